"""Load the golden fixtures written by make_golden.py."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    return np.load(os.path.join(HERE, name), allow_pickle=False)


def potentials(npz):
    """Potential dicts (the layout of oracle.nnfile.parse_nn) by species."""
    out = {}
    for t in [str(x) for x in npz["types"]]:
        pot = {"net": {}, "stp": {}, "ts": {}, "legacy": bool(npz["pot.%s.legacy" % t])}
        pre = "pot.%s." % t
        for key in npz.files:
            if not key.startswith(pre) or key.endswith(".legacy"):
                continue
            part, field = key[len(pre):].split(".", 1)
            v = npz[key]
            if v.dtype.kind == "U":
                v = [str(x) for x in v] if v.ndim else str(v)
            elif v.ndim == 0:
                v = v.item()
            pot[part][field] = v
        if "sfval_cov" not in pot["stp"]:
            pot["stp"]["sfval_cov"] = None
        out[t] = pot
    return out


def write_potential_files(pots, directory):
    """Write each potential as a .nn file (product writer); returns paths."""
    from aenet_gb300.nnfile import write_nn
    paths = {}
    for t, pot in pots.items():
        p = os.path.join(directory, "%s.nn" % t)
        write_nn(p, pot["net"], pot["stp"], pot["ts"], legacy=pot["legacy"])
        paths[t] = p
    return paths
