"""Regenerate the golden fixtures from the reference tree (run by hand).

Reads the reference's own test inputs and recorded outputs -- nothing is
computed here -- and stores them as small ``.npz`` files:

* ``k1_ti2o4.npz``   python3/aenet/tests/test_ase.py:31-44,58 and
                     test_core.py:29-30: the Ti2O4 cell, the Ti/O Chebyshev
                     potentials (Ti.15t-15t.nn, O.15t-15t.nn) and the
                     expected total energy -4990.310783539421 eV.
* ``k3_cu_dimer.npz`` unittests/Cu-dimer-forces: the four Behler potentials
                     (16-record legacy setups), predict.in's type order and,
                     for each of the 81 dimer distances, the cohesive and
                     total energies (F20.8) and the forces (F12.6) printed in
                     output-reference/dimer-x*.xsf.out.

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT
        (or with the environment variable AENET_REFERENCE_ROOT set)
"""
import glob
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.nnfile import parse_nn  # noqa: E402


def pack_potential(prefix, pot, out):
    for part in ("net", "stp", "ts"):
        for k, v in pot[part].items():
            key = "%s.%s.%s" % (prefix, part, k)
            if v is None:
                continue
            if isinstance(v, list):
                v = np.array(v, dtype=str)
            out[key] = np.asarray(v)
    out[prefix + ".legacy"] = np.asarray(pot["legacy"])


def main(ref):
    out = {}
    tdir = os.path.join(ref, "python3", "aenet", "tests")
    for t in ("Ti", "O"):
        pack_potential("pot." + t, parse_nn(os.path.join(tdir, "%s.15t-15t.nn" % t)), out)
    out["types"] = np.array(["Ti", "O"])
    out["cell"] = np.array([(3.81382872, 0.00000000, 0.00000000),
                            (0.56886601, 3.77116440, 0.00000000),
                            (-2.19138173, -1.88561177, 4.88111931)])
    out["positions"] = np.array([
        (0.42651082, 2.82851745, 1.22027956), (1.76480257, -0.94296447, 3.66083922),
        (0.14225662, 0.94278546, 0.79509432), (2.04905661, 0.94276737, 4.08602446),
        (-0.14223328, -0.94276538, 3.23565398), (2.33354646, 2.82831821, 1.64546480)])
    out["symbols"] = np.array(["Ti", "Ti", "O", "O", "O", "O"])
    out["E_total"] = np.asarray(-4990.310783539421)
    out["Rc_min"] = np.asarray(0.55)
    out["Rc_max"] = np.asarray(8.0)
    np.savez_compressed(os.path.join(HERE, "k1_ti2o4.npz"), **out)

    out = {}
    ddir = os.path.join(ref, "unittests", "Cu-dimer-forces")
    types = ["Au", "Cu", "O", "H"]          # predict.in TYPES order
    for t in types:
        pack_potential("pot." + t, parse_nn(os.path.join(ddir, "%s.05t-05t.nn" % t)), out)
    out["types"] = np.array(types)
    rows = []
    for f in sorted(glob.glob(os.path.join(ddir, "output-reference", "dimer-x*.xsf.out"))):
        txt = open(f).read()
        ec = float(re.search(r"Cohesive energy\s*:\s*(\S+)", txt).group(1))
        et = float(re.search(r"Total energy\s*:\s*(\S+)", txt).group(1))
        atoms = [l.split() for l in txt.splitlines() if l.startswith(" Cu ")]
        x = [[float(v) for v in a[1:4]] for a in atoms]
        F = [[float(v) for v in a[4:7]] for a in atoms]
        rows.append((x, F, ec, et))
    out["positions"] = np.array([r[0] for r in rows])
    out["forces"] = np.array([r[1] for r in rows])
    out["E_coh"] = np.array([r[2] for r in rows])
    out["E_total"] = np.array([r[3] for r in rows])
    np.savez_compressed(os.path.join(HERE, "k3_cu_dimer.npz"), **out)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AENET_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set AENET_REFERENCE_ROOT)")
    main(root)
