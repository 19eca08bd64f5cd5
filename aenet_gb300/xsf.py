"""XCrySDen structure files (XSF), as predict.x reads them (src/xsflib.f90
via geo_init_xsf, src/geometry.f90:655-720).

Supported: ``ATOMS`` (isolated structure, Cartesian coordinates) and
``CRYSTAL`` with ``PRIMVEC`` and ``PRIMCOORD`` (periodic); optional force
columns after the coordinates; ``#`` starts a comment.
"""
import numpy as np

__all__ = ["read_xsf", "write_xsf"]


def _records(path):
    with open(path) as fh:
        for line in fh:
            line = line.split("#", 1)[0].strip()
            if line:
                yield line


def read_xsf(path):
    """Return dict(symbols, positions (N,3), cell (3,3) rows or None, pbc,
    forces (N,3) or None)."""
    lines = list(_records(path))
    symbols, pos, forces = [], [], []
    cell = None
    pbc = False
    i = 0
    while i < len(lines):
        key = lines[i].split()[0].upper()
        if key == "ATOMS":
            i += 1
            while i < len(lines) and lines[i].split()[0].upper() not in (
                    "ATOMS", "CRYSTAL", "PRIMVEC", "PRIMCOORD", "CONVVEC", "SLAB", "POLYMER",
                    "MOLECULE"):
                f = lines[i].split()
                symbols.append(f[0])
                pos.append([float(x) for x in f[1:4]])
                if len(f) >= 7:
                    forces.append([float(x) for x in f[4:7]])
                i += 1
            continue
        if key == "CRYSTAL":
            pbc = True
        elif key == "PRIMVEC":
            cell = np.array([[float(x) for x in lines[i + k].split()[:3]] for k in (1, 2, 3)])
            i += 4
            continue
        elif key == "PRIMCOORD":
            n = int(lines[i + 1].split()[0])
            for k in range(n):
                f = lines[i + 2 + k].split()
                symbols.append(f[0])
                pos.append([float(x) for x in f[1:4]])
                if len(f) >= 7:
                    forces.append([float(x) for x in f[4:7]])
            i += 2 + n
            continue
        i += 1
    if not symbols:
        raise ValueError("%s: no atoms" % path)
    if pbc and cell is None:
        raise ValueError("%s: CRYSTAL without PRIMVEC" % path)
    return {"symbols": symbols, "positions": np.array(pos, dtype=np.float64),
            "cell": cell, "pbc": bool(pbc),
            "forces": np.array(forces) if len(forces) == len(symbols) else None}


def write_xsf(path, symbols, positions, cell=None, forces=None, comment=None):
    with open(path, "w") as fh:
        if comment:
            fh.write("# %s\n\n" % comment)
        rows = []
        for k, s in enumerate(symbols):
            r = "%-3s %16.10f %16.10f %16.10f" % ((s,) + tuple(positions[k]))
            if forces is not None:
                r += " %16.10f %16.10f %16.10f" % tuple(forces[k])
            rows.append(r)
        if cell is None:
            fh.write("ATOMS\n" + "\n".join(rows) + "\n")
        else:
            fh.write("CRYSTAL\nPRIMVEC\n")
            for v in np.asarray(cell):
                fh.write("%16.10f %16.10f %16.10f\n" % tuple(v))
            fh.write("PRIMCOORD\n%d 1\n" % len(symbols) + "\n".join(rows) + "\n")
