"""predict.x on the GPU: energies (and forces, atomic energies, relaxed
geometries) of the structures listed in a predict.x input file.

    python -m aenet_gb300.predict <input-file> [<structure files>] [--mixed]

Reads the same input file as the reference's predict.x (keywords of
read_InpPredict, src/input.f90:358-400: TYPES, NETWORKS, FORCES,
PRINT_ATOMIC_ENERGIES, RELAX, FILES, VERBOSITY) and XSF structures, and
prints the reference's report (print_fileinfo / print_coordinates /
print_energy, src/predict.F90:436-575) with each structure evaluated in one
GPU call (neighbour search included) instead of predict.x's per-atom loop.

RELAX minimises the cohesive energy in Cartesian coordinates with L-BFGS-B
(F_conv on the RMS force, E_conv on the energy change, steps).  The
reference hands lattice coordinates and Cartesian forces to its optimiser
(opt_bfgs_coords, src/optimize.f90:1775-1843); here coordinates and
gradient are both Cartesian, so relaxation paths differ from predict.x's.
"""
import argparse
import os
import sys

import numpy as np

from .core import ANNPotentials, FP64, MIXED
from .xsf import read_xsf

__all__ = ["read_input", "main"]


def _clean(line):
    return line.split("!", 1)[0].split("#", 1)[0].strip()


def read_input(path):
    """Parse a predict.x input file into a dict."""
    lines = [_clean(l) for l in open(path)]
    lines = [l for l in lines if l]
    inp = {"types": [], "networks": {}, "forces": False, "print_atomic_energies": False,
           "relax": None, "files": [], "verbosity": 1, "timing": False}
    base = os.path.dirname(os.path.abspath(path))
    i = 0
    while i < len(lines):
        f = lines[i].split()
        key = f[0].lower()
        if key == "types":
            n = int(lines[i + 1].split()[0])
            inp["types"] = [lines[i + 2 + k].split()[0] for k in range(n)]
            i += 2 + n
            continue
        if key == "networks":
            n = len(inp["types"])
            for k in range(n):
                t, fn = lines[i + 1 + k].split()[:2]
                inp["networks"][t] = fn if os.path.isabs(fn) else os.path.join(base, fn)
            i += 1 + n
            continue
        if key == "files":
            n = int(lines[i + 1].split()[0])
            for k in range(n):
                fn = lines[i + 2 + k].split()[0]
                inp["files"].append(fn if os.path.isabs(fn) else os.path.join(base, fn))
            i += 2 + n
            continue
        if key == "relax":
            opts = {"method": "bfgs", "F_conv": 0.01, "E_conv": 0.001, "steps": 99}
            if i + 1 < len(lines):
                for tok in lines[i + 1].split():
                    if "=" in tok:
                        k, v = tok.split("=", 1)
                        v = v.lower().replace("d", "e")
                        if k.lower() == "method":
                            opts["method"] = v
                        elif k.lower() == "steps":
                            opts["steps"] = int(float(v))
                        elif k.lower() in ("f_conv", "e_conv"):
                            opts["F_conv" if k.lower() == "f_conv" else "E_conv"] = float(v)
            inp["relax"] = opts
            inp["forces"] = True
            i += 1
            continue
        if key == "forces":
            inp["forces"] = True
        elif key == "print_atomic_energies":
            inp["print_atomic_energies"] = True
        elif key == "timing":
            inp["timing"] = True
        elif key == "verbosity" and len(f) > 1:
            inp["verbosity"] = int(f[1])
        i += 1
    if not inp["types"]:
        raise ValueError("no atom TYPES specified in file `%s'" % path)
    if len(inp["networks"]) != len(inp["types"]):
        raise ValueError("no NETWORKS specified in file `%s'" % path)
    return inp


def force_stats(F):
    """calc_rms_force (src/predict.F90:712-749): mean, mean absolute, the
    force of the atom with the largest |F| (1-based index) and the RMS."""
    F = np.asarray(F).reshape(-1, 3)
    f2 = (F * F).sum(1)
    imax = int(np.argmax(f2)) if np.any(f2 > 0) else 0
    return F.mean(0), np.abs(F).mean(0), (F[imax] if np.any(f2 > 0) else np.zeros(3)), imax + 1, \
        float(np.sqrt(f2.mean()))


class Report:
    def __init__(self, out):
        self.out = out

    def w(self, s=""):
        self.out.write(" " + s + "\n")

    def fileinfo(self, istruc, fn, cell, n, ntypes):
        self.w("Structure number  : %d" % istruc)
        self.w("File name         : %s" % fn)
        self.w("Number of atoms   : %d" % n)
        self.w("Number of species : %d" % ntypes)
        self.w()
        self.w("Lattice vectors (Angstrom):")
        self.w()
        for name, v in zip("abc", cell):
            self.out.write("   %s = ( %s )\n" % (name, "".join("  %15.8f" % x for x in v)))
        self.w()

    def coordinates(self, relaxed, symbols, pos, F=None, Ea=None):
        h = "Cartesian atomic coordinates" + (" (optimized)" if relaxed else " (input)")
        if F is not None:
            h += " and corresponding atomic forces"
        self.w(h + ":")
        self.w()
        hdr = "  " + "".join("  %-12s" % c for c in ("     x", "     y", "     z"))
        units = "  " + "".join("  %-12s" % "    (Ang)" for _ in range(3))
        dash = 44
        if F is not None:
            hdr += "".join("  %-12s" % c for c in ("     Fx", "    Fy", "    Fz"))
            units += "".join("  %-12s" % "  (eV/Ang)" for _ in range(3))
            dash += 42
        if Ea is not None:
            hdr += "  %-12s" % "   E_atom"
            units += "  %-12s" % "    (eV)"
            dash += 14
        self.w(hdr)
        self.w(units)
        self.w("-" * dash)
        for k, s in enumerate(symbols):
            line = "%-2s" % s + "".join("  %12.6f" % x for x in pos[k])
            if F is not None:
                line += "".join("  %12.6f" % x for x in F[k])
            if Ea is not None:
                line += "  %12.6f" % Ea[k]
            self.w(line)
        self.w()

    def energy(self, Ecoh, Etot, F=None):
        self.w("Cohesive energy            :  %20.8f eV" % Ecoh)
        self.w("Total energy               :  %20.8f eV" % Etot)
        if F is not None:
            avg, mav, mx, imax, rms = force_stats(F)
            self.w("Mean force (must be zero)  :" + "".join("  %12.6f" % x for x in avg))
            self.w("Mean absolute force        :" + "".join("  %12.6f" % x for x in mav))
            self.w("Maximum force              :" + "".join("  %12.6f" % x for x in mx))
            self.w("RMS force                  :  %12.6f" % rms)
            self.w("The maximum force is acting on atom %d." % imax)
            self.w("All forces are given in eV/Angstrom.")
        self.w()


def _bounding_box(pos):
    """geo_get_bounds (src/geometry.f90:538-580): the box predict.x reports
    for an isolated structure."""
    eps = 2.0e-6
    return np.diag(pos.max(0) - pos.min(0) + eps)


def evaluate(pot, s, forces, atomic, precision):
    r = pot.structure_energy_forces(s["positions"], s["symbols"], s["cell"], pbc=s["pbc"],
                                    precision=precision, forces=forces)
    return r


def main(argv=None, out=sys.stdout):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("input")
    ap.add_argument("structures", nargs="*")
    ap.add_argument("--mixed", action="store_true",
                    help="mixed precision (FP32 descriptors, networks, forces)")
    args = ap.parse_args(argv)
    inp = read_input(args.input)
    files = args.structures or inp["files"]
    if not files:
        sys.stderr.write("Error: no input structures specified in %s\n" % args.input)
        return 1
    precision = MIXED if args.mixed else FP64
    pot = ANNPotentials({t: inp["networks"][t] for t in inp["types"]})
    rep = Report(out)
    try:
        for k, fn in enumerate(files, start=1):
            s = read_xsf(fn)
            n = len(s["symbols"])
            cell = s["cell"] if s["pbc"] else _bounding_box(s["positions"])
            if inp["verbosity"] > 0:
                rep.fileinfo(k, fn, cell, n, len(set(s["symbols"])))
            r = evaluate(pot, s, inp["forces"], inp["print_atomic_energies"], precision)
            F = r["forces"] if inp["forces"] else None
            Ea = r["atomic_energies"] if inp["print_atomic_energies"] else None
            rep.coordinates(False, s["symbols"], s["positions"], F, Ea)
            if inp["relax"] is not None:
                x = _relax(pot, s, inp["relax"], precision, rep)
                s = dict(s, positions=x.reshape(-1, 3))
                r = evaluate(pot, s, True, False, precision)
                F = r["forces"]
                rep.w()
                rep.coordinates(True, s["symbols"], s["positions"], F)
            rep.energy(r["cohesive_energy"], r["energy"], F)
            if k < len(files):
                rep.w("+" * 70)
                rep.w()
    finally:
        pot.release()
    return 0


def _relax(pot, s, opts, precision, rep):
    """L-BFGS-B relaxation with the reference's convergence knobs."""
    from scipy.optimize import minimize
    E0 = {"v": None}
    hist = {"it": 0, "prev": None, "x": s["positions"].ravel().copy()}

    def fg(x):
        r = pot.structure_energy_forces(x.reshape(-1, 3), s["symbols"], s["cell"], pbc=s["pbc"],
                                        precision=precision)
        if E0["v"] is None:
            E0["v"] = r["cohesive_energy"]
        return r["cohesive_energy"], -r["forces"].ravel()

    rep.w("Geometry optimization:")
    rep.w()
    rep.w("       " + "   energy change  " + "     rms force    ")
    rep.w("       " + "        (eV)      " + "     (eV/Ang)     ")
    rep.w("-" * 60)

    class Converged(Exception):
        pass

    last = {"E": None}

    def cb(x):
        hist["it"] += 1
        hist["x"] = x.copy()
        E, g = fg(x)
        rms = float(np.sqrt((g.reshape(-1, 3) ** 2).sum(1).mean()))
        if hist["prev"] is None:
            rep.out.write(" %5d  %16.8f  %16.8f\n" % (hist["it"], E - E0["v"], rms))
        else:
            rep.out.write(" %5d  %16.8f  %16.8f  %16.8f\n"
                          % (hist["it"], E - E0["v"], rms, rms - hist["prev"]))
        hist["prev"] = rms
        dE = None if last["E"] is None else abs(E - last["E"])
        last["E"] = E
        if rms < opts["F_conv"] or (dE is not None and dE < opts["E_conv"]):
            raise Converged()

    try:
        res = minimize(fg, hist["x"], jac=True, method="L-BFGS-B", callback=cb,
                       options={"maxiter": opts["steps"], "maxcor": 20, "gtol": 1e-12,
                                "ftol": 1e-15})
        hist["x"] = res.x
    except Converged:
        rep.w("   converged after %d iterations." % hist["it"])
    return hist["x"]


if __name__ == "__main__":
    sys.exit(main())
