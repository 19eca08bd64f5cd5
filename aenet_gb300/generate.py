"""generate.x on the GPU: descriptors of every atom of a set of structures,
written as an aenet training-set file.

Replaces the structure loop of src/generate.f90: per structure the cohesive
energy E_total - sum_i E_atom(type_i) (generate.f90:304-313) and, per atom,
type, Cartesian coordinates, forces and the raw (unnormalised) descriptor;
the footer carries each species' Setup with the running statistics of its
descriptors (stp_eval's min/max/avg/cov, src/sfsetup.f90:960-975), as
generate.x leaves them for train.x's normalisation.

The descriptors come from the GPU FP64 path: the potentials are loaded with
identity normalisation, so the plan's descriptor rows are the raw values.
With ``forces_percent`` the descriptor Jacobians of that share of the
structures are written beside the training set in the PyTorch export
format of generate.x's FORCES keyword (aenet_gb300/pytorch_export.py).
"""
import os
import tempfile

import numpy as np
import torch

from . import nnfile
from .core import ANNPotentials, FP64
from .plan import Plan
from .pytorch_export import select_structures, write_forces_file
from .trainset import TrainSet, write_trainset
from .workloads import running_stats

__all__ = ["generate_trainset"]


def generate_trainset(potential_files, structures, path, forces_percent=None, seed=0):
    """``potential_files``: species -> .nn (their setups define the
    descriptors); ``structures``: dicts with positions, symbols, cell (None
    for isolated), energy (total, eV), optional forces and name.  Writes
    ``path`` and returns the TrainSet.  ``forces_percent`` (the FORCESPERCENT
    keyword, 0-100) also writes ``path + ".forces"`` with the descriptor
    Jacobians of that share of the structures (chosen with ``seed``)."""
    types = list(potential_files.keys())
    setups, E_atom = {}, {}
    tmp = tempfile.mkdtemp(prefix="aenet_generate_")
    ident_paths = {}
    legacy = False
    for t in types:
        net, stp, ts, leg = nnfile.read_nn(potential_files[t])
        legacy = legacy or leg
        setups[t] = stp
        E_atom[t] = float(ts["E_atom"][list(ts["typeName"]).index(t)])
        nsf = stp["nsf"]
        ident = dict(stp, sfval_min=np.zeros(nsf), sfval_max=np.zeros(nsf),
                     sfval_avg=np.zeros(nsf), sfval_cov=np.ones(nsf))
        ident_paths[t] = os.path.join(tmp, "%s.identity.nn" % t)
        nnfile.write_nn(ident_paths[t], net, ident, ts, legacy=False)
    ann = ANNPotentials(ident_paths)
    try:
        natoms = [len(s["symbols"]) for s in structures]
        pbc = np.array([0 if s.get("cell") is None else 1 for s in structures], dtype=np.int32)
        cells = np.stack([np.eye(3) if s.get("cell") is None else np.asarray(s["cell"], dtype=float)
                          for s in structures])
        pos = np.concatenate([np.asarray(s["positions"], dtype=float).reshape(-1, 3)
                              for s in structures])
        tid = np.concatenate([[types.index(x) + 1 for x in s["symbols"]] for s in structures])
        plan = Plan(natoms, cells, pbc, precision=FP64, coords0=pos)
        p = torch.tensor(pos, device="cuda")
        t = torch.tensor(tid.astype(np.int32), device="cuda")
        out = plan.run(p, t, forces=False)
        plan.check()
        G = plan.descriptors().cpu().numpy()
        if forces_percent is not None:
            _write_jacobians(plan, structures, natoms, tid, len(types), setups, types,
                             path + ".forces", forces_percent / 100.0, seed)
        plan.close()
    finally:
        ann.release()
    ts = TrainSet(types, [E_atom[x] for x in types], normalized=False, scale=1.0, shift=0.0)
    row = 0
    per_species = {k: [] for k in range(1, len(types) + 1)}
    for k, s in enumerate(structures):
        n = natoms[k]
        tt = tid[row:row + n]
        sf = [G[row + a, :setups[types[tt[a] - 1]]["nsf"]] for a in range(n)]
        for a in range(n):
            per_species[int(tt[a])].append(sf[a])
        ecoh = float(s["energy"]) - sum(E_atom[types[x - 1]] for x in tt)
        forces = s.get("forces")
        forces = np.zeros((n, 3)) if forces is None else np.asarray(forces, dtype=float)
        ts.add(s.get("name", "structure-%d" % (k + 1)), ecoh, tt, pos[row:row + n], forces, sf)
        row += n
    ts.E_av, ts.E_min, ts.E_max = ts.energy_range()
    ts.setup_records = []
    for k, name in enumerate(types, start=1):
        stp = dict(setups[name])
        if per_species[k]:
            mn, mx, av, cv = running_stats(np.array(per_species[k]))
            stp.update(sfval_min=mn, sfval_max=mx, sfval_avg=av, sfval_cov=cv,
                       neval=len(per_species[k]))
        ts.setup_records.append(nnfile.setup_payloads(stp, legacy=legacy))
    write_trainset(path, ts)
    return ts


def _write_jacobians(plan, structures, natoms, tid, ntypes, setups, types, path, fraction, seed):
    """Jacobians of the selected structures from the plan's last run, one
    structure at a time, in the PyTorch export format."""
    flags = select_structures(len(structures), fraction, seed)
    recs = []
    row = 0
    for k, s in enumerate(structures):
        n = natoms[k]
        rec = {"name": s.get("name", "structure-%d" % (k + 1)), "natoms": n, "ntypes": ntypes,
               "selected": bool(flags[k]), "atoms": []}
        if flags[k]:
            Ji, Jj, nbl, nnb = plan.jacobian(row, n)
            Ji, Jj, nbl, nnb = (x.cpu().numpy() for x in (Ji, Jj, nbl, nnb))
            for a in range(n):
                it = int(tid[row + a])
                nsf = setups[types[it - 1]]["nsf"]
                m = int(nnb[a])
                rec["atoms"].append((it, nbl[a, :m] - row + 1, Ji[a, :nsf],
                                     Jj[a, :m, :nsf]))
        recs.append(rec)
        row += n
    write_forces_file(path, recs)
