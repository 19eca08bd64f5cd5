"""Measured choice of the evaluator's launch shapes.

Four knobs decide most of the run time of a batch: the neighbour-search
kernel (one warp per atom over the full or the half stencil, or per home
cell with a lane per home atom or a lane per candidate), the number of neighbour-search cells per cut-off
length (1, 2 or 3), their refinement along the third axis (1, 2 or 4) and
the number of lanes that cooperate on one atom in the descriptor and
adjoint kernels (8, 16 or 32).  The first three only change the neighbour
search and the last only the descriptor kernels, so :func:`tune` times a
full energy-and-force pass of the caller's batch (CUDA events on the
current stream) over the kernel and cell size at a fixed lane count, then
the refinement, then the lane counts of the forward and of the adjoint;
results are cached per workload key in a JSON file.
"""
import json
import os

import torch

from . import core
from .plan import Plan

LANES = (8, 16, 32)
CELL_DIVS = (1, 2, 3)
Z_REFINES = (1, 2, 4)
NB_KERNELS = ("cell", "atom", "stream", "half", "struct", "struct_half")
CACHE = os.path.join(os.path.expanduser("~"), ".cache", "aenet_gb300", "autotune.json")


def _time(plan, p, t, reps):
    out = plan.run(p, t)
    plan.check()
    for _ in range(2):
        plan.run(p, t, out=out)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        plan.run(p, t, out=out)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(natoms, cells, pbc, positions, types, precision=core.MIXED, key=None, reps=3,
         cache=CACHE, lanes=LANES, cell_divs=CELL_DIVS, nb_kernels=NB_KERNELS,
         z_refines=Z_REFINES):
    """Return the chosen {neighbour_kernel, cell_div, z_refine,
    lanes_per_atom, adjoint_lanes_per_atom, ms} and apply them as options."""
    entries = {}
    if key and cache and os.path.exists(cache):
        try:
            entries = json.load(open(cache))
        except Exception:
            entries = {}
    if key and key in entries:
        best = entries[key]
    else:
        p = torch.as_tensor(positions, dtype=torch.float64, device="cuda").contiguous()
        t = torch.as_tensor(types, dtype=torch.int32, device="cuda").contiguous()
        results = []
        lp0 = lanes[0]
        core.set_option("lanes_per_atom", lp0)
        core.set_option("z_refine", 1)
        for cd in cell_divs:
            core.set_option("cell_div", cd)
            plan = Plan(natoms, cells, pbc, precision=precision, coords0=positions)
            for nk in nb_kernels:
                core.set_option("neighbour_kernel", nk)
                results.append((_time(plan, p, t, reps), lp0, cd, nk))
            plan.close()
        _, _, cd, nk = min(results)
        core.set_option("cell_div", cd)
        core.set_option("neighbour_kernel", nk)
        # finer cells along the third axis at the chosen search shape
        zres = [(min(results)[0], 1)]
        for zr in z_refines:
            if zr == 1:
                continue
            core.set_option("z_refine", zr)
            plan = Plan(natoms, cells, pbc, precision=precision, coords0=positions)
            zres.append((_time(plan, p, t, reps), zr))
            plan.close()
        zr = min(zres)[1]
        core.set_option("z_refine", zr)
        plan = Plan(natoms, cells, pbc, precision=precision, coords0=positions)
        for lp in lanes[1:]:
            core.set_option("lanes_per_atom", lp)
            results.append((_time(plan, p, t, reps), lp, cd, nk))
        plan.close()
        ms, lp, cd, nk = min(results)
        # the adjoint's lanes per atom, at the chosen forward shape
        core.set_option("lanes_per_atom", lp)
        plan = Plan(natoms, cells, pbc, precision=precision, coords0=positions)
        adj = [(ms, 0)]
        for la in lanes:
            if la == lp:
                continue
            core.set_option("adjoint_lanes_per_atom", la)
            adj.append((_time(plan, p, t, reps), la))
        core.set_option("adjoint_lanes_per_atom", 0)
        plan.close()
        ms, la = min(adj)
        best = {"neighbour_kernel": nk, "cell_div": cd, "z_refine": zr, "lanes_per_atom": lp,
                "adjoint_lanes_per_atom": la, "ms": ms,
                "all": [[r[3], r[2], r[1], r[0]] for r in results] +
                       [["z_refine", z[1], z[0]] for z in zres[1:]] +
                       [["adjoint", a[1], a[0]] for a in adj[1:]]}
        if key and cache:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            entries[key] = best
            tmp = cache + ".tmp%d" % os.getpid()
            json.dump(entries, open(tmp, "w"), indent=1)
            os.replace(tmp, cache)
    core.set_option("lanes_per_atom", best["lanes_per_atom"])
    core.set_option("cell_div", best["cell_div"])
    core.set_option("z_refine", best.get("z_refine", 1))
    core.set_option("neighbour_kernel", best.get("neighbour_kernel", "atom"))
    core.set_option("adjoint_lanes_per_atom", best.get("adjoint_lanes_per_atom", 0))
    return best
