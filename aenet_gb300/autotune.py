"""Measured choice of the evaluator's launch shapes.

Two knobs decide most of the run time of a batch: the number of lanes that
cooperate on one atom in the descriptor and adjoint kernels (8, 16 or 32)
and the number of neighbour-search cells per cut-off length (1, 2 or 3).
:func:`tune` times a full energy-and-force pass of the caller's batch for
every combination (CUDA events on the current stream) and keeps the
fastest; results are cached per workload key in a JSON file.
"""
import json
import os

import torch

from . import core
from .plan import Plan

LANES = (8, 16, 32)
CELL_DIVS = (1, 2, 3)
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
         cache=CACHE, lanes=LANES, cell_divs=CELL_DIVS):
    """Return (lanes_per_atom, cell_div, ms) and apply them as options."""
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
        for cd in cell_divs:
            core.set_option("cell_div", cd)
            plan = Plan(natoms, cells, pbc, precision=precision, coords0=positions)
            for lp in lanes:
                core.set_option("lanes_per_atom", lp)
                results.append((_time(plan, p, t, reps), lp, cd))
            plan.close()
        ms, lp, cd = min(results)
        best = {"lanes_per_atom": lp, "cell_div": cd, "ms": ms,
                "all": [[r[1], r[2], r[0]] for r in results]}
        if key and cache:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            entries[key] = best
            tmp = cache + ".tmp%d" % os.getpid()
            json.dump(entries, open(tmp, "w"), indent=1)
            os.replace(tmp, cache)
    core.set_option("lanes_per_atom", best["lanes_per_atom"])
    core.set_option("cell_div", best["cell_div"])
    return best
