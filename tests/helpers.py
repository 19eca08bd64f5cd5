"""Shared test helpers (oracle-side workload statistics, tolerances)."""
import numpy as np

from aenet_gb300 import workloads


def oracle_descriptor_fn(oracle):
    """Raw descriptors of selected atoms computed by the FP64 oracle."""
    def fn(workload, paths, ids):
        oracle.load(workload.types, paths)
        rows, spec = [], []
        offset = 0
        ids = set(int(i) for i in ids)
        for s in workload.structures:
            local = [i - offset for i in range(offset, offset + s.natoms) if i in ids]
            offset += s.natoms
            if not local:
                continue
            _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types, pbc=s.pbc,
                                              atoms=local)
            for q, a in enumerate(local):
                nbcoo, _, nbl, nbt = nb[q]
                rows.append(oracle.descriptor(centres[a], int(s.types[a]), nbcoo, nbt,
                                              scaled=False))
                spec.append(int(s.types[a]))
        return np.array(rows), np.array(spec)
    return fn


def make_potentials(oracle, workload, directory, max_atoms=4000):
    return workloads.write_potentials(workload, directory, oracle_descriptor_fn(oracle),
                                      max_atoms_for_stats=max_atoms)
