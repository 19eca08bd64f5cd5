"""The neighbour-list entry point (MD engines with local + ghost atoms):
a periodic cell expressed as local atoms plus one shell of ghost images and
a full neighbour list built with a skin, against the same structure through
the periodic entry point (FP64: energy 1e-10 eV/atom, forces after folding
ghost forces onto their owners 1e-9 eV/A, virial 1e-8 eV)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _ghosts_and_list(pos, cell, rc):
    n = len(pos)
    shifts = [np.array([a, b, c]) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)
              if (a, b, c) != (0, 0, 0)]
    x = [pos] + [pos + s @ cell for s in shifts]
    owner = np.concatenate([np.arange(n)] * (1 + len(shifts)))
    x = np.concatenate(x)
    offs, nbr = [0], []
    for i in range(n):
        d = np.linalg.norm(x - pos[i], axis=1)
        js = np.where((d <= rc) & (np.arange(len(x)) != i))[0]
        nbr.extend(js.tolist())
        offs.append(len(nbr))
    return x, owner, np.array(offs, dtype=np.int32), np.array(nbr, dtype=np.int32)


def test_neighbor_list_entry_matches_periodic(cuda, oracle, tmp_path):
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials, FP64, MIXED
    from tests import helpers
    w = workloads.aucu_fcc_4000()
    keep = np.all(workloads.fcc_positions(10, 3.90)[0] < 4 * 3.90 - 0.1, axis=1)
    s = w.structures[0]
    pos, typ = s.positions[keep], s.types[keep]
    cell = np.eye(3) * 4 * 3.90
    sub = workloads.Workload(w.name, w.types, w.setups, w.arch,
                             [workloads.Structure(pos, typ, cell)], w.seed)
    sub.networks = w.networks
    paths = helpers.make_potentials(oracle, sub, str(tmp_path))
    ann = ANNPotentials({t: paths[t] for t in w.types}, angular_domain="current")
    try:
        x, owner, offs, nbr = _ghosts_and_list(pos, cell, ann.Rc_max + 0.5)
        types_all = typ[owner]
        n = len(pos)
        for prec, etol, ftol in ((FP64, 1e-10, 1e-9), (MIXED, 1e-3, 2e-2)):
            ref = ann.structure_energy_forces(pos, typ, cell, precision=prec, virial=True)
            r = ann.neighbor_list_energy_forces(x, types_all, offs, nbr, n, precision=prec,
                                                virial=True)
            folded = np.zeros((n, 3))
            np.add.at(folded, owner, r["forces"])
            assert abs(r["energy"] - ref["energy"]) / n < etol
            if prec == FP64:
                assert np.abs(folded - ref["forces"]).max() < ftol
                assert np.abs(r["virial"] - ref["virial"]).max() < 1e-8
                assert np.abs(r["atomic_energies"] - ref["atomic_energies"]).max() < 1e-10
            else:
                assert np.sqrt(np.mean((folded - ref["forces"]) ** 2)) < ftol
    finally:
        ann.release()
