"""The two largest workloads at their full sizes.

  lisio_batch_4096   4096 periodic Li/Si/O cells, 16-512 atoms each
                     (~597k atoms), Chebyshev r10/6.0 a4/4.0, species-weighted
  cuau_fcc_1m        one 1,048,576-atom Cu/Au FCC crystal, Chebyshev
                     r16/6.0 a8/4.0, species-weighted

The oracle is too slow for every atom of these, so it pins a sample (whole
structures of the batch; the first atoms of the crystal), and the rest is
checked through properties that hold at any size:
  - FP64 forces of each structure sum to zero (the energy depends on the
    interatomic vectors only), to rounding;
  - FP64 virials are symmetric (the energy is rotation invariant);
  - the mixed path stays within 1 meV/atom and 20 meV/A RMS of FP64 on
    every structure;
  - the host-buffer call (chunks on several streams) and one device plan
    over the whole batch give the same energies.
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu

E_TOL_FP64 = 1e-10      # eV/atom against the oracle
F_TOL_FP64 = 1e-9       # eV/A against the oracle
E_TOL_MIXED = 1e-3      # eV/atom, mixed against FP64
F_RMS_MIXED = 2e-2      # eV/A, mixed against FP64


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _force_sum_tol(n, F):
    # FP64 rounding of n per-atom sums of pair terms, each of size |F|
    return 1e-12 * n * max(1.0, float(np.abs(F).max()))


def test_lisio_batch_4096_full_size(cuda, oracle, tmp_path):
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials, FP64, MIXED
    w = workloads.lisio_batch_4096()
    assert len(w.structures) == 4096
    oracle.set_candidates("cells")
    try:
        paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=2000)
    finally:
        oracle.set_candidates("complete")
    structs = [(s.positions, s.types, s.cell, True) for s in w.structures]
    nat = np.array([s.natoms for s in w.structures])
    off = np.concatenate([[0], np.cumsum(nat)])
    ann = ANNPotentials({t: paths[t] for t in w.types})
    try:
        r64 = ann.batch_energy_forces(structs, precision=FP64, virial=True)
        r32 = ann.batch_energy_forces(structs, precision=MIXED)
        # one device plan over the whole batch (the bench's device-resident path)
        from aenet_gb300.plan import Plan
        nat_p, pos, typ, cells, pbc = w.packed()
        plan = Plan(nat_p, cells, pbc, precision=FP64)
        out = plan.run(cuda.tensor(pos, device="cuda"), cuda.tensor(typ, device="cuda"),
                       forces=False)
        plan.check()
        Ep = out["E"].cpu().numpy()
        plan.close()
    finally:
        ann.release()
    assert int(off[-1]) == r64["forces"].shape[0]

    # oracle: the smallest and largest cells and four others
    rng = np.random.default_rng(7)
    pick = sorted({int(np.argmin(nat)), int(np.argmax(nat)),
                   *rng.choice(len(nat), 4, replace=False).tolist()})
    oracle.load(w.types, paths)
    oracle.set_candidates("cells")
    try:
        for k in pick:
            s = w.structures[k]
            _, et, F, _ = oracle.structure(s.cell, s.positions, s.types, nthreads=8)
            assert abs(r64["energy"][k] - et) / s.natoms < E_TOL_FP64, k
            assert np.abs(r64["forces"][off[k]:off[k + 1]] - F).max() < F_TOL_FP64, k
    finally:
        oracle.set_candidates("complete")

    # properties of every structure
    F64 = r64["forces"]
    for k in range(len(nat)):
        Fk = F64[off[k]:off[k + 1]]
        assert np.abs(Fk.sum(axis=0)).max() < _force_sum_tol(nat[k], Fk), k
    W = r64["virial"]
    asym = np.abs(W - W.transpose(0, 2, 1)).max(axis=(1, 2))
    assert (asym <= 1e-9 * np.maximum(1.0, np.abs(W).max(axis=(1, 2)))).all()
    dE = np.abs(r32["energy"] - r64["energy"]) / nat
    assert dE.max() < E_TOL_MIXED, dE.max()
    dF = r32["forces"] - F64
    assert np.sqrt(np.mean(dF ** 2)) < F_RMS_MIXED
    assert np.abs(dF).max() < 10 * F_RMS_MIXED
    # host-buffer chunks and one device plan: same FP64 energies
    assert (np.abs(Ep - r64["energy"]) / nat).max() < 1e-11


def test_cuau_fcc_1m_full_size(cuda, oracle, tmp_path):
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials, FP64, MIXED
    w = workloads.cuau_fcc_1m()
    s = w.structures[0]
    assert s.natoms == 1048576
    oracle.set_candidates("cells")
    try:
        paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=1000)
    finally:
        oracle.set_candidates("complete")
    ann = ANNPotentials({t: paths[t] for t in w.types})
    try:
        r64 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64,
                                          virial=True)
        r32 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=MIXED)
    finally:
        ann.release()
    n = s.natoms

    # oracle: the first 2000 atoms' energies
    oracle.load(w.types, paths)
    oracle.set_candidates("cells")
    try:
        _, _, _, Ea = oracle.structure(s.cell, s.positions, s.types, forces=False,
                                       nthreads=16, atom_limit=2000)
    finally:
        oracle.set_candidates("complete")
    assert np.abs(r64["atomic_energies"][:2000] - Ea[:2000]).max() < E_TOL_FP64

    F64 = r64["forces"]
    assert np.abs(F64.sum(axis=0)).max() < _force_sum_tol(n, F64)
    W = r64["virial"]
    assert np.abs(W - W.T).max() <= 1e-9 * max(1.0, np.abs(W).max())
    assert abs(r64["energy"] - r64["atomic_energies"].sum()) < 1e-9 * n
    assert abs(r32["energy"] - r64["energy"]) / n < E_TOL_MIXED
    dF = r32["forces"] - F64
    assert np.sqrt(np.mean(dF ** 2)) < F_RMS_MIXED
    assert np.abs(dF).max() < 10 * F_RMS_MIXED


def test_tio2_rutile_9000_full_size(cuda, oracle, tmp_path):
    """The Behler-Parrinello configuration at its stated size: rutile Ti/O
    10x10x15 unit cells (9000 atoms), 8 G2 per pair and 16 G4 per triple
    (64 features), Rc 6.5 A, 64-30-30-1 networks.  FP64 energies and
    forces of every atom against the oracle (the whole structure, the
    reference's per-atom loop on all host cores); the FP64 virial against
    central differences of the FP64 energy under strain; the mixed path
    within 1 meV/atom and 20 meV/A RMS of FP64."""
    import os
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials, FP64, MIXED
    w = workloads.tio2_rutile_9000()
    s = w.structures[0]
    assert s.natoms == 9000
    paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=600)
    ann = ANNPotentials({t: paths[t] for t in w.types})
    try:
        r64 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64,
                                          virial=True)
        r32 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=MIXED,
                                          virial=True)
        h = 1e-5
        W = np.zeros((3, 3))
        for a in range(3):
            for b in range(3):
                E = []
                for sgn in (-1, 1):
                    eps = np.eye(3)
                    eps[a, b] += sgn * h
                    E.append(ann.structure_energy_forces(s.positions @ eps, s.types,
                                                         s.cell @ eps, precision=FP64,
                                                         forces=False)["energy"])
                W[a, b] = -(E[1] - E[0]) / (2 * h)
    finally:
        ann.release()
    n = s.natoms
    oracle.load(w.types, paths)
    oracle.set_candidates("cells")
    try:
        ec, et, F, Ea = oracle.structure(s.cell, s.positions, s.types,
                                         nthreads=os.cpu_count() or 1)
    finally:
        oracle.set_candidates("complete")
    assert abs(r64["energy"] - et) / n < E_TOL_FP64
    assert np.abs(r64["atomic_energies"] - Ea).max() < E_TOL_FP64
    assert np.abs(r64["forces"] - F).max() < F_TOL_FP64
    F64 = r64["forces"]
    assert np.abs(F64.sum(axis=0)).max() < _force_sum_tol(n, F64)
    # central differences of an energy of ~-2e4 eV at h = 1e-5: ~1e-6 relative
    assert np.abs(r64["virial"] - W).max() < 1e-5 * max(1.0, np.abs(W).max())
    assert np.abs(W - W.T).max() <= 1e-5 * max(1.0, np.abs(W).max())
    assert abs(r32["energy"] - r64["energy"]) / n < E_TOL_MIXED
    dF = r32["forces"] - F64
    assert np.sqrt(np.mean(dF ** 2)) < F_RMS_MIXED
    assert np.abs(dF).max() < 10 * F_RMS_MIXED
    dV = r32["virial"] - r64["virial"]
    assert np.abs(dV).max() < 1e-3 * max(1.0, np.abs(r64["virial"]).max())
