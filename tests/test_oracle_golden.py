"""The oracle against the reference's own golden values (no GPU).

K-1  python3/aenet/tests/test_ase.py:58      Ti2O4 total energy
K-2  python3/aenet/tests/test_core.py:29-30  Rc_min / Rc_max of the Ti/O pair
K-3  unittests/Cu-dimer-forces               81-point Behler dimer scan
"""
import numpy as np
import pytest

from tests.golden import fixtures


@pytest.fixture(scope="module")
def k1():
    return fixtures.load("k1_ti2o4.npz")


@pytest.fixture(scope="module")
def k3():
    return fixtures.load("k3_cu_dimer.npz")


def _types(npz, symbols):
    names = [str(t) for t in npz["types"]]
    return np.array([names.index(str(s)) + 1 for s in symbols], dtype=np.int32)


def test_k1_ti2o4_energy_legacy_angular(oracle, k1):
    pots = fixtures.potentials(k1)
    oracle.load(["Ti", "O"], pots, angular="legacy")
    types = _types(k1, k1["symbols"])
    ec, et, F, Ea = oracle.structure(k1["cell"], k1["positions"], types)
    # test_ase.py:58 uses assertAlmostEqual (7 places); the restatement is
    # exact to the 12 printed digits.
    assert abs(et - float(k1["E_total"])) < 1e-9
    assert abs(Ea.sum() - et) < 1e-9
    # forces sum to zero (translation invariance)
    assert np.abs(F.sum(axis=0)).max() < 1e-10


def test_k1_forces_match_central_differences(oracle, k1):
    """test_ase.py:62-86: forces vs central differences (d = 0.01)."""
    pots = fixtures.potentials(k1)
    oracle.load(["Ti", "O"], pots, angular="legacy")
    types = _types(k1, k1["symbols"])
    pos = np.array(k1["positions"])
    _, _, F, _ = oracle.structure(k1["cell"], pos, types)
    d = 0.01
    for ia in range(len(pos)):
        for c in range(3):
            p1 = pos.copy(); p1[ia, c] -= d
            p2 = pos.copy(); p2[ia, c] += d
            e1 = oracle.structure(k1["cell"], p1, types, forces=False)[1]
            e2 = oracle.structure(k1["cell"], p2, types, forces=False)[1]
            assert abs(F[ia, c] + (e2 - e1) / (2 * d)) < 5e-3


def test_k2_cutoff_range(oracle, k1):
    oracle.load(["Ti", "O"], fixtures.potentials(k1))
    assert oracle.Rc_min == float(k1["Rc_min"])
    assert oracle.Rc_max == float(k1["Rc_max"])


def test_k3_cu_dimer_scan(oracle, k3):
    types = [str(t) for t in k3["types"]]
    oracle.load(types, fixtures.potentials(k3))
    cu = types.index("Cu") + 1
    for x, F, ec, et in zip(k3["positions"], k3["forces"], k3["E_coh"], k3["E_total"]):
        ecm, etm, Fm, _ = oracle.structure(None, x, [cu, cu], pbc=False)
        assert abs(ecm - ec) <= 5.1e-9       # printed with F20.8
        assert abs(etm - et) <= 5.1e-9
        assert np.abs(Fm - F).max() <= 5.1e-7  # printed with F12.6


def test_k3_cell_list_as_written_misses_far_dimer_partner(oracle, k3):
    """The linked-cell search of lclist.f90 as written misses the partner of
    a dimer beyond ~4.6 A in the thin isolated bounding box, so the current
    reference source would not reproduce its own 2013 outputs there; the
    complete candidate mode does."""
    types = [str(t) for t in k3["types"]]
    oracle.load(types, fixtures.potentials(k3))
    cu = types.index("Cu") + 1
    x = k3["positions"][32]            # 5.2 A
    try:
        oracle.set_candidates("cells")
        ec_cells = oracle.structure(None, x, [cu, cu], pbc=False)[0]
    finally:
        oracle.set_candidates("complete")
    ec_full = oracle.structure(None, x, [cu, cu], pbc=False)[0]
    assert abs(ec_full - k3["E_coh"][32]) < 5.1e-9
    assert abs(ec_cells - k3["E_coh"][32]) > 1e-3


def test_nn_roundtrip_product_writer_oracle_reader(tmp_path, k1, k3):
    from oracle.nnfile import parse_nn
    for npz in (k1, k3):
        pots = fixtures.potentials(npz)
        paths = fixtures.write_potential_files(pots, str(tmp_path))
        for t, p in paths.items():
            back = parse_nn(p)
            assert back["legacy"] == pots[t]["legacy"]
            np.testing.assert_array_equal(back["net"]["W"], pots[t]["net"]["W"])
            np.testing.assert_array_equal(back["stp"]["sfval_avg"], pots[t]["stp"]["sfval_avg"])
            assert back["stp"]["envtypes"] == list(pots[t]["stp"]["envtypes"])
            assert back["ts"]["E_atom"].tolist() == list(pots[t]["ts"]["E_atom"])


def test_cell_search_as_written_is_complete_on_small_cells(oracle):
    """On the batch workload's cells (some shorter than the cut-off) the
    linked-cell search of lclist.f90 finds the same neighbour sets as the
    complete search, so the reference's own lists are the oracle's."""
    from aenet_gb300 import workloads
    w = workloads.lisio_batch_4096(nstruc=5)
    from tests.golden import fixtures
    k1 = fixtures.load("k1_ti2o4.npz")
    oracle.load(["Ti", "O"], fixtures.potentials(k1))
    for s in w.structures:
        sets = []
        for mode in ("cells", "complete"):
            oracle.set_candidates(mode)
            _, _, nb = oracle.neighbors(s.cell, s.positions, np.minimum(s.types, 2))
            sets.append([sorted(zip(x[2].tolist(), map(tuple, x[0].tolist()))) for x in nb])
        oracle.set_candidates("complete")
        assert sets[0] == sets[1]


def test_oracle_weight_gradient_matches_finite_differences(oracle, k1, tmp_path):
    """ff_wderiv restatement (feedforward.f90:763-860) against central
    differences of the atomic energy with respect to single weights of the
    K-1 Ti network (44-15-15-1): hidden-layer weights, biases and the
    output layer."""
    import copy
    pots = fixtures.potentials(k1)
    paths = fixtures.write_potential_files(pots, str(tmp_path))
    oracle.load(["Ti", "O"], paths, angular="legacy")
    types = _types(k1, k1["symbols"])
    _, centres, nb = oracle.neighbors(k1["cell"], k1["positions"], types, atoms=[0])
    nbcoo, _, _, nbt = nb[0]
    E0, g = oracle.atomic_energy_wgrad(centres[0], int(types[0]), nbcoo, nbt)
    assert abs(E0 - oracle.atomic_energy(centres[0], int(types[0]), nbcoo, nbt)) < 1e-12
    W = np.array(pots["Ti"]["net"]["W"], dtype=np.float64)
    nw = W.size
    # first layer (weight, bias), second layer, output weight and bias
    picks = [0, 7, 44 * 15 + 3, 45 * 15 + 2, 45 * 15 + 16 * 15 - 1, nw - 2, nw - 1]

    def energy(w):
        p = copy.deepcopy(pots)
        p["Ti"]["net"]["W"] = w
        ps = fixtures.write_potential_files(p, str(tmp_path))
        oracle.load(["Ti", "O"], ps, angular="legacy")
        return oracle.atomic_energy(centres[0], int(types[0]), nbcoo, nbt)

    for k in picks:
        h = 1e-4 * max(1.0, abs(W[k]))
        f = {}
        for m in (-2, -1, 1, 2):
            w = W.copy()
            w[k] += m * h
            f[m] = energy(w)
        fd = (8 * (f[1] - f[-1]) - (f[2] - f[-2])) / (12 * h)
        assert abs(fd - g[k]) <= 1e-7 * max(1.0, abs(g[k])), (k, fd, g[k])


def test_k5_fcc_neighbour_count_and_rotation_invariance(oracle, tmp_path):
    """K-5 (src/tests/*.f90 properties): 12 nearest neighbours in FCC, and
    energies invariant under a rotation of the structure with its cell."""
    from aenet_gb300 import workloads
    from tests import helpers
    w = workloads.cu_fcc_256()
    paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=64)
    oracle.load(w.types, paths)
    pos, cell = workloads.fcc_positions(4, 3.61)
    types = np.ones(len(pos), dtype=np.int32)
    _, _, nb = oracle.neighbors(cell, pos, types, Rc=3.61 / np.sqrt(2) + 0.05, atoms=[0, 17, 100])
    assert [len(x[0]) for x in nb] == [12, 12, 12]
    s = w.structures[0]
    rng = np.random.default_rng(11)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    e0 = oracle.structure(s.cell, s.positions, s.types, forces=False)[1]
    e1 = oracle.structure(s.cell @ q, s.positions @ q, s.types, forces=False)[1]
    assert abs(e1 - e0) / s.natoms < 1e-10


@pytest.mark.parametrize("which", ["behler", "chebyshev"])
def test_oracle_descriptor_derivatives_match_finite_differences(oracle, tmp_path, which):
    """The oracle's raw descriptor derivatives (what the GPU Jacobian export
    is checked against) against central differences of its descriptors,
    with respect to the central atom and to single neighbours: Behler
    G2/G4 (symmfunc, rutile Ti/O) and the species-weighted Chebyshev basis
    (sfbasis, Li/Si/O)."""
    from aenet_gb300 import workloads
    from tests import helpers
    if which == "behler":
        w = workloads.tio2_rutile_9000(cells=(1, 1, 2))
    else:
        w = workloads.lisio_batch_4096(nstruc=2)
    s = w.structures[0]
    paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=64)
    oracle.load(w.types, paths)
    _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types, atoms=[0, 1])
    h = 1e-5
    for a in (0, 1):
        nbcoo, _, _, nbt = nb[a]
        ti = int(s.types[a])

        def G(ci, cj):
            return oracle.descriptor(ci, ti, cj, nbt, scaled=False)

        G0, di, dj = oracle.descriptor(centres[a], ti, nbcoo, nbt, scaled=False, deriv=True)
        tol = 1e-6 * max(1.0, np.abs(di).max(), np.abs(dj).max())
        for c in range(3):
            e = np.zeros(3)
            e[c] = h
            fd = (G(centres[a] + e, nbcoo) - G(centres[a] - e, nbcoo)) / (2 * h)
            assert np.abs(fd - di[:, c]).max() <= tol, (a, c)
        for j in (0, len(nbt) // 2, len(nbt) - 1):
            for c in range(3):
                cp, cm = nbcoo.copy(), nbcoo.copy()
                cp[j, c] += h
                cm[j, c] -= h
                fd = (G(centres[a], cp) - G(centres[a], cm)) / (2 * h)
                assert np.abs(fd - dj[j, :, c]).max() <= tol, (a, j, c)
