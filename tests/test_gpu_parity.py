"""GPU evaluator against the FP64 oracle and the reference's golden values.

Tolerances (stated by the evaluation contract):
  FP64 path   energy within 1e-10 eV/atom of the oracle, forces 1e-9 eV/A;
              neighbour sets identical (bit for bit).
  mixed path  energy within 1 meV/atom, force RMS within 20 meV/A of FP64.
"""
import ctypes as C

import numpy as np
import pytest

from tests import helpers
from tests.golden import fixtures

pytestmark = pytest.mark.gpu

E_TOL_FP64 = 1e-10      # eV/atom
F_TOL_FP64 = 1e-9       # eV/A
E_TOL_MIXED = 1e-3      # eV/atom
F_RMS_MIXED = 2e-2      # eV/A


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


@pytest.fixture(scope="module")
def cu256(oracle, tmp_path_factory):
    from aenet_gb300 import workloads
    w = workloads.cu_fcc_256()
    d = tmp_path_factory.mktemp("cu256")
    oracle.set_candidates("cells")
    paths = helpers.make_potentials(oracle, w, str(d))
    oracle.set_candidates("complete")
    return w, paths


@pytest.fixture(scope="module")
def aucu(oracle, tmp_path_factory):
    from aenet_gb300 import workloads
    w = workloads.aucu_fcc_4000()
    d = tmp_path_factory.mktemp("aucu")
    paths = helpers.make_potentials(oracle, w, str(d), max_atoms=1000)
    return w, paths


@pytest.fixture(params=["atom", "cell", "stream", "half", "struct", "atom_z4", "stream_z2",
                        "half_z4", "struct_z4"])
def nb_kernel(request, cuda):
    """Run a test with each neighbour-search kernel (one warp per atom over
    the full or the half stencil, or one warp per home cell with a lane per
    home atom or per candidate), also on grids refined along the third
    axis; restores the defaults afterwards."""
    from aenet_gb300.core import set_option
    kernel, _, z = request.param.partition("_z")
    set_option("neighbour_kernel", kernel)
    set_option("z_refine", int(z or 1))
    yield request.param
    set_option("neighbour_kernel", "atom")
    set_option("z_refine", 1)


def _ann(paths, types, angular=None):
    from aenet_gb300.core import ANNPotentials
    return ANNPotentials({t: paths[t] for t in types}, angular_domain=angular or "current")


def test_k1_ti2o4_golden_energy_on_gpu(cuda, oracle, tmp_path):
    from aenet_gb300.core import FP64
    k1 = fixtures.load("k1_ti2o4.npz")
    pots = fixtures.potentials(k1)
    paths = fixtures.write_potential_files(pots, str(tmp_path))
    sym = [str(s) for s in k1["symbols"]]
    ann = _ann(paths, ["Ti", "O"], "legacy")
    try:
        r = ann.structure_energy_forces(k1["positions"], sym, k1["cell"], precision=FP64)
        assert ann.Rc_min == 0.55 and ann.Rc_max == 8.0
    finally:
        ann.release()
    assert abs(r["energy"] - float(k1["E_total"])) < 1e-9
    oracle.load(["Ti", "O"], pots, angular="legacy")
    types = np.array([1 if s == "Ti" else 2 for s in sym], dtype=np.int32)
    ec, et, F, Ea = oracle.structure(k1["cell"], k1["positions"], types)
    assert np.abs(r["forces"] - F).max() < F_TOL_FP64
    assert np.abs(r["atomic_energies"] - Ea).max() < E_TOL_FP64
    assert abs(r["cohesive_energy"] - ec) < 1e-9


def test_cu256_fp64_matches_oracle(cuda, oracle, cu256):
    from aenet_gb300.core import FP64
    w, paths = cu256
    s = w.structures[0]
    ann = _ann(paths, w.types)
    try:
        r = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64, virial=True)
    finally:
        ann.release()
    oracle.load(w.types, paths)
    ec, et, F, Ea = oracle.structure(s.cell, s.positions, s.types)
    n = s.natoms
    assert abs(r["energy"] - et) / n < E_TOL_FP64
    assert np.abs(r["atomic_energies"] - Ea).max() < E_TOL_FP64
    assert np.abs(r["forces"] - F).max() < F_TOL_FP64
    assert np.abs(r["forces"].sum(0)).max() < 1e-9


def test_cu256_virial_matches_strain_derivative(cuda, oracle, cu256):
    """W = -dE/d(strain) by central differences of the oracle energy."""
    from aenet_gb300.core import FP64
    w, paths = cu256
    s = w.structures[0]
    ann = _ann(paths, w.types)
    try:
        r = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64, virial=True)
    finally:
        ann.release()
    oracle.load(w.types, paths)
    h = 1e-5
    W = np.zeros((3, 3))
    for a in range(3):
        for b in range(3):
            E = []
            for sgn in (-1, 1):
                eps = np.eye(3)
                eps[a, b] += sgn * h
                E.append(oracle.structure(s.cell @ eps, s.positions @ eps, s.types,
                                          forces=False)[1])
            W[a, b] = -(E[1] - E[0]) / (2 * h)
    assert np.abs(r["virial"] - W).max() < 1e-5 * max(1.0, np.abs(W).max())


def test_neighbour_sets_bit_exact(cuda, oracle, cu256, nb_kernel):
    """aenet_nbl_* against the oracle's complete lcl_nbdist_cart lists on the
    same lattice coordinates: identical (atom, image) sets and coordinates."""
    from aenet_gb300 import _lib, workloads
    lib = _lib.lib()
    w, paths = cu256
    rng = np.random.default_rng(7)
    cases = [(w.structures[0].cell, w.structures[0].positions, w.structures[0].types)]
    k1 = fixtures.load("k1_ti2o4.npz")
    cases.append((k1["cell"], k1["positions"], np.array([1, 1, 1, 1, 1, 1], dtype=np.int32)))
    for n in (16, 40, 120):      # cells shorter than the cut-off: many images
        pos, cell = workloads.random_cell(rng, n)
        cases.append((cell, pos, np.ones(n, dtype=np.int32)))
    tric = np.array([[5.1, 0.0, 0.0], [1.7, 4.9, 0.0], [-1.2, 0.8, 6.3]])
    cases.append((tric, rng.uniform(0, 5, (30, 3)), np.ones(30, dtype=np.int32)))
    # orthorhombic, different heights per axis (pruned stencil rows)
    box = np.diag([18.3, 25.1, 31.7])
    cases.append((box, rng.uniform(0, 1, (900, 3)) @ box, np.ones(900, dtype=np.int32)))
    ann = _ann(paths, w.types)
    oracle.load(w.types, paths)
    try:
        for cell, pos, types in cases:
            latt, centres, ref = oracle.neighbors(cell, pos, types)
            # give the GPU the same lattice coordinates (cartesian = False)
            s_in = oracle.cart_to_latt(np.ascontiguousarray(cell, dtype=np.float64), pos)
            coords = np.ascontiguousarray(s_in.copy())
            L = np.ascontiguousarray(cell, dtype=np.float64)
            tt = np.ascontiguousarray(types, dtype=np.int32)
            lib.aenet_nbl_init(L.ctypes.data_as(C.c_void_p), len(pos),
                               tt.ctypes.data_as(C.c_void_p), coords.ctypes.data_as(C.c_void_p),
                               False, True)
            for i in range(len(pos)):
                cap = 4096
                nnb = C.c_int(cap)
                nbcoo = np.zeros((cap, 3))
                nbdist = np.zeros(cap)
                nbl = np.zeros(cap, dtype=np.int32)
                nbt = np.zeros(cap, dtype=np.int32)
                lib.aenet_nbl_neighbors(i + 1, C.byref(nnb), nbcoo.ctypes.data_as(C.c_void_p),
                                        nbdist.ctypes.data_as(C.c_void_p),
                                        nbl.ctypes.data_as(C.c_void_p),
                                        nbt.ctypes.data_as(C.c_void_p))
                k = nnb.value
                got = sorted(zip(nbl[:k].tolist(), map(tuple, nbcoo[:k].tolist())))
                rc, _, rl, _ = ref[i]
                exp = sorted(zip(rl.tolist(), map(tuple, rc.tolist())))
                assert len(got) == len(exp), (i, len(got), len(exp))
                assert got == exp
            np.testing.assert_allclose(coords, latt @ L, rtol=0, atol=1e-12)
            lib.aenet_nbl_final()
    finally:
        ann.release()


def test_per_atom_api_matches_oracle(cuda, oracle, cu256):
    """aenet_atomic_energy(_and_forces) with caller-supplied neighbours."""
    w, paths = cu256
    s = w.structures[0]
    oracle.load(w.types, paths)
    _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types)
    ann = _ann(paths, w.types)
    try:
        F_gpu = np.zeros((s.natoms, 3))
        F_or = np.zeros((s.natoms, 3))
        for i in (0, 17, 255):
            nbcoo, _, nbl, nbt = nb[i]
            sym = [w.types[t - 1] for t in nbt]
            e_gpu = ann.atomic_energy_and_forces(centres[i], w.types[s.types[i] - 1], i + 1,
                                                 nbcoo, sym, nbl, F_gpu)
            e_or = oracle.atomic_energy_and_forces(centres[i], int(s.types[i]), i + 1, nbcoo,
                                                   nbt, nbl, F_or)
            assert abs(e_gpu - e_or) < E_TOL_FP64
            e2 = ann.atomic_energy(centres[i], w.types[s.types[i] - 1], nbcoo, sym)
            assert abs(e2 - e_or) < E_TOL_FP64
        assert np.abs(F_gpu - F_or).max() < F_TOL_FP64
    finally:
        ann.release()


def test_aucu4000_mixed_vs_fp64(cuda, oracle, aucu):
    from aenet_gb300.core import FP64, MIXED
    w, paths = aucu
    s = w.structures[0]
    ann = _ann(paths, w.types)
    try:
        r64 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64)
        r32 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=MIXED)
    finally:
        ann.release()
    oracle.load(w.types, paths)
    oracle.set_candidates("cells")
    try:
        ec, et, F, Ea = oracle.structure(s.cell, s.positions, s.types, nthreads=8)
    finally:
        oracle.set_candidates("complete")
    n = s.natoms
    assert abs(r64["energy"] - et) / n < E_TOL_FP64
    assert np.abs(r64["forces"] - F).max() < F_TOL_FP64
    dE = abs(r32["energy"] - r64["energy"]) / n
    dF = r32["forces"] - r64["forces"]
    assert dE < E_TOL_MIXED, dE
    assert np.sqrt(np.mean(dF ** 2)) < F_RMS_MIXED
    assert np.abs(dF).max() < 10 * F_RMS_MIXED


def test_autograd_adjoint_and_finite_differences(cuda, aucu):
    """Forces from torch.autograd through the adjoint kernels equal the
    plan's forces, and match central differences (h = 1e-4 A, Richardson
    extrapolated) of the FP64 energy on 64 random atoms: tightly for the
    FP64 path, within the mixed-precision force tolerance for FP32."""
    torch = cuda
    from aenet_gb300.core import FP64, MIXED
    from aenet_gb300.plan import Plan, potential_energy
    w, paths = aucu
    s = w.structures[0]
    ann = _ann(paths, w.types)
    try:
        types = torch.tensor(s.types, device="cuda", dtype=torch.int32)
        grads = {}
        for prec, atol in ((FP64, 1e-9), (MIXED, 1e-3)):
            plan = Plan([s.natoms], [s.cell], precision=prec)
            pos = torch.tensor(s.positions, device="cuda", requires_grad=True)
            E = potential_energy(pos, plan, types)
            E.sum().backward()
            grads[prec] = pos.grad.clone()
            out = plan.run(pos.detach(), types, forces=True)
            # same kernels; in FP32 the atomic summation order differs
            torch.testing.assert_close(grads[prec], -out["F"], rtol=0, atol=atol)
            plan.close()
        plan = Plan([s.natoms], [s.cell], precision=FP64)
        p0 = torch.tensor(s.positions, device="cuda")
        rng = np.random.default_rng(11)
        h = 1e-4

        def central(a, c, hh):
            pp = p0.clone(); pp[a, c] += hh
            pm = p0.clone(); pm[a, c] -= hh
            return (plan.forward(pp, types)[0].item()
                    - plan.forward(pm, types)[0].item()) / (2 * hh)

        for a in rng.choice(s.natoms, 64, replace=False):
            c = int(rng.integers(3))
            fd = (4 * central(a, c, h / 2) - central(a, c, h)) / 3
            assert abs(fd - grads[FP64][a, c].item()) < 1e-6, (a, c, fd)
            assert abs(fd - grads[MIXED][a, c].item()) < F_RMS_MIXED, (a, c, fd)
        plan.close()
    finally:
        ann.release()


def test_batch_of_small_cells_matches_oracle(cuda, oracle, tmp_path, nb_kernel):
    """Several small periodic cells (cut-off longer than the cell: many
    images) in one batched call, FP64 against the oracle per structure."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64
    w = workloads.lisio_batch_4096(nstruc=6)
    oracle.set_candidates("cells")
    paths = helpers.make_potentials(oracle, w, str(tmp_path))
    oracle.set_candidates("complete")
    ann = _ann(paths, w.types)
    try:
        structs = [(s.positions, s.types, s.cell, True) for s in w.structures]
        r = ann.batch_energy_forces(structs, precision=FP64)
    finally:
        ann.release()
    oracle.load(w.types, paths)
    off = 0
    for k, s in enumerate(w.structures):
        ec, et, F, _ = oracle.structure(s.cell, s.positions, s.types)
        assert abs(r["energy"][k] - et) / s.natoms < E_TOL_FP64
        assert np.abs(r["forces"][off:off + s.natoms] - F).max() < F_TOL_FP64
        off += s.natoms


def test_sfb_api_matches_oracle(cuda, oracle):
    from aenet_gb300 import _lib
    lib = _lib.lib()
    names = (C.c_char_p * 2)(b"Au", b"Cu")
    st = C.c_int(-1)
    lib.aenet_sfb_init(2, names, 12, 6, 6.5, 4.5, C.byref(st))
    assert st.value == 0
    try:
        nv = lib.aenet_sfb_nvalues()
        assert nv == 40
        rng = np.random.default_rng(3)
        coo1 = rng.uniform(-4, 4, (30, 3))
        it = rng.integers(1, 3, 30).astype(np.int32)
        coo0 = np.zeros(3)
        vals = np.zeros(nv)
        lib.aenet_sfb_eval(1, coo0.ctypes.data_as(C.c_void_p), 30, it.ctypes.data_as(C.c_void_p),
                           coo1.ctypes.data_as(C.c_void_p), nv, vals.ctypes.data_as(C.c_void_p),
                           C.byref(st))
        assert st.value == 0
        olib = oracle.lib
        olib.orc_sfb_init(2, 12, 6, 6.5, 4.5)
        ref = np.zeros(nv)
        olib.orc_sfb_eval(1, coo0, 30, it, np.ascontiguousarray(coo1), nv, ref, None, None)
        olib.orc_sfb_final()
        np.testing.assert_allclose(vals, ref, rtol=0, atol=1e-11)
    finally:
        lib.aenet_sfb_final(C.byref(st))


def test_capacity_overflow_is_reported_and_retried(cuda, cu256):
    torch = cuda
    from aenet_gb300.core import FP64
    from aenet_gb300.plan import Plan, PlanStatusError
    w, paths = cu256
    s = w.structures[0]
    ann = _ann(paths, w.types)
    try:
        plan = Plan([s.natoms], [s.cell], precision=FP64)
        pos = torch.tensor(s.positions, device="cuda")
        types = torch.tensor(s.types, device="cuda", dtype=torch.int32)
        plan.run(pos, types)
        plan.check()
        # squeeze the structure to 60% volume: more neighbours than the
        # capacity sized for the original density
        dense = torch.tensor(s.positions * 0.6, device="cuda")
        plan.set_cells([s.cell * 0.6])
        plan.run(dense, types)
        with pytest.raises(PlanStatusError):
            plan.check()
        plan.close()
        # the host-buffer entry point resizes and retries on its own
        r = ann.structure_energy_forces(s.positions * 0.6, s.types, s.cell * 0.6, precision=FP64)
        assert np.isfinite(r["energy"])
    finally:
        ann.release()


def _neighbour_keys(torch, plan, pos, cells, nat):
    """Per-row sorted keys (neighbour index, lattice image) of a plan's
    table.  The image n of a pair follows from its vector: R_ij = r_j - r_i
    + n L with the unwrapped input positions, so n = round((R_ij - r_j +
    r_i) L^-1) -- exact for FP32 vectors too (their error is ~1e-6 A against
    lattice vectors of several A)."""
    cap, cnt, jt, vec = plan.neighbors()
    n = plan.natoms
    dev = vec.device
    sid = torch.repeat_interleave(torch.arange(len(nat), device=dev),
                                  torch.as_tensor(nat, device=dev).long())
    Linv = torch.linalg.inv(torch.as_tensor(cells, device=dev, dtype=torch.float64))[sid]
    j = (jt & ((1 << 26) - 1)).long()
    valid = torch.arange(cap, device=dev)[None, :] < cnt[:, None].long()
    j = torch.where(valid, j, torch.zeros_like(j))
    d = vec[..., :3].double() - (pos[j] - pos[:, None, :])
    img = torch.einsum("ncx,nxy->ncy", d, Linv)
    imgr = torch.round(img)
    assert (img - imgr)[valid].abs().max().item() < 1e-3
    code = (imgr.long() + 8)
    assert ((code >= 0) & (code < 16))[valid].all()
    key = j * 4096 + code[..., 0] * 256 + code[..., 1] * 16 + code[..., 2]
    key = torch.where(valid, key, torch.full_like(key, 1 << 62))
    return cnt.clone(), torch.sort(key, dim=1).values, vec.clone(), jt.clone()


def test_fp32_and_fp64_plans_find_the_same_neighbours(cuda, oracle, tmp_path, nb_kernel):
    """Both precisions decide the cut-off with the same FP64 predicate:
    every row of the FP32 (mixed) plan's table holds the same set of
    (neighbour, lattice image) pairs as the FP64 plan's, and the pair
    vectors agree to FP32 rounding."""
    torch = cuda
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED
    from aenet_gb300.plan import Plan
    w = workloads.lisio_batch_4096(nstruc=64)
    paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=500)
    ann = _ann(paths, w.types)
    try:
        nat, pos, typ, cells, pbc = w.packed()
        p = torch.tensor(pos, device="cuda")
        t = torch.tensor(typ, device="cuda")
        got = []
        for prec in (FP64, MIXED):
            plan = Plan(nat, cells, pbc, precision=prec)
            plan.run(p, t)
            plan.check()
            got.append(_neighbour_keys(torch, plan, p, cells, nat))
            plan.close()
        (c64, k64, v64, _), (c32, k32, v32, _) = got
        assert torch.equal(c64, c32)
        assert torch.equal(k64, k32)
        assert int(c64.sum().item()) > 60 * len(pos)
        # same pair vectors (matched through the sorted keys)
        cap = k64.shape[1]
        for v, c in ((v64, c64), (v32, c32)):
            assert v.shape[1] == cap
        d64 = torch.sort(v64[..., 3].double().masked_fill(
            torch.arange(cap, device="cuda")[None] >= c64[:, None], 1e9), dim=1).values
        d32 = torch.sort(v32[..., 3].double().masked_fill(
            torch.arange(cap, device="cuda")[None] >= c32[:, None], 1e9), dim=1).values
        assert (d64 - d32).abs().max().item() < 1e-5
    finally:
        ann.release()


@pytest.mark.parametrize("acts", [((2, 3, 0), (3, 4, 0), (4, 2, 0)),
                                  ((2, 2, 2), (3, 3, 3), (4, 4, 4))])
def test_activation_codes_2_to_4(cuda, oracle, tmp_path, acts):
    """ff_activate's sigmoid (2), scaled tanh 1.7159 tanh(2x/3) (3) and the
    same plus 0.1x (4) (feedforward.f90:932-969) in hidden and output
    layers: FP64 against the oracle to 1e-10 eV/atom, the mixed path on the
    tensor-core kernel (its generic-activation instantiation) and on the
    SIMT kernel within the mixed tolerance of FP64."""
    from aenet_gb300 import nnfile, workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    w = workloads.lisio_batch_4096(nstruc=12)
    rng = np.random.default_rng(21)
    base = workloads.glorot_networks(rng, w.types, w.arch)
    # activation codes of (hidden 1, hidden 2, output), one layout per species
    for t, a in zip(w.types, acts):
        base[t] = nnfile.make_network(w.arch, base[t]["W"], activations=list(a))
    w.networks = base
    paths = helpers.make_potentials(oracle, w, str(tmp_path))
    ann = _ann(paths, w.types)
    try:
        structs = [(s.positions, s.types, s.cell, True) for s in w.structures]
        r64 = ann.batch_energy_forces(structs, precision=FP64)
        out = {}
        for mode in ("simt", "tensor"):
            set_option("networks", mode)
            out[mode] = ann.batch_energy_forces(structs, precision=MIXED)
    finally:
        set_option("networks", "tensor")
        ann.release()
    oracle.load(w.types, paths)
    off = 0
    for k, s in enumerate(w.structures):
        _, et, F, _ = oracle.structure(s.cell, s.positions, s.types)
        assert abs(r64["energy"][k] - et) / s.natoms < E_TOL_FP64, k
        assert np.abs(r64["forces"][off:off + s.natoms] - F).max() < F_TOL_FP64, k
        off += s.natoms
    nat = np.array([s.natoms for s in w.structures])
    for mode in ("simt", "tensor"):
        dE = np.abs(out[mode]["energy"] - r64["energy"]) / nat
        dF = out[mode]["forces"] - r64["forces"]
        assert dE.max() < E_TOL_MIXED, (mode, dE.max())
        assert np.sqrt((dF ** 2).mean()) < F_RMS_MIXED, mode


def test_k3_cu_dimer_scan_on_gpu(cuda, tmp_path):
    """unittests/Cu-dimer-forces on the GPU: 81 isolated dimers, Behler G2/G4
    with 16-record (legacy) setups; energies and forces at the printed
    precision of the reference's output files."""
    from aenet_gb300.core import FP64
    k3 = fixtures.load("k3_cu_dimer.npz")
    pots = fixtures.potentials(k3)
    paths = fixtures.write_potential_files(pots, str(tmp_path))
    types = [str(t) for t in k3["types"]]
    ann = _ann(paths, types)
    cu = types.index("Cu") + 1
    try:
        for x, F, ec, et in zip(k3["positions"], k3["forces"], k3["E_coh"], k3["E_total"]):
            r = ann.structure_energy_forces(x, np.array([cu, cu], dtype=np.int32), None,
                                            pbc=False, precision=FP64)
            assert abs(r["cohesive_energy"] - ec) <= 5.1e-9
            assert abs(r["energy"] - et) <= 5.1e-9
            assert np.abs(r["forces"] - F).max() <= 5.1e-7
    finally:
        ann.release()


@pytest.fixture(scope="module")
def rutile(oracle, tmp_path_factory):
    from aenet_gb300 import workloads
    w = workloads.tio2_rutile_9000(cells=(2, 2, 3))
    d = tmp_path_factory.mktemp("rutile")
    paths = helpers.make_potentials(oracle, w, str(d))
    return w, paths


def test_rutile_behler_fp64_parity_virial_and_mixed(cuda, oracle, rutile):
    from aenet_gb300.core import FP64, MIXED
    w, paths = rutile
    s = w.structures[0]
    ann = _ann(paths, w.types)
    try:
        r64 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64,
                                          virial=True)
        r32 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=MIXED,
                                          virial=True)
    finally:
        ann.release()
    oracle.load(w.types, paths)
    ec, et, F, Ea = oracle.structure(s.cell, s.positions, s.types)
    n = s.natoms
    assert abs(r64["energy"] - et) / n < E_TOL_FP64
    assert np.abs(r64["atomic_energies"] - Ea).max() < E_TOL_FP64
    assert np.abs(r64["forces"] - F).max() < F_TOL_FP64
    # virial against central differences of the oracle energy under strain
    h = 1e-5
    W = np.zeros((3, 3))
    for a in range(3):
        for b in range(3):
            E = []
            for sgn in (-1, 1):
                eps = np.eye(3)
                eps[a, b] += sgn * h
                E.append(oracle.structure(s.cell @ eps, s.positions @ eps, s.types,
                                          forces=False)[1])
            W[a, b] = -(E[1] - E[0]) / (2 * h)
    assert np.abs(r64["virial"] - W).max() < 1e-5 * max(1.0, np.abs(W).max())
    # mixed precision against FP64
    assert abs(r32["energy"] - r64["energy"]) / n < E_TOL_MIXED
    dF = r32["forces"] - r64["forces"]
    assert np.sqrt(np.mean(dF ** 2)) < F_RMS_MIXED


@pytest.mark.parametrize("which", ["lisio", "aucu"])
def test_tensor_core_networks_match_simt_and_fp64(cuda, oracle, aucu, tmp_path, which):
    """tcgen05 networks (split BF16, FP32 accumulation in TMEM) against the
    SIMT FP32 kernel and the FP64 path: 32-32-32-1 x3 (kin 32) and
    40-25-25-1 x2 (kin 64, hidden padded to 32)."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    if which == "lisio":
        w = workloads.lisio_batch_4096(nstruc=24)
        paths = helpers.make_potentials(oracle, w, str(tmp_path))
    else:
        w, paths = aucu
    ann = _ann(paths, w.types)
    try:
        structs = [(s.positions, s.types, s.cell, True) for s in w.structures]
        r64 = ann.batch_energy_forces(structs, precision=FP64)
        out = {}
        for mode in ("simt", "tensor"):
            set_option("networks", mode)
            out[mode] = ann.batch_energy_forces(structs, precision=MIXED)
    finally:
        set_option("networks", "tensor")
        ann.release()
    nat = np.array([s.natoms for s in w.structures])
    for mode in ("simt", "tensor"):
        dE = np.abs(out[mode]["energy"] - r64["energy"]) / nat
        dF = out[mode]["forces"] - r64["forces"]
        assert dE.max() < E_TOL_MIXED, (mode, dE.max())
        assert np.sqrt((dF ** 2).mean()) < F_RMS_MIXED, mode
    # split BF16 keeps ~16 bits: far inside the mixed tolerance
    dE = np.abs(out["tensor"]["energy"] - out["simt"]["energy"]) / nat
    assert dE.max() < 1e-4
    dF = out["tensor"]["forces"] - out["simt"]["forces"]
    assert np.sqrt((dF ** 2).mean()) < 1e-3


def test_k5_rotation_invariance_and_fcc_shell_on_gpu(cuda, cu256):
    """K-5 on the GPU: energies invariant under a rotation of structure and
    cell (FP64 1e-10 eV/atom, mixed 1e-5 eV/atom), forces rotate with it,
    and every atom of a perfect FCC crystal has 12 neighbours in its first
    shell."""
    torch = cuda
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED
    from aenet_gb300.plan import Plan
    w, paths = cu256
    s = w.structures[0]
    rng = np.random.default_rng(11)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    ann = _ann(paths, w.types)
    try:
        for prec, tol in ((FP64, 1e-10), (MIXED, 1e-5)):
            r0 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=prec)
            r1 = ann.structure_energy_forces(s.positions @ q, s.types, s.cell @ q, precision=prec)
            assert abs(r1["energy"] - r0["energy"]) / s.natoms < tol
            ftol = 1e-9 if prec == FP64 else 1e-3
            assert np.abs(r1["forces"] - r0["forces"] @ q).max() < ftol
        pos, cell = workloads.fcc_positions(4, 3.61)
        plan = Plan([len(pos)], cell[None], precision=FP64)
        p = torch.tensor(pos, device="cuda")
        t = torch.ones(len(pos), dtype=torch.int32, device="cuda")
        plan.run(p, t)
        plan.check()
        _, cnt, _, vec = plan.neighbors()
        d = vec[..., 3].cpu().numpy()
        c = cnt.cpu().numpy()
        first = [(d[i, :c[i]] < 3.61 / np.sqrt(2) + 0.05).sum() for i in range(len(pos))]
        assert set(first) == {12}
        plan.close()
    finally:
        ann.release()


@pytest.mark.parametrize("case", ["lisio", "lisio_legacy", "lisio_a7", "cu256"])
def test_angular_moment_form_matches_pairs(cuda, oracle, cu256, tmp_path, case):
    """FP32 angular terms in moment form (power spectra of the neighbours'
    harmonics, linear in the neighbour count) against the FP32 pair sums
    and the FP64 path: energies, forces and virials for angular orders 4
    and 6, the current and the legacy angular domain, one and three
    species."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    angular = "legacy" if case == "lisio_legacy" else "current"
    if case == "cu256":
        w, paths = cu256
    else:
        w = workloads.lisio_batch_4096(nstruc=24)
        if case == "lisio_a7":
            w.setups = workloads.cheb_setups(w.types, 12, 6.0, 6, 4.0)
            w.networks = workloads.glorot_networks(np.random.default_rng(7), w.types,
                                                   [40, 32, 32, 1])
        paths = helpers.make_potentials(oracle, w, str(tmp_path))
    ann = _ann(paths, w.types, angular)
    try:
        structs = [(s.positions, s.types, s.cell, True) for s in w.structures]
        r64 = ann.batch_energy_forces(structs, precision=FP64, virial=True)
        out = {}
        for mode in ("pairs", "moments"):
            set_option("angular_terms", mode)
            out[mode] = ann.batch_energy_forces(structs, precision=MIXED, virial=True)
    finally:
        set_option("angular_terms", "moments")
        ann.release()
    nat = np.array([s.natoms for s in w.structures])
    for mode in ("pairs", "moments"):
        dE = np.abs(out[mode]["energy"] - r64["energy"]) / nat
        dF = out[mode]["forces"] - r64["forces"]
        assert dE.max() < E_TOL_MIXED, (mode, dE.max())
        assert np.sqrt((dF ** 2).mean()) < F_RMS_MIXED, mode
    # both FP32 forms round differently but evaluate the same sums
    scale_F = np.sqrt((r64["forces"] ** 2).mean())
    dE = np.abs(out["moments"]["energy"] - out["pairs"]["energy"]) / nat
    assert dE.max() < 2e-5, dE.max()
    dF = out["moments"]["forces"] - out["pairs"]["forces"]
    assert np.sqrt((dF ** 2).mean()) < 1e-4 * max(1.0, scale_F)
    dV = out["moments"]["virial"] - r64["virial"]
    assert np.abs(dV).max() < 1e-3 * max(1.0, np.abs(r64["virial"]).max())


def test_moment_form_on_isolated_and_sparse_structures(cuda, oracle, tmp_path):
    """Moment form where the pair sum is small or empty: isolated molecules
    (no periodic images) and a sparse gas in which atoms have zero or one
    angular neighbour; energies and forces against FP64 and the pair form."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    w = workloads.lisio_batch_4096(nstruc=6)
    paths = helpers.make_potentials(oracle, w, str(tmp_path))
    rng = np.random.default_rng(11)
    structs = []
    for n in (3, 8, 20):          # molecules: compact clusters, no lattice
        pos = rng.normal(scale=1.4, size=(n, 3))
        structs.append((pos, rng.integers(1, 4, n).astype(np.int32), None, False))
    for n in (12, 30):            # gas: most atoms far apart
        pos, cell = workloads.random_cell(rng, n, density=0.004, dmin=2.5)
        structs.append((pos, rng.integers(1, 4, n).astype(np.int32), cell, True))
    ann = _ann(paths, w.types)
    try:
        r64 = ann.batch_energy_forces(structs, precision=FP64)
        out = {}
        for mode in ("pairs", "moments"):
            set_option("angular_terms", mode)
            out[mode] = ann.batch_energy_forces(structs, precision=MIXED)
    finally:
        set_option("angular_terms", "moments")
        ann.release()
    nat = np.array([len(s[1]) for s in structs])
    for mode in ("pairs", "moments"):
        assert np.all(np.isfinite(out[mode]["energy"])) and np.all(np.isfinite(out[mode]["forces"]))
        dE = np.abs(out[mode]["energy"] - r64["energy"]) / nat
        assert dE.max() < 1e-4, (mode, dE.max())
        assert np.abs(out[mode]["forces"] - r64["forces"]).max() < 1e-3, mode
    dE = np.abs(out["moments"]["energy"] - out["pairs"]["energy"]) / nat
    assert dE.max() < 2e-5


def test_behler_descriptor_jacobians_match_oracle(cuda, oracle, rutile):
    """PyTorch-export Jacobians for Behler bases (G1-G5): every neighbour
    slot's and the central atom's FP64 derivatives against the oracle's
    symmfunc restatement (stp_eval with derivatives), matched by pair
    vector."""
    import torch
    from aenet_gb300.core import FP64
    from aenet_gb300.plan import Plan
    w, paths = rutile
    s = w.structures[0]
    oracle.load(w.types, paths)
    ann = _ann(paths, w.types)
    try:
        plan = Plan([s.natoms], s.cell[None], np.array([1], dtype=np.int32), precision=FP64)
        plan.run(torch.tensor(s.positions, device="cuda"),
                 torch.tensor(s.types.astype(np.int32), device="cuda"), forces=False)
        plan.check()
        Ji, Jj, nbl, nnb = (x.cpu().numpy() for x in plan.jacobian())
        vec = plan.neighbors()[3].cpu().numpy()
        plan.close()
    finally:
        ann.release()
    _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types)
    for a in range(0, s.natoms, 7):
        nbcoo, _, nblist, nbt = nb[a]
        G, di, dj = oracle.descriptor(centres[a], int(s.types[a]), nbcoo, nbt, scaled=False,
                                      deriv=True)
        nsf = G.size
        m = int(nnb[a])
        assert m == len(nblist)
        scale = max(1.0, np.abs(dj).max())
        np.testing.assert_allclose(Ji[a, :nsf], di, rtol=0, atol=1e-9 * scale)
        R_ref = nbcoo - centres[a]
        for q in range(m):
            k = int(np.argmin(np.abs(R_ref - vec[a, q, :3]).sum(1)))
            assert np.abs(R_ref[k] - vec[a, q, :3]).max() < 1e-9
            assert nbl[a, q] + 1 == nblist[k]
            np.testing.assert_allclose(Jj[a, q, :nsf], dj[k], rtol=0, atol=1e-9 * scale)


def test_host_batch_runs_in_chunks_like_one_plan(cuda, oracle, tmp_path):
    """Large host-buffer batches run as chunks of whole structures on
    separate streams: 16 cells repeated to ~300k atoms give, copy for copy,
    the energies, forces and virials of the 16 cells evaluated alone (FP64:
    identical to rounding of the force sums; mixed: same kernels, FP32
    noise only)."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED
    w = workloads.lisio_batch_4096(nstruc=16)
    paths = helpers.make_potentials(oracle, w, str(tmp_path))
    base = [(s.positions, s.types, s.cell, True) for s in w.structures]
    nat = np.array([len(s[1]) for s in base])
    reps = int(np.ceil(300000 / nat.sum()))
    big = base * reps
    ann = _ann(paths, w.types)
    try:
        for prec, tol in ((FP64, 1e-11), (MIXED, 1e-5)):
            one = ann.batch_energy_forces(base, precision=prec, virial=True)
            many = ann.batch_energy_forces(big, precision=prec, virial=True)
            E = many["energy"].reshape(reps, len(base))
            assert np.abs(E - one["energy"][None]).max() / nat.min() < tol
            F = many["forces"].reshape(reps, nat.sum(), 3)
            assert np.abs(F - one["forces"][None]).max() < 100 * tol
            V = many["virial"].reshape(reps, len(base), 3, 3)
            assert np.abs(V - one["virial"][None]).max() < 1e3 * tol * max(1, np.abs(one["virial"]).max())
    finally:
        ann.release()


def test_stale_spin_option_matches_oracle(cuda, oracle, tmp_path):
    """sfb_eval refreshes s_j only inside the radial branch (sfbasis.f90:514)
    and reuses it for the angular pairs (:556): with a_Rc > r_Rc a neighbour
    beyond r_Rc weighs its pairs with the spin of the last earlier neighbour
    inside r_Rc.  Option angular_spin = stale reproduces that: the
    structure path in the reference's lcl_nbdist_cart order (the oracle's
    complete candidate order) and the per-atom libaenet calls in the
    caller's order (also shuffled).  FP64 to 1e-10 eV/atom and 1e-9 eV/A;
    with each neighbour's own spin the same potential differs from the
    oracle; the mixed path stays within its tolerance."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    rng = np.random.default_rng(41)
    w = workloads.aucu_fcc_4000()
    s0 = w.structures[0]
    sites, _ = workloads.fcc_positions(10, 3.90)
    keep = np.all(sites < 3 * 3.90 - 0.1, axis=1)
    s = workloads.Structure(s0.positions[keep], s0.types[keep], np.eye(3) * (3 * 3.90))
    arch = [28, 16, 16, 1]
    w = workloads.Workload("aucu_stale", w.types, workloads.cheb_setups(w.types, 8, 4.0, 4, 5.2),
                           arch, [s], 2)
    w.networks = workloads.glorot_networks(rng, w.types, arch)
    paths = helpers.make_potentials(oracle, w, str(tmp_path))
    oracle.load(w.types, paths)
    ec, et, F_or, Ea_or = oracle.structure(s.cell, s.positions, s.types)
    _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types)
    ann = _ann(paths, w.types)
    n = s.natoms
    try:
        set_option("angular_spin", "stale")
        r64 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64)
        r32 = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=MIXED)
        assert abs(r64["energy"] - et) / n < E_TOL_FP64
        assert np.abs(r64["atomic_energies"] - Ea_or).max() < E_TOL_FP64
        assert np.abs(r64["forces"] - F_or).max() < F_TOL_FP64
        assert abs(r32["energy"] - r64["energy"]) / n < E_TOL_MIXED
        assert np.sqrt(np.mean((r32["forces"] - r64["forces"]) ** 2)) < F_RMS_MIXED
        # per-atom calls: the caller's order decides, as in libaenet
        for i in (0, 37, 101):
            nbcoo, _, nbl, nbt = nb[i]
            for perm in (np.arange(len(nbl)), rng.permutation(len(nbl))):
                sym = [w.types[t - 1] for t in nbt[perm]]
                Fg = np.zeros((n, 3))
                Fo = np.zeros((n, 3))
                eg = ann.atomic_energy_and_forces(centres[i], w.types[s.types[i] - 1], i + 1,
                                                  nbcoo[perm], sym, nbl[perm], Fg)
                eo = oracle.atomic_energy_and_forces(centres[i], int(s.types[i]), i + 1,
                                                     nbcoo[perm], nbt[perm], nbl[perm], Fo)
                assert abs(eg - eo) < E_TOL_FP64, (i, eg, eo)
                assert np.abs(Fg - Fo).max() < F_TOL_FP64
        set_option("angular_spin", "own")
        own = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=FP64)
    finally:
        set_option("angular_spin", "own")
        ann.release()
    # the option matters for this basis: own spins miss the reference
    assert np.abs(own["atomic_energies"] - Ea_or).max() > 1e-6


@pytest.mark.parametrize("angular", ["current", "legacy"])
def test_fused_per_atom_kernel_matches_oracle_and_graph_path(cuda, oracle, aucu, angular,
                                                              tmp_path):
    """The fused per-atom launch (FP64; a cluster of eight blocks, and one
    block) against the oracle and against the graph of the batch kernels
    (per_atom_kernel = cluster, block, graph): two species with the spin block, both angular domains, rows of
    the alloy cell (about 80 neighbours, 24 angular), rows of a dense
    random cell (over 300 neighbours, about 110 angular: several staging
    chunks and pair rounds), a row beyond the fused kernel's 512
    neighbours (taken by the graph path), one neighbour and none;
    energy-only calls give the same energy; repeated calls the same bits."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import set_option
    w, paths = aucu
    s0 = w.structures[0]
    sites, _ = workloads.fcc_positions(10, 3.90)
    keep = np.all(sites < 3 * 3.90 - 0.1, axis=1)
    s = workloads.Structure(s0.positions[keep], s0.types[keep], np.eye(3) * (3 * 3.90))
    # a dense random cell (0.3 atoms/A^3, ~340 neighbours and ~110 angular
    # ones per atom) with a potential normalised on it, so that its rows
    # reach real forces
    rng = np.random.default_rng(7)
    box = 12.0
    pts = np.zeros((0, 3))
    while len(pts) < int(0.3 * box ** 3):
        p = rng.random(3) * box
        if len(pts) == 0 or np.linalg.norm((p - pts + box / 2) % box - box / 2, axis=1).min() > 0.9:
            pts = np.vstack([pts, p])
    dense = workloads.Structure(pts, 1 + rng.integers(0, 2, len(pts)), np.eye(3) * box)
    wd = workloads.Workload("dense", w.types, w.setups, w.arch, [dense], 11)
    wd.networks = workloads.glorot_networks(rng, w.types, w.arch)
    dpaths = helpers.make_potentials(oracle, wd, str(tmp_path))
    rows = []
    for ws, ps, st, picks in ((w, paths, s, (0, 51)), (wd, dpaths, dense, (3, 200))):
        oracle.load(w.types, ps, angular=angular)
        _, centres, nb = oracle.neighbors(st.cell, st.positions, st.types)
        for i in picks:
            nbcoo, _, nbl, nbt = nb[i]
            rows.append((ps, centres[i], int(st.types[i]), nbcoo, nbt))
    for m in (600, 1, 0):
        c = np.array([0.3, -0.2, 0.1])
        d = rng.normal(size=(m, 3))
        d *= (6.6 * rng.random(m) ** (1 / 3) / np.linalg.norm(d, axis=1))[:, None]
        rows.append((dpaths, c, 1 + (m % 2), c + d, 1 + rng.integers(0, 2, m)))
    assert max(len(r[4]) for r in rows[2:4]) > 300
    ann = None
    try:
        for ps, coo_i, ti, coo_j, tj in rows:
            if ann is None or ann.potential_files != {t: ps[t] for t in w.types}:
                if ann is not None:
                    ann.release()
                ann = _ann(ps, w.types, angular)
                oracle.load(w.types, ps, angular=angular)
            m = len(tj)
            n = m + 1
            idx = np.arange(2, m + 2, dtype=np.int32)
            sym = [w.types[t - 1] for t in tj]
            Fo = np.zeros((n, 3))
            eo = oracle.atomic_energy_and_forces(coo_i, ti, 1, coo_j, tj, idx, Fo)
            res = {}
            for path in ("cluster", "block", "graph"):
                set_option("per_atom_kernel", path)
                F = np.zeros((n, 3))
                e = ann.atomic_energy_and_forces(coo_i, w.types[ti - 1], 1, coo_j, sym, idx, F)
                e2 = ann.atomic_energy(coo_i, w.types[ti - 1], coo_j, sym)
                F3 = np.zeros((n, 3))
                e3 = ann.atomic_energy_and_forces(coo_i, w.types[ti - 1], 1, coo_j, sym, idx, F3)
                assert abs(e - eo) < E_TOL_FP64, (path, m, e, eo)
                assert np.abs(F - Fo).max() < F_TOL_FP64, (path, m)
                assert abs(e2 - e) < E_TOL_FP64
                assert e3 == e and np.array_equal(F3, F)
                res[path] = (e, F)
            for path in ("cluster", "block"):
                assert abs(res[path][0] - res["graph"][0]) < E_TOL_FP64
                assert np.abs(res[path][1] - res["graph"][1]).max() < F_TOL_FP64
            if m >= 300 and angular == "current":
                # the dense rows exercise real forces (the dense potential is
                # normalised on current-domain descriptors)
                assert np.abs(Fo).max() > 1e-2
    finally:
        set_option("per_atom_kernel", "fused")
        if ann is not None:
            ann.release()


def test_per_atom_calls_reuse_their_buffers(cuda, oracle, cu256):
    """Repeated aenet_atomic_energy_and_forces calls (the predict.x calling
    pattern) give identical results call after call and across neighbour
    counts that grow and shrink (the staging buffers are grown once and
    reused)."""
    w, paths = cu256
    s = w.structures[0]
    oracle.load(w.types, paths)
    _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types)
    ann = _ann(paths, w.types)
    try:
        first = {}
        for rep in range(3):
            for i in (5, 0, 200):
                nbcoo, _, nbl, nbt = nb[i]
                m = len(nbl) if rep != 1 else len(nbl) // 2
                F = np.zeros((s.natoms, 3))
                e = ann.atomic_energy_and_forces(centres[i], "Cu", i + 1, nbcoo[:m],
                                                 ["Cu"] * m, nbl[:m], F)
                key = (i, m)
                if key in first:
                    assert e == first[key][0]
                    assert np.array_equal(F, first[key][1])
                else:
                    first[key] = (e, F)
    finally:
        ann.release()


def test_per_structure_search_matches_per_atom_search(cuda, oracle, tmp_path):
    """The block-per-structure searches, full and half stencil (taken for
    batches of more than twice as many structures as SMs), against the
    warp-per-atom search on 320 small cells: identical (neighbour, image)
    sets per row, in both precisions, on the plain and the refined grid;
    FP64 energies equal to rounding and against the oracle on a sample of
    cells; invalid type ids are reported by the searches (which convert
    the caller's ids themselves)."""
    torch = cuda
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    from aenet_gb300.plan import Plan
    w = workloads.lisio_batch_4096(nstruc=320)
    paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=500)
    ann = _ann(paths, w.types)
    try:
        nat, pos, typ, cells, pbc = w.packed()
        p = torch.tensor(pos, device="cuda")
        t = torch.tensor(typ, device="cuda")
        for z in (1, 4):
            set_option("z_refine", z)
            for prec in (FP64, MIXED):
                got = {}
                for kern in ("atom", "struct", "struct_half"):
                    set_option("neighbour_kernel", kern)
                    plan = Plan(nat, cells, pbc, precision=prec)
                    o = plan.run(p, t)
                    plan.check()
                    got[kern] = _neighbour_keys(torch, plan, p, cells, nat) + (o["E"].clone(),)
                    plan.close()
                a = got["atom"]
                tol = 1e-11 if prec == FP64 else 1e-5
                for kern in ("struct", "struct_half"):
                    s = got[kern]
                    assert torch.equal(a[0], s[0]), kern
                    assert torch.equal(a[1], s[1]), kern
                    assert ((a[4] - s[4]).abs() / torch.as_tensor(nat, device="cuda")).max() < tol
                s = got["struct"]
                if prec == FP64 and z == 4:
                    E = s[4].cpu().numpy()
        # the per-structure searches check the caller's type ids themselves
        from aenet_gb300.plan import ST_BAD_TYPE
        for kern in ("struct", "struct_half"):
            set_option("neighbour_kernel", kern)
            plan = Plan(nat, cells, pbc, precision=MIXED)
            t_bad = t.clone()
            t_bad[3] = 0
            t_bad[11] = 99
            plan.run(p, t_bad)
            assert plan.status() & ST_BAD_TYPE, kern
            plan.close()
        oracle.load(w.types, paths)
        for k in (0, 7, 160, 319):
            st = w.structures[k]
            _, et, _, _ = oracle.structure(st.cell, st.positions, st.types)
            assert abs(E[k] - et) / st.natoms < E_TOL_FP64, k
    finally:
        set_option("neighbour_kernel", "atom")
        set_option("z_refine", 1)
        ann.release()
