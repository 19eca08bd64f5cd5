"""Loss and weight gradients on the GPU (training), against the oracle.

Energy loss (the reference's, src/train.f90:799-889 + optimize.f90:698-734):
the FP64 GPU gradient equals sum_s dE_s Dw_s assembled from the oracle's
per-atom ff_wderiv restatement, to 1e-10 relative.
Energy + force loss (no reference counterpart): FP64 gradient against
central differences of the FP64 GPU loss (Richardson, relative 1e-6);
mixed-precision gradient against FP64 (relative 2e-3 of the norm).
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu

G_REL_FP64 = 1e-10
G_REL_FD = 1e-6
G_REL_MIXED = 2e-3


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


@pytest.fixture(scope="module")
def batch(oracle, tmp_path_factory):
    """Eight small Li/Si/O cells (many periodic images) with targets from a
    teacher network of the same architecture and another seed."""
    from aenet_gb300 import workloads
    w = workloads.lisio_batch_4096(nstruc=8)
    d = tmp_path_factory.mktemp("train")
    paths = helpers.make_potentials(oracle, w, str(d))
    rng = np.random.default_rng(104)
    teacher = workloads.glorot_networks(rng, w.types, w.arch)
    tpaths = workloads.write_potentials(w, str(d / "teacher"), stats=_stats_of(paths, w),
                                        networks=teacher)
    return w, paths, tpaths


@pytest.fixture(scope="module")
def batch_odd(oracle, tmp_path_factory):
    """The same eight cells under a 40-feature descriptor (radial order 12,
    angular order 6) and 40-25-25-1 networks: odd layer widths, and more
    inputs than the weight-gradient kernel stages ahead in registers."""
    from aenet_gb300 import workloads
    base = workloads.lisio_batch_4096(nstruc=8)
    arch = [40, 25, 25, 1]
    w = workloads.Workload("lisio_odd", base.types,
                           workloads.cheb_setups(base.types, 12, 6.0, 6, 4.0), arch,
                           base.structures, base.seed)
    w.networks = workloads.glorot_networks(np.random.default_rng(5), w.types, arch)
    d = tmp_path_factory.mktemp("train_odd")
    paths = helpers.make_potentials(oracle, w, str(d))
    teacher = workloads.glorot_networks(np.random.default_rng(105), w.types, arch)
    tpaths = workloads.write_potentials(w, str(d / "teacher"), stats=_stats_of(paths, w),
                                        networks=teacher)
    return w, paths, tpaths


def _stats_of(paths, w):
    from aenet_gb300.nnfile import read_nn
    out = {}
    for t in w.types:
        _, stp, _, _ = read_nn(paths[t])
        out[t] = (stp["sfval_min"], stp["sfval_max"], stp["sfval_avg"], stp["sfval_cov"])
    return out


def _ann(paths, types):
    from aenet_gb300.core import ANNPotentials
    return ANNPotentials({t: paths[t] for t in types}, angular_domain="current")


def _structs(w):
    return [(s.positions, s.types, s.cell, True) for s in w.structures]


def _targets(w, tpaths):
    from aenet_gb300.core import FP64
    ann = _ann(tpaths, w.types)
    try:
        r = ann.batch_energy_forces(_structs(w), precision=FP64)
    finally:
        ann.release()
    return r["energy"], r["forces"]


@pytest.mark.parametrize("which", ["batch", "batch_odd"])
def test_energy_loss_gradient_matches_oracle(cuda, oracle, request, which):
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64
    from aenet_gb300.train import LOSS_ENERGY, Trainer
    w, paths, tpaths = request.getfixturevalue(which)
    E_t, _ = _targets(w, tpaths)
    ann = _ann(paths, w.types)
    try:
        tr = Trainer(ann, _structs(w), E_t, mode=LOSS_ENERGY, precision=FP64)
        loss, g = tr.loss_and_grad()
        loss2, g2 = tr.loss_and_grad()
        nws = [ann.nweights(t) for t in w.types]
        tr.close()
    finally:
        ann.release()
    # the reduction of the weight gradient is order-fixed; the forces and
    # the cell lists upstream use atomics, so reruns agree to rounding
    assert abs(loss - loss2) <= 1e-12 * loss
    assert np.abs(g - g2).max() <= 1e-10 * np.abs(g).max()
    # oracle: per structure dE_s and Dw_s from per-atom ff_wderiv
    oracle.load(w.types, paths)
    offs = np.concatenate([[0], np.cumsum(nws)])
    ref = np.zeros(offs[-1])
    sse = 0.0
    for k, s in enumerate(w.structures):
        _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types)
        E = 0.0
        Dw = np.zeros_like(ref)
        for a in range(s.natoms):
            nbcoo, _, _, nbt = nb[a]
            t = int(s.types[a])
            Ei, gi = oracle.atomic_energy_wgrad(centres[a], t, nbcoo, nbt)
            E += Ei
            Dw[offs[t - 1]:offs[t]] -= gi / s.natoms
        E_scale = 1.0 / workloads.TS_SCALE
        dE = (E_t[k] - E) / (E_scale * s.natoms)
        sse += 0.5 * dE * dE
        ref += dE * Dw / E_scale
    assert abs(loss - sse) <= G_REL_FP64 * max(sse, 1e-30) + 1e-18
    assert np.abs(g - ref).max() <= G_REL_FP64 * np.abs(ref).max()


@pytest.mark.parametrize("which", ["batch", "batch_odd"])
def test_force_loss_gradient_matches_finite_differences(cuda, request, which):
    from aenet_gb300.core import FP64
    from aenet_gb300.train import LOSS_ENERGY_FORCES, Trainer
    w, paths, tpaths = request.getfixturevalue(which)
    E_t, F_t = _targets(w, tpaths)
    ann = _ann(paths, w.types)
    try:
        tr = Trainer(ann, _structs(w), E_t, F_t, mode=LOSS_ENERGY_FORCES, w_E=1.0, w_F=0.1,
                     precision=FP64)
        W0 = ann.get_weights()
        loss, g = tr.loss_and_grad()
        nws = [ann.nweights(t) for t in w.types]
        offs = np.concatenate([[0], np.cumsum(nws)])
        # per species: a first-layer weight, a first-layer bias, a hidden
        # weight and the output bias (W per layer column-major (nout, nin+1),
        # bias in the last column)
        n0, n1 = w.arch[0], w.arch[1]
        picks = []
        for t in range(len(w.types)):
            o = offs[t]
            picks += [o + 5, o + n1 * n0 + 7, o + (n0 + 1) * n1 + 40, offs[t + 1] - 1]
        for k in picks:
            h = 1e-4 * max(1.0, abs(W0[k]))
            f = {}
            for m in (-2, -1, 1, 2):
                Wm = W0.copy()
                Wm[k] += m * h
                f[m] = tr.loss_and_grad(Wm)[0]
            fd = (8 * (f[1] - f[-1]) - (f[2] - f[-2])) / (12 * h)
            assert abs(fd - g[k]) <= G_REL_FD * max(abs(g[k]), 1e-3 * np.abs(g).max()), (k, fd, g[k])
        tr.loss_and_grad(W0)
        tr.close()
    finally:
        ann.release()


@pytest.mark.parametrize("which", ["batch", "batch_odd"])
def test_mixed_gradient_close_to_fp64(cuda, request, which):
    from aenet_gb300.core import FP64, MIXED
    from aenet_gb300.train import LOSS_ENERGY_FORCES, Trainer
    w, paths, tpaths = request.getfixturevalue(which)
    E_t, F_t = _targets(w, tpaths)
    ann = _ann(paths, w.types)
    try:
        out = {}
        for prec in (FP64, MIXED):
            tr = Trainer(ann, _structs(w), E_t, F_t, mode=LOSS_ENERGY_FORCES, precision=prec)
            out[prec] = tr.loss_and_grad()
            tr.close()
    finally:
        ann.release()
    (l64, g64), (l32, g32) = out[FP64], out[MIXED]
    assert abs(l32 - l64) <= G_REL_MIXED * l64
    assert np.linalg.norm(g32 - g64) <= G_REL_MIXED * np.linalg.norm(g64)


def test_lbfgs_fit_reduces_loss_and_saves_weights(cuda, batch, tmp_path):
    from aenet_gb300.core import MIXED
    from aenet_gb300.nnfile import read_nn
    from aenet_gb300.train import LOSS_ENERGY_FORCES, Trainer
    w, paths, tpaths = batch
    E_t, F_t = _targets(w, tpaths)
    ann = _ann(paths, w.types)
    try:
        tr = Trainer(ann, _structs(w), E_t, F_t, mode=LOSS_ENERGY_FORCES, precision=MIXED)
        l0, _ = tr.loss_and_grad()
        res = tr.fit(maxiter=25)
        l1, _ = tr.loss_and_grad()
        tr.close()
        assert l1 < 0.5 * l0, (l0, l1, res.message)
        W = ann.get_weights()
        ann.save_potential(w.types[0], tmp_path / "saved.nn")
        net, _, _, _ = read_nn(str(tmp_path / "saved.nn"))
        assert np.array_equal(net["W"], W[:ann.nweights(w.types[0])])
    finally:
        ann.release()


def test_generate_and_train_from_trainset_file(cuda, oracle, batch, tmp_path):
    """generate.x -> training-set file -> ts_normalize -> train.x energy
    loss from the stored descriptors: raw descriptors match the oracle, and
    the loss and gradient equal those of the positional path."""
    from aenet_gb300 import workloads
    from aenet_gb300.core import FP64
    from aenet_gb300.generate import generate_trainset
    from aenet_gb300.nnfile import read_nn
    from aenet_gb300.trainset import normalize, read_trainset
    from aenet_gb300.train import DescriptorTrainer, LOSS_ENERGY, Trainer
    w, paths, tpaths = batch
    E_t, F_t = _targets(w, tpaths)
    structs = [{"positions": s.positions, "symbols": [w.types[t - 1] for t in s.types],
                "cell": s.cell, "energy": E_t[k],
                "name": "s%d" % k} for k, s in enumerate(w.structures)]
    generate_trainset({t: paths[t] for t in w.types}, structs, str(tmp_path / "set.train"))
    raw = read_trainset(str(tmp_path / "set.train"))
    assert raw.setup_records is not None and len(raw.structures) == len(w.structures)
    # raw descriptors of a few atoms against the oracle
    oracle.load(w.types, paths)
    s0 = w.structures[0]
    _, centres, nb = oracle.neighbors(s0.cell, s0.positions, s0.types, atoms=[0, 1, 2])
    for q in range(3):
        nbcoo, _, _, nbt = nb[q]
        ref = oracle.descriptor(centres[q], int(s0.types[q]), nbcoo, nbt, scaled=False)
        assert np.abs(raw.structures[0]["sfval"][q] - ref).max() < 1e-10 * max(1, np.abs(ref).max())
    # normalise with the potentials' own statistics and energy scale
    stats = {}
    for k, t in enumerate(w.types, start=1):
        _, stp, tsi, _ = read_nn(paths[t])
        sd = np.sqrt(np.asarray(stp["sfval_cov"]) - np.asarray(stp["sfval_avg"]) ** 2)
        stats[k] = (np.asarray(stp["sfval_avg"]), np.where(sd <= 1e-10, 0.0, 1.0 / sd))
    norm = normalize(raw, stats, scale=workloads.TS_SCALE, shift=workloads.TS_SHIFT)
    ann = _ann(paths, w.types)
    try:
        dt = DescriptorTrainer(ann, norm, precision=FP64)
        l1, g1 = dt.loss_and_grad()
        dt.close()
        tr = Trainer(ann, _structs(w), E_t, mode=LOSS_ENERGY, precision=FP64)
        l0, g0 = tr.loss_and_grad()
        tr.close()
    finally:
        ann.release()
    assert abs(l1 - l0) <= 1e-9 * l0
    assert np.abs(g1 - g0).max() <= 1e-9 * np.abs(g0).max()


def test_descriptor_jacobians_match_oracle_and_export_file(cuda, oracle, batch, tmp_path):
    """generate.x's PyTorch export: the FP64 descriptor Jacobians of every
    neighbour slot and of the central atom against the oracle's stp_eval
    derivatives (sfb_radial / sfb_angular restated), matched by pair
    vector; then the .forces file written by generate_trainset holds the
    same numbers in the reference's record layout."""
    import torch
    from aenet_gb300.core import FP64
    from aenet_gb300.generate import generate_trainset
    from aenet_gb300.plan import Plan
    from aenet_gb300.pytorch_export import read_forces_file
    w, paths, tpaths = batch
    oracle.load(w.types, paths)
    ann = _ann(paths, w.types)
    try:
        for s in w.structures[:3]:
            plan = Plan([s.natoms], s.cell[None], np.array([1], dtype=np.int32), precision=FP64)
            p = torch.tensor(s.positions, device="cuda")
            t = torch.tensor(s.types.astype(np.int32), device="cuda")
            plan.run(p, t, forces=False)
            plan.check()
            Ji, Jj, nbl, nnb = (x.cpu().numpy() for x in plan.jacobian())
            _, _, _, vec = plan.neighbors()
            vec = vec.cpu().numpy()
            plan.close()
            _, centres, nb = oracle.neighbors(s.cell, s.positions, s.types)
            for a in range(s.natoms):
                nbcoo, _, nblist, nbt = nb[a]
                G, di, dj = oracle.descriptor(centres[a], int(s.types[a]), nbcoo, nbt,
                                              scaled=False, deriv=True)
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
    finally:
        ann.release()
    # generate_trainset loads its own (identity-normalised) potentials
    structs = [{"positions": s.positions, "symbols": [w.types[t - 1] for t in s.types],
                "cell": s.cell, "energy": -1.0, "name": "s%d" % k}
               for k, s in enumerate(w.structures[:4])]
    generate_trainset({t: paths[t] for t in w.types}, structs, str(tmp_path / "set.train"),
                      forces_percent=50.0, seed=3)
    recs, max_nnb = read_forces_file(str(tmp_path / "set.train.forces"))
    assert len(recs) == 4 and sum(r["selected"] for r in recs) == 2
    seen = 0
    for k, r in enumerate(recs):
        s = w.structures[k]
        assert r["name"] == "s%d" % k and r["natoms"] == s.natoms and r["ntypes"] == 3
        if not r["selected"]:
            assert r["atoms"] == []
            continue
        for a, (itype, nbl1, dGi, dGj) in enumerate(r["atoms"]):
            assert itype == s.types[a]
            assert nbl1.min() >= 1 and nbl1.max() <= s.natoms
            np.testing.assert_allclose(dGi, -dGj.sum(0), rtol=0, atol=1e-9 * max(1, np.abs(dGj).max()))
            seen = max(seen, len(nbl1))
    assert max_nnb == seen


def test_fit_resumes_from_restart_file(cuda, batch, tmp_path):
    """train.restart semantics: 3 + 3 iterations through the restart file
    reach the weights of 6 uninterrupted iterations (FP64 energy loss)."""
    from aenet_gb300.core import FP64
    from aenet_gb300.train import LOSS_ENERGY, Trainer
    w, paths, tpaths = batch
    E_t, _ = _targets(w, tpaths)
    ann = _ann(paths, w.types)
    try:
        W0 = ann.get_weights()
        tr = Trainer(ann, _structs(w), E_t, mode=LOSS_ENERGY, precision=FP64)
        r6 = tr.fit(maxiter=6)
        ann.set_weights(W0)
        path = str(tmp_path / "train.restart")
        r3 = tr.fit(maxiter=3, restart=path, nn_files={w.types[0]: str(tmp_path / "a.nn")})
        ann.set_weights(W0 * 0.0)     # the restart file, not the loaded weights, decides
        r33 = tr.fit(maxiter=3, restart=path)
        tr.close()
    finally:
        ann.release()
    assert r3.nit == 3 and r33.nit == 6 and r6.nit == 6
    from aenet_gb300.nnfile import read_nn
    net, _, _, _ = read_nn(str(tmp_path / "a.nn"))
    assert np.array_equal(net["W"], r3.x[:net["W"].size])
    assert abs(r33.fun - r6.fun) <= 1e-9 * abs(r6.fun)
    np.testing.assert_allclose(r33.x, r6.x, rtol=0, atol=1e-8 * np.abs(r6.x).max())


def test_moment_tangent_matches_pair_tangent(cuda, batch):
    """The FP32 E+F loss gradient with the angular tangent in moment form
    (reusing the forward's moments) against the pair form: same loss and
    gradient up to FP32 rounding."""
    from aenet_gb300.core import MIXED, set_option
    from aenet_gb300.train import LOSS_ENERGY_FORCES, Trainer
    w, paths, tpaths = batch
    E_t, F_t = _targets(w, tpaths)
    ann = _ann(paths, w.types)
    out = {}
    try:
        for mode in ("pairs", "moments"):
            set_option("angular_terms", mode)
            tr = Trainer(ann, _structs(w), E_t, F_t, mode=LOSS_ENERGY_FORCES, precision=MIXED)
            out[mode] = tr.loss_and_grad()
            tr.close()
    finally:
        set_option("angular_terms", "moments")
        ann.release()
    (l0, g0), (l1, g1) = out["pairs"], out["moments"]
    assert abs(l1 - l0) <= 1e-5 * l0
    assert np.linalg.norm(g1 - g0) <= 1e-4 * np.linalg.norm(g0)
