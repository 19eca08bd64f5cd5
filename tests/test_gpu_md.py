"""GPU molecular dynamics (velocity Verlet with a Verlet skin).

- FP64 trajectory against a host velocity-Verlet integration that takes
  its forces from the FP64 oracle (positions 1e-9 A, energies 1e-9 eV);
- neighbour refresh inside the skin against a rebuild every step
  (positions 1e-9 A after 40 steps);
- NVE energy conservation of the mixed-precision run and its FP64 monitor.
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


@pytest.fixture(scope="module")
def cuau(oracle, tmp_path_factory):
    """256-atom Cu/Au FCC cut of the 1M-atom workload (same potentials
    layout: 52-20-20-1, Chebyshev r16/6.0 a8/4.0), velocities at 600 K."""
    from aenet_gb300 import workloads
    w = workloads.cuau_fcc_1m(n=4)
    paths = helpers.make_potentials(oracle, w, str(tmp_path_factory.mktemp("md")))
    return w, paths


def _ann(paths, types):
    from aenet_gb300.core import ANNPotentials
    return ANNPotentials({t: paths[t] for t in types}, angular_domain="current")


def _md(w, paths, precision, skin, dt=2.0):
    from aenet_gb300.md import MolecularDynamics
    s = w.structures[0]
    ann = _ann(paths, w.types)
    md = MolecularDynamics(ann, s.positions, s.types, s.cell, velocities=w.velocities,
                           dt=dt, skin=skin, precision=precision)
    return ann, md


def test_md_fp64_matches_host_verlet_with_oracle_forces(cuda, oracle, cuau):
    from aenet_gb300.core import FP64
    from aenet_gb300.md import MASS_UNIT
    from aenet_gb300.workloads import MASSES
    w, paths = cuau
    s = w.structures[0]
    ann, md = _md(w, paths, FP64, skin=0.3)
    try:
        md.run(5)
        r_gpu, v_gpu, f_gpu = md.state()
        e_gpu = md.E_pot
        md.close()
    finally:
        ann.release()
    oracle.load(w.types, paths)
    m = np.array([MASSES[w.types[t - 1]] for t in s.types])[:, None] * MASS_UNIT
    r = s.positions.copy()
    v = w.velocities.copy()
    _, _, F, _ = oracle.structure(s.cell, r, s.types)
    dt = 2.0
    for _ in range(5):
        v += 0.5 * dt * F / m
        r += dt * v
        _, e, F, _ = oracle.structure(s.cell, r, s.types)
        v += 0.5 * dt * F / m
    assert np.abs(r_gpu - r).max() < 1e-9
    assert np.abs(v_gpu - v).max() < 1e-10
    assert np.abs(f_gpu - F).max() < 1e-8
    assert abs(e_gpu - e) < 1e-9 * s.natoms


def test_md_skin_refresh_matches_rebuild_every_step(cuda, cuau):
    from aenet_gb300.core import FP64
    w, paths = cuau
    out = {}
    for skin in (0.3, 0.0):
        ann, md = _md(w, paths, FP64, skin=skin)
        try:
            md.run(40)
            out[skin] = md.state()[0], md.counters()
            md.close()
        finally:
            ann.release()
    (r_skin, (steps, builds)), (r_every, (_, builds0)) = out[0.3], out[0.0]
    assert steps == 40 and builds0 == 41 and builds < 41
    assert np.abs(r_skin - r_every).max() < 1e-9


def test_md_mixed_energy_conservation_and_fp64_monitor(cuda, cuau):
    from aenet_gb300.core import MIXED
    w, paths = cuau
    n = w.structures[0].natoms
    ann, md = _md(w, paths, MIXED, skin=0.3, dt=0.5)
    try:
        e0 = md.E_pot + md.E_kin
        drift = []
        for _ in range(10):
            ep, ek = md.run(20)
            drift.append(abs(ep + ek - e0) / n)
            # the FP64 re-evaluation of the same positions
            assert abs(md.energy_fp64() - ep) / n < 1e-3
        md.close()
    finally:
        ann.release()
    assert max(drift) < 2e-3, drift
