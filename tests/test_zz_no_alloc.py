"""The allocation-free entry point against the allocating one.

aenet_gpu_structure_energy_forces_noalloc serves callers that cannot
allocate device memory while they run (MD engines that reserve all GPU
memory up front and forbid allocation in their time loop, plugin hosts
whose application owns the memory pool): it takes device buffers and keeps
its scratch in an array compiled into the library.  Here it is called through the C-ABI twice in a row -- the second
call sees the first call's leftovers in the shared scratch -- and each
result must match aenet_gpu_structure_energy_forces on the same structure
within the tolerances the other GPU tests use.  The file runs last so that a
failure here cannot hide failures elsewhere; it also passes on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu

E_TOL_FP64 = 1e-10      # eV/atom, as in test_gpu_parity.py
F_TOL_FP64 = 1e-9       # eV/A
E_TOL_MIXED = 1e-3      # eV/atom
F_RMS_MIXED = 2e-2      # eV/A


@pytest.fixture(scope="module")
def setup(oracle, tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from aenet_gb300 import workloads
    from aenet_gb300.core import ANNPotentials
    w = workloads.aucu_fcc_4000()
    # a 4x4x4 cut (256 atoms) of the alloy stays inside the scratch limits
    s = w.structures[0]
    sites, _ = workloads.fcc_positions(10, 3.90)
    keep = np.all(sites < 4 * 3.90 - 0.1, axis=1)
    pos = s.positions[keep]
    types = s.types[keep]
    cell = np.eye(3) * (4 * 3.90)
    sub = workloads.Workload(w.name, w.types, w.setups, w.arch,
                             [workloads.Structure(pos, types, cell)], w.seed)
    sub.networks = w.networks
    paths = helpers.make_potentials(oracle, sub, str(tmp_path_factory.mktemp("noalloc")))
    ann = ANNPotentials({t: paths[t] for t in w.types})
    # the allocation-free call reads the device tables that the first
    # allocating evaluation builds
    st = sub.structures[0]
    ann.structure_energy_forces(st.positions, st.types, st.cell)
    yield torch, ann, st
    ann.release()


def _noalloc(torch, lib, s, precision, status=0):
    n = s.natoms
    d_pos = torch.tensor(s.positions, device="cuda")
    d_typ = torch.tensor(s.types, device="cuda", dtype=torch.int32)
    d_E = torch.zeros(1, dtype=torch.float64, device="cuda")
    d_F = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    d_W = torch.zeros(9, dtype=torch.float64, device="cuda")
    d_st = torch.full((1,), 0xFFFF, dtype=torch.int32, device="cuda")
    lat = np.ascontiguousarray(s.cell, dtype=np.float64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.aenet_gpu_structure_energy_forces_noalloc(
        n, C.c_void_p(d_pos.data_ptr()), C.c_void_p(d_typ.data_ptr()),
        lat.ctypes.data_as(C.c_void_p), precision, C.c_void_p(d_E.data_ptr()),
        C.c_void_p(d_F.data_ptr()), C.c_void_p(d_W.data_ptr()), C.c_void_p(d_st.data_ptr()),
        stream)
    assert rc == 0, rc
    torch.cuda.synchronize()
    assert int(d_st.item()) == status, int(d_st.item())
    return d_E.item(), d_F.cpu().numpy(), d_W.cpu().numpy().reshape(3, 3)


def _compare(ref, got, n, prec, FP64):
    E, F, W = got
    if prec == FP64:
        assert abs(E - ref["energy"]) / n < E_TOL_FP64, (E, ref["energy"])
        assert np.abs(F - ref["forces"]).max() < F_TOL_FP64
        assert np.abs(W - ref["virial"]).max() < 1e-8
    else:
        assert abs(E - ref["energy"]) / n < E_TOL_MIXED
        assert np.sqrt(np.mean((F - ref["forces"]) ** 2)) < F_RMS_MIXED
        assert np.abs(W - ref["virial"]).max() < 1e-2 * max(1.0, np.abs(ref["virial"]).max())


def test_noalloc_matches_allocating_entry_point(setup):
    torch, ann, s = setup
    from aenet_gb300 import _lib
    from aenet_gb300.core import FP64, MIXED
    lib = _lib.lib()
    n = s.natoms
    for prec in (FP64, MIXED):
        # the allocating entry point first: it also builds the device tables
        ref = ann.structure_energy_forces(s.positions, s.types, s.cell, precision=prec,
                                          virial=True)
        for call in range(2):
            _compare(ref, _noalloc(torch, lib, s, prec), n, prec, FP64)


def test_noalloc_eight_lanes_and_triclinic_cell(setup):
    """Eight lanes per atom (the descriptor kernels' smallest groups, whose
    FP64 adjoint needs the most shared memory) and a sheared cell, both
    precisions, two calls each, against the allocating entry point."""
    torch, ann, s = setup
    from aenet_gb300 import _lib, workloads
    from aenet_gb300.core import FP64, MIXED, set_option
    lib = _lib.lib()
    shear = np.array([[1.0, 0.0, 0.0], [0.18, 1.0, 0.0], [-0.11, 0.07, 1.0]])
    tric = workloads.Structure(s.positions @ shear, s.types, s.cell @ shear)
    try:
        set_option("lanes_per_atom", 8)
        for st in (s, tric):
            for prec in (FP64, MIXED):
                ref = ann.structure_energy_forces(st.positions, st.types, st.cell, precision=prec,
                                                  virial=True)
                for call in range(2):
                    _compare(ref, _noalloc(torch, lib, st, prec), st.natoms, prec, FP64)
    finally:
        set_option("lanes_per_atom", 16)


def test_noalloc_reports_neighbour_overflow(setup):
    """A cell compressed until its atoms have more neighbours than the
    fixed per-atom limit (192): the call returns, and the status word it
    writes carries the neighbour-overflow bit."""
    torch, ann, s = setup
    from aenet_gb300 import _lib, workloads
    from aenet_gb300.core import FP64
    lib = _lib.lib()
    dense = workloads.Structure(s.positions * 0.62, s.types, s.cell * 0.62)
    _noalloc(torch, lib, dense, FP64, status=1)     # AENET_GPU_ST_NB_OVERFLOW


def test_noalloc_rejects_oversized_input(setup):
    torch, ann, s = setup
    from aenet_gb300 import _lib
    from aenet_gb300.core import FP64
    lib = _lib.lib()
    too_many = 2049        # AENET_NOALLOC_MAX_ATOMS + 1
    d = torch.zeros((too_many, 3), dtype=torch.float64, device="cuda")
    t = torch.ones(too_many, dtype=torch.int32, device="cuda")
    lat = np.ascontiguousarray(np.eye(3) * 50.0)
    rc = lib.aenet_gpu_structure_energy_forces_noalloc(
        too_many, C.c_void_p(d.data_ptr()), C.c_void_p(t.data_ptr()),
        lat.ctypes.data_as(C.c_void_p), FP64, None, None, None, None,
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 2         # AENET_ERR_MALLOC: beyond the scratch capacity
