"""The C-ABI library on the host (no GPU needed): loading, exports, potential
files, status codes, and that evaluation refuses to run without a GPU."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from tests.golden import fixtures


@pytest.fixture(scope="module")
def lib():
    from aenet_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from aenet_gb300 import build
        build.build()
    return _lib.lib()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_every_declared_symbol_is_exported(lib):
    from aenet_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    defined = {l.split()[-1] for l in out.splitlines() if l.strip()}
    declared = _lib.exported_symbols()
    assert "aenet_atomic_energy_and_forces" in declared
    assert "aenet_gpu_plan_run" in declared
    missing = [s for s in declared if s not in defined]
    assert not missing, missing


def _init(lib, names):
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    st = C.c_int(-1)
    lib.aenet_init(len(names), arr, C.byref(st))
    return st.value


def _final(lib):
    st = C.c_int(-1)
    lib.aenet_final(C.byref(st))
    return st.value


def test_load_potentials_and_range(lib, tmp_path):
    """K-2: python3/aenet/tests/test_core.py:29-30 through the C-ABI."""
    k1 = fixtures.load("k1_ti2o4.npz")
    paths = fixtures.write_potential_files(fixtures.potentials(k1), str(tmp_path))
    assert _init(lib, ["Ti", "O"]) == 0
    try:
        assert _init(lib, ["Ti", "O"]) == 1          # AENET_ERR_INIT
        assert not lib.aenet_all_loaded()
        st = C.c_int(-1)
        lib.aenet_load_potential(3, paths["Ti"].encode(), C.byref(st))
        assert st.value == 4                          # AENET_ERR_TYPE
        lib.aenet_load_potential(1, str(tmp_path / "missing.nn").encode(), C.byref(st))
        assert st.value == 3                          # AENET_ERR_IO
        lib.aenet_load_potential(1, paths["Ti"].encode(), C.byref(st))
        assert st.value == 0
        lib.aenet_load_potential(2, paths["O"].encode(), C.byref(st))
        assert st.value == 0
        assert lib.aenet_all_loaded()
        assert C.c_double.in_dll(lib, "aenet_Rc_min").value == 0.55
        assert C.c_double.in_dll(lib, "aenet_Rc_max").value == 8.0
        assert C.c_int.in_dll(lib, "aenet_nsf_max").value == 44
        # lcl_nmax_nbdist(0.55, 8.0)
        assert C.c_int.in_dll(lib, "aenet_nnb_max").value == int(
            np.ceil((8.0 + 0.275) ** 3 / 0.275 ** 3 * 0.7405))
        ti = fixtures.potentials(k1)["Ti"]["ts"]
        assert lib.aenet_free_atom_energy(1) == ti["E_atom"][ti["typeName"].index("Ti")]
        # aenet_convert_atom_types: ["O","Ti"] ids -> library ids
        names = (C.c_char_p * 2)(b"O", b"Ti")
        tin = np.array([1, 2, 2, 1], dtype=np.int32)
        tout = np.zeros(4, dtype=np.int32)
        lib.aenet_convert_atom_types(2, names, 4, tin.ctypes.data_as(C.c_void_p),
                                     tout.ctypes.data_as(C.c_void_p), C.byref(st))
        assert st.value == 0 and tout.tolist() == [2, 1, 1, 2]
    finally:
        assert _final(lib) == 0


def test_truncated_potential_file_is_an_io_error(lib, tmp_path):
    k1 = fixtures.load("k1_ti2o4.npz")
    paths = fixtures.write_potential_files(fixtures.potentials(k1), str(tmp_path))
    data = open(paths["Ti"], "rb").read()
    bad = tmp_path / "trunc.nn"
    bad.write_bytes(data[: len(data) // 2])
    assert _init(lib, ["Ti"]) == 0
    try:
        st = C.c_int(-1)
        lib.aenet_load_potential(1, str(bad).encode(), C.byref(st))
        assert st.value == 3
    finally:
        _final(lib)


def test_uninitialised_calls_report_init_error(lib):
    st = C.c_int(-1)
    E = C.c_double(0)
    coo = np.zeros(3)
    lib.aenet_atomic_energy(coo.ctypes.data_as(C.c_void_p), 1, 0, None, None, C.byref(E),
                            C.byref(st))
    assert st.value == 1


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback_without_gpu(lib, tmp_path):
    """Evaluation needs the GPU: without one the call fails with
    AENET_ERR_CUDA instead of computing on the CPU."""
    k1 = fixtures.load("k1_ti2o4.npz")
    paths = fixtures.write_potential_files(fixtures.potentials(k1), str(tmp_path))
    assert _init(lib, ["Ti", "O"]) == 0
    try:
        st = C.c_int(-1)
        for i, t in enumerate(["Ti", "O"], start=1):
            lib.aenet_load_potential(i, paths[t].encode(), C.byref(st))
            assert st.value == 0
        coo_i = np.zeros(3)
        coo_j = np.array([[1.9, 0.0, 0.0]])
        tj = np.array([2], dtype=np.int32)
        E = C.c_double(0)
        lib.aenet_atomic_energy(coo_i.ctypes.data_as(C.c_void_p), 1, 1,
                                coo_j.ctypes.data_as(C.c_void_p), tj.ctypes.data_as(C.c_void_p),
                                C.byref(E), C.byref(st))
        assert st.value == 5
    finally:
        _final(lib)


def test_noalloc_entry_point_requires_loaded_tables():
    """Without loaded potentials the allocation-free entry point returns
    AENET_ERR_INIT before it touches the GPU or any of its pointers."""
    import ctypes as C
    import numpy as np
    from aenet_gb300 import _lib
    lib = _lib.lib()
    lat = np.ascontiguousarray(np.eye(3) * 10.0)
    fake = C.c_void_p(256)     # never dereferenced: the call returns first
    rc = lib.aenet_gpu_structure_energy_forces_noalloc(
        4, fake, fake, lat.ctypes.data_as(C.c_void_p), 0, None, None, None, None, None)
    assert rc == 1


def test_every_declared_function_has_ctypes_signature():
    """Each function of include/*.h is bound with argtypes in the ctypes
    layer: without them ctypes passes Python ints (handles, pointers) as
    32-bit C ints, which truncates pointers above 4 GB."""
    import ctypes as C
    import os
    import re
    from aenet_gb300 import _lib
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    text = "".join(open(os.path.join(root, "include", h)).read()
                   for h in ("aenet.h", "aenet_gb300.h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(aenet_\w+)\s*\(", text)))
    lib = _lib._declare(C.CDLL(_lib.LIB_PATH))
    missing = [n for n in names if getattr(lib, n).argtypes is None]
    assert not missing, missing


def test_options_accept_documented_values_only(lib):
    """aenet_gpu_set_option takes the keys and values include/aenet_gb300.h
    documents (host state only, no GPU needed) and returns AENET_ERR_INPUT
    for anything else; the defaults are restored afterwards."""
    from aenet_gb300.core import AENET_ERR_INPUT
    ok = {
        "angular_domain": ["current", "legacy"],
        "angular_terms": ["moments", "pairs"],
        "angular_spin": ["own", "stale"],
        "neighbour_kernel": ["atom", "cell", "stream", "half", "struct", "struct_half"],
        "networks": ["tensor", "simt"],
        "per_atom_kernel": ["fused", "cluster", "block", "graph"],
        "lanes_per_atom": ["8", "16", "32"],
        "cell_div": ["1", "2", "3"],
        "z_refine": ["1", "2", "3", "4"],
    }
    defaults = {"angular_domain": "current", "angular_terms": "moments", "angular_spin": "own",
                "neighbour_kernel": "atom", "networks": "tensor", "per_atom_kernel": "fused",
                "lanes_per_atom": "16", "cell_div": "2", "z_refine": "1"}
    try:
        for key, values in ok.items():
            for v in values:
                assert lib.aenet_gpu_set_option(key.encode(), v.encode()) == 0, (key, v)
            assert lib.aenet_gpu_set_option(key.encode(), b"bogus") == AENET_ERR_INPUT, key
        assert lib.aenet_gpu_set_option(b"no_such_key", b"1") == AENET_ERR_INPUT
    finally:
        for key, v in defaults.items():
            lib.aenet_gpu_set_option(key.encode(), v.encode())
