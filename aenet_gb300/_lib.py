"""ctypes binding of libaenet_gb300.so.

The library is the only compute path: importing this module without the
built library, or calling into it without a CUDA device, raises instead of
falling back to anything else.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaenet_gb300.so")

_lib = None

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
vp = C.c_void_p


class LibraryMissing(RuntimeError):
    pass


def _declare(lib):
    lib.aenet_init.argtypes = [C.c_int, C.POINTER(C.c_char_p), ip]
    lib.aenet_init.restype = None
    lib.aenet_final.argtypes = [ip]
    lib.aenet_final.restype = None
    lib.aenet_print_info.argtypes = []
    lib.aenet_print_info.restype = None
    lib.aenet_load_potential.argtypes = [C.c_int, C.c_char_p, ip]
    lib.aenet_load_potential.restype = None
    lib.aenet_all_loaded.argtypes = []
    lib.aenet_all_loaded.restype = C.c_bool
    lib.aenet_free_atom_energy.argtypes = [C.c_int]
    lib.aenet_free_atom_energy.restype = C.c_double
    lib.aenet_atomic_energy.argtypes = [vp, C.c_int, C.c_int, vp, vp, dp, ip]
    lib.aenet_atomic_energy.restype = None
    lib.aenet_atomic_energy_and_forces.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp,
                                                   C.c_int, dp, vp, ip]
    lib.aenet_atomic_energy_and_forces.restype = None
    lib.aenet_convert_atom_types.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_int, vp, vp, ip]
    lib.aenet_convert_atom_types.restype = None
    lib.aenet_sfb_init.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.c_int, C.c_int, C.c_double,
                                   C.c_double, ip]
    lib.aenet_sfb_init.restype = None
    lib.aenet_sfb_final.argtypes = [ip]
    lib.aenet_sfb_final.restype = None
    lib.aenet_sfb_nvalues.argtypes = []
    lib.aenet_sfb_nvalues.restype = C.c_int
    lib.aenet_sfb_eval.argtypes = [C.c_int, vp, C.c_int, vp, vp, C.c_int, vp, ip]
    lib.aenet_sfb_eval.restype = None
    lib.aenet_sfb_reconstruct_radial.argtypes = [C.c_int, vp, C.c_int, vp, vp, ip]
    lib.aenet_sfb_reconstruct_radial.restype = None
    lib.aenet_nbl_init.argtypes = [vp, C.c_int, vp, vp, C.c_bool, C.c_bool]
    lib.aenet_nbl_init.restype = None
    lib.aenet_nbl_final.argtypes = []
    lib.aenet_nbl_final.restype = None
    lib.aenet_nbl_neighbors.argtypes = [C.c_int, ip, vp, vp, vp, vp]
    lib.aenet_nbl_neighbors.restype = None
    lib.aenet_gpu_set_option.argtypes = [C.c_char_p, C.c_char_p]
    lib.aenet_gpu_set_option.restype = C.c_int
    lib.aenet_gpu_structure_energy_forces.argtypes = [C.c_int, vp, vp, vp, C.c_int, C.c_int, dp, dp,
                                                      vp, vp, vp, ip]
    lib.aenet_gpu_structure_energy_forces.restype = None
    lib.aenet_gpu_batch_energy_forces.argtypes = [C.c_int, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp,
                                                  ip]
    lib.aenet_gpu_batch_energy_forces.restype = None
    lib.aenet_gpu_plan_create.argtypes = [C.c_int, vp, vp, vp, vp, C.c_int, ip]
    lib.aenet_gpu_plan_create.restype = vp
    lib.aenet_gpu_plan_destroy.argtypes = [vp]
    lib.aenet_gpu_plan_destroy.restype = None
    lib.aenet_gpu_plan_natoms.argtypes = [vp]
    lib.aenet_gpu_plan_natoms.restype = C.c_int
    lib.aenet_gpu_plan_set_lattices.argtypes = [vp, vp]
    lib.aenet_gpu_plan_set_lattices.restype = C.c_int
    lib.aenet_gpu_plan_run.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_uint, vp]
    lib.aenet_gpu_plan_run.restype = C.c_int
    lib.aenet_gpu_plan_forward.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.aenet_gpu_plan_forward.restype = C.c_int
    lib.aenet_gpu_plan_backward.argtypes = [vp, vp, vp, vp, vp]
    lib.aenet_gpu_plan_backward.restype = C.c_int
    lib.aenet_gpu_plan_profile.argtypes = [vp, vp, vp, vp, vp, C.POINTER(C.c_float), vp]
    lib.aenet_gpu_plan_profile.restype = C.c_int
    lib.aenet_gpu_measure_fp32_peak.argtypes = [dp, vp]
    lib.aenet_gpu_measure_fp32_peak.restype = C.c_int
    lib.aenet_gpu_plan_status.argtypes = [vp, vp]
    lib.aenet_gpu_plan_status.restype = C.c_uint
    lib.aenet_gpu_plan_neighbors.argtypes = [vp, ip, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]
    lib.aenet_gpu_plan_neighbors.restype = C.c_int
    lib.aenet_gpu_plan_descriptors.argtypes = [vp, C.POINTER(vp), ip]
    lib.aenet_gpu_plan_descriptors.restype = C.c_int
    lib.aenet_gpu_structure_energy_forces_noalloc.argtypes = [C.c_int, vp, vp, vp, C.c_int, vp, vp,
                                                              vp, vp, vp]
    lib.aenet_gpu_structure_energy_forces_noalloc.restype = C.c_int
    lib.aenet_gpu_plan_loss_gradient.argtypes = [vp, vp, vp, vp, vp, C.c_int, C.c_double,
                                                 C.c_double, vp, vp, vp, vp, vp]
    lib.aenet_gpu_plan_loss_gradient.restype = C.c_int
    lib.aenet_gpu_network_nweights.argtypes = [C.c_int]
    lib.aenet_gpu_network_nweights.restype = C.c_int
    lib.aenet_gpu_get_weights.argtypes = [vp]
    lib.aenet_gpu_get_weights.restype = C.c_int
    lib.aenet_gpu_set_weights.argtypes = [vp]
    lib.aenet_gpu_set_weights.restype = C.c_int
    lib.aenet_gpu_save_potential.argtypes = [C.c_int, C.c_char_p]
    lib.aenet_gpu_save_potential.restype = C.c_int
    lib.aenet_gpu_plan_load_descriptors.argtypes = [vp, vp, C.c_int]
    lib.aenet_gpu_plan_load_descriptors.restype = C.c_int
    lib.aenet_gpu_plan_neighbour_capacity.argtypes = [vp]
    lib.aenet_gpu_plan_neighbour_capacity.restype = C.c_int
    lib.aenet_gpu_plan_descriptor_jacobian.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp]
    lib.aenet_gpu_plan_descriptor_jacobian.restype = C.c_int
    lib.aenet_gpu_plan_descriptor_loss_gradient.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    lib.aenet_gpu_plan_descriptor_loss_gradient.restype = C.c_int
    lib.aenet_gpu_neighbor_list_energy_forces.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, C.c_int,
                                                           vp, vp, vp, vp]
    lib.aenet_gpu_neighbor_list_energy_forces.restype = C.c_int
    lib.aenet_gpu_md_create.argtypes = [C.c_int, vp, vp, vp, vp, vp, C.c_double, C.c_double,
                                        C.c_int, ip]
    lib.aenet_gpu_md_create.restype = vp
    lib.aenet_gpu_md_destroy.argtypes = [vp]
    lib.aenet_gpu_md_destroy.restype = None
    lib.aenet_gpu_md_run.argtypes = [vp, C.c_int, dp, dp]
    lib.aenet_gpu_md_run.restype = C.c_int
    lib.aenet_gpu_md_get.argtypes = [vp, vp, vp, vp]
    lib.aenet_gpu_md_get.restype = C.c_int
    lib.aenet_gpu_md_counters.argtypes = [vp, C.POINTER(C.c_longlong), ip]
    lib.aenet_gpu_md_counters.restype = C.c_int
    lib.aenet_gpu_md_phase_times.argtypes = [vp, dp, C.POINTER(C.c_longlong), dp,
                                             C.POINTER(C.c_longlong)]
    lib.aenet_gpu_md_phase_times.restype = C.c_int
    lib.aenet_gpu_md_energy_fp64.argtypes = [vp, dp]
    lib.aenet_gpu_md_energy_fp64.restype = C.c_int
    return lib


def lib():
    """Load (once) and return the library; raises LibraryMissing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                "libaenet_gb300.so is not built (run `python -c 'import __graft_entry__ as g; "
                "g.build()'` or `python aenet_gb300/build.py`)")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def exported_symbols():
    """Names declared in include/aenet.h and include/aenet_gb300.h."""
    import re
    root = os.path.dirname(HERE)
    names = []
    for h in ("aenet.h", "aenet_gb300.h"):
        txt = open(os.path.join(root, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = "\n".join(l for l in txt.splitlines() if not l.lstrip().startswith("typedef"))
        for m in re.finditer(r"\b(aenet_\w+|AENET_\w+)\s*(\(|;)", txt):
            names.append(m.group(1))
        for m in re.finditer(r"extern\s+\w+\s+(\w+)\s*;", txt):
            names.append(m.group(1))
    return sorted(set(n for n in names
                       if not (n.startswith("AENET_GPU_") or n.startswith("AENET_NOALLOC_"))))


def ntypes():
    """Number of loaded species (0 when nothing is loaded)."""
    n = 0
    while n < 8 and lib().aenet_gpu_network_nweights(n + 1) >= 0:
        n += 1
    return n
