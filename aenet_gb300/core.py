"""Python surface of the drop-in: ``ANNPotentials`` (python3/aenet/core.pyx).

Same constructor, methods, read-only attributes and exceptions as the
reference's Cython class (core.pyx:38-202), backed by libaenet_gb300.so.
Beyond the reference it evaluates whole structures and batches on the GPU
(:meth:`structure_energy_forces`, :meth:`batch_energy_forces`).
"""
import ctypes as C

import numpy as np

from . import _lib

AENET_OK = 0
AENET_ERR_INIT = 1
AENET_ERR_MALLOC = 2
AENET_ERR_IO = 3
AENET_ERR_TYPE = 4
AENET_ERR_CUDA = 5
AENET_ERR_INPUT = 6

FP64 = 0
MIXED = 1


class AenetError(Exception):
    pass


class InitError(Exception):
    pass


class SpeciesError(Exception):
    pass


def check_status(stat):
    """core.pyx:190-202 plus the GPU codes."""
    if stat == AENET_ERR_MALLOC:
        raise MemoryError("aenetLib: Memory allocation failed.")
    elif stat == AENET_ERR_INIT:
        raise InitError("aenetLib: Module not initialized "
                        "(or attempt to re-initialize module).")
    elif stat == AENET_ERR_IO:
        raise IOError("aenetLib: I/O error encountered.")
    elif stat == AENET_ERR_TYPE:
        raise SpeciesError("aenetLib: Invalid atomic species.")
    elif stat == AENET_ERR_CUDA:
        raise AenetError("aenetLib: CUDA error (is a GPU available?).")
    elif stat == AENET_ERR_INPUT:
        raise AenetError("aenetLib: invalid input.")
    elif stat != 0:
        raise AenetError("aenetLib: Unspecified error encountered.")


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def set_option(key, value):
    """aenet_gpu_set_option: angular_domain, angular_spin, angular_terms,
    cell_div, z_refine, lanes_per_atom, adjoint_lanes_per_atom,
    neighbour_kernel, networks, per_atom_kernel (include/aenet_gb300.h)."""
    st = _lib.lib().aenet_gpu_set_option(key.encode(), str(value).encode())
    check_status(st)


class ANNPotentials:
    """Artificial Neural Network (ANN) potentials, one per species.

    ``potential_files`` maps species names to ``.nn`` files; the dict order
    defines the 1-based type ids.
    """

    def __init__(self, potential_files, angular_domain=None):
        lib = _lib.lib()
        self.atom_types = [str(t) for t in potential_files.keys()]
        self.potential_files = dict(potential_files)
        self.ntypes = len(self.atom_types)
        self.Rc_min = 0.0
        self.Rc_max = 0.0
        if angular_domain is not None:
            set_option("angular_domain", angular_domain)
        names = (C.c_char_p * self.ntypes)(*[t.encode() for t in self.atom_types])
        stat = C.c_int(0)
        lib.aenet_init(self.ntypes, names, C.byref(stat))
        check_status(stat.value)
        self._alive = True
        for t in self.atom_types:
            self._load_potential(t, str(self.potential_files[t]))
        assert lib.aenet_all_loaded()
        self.Rc_min = C.c_double.in_dll(lib, "aenet_Rc_min").value
        self.Rc_max = C.c_double.in_dll(lib, "aenet_Rc_max").value
        self.nnb_max = C.c_int.in_dll(lib, "aenet_nnb_max").value
        self.nsf_max = C.c_int.in_dll(lib, "aenet_nsf_max").value

    def release(self):
        if getattr(self, "_alive", False):
            stat = C.c_int(0)
            _lib.lib().aenet_final(C.byref(stat))
            self._alive = False

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def __str__(self):
        return " ANN Potentials\n   Atomic species: %s\n" % " ".join(self.atom_types)

    def _load_potential(self, atom_type, filename):
        type_id = self.get_type_id(atom_type)
        stat = C.c_int(0)
        _lib.lib().aenet_load_potential(type_id, filename.encode(), C.byref(stat))
        if stat.value == AENET_ERR_TYPE:
            raise SpeciesError("Unknown type ID: %d" % (type_id,))
        elif stat.value == AENET_ERR_IO:
            raise IOError("File not found: %s" % (filename,))
        check_status(stat.value)

    # ---- network weights (training) ----------------------------------
    def nweights(self, atom_type=None):
        """Wsize of one species, or of all species together."""
        lib = _lib.lib()
        if atom_type is not None:
            return lib.aenet_gpu_network_nweights(self.get_type_id(atom_type))
        return sum(lib.aenet_gpu_network_nweights(t) for t in range(1, self.ntypes + 1))

    def get_weights(self):
        """All weights: species in type order, each the network's W(1:Wsize)."""
        W = np.empty(self.nweights(), dtype=np.float64)
        check_status(_lib.lib().aenet_gpu_get_weights(W.ctypes.data_as(C.c_void_p)))
        return W

    def set_weights(self, W):
        W = np.ascontiguousarray(W, dtype=np.float64).reshape(-1)
        if W.size != self.nweights():
            raise ValueError("expected %d weights, got %d" % (self.nweights(), W.size))
        check_status(_lib.lib().aenet_gpu_set_weights(W.ctypes.data_as(C.c_void_p)))

    def save_potential(self, atom_type, filename):
        """Write the species' potential with its current weights (.nn)."""
        check_status(_lib.lib().aenet_gpu_save_potential(self.get_type_id(atom_type),
                                                         str(filename).encode()))

    def print_info_to_stdout(self):
        _lib.lib().aenet_print_info()

    def get_type_id(self, atom_type):
        for i, t in enumerate(self.atom_types):
            if t.strip() == str(atom_type).strip():
                return i + 1
        raise SpeciesError("Unknown atomic species: {}".format(atom_type))

    def free_atom_energy(self, atom_type):
        return _lib.lib().aenet_free_atom_energy(self.get_type_id(atom_type))

    # ---------------------------------------------------- per atom (core.pyx)
    def atomic_energy(self, coo_i, type_i, coo_j, type_j):
        coo_i = _f64(coo_i)
        coo_j = _f64(np.asarray(coo_j).reshape(-1, 3))
        itype_j = _i32([self.get_type_id(str(t)) for t in type_j])
        E = C.c_double(0.0)
        stat = C.c_int(0)
        _lib.lib().aenet_atomic_energy(_ptr(coo_i), self.get_type_id(type_i), len(type_j),
                                       _ptr(coo_j), _ptr(itype_j), C.byref(E), C.byref(stat))
        check_status(stat.value)
        return E.value

    def atomic_energy_and_forces(self, coo_i, type_i, index_i, coo_j, type_j, index_j, F):
        """F is (natoms, 3) float64, C-contiguous, accumulated in place;
        index_i / index_j are 1-based."""
        if not (isinstance(F, np.ndarray) and F.dtype == np.float64 and F.flags.c_contiguous):
            raise TypeError("F must be a C-contiguous float64 array")
        coo_i = _f64(coo_i)
        coo_j = _f64(np.asarray(coo_j).reshape(-1, 3))
        itype_j = _i32([self.get_type_id(str(t)) for t in type_j])
        idx_j = _i32(index_j)
        E = C.c_double(0.0)
        stat = C.c_int(0)
        _lib.lib().aenet_atomic_energy_and_forces(
            _ptr(coo_i), self.get_type_id(type_i), int(index_i), len(type_j), _ptr(coo_j),
            _ptr(itype_j), _ptr(idx_j), F.shape[0], C.byref(E), _ptr(F), C.byref(stat))
        check_status(stat.value)
        return E.value

    # -------------------------------------------------- whole structures
    def type_ids(self, symbols):
        return _i32([self.get_type_id(s) for s in symbols])

    def structure_energy_forces(self, positions, symbols_or_types, cell=None, pbc=True,
                                precision=FP64, forces=True, virial=False):
        """Energy (total, cohesive, per atom), forces and virial of one
        structure evaluated on the GPU (predict.x's get_energy)."""
        pos = _f64(positions).reshape(-1, 3)
        n = pos.shape[0]
        types = self._types(symbols_or_types)
        lat = _f64(np.zeros((3, 3)) if cell is None else cell).reshape(9)
        Et, Ec = C.c_double(0.0), C.c_double(0.0)
        Ea = np.zeros(n)
        F = np.zeros((n, 3)) if forces else None
        W = np.zeros((3, 3)) if virial else None
        stat = C.c_int(0)
        _lib.lib().aenet_gpu_structure_energy_forces(
            n, _ptr(pos), _ptr(types), _ptr(lat), int(bool(pbc)), int(precision), C.byref(Et),
            C.byref(Ec), _ptr(Ea), _ptr(F), _ptr(W), C.byref(stat))
        check_status(stat.value)
        out = {"energy": Et.value, "cohesive_energy": Ec.value, "atomic_energies": Ea}
        if forces:
            out["forces"] = F
        if virial:
            out["virial"] = W
        return out

    def batch_energy_forces(self, structures, precision=MIXED, forces=True, virial=False):
        """structures: list of (positions, symbols_or_types, cell, pbc)."""
        natoms = _i32([np.asarray(s[0]).reshape(-1, 3).shape[0] for s in structures])
        pos = _f64(np.concatenate([np.asarray(s[0], dtype=np.float64).reshape(-1, 3)
                                   for s in structures]))
        types = np.concatenate([self._types(s[1]) for s in structures]).astype(np.int32)
        lat = _f64(np.concatenate([np.asarray(s[2] if s[2] is not None else np.zeros((3, 3)),
                                              dtype=np.float64).reshape(9) for s in structures]))
        pbc = _i32([int(bool(s[3])) for s in structures])
        ns = len(structures)
        E = np.zeros(ns)
        F = np.zeros((pos.shape[0], 3)) if forces else None
        W = np.zeros((ns, 3, 3)) if virial else None
        stat = C.c_int(0)
        _lib.lib().aenet_gpu_batch_energy_forces(ns, _ptr(natoms), _ptr(pos), _ptr(types),
                                                 _ptr(lat), _ptr(pbc), int(precision), _ptr(E),
                                                 _ptr(F), _ptr(W), C.byref(stat))
        check_status(stat.value)
        out = {"energy": E}
        if forces:
            out["forces"] = F
        if virial:
            out["virial"] = W
        return out

    def neighbor_list_energy_forces(self, x, types, neigh_offset, neighbors, nlocal,
                                    precision=MIXED, virial=False):
        """Energy and forces from a caller's neighbour list: ``x`` holds the
        ``nlocal`` local atoms then the ghosts, ``neigh_offset``/``neighbors``
        the CSR lists of the local atoms.  Forces are returned for all atoms
        (ghosts included)."""
        x = _f64(x).reshape(-1, 3)
        nall = x.shape[0]
        t = self._types(types)
        off = _i32(neigh_offset)
        nb = _i32(neighbors)
        E = C.c_double(0.0)
        Ea = np.zeros(nlocal)
        F = np.zeros((nall, 3))
        W = np.zeros((3, 3)) if virial else None
        st = _lib.lib().aenet_gpu_neighbor_list_energy_forces(
            int(nlocal), nall, _ptr(x), _ptr(t), _ptr(off), _ptr(nb) if nb.size else None,
            int(precision), C.byref(E), _ptr(Ea), _ptr(F), _ptr(W))
        check_status(st)
        out = {"energy": E.value, "atomic_energies": Ea, "forces": F}
        if virial:
            out["virial"] = W
        return out

    def _types(self, symbols_or_types):
        a = np.asarray(symbols_or_types)
        if a.dtype.kind in "iu":
            return _i32(a)
        return self.type_ids([str(s) for s in a])
