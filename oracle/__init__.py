"""FP64 CPU oracle for aenet's energy-and-force path -- TEST INFRASTRUCTURE.

Only the test suite, ``__graft_entry__.smoke()`` and the benchmark's CPU
baseline leg import this package, and only to check or time against: the
product library never loads it.  The numerics live in ``aenet_oracle.c`` (a plain-C
restatement of the reference Fortran, built by ``oracle/build.py``); this
module is a thin ctypes front end.

Conventions: ``cell`` is a (3, 3) array whose rows are the lattice vectors
(the same memory layout as the reference's column-major ``latticeVec``);
coordinates are (N, 3) Cartesian in Angstrom; ``types`` are 1-based global
type ids in the order the species were passed to :meth:`Oracle.load`.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build
from .nnfile import parse_nn

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        lib = C.CDLL(path)
        vp = C.c_void_p
        lib.orc_init.argtypes = [C.c_int]
        lib.orc_set_network.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_int]
        lib.orc_set_setup.argtypes = [C.c_int, C.c_int, C.c_int, _ip, C.c_double,
                                      C.c_double, C.c_int, _ip, _dp, _ip, _dp, _dp,
                                      _dp, vp, C.c_int]
        lib.orc_set_energy.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
        lib.orc_finalize.argtypes = [C.c_int]
        lib.orc_Rc_min.restype = C.c_double
        lib.orc_Rc_max.restype = C.c_double
        lib.orc_descriptor.argtypes = [_dp, C.c_int, C.c_int, _dp, _ip, C.c_int,
                                       _dp, vp, vp]
        lib.orc_stp_stats.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        lib.orc_atomic_energy.argtypes = [_dp, C.c_int, C.c_int, _dp, _ip,
                                          C.POINTER(C.c_double)]
        lib.orc_atomic_energy_and_forces.argtypes = [
            _dp, C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, C.c_int,
            C.POINTER(C.c_double), _dp]
        lib.orc_atomic_energy_wgrad.argtypes = [_dp, C.c_int, C.c_int, _dp, _ip,
                                                C.POINTER(C.c_double), _dp]
        lib.orc_nbl_init.argtypes = [_dp, C.c_int, _ip, _dp, C.c_int, C.c_double,
                                     C.c_double]
        lib.orc_nbl_neighbors.argtypes = [C.c_int, C.c_int, _dp, _dp, _ip, _ip,
                                          C.c_double]
        lib.orc_nbl_wrapped.argtypes = [_dp]
        lib.orc_cart_to_latt.argtypes = [_dp, C.c_int, _dp, _dp]
        lib.orc_bounding_box.argtypes = [C.c_int, _dp, _dp]
        lib.orc_structure_energy_forces.argtypes = [
            _dp, C.c_int, _dp, _ip, C.c_int, C.c_int, C.c_int,
            C.POINTER(C.c_double), C.POINTER(C.c_double), vp, vp]
        lib.orc_set_complete_candidates.argtypes = [C.c_int]
        lib.orc_sfb_init.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
        lib.orc_sfb_eval.argtypes = [C.c_int, _dp, C.c_int, _ip, _dp, C.c_int, _dp,
                                     vp, vp]
        lib.orc_sfb_reconstruct_radial.argtypes = [_dp, C.c_int, _dp, _dp]
        _LIB = lib
    return _LIB


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleError(RuntimeError):
    pass


class Oracle:
    """Single-instance oracle, like the reference library (module globals)."""

    def __init__(self):
        self.lib = _lib()
        self.types = []
        self.loaded = False

    # -------------------------------------------------------------- setup
    def load(self, types, potentials, angular="current", normalizer="auto"):
        """Load one potential per species.

        ``potentials`` maps species name to a ``.nn`` path or to the dict
        returned by :func:`oracle.nnfile.parse_nn`.
        """
        lib = self.lib
        lib.orc_final()
        self.types = list(types)
        self._check(lib.orc_init(len(types)))
        self.pots = {}
        for it, name in enumerate(types, start=1):
            pot = potentials[name]
            if isinstance(pot, (str, os.PathLike)):
                pot = parse_nn(pot)
            self.pots[name] = pot
            net, stp, ts = pot["net"], pot["stp"], pot["ts"]
            self._check(lib.orc_set_network(
                it, int(net["nlayers"]), _i32(net["nnodes"]), _i32(net["f_a"]),
                _f64(net["W"]), int(net["Wsize"])))
            env_global = _i32([self.types.index(e) + 1 if e in self.types else 0
                               for e in stp["envtypes"]])
            sftype = {"chebyshev": 1, "behler2011": 2}[stp["sftype"].lower()]
            legacy = stp["sfval_cov"] is None
            norm = {"auto": int(legacy), "current": 0, "legacy": 1}[normalizer]
            cov = None if stp["sfval_cov"] is None else _f64(stp["sfval_cov"])
            sfparam = np.zeros((stp["nsf"], 4))
            sfparam[:, :stp["sfparam"].shape[1]] = stp["sfparam"]
            sfenv = np.zeros((stp["nsf"], 2), dtype=np.int32)
            sfenv[:, :stp["sfenv"].shape[1]] = stp["sfenv"]
            self._check(lib.orc_set_setup(
                it, sftype, int(stp["nenv"]), env_global, stp["Rc_min"],
                stp["Rc_max"], int(stp["nsf"]), _i32(stp["sf"]), _f64(sfparam),
                _i32(sfenv), _f64(stp["sfval_min"]), _f64(stp["sfval_max"]),
                _f64(stp["sfval_avg"]), _ptr(cov), norm))
            k = ts["typeName"].index(stp["atomtype"])
            self._check(lib.orc_set_energy(it, ts["scale"], ts["shift"],
                                           float(ts["E_atom"][k])))
        self._check(lib.orc_finalize(1 if angular == "legacy" else 0))
        self.loaded = True
        self.Rc_min = lib.orc_Rc_min()
        self.Rc_max = lib.orc_Rc_max()
        self.nnb_max = lib.orc_nnb_max()
        self.nsf_max = lib.orc_nsf_max()

    def set_candidates(self, mode):
        """"complete" (default): every atom/image within the cut-off;
        "cells": the linked-cell candidate search of lclist.f90 as written."""
        self.lib.orc_set_complete_candidates(1 if mode == "complete" else 0)

    def E_atom(self, name):
        pot = self.pots[name]
        ts = pot["ts"]
        return float(ts["E_atom"][ts["typeName"].index(pot["stp"]["atomtype"])])

    @staticmethod
    def _check(st):
        if st != 0:
            raise OracleError("oracle status %d" % st)

    # ---------------------------------------------------------- per atom
    def descriptor(self, coo_i, type_i, coo_j, type_j, scaled=True, deriv=False):
        coo_j = _f64(np.asarray(coo_j).reshape(-1, 3))
        n = coo_j.shape[0]
        nsf = self.lib.orc_nsf(type_i)
        G = np.zeros(nsf)
        di = np.zeros((nsf, 3)) if deriv else None
        dj = np.zeros((max(n, 1), nsf, 3)) if deriv else None
        self._check(self.lib.orc_descriptor(_f64(coo_i), type_i, n, coo_j,
                                            _i32(type_j), int(scaled), G,
                                            _ptr(di), _ptr(dj)))
        if deriv:
            return G, di, dj[:n]
        return G

    def atomic_energy(self, coo_i, type_i, coo_j, type_j):
        coo_j = _f64(np.asarray(coo_j).reshape(-1, 3))
        E = C.c_double()
        self._check(self.lib.orc_atomic_energy(_f64(coo_i), type_i, coo_j.shape[0],
                                               coo_j, _i32(type_j), C.byref(E)))
        return E.value

    def atomic_energy_and_forces(self, coo_i, type_i, index_i, coo_j, type_j,
                                 index_j, F):
        coo_j = _f64(np.asarray(coo_j).reshape(-1, 3))
        E = C.c_double()
        assert F.dtype == np.float64 and F.flags.c_contiguous
        self._check(self.lib.orc_atomic_energy_and_forces(
            _f64(coo_i), type_i, index_i, coo_j.shape[0], coo_j, _i32(type_j),
            _i32(index_j), F.shape[0], C.byref(E), F))
        return E.value

    def atomic_energy_wgrad(self, coo_i, type_i, coo_j, type_j):
        coo_j = _f64(np.asarray(coo_j).reshape(-1, 3))
        name = self.types[type_i - 1]
        nw = int(self.pots[name]["net"]["Wsize"])
        g = np.zeros(nw)
        E = C.c_double()
        self._check(self.lib.orc_atomic_energy_wgrad(
            _f64(coo_i), type_i, coo_j.shape[0], coo_j, _i32(type_j), C.byref(E), g))
        return E.value, g

    # -------------------------------------------------------- structures
    def cart_to_latt(self, cell, cart):
        cart = _f64(cart)
        out = np.zeros_like(cart)
        self.lib.orc_cart_to_latt(_f64(cell), cart.shape[0], cart, out)
        return out

    def neighbors(self, cell, cart, types, pbc=True, Rc=None, atoms=None):
        """Per-atom neighbour lists of lcl_nbdist_cart (predict.x order).

        Returns the wrapped lattice coordinates, the Cartesian centre
        positions and a list of (nbcoo, nbdist, nblist, nbtype) per atom
        (nblist 1-based).  ``atoms`` (0-based ids) restricts the queries;
        the list then holds entries only for those atoms, in that order.
        """
        cart = _f64(cart).copy()
        cell = _f64(cell)
        if not pbc:
            box = np.zeros(9)
            self.lib.orc_bounding_box(cart.shape[0], cart, box)
            cell = box.reshape(3, 3)
        latt = self.cart_to_latt(cell, cart)
        n = cart.shape[0]
        self._check(self.lib.orc_nbl_init(cell, n, _i32(types), latt, int(pbc),
                                          self.Rc_min, self.Rc_max))
        self.lib.orc_nbl_wrapped(latt)
        Rc = self.Rc_max if Rc is None else Rc
        cap = max(self.nnb_max, 64)
        out = []
        for i in ((np.arange(n) + 1) if atoms is None else (np.asarray(atoms) + 1)):
            i = int(i)
            while True:
                nbcoo = np.zeros((cap, 3)); nbdist = np.zeros(cap)
                nbl = np.zeros(cap, dtype=np.int32); nbt = np.zeros(cap, dtype=np.int32)
                nnb = self.lib.orc_nbl_neighbors(i, cap, nbcoo, nbdist, nbl, nbt, Rc)
                if nnb >= 0:
                    break
                cap *= 2
            out.append((nbcoo[:nnb].copy(), nbdist[:nnb].copy(), nbl[:nnb].copy(),
                        nbt[:nnb].copy()))
        self.lib.orc_nbl_final()
        centres = latt @ cell
        return latt, centres, out

    def structure(self, cell, cart, types, pbc=True, forces=True, nthreads=1,
                  atom_limit=0):
        """predict.x get_energy: returns (Ecoh, Etot, F or None, E_atoms)."""
        cart = _f64(cart)
        n = cart.shape[0]
        cell = _f64(np.zeros((3, 3)) if cell is None else cell)
        F = np.zeros((n, 3)) if forces else None
        Ea = np.zeros(n)
        ec, et = C.c_double(), C.c_double()
        self._check(self.lib.orc_structure_energy_forces(
            cell, n, cart, _i32(types), int(pbc), int(nthreads), int(atom_limit),
            C.byref(ec), C.byref(et), _ptr(F), _ptr(Ea)))
        return ec.value, et.value, F, Ea

    # ----------------------------------------------------------- helpers
    def stp_stats(self, vecs):
        vecs = _f64(vecs)
        nvec, nsf = vecs.shape
        mn, mx, av, cv = (np.zeros(nsf) for _ in range(4))
        self.lib.orc_stp_stats(nsf, nvec, vecs, mn, mx, av, cv)
        return mn, mx, av, cv

    def close(self):
        self.lib.orc_final()
        self.loaded = False
