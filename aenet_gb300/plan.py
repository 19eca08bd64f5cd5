"""Device-resident evaluation plans over torch tensors, and the autograd
function that turns the adjoint kernels into a backward pass.

A :class:`Plan` fixes a batch layout (structure sizes, lattices, pbc) and
owns the device workspace inside libaenet_gb300.so; every run reads
positions from and writes results into CUDA tensors on the current torch
stream without allocating, so runs can be captured in CUDA graphs.
PyTorch provides only the tensors, the stream and autograd.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from .core import FP64, MIXED, check_status

FORCES = 1
VIRIAL = 2

LOSS_ENERGY = 1
LOSS_ENERGY_FORCES = 2

ST_NB_OVERFLOW = 1
ST_BAD_COORD = 2
ST_BAD_TYPE = 4
ST_CELL_OVERFLOW = 8
ST_TC_TIMEOUT = 16


class PlanStatusError(RuntimeError):
    pass


def _ntypes():
    return _lib.ntypes()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class _DeviceArray:
    """Zero-copy view of library-owned device memory for torch.as_tensor."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}


class Plan:
    def __init__(self, natoms, cells=None, pbc=None, precision=MIXED, coords0=None):
        lib = _lib.lib()
        self.natoms_per = np.ascontiguousarray(natoms, dtype=np.int32).reshape(-1)
        self.nstruc = int(self.natoms_per.size)
        self.precision = precision
        pbc = np.ones(self.nstruc, dtype=np.int32) if pbc is None else np.ascontiguousarray(
            np.asarray(pbc, dtype=np.int32).reshape(-1))
        self.pbc = pbc
        lat = None
        if cells is not None:
            lat = np.ascontiguousarray(np.asarray(cells, dtype=np.float64).reshape(self.nstruc, 9))
        c0 = None if coords0 is None else np.ascontiguousarray(
            np.asarray(coords0, dtype=np.float64).reshape(-1, 3))
        stat = C.c_int(0)
        self._h = lib.aenet_gpu_plan_create(
            self.nstruc, self.natoms_per.ctypes.data_as(C.c_void_p),
            None if lat is None else lat.ctypes.data_as(C.c_void_p),
            pbc.ctypes.data_as(C.c_void_p),
            None if c0 is None else c0.ctypes.data_as(C.c_void_p), int(precision), C.byref(stat))
        check_status(stat.value)
        if not self._h:
            raise PlanStatusError("plan creation failed")
        self.natoms = lib.aenet_gpu_plan_natoms(self._h)
        self.generation = 0
        dev = torch.device("cuda")
        self.atom_struct = torch.repeat_interleave(
            torch.arange(self.nstruc, device=dev), torch.as_tensor(self.natoms_per, device=dev).long())

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().aenet_gpu_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cells(self, cells):
        lat = np.ascontiguousarray(np.asarray(cells, dtype=np.float64).reshape(self.nstruc, 9))
        check_status(_lib.lib().aenet_gpu_plan_set_lattices(self._h, lat.ctypes.data_as(C.c_void_p)))

    @staticmethod
    def _check_inputs(pos, types):
        if not (pos.is_cuda and pos.dtype == torch.float64 and pos.is_contiguous()):
            raise TypeError("positions must be a contiguous float64 CUDA tensor (N, 3)")
        if not (types.is_cuda and types.dtype == torch.int32 and types.is_contiguous()):
            raise TypeError("types must be a contiguous int32 CUDA tensor (1-based)")

    def run(self, pos, types, forces=True, virial=False, atomic=False, out=None):
        """One full pass; returns a dict of CUDA tensors (E, F, virial,
        E_atoms).  ``out`` may provide preallocated tensors (graph capture)."""
        self._check_inputs(pos, types)
        dev = pos.device
        out = {} if out is None else out
        E = out.get("E")
        if E is None:
            E = out["E"] = torch.empty(self.nstruc, dtype=torch.float64, device=dev)
        F = out.get("F") if forces else None
        if forces and F is None:
            F = out["F"] = torch.empty((self.natoms, 3), dtype=torch.float64, device=dev)
        W = out.get("virial") if virial else None
        if virial and W is None:
            W = out["virial"] = torch.empty((self.nstruc, 3, 3), dtype=torch.float64, device=dev)
        Ea = out.get("E_atoms") if atomic else None
        if atomic and Ea is None:
            Ea = out["E_atoms"] = torch.empty(self.natoms, dtype=torch.float64, device=dev)
        flags = (FORCES if forces else 0) | (VIRIAL if virial else 0)
        st = _lib.lib().aenet_gpu_plan_run(self._h, _p(pos), _p(types), _p(E), _p(Ea), _p(F),
                                           _p(W), flags, _stream())
        check_status(st)
        self.generation += 1
        return out

    def forward(self, pos, types, E=None, E_atoms=None):
        self._check_inputs(pos, types)
        if E is None:
            E = torch.empty(self.nstruc, dtype=torch.float64, device=pos.device)
        st = _lib.lib().aenet_gpu_plan_forward(self._h, _p(pos), _p(types), _p(E), _p(E_atoms),
                                               _stream())
        check_status(st)
        self.generation += 1
        return E

    def backward(self, weights=None, grad=None, virial=None):
        """grad[i] = sum_s w_s dE_s/dR_i of the last forward."""
        dev = torch.device("cuda")
        if grad is None:
            grad = torch.empty((self.natoms, 3), dtype=torch.float64, device=dev)
        if weights is not None:
            weights = weights.to(dtype=torch.float64).contiguous()
        st = _lib.lib().aenet_gpu_plan_backward(self._h, _p(weights), _p(grad), _p(virial),
                                                _stream())
        check_status(st)
        return grad

    def loss_gradient(self, pos, types, E_target, F_target=None, mode=None, w_E=1.0, w_F=0.1,
                      grad=None, loss=None, E=None, F=None):
        """Loss of the batch and its gradient with respect to every network
        weight (flattened like :func:`aenet_gb300.core.ANNPotentials.get_weights`).

        mode LOSS_ENERGY: the reference's energy loss (train.f90:799-889);
        mode LOSS_ENERGY_FORCES: w_E sum (E-E_t)^2/N^2 + w_F sum |F-F_t|^2.
        Returns (loss[1], grad) as CUDA float64 tensors."""
        self._check_inputs(pos, types)
        dev = pos.device
        lib = _lib.lib()
        if mode is None:
            mode = LOSS_ENERGY_FORCES if F_target is not None else LOSS_ENERGY
        if grad is None:
            nw = sum(lib.aenet_gpu_network_nweights(t) for t in range(1, _ntypes() + 1))
            grad = torch.empty(nw, dtype=torch.float64, device=dev)
        if loss is None:
            loss = torch.empty(1, dtype=torch.float64, device=dev)
        E_target = E_target.to(device=dev, dtype=torch.float64).contiguous()
        if F_target is not None:
            F_target = F_target.to(device=dev, dtype=torch.float64).contiguous()
        st = lib.aenet_gpu_plan_loss_gradient(self._h, _p(pos), _p(types), _p(E_target),
                                              _p(F_target), int(mode), float(w_E), float(w_F),
                                              _p(loss), _p(grad), _p(E), _p(F), _stream())
        check_status(st)
        self.generation += 1
        return loss, grad

    STAGES = ("types", "neighbours", "descriptor", "networks", "energy_reduce", "adjoint",
              "forces_out", "neighbour_search")

    def profile(self, pos, types, E=None, F=None):
        """Stage durations (ms) of one full pass, CUDA events on the stream."""
        self._check_inputs(pos, types)
        ms = (C.c_float * 8)()
        check_status(_lib.lib().aenet_gpu_plan_profile(self._h, _p(pos), _p(types), _p(E), _p(F),
                                                       ms, _stream()))
        self.generation += 1
        return dict(zip(self.STAGES, [float(x) for x in ms]))

    def status(self):
        return int(_lib.lib().aenet_gpu_plan_status(self._h, _stream()))

    def check(self):
        st = self.status()
        if st:
            names = [n for b, n in ((ST_NB_OVERFLOW, "neighbour capacity overflow"),
                                    (ST_BAD_COORD, "non-finite coordinate"),
                                    (ST_BAD_TYPE, "invalid type id"),
                                    (ST_CELL_OVERFLOW, "cell capacity overflow"),
                                    (ST_TC_TIMEOUT, "tensor-core wait timed out")) if st & b]
            raise PlanStatusError("plan status %d: %s" % (st, ", ".join(names)))

    def neighbors(self):
        """(cap, counts[N], packed index|species<<26 [N, cap], vectors
        [N, cap, 4]) as zero-copy CUDA tensors of the last run."""
        cap = C.c_int(0)
        pc, pj, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check_status(_lib.lib().aenet_gpu_plan_neighbors(self._h, C.byref(cap), C.byref(pc),
                                                         C.byref(pj), C.byref(pv)))
        n, c = self.natoms, cap.value
        cnt = torch.as_tensor(_DeviceArray(pc.value, (n,), "<i4"), device="cuda")
        jt = torch.as_tensor(_DeviceArray(pj.value, (n, c), "<i4"), device="cuda")
        vt = "<f8" if self.precision == FP64 else "<f4"
        vec = torch.as_tensor(_DeviceArray(pv.value, (n, c, 4), vt), device="cuda")
        return c, cnt, jt, vec

    def jacobian(self, atom0=0, count=None, nsf_max=None):
        """Raw FP64 descriptor Jacobians of atoms [atom0, atom0 + count) from
        the neighbour table of the last run (FP64 plans, Chebyshev or Behler):
        (dG/dR_i [count, nsf_max, 3], dG/dR_j [count, cap, nsf_max, 3],
        neighbour atom indices [count, cap], neighbour counts [count]) as
        CUDA tensors (aenet_gpu_plan_descriptor_jacobian)."""
        lib = _lib.lib()
        count = self.natoms - atom0 if count is None else count
        if nsf_max is None:
            nsf_max = C.c_int.in_dll(lib, "aenet_nsf_max").value
        cap = lib.aenet_gpu_plan_neighbour_capacity(self._h)
        dev = torch.device("cuda")
        Ji = torch.empty((count, nsf_max, 3), dtype=torch.float64, device=dev)
        Jj = torch.empty((count, cap, nsf_max, 3), dtype=torch.float64, device=dev)
        nbl = torch.empty((count, cap), dtype=torch.int32, device=dev)
        nnb = torch.empty((count,), dtype=torch.int32, device=dev)
        check_status(lib.aenet_gpu_plan_descriptor_jacobian(self._h, int(atom0), int(count), _p(Ji),
                                                            _p(Jj), _p(nbl), _p(nnb), _stream()))
        return Ji, Jj, nbl, nnb

    def descriptors(self):
        pg = C.c_void_p()
        pad = C.c_int(0)
        check_status(_lib.lib().aenet_gpu_plan_descriptors(self._h, C.byref(pg), C.byref(pad)))
        vt = "<f8" if self.precision == FP64 else "<f4"
        return torch.as_tensor(_DeviceArray(pg.value, (self.natoms, pad.value), vt), device="cuda")


class PotentialEnergy(torch.autograd.Function):
    """E_s(R) per structure; backward runs the adjoint kernels.

    The descriptor Jacobian is never stored: the backward pass recomputes
    the descriptor partials from the neighbour table kept by the forward.
    """

    @staticmethod
    def forward(ctx, positions, plan, types):
        E = plan.forward(positions.detach().contiguous(), types)
        ctx.plan = plan
        ctx.generation = plan.generation
        return E

    @staticmethod
    def backward(ctx, gE):
        plan = ctx.plan
        if plan.generation != ctx.generation:
            raise RuntimeError("the plan ran again between forward and backward")
        grad = plan.backward(gE.detach())
        return grad, None, None


def potential_energy(positions, plan, types):
    """Differentiable per-structure energies (autograd over positions)."""
    return PotentialEnergy.apply(positions, plan, types)
