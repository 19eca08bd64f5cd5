"""Training of the network weights on the GPU.

Replaces the optimisation loop of train.x: per epoch, eval_next_structure
for every structure (src/train.f90:799-889) accumulates the loss and the
weight gradient, and opt_bfgs_weights (src/optimize.f90:1721-1771) takes one
L-BFGS-B step over the flattened weights of all species.  Here the loss and
gradient of the whole training set come from one GPU pass
(``aenet_gpu_plan_loss_gradient``: neighbours, descriptors, networks,
forces, descriptor tangents and weight gradients), and the optimiser is
L-BFGS with m = 20 correction pairs and no bounds, as opt_init_bfgs sets
up L-BFGS-B (src/optimize.f90:1600-1609), one iteration per epoch.  The
optimiser (aenet_gb300/lbfgs.py) runs on the host -- a vector of a few
thousand weights per step, negligible next to the GPU pass -- and saves
its state to a restart file after each epoch when asked, as train.x saves
`train.restart`; a run started with an existing restart file resumes from
it.  scipy's L-BFGS-B (the same algorithm as the reference's library) is
available as ``optimizer="scipy"``, without restarts.

Two losses (``mode``):
  LOSS_ENERGY         the reference's: sum_s dE_s^2/2 with
                      dE_s = (E_t,s - E_s)/(E_scale N_s);
  LOSS_ENERGY_FORCES  w_E sum_s (E_s - E_t,s)^2/N_s^2 + w_F sum_i |F_i - F_t,i|^2.
"""
import ctypes as C
import os
from types import SimpleNamespace

import numpy as np
import torch

from . import _lib
from .core import FP64, check_status
from .lbfgs import LBFGS
from .plan import LOSS_ENERGY, LOSS_ENERGY_FORCES, Plan, _p, _stream

__all__ = ["Trainer", "DescriptorTrainer", "LOSS_ENERGY", "LOSS_ENERGY_FORCES"]


class _Fit:
    """L-BFGS over all weights (opt_bfgs_weights, src/optimize.f90:1721-1771)."""

    def fit(self, maxiter=100, m=20, gtol=0.0, ftol=0.0, callback=None, restart=None,
            save_every=1, optimizer="lbfgs", nn_files=None):
        """``maxiter`` iterations (epochs) at most; stops early when the
        largest gradient component is at most ``gtol`` or the relative
        decrease of one iteration is at most ``ftol``.  ``restart``: path of
        the optimiser's state, resumed from when the file exists and written
        every ``save_every`` iterations; ``nn_files`` (species -> path): the
        potentials written at the same times and at the end, as train.x
        writes its .nn files.  Leaves the final weights loaded and returns
        (x, fun, jac, nit, nfev, success, message)."""
        if optimizer == "scipy":
            from scipy.optimize import minimize
            x0 = self.pot.get_weights()
            res = minimize(self.loss_and_grad, x0, jac=True, method="L-BFGS-B",
                           callback=callback, options={"maxcor": int(m), "maxiter": int(maxiter),
                                                       "gtol": gtol, "ftol": ftol})
            self.pot.set_weights(res.x)
            return res
        if restart is not None and os.path.exists(restart):
            opt = LBFGS.load(self.loss_and_grad, restart, m=m)
        else:
            opt = LBFGS(self.loss_and_grad, self.pot.get_weights(), m=m)
        message = "maximum number of iterations"
        success = True
        for _ in range(int(maxiter)):
            if np.abs(opt.g).max() <= gtol:
                message = "gradient below gtol"
                break
            f_old = opt.f
            if not opt.step():
                message, success = "no decrease along the search direction", False
                break
            if callback is not None:
                callback(opt.x)
            if opt.k % max(1, int(save_every)) == 0:
                if restart is not None:
                    opt.save(restart)
                self._save_nn(nn_files, opt.x)
            if ftol and f_old - opt.f <= ftol * max(abs(f_old), abs(opt.f), 1.0):
                message = "relative decrease below ftol"
                break
        if restart is not None:
            opt.save(restart)
        self.pot.set_weights(opt.x)
        self._save_nn(nn_files, opt.x)
        return SimpleNamespace(x=opt.x, fun=opt.f, jac=opt.g, nit=opt.k, nfev=opt.nfev,
                               success=success, message=message)


    def _save_nn(self, nn_files, x):
        if not nn_files:
            return
        self.pot.set_weights(x)
        for name, path in nn_files.items():
            self.pot.save_potential(name, path)


class Trainer(_Fit):
    """Loss, gradient and L-BFGS-B fit of the loaded potentials on a fixed
    training set held in device memory.

    ``structures``: sequence of (positions (N, 3), type ids (N,) 1-based,
    cell (3, 3) or None, pbc).  ``E_target``: total energies (eV) per
    structure; ``F_target``: forces (sum N, 3) in eV/A (LOSS_ENERGY_FORCES).
    """

    def __init__(self, potentials, structures, E_target, F_target=None, mode=None, w_E=1.0,
                 w_F=0.1, precision=FP64):
        self.pot = potentials
        structures = list(structures)
        natoms = [len(s[1]) for s in structures]
        cells = np.stack([np.eye(3) if s[2] is None else np.asarray(s[2], dtype=np.float64)
                          for s in structures])
        pbc = np.array([1 if s[3] else 0 for s in structures], dtype=np.int32)
        pos = np.concatenate([np.asarray(s[0], dtype=np.float64).reshape(-1, 3)
                              for s in structures])
        types = np.concatenate([np.asarray(s[1], dtype=np.int32) for s in structures])
        self.mode = mode if mode is not None else (
            LOSS_ENERGY_FORCES if F_target is not None else LOSS_ENERGY)
        self.w_E, self.w_F = float(w_E), float(w_F)
        self.plan = Plan(natoms, cells, pbc, precision=precision,
                         coords0=None if pbc.all() else pos)
        dev = torch.device("cuda")
        self.pos = torch.as_tensor(pos, device=dev).contiguous()
        self.types = torch.as_tensor(types, device=dev).contiguous()
        self.E_t = torch.as_tensor(np.asarray(E_target, dtype=np.float64), device=dev).contiguous()
        self.F_t = None if F_target is None else torch.as_tensor(
            np.asarray(F_target, dtype=np.float64).reshape(-1, 3), device=dev).contiguous()
        self.nw = potentials.nweights()
        self.grad = torch.empty(self.nw, dtype=torch.float64, device=dev)
        self.loss = torch.empty(1, dtype=torch.float64, device=dev)
        self.evaluations = 0

    def loss_and_grad(self, W=None):
        """(loss, gradient) at the weights W (the current ones if None)."""
        if W is not None:
            self.pot.set_weights(W)
        self.plan.loss_gradient(self.pos, self.types, self.E_t, self.F_t, mode=self.mode,
                                w_E=self.w_E, w_F=self.w_F, grad=self.grad, loss=self.loss)
        self.plan.check()
        self.evaluations += 1
        return float(self.loss.item()), self.grad.cpu().numpy().copy()

    def close(self):
        self.plan.close()


class DescriptorTrainer(_Fit):
    """train.x on a normalised training set (aenet training-set file): the
    reference's energy loss and gradient (eval_next_structure,
    src/train.f90:799-889) from the stored descriptors, on the GPU.

    ``ts`` is a normalised :class:`aenet_gb300.trainset.TrainSet`; its
    species names must be loaded in ``potentials``, whose energy scale and
    shift are those of the training set (as train.x writes them)."""

    def __init__(self, potentials, ts, precision=FP64):
        from .nnfile import read_nn
        if not ts.normalized:
            raise ValueError("normalise the training set first (trainset.normalize)")
        self.pot = potentials
        lib = _lib.lib()
        natoms = np.array([len(st["types"]) for st in ts.structures], dtype=np.int32)
        N = int(natoms.sum())
        ids = [potentials.get_type_id(n) for n in ts.type_names]
        types = np.concatenate([np.array([ids[t - 1] for t in st["types"]], dtype=np.int32)
                                for st in ts.structures])
        ld = max(len(v) for st in ts.structures for v in st["sfval"])
        G = np.zeros((N, ld))
        row = 0
        for st in ts.structures:
            for v in st["sfval"]:
                G[row, :len(v)] = v
                row += 1
        # totals in eV whose normalised cohesive part is the file's energy
        sc, sh, ea = {}, {}, {}
        for name in potentials.atom_types:
            _, _, tsi, _ = read_nn(potentials.potential_files[name])
            sc[name], sh[name] = 1.0 / tsi["scale"], tsi["shift"]
            ea[name] = potentials.free_atom_energy(name)
        names = potentials.atom_types
        E_t = np.array([st["energy"] * sc[names[0]] + len(st["types"]) * sh[names[0]] +
                        sum(ea[ts.type_names[t - 1]] for t in st["types"])
                        for st in ts.structures])
        self.plan = Plan(natoms, None, np.zeros(len(natoms), dtype=np.int32), precision=precision,
                         coords0=np.zeros((N, 3)))
        G = np.ascontiguousarray(G)
        check_status(lib.aenet_gpu_plan_load_descriptors(self.plan._h,
                                                         G.ctypes.data_as(C.c_void_p), ld))
        dev = torch.device("cuda")
        self.types = torch.as_tensor(types, device=dev).contiguous()
        self.E_t = torch.as_tensor(E_t, device=dev).contiguous()
        self.grad = torch.empty(potentials.nweights(), dtype=torch.float64, device=dev)
        self.loss = torch.empty(1, dtype=torch.float64, device=dev)
        self.E = torch.empty(len(natoms), dtype=torch.float64, device=dev)

    def loss_and_grad(self, W=None):
        if W is not None:
            self.pot.set_weights(W)
        check_status(_lib.lib().aenet_gpu_plan_descriptor_loss_gradient(
            self.plan._h, _p(self.types), _p(self.E_t), _p(self.loss), _p(self.grad),
            _p(self.E), _stream()))
        return float(self.loss.item()), self.grad.cpu().numpy().copy()

    def close(self):
        self.plan.close()
