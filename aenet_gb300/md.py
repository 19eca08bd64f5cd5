"""Molecular dynamics with the GPU evaluator, without ASE.

Mirrors python3/scripts/aenet-md.py (Maxwell-Boltzmann velocities, NVE
velocity Verlet, the "step E_pot E_kin T E_tot" log of printenergy,
aenet-md.py:45-51) with the whole integration on the GPU
(``aenet_gpu_md_*``): a step is kick-drift, neighbour refresh (or rebuild
past the skin), descriptors, networks, forces and the second kick, with
no host round trip besides the one-word skin check.

Units: A, fs, amu, eV.
"""
import ctypes as C
import sys

import numpy as np

from . import _lib
from .core import MIXED, check_status

KB = 8.617333262e-5                                   # eV / K
MASS_UNIT = 1.66053906660e-27 * 1e10 / 1.602176634e-19  # amu A^2/fs^2 in eV

__all__ = ["MolecularDynamics", "maxwell_boltzmann", "KB", "MASS_UNIT"]


def maxwell_boltzmann(masses, temperature, rng, remove_com=True):
    """Velocities (A/fs) drawn at ``temperature`` (K) for per-atom masses
    (amu), centre-of-mass motion removed."""
    m = np.asarray(masses, dtype=np.float64)
    v = rng.normal(0.0, 1.0, (m.size, 3)) * np.sqrt(KB * temperature / (m * MASS_UNIT))[:, None]
    if remove_com:
        v -= (m[:, None] * v).sum(0) / m.sum()
    return v


class MolecularDynamics:
    """NVE velocity-Verlet run of one periodic structure.

    ``potentials`` is a loaded :class:`aenet_gb300.core.ANNPotentials`;
    ``types`` are 1-based type ids; ``masses`` maps species to amu.
    """

    def __init__(self, potentials, positions, types, cell, velocities=None, masses=None,
                 dt=2.0, skin=0.3, precision=MIXED):
        from .workloads import MASSES
        self.pot = potentials
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        self.n = pos.shape[0]
        self.types = np.ascontiguousarray(types, dtype=np.int32).reshape(-1)
        masses = masses or {t: MASSES[t] for t in potentials.atom_types}
        self.mass_by_type = np.array([masses[t] for t in potentials.atom_types], dtype=np.float64)
        self.masses = self.mass_by_type[self.types - 1]
        lat = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64)
        self.dt, self.skin = float(dt), float(skin)
        stat = C.c_int(0)
        self._h = _lib.lib().aenet_gpu_md_create(
            self.n, lat.ctypes.data_as(C.c_void_p), pos.ctypes.data_as(C.c_void_p),
            None if vel is None else vel.ctypes.data_as(C.c_void_p),
            self.types.ctypes.data_as(C.c_void_p), self.mass_by_type.ctypes.data_as(C.c_void_p),
            self.dt, self.skin, int(precision), C.byref(stat))
        check_status(stat.value)
        self.E_pot, self.E_kin = self._energies()

    def _energies(self):
        ep, ek = C.c_double(), C.c_double()
        check_status(_lib.lib().aenet_gpu_md_run(self._h, 0, C.byref(ep), C.byref(ek)))
        return ep.value, ek.value

    def run(self, steps):
        """Advance ``steps`` steps; returns (E_pot, E_kin) after the last."""
        ep, ek = C.c_double(), C.c_double()
        check_status(_lib.lib().aenet_gpu_md_run(self._h, int(steps), C.byref(ep), C.byref(ek)))
        self.E_pot, self.E_kin = ep.value, ek.value
        return self.E_pot, self.E_kin

    def temperature(self):
        return self.E_kin / self.n / (1.5 * KB)

    def state(self):
        """(positions, velocities, forces) as host arrays."""
        r, v, f = (np.empty((self.n, 3)) for _ in range(3))
        check_status(_lib.lib().aenet_gpu_md_get(self._h, r.ctypes.data_as(C.c_void_p),
                                                 v.ctypes.data_as(C.c_void_p),
                                                 f.ctypes.data_as(C.c_void_p)))
        return r, v, f

    def phase_times(self):
        """Device time of the force part of the steps so far: (ms of steps
        that rebuilt the neighbour table, their count, ms of steps that
        refreshed the stored pair vectors, their count)."""
        bm, bs, rm, rs = C.c_double(), C.c_longlong(), C.c_double(), C.c_longlong()
        check_status(_lib.lib().aenet_gpu_md_phase_times(self._h, C.byref(bm), C.byref(bs),
                                                         C.byref(rm), C.byref(rs)))
        return bm.value, bs.value, rm.value, rs.value

    def counters(self):
        steps, builds = C.c_longlong(), C.c_int()
        check_status(_lib.lib().aenet_gpu_md_counters(self._h, C.byref(steps), C.byref(builds)))
        return steps.value, builds.value

    def energy_fp64(self):
        e = C.c_double()
        check_status(_lib.lib().aenet_gpu_md_energy_fp64(self._h, C.byref(e)))
        return e.value

    def printenergy(self, istep, out=sys.stdout):
        """aenet-md.py's log line: step, E_pot/atom, E_kin/atom, T, E_tot/atom."""
        epot, ekin = self.E_pot / self.n, self.E_kin / self.n
        out.write("{:5d} {:15.8e} {:15.8e} {:7.1f} {:15.8e}\n".format(
            istep, epot, ekin, ekin / (1.5 * KB), epot + ekin))

    def simulate(self, md_steps, print_steps, out=sys.stdout):
        """aenet-md.py's main loop: log, then md_steps/print_steps blocks."""
        out.write("# {:5s} {:15s} {:15s} {:7s} {:15s}\n".format("step", "E_pot", "E_kin", "T",
                                                                "E_tot"))
        self.printenergy(0, out)
        istep = 0
        for _ in range(int(md_steps / print_steps)):
            self.run(print_steps)
            istep += print_steps
            self.printenergy(istep, out)

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().aenet_gpu_md_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
