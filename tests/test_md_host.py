"""Host-side MD logic (no GPU): Maxwell-Boltzmann velocities and units."""
import numpy as np

from aenet_gb300.md import KB, MASS_UNIT, maxwell_boltzmann


def test_mass_unit_is_amu_angstrom2_per_fs2_in_ev():
    # 1 amu (1 A/fs)^2 = 1.66053906660e-27 kg * 1e10 m^2/s^2
    assert abs(MASS_UNIT - 103.6426965) < 1e-6


def test_maxwell_boltzmann_temperature_and_momentum():
    rng = np.random.default_rng(5)
    m = np.where(np.arange(200000) % 4 == 0, 196.96657, 63.546)
    v = maxwell_boltzmann(m, 600.0, rng)
    p = (m[:, None] * v).sum(0)
    assert np.abs(p).max() < 1e-9 * np.abs(m[:, None] * v).sum()
    ekin = 0.5 * (m[:, None] * v * v).sum() * MASS_UNIT
    T = ekin / len(m) / (1.5 * KB)
    assert abs(T - 600.0) < 6.0
