"""ANNCalculator (the reference's ase_calculator.py surface) on the GPU,
against the FP64 oracle; works without ASE through a duck-typed Atoms."""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu


class _Atoms:
    """The four Atoms methods the calculator reads."""

    def __init__(self, positions, symbols, cell, pbc=True):
        self.positions = np.array(positions, dtype=np.float64)
        self.symbols = list(symbols)
        self.cell = np.array(cell, dtype=np.float64)
        self.pbc = np.array([pbc] * 3)

    def get_positions(self):
        return self.positions.copy()

    def get_chemical_symbols(self):
        return list(self.symbols)

    def get_cell(self):
        return self.cell.copy()

    def get_pbc(self):
        return self.pbc.copy()


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def test_ann_calculator_energy_forces_stress(cuda, oracle, tmp_path):
    from aenet_gb300 import workloads
    from aenet_gb300.ase_calculator import ANNCalculator
    from aenet_gb300.core import FP64
    w = workloads.aucu_fcc_4000()
    s = w.structures[0]
    keep = np.all(workloads.fcc_positions(10, 3.90)[0] < 4 * 3.90 - 0.1, axis=1)
    pos, typ = s.positions[keep], s.types[keep]
    cell = np.eye(3) * 4 * 3.90
    sub = workloads.Workload(w.name, w.types, w.setups, w.arch,
                             [workloads.Structure(pos, typ, cell)], w.seed)
    sub.networks = w.networks
    paths = helpers.make_potentials(oracle, sub, str(tmp_path))
    symbols = [w.types[t - 1] for t in typ]
    calc = ANNCalculator({t: paths[t] for t in w.types}, precision=FP64)
    try:
        atoms = _Atoms(pos, symbols, cell)
        E = calc.get_potential_energy(atoms)
        F = calc.get_forces(atoms)
        S = calc.get_stress(atoms)
        # unchanged atoms: cached results
        assert calc.get_potential_energy(atoms) == E
        # stress against a strain derivative of the energy
        h = 1e-5
        eps = np.zeros((3, 3))
        eps[0, 1] = eps[1, 0] = h
        ep = calc.get_potential_energy(_Atoms(pos @ (np.eye(3) + eps), symbols,
                                              cell @ (np.eye(3) + eps)))
        em = calc.get_potential_energy(_Atoms(pos @ (np.eye(3) - eps), symbols,
                                              cell @ (np.eye(3) - eps)))
        vol = abs(np.linalg.det(cell))
        # dE/d(eps_xy + eps_yx) = V (sigma_xy + sigma_yx) = 2 V sigma_xy
        assert abs((ep - em) / (2 * h) - 2 * vol * S[5]) < 1e-6 * max(1.0, abs(ep - em) / h)
    finally:
        calc.release()
    oracle.load(w.types, paths)
    _, et, Fo, _ = oracle.structure(cell, pos, typ)
    assert abs(E - et) / len(pos) < 1e-10
    assert np.abs(F - Fo).max() < 1e-9
