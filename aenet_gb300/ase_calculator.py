"""ASE calculator backed by the GPU evaluator.

Same class name, constructor and properties as the reference's
python3/aenet/ase_calculator.py:26-123 (``ANNCalculator(potentials)``
with ``energy`` and ``forces``), plus ``stress``.  The reference builds an
ASE NeighborList and calls the library once per atom; here the whole
structure goes to the GPU in one call (neighbour search included).

When ASE is importable the class derives from ``ase.calculators.calculator
.Calculator``; otherwise it is a small stand-alone class with the same
methods (``calculate``, ``get_potential_energy``, ``get_forces``,
``get_stress``) working on any object that provides ``get_positions()``,
``get_chemical_symbols()``, ``get_cell()`` and ``get_pbc()``.

Periodicity must be all three directions or none (isolated structures).
"""
import numpy as np

from .core import ANNPotentials, MIXED

try:  # pragma: no cover - ASE is optional
    from ase.calculators.calculator import Calculator as _Base
    from ase.calculators.calculator import all_changes as _all_changes
    HAVE_ASE = True
except ImportError:
    HAVE_ASE = False
    _all_changes = ["positions", "numbers", "cell", "pbc"]

    class _Base:
        """Minimal stand-in for ase.calculators.calculator.Calculator."""

        def __init__(self, **kwargs):
            self.atoms = None
            self.results = {}
            self.parameters = dict(kwargs)

        def _changes(self, atoms):
            if self.atoms is None:
                return list(_all_changes)
            ch = []
            if not np.array_equal(self.atoms["positions"], atoms.get_positions()):
                ch.append("positions")
            if list(self.atoms["symbols"]) != list(atoms.get_chemical_symbols()):
                ch.append("numbers")
            if not np.array_equal(self.atoms["cell"], np.asarray(atoms.get_cell())):
                ch.append("cell")
            if not np.array_equal(self.atoms["pbc"], np.asarray(atoms.get_pbc())):
                ch.append("pbc")
            return ch

        def calculate(self, atoms=None, properties=("energy",), system_changes=None):
            if atoms is not None:
                self.atoms = {"positions": np.array(atoms.get_positions(), dtype=np.float64),
                              "symbols": list(atoms.get_chemical_symbols()),
                              "cell": np.array(atoms.get_cell(), dtype=np.float64),
                              "pbc": np.array(atoms.get_pbc(), dtype=bool)}

        def get_property(self, name, atoms):
            changes = self._changes(atoms)
            if changes or name not in self.results:
                self.results = {}
                self.calculate(atoms, [name], changes)
            return self.results[name]

        def get_potential_energy(self, atoms=None, force_consistent=False):
            return self.get_property("energy", atoms)

        def get_forces(self, atoms=None):
            return self.get_property("forces", atoms).copy()

        def get_stress(self, atoms=None):
            return self.get_property("stress", atoms).copy()


class ANNCalculator(_Base):
    implemented_properties = ["energy", "forces", "stress"]

    def __init__(self, potentials, precision=MIXED, **kwargs):
        _Base.__init__(self, **kwargs)
        self.ann = ANNPotentials(potentials)
        self.cutoff = self.ann.Rc_max
        self.precision = precision
        self.results = {}

    def release(self):
        self.ann.release()

    def _state(self, atoms):
        if HAVE_ASE:
            a = self.atoms
            return (a.get_positions(), a.get_chemical_symbols(), np.asarray(a.get_cell()),
                    np.asarray(a.get_pbc()))
        a = self.atoms
        return a["positions"], a["symbols"], a["cell"], a["pbc"]

    def calculate(self, atoms=None, properties=("energy",), system_changes=_all_changes):
        _Base.calculate(self, atoms, properties, system_changes)
        pos, symbols, cell, pbc = self._state(atoms)
        pbc = np.asarray(pbc, dtype=bool).reshape(-1)
        if pbc.any() and not pbc.all():
            raise NotImplementedError("mixed periodicity (periodic in some directions only)")
        periodic = bool(pbc.all())
        want_stress = "stress" in properties and periodic
        r = self.ann.structure_energy_forces(pos, symbols, cell if periodic else None,
                                             pbc=periodic, precision=self.precision,
                                             virial=want_stress)
        self.results["energy"] = float(r["energy"])
        self.results["free_energy"] = float(r["energy"])
        self.results["forces"] = np.array(r["forces"])
        if "stress" in properties:
            if not periodic:
                raise NotImplementedError("stress of a non-periodic structure")
            W = np.asarray(r["virial"]).reshape(3, 3)
            vol = abs(np.linalg.det(np.asarray(cell, dtype=np.float64)))
            s = -0.5 * (W + W.T) / vol   # sigma = -W / V, Voigt xx yy zz yz xz xy
            self.results["stress"] = np.array([s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2],
                                               s[0, 1]])
