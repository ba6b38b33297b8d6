"""ASE objects the calculator and the MD driver need.

When the ``ase`` package is importable its ``Atoms``, ``Calculator`` and
``all_changes`` are used unchanged, so the calculator is a real ASE
calculator.  Without it, a small stand-in with the same names, call
signatures and caching behaviour is provided (enough for
``atoms.calc = calc; atoms.get_potential_energy()``, ``get_forces``,
``get_stress``, velocities, kinetic energy and temperature).
"""
from typing import Dict, List, Optional

import numpy as np

from . import units

try:  # pragma: no cover - depends on the environment
    from ase import Atoms  # type: ignore
    from ase.calculators.calculator import Calculator, all_changes  # type: ignore
    HAVE_ASE = True
except ImportError:
    HAVE_ASE = False

    all_changes = ["positions", "numbers", "cell", "pbc", "initial_charges", "initial_magmoms"]

    class Calculator:
        """Minimal ase.calculators.calculator.Calculator: results cache keyed
        on the atoms' positions, numbers, cell and pbc."""

        implemented_properties: List[str] = []

        def __init__(self, **kwargs):
            self.parameters = dict(kwargs)
            self.results: Dict[str, object] = {}
            self.atoms: Optional["Atoms"] = None

        def reset(self):
            self.results = {}
            self.atoms = None

        def check_state(self, atoms: "Atoms", tol: float = 1e-15) -> List[str]:
            if self.atoms is None:
                return list(all_changes)
            changes = []
            if len(atoms) != len(self.atoms) or not np.allclose(atoms.positions, self.atoms.positions,
                                                                 rtol=0, atol=tol):
                changes.append("positions")
            if len(atoms) != len(self.atoms) or not np.array_equal(atoms.numbers, self.atoms.numbers):
                changes.append("numbers")
            if not np.allclose(atoms.cell, self.atoms.cell, rtol=0, atol=tol):
                changes.append("cell")
            if not np.array_equal(atoms.pbc, self.atoms.pbc):
                changes.append("pbc")
            return changes

        def calculate(self, atoms: "Atoms" = None, properties=("energy",), system_changes=all_changes):
            if atoms is not None:
                self.atoms = atoms.copy()

        def get_property(self, name: str, atoms: "Atoms" = None, allow_calculation: bool = True):
            if name not in self.implemented_properties:
                raise NotImplementedError(f"{name} property not implemented")
            if atoms is None:
                atoms = self.atoms
                system_changes: List[str] = []
            else:
                system_changes = self.check_state(atoms)
                if system_changes:
                    self.results = {}
            if name not in self.results:
                if not allow_calculation:
                    return None
                self.calculate(atoms, [name], system_changes)
            value = self.results[name]
            return value.copy() if isinstance(value, np.ndarray) else value

    class Atoms:
        """Minimal ase.Atoms: numbers, positions (Angstrom), cell, pbc,
        masses (amu) and momenta."""

        def __init__(self, numbers=None, positions=None, cell=None, pbc=None, masses=None,
                     momenta=None, velocities=None, calculator=None):
            self.numbers = np.asarray(numbers if numbers is not None else [], dtype=np.int64).copy()
            n = len(self.numbers)
            self.positions = (np.zeros((n, 3)) if positions is None
                              else np.asarray(positions, dtype=np.float64).reshape(n, 3).copy())
            c = np.zeros((3, 3)) if cell is None else np.asarray(cell, dtype=np.float64)
            self.cell = np.diag(c) if c.shape == (3,) else c.reshape(3, 3).copy()
            p = False if pbc is None else pbc
            self.pbc = np.array([p] * 3 if np.ndim(p) == 0 else p, dtype=bool)
            self._masses = None if masses is None else np.asarray(masses, dtype=np.float64).copy()
            self._momenta = np.zeros((n, 3))
            if momenta is not None:
                self.set_momenta(momenta)
            if velocities is not None:
                self.set_velocities(velocities)
            self.calc = calculator

        def __len__(self) -> int:
            return len(self.numbers)

        def copy(self) -> "Atoms":
            a = Atoms(self.numbers, self.positions, self.cell, self.pbc, self._masses, self._momenta)
            return a

        # geometry
        def get_positions(self) -> np.ndarray:
            return self.positions.copy()

        def set_positions(self, positions):
            self.positions = np.asarray(positions, dtype=np.float64).reshape(len(self), 3).copy()

        def get_atomic_numbers(self) -> np.ndarray:
            return self.numbers.copy()

        def get_cell(self) -> np.ndarray:
            return self.cell.copy()

        def get_pbc(self) -> np.ndarray:
            return self.pbc.copy()

        def get_volume(self) -> float:
            return float(abs(np.linalg.det(self.cell)))

        # masses and motion
        def get_masses(self) -> np.ndarray:
            return units.masses_of(self.numbers) if self._masses is None else self._masses.copy()

        def set_masses(self, masses):
            self._masses = np.asarray(masses, dtype=np.float64).copy()

        def get_momenta(self) -> np.ndarray:
            return self._momenta.copy()

        def set_momenta(self, momenta):
            self._momenta = np.asarray(momenta, dtype=np.float64).reshape(len(self), 3).copy()

        def get_velocities(self) -> np.ndarray:
            return self._momenta / self.get_masses()[:, None]

        def set_velocities(self, velocities):
            self.set_momenta(np.asarray(velocities, dtype=np.float64) * self.get_masses()[:, None])

        def get_kinetic_energy(self) -> float:
            return float(0.5 * np.sum(self._momenta * self.get_velocities()))

        def get_temperature(self) -> float:
            dof = 3 * len(self)
            return 2.0 * self.get_kinetic_energy() / (dof * units.kB) if dof else 0.0

        # calculator
        def _calc(self):
            if self.calc is None:
                raise RuntimeError("Atoms object has no calculator.")
            return self.calc

        def get_potential_energy(self) -> float:
            return self._calc().get_property("energy", self)

        def get_forces(self) -> np.ndarray:
            return self._calc().get_property("forces", self)

        def get_stress(self) -> np.ndarray:
            return self._calc().get_property("stress", self)

        def get_total_energy(self) -> float:
            return self.get_potential_energy() + self.get_kinetic_energy()
