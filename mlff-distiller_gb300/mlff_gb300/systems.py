"""Seeded synthetic systems with the shapes of the benchmark workloads.

No datasets ship with the reference; these generators stand in for them
with fixed seeds:

* ``lattice_molecule``   -- an open H/C/N/O molecule: the first n sites of a
  ceil(n^(1/3))^3 cubic lattice (a = 1.5 A) plus N(0, 0.1^2) jitter.
* ``molecule_batch``     -- many such molecules of uniform-random size
  (ragged CSR batch, no cross-molecule edges).
* ``water_box``          -- 1000 O by random sequential addition (minimum
  image O-O >= 2.5 A) in a periodic 31 A box, 2 H per O at 0.96 A and
  104.5 deg in random orientation.
* ``replicas``           -- copies of one 64-atom molecule for MD.
* ``large_box``          -- 1e5 atoms on a jittered 47^3 lattice in a
  periodic 100 A box.

Each returns a ``System`` with float64 positions, int64 atomic numbers,
molecule offsets (``mol_ptr``), per-molecule orthorhombic box lengths and
periodic flags.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

ELEMENTS = np.array([1, 6, 7, 8], dtype=np.int64)
ELEMENT_P = np.array([0.5, 0.3, 0.1, 0.1])


@dataclasses.dataclass
class System:
    Z: np.ndarray          # int64 [N]
    pos: np.ndarray        # float64 [N,3]
    mol_ptr: np.ndarray    # int64 [B+1]
    box: np.ndarray        # float64 [B,3] (0 for open molecules)
    pbc: np.ndarray        # bool [B]
    name: str = ""

    @property
    def n_atoms(self) -> int:
        return int(self.Z.shape[0])

    @property
    def n_mol(self) -> int:
        return int(self.mol_ptr.shape[0] - 1)

    def molecule(self, m: int) -> "System":
        a, b = int(self.mol_ptr[m]), int(self.mol_ptr[m + 1])
        return System(self.Z[a:b].copy(), self.pos[a:b].copy(),
                      np.array([0, b - a], np.int64), self.box[m:m + 1].copy(),
                      self.pbc[m:m + 1].copy(), f"{self.name}[{m}]")

    def subset(self, mols: List[int]) -> "System":
        parts = [self.molecule(m) for m in mols]
        return concat(parts, name=f"{self.name}[subset]")


def concat(systems: List[System], name: str = "") -> System:
    Z = np.concatenate([s.Z for s in systems])
    pos = np.concatenate([s.pos for s in systems])
    sizes = np.concatenate([np.diff(s.mol_ptr) for s in systems])
    mol_ptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    box = np.concatenate([s.box for s in systems])
    pbc = np.concatenate([s.pbc for s in systems])
    return System(Z, pos, mol_ptr, box, pbc, name)


def _lattice_sites(n_side: int, a: float) -> np.ndarray:
    idx = np.arange(n_side)
    g = np.stack(np.meshgrid(idx, idx, idx, indexing="ij"), axis=-1).reshape(-1, 3)
    return g.astype(np.float64) * a


def lattice_molecule(n_atoms: int = 60, seed: int = 0, a: float = 1.5,
                     jitter: float = 0.1, rng: Optional[np.random.Generator] = None) -> System:
    """Open molecule of n_atoms H/C/N/O (p = .5/.3/.1/.1) on a jittered
    cubic lattice.  60 atoms with seed 0 is the CPU-runnable case."""
    rng = np.random.default_rng(seed) if rng is None else rng
    n_side = int(math.ceil(n_atoms ** (1.0 / 3.0) - 1e-9))
    while n_side ** 3 < n_atoms:
        n_side += 1
    sites = _lattice_sites(n_side, a)[:n_atoms]
    pos = sites + rng.normal(0.0, jitter, size=sites.shape)
    Z = rng.choice(ELEMENTS, size=n_atoms, p=ELEMENT_P)
    return System(Z.astype(np.int64), pos, np.array([0, n_atoms], np.int64),
                  np.zeros((1, 3)), np.zeros(1, bool), f"molecule{n_atoms}")


def molecule_batch(n_mol: int = 256, n_min: int = 10, n_max: int = 120, seed: int = 1) -> System:
    """n_mol open molecules with sizes uniform in [n_min, n_max] (about
    16-17k atoms for 256 molecules), concatenated as a ragged batch."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(n_min, n_max + 1, size=n_mol)
    mols = [lattice_molecule(int(n), rng=rng) for n in sizes]
    return concat(mols, name=f"batch{n_mol}")


def _min_image(d: np.ndarray, L: float) -> np.ndarray:
    return d - L * np.round(d / L)


def water_box(n_water: int = 1000, L: float = 31.0, d_oo: float = 2.5, seed: int = 2) -> System:
    """Periodic water-like box: O by random sequential addition with
    minimum-image O-O >= d_oo, two H at 0.96 A, HOH 104.5 deg, random
    orientation.  Atom order: O, H, H per molecule."""
    rng = np.random.default_rng(seed)
    O = np.empty((n_water, 3))
    k = 0
    tries = 0
    while k < n_water:
        tries += 1
        if tries > 10_000_000:
            raise RuntimeError("random sequential addition did not converge")
        c = rng.uniform(0.0, L, size=3)
        if k:
            dd = _min_image(O[:k] - c, L)
            if np.min(np.einsum("ij,ij->i", dd, dd)) < d_oo * d_oo:
                continue
        O[k] = c
        k += 1
    theta = math.radians(104.5)
    r_oh = 0.96
    # H positions in a local frame (bisector along x), rotated randomly
    h_local = np.array([[r_oh * math.cos(theta / 2), r_oh * math.sin(theta / 2), 0.0],
                        [r_oh * math.cos(theta / 2), -r_oh * math.sin(theta / 2), 0.0]])
    pos = np.empty((3 * n_water, 3))
    for i in range(n_water):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        pos[3 * i] = O[i]
        pos[3 * i + 1:3 * i + 3] = O[i] + h_local @ R.T
    Z = np.tile(np.array([8, 1, 1], np.int64), n_water)
    return System(Z, pos, np.array([0, 3 * n_water], np.int64), np.array([[L, L, L]]),
                  np.ones(1, bool), f"water{n_water}")


def replicas(n_rep: int = 128, n_atoms: int = 64, seed: int = 3) -> System:
    """n_rep copies of one n_atoms lattice molecule (MD replica batch)."""
    mol = lattice_molecule(n_atoms, seed=seed)
    return concat([mol] * n_rep, name=f"replicas{n_rep}x{n_atoms}")


def large_box(n_atoms: int = 100_000, density: float = 0.1, jitter: float = 0.15,
              seed: int = 4) -> System:
    """Periodic cubic box at the given number density: first n_atoms sites
    of a jittered ceil(n^(1/3))^3 lattice, wrapped into the box."""
    rng = np.random.default_rng(seed)
    L = (n_atoms / density) ** (1.0 / 3.0)
    n_side = int(math.ceil(n_atoms ** (1.0 / 3.0) - 1e-9))
    while n_side ** 3 < n_atoms:
        n_side += 1
    a = L / n_side
    sites = _lattice_sites(n_side, a)[:n_atoms]
    pos = sites + rng.normal(0.0, jitter, size=sites.shape)
    pos = pos - L * np.floor(pos / L)
    Z = rng.choice(ELEMENTS, size=n_atoms, p=ELEMENT_P)
    return System(Z.astype(np.int64), pos, np.array([0, n_atoms], np.int64),
                  np.array([[L, L, L]]), np.ones(1, bool), f"box{n_atoms}")


def workload(name: str) -> System:
    """Named workloads: molecule60, batch256, water3000, replicas128x64, box100k."""
    if name == "molecule60":
        return lattice_molecule(60, seed=0)
    if name == "batch256":
        return molecule_batch(256)
    if name == "water3000":
        return water_box()
    if name == "replicas128x64":
        return replicas()
    if name == "box100k":
        return large_box()
    raise KeyError(name)
