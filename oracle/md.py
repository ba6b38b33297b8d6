"""ORACLE -- test infrastructure only.

Float64 velocity-Verlet restated from the NVE loop the reference drives
(src/mlff_distiller/testing/nve_harness.py:173-261: ASE's VelocityVerlet,
un-vendored, not installed here, so parity with ASE itself is unpinned).
Per step, as ASE's VelocityVerlet.step does it:

    v += dt/2 F(r)/m ;  r += dt v ;  F = F(r) ;  v += dt/2 F/m

The force callback receives float64 positions and returns float64 forces and
the per-structure potential energy.
"""
from typing import Callable, Tuple

import numpy as np


def velocity_verlet(pos: np.ndarray, vel: np.ndarray, masses: np.ndarray,
                    force_fn: Callable[[np.ndarray], Tuple[np.ndarray, np.ndarray]], dt: float, n_steps: int,
                    mol_ptr: np.ndarray):
    """Returns final (pos, vel, forces) and per-step [n_steps, B] potential
    and kinetic energies."""
    r = np.array(pos, dtype=np.float64)
    v = np.array(vel, dtype=np.float64)
    m = np.asarray(masses, dtype=np.float64)[:, None]
    e, F = force_fn(r)
    B = len(mol_ptr) - 1
    epot = np.zeros((n_steps, B))
    ekin = np.zeros((n_steps, B))
    for s in range(n_steps):
        v = v + 0.5 * dt * F / m
        r = r + dt * v
        e, F = force_fn(r)
        v = v + 0.5 * dt * F / m
        ke = 0.5 * m * v * v
        epot[s] = e
        ekin[s] = [ke[mol_ptr[b]:mol_ptr[b + 1]].sum() for b in range(B)]
    return r, v, F, epot, ekin


def langevin_baoab(pos: np.ndarray, vel: np.ndarray, masses: np.ndarray,
                   force_fn: Callable[[np.ndarray], Tuple[np.ndarray, np.ndarray]], dt: float, friction: float,
                   kT: float, seed: int, step0: int, n_steps: int, mol_ptr: np.ndarray):
    """Float64 BAOAB Langevin (Leimkuhler and Matthews, J. Chem. Phys. 138,
    174102 (2013)) with the normals of oracle/philox.py keyed by
    (seed, step0 + step, atom), as the GPU integrator draws them:
        v += dt/2 F/m; r += dt/2 v; v = c1 v + sqrt((1 - c1^2) kT/m) xi;
        r += dt/2 v; F = F(r); v += dt/2 F/m,   c1 = exp(-friction dt)."""
    from oracle.philox import langevin_normals
    r = np.array(pos, dtype=np.float64)
    v = np.array(vel, dtype=np.float64)
    m = np.asarray(masses, dtype=np.float64)[:, None]
    c1 = np.exp(-friction * dt)
    c2 = np.sqrt(max(0.0, 1.0 - c1 * c1))
    e, F = force_fn(r)
    B = len(mol_ptr) - 1
    epot = np.zeros((n_steps, B))
    ekin = np.zeros((n_steps, B))
    for s in range(n_steps):
        xi = langevin_normals(seed, step0 + s, r.shape[0])
        v = v + 0.5 * dt * F / m
        r = r + 0.5 * dt * v
        v = c1 * v + c2 * np.sqrt(kT / m) * xi
        r = r + 0.5 * dt * v
        e, F = force_fn(r)
        v = v + 0.5 * dt * F / m
        ke = 0.5 * m * v * v
        epot[s] = e
        ekin[s] = [ke[mol_ptr[b]:mol_ptr[b + 1]].sum() for b in range(B)]
    return r, v, F, epot, ekin
