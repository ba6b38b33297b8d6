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
