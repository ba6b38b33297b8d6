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


def langevin_vec(pos: np.ndarray, vel: np.ndarray, masses: np.ndarray,
                 force_fn: Callable[[np.ndarray], Tuple[np.ndarray, np.ndarray]], dt: float, friction: float,
                 kT: float, seed: int, step0: int, n_steps: int, mol_ptr: np.ndarray, fix_com: bool = True):
    """Float64 Langevin of Vanden-Eijnden and Ciccotti (Chem. Phys. Lett.
    429, 310 (2006), Eq. 23), the scheme of ASE's Langevin (the reference's
    NVT protocol, benchmarks/md_trajectory.py:407-413), with its default
    fixed centre of mass, and the normals of oracle/philox.py:vec_normals
    keyed by (seed, step0 + step, atom) as the GPU integrator draws them.
    sigma = sqrt(2 kT gamma / m); c1 = dt/2 - dt^2 gamma/8, c2 = gamma dt/2 -
    gamma^2 dt^2/8, c3 = sqrt(dt) sigma/2 - dt^1.5 gamma sigma/8, c5 =
    dt^1.5 sigma/(2 sqrt 3), c4 = gamma c5/2;
        v += c1 F/m - c2 v + c3 xi - c4 eta;  r += dt v + c5 eta
        (fix_com: shift each structure back to its old centre of mass,
         v = (r_new - r - c5 eta) / dt);  F = F(r);
        v += c1 F/m - c2 v + c3 xi - c4 eta;  (fix_com: v -= v_com)."""
    from oracle.philox import vec_normals
    r = np.array(pos, dtype=np.float64)
    v = np.array(vel, dtype=np.float64)
    m = np.asarray(masses, dtype=np.float64)[:, None]
    g = float(friction)
    sig = np.sqrt(2.0 * kT * g / m)
    c1 = dt / 2.0 - dt * dt * g / 8.0
    c2 = g * dt / 2.0 - g * g * dt * dt / 8.0
    c3 = np.sqrt(dt) * sig / 2.0 - dt ** 1.5 * g * sig / 8.0
    c5 = dt ** 1.5 * sig / (2.0 * np.sqrt(3.0))
    c4 = g / 2.0 * c5
    e, F = force_fn(r)
    B = len(mol_ptr) - 1
    epot = np.zeros((n_steps, B))
    ekin = np.zeros((n_steps, B))
    groups = [slice(mol_ptr[b], mol_ptr[b + 1]) for b in range(B)]
    for s in range(n_steps):
        nz = vec_normals(seed, step0 + s, r.shape[0])
        xi, eta = nz[:, :3], nz[:, 3:]
        v = v + (c1 * F / m - c2 * v + c3 * xi - c4 * eta)
        x_old = r
        r = r + dt * v + c5 * eta
        if fix_com:
            for sl in groups:
                mm = m[sl]
                shift = ((mm * x_old[sl]).sum(axis=0) - (mm * r[sl]).sum(axis=0)) / mm.sum()
                r[sl] = r[sl] + shift
                v[sl] = v[sl] + shift / dt
        e, F = force_fn(r)
        v = v + (c1 * F / m - c2 * v + c3 * xi - c4 * eta)
        if fix_com:
            for sl in groups:
                mm = m[sl]
                v[sl] = v[sl] - (mm * v[sl]).sum(axis=0) / mm.sum()
        ke = 0.5 * m * v * v
        epot[s] = e
        ekin[s] = [ke[sl].sum() for sl in groups]
    return r, v, F, epot, ekin


def npt_melchionna(pos: np.ndarray, vel: np.ndarray, masses: np.ndarray, box: np.ndarray,
                   force_fn: Callable[[np.ndarray, np.ndarray], Tuple[float, np.ndarray, np.ndarray]], dt: float,
                   kT: float, ttime: float, pfactor: float, pressure: float, n_steps: int,
                   zeta: float = 0.0, eta=None, xi: float = 0.0):
    """Float64 NPT for one orthorhombic periodic structure with the
    equations of motion of ASE's NPT (Melchionna, Ciccotti and Holian, Mol.
    Phys. 78, 533 (1993); diagonal strain rate):
        dr/dt = v + eta (r - R_com),  dv/dt = F/m - (zeta + eta) v,
        dzeta/dt = (2K / (3 n kT) - 1) / ttime^2,
        deta/dt = V / pfactor (diag(sum m v v - W) / V - pressure),  dL/dt = eta L,
    W = dE/d(strain), and the time-reversible splitting the GPU integrator
    uses: half step of zeta (then xi += dt/2 zeta) and eta; v scaled by
    exp(-(zeta + eta) dt/2) and half-kicked; exact drift for constant v of
    positions relative to the moving centre of mass and of the box; force
    and virial; half kick and scaling; xi += dt/2 zeta, half step of zeta
    and eta.  force_fn(pos, box) -> (E, F [n,3], W [3,3]).  Returns the
    final state and per-step potential energy, kinetic energy, volume,
    zeta, eta and xi."""
    r = np.array(pos, dtype=np.float64)
    v = np.array(vel, dtype=np.float64)
    L = np.array(box, dtype=np.float64).reshape(3)
    m = np.asarray(masses, dtype=np.float64)[:, None]
    eta = np.zeros(3) if eta is None else np.array(eta, dtype=np.float64)
    n = r.shape[0]
    g = 3.0 * n
    E, F, W = force_fn(r, L)
    out = {"epot": np.zeros(n_steps), "ekin": np.zeros(n_steps), "volume": np.zeros(n_steps),
           "zeta_t": np.zeros(n_steps), "eta_t": np.zeros((n_steps, 3)), "xi_t": np.zeros(n_steps)}

    def half(zeta, eta, K):
        V = float(np.prod(L))
        if ttime > 0:
            zeta = zeta + 0.5 * dt * (K.sum() / (g * kT) - 1.0) / ttime ** 2
        if pfactor > 0:
            eta = eta + 0.5 * dt * (V / pfactor) * ((K - np.diag(W)) / V - pressure)
        return zeta, eta

    for s in range(n_steps):
        K = (m * v * v).sum(axis=0)
        zeta, eta = half(zeta, eta, K)
        xi += 0.5 * dt * zeta
        v = v * np.exp(-0.5 * dt * (zeta + eta)) + 0.5 * dt * F / m
        M = m.sum()
        R0 = (m * r).sum(axis=0) / M
        vc = (m * v).sum(axis=0) / M
        x = eta * dt
        ph = dt * np.where(np.abs(x) < 1e-12, 1.0 + 0.5 * x, np.expm1(x) / np.where(x == 0, 1.0, x))
        r = R0 + vc * dt + np.exp(x) * (r - R0) + (v - vc) * ph
        L = L * np.exp(x)
        E, F, W = force_fn(r, L)
        v = (v + 0.5 * dt * F / m) * np.exp(-0.5 * dt * (zeta + eta))
        K = (m * v * v).sum(axis=0)
        xi += 0.5 * dt * zeta
        zeta, eta = half(zeta, eta, K)
        out["epot"][s] = E
        out["ekin"][s] = 0.5 * K.sum()
        out["volume"][s] = np.prod(L)
        out["zeta_t"][s], out["eta_t"][s], out["xi_t"][s] = zeta, eta, xi
    out.update(pos=r, vel=v, box=L, zeta=zeta, eta=eta, xi=xi, forces=F, virial=W)
    return out


def npt_conserved(epot: float, ekin: float, volume: float, n_atoms: int, kT: float, ttime: float, pfactor: float,
                  pressure: float, zeta: float, eta: np.ndarray, xi: float) -> float:
    """E + K + P V + 3 n kT (ttime^2 zeta^2 / 2 + xi) + pfactor |eta|^2 / 2,
    conserved by the NPT equations of motion above."""
    g = 3.0 * n_atoms
    return (epot + ekin + pressure * volume + g * kT * (0.5 * ttime ** 2 * zeta ** 2 + xi) +
            0.5 * pfactor * float(np.dot(eta, eta)))
