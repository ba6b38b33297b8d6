"""Langevin NVT on the GPU (GPU only), both schemes: ASE's
(Vanden-Eijnden-Ciccotti, fixed centre of mass; the default) and BAOAB.

The float64 GPU integrators are checked against the float64 restatements in
oracle/md.py driven by oracle forces and the same Philox normals, a
CUDA-graph replay against eager steps (bit for bit: the draws are keyed by a
device-side step counter), and the thermostat's equilibrium kinetic
temperature on non-interacting atoms.
"""
import numpy as np
import pytest
import torch

from oracle import painn
from oracle.md import langevin_baoab, langevin_vec

pytestmark = pytest.mark.gpu


def _langevin(weights, sysm, T, friction, seed, precision="tuned_fp32", scheme="ase"):
    from mlff_gb300.md import LangevinGPU
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision=precision).to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    m.eval()
    return LangevinGPU(m, sysm.Z, sysm.pos, sysm.mol_ptr, temperature_K=T, friction=friction, seed=seed,
                       timestep_fs=0.5, scheme=scheme)


@pytest.mark.parametrize("scheme", ["ase", "baoab"])
def test_langevin_vs_oracle_integrator(weights_seed0, scheme):
    from mlff_gb300 import systems, units
    s = systems.concat([systems.lattice_molecule(60, seed=0), systems.lattice_molecule(23, seed=4)])
    d = _langevin(weights_seed0, s, 300.0, 0.02, seed=11, scheme=scheme)
    d.initialize_velocities(300.0, seed=2)
    v0, x0 = d.velocities(), d.positions()
    tr = d.run(20, graph=True, block=10)

    def force_fn(r):
        E, F = painn.energy_forces(weights_seed0, s.Z, r.astype(np.float32).astype(np.float64), s.mol_ptr)
        return E.numpy(), F.numpy()

    integrate = langevin_vec if scheme == "ase" else langevin_baoab
    r, v, F, ep, ek = integrate(x0, v0, d.masses, force_fn, d.dt, 0.02, units.kB * 300.0, 11, 0, 20, s.mol_ptr)
    assert np.abs(d.positions() - r).max() < 1e-5
    assert np.abs(d.velocities() - v).max() < 1e-4
    np.testing.assert_allclose(tr["kinetic_energy"], ek, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("scheme", ["ase", "baoab"])
def test_langevin_graph_equals_eager(weights_seed0, scheme):
    from mlff_gb300 import systems
    s = systems.replicas(4, 64, seed=3)
    runs = []
    for graph in (False, True):
        d = _langevin(weights_seed0, s, 300.0, 0.05, seed=5, precision="fp16x3", scheme=scheme)
        d.initialize_velocities(300.0, seed=1)
        tr = d.run(30, graph=graph, block=10)
        runs.append((d.positions(), d.velocities(), tr["kinetic_energy"]))
    for a, b in zip(*runs):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("scheme", ["ase", "baoab"])
def test_langevin_equilibrium_temperature(weights_seed0, scheme):
    """Atoms more than 7 A apart (beyond the 5 A cutoff) feel no force: the
    thermostat must hold the kinetic temperature at T (3n - 3 degrees of
    freedom per structure with the centre of mass fixed)."""
    from mlff_gb300 import systems, units
    s = systems.replicas(8, 64, seed=3)
    s.pos = s.pos * 8.0                         # nearest neighbours >= 7.4 A apart
    # 1/friction ~ 5 ASE time units
    d = _langevin(weights_seed0, s, 300.0, 0.2, seed=9, precision="fp16x3", scheme=scheme)
    _, F0 = d.compute_forces()
    assert float(np.abs(F0).max()) == 0.0         # no edges at the start
    tr = d.run(1200, graph=True, block=50)
    dof = 3 * s.n_atoms - (3 * s.n_mol if scheme == "ase" else 0)
    T = tr["kinetic_energy"].sum(axis=1) / (0.5 * dof * units.kB)
    assert abs(T[600:].mean() / 300.0 - 1.0) < 0.05


def test_ase_scheme_keeps_the_centre_of_mass(weights_seed0):
    from mlff_gb300 import systems
    s = systems.replicas(4, 64, seed=3)
    d = _langevin(weights_seed0, s, 300.0, 0.05, seed=7, precision="fp16x3")
    d.initialize_velocities(300.0, seed=3)
    m = d.masses[:, None]

    def com(x):
        return np.stack([(m[a:b] * x[a:b]).sum(0) / m[a:b].sum() for a, b in zip(s.mol_ptr[:-1], s.mol_ptr[1:])])
    c0 = com(d.positions())
    d.run(40, graph=True, block=20)
    assert np.abs(com(d.positions()) - c0).max() < 1e-9
    assert np.abs(com(d.velocities())).max() < 1e-12
