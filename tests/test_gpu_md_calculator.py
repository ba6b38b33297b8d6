"""Drop-in ASE calculator and the GPU velocity-Verlet driver (GPU only).

Calculator results are checked against the float64 oracle with the bars of
the parity tests (forces max |dF| <= 1e-3 eV/A, energy <= 5e-5 eV/atom).
The integrator is checked against the float64 Verlet restatement in
oracle/md.py driven by oracle forces, the CUDA-graph replay against eager
steps (bit for bit), and the NVE energy drift of MD replicas.
"""
import numpy as np
import pytest
import torch

from oracle import painn
from oracle.md import velocity_verlet

pytestmark = pytest.mark.gpu

F_TOL = 1e-3
E_TOL_PER_ATOM = 5e-5


@pytest.fixture(scope="module")
def ckpt(tmp_path_factory, weights_bias):
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField()
    m.load_state_dict({k: torch.tensor(v) for k, v in weights_bias.items()})
    p = tmp_path_factory.mktemp("ckpt") / "model.pt"
    m.save(p)
    return p


def _atoms(sysm, m=0):
    from mlff_gb300.ase_compat import Atoms
    s = sysm.molecule(m) if sysm.n_mol > 1 else sysm
    a = Atoms(numbers=s.Z, positions=s.pos)
    if s.pbc is not None and bool(np.asarray(s.pbc).any()):
        a = Atoms(numbers=s.Z, positions=s.pos, cell=np.diag(s.box[0]), pbc=True)
    return a


def test_calculator_energy_forces_vs_oracle(ckpt, weights_bias):
    from mlff_gb300 import systems
    from mlff_gb300.ase_calculator import StudentForceFieldCalculator
    s = systems.lattice_molecule(60, seed=0)
    calc = StudentForceFieldCalculator(ckpt, enable_timing=True)
    atoms = _atoms(s)
    atoms.calc = calc
    e = atoms.get_potential_energy()
    f = atoms.get_forces()
    atoms.get_forces()                       # cached: no second evaluation
    assert calc.n_calls == 1 and calc.get_timing_stats()["n_calls"] == 1
    E0, F0 = painn.energy_forces(weights_bias, s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr)
    assert abs(e - float(E0[0])) <= E_TOL_PER_ATOM * s.n_atoms
    assert np.abs(f - F0.numpy()).max() <= F_TOL
    assert isinstance(e, float) and f.dtype == np.float64 and f.shape == (60, 3)


def test_calculate_batch_equals_single(ckpt):
    from mlff_gb300 import systems
    from mlff_gb300.ase_calculator import StudentForceFieldCalculator
    s = systems.molecule_batch(5, 10, 60, seed=7)
    calc = StudentForceFieldCalculator(ckpt)
    batch = calc.calculate_batch([_atoms(s, m) for m in range(s.n_mol)])
    for m in range(s.n_mol):
        a = _atoms(s, m)
        a.calc = calc
        assert abs(batch[m]["energy"] - a.get_potential_energy()) <= 1e-6 * max(1.0, abs(batch[m]["energy"]))
        np.testing.assert_allclose(batch[m]["forces"], a.get_forces(), rtol=0, atol=1e-5)


def test_stress_periodic_vs_oracle(ckpt, weights_bias):
    from mlff_gb300 import systems
    from mlff_gb300.ase_calculator import StudentForceFieldCalculator
    s = systems.water_box(n_water=50, L=11.0, seed=3)
    calc = StudentForceFieldCalculator(ckpt, enable_stress=True)
    a = _atoms(s)
    a.calc = calc
    stress = a.get_stress()
    E0, F0, V0 = painn.energy_forces(weights_bias, s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr,
                                     box=s.box, pbc=s.pbc, virial=True)
    ref = painn.stress_voigt(V0.numpy()[0], s.box[0])
    assert np.abs(stress - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())
    assert np.abs(a.get_forces() - F0.numpy()).max() <= F_TOL


def _driver(weights, sysm, precision="fp16x3"):
    from mlff_gb300.md import VelocityVerletGPU
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision=precision).to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    m.eval()
    return VelocityVerletGPU(m, sysm.Z, sysm.pos, sysm.mol_ptr, timestep_fs=0.5)


def test_verlet_graph_equals_eager(weights_seed0):
    from mlff_gb300 import systems
    s = systems.replicas(4, 64, seed=3)
    runs = []
    for graph in (False, True):
        d = _driver(weights_seed0, s)
        d.initialize_velocities(300.0, seed=1)
        tr = d.run(30, graph=graph, block=10)
        runs.append((d.positions(), d.velocities(), tr["potential_energy"], tr["kinetic_energy"]))
    for a, b in zip(*runs):
        np.testing.assert_array_equal(a, b)


def test_verlet_vs_oracle_integrator(weights_seed0):
    """20 steps of the float64 GPU integrator against the float64 oracle
    Verlet driven by oracle forces evaluated at float32-rounded positions
    (what the device force call sees)."""
    from mlff_gb300 import systems
    from mlff_gb300.md import kinetic_energy
    s = systems.lattice_molecule(60, seed=0)
    d = _driver(weights_seed0, s, precision="tuned_fp32")
    d.initialize_velocities(300.0, seed=2)
    v0, x0 = d.velocities(), d.positions()
    tr = d.run(20, graph=True, block=10)

    def force_fn(r):
        E, F = painn.energy_forces(weights_seed0, s.Z, r.astype(np.float32).astype(np.float64), s.mol_ptr)
        return E.numpy(), F.numpy()

    r, v, F, ep, ek = velocity_verlet(x0, v0, d.masses, force_fn, d.dt, 20, s.mol_ptr)
    assert np.abs(d.positions() - r).max() < 1e-5
    assert np.abs(d.velocities() - v).max() < 1e-4
    assert np.abs(tr["potential_energy"] - ep).max() <= E_TOL_PER_ATOM * s.n_atoms
    np.testing.assert_allclose(tr["kinetic_energy"], ek, rtol=1e-5, atol=1e-6)
    assert np.allclose(kinetic_energy(d.velocities(), d.masses, s.mol_ptr), tr["kinetic_energy"][-1])


def test_nve_replicas_energy_drift(weights_seed0):
    """MD replicas (64-atom molecules, 300 K, 0.5 fs, 400 steps): the total
    energy of every replica stays within 2 meV/atom of its start."""
    from mlff_gb300 import systems
    from mlff_gb300.md import kinetic_energy
    s = systems.replicas(16, 64, seed=3)
    d = _driver(weights_seed0, s)
    d.initialize_velocities(300.0, seed=4)
    E0, _ = d.compute_forces()
    K0 = kinetic_energy(d.velocities(), d.masses, s.mol_ptr)
    tr = d.run(400, graph=True, block=50)
    et = tr["potential_energy"] + tr["kinetic_energy"]
    per_atom = np.abs(et - (E0 + K0)[None, :]) / 64
    print("max |E - E0| per atom", per_atom.max())
    assert np.isfinite(et).all()
    assert per_atom.max() < 2e-3


def test_nve_energy_error_no_worse_than_fp64_reference_algorithm(weights_seed0):
    """Total-energy excursion of the GPU trajectory (split-FP16 filters,
    float64 state) against the float64 oracle integrator with float64
    forces from the same start, 200 steps: the GPU's max |E(t) - E(0)| is
    within 25 % (plus 0.05 meV/atom) of the float64 one."""
    from mlff_gb300 import systems
    from mlff_gb300.md import kinetic_energy
    s = systems.lattice_molecule(60, seed=0)
    d = _driver(weights_seed0, s)
    d.initialize_velocities(300.0, seed=5)
    x0, v0 = d.positions(), d.velocities()
    E0, _ = d.compute_forces()
    K0 = kinetic_energy(v0, d.masses, s.mol_ptr)
    tr = d.run(200, graph=True, block=50)
    gpu = np.abs(tr["potential_energy"] + tr["kinetic_energy"] - (E0 + K0)).max()

    def force_fn(r):
        E, F = painn.energy_forces(weights_seed0, s.Z, r, s.mol_ptr)
        return E.numpy(), F.numpy()

    e_ref0, _ = force_fn(x0)
    _, _, _, ep, ek = velocity_verlet(x0, v0, d.masses, force_fn, d.dt, 200, s.mol_ptr)
    ref = np.abs(ep + ek - (e_ref0 + K0)).max()
    print("max |E - E0|: gpu", gpu, "float64 oracle", ref)
    assert gpu <= 1.25 * ref + 5e-5 * s.n_atoms


def test_harness_interface(ckpt):
    from mlff_gb300 import systems
    from mlff_gb300.ase_calculator import StudentForceFieldCalculator
    from mlff_gb300.md import NVEMDHarness
    s = systems.lattice_molecule(60, seed=0)
    calc = StudentForceFieldCalculator(ckpt)
    h = NVEMDHarness(_atoms(s), calc, temperature=300.0, timestep=0.5, log_interval=10)
    res = h.run_simulation(steps=30)
    td = res["trajectory_data"]
    assert res["n_steps"] == 30 and h.is_complete
    assert len(td["total_energy"]) == 31 and len(td["positions"]) == 4
    assert np.isfinite(res["energy_drift_pct"])
    assert abs(res["total_time_ps"] - 0.015) < 1e-12
    for k in ("energy_drift_abs", "avg_temperature", "std_temperature", "initial_energy", "final_energy",
              "avg_potential_energy", "avg_kinetic_energy", "wall_time_s"):
        assert k in res
    with pytest.raises(ValueError):
        h.run_simulation(steps=0)


def test_student_calculator_equals_force_field_calculator(ckpt):
    """The generic dict-in/dict-out StudentCalculator on a StudentForceField
    checkpoint gives the drop-in calculator's results (molecule and
    periodic box with stress)."""
    from mlff_gb300 import systems
    from mlff_gb300.ase_calculator import StudentForceFieldCalculator
    from mlff_gb300.student_calculator import StudentCalculator
    gen = StudentCalculator(model_path=ckpt)
    ref = StudentForceFieldCalculator(ckpt, enable_stress=True)
    for s in (systems.lattice_molecule(60, seed=0), systems.water_box(n_water=50, L=11.0, seed=3)):
        a, b = _atoms(s), _atoms(s)
        a.calc, b.calc = gen, ref
        assert a.get_potential_energy() == b.get_potential_energy()
        np.testing.assert_array_equal(a.get_forces(), b.get_forces())
        if s.pbc is not None and bool(np.asarray(s.pbc).any()):
            np.testing.assert_allclose(a.get_stress(), b.get_stress(), rtol=1e-12, atol=1e-12)
