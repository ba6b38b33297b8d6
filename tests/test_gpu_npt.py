"""NPT (Nose-Hoover + Parrinello-Rahman equations of motion, orthorhombic
boxes) on the GPU (GPU only).

The float64 GPU integrator is checked against the float64 restatement of the
same splitting in oracle/md.py driven by oracle forces and virials, a
CUDA-graph replay against eager steps, conservation of the extended energy
the equations of motion conserve, and the barostat's response: a target
pressure above the box's pressure shrinks it, one below expands it; a
runaway barostat (pfactor far too small) stops with an error status instead
of blowing the box up.
"""
import numpy as np
import pytest
import torch

from oracle import painn
from oracle.md import npt_conserved, npt_melchionna

pytestmark = pytest.mark.gpu

KT300 = 8.617333262e-5 * 300.0


def _npt(weights, s, T=300.0, ttime_fs=25.0, pfactor=2000.0, pressure=0.0, precision="tuned_fp32"):
    from mlff_gb300 import units
    from mlff_gb300.md import NPTGPU
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision=precision).to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    m.eval()
    d = NPTGPU(m, s.Z, s.pos, s.mol_ptr, s.box, temperature_K=T, externalstress=pressure,
               ttime=ttime_fs * units.fs, pfactor=pfactor, timestep_fs=0.5)
    d.initialize_velocities(T, seed=5, remove_com_rotation=False)
    return d


def _box():
    from mlff_gb300 import systems
    return systems.water_box(n_water=60, L=11.5, d_oo=2.2, seed=8)


def test_npt_vs_oracle_integrator(weights_bias):
    from mlff_gb300 import units
    s = _box()
    d = _npt(weights_bias, s)
    v0, x0 = d.velocities(), d.positions()
    tr = d.run(12, graph=False)

    def force_fn(r, L):
        # the library evaluates the float32 copies of positions and box
        E, F, W = painn.energy_forces(weights_bias, s.Z, r.astype(np.float32).astype(np.float64), s.mol_ptr,
                                      box=L.astype(np.float32).astype(np.float64).reshape(1, 3), pbc=s.pbc,
                                      virial=True)
        return float(E[0]), F.numpy(), W.numpy()[0]

    o = npt_melchionna(x0, v0, d.masses, s.box[0], force_fn, d.dt, KT300, 25.0 * units.fs, 2000.0, 0.0, 12)
    dx = np.abs(d.positions() - o["pos"]).max()
    dv = np.abs(d.velocities() - o["vel"]).max() / np.abs(o["vel"]).max()
    dL = np.abs(d.box64.cpu().numpy()[0] - o["box"]).max()
    deta = np.abs(d.eta.cpu().numpy()[0] - o["eta"]).max() / max(np.abs(o["eta"]).max(), 1e-12)
    dz = abs(float(d.zeta[0]) - o["zeta"]) / max(abs(o["zeta"]), 1e-12)
    print(f"max |dx| {dx:.2e} A, rel dv {dv:.2e}, |dL| {dL:.2e} A, rel deta {deta:.2e}, rel dzeta {dz:.2e}; "
          f"volume {o['volume'][0]:.2f} -> {o['volume'][-1]:.2f}")
    assert abs(o["volume"][-1] - o["volume"][0]) > 1e-3   # the barostat acted
    assert dx < 1e-4 and dv < 1e-4 and dL < 1e-5 and deta < 1e-3 and dz < 1e-3
    np.testing.assert_allclose(tr["potential_energy"][:, 0], o["epot"], rtol=0, atol=2e-3)
    np.testing.assert_allclose(tr["kinetic_energy"][:, 0], o["ekin"], rtol=1e-4, atol=1e-6)


def test_npt_graph_equals_eager(weights_bias):
    s = _box()
    a, b = _npt(weights_bias, s), _npt(weights_bias, s)
    b.set_velocities(a.velocities())
    ta = a.run(20, graph=True, block=10)
    tb = b.run(20, graph=False)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.box64.cpu().numpy(), b.box64.cpu().numpy())
    assert np.array_equal(ta["potential_energy"], tb["potential_energy"])


def test_npt_extended_energy_error_no_worse_than_fp64_algorithm(weights_seed0):
    """The conserved quantity E + K + P V + 3 n kT (ttime^2 zeta^2 / 2 + xi)
    + pfactor |eta|^2 / 2 along the GPU trajectory (float32 forces, float64
    state), read every 10 steps for 200 steps, against the same splitting in
    float64 with float64 forces from the same start: the GPU's largest
    excursion is within 25 % (plus 0.05 meV/atom) of the float64 one."""
    from mlff_gb300 import units
    s = _box()
    tt, pf = 25.0 * units.fs, 20000.0
    d = _npt(weights_seed0, s, pfactor=pf)
    x0, v0 = d.positions(), d.velocities()
    d.compute_forces()
    H0 = d.npt_conserved()[0]
    gpu = 0.0
    for _ in range(20):
        d.run(10, graph=True, block=10)
        gpu = max(gpu, abs(d.npt_conserved()[0] - H0))

    def force_fn(r, L):
        E, F, W = painn.energy_forces(weights_seed0, s.Z, r, s.mol_ptr, box=L.reshape(1, 3), pbc=s.pbc, virial=True)
        return float(E[0]), F.numpy(), W.numpy()[0]

    o = npt_melchionna(x0, v0, d.masses, s.box[0], force_fn, d.dt, KT300, tt, pf, 0.0, 200)
    E0, _, _ = force_fn(x0, s.box[0])
    K0 = 0.5 * float((d.masses[:, None] * v0 * v0).sum())
    h0 = npt_conserved(E0, K0, float(np.prod(s.box[0])), s.n_atoms, KT300, tt, pf, 0.0, 0.0, np.zeros(3), 0.0)
    h = np.array([npt_conserved(o["epot"][i], o["ekin"][i], o["volume"][i], s.n_atoms, KT300, tt, pf, 0.0,
                                o["zeta_t"][i], o["eta_t"][i], o["xi_t"][i]) for i in range(9, 200, 10)])
    ref = np.abs(h - h0).max()
    print(f"max |H - H0| every 10 steps: gpu {gpu:.3e} eV, float64 algorithm {ref:.3e} eV; "
          f"volume {o['volume'][0]:.2f} -> {o['volume'][-1]:.2f}")
    assert gpu <= 1.25 * ref + 5e-5 * s.n_atoms


def test_npt_barostat_direction(weights_seed0):
    """From the same start, a target pressure well above the box's own
    pressure compresses it and one well below expands it (20 steps, no
    thermostat)."""
    s = _box()
    d = _npt(weights_seed0, s, ttime_fs=0.0)
    d.compute_forces()
    W = d.virial.cpu().numpy()[0]
    V0 = float(d.volumes()[0])
    K = (d.masses[:, None] * d.velocities() ** 2).sum(axis=0)
    P0 = float((K - np.diag(W)).sum() / (3.0 * V0))
    snap = d.snapshot()
    vols = {}
    for tag, dp in (("high", 0.05), ("low", -0.05)):
        d.set_npt(300.0, externalstress=P0 + dp, ttime=0.0, pfactor=2000.0)
        d.restore(snap)
        d.run(20, graph=False)
        vols[tag] = float(d.volumes()[0])
    print(f"P0 {P0:.3e} eV/A^3, V0 {V0:.2f}; V(P0 + 0.05) {vols['high']:.2f}, V(P0 - 0.05) {vols['low']:.2f}")
    assert vols["high"] < V0 < vols["low"]


def test_npt_runaway_barostat_reports_error(weights_bias):
    """pfactor far too small: the strain rate grows until the box would
    change by more than 20 % in a step; the integrator sets the box error
    instead (the run raises), and the positions stay finite."""
    from mlff_gb300 import _lib
    s = _box()
    d = _npt(weights_bias, s, pfactor=0.5)
    with pytest.raises(_lib.MLFFError):
        d.run(400, graph=False)
    assert np.isfinite(d.positions()).all()
