"""Device energy-conservation statistics (mlff_md_energy_stats) against the
numpy restatement of the reference's metrics in oracle/energy_metrics.py
(GPU only), per replica and through the reference-named functions."""
import numpy as np
import pytest
import torch

from oracle.energy_metrics import stats as oracle_stats

pytestmark = pytest.mark.gpu


def test_replica_stats_vs_oracle():
    from mlff_gb300.energy_metrics import STAT_NAMES, replica_energy_stats
    rng = np.random.default_rng(0)
    n, B = 1001, 5
    t = np.arange(n)
    ep = -50.0 - 0.3 * np.sin(t / 17.0)[:, None] + 0.01 * rng.standard_normal((n, B)) + 1e-4 * t[:, None]
    ek = 2.0 + 0.3 * np.sin(t / 17.0)[:, None] + 0.01 * rng.standard_normal((n, B))
    mol_ptr = np.array([0, 10, 30, 31, 95, 160])
    st = replica_energy_stats(torch.tensor(ep[1:], device="cuda"), torch.tensor(ek[1:], device="cuda"), 5e-4,
                              mol_ptr=torch.tensor(mol_ptr), epot0=torch.tensor(ep[0]), ekin0=torch.tensor(ek[0]))
    for b in range(B):
        ref = oracle_stats(ep[:, b] + ek[:, b], ek[:, b], ep[:, b], 5e-4, n_atoms=mol_ptr[b + 1] - mol_ptr[b])
        got = np.array([float(st[name][b]) for name in STAT_NAMES])
        np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12)
    # fixed-order reductions: bit-identical on a second run
    st2 = replica_energy_stats(torch.tensor(ep[1:], device="cuda"), torch.tensor(ek[1:], device="cuda"), 5e-4,
                               mol_ptr=torch.tensor(mol_ptr), epot0=torch.tensor(ep[0]), ekin0=torch.tensor(ek[0]))
    for name in STAT_NAMES:
        assert torch.equal(st[name], st2[name])


def test_reference_named_metrics():
    from mlff_gb300 import energy_metrics as em
    e = np.array([-100.0, -100.1, -100.2, -99.9])
    assert abs(em.compute_energy_drift(e) - 0.1) < 1e-9
    assert abs(em.compute_energy_drift(e, "absolute") - 0.1) < 1e-9
    assert abs(em.compute_energy_drift(e, "max_deviation") - 0.2) < 1e-9
    assert abs(em.compute_energy_conservation_ratio(e) - (1 - e.std() / abs(e.mean()))) < 1e-12
    fl = em.compute_energy_fluctuations(e)
    assert abs(fl["range"] - 0.3) < 1e-9 and abs(fl["std"] - e.std()) < 1e-12
    ke, pe = np.array([10.0, 11.0, 9.0, 10.0]), np.array([-110.0, -111.0, -109.0, -110.0])
    kp = em.compute_kinetic_potential_stability(ke, pe)
    assert abs(kp["ke_pe_correlation"] + 1.0) < 1e-12
    times = np.linspace(0, 10, 100)
    en = -100.0 + 0.01 * times
    td = em.compute_time_resolved_drift(times, en)
    assert abs(td["drift_rate"] - 0.01) < 1e-9 and abs(td["r_squared"] - 1.0) < 1e-9
    assert abs(td["initial_energy"] + 100.0) < 1e-9
    traj = {"time": list(times), "kinetic_energy": list(10.0 + 0.1 * np.sin(times)),
            "potential_energy": list(-110.0 - 0.1 * np.sin(times))}
    a = em.assess_energy_conservation(traj, tolerance_pct=1.0)
    assert a["passed"] and abs(a["energy_drift_pct"]) < 1e-9
