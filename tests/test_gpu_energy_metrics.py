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


def _golden():
    import os
    from conftest import GOLDEN
    return np.load(os.path.join(GOLDEN, "golden_metrics.npz"))


def test_energy_metrics_vs_reference_outputs():
    """The reference-named functions against the reference's own
    energy_metrics outputs (golden_metrics.npz)."""
    from mlff_gb300 import energy_metrics as em
    g = _golden()
    # absolute 1e-10: R^2 = 1 - ss_res / ss_tot cancels where a fit explains nothing
    close = lambda a, b, key: np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-10, err_msg=key)
    for i in range(4):
        pre = f"e{i}/"
        t, k, p = g[pre + "time"], g[pre + "kinetic"], g[pre + "potential"]
        e = k + p
        close(em.compute_energy_drift(e, "relative"), g[pre + "drift_relative"], "relative")
        close(em.compute_energy_drift(e, "absolute"), g[pre + "drift_absolute"], "absolute")
        close(em.compute_energy_drift(e, "max_deviation"), g[pre + "drift_max_deviation"], "max_deviation")
        close(em.compute_energy_conservation_ratio(e), g[pre + "conservation_ratio"], "ratio")
        close(em.compute_energy_conservation_ratio(e, window=10), g[pre + "conservation_ratio_w10"], "ratio w10")
        for key, v in em.compute_energy_fluctuations(e).items():
            close(v, g[pre + "fluct/" + key], key)
        for key, v in em.compute_kinetic_potential_stability(k, p).items():
            close(v, g[pre + "kp/" + key], key)
        for key, v in em.compute_time_resolved_drift(t, e).items():
            close(v, g[pre + "trd/" + key], key)
        for key, v in em.compute_time_resolved_drift(t, e, method="cumulative").items():
            close(v, g[pre + "trc/" + key], key)
        a = em.assess_energy_conservation({"time": t, "kinetic_energy": k, "potential_energy": p})
        assert a["passed"] == bool(g[pre + "assess/passed"])
        for key in ("energy_drift_pct", "energy_drift_max_pct", "conservation_ratio"):
            close(a[key], g[pre + "assess/" + key], key)
        for key, v in a["criteria"].items():
            assert v == bool(g[pre + "assess/criteria/" + key]), key


def test_force_metrics_vs_reference_outputs():
    """Device force-accuracy statistics through the reference-named
    functions against the reference's own force_metrics outputs."""
    from mlff_gb300 import force_metrics as fm
    g = _golden()
    # absolute 1e-10: R^2 = 1 - ss_res / ss_tot cancels where a fit explains nothing
    close = lambda a, b, key: np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-10, err_msg=key)
    for i in range(3):
        pre = f"f{i}/"
        pred, ref = g[pre + "pred"], g[pre + "ref"]
        close(fm.compute_force_rmse(pred, ref), g[pre + "rmse"], "rmse")
        close(fm.compute_force_rmse(pred, ref, per_component=True), g[pre + "rmse_comp"], "rmse comp")
        close(fm.compute_force_mae(pred, ref), g[pre + "mae"], "mae")
        close(fm.compute_force_mae(pred, ref, per_component=True), g[pre + "mae_comp"], "mae comp")
        for key, v in fm.compute_force_magnitude_error(pred, ref).items():
            close(v, g[pre + "mag/" + key], key)
        close(fm.compute_angular_error(pred, ref), g[pre + "angular_median"], "angle median")
        close(fm.compute_angular_error(pred, ref, return_distribution=True), g[pre + "angular_dist"], "angles")
        for key, v in fm.compute_force_correlation(pred, ref).items():
            close(v, g[pre + "corr/" + key], key)
        if pred.ndim == 2:
            for key, v in fm.compute_per_atom_force_errors(pred, ref).items():
                close(v, g[pre + "atom/" + key], key)
        a = fm.assess_force_accuracy(torch.tensor(pred, device="cuda"), torch.tensor(ref), verbose=False)
        assert a["passed"] == bool(g[pre + "assess/passed"])
        for key, v in a["angular_percentiles"].items():
            close(v, g[pre + "assess/pct/" + key], key)
        for key, v in a["criteria"].items():
            assert v == bool(g[pre + "assess/criteria/" + key]), key
    with pytest.raises(ValueError):
        fm.compute_force_rmse(np.zeros((4, 3)), np.zeros((5, 3)))
