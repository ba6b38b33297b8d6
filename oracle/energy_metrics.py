"""ORACLE -- test infrastructure only.

The reference's energy-conservation metrics (src/mlff_distiller/testing/
energy_metrics.py) restated in numpy; the tests compare the device
statistics kernel (mlff_md_energy_stats) with it:
  drift (relative / max deviation)           energy_metrics.py:48-94
  conservation ratio 1 - std/|mean|          :97-157
  fluctuations (std, range, mean abs dev)    :160-200
  kinetic / potential stability              :203-267
  linear-fit drift rate, R^2, standard error :270-354
"""
import numpy as np

KB = 8.617333262e-5


def stats(etot: np.ndarray, ekin: np.ndarray, epot: np.ndarray, dt_ps: float, n_atoms=None) -> np.ndarray:
    """The 20 quantities of mlff_md_energy_stats for one replica."""
    e = np.asarray(etot, np.float64)
    k = np.asarray(ekin, np.float64)
    p = np.asarray(epot, np.float64)
    n = len(e)
    t = np.arange(n) * dt_ps
    e0, ef, me, sd = e[0], e[-1], e.mean(), e.std()
    drift = 100.0 * (ef - e0) / abs(e0) if abs(e0) >= 1e-10 else 0.0
    maxdev = 100.0 * np.abs(e - e0).max() / abs(e0) if abs(e0) >= 1e-10 else 0.0
    ratio = max(0.0, 1.0 - sd / abs(me)) if abs(me) >= 1e-10 else 1.0
    corr = float(np.corrcoef(k, p)[0, 1]) if k.std() > 0 and p.std() > 0 else 0.0
    part = k.mean() / abs(p.mean()) if abs(p.mean()) > 1e-10 else 0.0
    if n >= 2:
        rate, icpt = np.polyfit(t, e, 1)
        res = e - (rate * t + icpt)
    else:
        rate, res = 0.0, np.zeros(1)
    ss_tot = ((e - me) ** 2).sum()
    r2 = 1.0 - (res ** 2).sum() / ss_tot if ss_tot > 1e-10 else 1.0
    rstd = res.std() / (t.std() * np.sqrt(n)) if t.std() > 1e-10 else 0.0
    tconv = 2.0 / (3.0 * n_atoms * KB) if n_atoms else 0.0
    return np.array([e0, ef, drift, maxdev, me, sd, np.ptp(e), np.abs(e - me).mean(), ratio,
                     k.mean(), k.std(), p.mean(), p.std(), corr, part, rate, r2, rstd,
                     k.mean() * tconv, k.std() * tconv])
