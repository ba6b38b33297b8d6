"""ORACLE -- test infrastructure only.

The reference's force-accuracy metrics (src/mlff_distiller/testing/
force_metrics.py) restated in numpy; pinned to the reference's own outputs
(tests/golden/golden_metrics.npz) and compared with the device statistics
(mlff_force_stats):
  component RMSE / MAE, overall and per component   force_metrics.py:46-120
  magnitude RMSE / MAE / mean relative error (%)     :123-179
  angle between vectors (degrees), |F| > 1e-6        :182-242
  per-atom errors                                    :245-306
  Pearson r, R^2, mean cosine similarity             :309-381
"""
import numpy as np

MIN_MAG = 1e-6


def metrics(pred: np.ndarray, ref: np.ndarray) -> dict:
    p = np.asarray(pred, np.float64).reshape(-1, 3)
    r = np.asarray(ref, np.float64).reshape(-1, 3)
    d = p - r
    pm, rm = np.linalg.norm(p, axis=1), np.linalg.norm(r, axis=1)
    dm = pm - rm
    nz = rm > MIN_MAG
    ok = (pm > MIN_MAG) & (rm > MIN_MAG)
    cos = (p[ok] * r[ok]).sum(axis=1) / (pm[ok] * rm[ok])
    ang = np.rad2deg(np.arccos(np.clip(cos, -1.0, 1.0)))
    pf, rf = p.ravel(), r.ravel()
    pearson = float(np.corrcoef(pf, rf)[0, 1]) if (pf.size > 1 and pf.std() > 1e-10 and rf.std() > 1e-10) else 0.0
    ss_tot = ((rf - rf.mean()) ** 2).sum()
    return {"rmse": float(np.sqrt((d ** 2).mean())), "rmse_comp": np.sqrt((d ** 2).mean(axis=0)),
            "mae": float(np.abs(d).mean()), "mae_comp": np.abs(d).mean(axis=0),
            "mag/rmse": float(np.sqrt((dm ** 2).mean())), "mag/mae": float(np.abs(dm).mean()),
            "mag/relative_error": float(100.0 * (np.abs(dm[nz]) / rm[nz]).mean()) if nz.any() else 0.0,
            "angular_dist": ang, "angular_median": float(np.median(ang)) if ang.size else 0.0,
            "corr/pearson_r": pearson,
            "corr/r_squared": float(1.0 - (d ** 2).sum() / ss_tot) if ss_tot > 1e-10 else 0.0,
            "corr/cosine_similarity": float(cos.mean()) if cos.size else 0.0}
