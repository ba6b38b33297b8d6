"""Force-accuracy metrics (testing/force_metrics.py:46-513) computed on the
device.

``force_stats`` runs ``mlff_force_stats`` over predicted and reference force
vectors -- [n_atoms, 3] or [n_frames, n_atoms, 3], numpy arrays or torch
tensors on any device -- and returns the sums every metric needs plus,
optionally, the per-vector errors.  The functions below keep the reference's
names, arguments, return types and result keys: ``compute_force_rmse``,
``compute_force_mae``, ``compute_force_magnitude_error``,
``compute_angular_error``, ``compute_per_atom_force_errors``,
``compute_force_correlation`` and ``assess_force_accuracy``.  Magnitudes at
or below 1e-6 eV/A have no direction and are left out of the angular
statistics, as in the reference.
"""
from __future__ import annotations

import logging
import math
from typing import Any, Dict

import numpy as np
import torch

from . import _lib
from .engine import _stream_handle

logger = logging.getLogger(__name__)

N_STATS = 20


def _as_device(x) -> torch.Tensor:
    t = torch.as_tensor(x)
    return t.to(device="cuda", dtype=torch.float64).reshape(-1, 3).contiguous()


def _check(pred, ref):
    ps, rs = tuple(pred.shape), tuple(ref.shape)
    if ps != rs:
        raise ValueError(f"Force arrays must have same shape: {ps} vs {rs}")
    if not ps or ps[-1] != 3:
        raise ValueError(f"Expected force arrays [..., 3], got {ps}")


def force_stats(pred, ref, per_vector: bool = False):
    """(stats [20] float64 device tensor, per_vector [n, 4] or None); see
    mlff_force_stats for the layout."""
    if not torch.cuda.is_available():
        raise RuntimeError("force metrics run on a CUDA device (GB300); none is available")
    _check(pred, ref)
    p, r = _as_device(pred), _as_device(ref)
    lib = _lib.load()
    n = p.shape[0]
    stats = torch.empty(N_STATS, dtype=torch.float64, device="cuda")
    pv = torch.empty(n, 4, dtype=torch.float64, device="cuda") if per_vector else None
    ws = torch.empty(lib.mlff_force_stats_workspace_size(), dtype=torch.uint8, device="cuda")
    _lib.check(lib.mlff_force_stats(p.data_ptr(), r.data_ptr(), n, stats.data_ptr(), _lib.ptr(pv), ws.data_ptr(),
                                    ws.numel(), _stream_handle()))
    return stats, pv


def _host(stats: torch.Tensor) -> np.ndarray:
    return stats.cpu().numpy()


def compute_force_rmse(predicted_forces, reference_forces, per_component: bool = False):
    """force_metrics.py:46-83: sqrt(mean squared component error), overall
    or per component (x, y, z)."""
    s = _host(force_stats(predicted_forces, reference_forces)[0])
    n = max(s[0], 1.0)
    if per_component:
        return np.sqrt(s[1:4] / n)
    return float(math.sqrt(s[1:4].sum() / (3 * n)))


def compute_force_mae(predicted_forces, reference_forces, per_component: bool = False):
    """force_metrics.py:86-120: mean absolute component error."""
    s = _host(force_stats(predicted_forces, reference_forces)[0])
    n = max(s[0], 1.0)
    if per_component:
        return s[4:7] / n
    return float(s[4:7].sum() / (3 * n))


def _magnitude(s: np.ndarray) -> Dict[str, float]:
    n = max(s[0], 1.0)
    rel = 100.0 * s[9] / s[10] if s[10] > 0 else 0.0
    return {"rmse": float(math.sqrt(s[7] / n)), "mae": float(s[8] / n), "relative_error": float(rel)}


def compute_force_magnitude_error(predicted_forces, reference_forces) -> Dict[str, float]:
    """force_metrics.py:123-179: RMSE and MAE of |F_pred| - |F_ref|, mean
    relative error (%) over |F_ref| > 1e-6."""
    return _magnitude(_host(force_stats(predicted_forces, reference_forces)[0]))


def _angles(pv: torch.Tensor) -> torch.Tensor:
    a = pv[:, 3]
    return a[~torch.isnan(a)]


def compute_angular_error(predicted_forces, reference_forces, return_distribution: bool = False):
    """force_metrics.py:182-242: median angle (degrees) between predicted and
    reference vectors, or all angles with return_distribution."""
    _, pv = force_stats(predicted_forces, reference_forces, per_vector=True)
    a = _angles(pv)
    if a.numel() == 0:
        logger.warning("No valid force vectors for angular error computation (all forces near zero)")
        return np.array([]) if return_distribution else 0.0
    if return_distribution:
        return a.cpu().numpy()
    return float(torch.quantile(a, 0.5))


def compute_per_atom_force_errors(predicted_forces, reference_forces) -> Dict[str, np.ndarray]:
    """force_metrics.py:245-306: per-atom RMSE, MAE, magnitude error and
    angular error (0 where undefined) of [n_atoms, 3] arrays."""
    _check(predicted_forces, reference_forces)
    if len(tuple(predicted_forces.shape)) != 2:
        raise ValueError(f"Expected shape [n_atoms, 3], got {tuple(predicted_forces.shape)}")
    _, pv = force_stats(predicted_forces, reference_forces, per_vector=True)
    h = pv.cpu().numpy()
    return {"rmse": h[:, 0], "mae": h[:, 1], "magnitude_error": h[:, 2], "angular_error": np.nan_to_num(h[:, 3])}


def _correlation(s: np.ndarray) -> Dict[str, float]:
    m = 3.0 * s[0]
    if m < 1:
        return {"pearson_r": 0.0, "r_squared": 0.0, "cosine_similarity": 0.0}
    mp, mr = s[13] / m, s[14] / m
    var_p = max(s[15] / m - mp * mp, 0.0)
    var_r = max(s[16] / m - mr * mr, 0.0)
    cov = s[17] / m - mp * mr
    pearson = cov / math.sqrt(var_p * var_r) if (m > 1 and math.sqrt(var_p) > 1e-10 and math.sqrt(var_r) > 1e-10) \
        else 0.0
    ss_res = s[1:4].sum()
    ss_tot = var_r * m
    r2 = 1.0 - ss_res / ss_tot if ss_tot > 1e-10 else 0.0
    cos = s[12] / s[11] if s[11] > 0 else 0.0
    return {"pearson_r": float(pearson), "r_squared": float(r2), "cosine_similarity": float(cos)}


def compute_force_correlation(predicted_forces, reference_forces) -> Dict[str, float]:
    """force_metrics.py:309-381: Pearson r and R^2 over all components, mean
    cosine similarity over vectors with a direction."""
    return _correlation(_host(force_stats(predicted_forces, reference_forces)[0]))


def assess_force_accuracy(predicted_forces, reference_forces, rmse_tolerance: float = 0.2,
                          mae_tolerance: float = 0.15, angular_tolerance: float = 15.0,
                          verbose: bool = True) -> Dict[str, Any]:
    """force_metrics.py:384-500: every metric from one device pass, the
    pass/fail criteria (RMSE, MAE, median angle within tolerance, R^2 >=
    0.9) and the angular percentiles."""
    st, pv = force_stats(predicted_forces, reference_forces, per_vector=True)
    s = _host(st)
    n = max(s[0], 1.0)
    rmse = float(math.sqrt(s[1:4].sum() / (3 * n)))
    mae = float(s[4:7].sum() / (3 * n))
    a = _angles(pv)
    if a.numel():
        q = torch.quantile(a, torch.tensor([0.5, 0.75, 0.9, 0.95], dtype=torch.float64, device=a.device)).tolist()
    else:
        q = [0.0, 0.0, 0.0, 0.0]
    corr = _correlation(s)
    criteria = {"rmse_within_tolerance": rmse <= rmse_tolerance, "mae_within_tolerance": mae <= mae_tolerance,
                "angular_error_acceptable": q[0] <= angular_tolerance, "high_correlation": corr["r_squared"] >= 0.9}
    out = {"passed": all(criteria.values()), "rmse": rmse, "mae": mae, "magnitude_errors": _magnitude(s),
           "angular_error_median": q[0],
           "angular_percentiles": {"p50": q[0], "p75": q[1], "p90": q[2], "p95": q[3]},
           "correlation": corr, "criteria": criteria,
           "tolerances": {"rmse": rmse_tolerance, "mae": mae_tolerance, "angular": angular_tolerance},
           "max_component_error": float(s[18])}
    if verbose:
        logger.info("force accuracy over %d vectors: RMSE %.4f eV/A, MAE %.4f eV/A, median angle %.2f deg, "
                    "R^2 %.6f -> %s", int(s[0]), rmse, mae, q[0], corr["r_squared"],
                    "PASSED" if out["passed"] else "FAILED")
    return out


__all__ = ["force_stats", "compute_force_rmse", "compute_force_mae", "compute_force_magnitude_error",
           "compute_angular_error", "compute_per_atom_force_errors", "compute_force_correlation",
           "assess_force_accuracy"]
