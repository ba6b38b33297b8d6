"""Energy-conservation metrics of MD trajectories (testing/energy_metrics.py:
48-357) computed on the device for many replicas at once.

``replica_energy_stats`` runs ``mlff_md_energy_stats`` on [n_samples, B]
potential / kinetic energy traces -- the per-step traces the GPU integrators
record, without copying them to the host -- and returns one [B] tensor per
quantity.  ``compute_energy_drift``, ``compute_energy_conservation_ratio``,
``compute_energy_fluctuations``, ``compute_kinetic_potential_stability``,
``compute_time_resolved_drift`` (linear fit) and ``assess_energy_conservation``
keep the reference's names, arguments and result keys for one trajectory
(host arrays or the NVE harness's trajectory_data) and use the same kernel.
"""
from typing import Any, Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .engine import _stream_handle

STAT_NAMES = ["initial_energy", "final_energy", "energy_drift_pct", "energy_drift_max_pct", "mean_energy",
              "std", "range", "mean_abs_dev", "conservation_ratio", "ke_mean", "ke_std", "pe_mean", "pe_std",
              "ke_pe_correlation", "energy_partition_ratio", "drift_rate", "r_squared", "drift_rate_std",
              "avg_temperature", "std_temperature"]


def replica_energy_stats(epot: torch.Tensor, ekin: torch.Tensor, dt_ps: float,
                         mol_ptr: Optional[torch.Tensor] = None, epot0: Optional[torch.Tensor] = None,
                         ekin0: Optional[torch.Tensor] = None) -> Dict[str, torch.Tensor]:
    """Statistics per replica of device traces epot, ekin [n_steps, B]
    (float64, eV) sampled dt_ps apart; epot0 / ekin0 [B] (optional) are the
    energies before the first step, prepended as sample 0."""
    dev = epot.device
    if dev.type != "cuda":
        raise RuntimeError("replica_energy_stats runs on a CUDA device")
    p = epot.to(torch.float64).reshape(epot.shape[0], -1)
    k = ekin.to(torch.float64).reshape(ekin.shape[0], -1)
    if epot0 is not None:
        p = torch.cat([epot0.to(device=dev, dtype=torch.float64).reshape(1, -1), p])
        k = torch.cat([ekin0.to(device=dev, dtype=torch.float64).reshape(1, -1), k])
    p, k = p.contiguous(), k.contiguous()
    n, B = p.shape
    out = torch.empty(B, len(STAT_NAMES), dtype=torch.float64, device=dev)
    mp = None if mol_ptr is None else torch.as_tensor(mol_ptr, dtype=torch.int64, device=dev).contiguous()
    _lib.check(_lib.load().mlff_md_energy_stats(p.data_ptr(), k.data_ptr(), n, B, _lib.ptr(mp), float(dt_ps),
                                                out.data_ptr(), _stream_handle()))
    return {name: out[:, i] for i, name in enumerate(STAT_NAMES)}


def _one(energies: Sequence[float], kinetic=None, potential=None, dt_ps: float = 1.0) -> Dict[str, float]:
    e = torch.as_tensor(np.asarray(energies, np.float64), device="cuda")
    if kinetic is None:
        k, p = torch.zeros_like(e), e
    else:
        k = torch.as_tensor(np.asarray(kinetic, np.float64), device="cuda")
        p = torch.as_tensor(np.asarray(potential, np.float64), device="cuda")
    st = replica_energy_stats(p.reshape(-1, 1), k.reshape(-1, 1), dt_ps)
    return {name: float(v[0]) for name, v in st.items()}


def compute_energy_drift(energies: np.ndarray, method: str = "relative") -> float:
    """energy_metrics.py:48-94 ('relative' %, 'absolute' eV, 'max_deviation' %)."""
    if len(energies) < 2:
        raise ValueError(f"Need at least 2 energy values, got {len(energies)}")
    s = _one(energies)
    if method == "relative":
        return s["energy_drift_pct"]
    if method == "absolute":
        return s["final_energy"] - s["initial_energy"]
    if method == "max_deviation":
        return s["energy_drift_max_pct"]
    raise ValueError(f"Unknown drift method: {method}")


def compute_energy_conservation_ratio(energies: np.ndarray, window: Optional[int] = None) -> float:
    """energy_metrics.py:97-157: 1 - std/|mean|, clamped at 0, over the whole
    trajectory or averaged over rolling windows of ``window`` samples
    (windows whose mean is within 1e-10 of zero are skipped)."""
    if len(energies) < 2:
        raise ValueError(f"Need at least 2 energy values, got {len(energies)}")
    if window is not None and window > len(energies):
        window = None
    if window is None:
        return _one(energies)["conservation_ratio"]
    e = torch.as_tensor(np.asarray(energies, np.float64), device="cuda")
    w = e.unfold(0, int(window), 1)                  # [n - window + 1, window] rolling windows
    mean = w.mean(dim=1)
    std = w.std(dim=1, unbiased=False)
    keep = mean.abs() > 1e-10
    if not bool(keep.any()):
        return 1.0
    return float(torch.clamp(1.0 - std[keep] / mean[keep].abs(), min=0.0).mean())


def compute_energy_fluctuations(energies: np.ndarray) -> Dict[str, float]:
    """energy_metrics.py:160-200."""
    if len(energies) < 2:
        raise ValueError(f"Need at least 2 energy values, got {len(energies)}")
    s = _one(energies)
    cv = s["std"] / abs(s["mean_energy"]) if abs(s["mean_energy"]) > 1e-10 else 0.0
    return {"std": s["std"], "range": s["range"], "mean_abs_dev": s["mean_abs_dev"], "coefficient_of_variation": cv}


def compute_kinetic_potential_stability(kinetic_energies: np.ndarray, potential_energies: np.ndarray) -> Dict[str, float]:
    """energy_metrics.py:203-267."""
    if len(kinetic_energies) != len(potential_energies):
        raise ValueError(f"Kinetic and potential energy arrays must have same length: "
                         f"{len(kinetic_energies)} vs {len(potential_energies)}")
    if len(kinetic_energies) < 2:
        raise ValueError(f"Need at least 2 energy values, got {len(kinetic_energies)}")
    k, p = np.asarray(kinetic_energies, np.float64), np.asarray(potential_energies, np.float64)
    s = _one(k + p, k, p)
    return {key: s[key] for key in ("ke_mean", "ke_std", "pe_mean", "pe_std", "ke_pe_correlation",
                                    "energy_partition_ratio")}


def compute_time_resolved_drift(times: np.ndarray, energies: np.ndarray, method: str = "linear_fit") -> Dict[str, Any]:
    """energy_metrics.py:270-354: 'linear_fit' (drift rate, its standard
    error, R^2, total drift, fitted initial energy; uniformly spaced times) or
    'cumulative' (average rate, total and largest drift from the first
    sample, the drift series)."""
    if len(times) != len(energies):
        raise ValueError(f"Times and energies must have same length: {len(times)} vs {len(energies)}")
    if len(times) < 3:
        raise ValueError(f"Need at least 3 data points for drift analysis, got {len(times)}")
    t = np.asarray(times, np.float64)
    if method == "cumulative":
        e = torch.as_tensor(np.asarray(energies, np.float64), device="cuda")
        cum = e - e[0]
        span = float(t[-1] - t[0])
        total = float(cum[-1])
        return {"drift_rate": total / span if span > 1e-10 else 0.0, "total_drift": total,
                "max_drift": float(cum.abs().max()), "cumulative_drift": cum.cpu().numpy()}
    if method != "linear_fit":
        raise ValueError(f"Unknown method: {method}")
    s = _one(energies, dt_ps=float(t[1] - t[0]))
    return {"drift_rate": s["drift_rate"], "drift_rate_std": s["drift_rate_std"], "r_squared": s["r_squared"],
            "total_drift": s["final_energy"] - s["initial_energy"],
            "initial_energy": s["mean_energy"] - s["drift_rate"] * 0.5 * (t[-1] - t[0]) - s["drift_rate"] * t[0]}


def assess_energy_conservation(trajectory_data: Dict[str, List], tolerance_pct: float = 1.0,
                               verbose: bool = False) -> Dict[str, Any]:
    """energy_metrics.py:357-460: all metrics of a harness trajectory and the
    pass/fail criteria (drift within tolerance, max drift within 1.5x,
    conservation ratio >= 0.99, KE-PE anti-correlated)."""
    times = np.asarray(trajectory_data["time"], np.float64)
    k = np.asarray(trajectory_data["kinetic_energy"], np.float64)
    p = np.asarray(trajectory_data["potential_energy"], np.float64)
    dt = float(times[1] - times[0]) if len(times) > 1 else 1.0
    s = _one(k + p, k, p, dt_ps=dt)
    cv = s["std"] / abs(s["mean_energy"]) if abs(s["mean_energy"]) > 1e-10 else 0.0
    criteria = {"drift_within_tolerance": abs(s["energy_drift_pct"]) <= tolerance_pct,
                "max_drift_within_tolerance": s["energy_drift_max_pct"] <= tolerance_pct * 1.5,
                "conservation_ratio_good": s["conservation_ratio"] >= 0.99,
                "ke_pe_anticorrelated": s["ke_pe_correlation"] < 0}
    out = {"passed": all(criteria.values()), "energy_drift_pct": s["energy_drift_pct"],
           "energy_drift_max_pct": s["energy_drift_max_pct"], "conservation_ratio": s["conservation_ratio"],
           "fluctuation_stats": {"std": s["std"], "range": s["range"], "mean_abs_dev": s["mean_abs_dev"],
                                 "coefficient_of_variation": cv},
           "ke_pe_stability": {key: s[key] for key in ("ke_mean", "ke_std", "pe_mean", "pe_std",
                                                       "ke_pe_correlation", "energy_partition_ratio")},
           "time_resolved_drift": {"drift_rate": s["drift_rate"], "drift_rate_std": s["drift_rate_std"],
                                   "r_squared": s["r_squared"], "total_drift": s["final_energy"] - s["initial_energy"]},
           "criteria": criteria, "tolerance_pct": tolerance_pct}
    if verbose:
        print(f"energy drift {s['energy_drift_pct']:.4f} %  conservation ratio {s['conservation_ratio']:.6f}  "
              f"{'PASSED' if out['passed'] else 'FAILED'}")
    return out
