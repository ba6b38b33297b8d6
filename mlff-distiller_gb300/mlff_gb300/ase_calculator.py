"""Drop-in ``StudentForceFieldCalculator`` (inference/ase_calculator.py:
57-890) on the GB300 engine.

Same constructor arguments, ``implemented_properties``, results
(``energy`` float eV, ``forces`` (N, 3) eV/A, ``stress`` Voigt (6,) eV/A^3),
``calculate_batch``, ``n_calls`` / ``avg_time`` / ``get_timing_stats`` /
``reset`` and error behaviour: ``ValueError`` for invalid input is re-raised
as is, anything else is wrapped in ``RuntimeError``, and a missing
checkpoint raises ``FileNotFoundError``.  Energies and forces come from one
call into the CUDA library (neighbour list, model and hand-written force
adjoint); there is no CPU path.

Differences, all on the side of the physics: periodic cells are honoured
(orthorhombic, all three axes periodic) in ``calculate`` and
``calculate_batch``, and ``stress`` is the virial stress of the periodic
model instead of zeros.
"""
import logging
import time
import warnings
from pathlib import Path
from typing import Any, Dict, List, Optional, Union

import numpy as np
import torch

from .ase_compat import Atoms, Calculator, all_changes
from .student_model import StudentForceField

logger = logging.getLogger(__name__)

_PRECISIONS = ("fp16x3", "tuned_fp32", "fp32")


class StudentForceFieldCalculator(Calculator):
    """ASE calculator for ``StudentForceField`` checkpoints.

    ``precision`` (extra keyword, default ``"fp16x3"``) selects the CUDA
    path: ``"fp16x3"`` tensor-core split-FP16 filters, ``"tuned_fp32"``
    fused CUDA-core FP32, ``"fp32"`` the plain per-op FP32 path.
    ``use_fp16`` is accepted for compatibility (the tensor-core path is the
    default already); ``use_compile`` is accepted and ignored (there is no
    tracing compiler on this path); ``use_analytical_forces`` is always in
    effect (forces come from the hand-written adjoint)."""

    def __init__(self, checkpoint_path: Union[str, Path], device: str = "cuda",
                 dtype: torch.dtype = torch.float32, enable_stress: bool = False,
                 batch_size: Optional[int] = None, enable_timing: bool = False,
                 use_compile: bool = False, use_fp16: bool = False, use_jit: bool = False,
                 jit_path: Optional[Union[str, Path]] = None, use_torch_cluster: bool = True,
                 use_analytical_forces: bool = False, precision: str = "fp16x3", **kwargs):
        super().__init__(**kwargs)
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {_PRECISIONS}, got {precision!r}")
        self.checkpoint_path = Path(checkpoint_path)
        self.device = torch.device(device)
        self.dtype = dtype
        self.enable_stress = enable_stress
        self.batch_size = batch_size
        self.enable_timing = enable_timing
        self.use_compile = use_compile
        self.use_fp16 = use_fp16
        self.use_jit = use_jit
        self.jit_path = Path(jit_path) if jit_path else None
        self.use_torch_cluster = use_torch_cluster
        self.use_analytical_forces = use_analytical_forces
        self.precision = precision
        self.implemented_properties = ["energy", "forces"]
        if self.enable_stress:
            self.implemented_properties.append("stress")
        if use_compile:
            logger.info("use_compile is ignored: the GB300 path runs hand-written CUDA kernels")
        self.model = self._load_model()
        self._n_calls = 0
        self._total_time = 0.0
        self._call_times: List[float] = []

    # ------------------------------------------------------------------ model
    def _load_model(self) -> StudentForceField:
        """Checkpoint (or TorchScript archive) -> StudentForceField on the
        device (ase_calculator.py:204-277)."""
        if self.use_jit:
            if not self.jit_path:
                raise ValueError("use_jit=True but jit_path not provided")
            if not self.jit_path.exists():
                raise FileNotFoundError(f"TorchScript model not found: {self.jit_path}")
            try:
                scripted = torch.jit.load(str(self.jit_path), map_location="cpu")
                sd = {k: v for k, v in scripted.state_dict().items()}
                model = StudentForceField.from_state_dict(sd, precision=self.precision)
                return model.to(self.device).eval()
            except Exception as e:
                raise RuntimeError(f"Failed to load TorchScript model from {self.jit_path}: {e}") from e
        if not self.checkpoint_path.exists():
            raise FileNotFoundError(f"Checkpoint not found: {self.checkpoint_path}\n"
                                    f"Please ensure the model has been trained and checkpoint saved.")
        try:
            model = StudentForceField.load(self.checkpoint_path, device="cpu", precision=self.precision)
            model.use_torch_cluster = self.use_torch_cluster
            model.eval()
            return model.to(self.device)
        except Exception as e:
            raise RuntimeError(f"Failed to load model from {self.checkpoint_path}: {e}") from e

    # ------------------------------------------------------------- validation
    @staticmethod
    def _validate_inputs(positions, numbers, cell, pbc):
        """ase_calculator.py:414-459."""
        if len(positions) == 0:
            raise ValueError("Cannot calculate properties for empty structure")
        if np.any(numbers < 1) or np.any(numbers > 118):
            raise ValueError(f"Invalid atomic numbers: must be 1-118, got {numbers}")
        if not np.isfinite(positions).all():
            raise ValueError("Positions contain NaN or Inf values")
        if np.asarray(pbc).any():
            if not np.isfinite(cell).all():
                raise ValueError("Cell contains NaN or Inf values")
            volume = abs(np.linalg.det(np.asarray(cell, dtype=np.float64).reshape(3, 3)))
            if volume < 1e-6:
                warnings.warn(f"Cell volume very small ({volume:.2e} A^3), may indicate degenerate cell",
                              stacklevel=3)

    def _host_inputs(self, numbers, positions):
        """Atomic numbers and positions in pinned host buffers reused from
        call to call (the model copies them straight into its CUDA graph's
        input buffers)."""
        n = len(numbers)
        buf = getattr(self, "_pinned", None)
        if buf is None or buf[0].shape[0] != n:
            buf = (torch.empty(n, dtype=torch.int64).pin_memory(), torch.empty(n, 3, dtype=torch.float32).pin_memory())
            self._pinned = buf
        buf[0].numpy()[:] = np.asarray(numbers, dtype=np.int64)
        buf[1].numpy()[:] = np.asarray(positions)
        return buf

    def _tensors(self, positions, numbers, cell, pbc, host: bool = False):
        dev = self.device
        if host and dev.type == "cuda":
            z, x = self._host_inputs(numbers, positions)
        else:
            z = torch.as_tensor(np.asarray(numbers, dtype=np.int64), device=dev)
            x = torch.as_tensor(np.asarray(positions, dtype=np.float32), device=dev)
        periodic = bool(np.asarray(pbc).any())
        # cell and pbc stay on the host: the model checks them there without a device sync
        c = torch.as_tensor(np.asarray(cell, dtype=np.float32).reshape(3, 3)) if periodic else None
        p = torch.as_tensor(np.asarray(pbc, dtype=bool)) if periodic else None
        return z, x, c, p

    # -------------------------------------------------------------- calculate
    def calculate(self, atoms: Optional[Atoms] = None, properties: List[str] = ("energy", "forces"),
                  system_changes: List[str] = all_changes):
        """ase_calculator.py:279-412."""
        Calculator.calculate(self, atoms, properties, system_changes)
        t0 = time.perf_counter()
        try:
            positions = atoms.get_positions()
            numbers = atoms.get_atomic_numbers()
            cell = np.asarray(atoms.get_cell())
            pbc = np.asarray(atoms.get_pbc())
            self._validate_inputs(positions, numbers, cell, pbc)
            want_stress = "stress" in properties and self.enable_stress
            # energy + forces: host buffers in, host results out (one synchronisation)
            z, x, c, p = self._tensors(positions, numbers, cell, pbc, host=not want_stress)
            E, F, V = self.model.energy_forces_virial(z, x, c, p) if want_stress else \
                (*self.model.energy_and_forces(z, x, None, c, p), None)
            results: Dict[str, Any] = {"energy": float(E.sum().item()),
                                       "forces": F.detach().cpu().numpy().astype(np.float64)}
            if want_stress:
                results["stress"] = self._stress(V, cell, pbc)
            self.results = results
            self._n_calls += 1
            if self.enable_timing:
                dt = time.perf_counter() - t0
                self._total_time += dt
                self._call_times.append(dt)
        except ValueError:
            raise
        except Exception as e:
            logger.error(f"Calculation failed: {e}")
            raise RuntimeError(f"Failed to calculate properties for {len(atoms)} atoms: {e}") from e

    @staticmethod
    def _stress(V, cell, pbc) -> np.ndarray:
        """Voigt stress (xx, yy, zz, yz, xz, xy) = sym(dE/d strain) / volume;
        zeros for a non-periodic structure (what the reference returns,
        ase_calculator.py:521-588)."""
        if V is None or not np.asarray(pbc).any():
            return np.zeros(6)
        g = V[0].detach().cpu().numpy().astype(np.float64)
        g = 0.5 * (g + g.T)
        vol = abs(np.linalg.det(np.asarray(cell, dtype=np.float64).reshape(3, 3)))
        s = g / vol
        return np.array([s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]])

    def calculate_batch(self, atoms_list: List[Atoms], properties: List[str] = ("energy", "forces")
                        ) -> List[Dict[str, Any]]:
        """All structures in one library call (ase_calculator.py:590-817)."""
        if not atoms_list:
            return []
        if len(atoms_list) == 1:
            atoms = atoms_list[0]
            atoms.calc = self
            return [{
                "energy": atoms.get_potential_energy() if "energy" in properties else None,
                "forces": atoms.get_forces() if "forces" in properties else None,
                "stress": atoms.get_stress() if "stress" in properties and self.enable_stress else None,
            }]
        try:
            pos, num, counts, cells, pbcs = [], [], [], [], []
            for a in atoms_list:
                p, n = a.get_positions(), a.get_atomic_numbers()
                c, b = np.asarray(a.get_cell()), np.asarray(a.get_pbc())
                self._validate_inputs(p, n, c, b)
                pos.append(p); num.append(n); counts.append(len(n)); cells.append(c); pbcs.append(b)
            periodic = [bool(b.any()) for b in pbcs]
            if any(periodic) and not all(periodic):
                raise ValueError("calculate_batch needs all structures periodic or all non-periodic")
            z, x = self._host_inputs(np.concatenate(num), np.concatenate(pos)) if self.device.type == "cuda" else \
                (torch.as_tensor(np.concatenate(num).astype(np.int64)),
                 torch.as_tensor(np.concatenate(pos).astype(np.float32)))
            # structure index, cells and pbc flags on the host (checked there, no device sync)
            bidx = torch.as_tensor(np.repeat(np.arange(len(atoms_list), dtype=np.int64), counts))
            c = p = None
            if all(periodic):
                c = torch.as_tensor(np.stack(cells).astype(np.float32))
                p = torch.as_tensor(np.stack(pbcs))
            E, F = self.model.energy_and_forces(z, x, bidx, c, p)
            E = E.detach().cpu().numpy()
            F = F.detach().cpu().numpy().astype(np.float64)
        except ValueError:
            raise
        except Exception as e:
            raise RuntimeError(f"Failed to calculate batch of {len(atoms_list)} structures: {e}") from e
        out, off = [], 0
        for i, n in enumerate(counts):
            r: Dict[str, Any] = {}
            if "energy" in properties:
                r["energy"] = float(E[i])
            if "forces" in properties:
                r["forces"] = F[off:off + n]
            if "stress" in properties and self.enable_stress:
                r["stress"] = None   # as the reference's batch path (ase_calculator.py:806-808)
            out.append(r)
            off += n
        self._n_calls += 1
        return out

    # ------------------------------------------------------------- bookkeeping
    def reset(self):
        Calculator.reset(self)

    @property
    def n_calls(self) -> int:
        return self._n_calls

    @property
    def avg_time(self) -> float:
        return self._total_time / self._n_calls if self._n_calls else 0.0

    def get_timing_stats(self) -> Dict[str, float]:
        if not self._call_times:
            return {"n_calls": 0, "total_time": 0.0, "avg_time": 0.0, "min_time": 0.0, "max_time": 0.0,
                    "median_time": 0.0}
        t = np.asarray(self._call_times)
        return {"n_calls": self._n_calls, "total_time": self._total_time, "avg_time": float(t.mean()),
                "min_time": float(t.min()), "max_time": float(t.max()), "median_time": float(np.median(t)),
                "std_time": float(t.std())}

    def __repr__(self) -> str:
        return (f"StudentForceFieldCalculator(checkpoint={self.checkpoint_path.name}, "
                f"device={self.device}, calls={self._n_calls})")


__all__ = ["StudentForceFieldCalculator"]
