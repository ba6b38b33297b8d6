"""Generic ``StudentCalculator`` (models/student_calculator.py:59-580), the
dict-in / dict-out ASE calculator of the reference, on the GB300 engine.

Same constructor (``model`` instance or factory, ``model_path``,
``model_config``, ``device``, ``dtype``, ``compile``, output keys),
``implemented_properties`` (energy, forces, stress), ``n_calls``, ``reset``
and error behaviour (``ValueError`` when neither a model nor a path is
given, ``FileNotFoundError`` for a missing checkpoint, ``RuntimeError``
wrapping a failed load).

A ``StudentForceField`` model (given, built by the factory or loaded from a
checkpoint) is evaluated by one call into the CUDA library: energy, forces
and, for periodic cells, the virial stress.  Any other module is called as
the reference calls it -- ``model(input_dict)`` returning a dict with the
energy / forces / stress keys -- so the calculator still wraps foreign
student models.  ``compile`` is accepted and ignored (no tracing compiler
on this path).
"""
import warnings
from pathlib import Path
from typing import Any, Callable, Dict, List, Optional, Union

import numpy as np
import torch
import torch.nn as nn

from .ase_compat import Calculator, all_changes
from .student_model import StudentForceField


class StudentCalculator(Calculator):
    implemented_properties = ["energy", "forces", "stress"]

    def __init__(self, model: Optional[Union[nn.Module, Callable]] = None,
                 model_path: Optional[Union[str, Path]] = None, model_config: Optional[Dict[str, Any]] = None,
                 device: str = "cuda", dtype: torch.dtype = torch.float32, compile: bool = False,
                 energy_key: str = "energy", forces_key: str = "forces", stress_key: str = "stress", **kwargs):
        super().__init__(**kwargs)
        self.model_path = Path(model_path) if model_path is not None else None
        self.model_config = dict(model_config or {})
        self.device = torch.device(device)
        self.dtype = dtype
        self.compile = compile
        self.energy_key, self.forces_key, self.stress_key = energy_key, forces_key, stress_key
        self.model = self._initialize_model(model)
        self._n_calls = 0

    # ------------------------------------------------------------ model
    def _initialize_model(self, model) -> nn.Module:
        if isinstance(model, nn.Module):
            return self._ready(model)
        if callable(model):
            inst = model(**self.model_config)
            if not isinstance(inst, nn.Module):
                raise ValueError(f"Model factory must return nn.Module, got {type(inst)}")
            return self._ready(inst)
        if self.model_path is not None:
            return self._load_from_checkpoint()
        raise ValueError("Either 'model' or 'model_path' must be provided to StudentCalculator")

    def _ready(self, model: nn.Module) -> nn.Module:
        # the CUDA path computes in float32 / split fp16 whatever dtype is asked for
        model = model.to(self.device)
        if not isinstance(model, StudentForceField):
            model = model.to(self.dtype)
        model.eval()
        return model

    def _load_from_checkpoint(self) -> nn.Module:
        if not self.model_path.exists():
            raise FileNotFoundError(f"Model checkpoint not found: {self.model_path}\n"
                                    f"Please ensure the student model has been trained and saved.")
        try:
            ckpt = torch.load(self.model_path, map_location="cpu", weights_only=False)
            if not isinstance(ckpt, dict):
                raise ValueError(f"Unexpected checkpoint format: {type(ckpt)}. "
                                 "Expected dict with 'model_state_dict' or 'state_dict' key.")
            if "model_state_dict" in ckpt:
                sd = ckpt["model_state_dict"]
                if "model_config" in ckpt and not self.model_config:
                    self.model_config = dict(ckpt["model_config"])
            elif "state_dict" in ckpt:
                sd = ckpt["state_dict"]
            else:
                sd = ckpt
            cfg = dict(self.model_config)
            cls = ckpt.get("model_class") or cfg.pop("model_class", None)
            if cls is None:
                # a StudentForceField checkpoint (the reference's own format) needs no class
                if not any(k.startswith("interactions.") or k.startswith("model.interactions.") for k in sd):
                    raise ValueError("Model class must be provided in model_config when loading from "
                                     "checkpoint that doesn't include model_class information. "
                                     "Use: model_config={'model_class': YourModelClass, ...}")
                cfg.update(ckpt.get("config", {}) if isinstance(ckpt.get("config"), dict) else {})
                model = StudentForceField.from_state_dict(sd, config=cfg)
            elif cls is StudentForceField or getattr(cls, "__name__", "") == "StudentForceField":
                model = StudentForceField.from_state_dict(sd, config=cfg)
            else:
                model = cls(**cfg)
                model.load_state_dict(sd)
            return self._ready(model)
        except Exception as e:
            raise RuntimeError(f"Failed to load model from {self.model_path}: {e}") from e

    # -------------------------------------------------------- calculate
    def calculate(self, atoms=None, properties: List[str] = ("energy",), system_changes: List[str] = all_changes):
        Calculator.calculate(self, atoms, properties, system_changes)
        positions = atoms.get_positions()
        numbers = atoms.get_atomic_numbers()
        cell = np.asarray(atoms.get_cell())
        pbc = np.asarray(atoms.get_pbc())
        if isinstance(self.model, StudentForceField):
            out = self._fused(positions, numbers, cell, pbc, "stress" in properties)
        else:
            with torch.no_grad():
                out = self.model(self._prepare_input(positions, numbers, cell, pbc))
        self.results = self._extract_results(out, properties)
        self._n_calls += 1

    def _fused(self, positions, numbers, cell, pbc, want_stress: bool) -> Dict[str, torch.Tensor]:
        dev = self.device
        periodic = bool(pbc.any())
        # energy + forces take host inputs and return host results (one synchronisation)
        host = not (want_stress and periodic)
        z = torch.as_tensor(np.asarray(numbers, dtype=np.int64), device="cpu" if host else dev)
        x = torch.as_tensor(np.asarray(positions, dtype=np.float32), device="cpu" if host else dev)
        c = torch.as_tensor(cell.astype(np.float32).reshape(3, 3)) if periodic else None
        p = torch.as_tensor(pbc.astype(bool)) if periodic else None
        out: Dict[str, torch.Tensor] = {}
        if want_stress and periodic:
            E, F, V = self.model.energy_forces_virial(z, x, c, p)
            vol = abs(float(np.linalg.det(cell.astype(np.float64))))
            g = V[0].double()
            out[self.stress_key] = 0.5 * (g + g.T) / vol
        else:
            E, F = self.model.energy_and_forces(z, x, None, c, p)
            if want_stress:
                out[self.stress_key] = torch.zeros(3, 3, dtype=torch.float64)
        out[self.energy_key] = E
        out[self.forces_key] = F
        return out

    def _prepare_input(self, positions, numbers, cell, pbc) -> Dict[str, torch.Tensor]:
        """The reference's model-input dict (models/student_calculator.py:363-440)."""
        dev = self.device
        inp = {"positions": torch.as_tensor(np.asarray(positions), dtype=self.dtype, device=dev),
               "atomic_numbers": torch.as_tensor(np.asarray(numbers), dtype=torch.long, device=dev),
               "batch": torch.zeros(len(positions), dtype=torch.long, device=dev)}
        if pbc.any():
            inp["cell"] = torch.as_tensor(cell, dtype=self.dtype, device=dev)
            inp["pbc"] = torch.as_tensor(pbc, device=dev)
        return inp

    def _extract_results(self, output: Dict[str, torch.Tensor], properties) -> Dict[str, Any]:
        """ASE-format results (models/student_calculator.py:442-520)."""
        results: Dict[str, Any] = {}
        if "energy" in properties:
            e = output.get(self.energy_key)
            if e is None:
                raise KeyError(f"Model output missing '{self.energy_key}' key. Available keys: {list(output.keys())}")
            e = e.detach().cpu()
            results["energy"] = float(e.reshape(-1)[0]) if e.dim() > 0 else float(e)
        if "forces" in properties:
            f = output.get(self.forces_key)
            if f is None:
                raise KeyError(f"Model output missing '{self.forces_key}' key. Available keys: {list(output.keys())}")
            f = f.detach().cpu().numpy()
            results["forces"] = f[0] if f.ndim == 3 else f
        if "stress" in properties:
            s = output.get(self.stress_key)
            if s is not None:
                s = s.detach().cpu().numpy()
                if s.shape == (3, 3):
                    s = np.array([s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]])
                elif s.ndim == 2 and s.shape[0] > 1:
                    s = s[0]
                results["stress"] = s
            else:
                warnings.warn(f"Model output missing '{self.stress_key}' key. Stress will not be available.",
                              stacklevel=2)
        return results

    # ------------------------------------------------------------ misc
    def reset(self):
        Calculator.reset(self)

    @property
    def n_calls(self) -> int:
        return self._n_calls

    def __repr__(self) -> str:
        if self.model_path:
            return f"StudentCalculator(model_path={self.model_path}, device={self.device})"
        return f"StudentCalculator(device={self.device})"
