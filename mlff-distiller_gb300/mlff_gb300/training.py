"""Training of the StudentForceField on the GPU with the library's own
forward and reverse kernels.

``param_grads`` returns sum_b w_b dE_b/dtheta for every trainable tensor
of the state_dict from one call of ``mlff_param_grads`` (plain FP32 path:
per-op forward, hand-written reverse pass with the weight-gradient
reductions), the parameter part of ``loss.backward()`` in
Trainer.train_epoch (training/trainer.py:288-393) for an energy loss.

``EnergyTrainer`` is the optimisation step around it with the reference's
defaults (configs/train_student.yaml: AdamW, lr 1e-3, weight decay 1e-5,
betas (0.9, 0.999), eps 1e-8, gradient-norm clip 1.0) and the energy
term of ForceFieldLoss (training/losses.py:106-246: mean squared error of
the per-structure energies).  The force term of that loss needs the
gradient of the forces with respect to the parameters (a second-order
reverse pass) and is not part of this module.
"""
import ctypes
from typing import Dict, Optional, Tuple

import numpy as np
import torch

from . import _lib
from .engine import Batch, _stream_handle, make_batch

_LAYER_KEYS = {
    "filter_w1": "message.rbf_to_scalar.0.weight", "filter_b1": "message.rbf_to_scalar.0.bias",
    "filter_w2": "message.rbf_to_scalar.2.weight", "filter_b2": "message.rbf_to_scalar.2.bias",
    "mixing": "update.mixing_matrix", "update_w1": "update.update_mlp.0.weight",
    "update_b1": "update.update_mlp.0.bias", "update_w2": "update.update_mlp.2.weight",
    "update_b2": "update.update_mlp.2.bias",
}
_HEAD_KEYS = {"head_w1": "energy_head.0.weight", "head_b1": "energy_head.0.bias",
              "head_w2": "energy_head.2.weight", "head_b2": "energy_head.2.bias",
              "head_w3": "energy_head.4.weight", "head_b3": "energy_head.4.bias"}


def trainable_names(model) -> list:
    return [n for n, p in model.named_parameters() if p.requires_grad]


def param_grads(model, batch: Batch, weights: torch.Tensor, forces: bool = False
                ) -> Tuple[torch.Tensor, Dict[str, torch.Tensor], Optional[torch.Tensor]]:
    """Energies [B] (float64), {name: sum_b w_b dE_b/d(name)} for every
    trainable parameter (float32, state_dict shapes) and, if asked,
    -sum_b w_b dE_b/dpos."""
    eng = model.engine()
    dev = eng.device
    N, B = batch.n_atoms, batch.n_mol
    w = torch.as_tensor(weights, dtype=torch.float64, device=dev).contiguous()
    if w.shape != (B,):
        raise ValueError(f"weights must have shape ({B},), got {tuple(w.shape)}")
    params = dict(model.named_parameters())
    grads = {n: torch.zeros_like(p, dtype=torch.float32, device=dev) for n, p in params.items() if p.requires_grad}
    g = _lib.Grads()
    g.embedding = _lib.ptr(grads.get("embedding.weight"))
    for l in range(model.num_interactions):
        for field, key in _LAYER_KEYS.items():
            getattr(g, field)[l] = _lib.ptr(grads.get(f"interactions.{l}.{key}"))
    for field, key in _HEAD_KEYS.items():
        setattr(g, field, _lib.ptr(grads.get(key)))
    E = torch.empty(B, dtype=torch.float64, device=dev)
    F = torch.empty(N, 3, dtype=torch.float32, device=dev) if forces else None
    out = _lib.Outputs()
    out.energy, out.forces, out.virial, out.atom_energy = E.data_ptr(), _lib.ptr(F), None, None
    sysd = batch.system()
    path = _lib.PATH_TRAIN
    for _ in range(4):
        cap = eng.capacity(N, path)
        ws = eng.workspace_for(N, B, cap, path)
        _lib.check(eng.lib.mlff_param_grads(ctypes.byref(eng.dims), eng.packed.data_ptr(), ctypes.byref(sysd), cap,
                                            w.data_ptr(), ctypes.byref(g), ctypes.byref(out), ws.data_ptr(),
                                            ws.numel(), _stream_handle()))
        code, n_edges, where = eng.status()
        if code == _lib.ERR_CAPACITY:
            eng.edge_capacity[path] = int(n_edges * 1.25) + 1024
            continue
        if code != _lib.OK:
            raise _lib.MLFFError(code, f"device status {code} at index {where}")
        eng.edge_capacity[path] = max(eng.edge_capacity.get(path, 0), int(n_edges * 1.15) + 1024)
        break
    else:
        raise _lib.MLFFError(_lib.ERR_CAPACITY, "edge capacity did not converge")
    return E, grads, F


class EnergyTrainer:
    """One optimisation step per call: energies, loss, parameter gradients
    from the CUDA reverse pass, gradient clipping and AdamW."""

    def __init__(self, model, lr: float = 1e-3, weight_decay: float = 1e-5, betas=(0.9, 0.999),
                 eps: float = 1e-8, grad_clip: float = 1.0, per_atom: bool = False):
        self.model = model
        self.opt = torch.optim.AdamW([p for p in model.parameters() if p.requires_grad], lr=lr,
                                     weight_decay=weight_decay, betas=betas, eps=eps)
        self.grad_clip = grad_clip
        self.per_atom = per_atom
        self.steps = 0

    def loss_weights(self, E: torch.Tensor, E_ref: torch.Tensor, n_atoms: torch.Tensor):
        """MSE of energies (or of energies per atom): loss and dL/dE_b."""
        B = E.shape[0]
        if self.per_atom:
            r = (E - E_ref) / n_atoms
            return (r * r).mean(), 2.0 * r / n_atoms / B
        r = E - E_ref
        return (r * r).mean(), 2.0 * r / B

    def step(self, batch: Batch, E_ref) -> float:
        dev = batch.Z.device
        E_ref = torch.as_tensor(E_ref, dtype=torch.float64, device=dev)
        n_atoms = (batch.mol_ptr[1:] - batch.mol_ptr[:-1]).to(torch.float64)
        # the loss weights need this step's energies: an energy-only forward first
        E0, _, _ = self.model.engine().energy_forces(batch, _lib.PATH_PLAIN_FP32, forces=False)
        loss, w = self.loss_weights(E0, E_ref, n_atoms)
        E, grads, _ = param_grads(self.model, batch, w)
        for n, p in self.model.named_parameters():
            if p.requires_grad:
                p.grad = grads[n].to(p.dtype)
        if self.grad_clip:
            torch.nn.utils.clip_grad_norm_(self.model.parameters(), self.grad_clip)
        self.opt.step()
        self.opt.zero_grad(set_to_none=True)
        self.steps += 1
        return float(loss.item())

    def evaluate(self, batch: Batch, E_ref) -> float:
        """Energy MSE (or per-atom MSE) without a parameter update."""
        dev = batch.Z.device
        E_ref = torch.as_tensor(E_ref, dtype=torch.float64, device=dev)
        n_atoms = (batch.mol_ptr[1:] - batch.mol_ptr[:-1]).to(torch.float64)
        E, _, _ = self.model.engine().energy_forces(batch, _lib.PATH_PLAIN_FP32, forces=False)
        loss, _ = self.loss_weights(E, E_ref, n_atoms)
        return float(loss.item())


__all__ = ["param_grads", "EnergyTrainer", "trainable_names", "make_batch"]
