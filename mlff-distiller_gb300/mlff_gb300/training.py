"""Training of the StudentForceField on the GPU with the library's own
forward and reverse kernels.

``param_grads`` returns the parameter part of ``loss.backward()`` in
Trainer.train_epoch (training/trainer.py:288-393) for every trainable
tensor of the state_dict, given the loss's derivatives with respect to the
predictions: w_b = dL/dE_b (one call of ``mlff_param_grads``: plain FP32
path forward, hand-written reverse pass with the weight-gradient
reductions) and, for a loss on forces, G_i = dL/dF_i (one call of
``mlff_param_grads_forces``: the same path in forward mode over the reverse
pass, which adds sum_i G_i . dF_i/dtheta -- what the reference gets by
taking forces with create_graph=True and differentiating again).

``ForceFieldLoss`` restates the reference's loss (training/losses.py:15-
246: energy, force, angular and stress terms with mse / mae / huber
components); the trainers evaluate it with torch on the predictions only
(energies, forces, stress) to get w, G and, for the stress term, S =
dL/dW with W = dE/d(strain) (one more direction of the same forward-mode
pass).  ``ForceFieldTrainer`` is the optimisation step with
the reference's defaults (configs/train_student.yaml: energy weight 1,
force weight 100, angular weight 10, AdamW lr 1e-3, weight decay 1e-5,
betas (0.9, 0.999), eps 1e-8, gradient-norm clip 1.0); ``EnergyTrainer``
the energy-only step.
"""
import ctypes
import warnings
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


def _grads_struct(model, grads: Dict[str, torch.Tensor]):
    g = _lib.Grads()
    g.embedding = _lib.ptr(grads.get("embedding.weight"))
    for l in range(model.num_interactions):
        for field, key in _LAYER_KEYS.items():
            getattr(g, field)[l] = _lib.ptr(grads.get(f"interactions.{l}.{key}"))
    for field, key in _HEAD_KEYS.items():
        setattr(g, field, _lib.ptr(grads.get(key)))
    return g


def param_grads(model, batch: Batch, weights: torch.Tensor, forces: bool = False,
                force_weights: Optional[torch.Tensor] = None, virial_weights: Optional[torch.Tensor] = None
                ) -> Tuple[torch.Tensor, Dict[str, torch.Tensor], Optional[torch.Tensor]]:
    """Energies [B] (float64), {name: dL/d(name)} for every trainable
    parameter (float32, state_dict shapes) and, if asked, the forces
    -sum_b w_b dE_b/dpos.

    dL/dtheta = sum_b w_b dE_b/dtheta (weights: w = dL/dE, [B]) plus, when
    force_weights G = dL/dF [N,3] is given, sum_i G_i . dF_i/dtheta, plus,
    when virial_weights S = dL/dW [B,3,3] is given (W = dE/d(strain), the
    virial the engine returns), sum_b S_b : dW_b/dtheta."""
    eng = model.engine()
    dev = eng.device
    N, B = batch.n_atoms, batch.n_mol
    w = torch.as_tensor(weights, dtype=torch.float64, device=dev).contiguous()
    if w.shape != (B,):
        raise ValueError(f"weights must have shape ({B},), got {tuple(w.shape)}")
    G = S = None
    if force_weights is not None:
        G = torch.as_tensor(force_weights, dtype=torch.float32, device=dev).contiguous()
        if G.shape != (N, 3):
            raise ValueError(f"force_weights must have shape ({N}, 3), got {tuple(G.shape)}")
    if virial_weights is not None:
        S = torch.as_tensor(virial_weights, dtype=torch.float64, device=dev).contiguous()
        if S.shape != (B, 3, 3):
            raise ValueError(f"virial_weights must have shape ({B}, 3, 3), got {tuple(S.shape)}")
    params = dict(model.named_parameters())
    grads = {n: torch.zeros_like(p, dtype=torch.float32, device=dev) for n, p in params.items() if p.requires_grad}
    g = _grads_struct(model, grads)
    E = torch.empty(B, dtype=torch.float64, device=dev)
    F = torch.empty(N, 3, dtype=torch.float32, device=dev) if forces else None
    out = _lib.Outputs()
    out.energy, out.forces, out.virial, out.atom_energy = E.data_ptr(), _lib.ptr(F), None, None
    sysd = batch.system()
    path = _lib.PATH_TRAIN
    second = G is not None or S is not None
    ws_path = _lib.PATH_TRAIN_FORCES if second else _lib.PATH_TRAIN
    for _ in range(4):
        cap = eng.capacity(N, path)
        ws = eng.workspace_for(N, B, cap, ws_path)
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
    if second:
        # same structures, same capacity: the edge list fits
        _lib.check(eng.lib.mlff_param_grads_forces(ctypes.byref(eng.dims), eng.packed.data_ptr(), ctypes.byref(sysd),
                                                   cap, _lib.ptr(G), _lib.ptr(S), ctypes.byref(g), ws.data_ptr(),
                                                   ws.numel(), _stream_handle()))
        code, _, where = eng.status()
        if code != _lib.OK:
            raise _lib.MLFFError(code, f"device status {code} at index {where}")
    return E, grads, F


def force_term_grads(model, batch: Batch, force_weights: torch.Tensor,
                     virial_weights: Optional[torch.Tensor] = None) -> Dict[str, torch.Tensor]:
    """{name: sum_i G_i . dF_i/dtheta (+ sum_b S_b : dW_b/dtheta)} for every
    trainable parameter: the forward-mode pass alone (mlff_param_grads_forces
    into zeroed gradients), without the energy term."""
    eng = model.engine()
    dev = eng.device
    N, B = batch.n_atoms, batch.n_mol
    G = None if force_weights is None else torch.as_tensor(force_weights, dtype=torch.float32,
                                                          device=dev).contiguous()
    S = None if virial_weights is None else torch.as_tensor(virial_weights, dtype=torch.float64,
                                                            device=dev).contiguous()
    if G is not None and G.shape != (N, 3):
        raise ValueError(f"force_weights must have shape ({N}, 3), got {tuple(G.shape)}")
    if S is not None and S.shape != (B, 3, 3):
        raise ValueError(f"virial_weights must have shape ({B}, 3, 3), got {tuple(S.shape)}")
    grads = {n: torch.zeros_like(p, dtype=torch.float32, device=dev)
             for n, p in model.named_parameters() if p.requires_grad}
    if G is None and S is None:
        return grads
    g = _grads_struct(model, grads)
    sysd = batch.system()
    path = _lib.PATH_TRAIN
    for _ in range(4):
        cap = eng.capacity(N, path)
        ws = eng.workspace_for(N, B, cap, _lib.PATH_TRAIN_FORCES)
        _lib.check(eng.lib.mlff_param_grads_forces(ctypes.byref(eng.dims), eng.packed.data_ptr(), ctypes.byref(sysd),
                                                   cap, _lib.ptr(G), _lib.ptr(S), ctypes.byref(g), ws.data_ptr(),
                                                   ws.numel(), _stream_handle()))
        code, n_edges, where = eng.status()
        if code == _lib.ERR_CAPACITY:
            eng.edge_capacity[path] = int(n_edges * 1.25) + 1024
            for t in grads.values():
                t.zero_()
            continue
        if code != _lib.OK:
            raise _lib.MLFFError(code, f"device status {code} at index {where}")
        eng.edge_capacity[path] = max(eng.edge_capacity.get(path, 0), int(n_edges * 1.15) + 1024)
        return grads
    raise _lib.MLFFError(_lib.ERR_CAPACITY, "edge capacity did not converge")


class ForceFieldLoss:
    """Weighted energy / force / angular loss on predicted energies [B] and
    forces [N,3] (ForceFieldLoss, training/losses.py:15-246): each term is an
    mse, mae or huber loss with the given reduction; the angular term is
    1 - cos between predicted and target force vectors (norms clamped at
    1e-8).  Stress enters only when both dicts hold it.  Returns the
    reference's dict of terms and monitoring metrics."""

    def __init__(self, energy_weight: float = 1.0, force_weight: float = 100.0, stress_weight: float = 0.1,
                 angular_weight: float = 10.0, energy_loss_type: str = "mse", force_loss_type: str = "mse",
                 stress_loss_type: str = "mse", huber_delta: float = 1.0, reduction: str = "mean"):
        self.energy_weight, self.force_weight = energy_weight, force_weight
        self.stress_weight, self.angular_weight = stress_weight, angular_weight
        self.energy_loss_type, self.force_loss_type = energy_loss_type, force_loss_type
        self.stress_loss_type = stress_loss_type
        self.huber_delta, self.reduction = huber_delta, reduction
        if force_weight > 0 and energy_weight > 0 and force_weight < energy_weight:
            warnings.warn(f"Force weight ({force_weight}) < energy weight ({energy_weight}). "
                          "For MD stability, forces should be weighted higher than energy.", UserWarning)

    def _component(self, pred, target, kind: str):
        import torch.nn.functional as tf
        if kind == "mse":
            return tf.mse_loss(pred, target, reduction=self.reduction)
        if kind == "mae":
            return tf.l1_loss(pred, target, reduction=self.reduction)
        if kind == "huber":
            return tf.huber_loss(pred, target, delta=self.huber_delta, reduction=self.reduction)
        raise ValueError(f"Unknown loss type: {kind}")

    def __call__(self, predictions: Dict[str, torch.Tensor], targets: Dict[str, torch.Tensor],
                 mask: Optional[Dict[str, torch.Tensor]] = None) -> Dict[str, torch.Tensor]:
        import torch.nn.functional as tf
        out: Dict[str, torch.Tensor] = {}
        total = 0.0

        def pair(key):
            p, t = predictions[key], targets[key]
            if mask is not None and key in mask:
                p, t = p[mask[key]], t[mask[key]]
            return p, t

        if "energy" in predictions and "energy" in targets and self.energy_weight > 0:
            p, t = pair("energy")
            out["energy"] = self._component(p, t, self.energy_loss_type)
            total = total + self.energy_weight * out["energy"]
            with torch.no_grad():
                out["energy_rmse"] = torch.sqrt(tf.mse_loss(p, t))
                out["energy_mae"] = tf.l1_loss(p, t)
        if "forces" in predictions and "forces" in targets and self.force_weight > 0:
            p, t = pair("forces")
            out["force"] = self._component(p, t, self.force_loss_type)
            total = total + self.force_weight * out["force"]
            if self.angular_weight > 0:
                pn = p / torch.norm(p, dim=-1, keepdim=True).clamp(min=1e-8)
                tn = t / torch.norm(t, dim=-1, keepdim=True).clamp(min=1e-8)
                cos = (pn * tn).sum(dim=-1)
                ang = 1.0 - cos
                out["angular"] = ang.mean() if self.reduction == "mean" else (
                    ang.sum() if self.reduction == "sum" else ang)
                total = total + self.angular_weight * out["angular"]
                with torch.no_grad():
                    deg = torch.acos(torch.clamp(cos, -1.0, 1.0)) * (180.0 / 3.14159265)
                    out["angular_error_mean_deg"], out["angular_error_max_deg"] = deg.mean(), deg.max()
            with torch.no_grad():
                out["force_rmse"] = torch.sqrt(tf.mse_loss(p, t))
                out["force_mae"] = tf.l1_loss(p, t)
                if p.dim() >= 2 and p.shape[-1] == 3:
                    sq = (p - t) ** 2
                    for i, ax in enumerate("xyz"):
                        out[f"force_rmse_{ax}"] = torch.sqrt(sq[..., i].mean())
        if "stress" in predictions and "stress" in targets and self.stress_weight > 0:
            p, t = pair("stress")
            out["stress"] = self._component(p, t, self.stress_loss_type)
            total = total + self.stress_weight * out["stress"]
            with torch.no_grad():
                out["stress_rmse"] = torch.sqrt(tf.mse_loss(p, t))
                out["stress_mae"] = tf.l1_loss(p, t)
        out["total"] = total
        return out

    def derivatives(self, E: torch.Tensor, F: torch.Tensor, E_ref: torch.Tensor, F_ref: torch.Tensor,
                    mask: Optional[Dict[str, torch.Tensor]] = None, W: Optional[torch.Tensor] = None,
                    volume: Optional[torch.Tensor] = None, S_ref: Optional[torch.Tensor] = None):
        """(loss dict, dL/dE [B] float64, dL/dF [N,3] float32 or None,
        dL/dW [B,3,3] float64 or None): the loss differentiated with respect
        to the predictions only.  With W = dE/d(strain) [B,3,3], the cell
        volumes [B] and stress targets S_ref ([B,3,3] or Voigt [B,6]), the
        predicted stress sym(W) / volume (the calculator's stress) enters
        the stress term."""
        Ed = E.detach().to(torch.float64).requires_grad_(True)
        Fd = F.detach().to(torch.float64).requires_grad_(True)
        pred = {"energy": Ed, "forces": Fd}
        tgt = {"energy": E_ref.to(torch.float64), "forces": F_ref.to(torch.float64)}
        Wd = None
        if W is not None and S_ref is not None:
            Wd = W.detach().to(torch.float64).requires_grad_(True)
            sym = 0.5 * (Wd + Wd.transpose(1, 2)) / volume.to(torch.float64).reshape(-1, 1, 1)
            if S_ref.shape[-1] == 6:
                sym = torch.stack([sym[:, 0, 0], sym[:, 1, 1], sym[:, 2, 2], sym[:, 1, 2], sym[:, 0, 2],
                                   sym[:, 0, 1]], dim=-1)
            pred["stress"], tgt["stress"] = sym, S_ref.to(torch.float64)
        out = self(pred, tgt, mask)
        total = out["total"]
        if not torch.is_tensor(total) or not total.requires_grad:
            return out, torch.zeros_like(Ed), None, None
        inputs = [Ed, Fd] + ([Wd] if Wd is not None else [])
        gr = torch.autograd.grad(total, inputs, allow_unused=True)
        gE = torch.zeros_like(Ed) if gr[0] is None else gr[0].detach()
        gF = None if gr[1] is None else gr[1].detach().to(torch.float32)
        gW = None if Wd is None or gr[2] is None else gr[2].detach()
        return out, gE, gF, gW


def _adamw(model, lr, weight_decay, betas, eps):
    return torch.optim.AdamW([p for p in model.parameters() if p.requires_grad], lr=lr,
                             weight_decay=weight_decay, betas=betas, eps=eps)


def _apply(model, opt, grads, grad_clip):
    for n, p in model.named_parameters():
        if p.requires_grad:
            p.grad = grads[n].to(p.dtype)
    if grad_clip:
        torch.nn.utils.clip_grad_norm_(model.parameters(), grad_clip)
    opt.step()
    opt.zero_grad(set_to_none=True)


class ForceFieldTrainer:
    """One optimisation step per call on energies and forces: forward and
    forces on the plain FP32 path, the loss and its derivatives w = dL/dE,
    G = dL/dF (``ForceFieldLoss``), parameter gradients from the CUDA
    reverse pass and its forward-mode derivative (``param_grads``),
    gradient clipping and AdamW."""

    def __init__(self, model, loss: Optional[ForceFieldLoss] = None, lr: float = 1e-3, weight_decay: float = 1e-5,
                 betas=(0.9, 0.999), eps: float = 1e-8, grad_clip: float = 1.0):
        self.model = model
        self.loss_fn = loss if loss is not None else ForceFieldLoss()
        self.opt = _adamw(model, lr, weight_decay, betas, eps)
        self.grad_clip = grad_clip
        self.steps = 0

    def _predict(self, batch: Batch, virial: bool = False):
        return self.model.engine().energy_forces(batch, _lib.PATH_PLAIN_FP32, forces=True, virial=virial)

    def step(self, batch: Batch, E_ref, F_ref, S_ref=None) -> Dict[str, float]:
        """One step on energy and force targets (and stress targets
        [B,3,3] or Voigt [B,6] for periodic batches)."""
        dev = batch.Z.device
        E_ref = torch.as_tensor(E_ref, dtype=torch.float64, device=dev)
        F_ref = torch.as_tensor(F_ref, dtype=torch.float64, device=dev)
        stress = S_ref is not None and self.loss_fn.stress_weight > 0
        if stress and batch.box is None:
            raise ValueError("stress targets need periodic structures (batch.box)")
        E, F, W = self._predict(batch, virial=stress)
        vol = torch.prod(batch.box.to(torch.float64), dim=1) if stress else None
        S_ref = torch.as_tensor(S_ref, dtype=torch.float64, device=dev) if stress else None
        out, w, G, S = self.loss_fn.derivatives(E, F, E_ref, F_ref, W=W, volume=vol, S_ref=S_ref)
        _, grads, _ = param_grads(self.model, batch, w, force_weights=G, virial_weights=S)
        _apply(self.model, self.opt, grads, self.grad_clip)
        self.steps += 1
        return {k: float(v.item()) for k, v in out.items() if torch.is_tensor(v) and v.numel() == 1}

    def evaluate(self, batch: Batch, E_ref, F_ref) -> Dict[str, float]:
        dev = batch.Z.device
        E, F, _ = self._predict(batch)
        out = self.loss_fn({"energy": E.to(torch.float64), "forces": F.to(torch.float64)},
                           {"energy": torch.as_tensor(E_ref, dtype=torch.float64, device=dev),
                            "forces": torch.as_tensor(F_ref, dtype=torch.float64, device=dev)})
        return {k: float(v.item()) for k, v in out.items() if torch.is_tensor(v) and v.numel() == 1}


class EnergyTrainer:
    """One optimisation step per call: energies, loss, parameter gradients
    from the CUDA reverse pass, gradient clipping and AdamW."""

    def __init__(self, model, lr: float = 1e-3, weight_decay: float = 1e-5, betas=(0.9, 0.999),
                 eps: float = 1e-8, grad_clip: float = 1.0, per_atom: bool = False):
        self.model = model
        self.opt = _adamw(model, lr, weight_decay, betas, eps)
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
        _apply(self.model, self.opt, grads, self.grad_clip)
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


__all__ = ["param_grads", "force_term_grads", "ForceFieldLoss", "ForceFieldTrainer", "EnergyTrainer", "trainable_names", "make_batch"]
