"""ORACLE -- test infrastructure only.

Functional CPU restatement of the reference StudentForceField
(src/mlff_distiller/models/student_model.py) that evaluates energy, forces
and the strain derivative (virial) in float64 with torch autograd.  It takes
an explicit edge list with integer image shifts so that periodic boxes (no
reference counterpart, student_model.py:694-703) use the same model algebra.

Parameters are a state_dict with the reference's key names
(student_model.py:566-628, StudentForceField.__init__).
"""
from __future__ import annotations

import math
from typing import Dict, Optional, Tuple

import numpy as np
import torch

Tensor = torch.Tensor


def _silu(x: Tensor) -> Tensor:
    return x * torch.sigmoid(x)


def rbf_times_cutoff(d: Tensor, centers: Tensor, widths: Tensor, cutoff: float) -> Tensor:
    """exp(-(d-mu)^2 / w^2) * 0.5*(cos(pi d / rc) + 1) * [d < rc].

    GaussianRBF.forward student_model.py:246-255 (gamma = 1/w^2, :253) times
    CosineCutoff.forward :284-292, multiplied at :718-722.
    """
    diff = d.unsqueeze(-1) - centers
    gamma = 1.0 / (widths ** 2)
    rbf = torch.exp(-gamma * diff ** 2)
    fc = 0.5 * (torch.cos(math.pi * d / cutoff) + 1.0)
    fc = fc * (d < cutoff).to(d.dtype)
    return rbf * fc.unsqueeze(-1)


def _linear(x: Tensor, p: Dict[str, Tensor], key: str) -> Tensor:
    return x @ p[key + ".weight"].T + p[key + ".bias"]


def _messages(s: Tensor, v: Tensor, e: Tensor, u: Tensor, src: Tensor, dst: Tensor, w1: Tensor, b1: Tensor,
              w2: Tensor, b2: Tensor):
    """(ds, dv) of one edge set: filter MLP (:350), split (:353-355), scalar
    and vector messages summed at the receivers (:359-385)."""
    H = s.shape[1]
    f = _silu(e @ w1.T + b1) @ w2.T + b2
    fs, fv1, fv2 = torch.split(f, H, dim=-1)
    ds = torch.zeros_like(s).index_add_(0, dst, s[src] * fs)
    dv = torch.zeros_like(v).index_add_(
        0, dst, v[src] * fv1.unsqueeze(1) + u.unsqueeze(-1) * fv2.unsqueeze(1))
    return ds, dv


def energy(p: Dict[str, Tensor], Z: Tensor, pos: Tensor, src: Tensor, dst: Tensor,
           shift_vec: Tensor, mol: Tensor, n_mol: int, cutoff: float = 5.0,
           edge_chunk: Optional[int] = None) -> Tensor:
    """Per-molecule energies [n_mol] (StudentForceField.forward :634-757).

    shift_vec [E,3] is added to pos[src]-pos[dst] (zero for open molecules).
    Messages flow src -> dst (PaiNNMessage.forward :346-387); the update is
    PaiNNUpdate.forward :434-470 with the 3x3 mixing over the xyz axis.

    edge_chunk: evaluate the messages over chunks of that many edges, each
    recomputed in the backward pass (torch.utils.checkpoint), so that large
    systems fit in host memory; the sums then add chunk by chunk (the same
    result up to float64 rounding).  None: one pass over all edges.
    """
    H = p["embedding.weight"].shape[1]
    s = p["embedding.weight"][Z]                                  # :684
    v = torch.zeros(Z.shape[0], 3, H, dtype=pos.dtype)           # :688-692
    r = pos[src] - pos[dst] + shift_vec                          # :709
    d = torch.linalg.vector_norm(r, dim=1)                       # :712
    u = r / (d.unsqueeze(1) + 1e-8)                              # :715
    e = rbf_times_cutoff(d, p["rbf.centers"], p["rbf.widths"], cutoff)   # :718-722
    n_layers = 1 + max(int(k.split(".")[1]) for k in p if k.startswith("interactions."))
    for l in range(n_layers):
        pre = f"interactions.{l}."
        if edge_chunk is None or src.shape[0] <= edge_chunk:
            f = _linear(_silu(_linear(e, p, pre + "message.rbf_to_scalar.0")), p,
                        pre + "message.rbf_to_scalar.2")              # :350
            fs, fv1, fv2 = torch.split(f, H, dim=-1)                   # :353-355
            ds = torch.zeros_like(s).index_add_(0, dst, s[src] * fs)   # :359-364
            dv = torch.zeros_like(v).index_add_(
                0, dst, v[src] * fv1.unsqueeze(1) + u.unsqueeze(-1) * fv2.unsqueeze(1))  # :370-385
        else:
            from torch.utils.checkpoint import checkpoint
            wts = [p[pre + "message.rbf_to_scalar.0.weight"], p[pre + "message.rbf_to_scalar.0.bias"],
                   p[pre + "message.rbf_to_scalar.2.weight"], p[pre + "message.rbf_to_scalar.2.bias"]]
            ds, dv = torch.zeros_like(s), torch.zeros_like(v)
            for c0 in range(0, src.shape[0], edge_chunk):
                c = slice(c0, c0 + edge_chunk)
                dsc, dvc = checkpoint(_messages, s, v, e[c], u[c], src[c], dst[c], *wts, use_reentrant=False)
                ds = ds + dsc
                dv = dv + dvc
        s = s + ds
        v = v + dv
        n = torch.linalg.vector_norm(v, dim=1)                     # :437
        a = _linear(_silu(_linear(torch.cat([s, n], dim=-1), p, pre + "update.update_mlp.0")),
                    p, pre + "update.update_mlp.2")               # :440-444
        a_s, g1, g2 = torch.split(a, H, dim=-1)                    # :447-449
        s = s + a_s                                                # :452
        mixed = torch.einsum("ij,njk->nik", p[pre + "update.mixing_matrix"], v)   # :458-462
        v = v * g1.unsqueeze(1) + mixed * g2.unsqueeze(1)          # :465-468
    h = _silu(_linear(s, p, "energy_head.0"))
    h = _silu(_linear(h, p, "energy_head.2"))
    e_atom = _linear(h, p, "energy_head.4").squeeze(-1)          # :736
    return torch.zeros(n_mol, dtype=pos.dtype).index_add_(0, mol, e_atom)   # :739-755


def params_to(p: Dict[str, Tensor], dtype=torch.float64) -> Dict[str, Tensor]:
    return {k: torch.as_tensor(np.asarray(v)).to(dtype) for k, v in p.items()}


def energy_forces(params, Z, pos, mol_ptr, cutoff=5.0, box=None, pbc=None,
                  edges=None, dtype=torch.float64, virial=False, edge_chunk=None):
    """Energies [B], forces [N,3] (= -dE/dpos) and optionally the strain
    derivative dE/d(eps) [B,3,3] for an affine strain of positions and cell.

    edges: (src, dst, shift) from oracle.nbr.radius_graph (computed here if
    None).  Forces follow predict_energy_and_forces :759-795 (autograd of
    the summed energy).
    """
    from . import nbr
    pos_np = np.asarray(pos)
    mol_ptr = np.asarray(mol_ptr, dtype=np.int64)
    n_mol = len(mol_ptr) - 1
    if edges is None:
        edges = nbr.radius_graph(pos_np.astype(np.float32), mol_ptr, cutoff, box, pbc)
    src, dst, shift = edges
    p = params_to(params, dtype)
    Zt = torch.as_tensor(np.asarray(Z), dtype=torch.long)
    mol = torch.repeat_interleave(torch.arange(n_mol), torch.as_tensor(np.diff(mol_ptr)))
    src_t = torch.as_tensor(np.asarray(src), dtype=torch.long)
    dst_t = torch.as_tensor(np.asarray(dst), dtype=torch.long)
    boxes = torch.zeros(n_mol, 3, dtype=dtype) if box is None else torch.as_tensor(
        np.asarray(box, dtype=np.float64).reshape(n_mol, 3), dtype=dtype)
    shift_t = torch.as_tensor(np.asarray(shift), dtype=dtype) * boxes[mol[dst_t]]
    x = torch.as_tensor(pos_np, dtype=dtype).clone().requires_grad_(True)
    eps = torch.zeros(n_mol, 3, 3, dtype=dtype, requires_grad=virial)
    if virial:
        # r' = (I + eps) r for every position and image shift, so that
        # dE/deps_ab = sum_edges (dE/dr_a) r_b
        strain = torch.eye(3, dtype=dtype) + eps
        xs = torch.einsum("nab,nb->na", strain[mol], x)
        sv = torch.einsum("eab,eb->ea", strain[mol[dst_t]], shift_t)
    else:
        xs, sv = x, shift_t
    E = energy(p, Zt, xs, src_t, dst_t, sv, mol, n_mol, cutoff, edge_chunk=edge_chunk)
    inputs = [x, eps] if virial else [x]
    grads = torch.autograd.grad(E.sum(), inputs)
    F = -grads[0]
    if virial:
        return E.detach(), F.detach(), grads[1].detach()
    return E.detach(), F.detach()


def stress_voigt(dEde: np.ndarray, box: np.ndarray) -> np.ndarray:
    """ASE-convention stress (1/V) dE/d(eps), symmetrised, Voigt order
    xx, yy, zz, yz, xz, xy (ase_calculator.py:578-583 uses that order)."""
    s = 0.5 * (dEde + dEde.T) / float(np.prod(box))
    return np.array([s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]])


def _train_setup(params, Z, pos, mol_ptr, cutoff, box, pbc, dtype):
    from . import nbr
    pos_np = np.asarray(pos)
    mol_ptr = np.asarray(mol_ptr, dtype=np.int64)
    n_mol = len(mol_ptr) - 1
    src, dst, shift = nbr.radius_graph(pos_np.astype(np.float32), mol_ptr, cutoff, box, pbc)
    p = params_to(params, dtype)
    train = [k for k in p if not k.startswith("rbf.")]
    for k in train:
        p[k].requires_grad_(True)
    mol = torch.repeat_interleave(torch.arange(n_mol), torch.as_tensor(np.diff(mol_ptr)))
    src_t = torch.as_tensor(np.asarray(src), dtype=torch.long)
    dst_t = torch.as_tensor(np.asarray(dst), dtype=torch.long)
    boxes = torch.zeros(n_mol, 3, dtype=dtype) if box is None else torch.as_tensor(
        np.asarray(box, dtype=np.float64).reshape(n_mol, 3), dtype=dtype)
    shift_t = torch.as_tensor(np.asarray(shift), dtype=dtype) * boxes[mol[dst_t]]
    Zt = torch.as_tensor(np.asarray(Z), dtype=torch.long)

    def energy_of(x, eps=None):
        # eps [B,3,3]: affine strain of positions and image shifts, r' = (I + eps) r
        if eps is None:
            return energy(p, Zt, x, src_t, dst_t, shift_t, mol, n_mol, cutoff)
        strain = torch.eye(3, dtype=dtype) + eps
        xs = torch.einsum("nab,nb->na", strain[mol], x)
        sv = torch.einsum("eab,eb->ea", strain[mol[dst_t]], shift_t)
        return energy(p, Zt, xs, src_t, dst_t, sv, mol, n_mol, cutoff)

    return p, train, energy_of, torch.as_tensor(pos_np, dtype=dtype)


def _grads_of(obj, p, train):
    # the last layer's mixing matrix only moves vector features the readout
    # never reads: its gradient is exactly zero
    g = torch.autograd.grad(obj, [p[k] for k in train], allow_unused=True)
    return {k: (torch.zeros_like(p[k]) if gi is None else gi).detach() for k, gi in zip(train, g)}


def param_grads(params, Z, pos, mol_ptr, weights, cutoff=5.0, box=None, pbc=None, dtype=torch.float64):
    """sum_b w_b dE_b/dtheta for every tensor of the state_dict except the
    RBF buffers, by autograd through `energy` (the parameter gradients
    loss.backward() gives the reference's Trainer, training/trainer.py:
    288-393, for an energy loss with dL/dE_b = w_b)."""
    p, train, energy_of, x = _train_setup(params, Z, pos, mol_ptr, cutoff, box, pbc, dtype)
    E = energy_of(x)
    w = torch.as_tensor(np.asarray(weights), dtype=dtype)
    return E.detach(), _grads_of((E * w).sum(), p, train)


def param_grads_forces(params, Z, pos, mol_ptr, energy_weights, force_weights, cutoff=5.0, box=None, pbc=None,
                       dtype=torch.float64, virial_weights=None):
    """sum_b w_b dE_b/dtheta + sum_i G_i . dF_i/dtheta (+ sum_b S_b :
    dW_b/dtheta with W_b = dE_b/d(strain)), F = -dE/dpos and W taken with
    create_graph=True (predict_energy_and_forces, student_model.py:759-795,
    in training mode) and differentiated again: the parameter gradients
    loss.backward() gives the reference's Trainer for a loss with dL/dE_b =
    w_b, dL/dF_i = G_i (and dL/dW_b = S_b).  Returns (E, F, grads)."""
    p, train, energy_of, x = _train_setup(params, Z, pos, mol_ptr, cutoff, box, pbc, dtype)
    x = x.clone().requires_grad_(True)
    n_mol = len(np.asarray(mol_ptr)) - 1
    eps = torch.zeros(n_mol, 3, 3, dtype=dtype, requires_grad=True)
    E = energy_of(x, eps if virial_weights is not None else None)
    inputs = [x, eps] if virial_weights is not None else [x]
    g = torch.autograd.grad(E.sum(), inputs, create_graph=True)
    F = -g[0]
    w = torch.as_tensor(np.asarray(energy_weights), dtype=dtype)
    obj = (E * w).sum()
    if force_weights is not None:
        obj = obj + (F * torch.as_tensor(np.asarray(force_weights), dtype=dtype)).sum()
    if virial_weights is not None:
        obj = obj + (g[1] * torch.as_tensor(np.asarray(virial_weights), dtype=dtype)).sum()
    return E.detach(), F.detach(), _grads_of(obj, p, train)
