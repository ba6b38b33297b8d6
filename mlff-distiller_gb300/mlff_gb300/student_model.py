"""Drop-in ``StudentForceField`` evaluated by the GB300 CUDA library.

Same constructor, same parameters and buffers, same state_dict keys and
shapes, same seeded initialisation and the same ``save``/``load`` checkpoint
format as the reference module
(src/mlff_distiller/models/student_model.py:532-1176).  ``forward`` and
``predict_energy_and_forces`` run the whole model -- radius graph, edge
filters, messages, updates, readout and the hand-written force adjoint --
in libmlff_gb300.so on the current CUDA stream.  There is no CPU path.

Differences from the reference, on purpose:
* ``cell``/``pbc`` are honoured (orthorhombic, minimum image) when
  ``periodic=True`` (default); the reference ignores them
  (student_model.py:694-703).  ``periodic=False`` reproduces that.
* ``precision`` picks the evaluation path: ``"fp16x3"`` (fused edge
  kernels, tcgen05 tensor cores with split-FP16 operands -- x = hi + lo,
  three MMAs -- and FP32 accumulation), ``"tuned_fp32"`` (same fused
  kernels on FP32 CUDA cores) or ``"fp32"`` (plain per-op FP32 kernels).
* Gradients flow to positions only (forces); parameter gradients for
  force-matching training come from ``mlff_gb300.training``.
"""
from __future__ import annotations

import logging
import math
from pathlib import Path
from typing import Dict, Optional, Tuple, Union

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from .engine import Batch, Engine, dims_of

logger = logging.getLogger(__name__)


class GaussianRBF(nn.Module):
    """exp(-(d - mu_k)^2 / w_k^2), mu = linspace(0, cutoff, n), w = cutoff/n
    (student_model.py:196-255).  ``centers``/``widths`` are buffers, or
    parameters when learnable."""

    def __init__(self, num_rbf: int = 20, cutoff: float = 5.0, learnable: bool = False):
        super().__init__()
        self.num_rbf = num_rbf
        self.cutoff = cutoff
        centers = torch.linspace(0, cutoff, num_rbf)
        widths = torch.ones(num_rbf) * (cutoff / num_rbf)
        if learnable:
            self.centers = nn.Parameter(centers)
            self.widths = nn.Parameter(widths)
        else:
            self.register_buffer("centers", centers)
            self.register_buffer("widths", widths)

    def forward(self, distances: torch.Tensor) -> torch.Tensor:
        diff = distances.unsqueeze(-1) - self.centers
        return torch.exp(-(1.0 / self.widths ** 2) * diff ** 2)


class CosineCutoff(nn.Module):
    """0.5 (cos(pi d / rc) + 1) for d < rc, else 0 (student_model.py:258-292)."""

    def __init__(self, cutoff: float = 5.0):
        super().__init__()
        self.cutoff = cutoff

    def forward(self, distances: torch.Tensor) -> torch.Tensor:
        return 0.5 * (torch.cos(math.pi * distances / self.cutoff) + 1.0) * (distances < self.cutoff).float()


def _dev_f32(t: torch.Tensor, name: str) -> torch.Tensor:
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor: mlff_gb300 has no CPU path")
    return t.detach().to(torch.float32).contiguous()


def _check_status(status: torch.Tensor, what: str):
    code, where = (int(x) for x in status[:3:2].tolist())
    if code == _lib.ERR_INVALID:
        raise IndexError(f"{what}: edge_index entry of edge {where} is out of range")
    if code != _lib.OK:
        raise _lib.MLFFError(code, f"{what}: device status {code} at {where}")


class _MessageFn(torch.autograd.Function):
    """PaiNNMessage.forward on the library's per-module kernels; backward
    returns the gradients of features, basis values, unit vectors and the
    filter parameters (mlff_painn_message_backward)."""

    @staticmethod
    def forward(ctx, s, v, edge_index, rbf, evec, w1, b1, w2, b2):
        lib = _lib.load()
        N, H = s.shape
        E, R = rbf.shape
        if v.shape != (N, 3, H) or edge_index.shape != (2, E) or evec.shape != (E, 3):
            raise ValueError(f"PaiNNMessage: inconsistent shapes scalar {tuple(s.shape)}, vector {tuple(v.shape)}, "
                             f"edge_index {tuple(edge_index.shape)}, edge_rbf {tuple(rbf.shape)}, "
                             f"edge_vector {tuple(evec.shape)}")
        args = [_dev_f32(x, n) for x, n in ((s, "scalar_features"), (v, "vector_features"), (rbf, "edge_rbf"),
                                            (evec, "edge_vector"), (w1, "weight"), (b1, "bias"), (w2, "weight"),
                                            (b2, "bias"))]
        ei = edge_index.detach().to(device=s.device, dtype=torch.int64).contiguous()
        so = torch.empty(N, H, device=s.device)
        vo = torch.empty(N, 3, H, device=s.device)
        status = torch.zeros(4, dtype=torch.int32, device=s.device)
        ws = torch.empty(lib.mlff_painn_message_workspace_size(H, R, E, 0), dtype=torch.uint8, device=s.device)
        sf, vf, rf, ef, w1f, b1f, w2f, b2f = args
        _lib.check(lib.mlff_painn_message(H, R, N, E, sf.data_ptr(), vf.data_ptr(), ei.data_ptr(), rf.data_ptr(),
                                          ef.data_ptr(), w1f.data_ptr(), b1f.data_ptr(), w2f.data_ptr(),
                                          b2f.data_ptr(), so.data_ptr(), vo.data_ptr(), status.data_ptr(),
                                          ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream))
        _check_status(status, "PaiNNMessage")
        ctx.save_for_backward(sf, vf, ei, rf, ef, w1f, b1f, w2f, b2f)
        ctx.dtypes = (s.dtype, v.dtype, rbf.dtype, evec.dtype, w1.dtype, b1.dtype, w2.dtype, b2.dtype)
        return so.to(s.dtype), vo.to(v.dtype)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gso, gvo):
        lib = _lib.load()
        sf, vf, ei, rf, ef, w1f, b1f, w2f, b2f = ctx.saved_tensors
        N, H = sf.shape
        E, R = rf.shape
        dev = sf.device
        gso = torch.zeros_like(sf) if gso is None else gso.to(torch.float32).contiguous()
        gvo = torch.zeros_like(vf) if gvo is None else gvo.to(torch.float32).contiguous()
        gs, gv = torch.empty_like(sf), torch.empty_like(vf)
        grbf, gev = torch.empty_like(rf), torch.empty_like(ef)
        gw1, gb1, gw2, gb2 = (torch.empty_like(w1f), torch.empty_like(b1f), torch.empty_like(w2f),
                              torch.empty_like(b2f))
        status = torch.zeros(4, dtype=torch.int32, device=dev)
        ws = torch.empty(lib.mlff_painn_message_workspace_size(H, R, E, 1), dtype=torch.uint8, device=dev)
        _lib.check(lib.mlff_painn_message_backward(
            H, R, N, E, sf.data_ptr(), vf.data_ptr(), ei.data_ptr(), rf.data_ptr(), ef.data_ptr(), w1f.data_ptr(),
            b1f.data_ptr(), w2f.data_ptr(), b2f.data_ptr(), gso.data_ptr(), gvo.data_ptr(), gs.data_ptr(),
            gv.data_ptr(), grbf.data_ptr(), gev.data_ptr(), gw1.data_ptr(), gb1.data_ptr(), gw2.data_ptr(),
            gb2.data_ptr(), status.data_ptr(), ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream))
        _check_status(status, "PaiNNMessage backward")
        d = ctx.dtypes
        return (gs.to(d[0]), gv.to(d[1]), None, grbf.to(d[2]), gev.to(d[3]), gw1.to(d[4]), gb1.to(d[5]),
                gw2.to(d[6]), gb2.to(d[7]))


class _UpdateFn(torch.autograd.Function):
    """PaiNNUpdate.forward on the library's per-module kernels, with its
    reverse pass (mlff_painn_update_backward)."""

    @staticmethod
    def forward(ctx, s, v, w1, b1, w2, b2, mix):
        lib = _lib.load()
        N, H = s.shape
        if v.shape != (N, 3, H):
            raise ValueError(f"PaiNNUpdate: scalar {tuple(s.shape)} and vector {tuple(v.shape)} do not match")
        sf, vf, w1f, b1f, w2f, b2f, mf = (_dev_f32(x, n) for x, n in (
            (s, "scalar_features"), (v, "vector_features"), (w1, "weight"), (b1, "bias"), (w2, "weight"),
            (b2, "bias"), (mix, "mixing_matrix")))
        so = torch.empty(N, H, device=s.device)
        vo = torch.empty(N, 3, H, device=s.device)
        ws = torch.empty(lib.mlff_painn_update_workspace_size(H, N, 0), dtype=torch.uint8, device=s.device)
        _lib.check(lib.mlff_painn_update(H, N, sf.data_ptr(), vf.data_ptr(), w1f.data_ptr(), b1f.data_ptr(),
                                         w2f.data_ptr(), b2f.data_ptr(), mf.data_ptr(), so.data_ptr(), vo.data_ptr(),
                                         ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream))
        ctx.save_for_backward(sf, vf, w1f, b1f, w2f, b2f, mf)
        ctx.dtypes = (s.dtype, v.dtype, w1.dtype, b1.dtype, w2.dtype, b2.dtype, mix.dtype)
        return so.to(s.dtype), vo.to(v.dtype)

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, gso, gvo):
        lib = _lib.load()
        sf, vf, w1f, b1f, w2f, b2f, mf = ctx.saved_tensors
        N, H = sf.shape
        dev = sf.device
        gso = torch.zeros_like(sf) if gso is None else gso.to(torch.float32).contiguous()
        gvo = torch.zeros_like(vf) if gvo is None else gvo.to(torch.float32).contiguous()
        outs = [torch.empty_like(x) for x in (sf, vf, w1f, b1f, w2f, b2f, mf)]
        ws = torch.empty(lib.mlff_painn_update_workspace_size(H, N, 1), dtype=torch.uint8, device=dev)
        _lib.check(lib.mlff_painn_update_backward(
            H, N, sf.data_ptr(), vf.data_ptr(), w1f.data_ptr(), b1f.data_ptr(), w2f.data_ptr(), b2f.data_ptr(),
            mf.data_ptr(), gso.data_ptr(), gvo.data_ptr(), *[o.data_ptr() for o in outs], ws.data_ptr(),
            ws.numel(), torch.cuda.current_stream().cuda_stream))
        return tuple(o.to(d) for o, d in zip(outs, ctx.dtypes))


class PaiNNMessage(nn.Module):
    """Message block: ``rbf_to_scalar`` = Linear(R, H) - SiLU - Linear(H, 3H)
    (student_model.py:297-322).  Inside StudentForceField the fused edge
    kernels evaluate it; called on its own (``forward``, student_model.py:
    324-387: messages from edge_index[0] to edge_index[1] added to the input
    features), it runs on the library's per-module kernels for any width,
    with gradients."""

    def __init__(self, hidden_dim: int, num_rbf: int):
        super().__init__()
        self.hidden_dim = hidden_dim
        self.rbf_to_scalar = nn.Sequential(nn.Linear(num_rbf, hidden_dim), nn.SiLU(),
                                           nn.Linear(hidden_dim, hidden_dim * 3))

    def forward(self, scalar_features: torch.Tensor, vector_features: torch.Tensor, edge_index: torch.Tensor,
                edge_rbf: torch.Tensor, edge_vector: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        l1, l2 = self.rbf_to_scalar[0], self.rbf_to_scalar[2]
        return _MessageFn.apply(scalar_features, vector_features, edge_index, edge_rbf, edge_vector,
                                l1.weight, l1.bias, l2.weight, l2.bias)


class PaiNNUpdate(nn.Module):
    """Update block: ``update_mlp`` = Linear(2H, H) - SiLU - Linear(H, 3H)
    and the 3x3 ``mixing_matrix`` over the xyz axis (student_model.py:
    390-416).  ``forward`` (:418-470) runs on the per-module kernels."""

    def __init__(self, hidden_dim: int):
        super().__init__()
        self.hidden_dim = hidden_dim
        self.update_mlp = nn.Sequential(nn.Linear(hidden_dim * 2, hidden_dim), nn.SiLU(),
                                        nn.Linear(hidden_dim, hidden_dim * 3))
        self.mixing_matrix = nn.Parameter(torch.randn(3, 3) / np.sqrt(3))

    def forward(self, scalar_features: torch.Tensor,
                vector_features: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        l1, l2 = self.update_mlp[0], self.update_mlp[2]
        return _UpdateFn.apply(scalar_features, vector_features, l1.weight, l1.bias, l2.weight, l2.bias,
                               self.mixing_matrix)


class PaiNNInteraction(nn.Module):
    """message + update (student_model.py:473-527)."""

    def __init__(self, hidden_dim: int, num_rbf: int):
        super().__init__()
        self.message = PaiNNMessage(hidden_dim, num_rbf)
        self.update = PaiNNUpdate(hidden_dim)

    def forward(self, scalar_features: torch.Tensor, vector_features: torch.Tensor, edge_index: torch.Tensor,
                edge_rbf: torch.Tensor, edge_vector: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
        s, v = self.message(scalar_features, vector_features, edge_index, edge_rbf, edge_vector)
        return self.update(s, v)


class _EnergyForces(torch.autograd.Function):
    """E = model(positions) with dE/dpos from the CUDA adjoint.  The forward
    computes forces eagerly; backward scales them by the incoming energy
    gradient of each structure."""

    @staticmethod
    def forward(ctx, positions, model, batch, mol_index):
        need_grad = positions.requires_grad
        E, F, _ = model._engine_call(batch, forces=need_grad)
        ctx.save_for_backward(F if need_grad else torch.empty(0, device=positions.device), mol_index)
        return E.to(positions.dtype)

    @staticmethod
    def backward(ctx, grad_E):
        F, mol_index = ctx.saved_tensors
        if F.numel() == 0:
            return None, None, None, None
        g = grad_E.to(torch.float32)[mol_index].unsqueeze(1)
        return (-F * g).to(grad_E.dtype), None, None, None


def _trainable(model):
    return [(n, p) for n, p in model.named_parameters() if p.requires_grad]


class _EnergyTrain(torch.autograd.Function):
    """Training-mode E = model(positions), differentiable in the parameters
    to second order.  The forward value and forces come from the fused FP32
    path (no per-edge activations are stored, so a forward-only call stays
    small); the parameter gradients from the plain FP32 path's reverse
    passes, recomputed in backward.  backward(g): the position gradient
    sum_b g_b dE_b/dpos and
    the parameter gradients sum_b g_b dE_b/dtheta (mlff_param_grads).  When
    the backward itself is recorded (torch.autograd.grad(E, pos,
    create_graph=True), the reference's forces in training mode,
    student_model.py:759-795) the position gradient is a _ForceTerm node
    instead, whose own backward gives the forces' parameter gradients; the
    energy term's parameter gradients then come from the later
    loss.backward()."""

    @staticmethod
    def forward(ctx, positions, model, batch, mol_index, *params):
        from . import _lib
        E, F, _ = model.engine().energy_forces(batch, _lib.PATH_TUNED_FP32, forces=True)
        ctx.model, ctx.batch = model, batch
        ctx.save_for_backward(F, mol_index, *params)
        return E.to(positions.dtype)

    @staticmethod
    def backward(ctx, grad_E):
        F, mol_index, *params = ctx.saved_tensors
        none = (None, None, None)
        if torch.is_grad_enabled():
            gpos = _ForceTerm.apply(grad_E, F, mol_index, ctx.model, ctx.batch, *params)
            return (gpos,) + none + (None,) * len(params)
        from .training import param_grads
        g = grad_E.detach()
        gpos = (-F * g.to(torch.float32)[mol_index].unsqueeze(1)).to(grad_E.dtype)
        _, grads, _ = param_grads(ctx.model, ctx.batch, g.to(torch.float64))
        return (gpos,) + none + tuple(grads[n].to(p.dtype) for (n, _), p in zip(_trainable(ctx.model), params))


class _ForceTerm(torch.autograd.Function):
    """sum_b g_b dE_b/dpos as a function of g and the parameters (the
    recorded position gradient of _EnergyTrain).  backward(G): the parameter
    gradients sum_i G'_i . d(dE/dpos_i)/dtheta with G'_i = g_b(i) G_i, by the
    forward-mode pass over the reverse pass (mlff_param_grads_forces), and
    dL/dg_b = sum over the atoms of b of G_i . dE/dpos_i.  The second
    derivative in the positions (a Hessian-vector product) is not formed:
    positions are training data."""

    @staticmethod
    def forward(ctx, grad_E, F, mol_index, model, batch, *params):
        ctx.model, ctx.batch = model, batch
        ctx.save_for_backward(grad_E, F, mol_index, *params)
        return -F * grad_E.detach().to(torch.float32)[mol_index].unsqueeze(1)

    @staticmethod
    def backward(ctx, grad_out):
        grad_E, F, mol_index, *params = ctx.saved_tensors
        from .training import force_term_grads
        G = grad_out.detach().to(torch.float32)
        Gp = G * grad_E.detach().to(torch.float32)[mol_index].unsqueeze(1)
        # the output is +dE/dpos = -F: its weights enter the forces' gradient with a minus sign
        grads = force_term_grads(ctx.model, ctx.batch, -Gp)
        gE = torch.zeros_like(grad_E).index_add_(0, mol_index, -(G * F).sum(dim=1).to(grad_E.dtype))
        return (gE, None, None, None, None) + tuple(grads[n].to(p.dtype)
                                                    for (n, _), p in zip(_trainable(ctx.model), params))


# Width of the fused whole-model CUDA paths (every reference configuration
# and checkpoint); other widths run the module-level path.
FUSED_HIDDEN = 128


class StudentForceField(nn.Module):
    """PaiNN-style energy model (student_model.py:532-1176) on GB300.

    hidden_dim = 128 runs the fused CUDA paths (``precision``).  Other widths
    (the reference's unit tests build width-64 models) run the module-level
    path: the reference's forward (student_model.py:675-757) with the radius
    graph and every message and update block on the library's CUDA kernels
    (``PaiNNMessage``, ``PaiNNUpdate``) and the edge geometry, radial basis,
    embedding lookup and energy head as tensor operations on the GPU; forces
    and the virial by autograd through the blocks' reverse kernels
    (first-order: a force loss cannot be differentiated again there)."""

    def __init__(self, hidden_dim: int = 128, num_interactions: int = 3, num_rbf: int = 20,
                 cutoff: float = 5.0, max_z: int = 118, learnable_rbf: bool = False,
                 use_torch_cluster: bool = True, precision: str = "fp16x3", periodic: bool = True):
        super().__init__()
        self.hidden_dim = hidden_dim
        self.num_interactions = num_interactions
        self.num_rbf = num_rbf
        self.cutoff = cutoff
        self.max_z = max_z
        self.use_torch_cluster = use_torch_cluster
        self.precision = precision
        self.periodic = periodic
        self.embedding = nn.Embedding(max_z + 1, hidden_dim)
        self.rbf = GaussianRBF(num_rbf, cutoff, learnable_rbf)
        self.cutoff_fn = CosineCutoff(cutoff)
        self.interactions = nn.ModuleList([PaiNNInteraction(hidden_dim, num_rbf)
                                           for _ in range(num_interactions)])
        self.energy_head = nn.Sequential(nn.Linear(hidden_dim, hidden_dim // 2), nn.SiLU(),
                                         nn.Linear(hidden_dim // 2, hidden_dim // 4), nn.SiLU(),
                                         nn.Linear(hidden_dim // 4, 1))
        self._initialize_parameters()
        self._engine: Optional[Engine] = None
        self._single_ptr: Dict[int, torch.Tensor] = {}   # device [0, N] offsets of single-structure calls
        self._cell_cache = None                            # last host cell -> checked device box / pbc
        self._batch_cache = None                           # last host structure index -> device offsets
        self._packed_version = None
        self._weight_slots = None                          # (tensor dict, name) of every parameter and buffer

    def _initialize_parameters(self):
        """Same initialisation as the reference (student_model.py:618-628)."""
        nn.init.uniform_(self.embedding.weight, -np.sqrt(3), np.sqrt(3))
        for module in self.modules():
            if isinstance(module, nn.Linear):
                nn.init.xavier_uniform_(module.weight)
                if module.bias is not None:
                    nn.init.zeros_(module.bias)

    def num_parameters(self) -> int:
        return sum(p.numel() for p in self.parameters() if p.requires_grad)

    @property
    def fused(self) -> bool:
        """True when the fused CUDA paths evaluate this model (hidden width 128)."""
        return self.hidden_dim == FUSED_HIDDEN

    # ------------------------------------------------- module-level path
    def _neighbor_engine(self) -> Engine:
        """Radius-graph builder of the module-level path.  The neighbour build
        reads only the cutoff and the species count, so it runs at the fused
        width with a one-layer, one-basis-function shape."""
        dev = self.embedding.weight.device
        eng = getattr(self, "_nbr_engine", None)
        if eng is None or eng.device != dev:
            eng = Engine(dims_of(FUSED_HIDDEN, 1, 1, self.max_z + 1, float(self.cutoff)), dev)
            self._nbr_engine = eng
        return eng

    def _module_energy(self, positions: torch.Tensor, bt: Batch, mol_index: torch.Tensor,
                       strain: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Energies [B] (float64) of the module-level path, differentiable
        with respect to positions, parameters and (given) the strain [B,3,3]
        applied to every edge vector (dE/dstrain at 0 is the virial)."""
        dev = positions.device
        N = bt.n_atoms
        row_ptr, col = self._neighbor_engine().neighbors(bt)
        # edge_index as the reference's radius graph: source-major, rows then columns
        src = torch.repeat_interleave(torch.arange(N, device=dev), (row_ptr[1:] - row_ptr[:-1]).to(torch.int64))
        dst = col.to(torch.int64)
        x = positions.to(torch.float32)
        vec = x[src] - x[dst]                                   # student_model.py:709
        if bt.box is not None:   # minimum image in orthorhombic periodic boxes
            L = bt.box[mol_index[dst]]
            per = bt.pbc[mol_index[dst]].to(torch.bool).unsqueeze(1)
            vec = torch.where(per, vec - L * torch.round(vec / L), vec)
        if strain is not None:
            vec = torch.einsum("eab,eb->ea", torch.eye(3, device=dev, dtype=vec.dtype) + strain[mol_index[dst]], vec)
        dist = torch.norm(vec, dim=1)
        unit = vec / (dist.unsqueeze(1) + 1e-8)
        rbf = self.rbf(dist) * self.cutoff_fn(dist).unsqueeze(-1)
        s = self.embedding(bt.Z)
        v = torch.zeros(N, 3, self.hidden_dim, device=dev, dtype=s.dtype)
        edge_index = torch.stack([src, dst])
        for block in self.interactions:
            s, v = block(s, v, edge_index, rbf, unit)
        e_atom = self.energy_head(s)[:, 0].to(torch.float64)
        # per-structure sums in a fixed order (atoms are grouped by structure)
        cs = torch.cat([e_atom.new_zeros(1), torch.cumsum(e_atom, 0)])
        return cs[bt.mol_ptr[1:]] - cs[bt.mol_ptr[:-1]]

    def _module_call(self, atomic_numbers, positions, cell, pbc, batch, forces=True, virial=False,
                     create_graph=False):
        """(energies [B] float64, forces [N,3] float32 or None, virial [B,3,3]
        or None, structures) of the module-level path."""
        dev = self.embedding.weight.device
        host = positions.device.type == "cpu"
        Zd = atomic_numbers.to(dev) if host else atomic_numbers
        Pd = positions.to(dev) if host else positions
        bt, mol_index, n_mol = self._make_batch(Zd, Pd, cell, pbc, batch)
        need = forces or virial
        x = Pd if (Pd.requires_grad or not need) else Pd.detach().requires_grad_(True)
        eps = torch.zeros(n_mol, 3, 3, device=dev, requires_grad=True) if virial else None
        with torch.enable_grad() if need else torch.no_grad():
            E = self._module_energy(x, bt, mol_index, eps)
            F = W = None
            if need:
                inputs = [x] + ([eps] if virial else [])
                g = torch.autograd.grad(E.sum(), inputs, create_graph=create_graph, allow_unused=True)
                if forces:
                    F = -(g[0] if g[0] is not None else torch.zeros_like(x))
                if virial:
                    W = g[1] if g[1] is not None else torch.zeros(n_mol, 3, 3, device=dev)
        return E, F, W, n_mol

    # ------------------------------------------------------------- engine
    @property
    def path(self) -> int:
        try:
            return _lib.PATHS[self.precision]
        except KeyError:
            raise ValueError(f"unknown precision {self.precision!r}; use one of {sorted(_lib.PATHS)}")

    def _weights_version(self):
        """(address, in-place version) of every parameter and buffer: changes
        when a weight is updated in place, reassigned or moved.  The slots
        are the modules' own parameter / buffer dicts, looked up once."""
        slots = self._weight_slots
        if slots is None:
            slots = [(m._parameters, n) for m in self.modules() for n in m._parameters] + \
                    [(m._buffers, n) for m in self.modules() for n in m._buffers]
            self._weight_slots = slots
        return tuple((t.data_ptr(), t._version) if t is not None else None
                     for t in (d[n] for d, n in slots))

    def engine(self) -> Engine:
        dev = self.embedding.weight.device
        if dev.type != "cuda":
            raise RuntimeError("mlff_gb300 computes on a CUDA device: move the model with .to('cuda')")
        if self._engine is None or self._engine.device != dev:
            self._engine = Engine(dims_of(self.hidden_dim, self.num_rbf, self.num_interactions,
                                          self.max_z + 1, float(self.cutoff)), dev)
            self._packed_version = None
        v = self._weights_version()
        if v != self._packed_version:
            self._engine.pack(self.state_dict())
            self._packed_version = v
        return self._engine

    def _engine_call(self, batch: Batch, forces: bool = True, virial: bool = False, to_host: bool = False):
        return self.engine().energy_forces(batch, self.path, forces=forces, virial=virial, to_host=to_host)

    def _make_batch(self, atomic_numbers, positions, cell, pbc, batch, need_index: bool = True,
                    host_inputs: bool = False):
        """Device Batch of one call.  A ``batch`` index or ``cell`` given on
        the host (as the calculator passes them) is validated and turned into
        molecule offsets on the host, with no device synchronisation; device
        tensors are validated on the device.  ``host_inputs``: atomic numbers
        and positions stay in host memory (the engine copies them into its
        graph's input buffers)."""
        dev = self.embedding.weight.device
        if dev.type != "cuda" or not torch.cuda.is_available():
            raise RuntimeError("mlff_gb300 needs a CUDA device (GB300, sm_103a): move the model to cuda")
        if host_inputs:
            if positions.device.type != "cpu" or atomic_numbers.device.type != "cpu":
                raise RuntimeError("host_inputs needs atomic numbers and positions in host memory")
        elif positions.device != dev:
            raise RuntimeError(f"positions on {positions.device} but model on {dev}")
        N = int(atomic_numbers.shape[0])
        if batch is None:
            mol_ptr = self._single_ptr.get(N)   # device [0, N], reused (the engine skips re-copying it)
            if mol_ptr is None:
                mol_ptr = torch.tensor([0, N], dtype=torch.int64, device=dev)
                self._single_ptr = {N: mol_ptr}
            mol_index = torch.zeros(N, dtype=torch.int64, device=dev) if need_index else None
            n_mol = 1
        elif batch.device.type == "cpu":
            b = batch.to(torch.int64)
            hit = self._batch_cache is not None and torch.equal(self._batch_cache[0], b)
            if hit:   # the same structure index as the last call: reuse its device offsets
                n_mol, mol_ptr = self._batch_cache[1], self._batch_cache[2]
            else:
                if N and bool((b[1:] < b[:-1]).any()):
                    raise ValueError("batch indices must be non-decreasing (atoms grouped by structure)")
                n_mol = int(b[-1]) + 1 if N else 0
                mp = torch.zeros(n_mol + 1, dtype=torch.int64)
                mp[1:] = torch.cumsum(torch.bincount(b, minlength=n_mol), 0)
                mol_ptr = mp.pin_memory().to(dev, non_blocking=True)
                self._batch_cache = (b.clone(), n_mol, mol_ptr)
            mol_index = b.to(dev, non_blocking=True) if need_index else None
        else:
            b = batch.to(torch.int64)
            if N and bool((b[1:] < b[:-1]).any()):
                raise ValueError("batch indices must be non-decreasing (atoms grouped by structure)")
            n_mol = int(b.max().item()) + 1 if N else 0
            counts = torch.bincount(b, minlength=n_mol)
            mol_ptr = torch.zeros(n_mol + 1, dtype=torch.int64, device=dev)
            mol_ptr[1:] = torch.cumsum(counts, 0)
            mol_index = b
        box = pbc_t = None
        if self.periodic and pbc is not None and cell is not None and bool(torch.as_tensor(pbc).any()):
            on_host = not (isinstance(cell, torch.Tensor) and cell.device.type != "cpu")
            if on_host:   # the same host cell as the last call: reuse its checked device copies
                ck = (n_mol, np.asarray(cell, dtype=np.float32).tobytes(), np.asarray(pbc, dtype=bool).tobytes())
                if self._cell_cache is not None and self._cell_cache[0] == ck:
                    box, pbc_t = self._cell_cache[1]
                    bt = Batch(atomic_numbers.to(torch.int64).contiguous(),
                               positions.detach().to(torch.float32).contiguous(), mol_ptr, box, pbc_t)
                    return bt, mol_index, n_mol
            vdev = torch.device("cpu") if on_host else dev   # where the cell is checked
            cell_t = torch.as_tensor(cell, dtype=torch.float32, device=vdev).reshape(-1, 3, 3)
            pbc_b = torch.as_tensor(pbc, device=vdev).reshape(-1, 3).to(torch.bool)
            if cell_t.shape[0] == 1 and n_mol > 1:
                cell_t = cell_t.expand(n_mol, 3, 3)
                pbc_b = pbc_b.expand(n_mol, 3)
            off = cell_t - torch.diag_embed(torch.diagonal(cell_t, dim1=1, dim2=2))
            if bool((off.abs() > 0).any()):
                raise NotImplementedError("periodic cells must be orthorhombic (diagonal cell matrix)")
            mixed = pbc_b.any(dim=1) & ~pbc_b.all(dim=1)
            if bool(mixed.any()):
                raise NotImplementedError("periodicity must be on all three axes or none")
            box = torch.diagonal(cell_t, dim1=1, dim2=2).contiguous()
            pbc_t = pbc_b.all(dim=1).to(torch.uint8).contiguous()
            if on_host:
                box = box.pin_memory().to(dev, non_blocking=True)
                pbc_t = pbc_t.pin_memory().to(dev, non_blocking=True)
                self._cell_cache = (ck, (box, pbc_t))
        bt = Batch(atomic_numbers.to(torch.int64).contiguous(),
                   positions.detach().to(torch.float32).contiguous(), mol_ptr, box, pbc_t)
        return bt, mol_index, n_mol

    # ------------------------------------------------------------- forward
    def forward(self, atomic_numbers: torch.Tensor, positions: torch.Tensor,
                cell: Optional[torch.Tensor] = None, pbc: Optional[torch.Tensor] = None,
                batch: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Total energy: 0-dim for one structure, [B] for a batch
        (student_model.py:634-757).  Differentiable w.r.t. positions."""
        if not self.fused:
            bt, mol_index, n_mol = self._make_batch(atomic_numbers, positions, cell, pbc, batch)
            E = self._module_energy(positions, bt, mol_index).to(positions.dtype)
            return E.sum() if n_mol <= 1 else E
        bt, mol_index, n_mol = self._make_batch(atomic_numbers, positions, cell, pbc, batch)
        train = _trainable(self) if self.training and torch.is_grad_enabled() else []
        if train:
            # parameter gradients (to second order, for force losses) from the CUDA passes
            E = _EnergyTrain.apply(positions, self, bt, mol_index, *[p for _, p in train])
        else:
            E = _EnergyForces.apply(positions, self, bt, mol_index)
        # one structure -> 0-dim, several -> [B]  (student_model.py:739-755)
        return E.sum() if n_mol <= 1 else E

    def predict_energy_and_forces(self, atomic_numbers: torch.Tensor, positions: torch.Tensor,
                                  cell: Optional[torch.Tensor] = None, pbc: Optional[torch.Tensor] = None
                                  ) -> Tuple[torch.Tensor, torch.Tensor]:
        """(energy, forces) with forces from the CUDA adjoint
        (student_model.py:759-795).  In training mode with trainable
        parameters the forces are -dE/dpos taken with create_graph=True, as
        the reference does, so a loss on them back-propagates into the
        parameters."""
        if not self.fused:
            train = self.training and torch.is_grad_enabled() and bool(_trainable(self))
            E, F, _, _ = self._module_call(atomic_numbers, positions, cell, pbc, None, create_graph=train)
            E = E.to(positions.dtype).sum()
            return (E, F.to(positions.dtype)) if train else (E.detach(), F.detach().to(positions.dtype))
        if self.training and torch.is_grad_enabled() and _trainable(self):
            x = positions if positions.requires_grad else positions.detach().requires_grad_(True)
            E = self.forward(atomic_numbers, x, cell=cell, pbc=pbc)
            F = -torch.autograd.grad(E, x, grad_outputs=torch.ones_like(E), create_graph=True)[0]
            return E, F
        bt, _, _ = self._make_batch(atomic_numbers, positions, cell, pbc, None)
        E, F, _ = self._engine_call(bt, forces=True)
        return E[0].to(positions.dtype), F.to(positions.dtype)

    def forward_with_analytical_forces(self, atomic_numbers: torch.Tensor, positions: torch.Tensor,
                                       cell: Optional[torch.Tensor] = None, pbc: Optional[torch.Tensor] = None,
                                       batch: Optional[torch.Tensor] = None
                                       ) -> Tuple[torch.Tensor, torch.Tensor]:
        """(energy, forces) without autograd (student_model.py:797-932, which
        differentiates the radial basis and cutoff by hand and the rest by
        autograd).  Here the whole reverse pass is hand-written: forces are
        the library's CUDA adjoint.  energy is 0-dim for one structure and
        [B] for a batch (as ``forward``); forces [N,3]; neither carries an
        autograd graph."""
        if not self.fused:
            E, F, _, n_mol = self._module_call(atomic_numbers, positions, cell, pbc, batch)
            E = E.detach().to(positions.dtype)
            return (E.sum() if n_mol <= 1 else E), F.detach().to(positions.dtype)
        bt, _, n_mol = self._make_batch(atomic_numbers, positions, cell, pbc, batch, need_index=False)
        E, F, _ = self._engine_call(bt, forces=True)
        E = E.to(positions.dtype)
        return (E.sum() if n_mol <= 1 else E), F.to(positions.dtype)

    def energy_and_forces(self, atomic_numbers: torch.Tensor, positions: torch.Tensor,
                          batch: Optional[torch.Tensor] = None, cell=None, pbc=None
                          ) -> Tuple[torch.Tensor, torch.Tensor]:
        """Batched (energies [B] float64, forces [N,3] float32) in one call,
        without autograd -- the batched calculator path
        (ase_calculator.py:708-770).  Atomic numbers and positions in host
        memory (pinned for asynchronous copies) give results in host memory:
        the inputs go straight into the cached CUDA graph's buffers and the
        results and status come back behind one synchronisation."""
        host = positions.device.type == "cpu" and atomic_numbers.device.type == "cpu"
        if not self.fused:
            E, F, _, _ = self._module_call(atomic_numbers, positions, cell, pbc, batch)
            E, F = E.detach(), F.detach().to(torch.float32)
            return (E.cpu(), F.cpu()) if host else (E, F)
        bt, _, _ = self._make_batch(atomic_numbers, positions, cell, pbc, batch, need_index=False,
                                    host_inputs=host)
        E, F, _ = self._engine_call(bt, forces=True, to_host=host)
        return E, F

    def energy_forces_virial(self, atomic_numbers, positions, cell=None, pbc=None, batch=None):
        """Energies [B], forces [N,3] and dE/d(strain) [B,3,3] in one call."""
        if not self.fused:
            E, F, W, _ = self._module_call(atomic_numbers, positions, cell, pbc, batch, virial=True)
            return E.detach(), F.detach().to(torch.float32), W.detach().to(torch.float64)
        bt, _, _ = self._make_batch(atomic_numbers, positions, cell, pbc, batch)
        return self._engine_call(bt, forces=True, virial=True)

    # ---------------------------------------------------------- checkpoint
    def save(self, path: Union[str, Path]):
        """Reference checkpoint format (student_model.py:1075-1099)."""
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        torch.save({"model_state_dict": self.state_dict(),
                    "config": {"hidden_dim": self.hidden_dim, "num_interactions": self.num_interactions,
                               "num_rbf": self.num_rbf, "cutoff": self.cutoff, "max_z": self.max_z,
                               "use_torch_cluster": self.use_torch_cluster},
                    "num_parameters": self.num_parameters()}, path)

    @classmethod
    def load(cls, path: Union[str, Path], device: str = "cpu", **kwargs):
        """Load a reference checkpoint, inferring missing config entries
        from state_dict shapes (student_model.py:1101-1176).  A trainer
        checkpoint's ``model.`` key prefix is stripped."""
        ckpt = torch.load(path, map_location="cpu", weights_only=False)
        return cls.from_state_dict(ckpt["model_state_dict"], config=ckpt.get("config", {}), **kwargs).to(device)

    @classmethod
    def from_state_dict(cls, sd: Dict[str, torch.Tensor], config: Optional[dict] = None, **kwargs):
        """Model from a reference-layout state_dict (checkpoint, trainer
        checkpoint with ``model.`` keys, or a TorchScript archive's
        state_dict), config entries missing from ``config`` inferred from the
        tensor shapes."""
        config = dict(config or {})
        config.setdefault("use_torch_cluster", True)
        keep = {"hidden_dim", "num_interactions", "num_rbf", "cutoff", "max_z", "learnable_rbf",
                "use_torch_cluster"}
        cfg = {k: v for k, v in config.items() if k in keep}
        if any(k.startswith("model.") for k in sd):
            sd = {k[len("model."):] if k.startswith("model.") else k: v for k, v in sd.items()}
        if "hidden_dim" not in cfg and "embedding.weight" in sd:
            cfg["hidden_dim"] = sd["embedding.weight"].shape[1]
        if "num_rbf" not in cfg and "rbf.centers" in sd:
            cfg["num_rbf"] = sd["rbf.centers"].shape[0]
        if "num_interactions" not in cfg:
            ids = {int(k.split(".")[1]) for k in sd if k.startswith("interactions.")}
            if ids:
                cfg["num_interactions"] = len(ids)
        cfg.setdefault("cutoff", 5.0)
        if "max_z" not in cfg and "embedding.weight" in sd:
            cfg["max_z"] = sd["embedding.weight"].shape[0] - 1
        cfg.update(kwargs)
        model = cls(**cfg)
        model.load_state_dict(sd)
        return model


__all__ = ["StudentForceField", "PaiNNInteraction", "PaiNNMessage", "PaiNNUpdate", "GaussianRBF",
           "CosineCutoff"]
