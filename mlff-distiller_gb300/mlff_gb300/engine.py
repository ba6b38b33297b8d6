"""Device-side evaluation engine: packed weights + one workspace + the
C-ABI calls, on the current torch CUDA stream.

``Engine.energy_forces`` is the single entry the module, the calculator,
the MD driver and the benchmark use.  It grows the edge capacity and the
workspace when the neighbour build reports that they were too small and
re-runs the call.  Calls whose shape repeats (same atom and structure
counts, path and outputs) replay a cached CUDA graph of the whole step: the
inputs are copied into the graph's own buffers, one graph launch replaces
the ~40 kernel launches, and the outputs are copied out.

Host inputs (``to_host=True``: Z and positions in host memory, ideally
pinned) are copied straight into the graph's input buffers, and the
outputs and the status word come back with asynchronous copies into pinned
host buffers behind one stream synchronisation -- the call a host-side
caller (the ASE calculator) makes once per step.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, Optional, Tuple

import torch

from . import _lib

DEFAULT_EDGES_PER_ATOM = 64
GRAPH_CACHE_SIZE = 4
AUTOTUNE_REPEATS = 6
_tuned_buckets = set()   # (path, ceil log2 atoms, ceil log2 structures) tuned in this process


def _bucket(path: int, n_atoms: int, n_mol: int):
    return (path, max(n_atoms - 1, 0).bit_length(), max(n_mol - 1, 0).bit_length())


def _stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


@dataclass
class Batch:
    """A ragged batch on the device (int64 Z, float32 positions, CSR
    molecule offsets, optional orthorhombic boxes and periodic flags)."""
    Z: torch.Tensor
    pos: torch.Tensor
    mol_ptr: torch.Tensor
    box: Optional[torch.Tensor] = None
    pbc: Optional[torch.Tensor] = None

    @property
    def n_atoms(self) -> int:
        return int(self.Z.shape[0])

    @property
    def n_mol(self) -> int:
        return int(self.mol_ptr.shape[0] - 1)

    def system(self) -> _lib.System:
        s = _lib.System()
        s.n_atoms = self.n_atoms
        s.n_mol = self.n_mol
        s.pos = self.pos.data_ptr()
        s.Z = self.Z.data_ptr()
        s.mol_ptr = self.mol_ptr.data_ptr()
        s.box = None if self.box is None else self.box.data_ptr()
        s.pbc = None if self.pbc is None else self.pbc.data_ptr()
        return s


def make_batch(Z, pos, mol_ptr, box=None, pbc=None, device="cuda") -> Batch:
    dev = torch.device(device)
    Zt = torch.as_tensor(Z).to(device=dev, dtype=torch.int64).contiguous()
    Pt = torch.as_tensor(pos).to(device=dev, dtype=torch.float32).contiguous()
    Mt = torch.as_tensor(mol_ptr).to(device=dev, dtype=torch.int64).contiguous()
    Bt = Ct = None
    if pbc is not None:
        pb = torch.as_tensor(pbc).to(dtype=torch.bool).reshape(-1)
        if bool(pb.any()):
            Bt = torch.as_tensor(box).to(device=dev, dtype=torch.float32).reshape(-1, 3).contiguous()
            Ct = pb.to(device=dev, dtype=torch.uint8).contiguous()
    return Batch(Zt, Pt, Mt, Bt, Ct)


def dims_of(hidden, n_rbf, n_layers, n_species, cutoff) -> _lib.Dims:
    d = _lib.Dims()
    d.hidden, d.n_rbf, d.n_layers, d.n_species, d.cutoff = hidden, n_rbf, n_layers, n_species, cutoff
    return d


class Engine:
    """Owns the packed weights and a growable workspace for one model."""

    def __init__(self, dims: _lib.Dims, device="cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("mlff_gb300 needs a CUDA device (GB300, sm_103a); none is available")
        self.lib = _lib.load()
        self.dims = dims
        self.device = torch.device(device)
        nbytes = self.lib.mlff_packed_weights_size(ctypes.byref(dims))
        if nbytes == 0:
            raise _lib.MLFFError(_lib.ERR_UNSUPPORTED, _lib.last_error())
        self.packed = torch.zeros(nbytes // 4, dtype=torch.float32, device=self.device)
        self.workspace: Optional[torch.Tensor] = None
        self.edge_capacity: Dict[int, int] = {}
        self._param_version = None
        self.use_graphs = True          # replay cached CUDA graphs for repeated shapes
        self.auto_tune = True           # tune the tensor-core path's partition factor once per size bucket
        self._graphs: Dict[tuple, dict] = {}

    # -------------------------------------------------------------- weights
    def pack(self, sd: Dict[str, torch.Tensor]):
        """Pack a reference-layout state_dict (float32 tensors on device)."""
        L = self.dims.n_layers
        t = {k: v.detach().to(device=self.device, dtype=torch.float32).contiguous() for k, v in sd.items()}
        self._keep = t
        p = _lib.Params()
        p.embedding = t["embedding.weight"].data_ptr()
        p.rbf_centers = t["rbf.centers"].data_ptr()
        p.rbf_widths = t["rbf.widths"].data_ptr()
        for l in range(L):
            pre = f"interactions.{l}."
            p.filter_w1[l] = t[pre + "message.rbf_to_scalar.0.weight"].data_ptr()
            p.filter_b1[l] = t[pre + "message.rbf_to_scalar.0.bias"].data_ptr()
            p.filter_w2[l] = t[pre + "message.rbf_to_scalar.2.weight"].data_ptr()
            p.filter_b2[l] = t[pre + "message.rbf_to_scalar.2.bias"].data_ptr()
            p.mixing[l] = t[pre + "update.mixing_matrix"].data_ptr()
            p.update_w1[l] = t[pre + "update.update_mlp.0.weight"].data_ptr()
            p.update_b1[l] = t[pre + "update.update_mlp.0.bias"].data_ptr()
            p.update_w2[l] = t[pre + "update.update_mlp.2.weight"].data_ptr()
            p.update_b2[l] = t[pre + "update.update_mlp.2.bias"].data_ptr()
        for i, k in ((1, "0"), (2, "2"), (3, "4")):
            setattr(p, f"head_w{i}", t[f"energy_head.{k}.weight"].data_ptr())
            setattr(p, f"head_b{i}", t[f"energy_head.{k}.bias"].data_ptr())
        _lib.check(self.lib.mlff_pack_weights(ctypes.byref(self.dims), ctypes.byref(p),
                                              self.packed.data_ptr(), self.packed.numel() * 4,
                                              _stream_handle()))
        torch.cuda.current_stream().synchronize()
        del self._keep

    # ------------------------------------------------------------ workspace
    def workspace_for(self, n_atoms: int, n_mol: int, cap: int, path: int) -> torch.Tensor:
        need = self.lib.mlff_workspace_size(ctypes.byref(self.dims), n_atoms, n_mol, cap, path)
        if need == 0:
            raise _lib.MLFFError(_lib.ERR_INVALID, _lib.last_error())
        if self.workspace is None or self.workspace.numel() < need:
            self.workspace = None
            self.workspace = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self.workspace

    def capacity(self, n_atoms: int, path: int) -> int:
        return max(self.edge_capacity.get(path, 0), DEFAULT_EDGES_PER_ATOM * n_atoms, 1024)

    def status(self):
        code = ctypes.c_int32()
        ne = ctypes.c_int64()
        where = ctypes.c_int32()
        _lib.check(self.lib.mlff_read_status(self.workspace.data_ptr(), ctypes.byref(code), ctypes.byref(ne),
                                             ctypes.byref(where), _stream_handle()))
        return code.value, ne.value, where.value

    # ---------------------------------------------------------------- calls
    def energy_forces(self, batch: Batch, path: int = _lib.PATH_TUNED_TC, forces: bool = True,
                      virial: bool = False, atom_energy: bool = False, check: bool = True,
                      graph: Optional[bool] = None, to_host: bool = False
                      ) -> Tuple[torch.Tensor, Optional[torch.Tensor], Optional[torch.Tensor]]:
        """Energies [B] (float64), forces [N,3] (float32), dE/dstrain [B,3,3].

        ``graph`` (default: ``self.use_graphs``) replays a cached CUDA graph
        when a call of the same shape was seen before; the first call of a
        shape runs eagerly and captures the graph for the next one.  The
        batch's ``mol_ptr``, ``box`` and ``pbc`` tensors are taken as
        immutable: passing the same tensor object again skips its copy.
        ``to_host``: the batch's Z and positions may live in host memory and
        the results are returned in host memory."""
        use_graph = self.use_graphs if graph is None else graph
        if use_graph and check and not torch.cuda.is_current_stream_capturing():
            res = self._graph_call(batch, path, forces, virial, atom_energy, to_host)
            if res is not None:
                return res
        if to_host:
            dev = self.device
            db = Batch(batch.Z.to(dev, non_blocking=True), batch.pos.to(dev, non_blocking=True), batch.mol_ptr,
                       batch.box, batch.pbc)
            res = self._eager_call(db, path, forces, virial, atom_energy, check)
            return tuple(None if t is None else t.cpu() for t in res)
        return self._eager_call(batch, path, forces, virial, atom_energy, check)

    def _eager_call(self, batch: Batch, path: int, forces: bool, virial: bool, atom_energy: bool, check: bool):
        N, B = batch.n_atoms, batch.n_mol
        dev = self.device
        E = torch.empty(B, dtype=torch.float64, device=dev)
        F = torch.empty(N, 3, dtype=torch.float32, device=dev) if forces else None
        V = torch.empty(B, 3, 3, dtype=torch.float64, device=dev) if virial else None
        A = torch.empty(N, dtype=torch.float32, device=dev) if atom_energy else None
        out = _lib.Outputs()
        out.energy, out.forces, out.virial = E.data_ptr(), _lib.ptr(F), _lib.ptr(V)
        out.atom_energy = _lib.ptr(A)
        sysd = batch.system()
        for _ in range(4):
            cap = self.capacity(N, path)
            ws = self.workspace_for(N, B, cap, path)
            _lib.check(self.lib.mlff_energy_forces(ctypes.byref(self.dims), self.packed.data_ptr(),
                                                   ctypes.byref(sysd), cap, path, ctypes.byref(out),
                                                   ws.data_ptr(), ws.numel(), _stream_handle()))
            if not check:
                break
            code, n_edges, where = self.status()
            if code == _lib.ERR_CAPACITY:
                self.edge_capacity[path] = int(n_edges * 1.25) + 1024
                continue
            if code != _lib.OK:
                raise _lib.MLFFError(code, f"device status {code} at index {where}")
            # keep headroom for the next call (MD steps change edge counts)
            self.edge_capacity[path] = max(self.edge_capacity.get(path, 0), int(n_edges * 1.15) + 1024)
            break
        else:
            raise _lib.MLFFError(_lib.ERR_CAPACITY, "edge capacity did not converge")
        if atom_energy:
            return E, F, V, A
        return E, F, V

    def _graph_call(self, batch: Batch, path: int, forces: bool, virial: bool, atom_energy: bool,
                    to_host: bool = False):
        """Replay (or, on the first call of a shape, run eagerly and capture)
        a CUDA graph of one energy_forces call.  Returns None when the graph
        must be rebuilt and the call redone eagerly."""
        N, B = batch.n_atoms, batch.n_mol
        key = (N, B, path, forces, virial, atom_energy, batch.box is not None, batch.pbc is not None)
        ent = self._graphs.get(key)
        cap = self.capacity(N, path)
        ws_ptr = None if self.workspace is None else self.workspace.data_ptr()
        if ent is not None and (ent["cap"] != cap or ent["ws"] != ws_ptr):
            del self._graphs[key]
            ent = None
        if ent is None:
            if self.auto_tune and path == _lib.PATH_TUNED_TC and _bucket(path, N, B) not in _tuned_buckets:
                db = batch if not to_host else Batch(batch.Z.to(self.device), batch.pos.to(self.device),
                                                     batch.mol_ptr, batch.box, batch.pbc)
                self.autotune(db, path)
            if to_host:
                dev = self.device
                db = Batch(batch.Z.to(dev), batch.pos.to(dev), batch.mol_ptr, batch.box, batch.pbc)
                res = self._eager_call(db, path, forces, virial, atom_energy, True)
                self._capture_call(key, db, path, forces, virial, atom_energy)
                return tuple(None if t is None else t.cpu() for t in res)
            res = self._eager_call(batch, path, forces, virial, atom_energy, True)
            self._capture_call(key, batch, path, forces, virial, atom_energy)
            return res
        st, src = ent["batch"], ent["src"]
        st.Z.copy_(batch.Z, non_blocking=True)
        st.pos.copy_(batch.pos, non_blocking=True)
        # molecule offsets and boxes are usually the caller's cached tensors:
        # copied only when a different tensor comes in
        for name in ("mol_ptr", "box", "pbc"):
            t = getattr(batch, name)
            if t is not None and src.get(name) is not t:
                getattr(st, name).copy_(t, non_blocking=True)
                src[name] = t
        ent["graph"].replay()
        if to_host:
            return self._host_results(key, ent, path)
        code, n_edges, where = self.status()
        if code == _lib.ERR_CAPACITY:
            self.edge_capacity[path] = int(n_edges * 1.25) + 1024
            del self._graphs[key]
            return None
        if code != _lib.OK:
            raise _lib.MLFFError(code, f"device status {code} at index {where}")
        self.edge_capacity[path] = max(self.edge_capacity.get(path, 0), int(n_edges * 1.15) + 1024)
        return tuple(None if t is None else t.clone() for t in ent["out"])

    def _host_results(self, key, ent, path: int):
        """Status word and outputs of a replayed graph copied into pinned
        host buffers behind one synchronisation; host copies returned."""
        hb = ent.get("host")
        if hb is None:
            hb = ent["host"] = {"status": torch.empty(4, dtype=torch.int32).pin_memory(),
                                "out": [None if t is None else torch.empty(t.shape, dtype=t.dtype).pin_memory()
                                        for t in ent["out"]]}
        # the status word sits at offset 0 of the workspace: code, n_edges (low 31 bits), where, n_edges >> 31
        hb["status"].copy_(self.workspace[:16].view(torch.int32), non_blocking=True)
        for t, h in zip(ent["out"], hb["out"]):
            if t is not None:
                h.copy_(t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        code, lo, where, hi = hb["status"].tolist()
        n_edges = (hi << 31) | (lo & 0x7FFFFFFF)
        if code == _lib.ERR_CAPACITY:
            self.edge_capacity[path] = int(n_edges * 1.25) + 1024
            del self._graphs[key]
            return None
        if code != _lib.OK:
            raise _lib.MLFFError(code, f"device status {code} at index {where}")
        self.edge_capacity[path] = max(self.edge_capacity.get(path, 0), int(n_edges * 1.15) + 1024)
        return tuple(None if h is None else h.clone() for h in hb["out"])

    def _capture_call(self, key, batch: Batch, path: int, forces: bool, virial: bool, atom_energy: bool):
        N, B = batch.n_atoms, batch.n_mol
        cap = self.capacity(N, path)
        self.workspace_for(N, B, cap, path)          # sized before capture: no allocation inside it
        st = Batch(batch.Z.clone(), batch.pos.clone(), batch.mol_ptr.clone(),
                   None if batch.box is None else batch.box.clone(),
                   None if batch.pbc is None else batch.pbc.clone())
        torch.cuda.current_stream().synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            out = self._eager_call(st, path, forces, virial, atom_energy, False)
        while len(self._graphs) >= GRAPH_CACHE_SIZE:
            self._graphs.pop(next(iter(self._graphs)))
        self._graphs[key] = {"graph": g, "batch": st, "out": out, "cap": cap, "ws": self.workspace.data_ptr(),
                             "src": {"mol_ptr": batch.mol_ptr, "box": batch.box, "pbc": batch.pbc}}

    def autotune(self, batch: Batch, path: int = _lib.PATH_TUNED_TC, repeats: int = AUTOTUNE_REPEATS) -> dict:
        """Choose the partition factor and the update tile of this batch's
        size bucket (mlff_autotune: a few timed calls per candidate, then
        cached by the library for every call of the bucket).  Returns the
        choices and the milliseconds per call of each partition factor.
        Synchronises the stream; not for use during stream capture."""
        self.energy_forces(batch, path, graph=False)       # sizes the edge capacity and workspace
        N, B = batch.n_atoms, batch.n_mol
        cap = self.capacity(N, path)
        ws = self.workspace_for(N, B, cap, path)
        E = torch.empty(B, dtype=torch.float64, device=self.device)
        F = torch.empty(N, 3, dtype=torch.float32, device=self.device)
        out = _lib.Outputs()
        out.energy, out.forces = E.data_ptr(), F.data_ptr()
        chosen = ctypes.c_int32(1)
        ms = (ctypes.c_double * 3)()
        sysd = batch.system()
        _lib.check(self.lib.mlff_autotune(ctypes.byref(self.dims), self.packed.data_ptr(), ctypes.byref(sysd), cap,
                                          path, ctypes.byref(out), ws.data_ptr(), ws.numel(), _stream_handle(),
                                          int(repeats), ctypes.byref(chosen), ms))
        _tuned_buckets.add(_bucket(path, N, B))
        f, ut = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self.lib.mlff_autotune_query_shape(path, N, B, ctypes.byref(f), ctypes.byref(ut)))
        return {"partition_factor": int(chosen.value), "update_tile_atoms": int(ut.value),
                "ms_per_call": {f: round(ms[i], 4) for i, f in enumerate((1, 2, 4))}}

    def capture(self, batch: Batch, path: int = _lib.PATH_TUNED_TC, forces: bool = True):
        """One energy_forces call captured in a CUDA graph, for repeated
        evaluation of a fixed batch (the edge capacity must already be known:
        call energy_forces once first).  Returns (replay, E, F): replay()
        launches the graph on the current stream and refreshes E and F."""
        self.energy_forces(batch, path, forces=forces, graph=False)   # sizes capacity and workspace
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            E, F, _ = self.energy_forces(batch, path, forces=forces, check=False, graph=False)
        self._graph_keep = g
        return g.replay, E, F

    def neighbors(self, batch: Batch):
        """CSR (row_ptr, col) of the radius graph, for tests and tools."""
        N, B = batch.n_atoms, batch.n_mol
        path = _lib.PATH_TUNED_FP32
        sysd = batch.system()
        for _ in range(4):
            cap = self.capacity(N, path)
            ws = self.workspace_for(N, B, cap, path)
            _lib.check(self.lib.mlff_build_neighbors(ctypes.byref(self.dims), ctypes.byref(sysd), cap,
                                                     ws.data_ptr(), ws.numel(), _stream_handle()))
            code, n_edges, where = self.status()
            if code == _lib.ERR_CAPACITY:
                self.edge_capacity[path] = int(n_edges * 1.25) + 1024
                continue
            if code != _lib.OK:
                raise _lib.MLFFError(code, f"device status {code} at index {where}")
            row_ptr = torch.empty(N + 1, dtype=torch.int32, device=self.device)
            col = torch.empty(max(cap, 1), dtype=torch.int32, device=self.device)
            _lib.check(self.lib.mlff_copy_neighbors(ws.data_ptr(), N, B, cap, path, row_ptr.data_ptr(),
                                                    col.data_ptr(), _stream_handle()))
            return row_ptr, col[:n_edges]
        raise _lib.MLFFError(_lib.ERR_CAPACITY, "edge capacity did not converge")
