"""Data-parallel replicas across GPUs (one process per GPU, no exchange on
the data path).

Independent structures -- a batch of molecules or MD replicas -- shard
across ranks by contiguous ranges of the CSR molecule list, balanced by atom
count; each rank evaluates its shard with its own engine, and the host
gathers the per-structure results.  The only collectives are host-level:
the gather of results and the max-over-ranks of the timed region.  A single
large periodic system would need a halo exchange after every interaction
layer; that is not built (the path shards only by structure).
"""
from typing import Optional, Tuple

import numpy as np
import torch


def shard_structures(mol_ptr, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous structure range [m0, m1) of ``rank``: the structure
    boundaries closest to rank/world of the total atom count (every rank
    gets whole structures; ranks may be empty when there are fewer
    structures than ranks)."""
    ptr = np.asarray(mol_ptr, dtype=np.int64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    B, N = len(ptr) - 1, int(ptr[-1])

    def cut(r: int) -> int:
        if r <= 0:
            return 0
        if r >= world:
            return B
        # first structure whose start is at or after the target atom
        return int(np.searchsorted(ptr[:-1], (N * r + world - 1) // world, side="left"))

    return cut(rank), cut(rank + 1)


def local_slice(mol_ptr, m0: int, m1: int):
    """Atom range and rebased molecule offsets of structures [m0, m1)."""
    ptr = np.asarray(mol_ptr, dtype=np.int64)
    a0, a1 = int(ptr[m0]), int(ptr[m1])
    return a0, a1, ptr[m0:m1 + 1] - a0


def gather_structure_values(local: torch.Tensor, m0: int, m1: int, n_mol: int,
                            group: Optional[object] = None) -> torch.Tensor:
    """Host-side gather of per-structure values (e.g. energies, float64)
    from all ranks into a [n_mol] tensor on every rank."""
    import torch.distributed as dist
    full = torch.zeros(n_mol, dtype=torch.float64)
    full[m0:m1] = local.detach().to("cpu", torch.float64)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(full, op=dist.ReduceOp.SUM, group=group)   # disjoint ranges: the sum is a gather
    return full


def aggregate_throughput(local_units: float, local_seconds: float, group: Optional[object] = None,
                         device: str = "cpu") -> Tuple[float, float, float]:
    """(total units, max seconds over ranks, units / s) of a timed region."""
    import torch.distributed as dist
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    units, secs = float(u.item()), float(t.item())
    return units, secs, units / secs if secs > 0 else 0.0
