"""Data-parallel replicas across ranks, host logic on CPU with two gloo
ranks (127.0.0.1): structure sharding covers every structure exactly once,
balanced by atoms; the host gather of per-structure values reproduces the
single-process result; throughput aggregates units by sum and time by max."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, mol_ptr, values, out_q):
    import torch.distributed as dist
    from mlff_gb300.replicas import aggregate_throughput, gather_structure_values, local_slice, shard_structures
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m0, m1 = shard_structures(mol_ptr, rank, world)
        a0, a1, lptr = local_slice(mol_ptr, m0, m1)
        # per-structure "energy" of the local shard from its own atoms only
        local = torch.tensor([values[a0 + lptr[i]:a0 + lptr[i + 1]].sum() for i in range(m1 - m0)],
                             dtype=torch.float64)
        full = gather_structure_values(local, m0, m1, len(mol_ptr) - 1)
        units, secs, rate = aggregate_throughput(a1 - a0, 0.5 + rank, device="cpu")
        out_q.put((rank, m0, m1, a1 - a0, full.numpy(), units, secs, rate))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharding_gather_and_throughput():
    from mlff_gb300 import systems
    s = systems.molecule_batch(37, 10, 120, seed=5)
    vals = np.random.default_rng(0).standard_normal(s.n_atoms)
    ref = np.array([vals[s.mol_ptr[i]:s.mol_ptr[i + 1]].sum() for i in range(s.n_mol)])
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, s.mol_ptr, vals, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, a0, b0, n0, f0, u0, t0, v0), (r1, a1, b1, n1, f1, u1, t1, v1) = res
    assert (a0, b1) == (0, s.n_mol) and b0 == a1                # contiguous, complete, disjoint
    assert abs(n0 - n1) <= 120                                  # balanced by atoms (one structure at most)
    np.testing.assert_allclose(f0, ref, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(f0, f1)
    assert u0 == u1 == s.n_atoms and t0 == t1 == 1.5 and abs(v0 - s.n_atoms / 1.5) < 1e-9


def _oracle_worker(rank: int, world: int, port: int, Z, pos, mol_ptr, weights, out_q):
    import torch.distributed as dist
    from mlff_gb300.replicas import gather_structure_values, local_slice, shard_structures
    from oracle import painn
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m0, m1 = shard_structures(mol_ptr, rank, world)
        a0, a1, lptr = local_slice(mol_ptr, m0, m1)
        E, _ = painn.energy_forces(weights, Z[a0:a1], pos[a0:a1], lptr)   # this rank's structures only
        full = gather_structure_values(torch.as_tensor(E), m0, m1, len(mol_ptr) - 1)
        out_q.put((rank, full.numpy()))
    finally:
        dist.destroy_process_group()


def test_two_rank_model_energies_equal_the_single_process_batch():
    """Each rank evaluates the model (the float64 oracle stands in for a
    rank's engine on CPU) on its own structures; the gathered per-structure
    energies equal one evaluation of the whole batch."""
    from mlff_gb300 import systems
    from oracle import painn
    golden = os.path.join(os.path.dirname(__file__), "golden")
    w = dict(np.load(os.path.join(golden, "weights_seed0.npz")))
    s = systems.molecule_batch(9, 10, 40, seed=6)
    pos = s.pos.astype(np.float32).astype(np.float64)
    E_ref, _ = painn.energy_forces(w, s.Z, pos, s.mol_ptr)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_oracle_worker, args=(r, 2, port, s.Z, pos, s.mol_ptr, w, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, full in res:
        np.testing.assert_allclose(full, E_ref.numpy(), rtol=1e-12, atol=1e-12)


def test_shard_edge_cases():
    from mlff_gb300.replicas import shard_structures
    ptr = np.array([0, 5, 10])
    assert [shard_structures(ptr, r, 4) for r in range(4)] in (
        [(0, 0), (0, 1), (1, 1), (1, 2)], [(0, 1), (1, 1), (1, 2), (2, 2)], [(0, 0), (0, 1), (1, 2), (2, 2)])
    cover = [shard_structures(ptr, r, 4) for r in range(4)]
    assert cover[0][0] == 0 and cover[-1][1] == 2 and all(cover[i][1] == cover[i + 1][0] for i in range(3))
    with pytest.raises(ValueError):
        shard_structures(ptr, 2, 2)
