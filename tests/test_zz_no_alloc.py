"""The allocation-free radius graph (mlff_radius_graph_noalloc).

Some callers cannot allocate device memory or give the library a
workspace; this entry point keeps its scratch in a fixed-size device array
inside the library instead.  The GPU test calls it through the C ABI twice
in a row (two different systems, so the second call must not see the
first call's leftovers) and compares each CSR with the one the
workspace-based entry point builds.  The CSR is integer data: equality is
exact.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch


def _system(Z, pos, mol_ptr, box=None, pbc=None):
    from mlff_gb300.engine import make_batch
    return make_batch(Z, pos, mol_ptr, box, pbc)


def _noalloc_csr(lib, batch, cap):
    row_ptr = torch.full((batch.n_atoms + 1,), -7, dtype=torch.int32, device="cuda")
    col = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
    status = torch.full((4,), -7, dtype=torch.int32, device="cuda")
    sysd = batch.system()
    r = lib.mlff_radius_graph_noalloc(ctypes.byref(sysd), 5.0, cap, row_ptr.data_ptr(), col.data_ptr(),
                                      status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert r == 0, lib.mlff_last_error_string()
    torch.cuda.synchronize()
    st = status.cpu().numpy()
    return row_ptr.cpu().numpy(), col.cpu().numpy(), st


def _workspace_csr(batch):
    from mlff_gb300.engine import Engine, dims_of
    eng = Engine(dims_of(128, 20, 3, 119, 5.0))
    row_ptr, col = eng.neighbors(batch)
    return row_ptr.cpu().numpy(), col.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_radius_graph_matches_workspace_entry_point():
    from mlff_gb300 import _lib, systems
    lib = _lib.load()
    mol = systems.molecule_batch(40, 10, 120, seed=21)
    water = systems.water_box(n_water=150, L=16.0, d_oo=2.3, seed=22)
    cases = [
        _system(mol.Z, mol.pos.astype(np.float32), mol.mol_ptr),
        _system(water.Z, water.pos.astype(np.float32), water.mol_ptr, water.box, water.pbc),
    ]
    for batch in cases:   # two calls in a row on the shared scratch
        ref_row, ref_col = _workspace_csr(batch)
        cap = min(len(ref_col) + 4096, 1 << 20)
        row, col, st = _noalloc_csr(lib, batch, cap)
        assert st[0] == 0, st
        n_edges = int(ref_row[-1])
        assert st[1] == n_edges
        np.testing.assert_array_equal(row, ref_row)
        np.testing.assert_array_equal(col[:n_edges], ref_col)


@pytest.mark.gpu
def test_noalloc_radius_graph_above_8192_atoms_and_at_the_limit():
    """Sizes whose row-pointer scan spans several blocks (the multi-block
    scan keeps its partial sums in the shared array): a 9,000-atom water box
    and a box of exactly MLFF_NOALLOC_MAX_ATOMS = 16,384 atoms, one call
    after the other."""
    from mlff_gb300 import _lib, systems
    lib = _lib.load()
    water = systems.water_box(n_water=3000, L=44.8, d_oo=2.5, seed=23)
    box = systems.large_box(n_atoms=16384, seed=24)
    assert water.n_atoms == 9000 and box.n_atoms == 16384
    for s in (water, box):
        batch = _system(s.Z, s.pos.astype(np.float32), s.mol_ptr, s.box, s.pbc)
        ref_row, ref_col = _workspace_csr(batch)
        n_edges = int(ref_row[-1])
        cap = min(n_edges + 4096, 1 << 20)
        assert n_edges < cap
        row, col, st = _noalloc_csr(lib, batch, cap)
        assert st[0] == 0, st
        assert st[1] == n_edges
        np.testing.assert_array_equal(row, ref_row)
        np.testing.assert_array_equal(col[:n_edges], ref_col)


@pytest.mark.gpu
def test_noalloc_capacity_reported():
    from mlff_gb300 import _lib, systems
    lib = _lib.load()
    mol = systems.lattice_molecule(60, seed=0)
    batch = _system(mol.Z, mol.pos.astype(np.float32), mol.mol_ptr)
    _, _, st = _noalloc_csr(lib, batch, 100)
    assert st[0] == _lib.ERR_CAPACITY and st[1] == 2794


def test_noalloc_rejects_sizes_beyond_the_static_limit():
    from mlff_gb300 import _lib
    lib = _lib.load()
    s = _lib.System()
    s.n_atoms = 16385
    s.n_mol = 1
    dummy = ctypes.c_void_p(16)
    r = lib.mlff_radius_graph_noalloc(ctypes.byref(s), 5.0, 1000, dummy, dummy, dummy, None)
    assert r == _lib.ERR_INVALID
    assert b"static scratch limit" in lib.mlff_last_error_string()
    s.n_atoms = 100
    r = lib.mlff_radius_graph_noalloc(ctypes.byref(s), 5.0, (1 << 20) + 1, dummy, dummy, dummy, None)
    assert r == _lib.ERR_INVALID
