"""CUDA path vs the oracle / the reference's golden vectors (GPU only).

Tolerances (float32 device arithmetic vs the float64 oracle): forces max
|dF| <= 1e-3 eV/A (the target bar); energies |dE| <= 5e-5 eV per atom
(0.05 meV/atom; the split-FP16 tensor-core path measures up to 2.3e-5 eV per
atom on the trained-like weights -- its FP32 accumulation truncates, so the
error exceeds a round-to-nearest emulation by about 5x).
The edge set is compared bit for bit.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import case_names
from oracle import nbr, painn

pytestmark = pytest.mark.gpu

F_TOL = 1e-3
E_TOL_PER_ATOM = 5e-5
PATHS = ["fp32", "tuned_fp32", "fp16x3"]
CASES = ["batch6", "cutoff_edge", "methane", "molecule60", "water"]


def engine_for(weights, precision="tuned_fp32"):
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision=precision).to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    m.eval()
    return m


def run(model, Z, pos, mol_ptr, box=None, pbc=None, virial=False):
    from mlff_gb300.engine import make_batch
    b = make_batch(Z, pos, mol_ptr, box, pbc)
    E, F, V = model.engine().energy_forces(b, model.path, forces=True, virial=virial)
    torch.cuda.synchronize()
    return E.cpu().numpy(), F.cpu().numpy(), (None if V is None else V.cpu().numpy())


@pytest.mark.parametrize("name", CASES)
def test_neighbors_bit_exact_vs_reference(golden_cases, weights_seed0, name):
    from mlff_gb300.engine import make_batch
    g = golden_cases
    m = engine_for(weights_seed0)
    b = make_batch(g[f"{name}/Z"], g[f"{name}/pos"], g[f"{name}/mol_ptr"])
    row_ptr, col = m.engine().neighbors(b)
    row_ptr = row_ptr.cpu().numpy().astype(np.int64)
    rows = np.repeat(np.arange(len(row_ptr) - 1), np.diff(row_ptr))
    ei = g[f"{name}/edge_index"]
    np.testing.assert_array_equal(rows, ei[0])
    np.testing.assert_array_equal(col.cpu().numpy(), ei[1])


@pytest.mark.parametrize("n_water,L,seed", [(1000, 31.0, 2), (50, 11.0, 3)])
def test_neighbors_periodic_bit_exact_vs_oracle(weights_seed0, n_water, L, seed):
    from mlff_gb300 import systems
    from mlff_gb300.engine import make_batch
    s = systems.water_box(n_water=n_water, L=L, seed=seed)
    pos32 = s.pos.astype(np.float32)
    src, dst, _ = nbr.radius_graph(pos32, s.mol_ptr, 5.0, s.box, s.pbc)
    m = engine_for(weights_seed0)
    row_ptr, col = m.engine().neighbors(make_batch(s.Z, pos32, s.mol_ptr, s.box, s.pbc))
    row_ptr = row_ptr.cpu().numpy().astype(np.int64)
    np.testing.assert_array_equal(np.repeat(np.arange(len(row_ptr) - 1), np.diff(row_ptr)), src)
    np.testing.assert_array_equal(col.cpu().numpy(), dst)


def test_neighbors_large_box_vs_oracle(weights_seed0):
    from mlff_gb300 import systems
    from mlff_gb300.engine import make_batch
    s = systems.large_box(n_atoms=20_000, seed=5)
    pos32 = s.pos.astype(np.float32)
    src, dst, _ = nbr.radius_graph(pos32, s.mol_ptr, 5.0, s.box, s.pbc)
    m = engine_for(weights_seed0)
    row_ptr, col = m.engine().neighbors(make_batch(s.Z, pos32, s.mol_ptr, s.box, s.pbc))
    assert int(row_ptr[-1]) == len(src)
    np.testing.assert_array_equal(col.cpu().numpy(), dst)


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("tag", ["seed", "bias"])
@pytest.mark.parametrize("name", CASES)
def test_energy_forces_vs_reference_fp64(golden_cases, weights_seed0, weights_bias, path, tag, name):
    g = golden_cases
    W = weights_seed0 if tag == "seed" else weights_bias
    m = engine_for(W, path)
    E, F, _ = run(m, g[f"{name}/Z"], g[f"{name}/pos"], g[f"{name}/mol_ptr"])
    n_atoms = len(g[f"{name}/Z"])
    dE = np.abs(E - g[f"{name}/{tag}/E64"]).max()
    assert dE <= E_TOL_PER_ATOM * n_atoms, dE
    if name == "methane":
        return  # |v| = 0 at the carbon by symmetry: forces undefined (see oracle test)
    dF = np.abs(F - g[f"{name}/{tag}/F64"]).max()
    assert dF <= F_TOL, dF


@pytest.mark.parametrize("path", PATHS)
def test_periodic_energy_forces_virial_vs_oracle(weights_bias, path):
    from mlff_gb300 import systems
    s = systems.water_box(n_water=60, L=11.5, d_oo=2.2, seed=8)
    pos32 = s.pos.astype(np.float32)
    m = engine_for(weights_bias, path)
    E, F, V = run(m, s.Z, pos32, s.mol_ptr, s.box, s.pbc, virial=True)
    E0, F0, V0 = painn.energy_forces(weights_bias, s.Z, pos32.astype(np.float64), s.mol_ptr, box=s.box,
                                     pbc=s.pbc, virial=True)
    assert abs(E[0] - float(E0[0])) <= E_TOL_PER_ATOM * s.n_atoms
    assert np.abs(F - F0.numpy()).max() <= F_TOL
    np.testing.assert_allclose(V[0], V0.numpy()[0], rtol=0, atol=2e-3 * max(1.0, np.abs(V0.numpy()).max()))


@pytest.mark.parametrize("path", PATHS)
def test_batch_equals_individual(golden_cases, weights_bias, path):
    g = golden_cases
    Z, pos, mp = g["batch6/Z"], g["batch6/pos"], g["batch6/mol_ptr"]
    m = engine_for(weights_bias, path)
    E, F, _ = run(m, Z, pos, mp)
    for i in range(len(mp) - 1):
        a, b = mp[i], mp[i + 1]
        Ei, Fi, _ = run(m, Z[a:b], pos[a:b], np.array([0, b - a]))
        assert abs(Ei[0] - E[i]) <= 1e-4 * max(1.0, abs(E[i]))
        assert np.abs(Fi - F[a:b]).max() <= 1e-4


@pytest.mark.parametrize("path", ["tuned_fp32", "fp16x3"])
def test_forces_match_fd_of_oracle_energy(golden_cases, weights_bias, path):
    """Central differences (step 1e-4 A) of the float64 model energy vs the
    device forces from the hand-written adjoint."""
    g = golden_cases
    Z, pos, mp = g["molecule60/Z"], g["molecule60/pos"].astype(np.float64), g["molecule60/mol_ptr"]
    m = engine_for(weights_bias, path)
    _, F, _ = run(m, Z, pos.astype(np.float32), mp)
    edges = nbr.radius_graph(pos.astype(np.float32), mp)
    h = 1e-4
    rng = np.random.default_rng(0)
    for a in rng.choice(len(Z), size=6, replace=False):
        for x in range(3):
            vals = []
            for sgn in (1, -1):
                p = pos.copy()
                p[a, x] += sgn * h
                Ep, _ = painn.energy_forces(weights_bias, Z, p, mp, edges=edges)
                vals.append(float(Ep[0]))
            fd = -(vals[0] - vals[1]) / (2 * h)
            assert abs(fd - F[a, x]) < 1e-3, (a, x, fd, F[a, x])


@pytest.mark.parametrize("path", ["tuned_fp32", "fp16x3"])
def test_fused_path_is_deterministic(golden_cases, weights_bias, path):
    g = golden_cases
    m = engine_for(weights_bias, path)
    E1, F1, _ = run(m, g["batch6/Z"], g["batch6/pos"], g["batch6/mol_ptr"])
    E2, F2, _ = run(m, g["batch6/Z"], g["batch6/pos"], g["batch6/mol_ptr"])
    np.testing.assert_array_equal(E1, E2)
    np.testing.assert_array_equal(F1, F2)


def test_capacity_overflow_reported_then_grown(golden_cases, weights_seed0):
    """A too-small edge capacity is reported through the status word (no
    fault, no write past the buffer) and the engine retries with room."""
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    g = golden_cases
    m = engine_for(weights_seed0)
    eng = m.engine()
    b = make_batch(g["molecule60/Z"], g["molecule60/pos"], g["molecule60/mol_ptr"])
    cap = 100
    ws = eng.workspace_for(b.n_atoms, b.n_mol, cap, _lib.PATH_TUNED_FP32)
    E = torch.empty(1, dtype=torch.float64, device="cuda")
    F = torch.empty(b.n_atoms, 3, device="cuda")
    out = _lib.Outputs()
    out.energy, out.forces = E.data_ptr(), F.data_ptr()
    sysd = b.system()
    r = eng.lib.mlff_energy_forces(ctypes.byref(eng.dims), eng.packed.data_ptr(), ctypes.byref(sysd), cap,
                                   _lib.PATH_TUNED_FP32, ctypes.byref(out), ws.data_ptr(), ws.numel(),
                                   torch.cuda.current_stream().cuda_stream)
    assert r == _lib.OK
    code, n_edges, _ = eng.status()
    assert code == _lib.ERR_CAPACITY and n_edges == g["molecule60/edge_index"].shape[1]
    assert np.isnan(E.item())
    eng.edge_capacity.clear()
    E2, _, _ = eng.energy_forces(b, _lib.PATH_TUNED_FP32)
    assert np.isfinite(E2.item())


def test_bad_inputs_reported(weights_seed0):
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    m = engine_for(weights_seed0)
    eng = m.engine()
    with pytest.raises(_lib.MLFFError) as ei:
        eng.energy_forces(make_batch([1, 200], [[0, 0, 0], [1, 0, 0]], [0, 2]), _lib.PATH_TUNED_FP32)
    assert ei.value.code == _lib.ERR_INVALID
    with pytest.raises(_lib.MLFFError) as ei:
        eng.energy_forces(make_batch([1, 1], [[0, 0, 0], [1, 0, 0]], [0, 2], box=[[6.0, 6.0, 6.0]],
                                     pbc=[True]), _lib.PATH_TUNED_FP32)
    assert ei.value.code == _lib.ERR_BOX


def _open_cluster(n_atoms, seed):
    """An open cluster at the 100k box's density: the jittered lattice of
    large_box without periodicity."""
    from mlff_gb300 import systems
    s = systems.large_box(n_atoms=n_atoms, seed=seed)
    s.pbc = np.zeros(1, bool)
    s.box = np.zeros((1, 3))
    return s


@pytest.mark.parametrize("n_atoms", [256, 20_000])
def test_neighbors_open_cluster_cell_grid_vs_oracle(weights_seed0, n_atoms):
    """Open structures of 256 atoms or more are binned into a bounding-box
    cell grid; the edge set must equal the oracle's all-pairs search bit for
    bit."""
    from mlff_gb300.engine import make_batch
    s = _open_cluster(n_atoms, seed=6)
    pos32 = s.pos.astype(np.float32)
    src, dst, _ = nbr.radius_graph(pos32, s.mol_ptr, 5.0)
    m = engine_for(weights_seed0)
    row_ptr, col = m.engine().neighbors(make_batch(s.Z, pos32, s.mol_ptr))
    row_ptr = row_ptr.cpu().numpy().astype(np.int64)
    assert int(row_ptr[-1]) == len(src)
    np.testing.assert_array_equal(np.repeat(np.arange(s.n_atoms), np.diff(row_ptr)), src)
    np.testing.assert_array_equal(col.cpu().numpy(), dst)


def test_neighbors_mixed_batch_vs_oracle(weights_seed0):
    """Small open molecules (all pairs), large open clusters (cell grid), an
    elongated open chain (few cells on two axes) and a periodic box in one
    batch."""
    from mlff_gb300 import systems
    from mlff_gb300.engine import make_batch
    rng = np.random.default_rng(7)
    chain = systems.lattice_molecule(300, seed=8)
    chain.pos = np.stack([np.arange(300) * 1.1, 0.3 * rng.standard_normal(300), 0.3 * rng.standard_normal(300)], 1)
    parts = [systems.lattice_molecule(50, seed=1), _open_cluster(1000, seed=2), chain,
             systems.water_box(n_water=60, L=11.5, d_oo=2.2, seed=8), _open_cluster(300, seed=3)]
    s = systems.concat(parts)
    pos32 = s.pos.astype(np.float32)
    src, dst, _ = nbr.radius_graph(pos32, s.mol_ptr, 5.0, s.box, s.pbc)
    m = engine_for(weights_seed0)
    row_ptr, col = m.engine().neighbors(make_batch(s.Z, pos32, s.mol_ptr, s.box, s.pbc))
    row_ptr = row_ptr.cpu().numpy().astype(np.int64)
    np.testing.assert_array_equal(np.repeat(np.arange(s.n_atoms), np.diff(row_ptr)), src)
    np.testing.assert_array_equal(col.cpu().numpy(), dst)


@pytest.mark.parametrize("path", ["fp16x3", "fp32"])
def test_open_cluster_energy_forces_vs_oracle(weights_bias, path):
    s = _open_cluster(600, seed=9)
    pos32 = s.pos.astype(np.float32)
    m = engine_for(weights_bias, path)
    E, F, _ = run(m, s.Z, pos32, s.mol_ptr)
    E0, F0 = painn.energy_forces(weights_bias, s.Z, pos32.astype(np.float64), s.mol_ptr)
    assert abs(E[0] - float(E0[0])) <= E_TOL_PER_ATOM * s.n_atoms
    assert np.abs(F - F0.numpy()).max() <= F_TOL
