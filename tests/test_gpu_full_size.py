"""Parity at the benchmark sizes (GPU only): the CUDA paths against the
float64 oracle on the full workloads the benchmark times.

* 256 open molecules of 10-120 atoms (16,858 atoms): every structure's
  energy and every force, tensor-core and plain FP32 paths;
* the 3,000-atom periodic water box: energy, forces and the strain
  derivative (virial);
* 128 replicas of a 64-atom molecule (the MD batch): every replica;
* the 100,000-atom periodic box: the edge set bit for bit against the C
  oracle, and energies and forces on a 20,000-atom box of the same density.

Tolerances as in test_gpu_parity: forces max |dF| <= 1e-3 eV/A, energies
|dE| <= 5e-5 eV per atom.  The oracle evaluates the messages in checkpointed
edge chunks here (same result up to float64 rounding) to stay within a few
GB of host memory.
"""
import numpy as np
import pytest
import torch

from oracle import nbr, painn

pytestmark = pytest.mark.gpu

F_TOL = 1e-3
E_TOL_PER_ATOM = 5e-5
CHUNK = 1 << 17


def seed_weights():
    from mlff_gb300.student_model import StudentForceField
    torch.manual_seed(0)
    return {k: v.numpy() for k, v in StudentForceField().state_dict().items()}


def gpu_eval(sysm, precision, virial=False):
    from mlff_gb300.engine import make_batch
    from mlff_gb300.student_model import StudentForceField
    torch.manual_seed(0)
    m = StudentForceField(precision=precision).cuda().eval()
    b = make_batch(sysm.Z, sysm.pos.astype(np.float32), sysm.mol_ptr, sysm.box if sysm.pbc.any() else None,
                   sysm.pbc if sysm.pbc.any() else None)
    E, F, V = m.engine().energy_forces(b, m.path, forces=True, virial=virial)
    torch.cuda.synchronize()
    return E.cpu().numpy(), F.cpu().numpy(), (None if V is None else V.cpu().numpy())


def oracle_eval(sysm, virial=False):
    out = painn.energy_forces(seed_weights(), sysm.Z, sysm.pos.astype(np.float32).astype(np.float64),
                              sysm.mol_ptr, box=sysm.box, pbc=sysm.pbc, virial=virial, edge_chunk=CHUNK)
    return tuple(t.numpy() for t in out)


def check_ef(sysm, E, F, E0, F0):
    per_atom = np.abs(E - E0) / np.diff(sysm.mol_ptr)
    assert per_atom.max() <= E_TOL_PER_ATOM, per_atom.max()
    dF = np.abs(F - F0).max()
    assert dF <= F_TOL, dF
    return per_atom.max(), dF


@pytest.fixture(scope="module")
def batch256():
    from mlff_gb300 import systems
    s = systems.workload("batch256")
    return s, oracle_eval(s)


@pytest.fixture(scope="module")
def water3000():
    from mlff_gb300 import systems
    s = systems.workload("water3000")
    return s, oracle_eval(s, virial=True)


@pytest.mark.parametrize("precision", ["fp16x3", "fp32"])
def test_batch256_all_structures_vs_fp64(batch256, precision):
    s, (E0, F0) = batch256
    assert s.n_mol == 256 and s.n_atoms == 16_858
    E, F, _ = gpu_eval(s, precision)
    check_ef(s, E, F, E0, F0)


@pytest.mark.parametrize("precision", ["fp16x3", "fp32"])
def test_water3000_energy_forces_virial_vs_fp64(water3000, precision):
    s, (E0, F0, V0) = water3000
    assert s.n_atoms == 3000 and bool(s.pbc[0])
    E, F, V = gpu_eval(s, precision, virial=True)
    check_ef(s, E, F, E0, F0)
    np.testing.assert_allclose(V[0], V0[0], rtol=0, atol=2e-3 * max(1.0, np.abs(V0).max()))


def test_replicas_128x64_vs_fp64():
    from mlff_gb300 import systems
    s = systems.workload("replicas128x64")
    one = s.molecule(0)
    E0, F0 = oracle_eval(one)
    E, F, _ = gpu_eval(s, "fp16x3")
    n = one.n_atoms
    assert s.n_mol == 128 and n == 64
    check_ef(s, E, F, np.repeat(E0, s.n_mol), np.tile(F0, (s.n_mol, 1)))
    # identical replicas give identical results: the batch layout adds no cross-talk
    np.testing.assert_array_equal(E, np.repeat(E[0], s.n_mol))
    np.testing.assert_array_equal(F.reshape(s.n_mol, n, 3), np.broadcast_to(F[:n], (s.n_mol, n, 3)))


def test_box100k_edges_bit_exact_vs_oracle():
    from mlff_gb300 import systems
    from mlff_gb300.engine import make_batch
    from mlff_gb300.student_model import StudentForceField
    s = systems.workload("box100k")
    pos32 = s.pos.astype(np.float32)
    src, dst, _ = nbr.radius_graph(pos32, s.mol_ptr, 5.0, s.box, s.pbc)
    m = StudentForceField(precision="fp16x3").cuda().eval()
    row_ptr, col = m.engine().neighbors(make_batch(s.Z, pos32, s.mol_ptr, s.box, s.pbc))
    row_ptr = row_ptr.cpu().numpy().astype(np.int64)
    assert int(row_ptr[-1]) == len(src) > 5_000_000
    np.testing.assert_array_equal(np.repeat(np.arange(s.n_atoms), np.diff(row_ptr)), src)
    np.testing.assert_array_equal(col.cpu().numpy(), dst)


def test_box20k_at_100k_density_vs_fp64():
    """Energies and forces on a 20,000-atom periodic box at the 100k box's
    number density (0.1 per A^3, about 55 neighbours per atom)."""
    from mlff_gb300 import systems
    s = systems.large_box(n_atoms=20_000, seed=5)
    E0, F0 = oracle_eval(s)
    E, F, _ = gpu_eval(s, "fp16x3")
    check_ef(s, E, F, E0, F0)
