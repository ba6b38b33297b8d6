"""Whole models at widths other than 128 (GPU only): the module-level path
(radius graph and every message / update block on the library's CUDA
kernels, geometry, basis, embedding and readout as tensor operations,
forces and virial by autograd) for the reference's small_model fixture
(tests/unit/test_student_model.py:44-54: hidden 64, 2 interactions, 10
basis functions, max_z 100), checked against the float64 oracle, central
differences and the other entry points."""
import tempfile
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import painn

pytestmark = pytest.mark.gpu

DEV = "cuda"


def small_model(seed=0):
    from mlff_gb300.student_model import StudentForceField
    torch.manual_seed(seed)
    m = StudentForceField(hidden_dim=64, num_interactions=2, num_rbf=10, cutoff=5.0, max_z=100).to(DEV)
    # non-zero biases, as a trained model has
    g = torch.Generator().manual_seed(seed + 1)
    with torch.no_grad():
        for name, p in m.named_parameters():
            if name.endswith("bias"):
                p.copy_(0.1 * torch.randn(p.shape, generator=g))
    return m.eval()


def weights(m):
    return {k: v.detach().cpu().numpy() for k, v in m.state_dict().items()}


def test_module_path_energy_forces_vs_float64_oracle():
    from mlff_gb300 import systems
    m = small_model()
    assert not m.fused
    s = systems.molecule_batch(6, 10, 40, seed=5)
    Z = torch.tensor(s.Z, device=DEV)
    pos = torch.tensor(s.pos, dtype=torch.float32, device=DEV)
    batch = torch.repeat_interleave(torch.arange(s.n_mol, device=DEV),
                                    torch.as_tensor(np.diff(s.mol_ptr), device=DEV))
    E, F = m.forward_with_analytical_forces(Z, pos, batch=batch)
    E0, F0 = painn.energy_forces(weights(m), s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr)
    n_per = np.diff(s.mol_ptr)
    e_err = np.abs(E.double().cpu().numpy() - E0.numpy()) / n_per
    f_err = np.abs(F.cpu().numpy() - F0.numpy()).max()
    print(f"width 64: energy error max {e_err.max():.2e} eV/atom, force error max {f_err:.2e} eV/A")
    assert e_err.max() < 2e-5
    assert f_err < 1e-3


def test_module_path_entry_points_agree():
    m = small_model()
    g = torch.Generator(device=DEV).manual_seed(2)
    Z = torch.randint(1, 9, (24,), device=DEV, generator=g)
    pos = torch.rand(24, 3, device=DEV, generator=g) * 6.0
    x = pos.clone().requires_grad_(True)
    E = m(Z, x)
    assert E.shape == torch.Size([])
    F = -torch.autograd.grad(E, x)[0]
    E2, F2 = m.predict_energy_and_forces(Z, pos)
    E3, F3 = m.forward_with_analytical_forces(Z, pos)
    Eh, Fh = m.energy_and_forces(Z.cpu(), pos.cpu())
    assert Fh.device.type == "cpu"
    # the per-module message kernels scatter with float atomics: results agree to rounding
    for f in (F2, F3, Fh.to(DEV)):
        torch.testing.assert_close(F, f, rtol=0, atol=1e-5)
    torch.testing.assert_close(E.detach(), E3, rtol=1e-6, atol=0)
    torch.testing.assert_close(E.detach().double(), Eh.to(DEV)[0], rtol=1e-6, atol=0)


def test_module_path_forces_match_central_differences():
    """The reference's finite-difference check (tests/unit/test_student_model
    .py:377-413, 5e-3 there), in float64 central differences of the
    module path's energy at step 1e-3 A."""
    m = small_model()
    g = torch.Generator(device=DEV).manual_seed(4)
    Z = torch.randint(1, 9, (12,), device=DEV, generator=g)
    pos = torch.rand(12, 3, device=DEV, generator=g) * 4.0
    _, F = m.forward_with_analytical_forces(Z, pos)
    h = 1e-3
    fd = torch.zeros_like(F)
    for i in range(12):
        for k in range(3):
            pp, pm = pos.clone(), pos.clone()
            pp[i, k] += h
            pm[i, k] -= h
            with torch.no_grad():
                fd[i, k] = -(m(Z, pp).double() - m(Z, pm).double()) / (2 * h)
    assert float((F - fd).abs().max()) < 5e-3


def test_module_path_virial_vs_oracle_strain_derivative():
    from mlff_gb300 import systems
    m = small_model()
    s = systems.water_box(n_water=40, L=10.0, d_oo=2.5, seed=3)
    Z = torch.tensor(s.Z, device=DEV)
    pos = torch.tensor(s.pos, dtype=torch.float32, device=DEV)
    cell = torch.diag(torch.tensor(s.box[0], dtype=torch.float32))
    pbc = torch.ones(3, dtype=torch.bool)
    E, F, W = m.energy_forces_virial(Z, pos, cell=cell, pbc=pbc)
    E0, F0, W0 = painn.energy_forces(weights(m), s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr,
                                     box=s.box, pbc=s.pbc, virial=True)
    assert abs(float(E[0]) - float(E0[0])) / s.n_atoms < 2e-5
    assert float(np.abs(F.cpu().numpy() - F0.numpy()).max()) < 1e-3
    np.testing.assert_allclose(W[0].cpu().numpy(), W0[0].numpy(), rtol=0, atol=2e-3)


def test_module_path_parameter_gradients_and_save_load():
    m = small_model()
    m.train()
    Z = torch.tensor([8, 1, 1, 6, 1], device=DEV)
    pos = torch.tensor([[0, 0, 0], [0.96, 0, 0], [-0.24, 0.93, 0], [2.5, 0.3, 0.1], [3.4, 0.9, 0.2]],
                       dtype=torch.float32, device=DEV)
    E = m(Z, pos)
    E.backward()
    grads = {n: p.grad for n, p in m.named_parameters()}
    assert grads["interactions.0.message.rbf_to_scalar.0.weight"].abs().sum() > 0
    assert grads["energy_head.0.weight"].abs().sum() > 0
    # a force loss needs second derivatives through the blocks' reverse kernels, which this path
    # does not provide: it raises instead of returning wrong gradients
    x = pos.clone().requires_grad_(True)
    _, F = m.predict_energy_and_forces(Z, x)
    with pytest.raises(RuntimeError):
        (F ** 2).sum().backward()
    m.eval()
    from mlff_gb300.student_model import StudentForceField
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "small.pt"
        m.save(path)
        m2 = StudentForceField.load(path, device=DEV).eval()
        assert m2.hidden_dim == 64 and m2.num_interactions == 2 and m2.num_rbf == 10
        for k, v in m.state_dict().items():
            torch.testing.assert_close(m2.state_dict()[k], v, rtol=0, atol=0)
        _, Fa = m.forward_with_analytical_forces(Z, pos)
        _, Fb = m2.forward_with_analytical_forces(Z, pos)
        torch.testing.assert_close(Fa, Fb, rtol=0, atol=1e-5)   # float-atomic scatters: equal to rounding
