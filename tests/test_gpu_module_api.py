"""The drop-in module surface on the GPU: the properties the reference's
unit tests check for StudentForceField and its blocks
(tests/unit/test_student_model.py), restated here for mlff_gb300, plus
numerical checks of the per-module kernels against a float64 torch
restatement of the blocks (student_model.py:324-470).

The reference's fixtures build the model without calling eval(), so most
checks run in training mode as they do there.  The full model supports
hidden_dim = 128 (the fused kernels); the blocks run at any width (the
reference's interaction test uses width 64 with 10 basis functions).
"""
import tempfile
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = "cuda"


def model(seed=0, train=True, **kw):
    from mlff_gb300.student_model import StudentForceField
    torch.manual_seed(seed)
    m = StudentForceField(**kw).to(DEV)
    return m.train(train)


def water():
    Z = torch.tensor([8, 1, 1], device=DEV)
    pos = torch.tensor([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0]], device=DEV)
    return Z, pos


def methane():
    Z = torch.tensor([6, 1, 1, 1, 1], device=DEV)
    a = 0.63
    pos = torch.tensor([[0, 0, 0], [a, a, a], [-a, -a, a], [-a, a, -a], [a, -a, -a]], dtype=torch.float32,
                       device=DEV)
    return Z, pos


# ------------------------------------------------------------ full model
@pytest.mark.parametrize("train", [True, False])
def test_forward_shapes_and_finite_for_many_sizes(train):
    m = model(train=train)
    g = torch.Generator(device=DEV).manual_seed(3)
    for n in (5, 10, 20, 50, 100, 200, 500):
        Z = torch.randint(1, 10, (n,), device=DEV, generator=g)
        pos = torch.randn(n, 3, device=DEV, generator=g) * 5.0
        E = m(Z, pos)
        assert E.shape == torch.Size([]) and torch.isfinite(E)


def test_autograd_forces_equal_the_other_force_entry_points():
    m = model(train=False)
    Z, pos = water()
    x = pos.clone().requires_grad_(True)
    E = m(Z, x)
    F = -torch.autograd.grad(E, x)[0]
    assert F.shape == pos.shape and torch.isfinite(F).all()
    E2, F2 = m.predict_energy_and_forces(Z, pos)
    E3, F3 = m.forward_with_analytical_forces(Z, pos)
    assert E3.shape == torch.Size([]) and not E3.requires_grad and not F3.requires_grad
    torch.testing.assert_close(F, F2, rtol=0, atol=1e-6)
    torch.testing.assert_close(F, F3, rtol=0, atol=1e-6)
    torch.testing.assert_close(E.detach(), E3, rtol=0, atol=1e-6)


def test_forward_with_analytical_forces_batch():
    m = model(train=False)
    Z, pos = water()
    Z2 = torch.cat([Z, Z])
    pos2 = torch.cat([pos, pos + torch.tensor([12.0, 0.0, 0.0], device=DEV)])
    batch = torch.tensor([0, 0, 0, 1, 1, 1], device=DEV)
    E, F = m.forward_with_analytical_forces(Z2, pos2, batch=batch)
    assert E.shape == (2,) and F.shape == (6, 3)
    torch.testing.assert_close(E[0], E[1], rtol=0, atol=1e-5)
    torch.testing.assert_close(F[:3], F[3:], rtol=0, atol=1e-5)


def test_predict_energy_and_forces_methane():
    m = model()
    Z, pos = methane()
    E, F = m.predict_energy_and_forces(Z, pos)
    assert E.shape == torch.Size([]) and F.shape == pos.shape
    assert torch.isfinite(E) and torch.isfinite(F).all()


def test_translation_permutation_and_extensivity():
    m = model()
    Z, pos = water()
    E1 = m(Z, pos)
    shift = torch.randn(3, device=DEV, generator=torch.Generator(device=DEV).manual_seed(1)) * 10.0
    assert abs(float(m(Z, pos + shift) - E1)) < 1e-5
    Zc = torch.tensor([6, 6, 6, 6], device=DEV)
    pc = torch.tensor([[0, 0, 0], [1.5, 0, 0], [0, 1.5, 0], [0, 0, 1.5]], dtype=torch.float32, device=DEV)
    perm = torch.tensor([2, 0, 3, 1], device=DEV)
    assert abs(float(m(Zc, pc) - m(Zc[perm], pc[perm]))) < 1e-5
    E2 = m(torch.cat([Z, Z]), torch.cat([pos, pos + torch.tensor([10.0, 0.0, 0.0], device=DEV)]))
    assert 1.9 < float(E2 / E1) < 2.1


def test_gradients_reach_positions_and_parameters():
    m = model()
    Z, pos = water()
    x = pos.clone().requires_grad_(True)
    m(Z, x).backward()
    assert x.grad is not None and torch.isfinite(x.grad).all()
    got = [n for n, p in m.named_parameters() if p.grad is not None and bool(p.grad.abs().sum() > 0)]
    assert "embedding.weight" in got and any(n.startswith("interactions.") for n in got)
    assert any(n.startswith("energy_head.") for n in got)


def test_forces_match_central_differences():
    m = model(train=False, precision="tuned_fp32")
    Z, pos = water()
    x = pos.clone().requires_grad_(True)
    F = -torch.autograd.grad(m(Z, x), x)[0]
    eps = 1e-3
    for i in range(3):
        for j in range(3):
            p1, p2 = pos.clone(), pos.clone()
            p1[i, j] += eps
            p2[i, j] -= eps
            fd = -(float(m(Z, p1)) - float(m(Z, p2))) / (2 * eps)
            assert abs(fd - float(F[i, j])) < 5e-3, (i, j, fd, float(F[i, j]))


def test_batch_of_two_structures():
    m = model()
    g = torch.Generator(device=DEV).manual_seed(2)
    Z = torch.randint(1, 10, (13,), device=DEV, generator=g)
    pos = torch.cat([torch.randn(5, 3, device=DEV, generator=g) * 2.0,
                     torch.randn(8, 3, device=DEV, generator=g) * 2.0 + torch.tensor([10.0, 0, 0], device=DEV)])
    batch = torch.cat([torch.zeros(5, dtype=torch.long, device=DEV), torch.ones(8, dtype=torch.long, device=DEV)])
    E = m(Z, pos, batch=batch)
    assert E.shape == (2,) and torch.isfinite(E).all()


def test_memory_of_a_1000_atom_forward_in_training_mode():
    m = model()
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats()
    g = torch.Generator(device=DEV).manual_seed(4)
    Z = torch.randint(1, 10, (1000,), device=DEV, generator=g)
    pos = torch.randn(1000, 3, device=DEV, generator=g) * 10.0
    E = m(Z, pos)
    torch.cuda.synchronize()
    assert torch.isfinite(E)
    assert torch.cuda.max_memory_allocated() / 2 ** 20 < 500


def test_save_and_load_roundtrip():
    m = model()
    Z, pos = water()
    E1 = m(Z, pos)
    from mlff_gb300.student_model import StudentForceField
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "model.pt"
        m.save(path)
        m2 = StudentForceField.load(path, device=DEV)
    assert abs(float(m2(Z, pos) - E1)) < 1e-6


# ----------------------------------------------------- blocks on their own
def ref_message(s, v, ei, rbf, evec, w1, b1, w2, b2):
    """float64 torch restatement of PaiNNMessage.forward (:346-387)."""
    H = s.shape[1]
    src, dst = ei
    h = rbf @ w1.T + b1
    f = (h * torch.sigmoid(h)) @ w2.T + b2
    fs, f1, f2 = torch.split(f, H, dim=-1)
    so = s + torch.zeros_like(s).index_add_(0, dst, s[src] * fs)
    vo = v + torch.zeros_like(v).index_add_(0, dst, v[src] * f1.unsqueeze(1) + evec.unsqueeze(-1) * f2.unsqueeze(1))
    return so, vo


def ref_update(s, v, w1, b1, w2, b2, mix):
    """float64 torch restatement of PaiNNUpdate.forward (:434-470)."""
    H = s.shape[1]
    z = torch.cat([s, torch.linalg.vector_norm(v, dim=1)], dim=-1) @ w1.T + b1
    a = (z * torch.sigmoid(z)) @ w2.T + b2
    a_s, g1, g2 = torch.split(a, H, dim=-1)
    return s + a_s, v * g1.unsqueeze(1) + torch.einsum("ij,njk->nik", mix, v) * g2.unsqueeze(1)


def block_inputs(H=64, R=10, N=10, E=30, seed=0):
    g = torch.Generator(device=DEV).manual_seed(seed)
    s = torch.randn(N, H, device=DEV, generator=g)
    v = torch.randn(N, 3, H, device=DEV, generator=g)
    ei = torch.randint(0, N, (2, E), device=DEV, generator=g)
    rbf = torch.randn(E, R, device=DEV, generator=g)
    evec = torch.randn(E, 3, device=DEV, generator=g)
    evec = evec / torch.linalg.vector_norm(evec, dim=1, keepdim=True)
    return s, v, ei, rbf, evec


def test_interaction_block_width_64():
    """The reference's interaction test: width 64, 10 basis functions, 10
    atoms, 30 random edges; shapes kept, no NaN."""
    from mlff_gb300.student_model import PaiNNInteraction
    torch.manual_seed(0)
    blk = PaiNNInteraction(hidden_dim=64, num_rbf=10).to(DEV)
    s, v, ei, rbf, evec = block_inputs()
    so, vo = blk(s, v, ei, rbf, evec)
    assert so.shape == s.shape and vo.shape == v.shape
    assert not torch.isnan(so).any() and not torch.isnan(vo).any()


@pytest.mark.parametrize("H,R", [(64, 10), (128, 20), (96, 7)])
def test_message_and_update_blocks_vs_float64(H, R):
    from mlff_gb300.student_model import PaiNNInteraction
    torch.manual_seed(1)
    blk = PaiNNInteraction(hidden_dim=H, num_rbf=R).to(DEV)
    s, v, ei, rbf, evec = block_inputs(H, R, N=40, E=300, seed=H)
    so, vo = blk(s, v, ei, rbf, evec)
    d = lambda t: t.detach().double()
    msg, upd = blk.message.rbf_to_scalar, blk.update.update_mlp
    s1, v1 = ref_message(d(s), d(v), ei, d(rbf), d(evec), d(msg[0].weight), d(msg[0].bias), d(msg[2].weight),
                         d(msg[2].bias))
    s2, v2 = ref_update(s1, v1, d(upd[0].weight), d(upd[0].bias), d(upd[2].weight), d(upd[2].bias),
                        d(blk.update.mixing_matrix))
    scale = max(1.0, float(s2.abs().max()), float(v2.abs().max()))
    assert float((so.double() - s2).abs().max()) < 1e-4 * scale
    assert float((vo.double() - v2).abs().max()) < 1e-4 * scale


def test_block_gradients_vs_float64_autograd():
    from mlff_gb300.student_model import PaiNNInteraction
    torch.manual_seed(2)
    H, R = 64, 10
    blk = PaiNNInteraction(hidden_dim=H, num_rbf=R).to(DEV)
    s, v, ei, rbf, evec = block_inputs(H, R, N=20, E=120, seed=5)
    ins = [t.clone().requires_grad_(True) for t in (s, v, rbf, evec)]
    so, vo = blk(ins[0], ins[1], ei, ins[2], ins[3])
    gw = torch.Generator(device=DEV).manual_seed(9)
    ws, wv = torch.randn(so.shape, device=DEV, generator=gw), torch.randn(vo.shape, device=DEV, generator=gw)
    ((so * ws).sum() + (vo * wv).sum()).backward()
    params = [blk.message.rbf_to_scalar[0].weight, blk.message.rbf_to_scalar[0].bias,
              blk.message.rbf_to_scalar[2].weight, blk.message.rbf_to_scalar[2].bias,
              blk.update.update_mlp[0].weight, blk.update.update_mlp[0].bias,
              blk.update.update_mlp[2].weight, blk.update.update_mlp[2].bias, blk.update.mixing_matrix]
    got = [t.grad for t in ins] + [p.grad for p in params]
    # float64 reference by autograd
    ri = [t.detach().double().requires_grad_(True) for t in (s, v, rbf, evec)]
    rp = [p.detach().double().requires_grad_(True) for p in params]
    s1, v1 = ref_message(ri[0], ri[1], ei, ri[2], ri[3], *rp[:4])
    s2, v2 = ref_update(s1, v1, *rp[4:])
    ((s2 * ws.double()).sum() + (v2 * wv.double()).sum()).backward()
    want = [t.grad for t in ri] + [p.grad for p in rp]
    for g, w in zip(got, want):
        scale = max(1.0, float(w.abs().max()))
        assert float((g.double() - w).abs().max()) < 2e-4 * scale


def test_block_rejects_out_of_range_edges():
    from mlff_gb300.student_model import PaiNNMessage
    blk = PaiNNMessage(64, 10).to(DEV)
    s, v, ei, rbf, evec = block_inputs()
    bad = ei.clone()
    bad[1, 7] = 10   # 10 atoms: index 10 is out of range
    with pytest.raises(IndexError):
        blk(s, v, bad, rbf, evec)
    so, _ = blk(s, v, ei, rbf, evec)   # the next call is unaffected
    assert torch.isfinite(so).all()
