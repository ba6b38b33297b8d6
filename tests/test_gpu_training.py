"""Training path (GPU only): parameter gradients of sum_b w_b E_b from the
CUDA reverse pass against float64 autograd through the oracle, determinism,
the force-loss term (sum_i G_i . dF_i/dtheta, forward mode over the reverse
pass) against float64 double backward through the oracle and against the
reference's own recorded training step, and what training buys: the
network fitted to a teacher's energies (and forces) on training molecules
predicts held-out molecules far better than the same network before
training.
"""
import numpy as np
import pytest
import torch

from oracle import painn

pytestmark = pytest.mark.gpu


def _model(weights, precision="fp32"):
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision=precision).to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    return m


def _batch(s):
    from mlff_gb300.engine import make_batch
    return make_batch(s.Z, s.pos, s.mol_ptr)


@pytest.mark.parametrize("wname", ["seed", "bias"])
def test_param_grads_vs_oracle(weights_seed0, weights_bias, wname):
    from mlff_gb300 import systems
    from mlff_gb300.training import param_grads
    W = weights_seed0 if wname == "seed" else weights_bias
    s = systems.molecule_batch(4, 10, 40, seed=11)
    rng = np.random.default_rng(0)
    w = rng.normal(size=s.n_mol)
    m = _model(W)
    E, grads, _ = param_grads(m, _batch(s), torch.tensor(w))
    E0, g0 = painn.param_grads(W, s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr, w)
    assert np.abs(E.cpu().numpy() - E0.numpy()).max() <= 2e-5 * s.n_atoms
    assert set(grads) == set(g0), set(grads) ^ set(g0)
    worst = 0.0
    for k, ref in g0.items():
        got = grads[k].double().cpu()
        scale = max(float(ref.abs().max()), 1e-6)
        err = float((got - ref).abs().max()) / scale
        worst = max(worst, err)
        assert err < 2e-4, (k, err)
    print("worst relative max error", worst)


def test_param_grads_repeatable(weights_bias):
    """Repeated calls give the same bits: the plain path sums messages and
    node adjoints per receiver row in edge order and the weight-gradient
    reductions in fixed splits (no float atomics), for the energy term and
    for the force term's forward-mode pass; so do its energies and forces."""
    from mlff_gb300 import _lib, systems
    from mlff_gb300.training import param_grads
    s = systems.molecule_batch(6, 10, 60, seed=12)
    m = _model(weights_bias)
    w = torch.linspace(-1, 1, s.n_mol, dtype=torch.float64)
    G = torch.tensor(np.random.default_rng(3).normal(size=(s.n_atoms, 3)))
    runs = [param_grads(m, _batch(s), w, forces=True, force_weights=G) for _ in range(2)]
    (E1, g1, F1), (E2, g2, F2) = runs
    torch.testing.assert_close(E1, E2, rtol=0, atol=0)
    torch.testing.assert_close(F1, F2, rtol=0, atol=0)
    for k in g1:
        torch.testing.assert_close(g1[k], g2[k], rtol=0, atol=0, msg=k)
    eng = m.engine()
    a = [t.cpu() for t in eng.energy_forces(_batch(s), _lib.PATH_PLAIN_FP32, graph=False)[:2]]
    b = [t.cpu() for t in eng.energy_forces(_batch(s), _lib.PATH_PLAIN_FP32, graph=False)[:2]]
    for x, y in zip(a, b):
        torch.testing.assert_close(x, y, rtol=0, atol=0)


def test_training_gain_over_untrained(weights_seed0, weights_bias):
    """Teacher: the model with the perturbed weights (float64 oracle
    energies).  Student: seed-0 weights, trained on 48 molecules with the
    library's gradients; evaluated on 16 held-out molecules with the
    tensor-core inference path."""
    from mlff_gb300 import systems
    from mlff_gb300.training import EnergyTrainer
    train = systems.molecule_batch(48, 10, 40, seed=21)
    test = systems.molecule_batch(16, 10, 40, seed=22)

    def teacher(s):
        E, _ = painn.energy_forces(weights_bias, s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr)
        return E.numpy()

    Et, Ev = teacher(train), teacher(test)
    m = _model(weights_seed0)
    tr = EnergyTrainer(m, lr=3e-3, per_atom=True)
    bt, bv = _batch(train), _batch(test)
    before = tr.evaluate(bv, Ev)
    losses = [tr.step(bt, Et) for _ in range(150)]
    after = tr.evaluate(bv, Ev)
    # the trained network, run on the tensor-core inference path
    from mlff_gb300.student_model import StudentForceField
    inf = StudentForceField(precision="fp16x3").to("cuda")
    inf.load_state_dict(m.state_dict())
    E_inf, _ = inf.energy_and_forces(bv.Z, bv.pos, torch.repeat_interleave(
        torch.arange(test.n_mol, device="cuda"), torch.as_tensor(np.diff(test.mol_ptr), device="cuda")))
    n = np.diff(test.mol_ptr)
    mse_inf = float(np.mean(((E_inf.cpu().numpy() - Ev) / n) ** 2))
    print(f"held-out per-atom energy MSE: untrained {before:.3e}, trained {after:.3e} (fp16x3 {mse_inf:.3e}); "
          f"train loss {losses[0]:.3e} -> {losses[-1]:.3e}")
    assert losses[-1] < 0.1 * losses[0]
    assert after < 0.1 * before
    assert mse_inf < 0.1 * before


def _compare_grads(grads, ref, tol):
    worst = 0.0
    for k, r in ref.items():
        got = grads[k].double().cpu()
        scale = max(float(r.abs().max()), 1e-6)
        err = float((got - r).abs().max()) / scale
        worst = max(worst, err)
        assert err < tol, (k, err)
    return worst


@pytest.mark.parametrize("wname", ["seed", "bias"])
def test_force_loss_grads_vs_oracle(weights_seed0, weights_bias, wname):
    """sum_b w_b dE_b/dtheta + sum_i G_i . dF_i/dtheta from the library
    (reverse pass + its forward-mode derivative along G, float32) against
    float64 double backward through the oracle."""
    from mlff_gb300 import systems
    from mlff_gb300.training import param_grads
    W = weights_seed0 if wname == "seed" else weights_bias
    s = systems.molecule_batch(4, 10, 40, seed=13)
    rng = np.random.default_rng(2)
    w = rng.normal(size=s.n_mol)
    G = (0.2 * rng.normal(size=(s.n_atoms, 3))).astype(np.float32)
    m = _model(W)
    E, grads, F = param_grads(m, _batch(s), torch.tensor(w), forces=True, force_weights=torch.tensor(G))
    pos = s.pos.astype(np.float32).astype(np.float64)
    E0, F0, g0 = painn.param_grads_forces(W, s.Z, pos, s.mol_ptr, w, G.astype(np.float64))
    assert np.abs(E.cpu().numpy() - E0.numpy()).max() <= 2e-5 * s.n_atoms
    # the float pass still returns -sum_b w_b dE_b/dpos
    _, Fa = painn.energy_forces(W, s.Z, pos, s.mol_ptr)
    Fw = Fa.numpy() * np.repeat(w, np.diff(s.mol_ptr))[:, None]
    assert np.abs(F.cpu().numpy() - Fw).max() <= 1e-3 * max(1.0, np.abs(Fw).max())
    assert set(grads) == set(g0)
    worst = _compare_grads(grads, g0, 2e-4)
    # the force term alone (w = 0) against the oracle
    _, gf, _ = param_grads(m, _batch(s), torch.zeros(s.n_mol), force_weights=torch.tensor(G))
    _, _, gf0 = painn.param_grads_forces(W, s.Z, pos, s.mol_ptr, np.zeros(s.n_mol), G.astype(np.float64))
    worst_f = _compare_grads(gf, gf0, 2e-4)
    print(f"worst relative max error: energy+force {worst:.2e}, force term {worst_f:.2e}")


def test_force_loss_grads_vs_reference_training_step(weights_bias):
    """The reference's own training step (golden_train.npz: its model in
    float64, forces with create_graph=True, ForceFieldLoss with energy 1 /
    force 100 / angular 10, loss.backward()) against the library's
    gradients for the loss derivatives of the same predictions."""
    import os
    from conftest import GOLDEN
    from mlff_gb300.engine import make_batch
    from mlff_gb300.training import ForceFieldLoss, param_grads
    g = np.load(os.path.join(GOLDEN, "golden_train.npz"))
    loss = ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=0.1, angular_weight=10.0)
    _, w, G, _ = loss.derivatives(torch.tensor(g["E"]), torch.tensor(g["F"]), torch.tensor(g["E_ref"]),
                               torch.tensor(g["F_ref"]))
    m = _model(weights_bias)
    _, grads, _ = param_grads(m, make_batch(g["Z"], g["pos"], g["mol_ptr"]), w, force_weights=G)
    worst = 0.0
    for k in grads:
        got = grads[k].double().cpu().reshape(-1).numpy()
        ref_norm = float(g[f"grad/{k}/norm"])
        val = g[f"grad/{k}/val"]
        scale = max(np.abs(val).max(), ref_norm / np.sqrt(got.size), 1e-9)
        err = np.abs(got[g[f"grad/{k}/idx"]] - val).max() / scale
        worst = max(worst, err)
        assert err < 2e-4, (k, err)
        assert abs(np.linalg.norm(got) - ref_norm) <= 2e-4 * ref_norm + 1e-9, k
    print(f"worst relative error vs the reference's training step: {worst:.2e}")


def test_force_training_gain(weights_seed0, weights_bias):
    """Force-matching training (ForceFieldTrainer on the force term: the
    parameter gradients are all second-order) on a teacher's float64
    forces: held-out force RMSE and loss drop well below the untrained
    network's, and the trained weights predict better forces on the
    tensor-core inference path too.  (With the reference's energy weight
    the first steps mostly remove the teacher's energy offset; the force
    term alone shows what the second-order gradients buy.)"""
    from mlff_gb300 import systems
    from mlff_gb300.training import ForceFieldLoss, ForceFieldTrainer
    train = systems.molecule_batch(32, 10, 40, seed=41)
    test = systems.molecule_batch(12, 10, 40, seed=42)

    def teacher(s):
        E, F = painn.energy_forces(weights_bias, s.Z, s.pos.astype(np.float32).astype(np.float64), s.mol_ptr)
        return E.numpy(), F.numpy()

    (Et, Ft), (Ev, Fv) = teacher(train), teacher(test)
    m = _model(weights_seed0)
    tr = ForceFieldTrainer(m, ForceFieldLoss(energy_weight=0.0, force_weight=100.0, angular_weight=0.0), lr=2e-3)
    bt, bv = _batch(train), _batch(test)
    before = tr.evaluate(bv, Ev, Fv)
    hist = [tr.step(bt, Et, Ft) for _ in range(60)]
    after = tr.evaluate(bv, Ev, Fv)
    from mlff_gb300.student_model import StudentForceField
    inf = StudentForceField(precision="fp16x3").to("cuda")
    inf.load_state_dict(m.state_dict())
    _, F_inf = inf.energy_and_forces(bv.Z, bv.pos, torch.repeat_interleave(
        torch.arange(test.n_mol, device="cuda"), torch.as_tensor(np.diff(test.mol_ptr), device="cuda")))
    rmse_inf = float(np.sqrt(np.mean((F_inf.cpu().numpy() - Fv) ** 2)))
    print(f"held-out force RMSE: untrained {before['force_rmse']:.3e}, trained {after['force_rmse']:.3e} "
          f"(fp16x3 {rmse_inf:.3e}); total loss {before['total']:.3e} -> {after['total']:.3e}; "
          f"train loss {hist[0]['total']:.3e} -> {hist[-1]['total']:.3e}")
    assert hist[-1]["total"] < 0.3 * hist[0]["total"]
    assert after["force_rmse"] < 0.6 * before["force_rmse"]
    assert rmse_inf < 0.6 * before["force_rmse"]


def test_stress_loss_grads_vs_oracle(weights_bias):
    """Periodic box: energy + force + strain-derivative (stress) loss
    gradients, and the strain term alone, against float64 double backward
    through the oracle."""
    from mlff_gb300 import systems
    from mlff_gb300.engine import make_batch
    from mlff_gb300.training import param_grads
    s = systems.water_box(n_water=60, L=11.5, d_oo=2.2, seed=8)
    pos32 = s.pos.astype(np.float32)
    rng = np.random.default_rng(6)
    w = rng.normal(size=1)
    G = (0.2 * rng.normal(size=(s.n_atoms, 3))).astype(np.float32)
    S = rng.normal(size=(1, 3, 3))
    m = _model(weights_bias)
    b = make_batch(s.Z, pos32, s.mol_ptr, s.box, s.pbc)
    pos = pos32.astype(np.float64)
    _, grads, _ = param_grads(m, b, torch.tensor(w), force_weights=torch.tensor(G), virial_weights=torch.tensor(S))
    _, _, g0 = painn.param_grads_forces(weights_bias, s.Z, pos, s.mol_ptr, w, G.astype(np.float64), box=s.box,
                                        pbc=s.pbc, virial_weights=S)
    worst = _compare_grads(grads, g0, 2e-4)
    _, gs, _ = param_grads(m, b, torch.zeros(1), virial_weights=torch.tensor(S))
    _, _, gs0 = painn.param_grads_forces(weights_bias, s.Z, pos, s.mol_ptr, np.zeros(1), None, box=s.box,
                                         pbc=s.pbc, virial_weights=S)
    worst_s = _compare_grads(gs, gs0, 2e-4)
    print(f"worst relative max error: energy+force+strain {worst:.2e}, strain term {worst_s:.2e}")


def test_force_field_trainer_with_stress(weights_seed0, weights_bias):
    """ForceFieldTrainer on periodic boxes with energy, force and stress
    targets (teacher: float64 oracle with the perturbed weights): the
    stress term is part of the loss and falls with training."""
    from mlff_gb300 import systems
    from mlff_gb300.engine import make_batch
    from mlff_gb300.training import ForceFieldLoss, ForceFieldTrainer
    boxes = [systems.water_box(n_water=50, L=11.5, d_oo=2.2, seed=20 + k) for k in range(4)]
    s = systems.concat(boxes)
    pos32 = s.pos.astype(np.float32)
    E0, F0, V0 = painn.energy_forces(weights_bias, s.Z, pos32.astype(np.float64), s.mol_ptr, box=s.box, pbc=s.pbc,
                                     virial=True)
    vol = np.prod(s.box, axis=1)
    sym = 0.5 * (V0.numpy() + V0.numpy().transpose(0, 2, 1)) / vol[:, None, None]
    S_ref = np.stack([sym[:, 0, 0], sym[:, 1, 1], sym[:, 2, 2], sym[:, 1, 2], sym[:, 0, 2], sym[:, 0, 1]], axis=1)
    m = _model(weights_seed0)
    loss = ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=1000.0, angular_weight=0.0)
    tr = ForceFieldTrainer(m, loss, lr=2e-3)
    b = make_batch(s.Z, pos32, s.mol_ptr, s.box, s.pbc)
    hist = [tr.step(b, E0.numpy(), F0.numpy(), S_ref) for _ in range(25)]
    print(f"stress term {hist[0]['stress']:.3e} -> {hist[-1]['stress']:.3e}; "
          f"total {hist[0]['total']:.3e} -> {hist[-1]['total']:.3e}")
    assert "stress" in hist[0]
    assert hist[-1]["total"] < 0.5 * hist[0]["total"]
    assert hist[-1]["stress"] < hist[0]["stress"]


def test_reference_training_loop_runs_on_the_cuda_gradients(weights_bias):
    """The reference's own training step, unchanged: model in train mode,
    E = model(Z, pos, batch), F = -autograd.grad(E, pos, create_graph=True),
    ForceFieldLoss(E, F) and loss.backward().  The parameters' .grad come
    from the library (energy term: reverse pass; force and angular terms:
    forward mode over it) and match the reference's recorded step
    (golden_train.npz) to float32 accuracy."""
    import os
    from conftest import GOLDEN
    from mlff_gb300.training import ForceFieldLoss
    g = np.load(os.path.join(GOLDEN, "golden_train.npz"))
    m = _model(weights_bias)
    m.train()
    Z = torch.tensor(g["Z"], device="cuda")
    x = torch.tensor(g["pos"], device="cuda", requires_grad=True)
    b = torch.repeat_interleave(torch.arange(len(g["mol_ptr"]) - 1, device="cuda"),
                                torch.as_tensor(np.diff(g["mol_ptr"]), device="cuda"))
    E = m(Z, x, batch=b)
    F = -torch.autograd.grad(E, x, grad_outputs=torch.ones_like(E), create_graph=True)[0]
    loss = ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=0.1, angular_weight=10.0)
    out = loss({"energy": E, "forces": F},
               {"energy": torch.tensor(g["E_ref"], dtype=torch.float32, device="cuda"),
                "forces": torch.tensor(g["F_ref"], dtype=torch.float32, device="cuda")})
    assert abs(float(out["total"].detach()) - float(g["loss"])) <= 1e-4 * abs(float(g["loss"]))
    out["total"].backward()
    worst = 0.0
    for k, p in m.named_parameters():
        got = p.grad.double().cpu().reshape(-1).numpy()
        ref_norm = float(g[f"grad/{k}/norm"])
        val = g[f"grad/{k}/val"]
        scale = max(np.abs(val).max(), ref_norm / np.sqrt(got.size), 1e-9)
        err = np.abs(got[g[f"grad/{k}/idx"]] - val).max() / scale
        worst = max(worst, err)
        assert err < 1e-3, (k, err)
    print(f"reference-style loss.backward(): worst relative error vs the reference's step {worst:.2e}")
    # predict_energy_and_forces in training mode builds the same graph
    m.zero_grad()
    s0 = slice(int(g["mol_ptr"][0]), int(g["mol_ptr"][1]))
    E1, F1 = m.predict_energy_and_forces(Z[s0], torch.tensor(g["pos"][s0], device="cuda"))
    (F1 * F1).sum().backward()
    assert all(p.grad is not None and torch.isfinite(p.grad).all() for p in m.parameters() if p.requires_grad)
    assert float(m.energy_head[0].weight.grad.abs().sum()) > 0
