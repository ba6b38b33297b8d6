"""Training path (GPU only): parameter gradients of sum_b w_b E_b from the
CUDA reverse pass against float64 autograd through the oracle, determinism,
and what training buys: the network fitted to a teacher's energies on
training molecules predicts held-out molecules far better than the same
network before training.
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
    """Repeated calls agree to rounding (the plain path scatter-adds with
    float atomics, as index_add_ does on a GPU)."""
    from mlff_gb300 import systems
    from mlff_gb300.training import param_grads
    s = systems.molecule_batch(6, 10, 60, seed=12)
    m = _model(weights_bias)
    w = torch.linspace(-1, 1, s.n_mol, dtype=torch.float64)
    _, g1, _ = param_grads(m, _batch(s), w)
    _, g2, _ = param_grads(m, _batch(s), w)
    for k in g1:
        scale = float(g1[k].abs().max()) + 1e-12
        assert float((g1[k] - g2[k]).abs().max()) <= 1e-5 * scale, k


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
