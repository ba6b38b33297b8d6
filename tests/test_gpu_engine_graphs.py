"""The engine's cached CUDA graphs of repeated call shapes (GPU only).

A call whose shape was seen before replays a captured graph of the whole
step on copies of the inputs; its results must equal an eager call bit for
bit, for changing positions, for structure indices and cells given on the
host, and across an edge-capacity overflow (the graph is dropped, the call
redone eagerly with a larger capacity and captured again).  Host inputs
(pinned host Z and positions, results returned in host memory) give the same
bits as device inputs, through capture, replay and a capacity overflow.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model(weights_bias):
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField()
    m.load_state_dict({k: torch.tensor(v) for k, v in weights_bias.items()})
    return m.cuda()


def _eager(model, Z, P, batch=None, cell=None, pbc=None):
    eng = model.engine()
    bt, _, _ = model._make_batch(Z, P, cell, pbc, batch, need_index=False)
    E, F, _ = eng.energy_forces(bt, model.path, forces=True, graph=False)
    return E, F


def test_graph_replay_equals_eager_batch(model):
    from mlff_gb300 import systems
    s = systems.molecule_batch(12, 10, 60, seed=5)
    Z = torch.as_tensor(s.Z, dtype=torch.int64, device="cuda")
    b = torch.as_tensor(np.repeat(np.arange(s.n_mol), np.diff(s.mol_ptr)))   # host index
    rng = np.random.default_rng(0)
    for it in range(4):   # call 1 captures, calls 2-4 replay
        pos = s.pos + 0.01 * it * rng.standard_normal(s.pos.shape)
        P = torch.as_tensor(pos, dtype=torch.float32, device="cuda")
        E, F = model.energy_and_forces(Z, P, batch=b)
        E0, F0 = _eager(model, Z, P, batch=b)
        assert torch.equal(E, E0) and torch.equal(F, F0)
    assert len(model.engine()._graphs) >= 1


def test_graph_replay_equals_eager_periodic_and_capacity(model):
    from mlff_gb300 import systems
    s = systems.water_box(150, 15.0, 2.5, seed=4)
    Z = torch.as_tensor(s.Z, dtype=torch.int64, device="cuda")
    cell = torch.as_tensor(np.diag(s.box[0]).astype(np.float32))   # host cell
    pbc = torch.ones(3, dtype=torch.bool)
    eng = model.engine()
    for scale in (1.0, 1.0, 1.0, 0.9, 0.9):   # the compressed box needs more edges than captured
        P = torch.as_tensor(s.pos * scale, dtype=torch.float32, device="cuda")
        c = cell * scale
        E, F = model.energy_and_forces(Z, P, cell=c, pbc=pbc)
        E0, F0 = _eager(model, Z, P, cell=c, pbc=pbc)
        assert torch.equal(E, E0) and torch.equal(F, F0)
        assert torch.isfinite(F).all()
    assert eng.status()[0] == 0


def test_host_buffers_equal_device_call(model):
    """energy_and_forces with host Z/positions: first call eager + capture,
    later calls copy straight into the graph's inputs and read results and
    status back behind one synchronisation; a compressed box overflows the
    captured edge capacity on the host path and is redone."""
    from mlff_gb300 import systems
    s = systems.water_box(150, 15.0, 2.5, seed=6)
    Zh = torch.as_tensor(s.Z, dtype=torch.int64).pin_memory()
    Zd = Zh.cuda()
    cell = torch.as_tensor(np.diag(s.box[0]).astype(np.float32))
    pbc = torch.ones(3, dtype=torch.bool)
    for scale in (1.0, 1.0, 1.0, 0.88, 0.88, 0.88):
        Ph = torch.as_tensor(s.pos * scale, dtype=torch.float32).pin_memory()
        E, F = model.energy_and_forces(Zh, Ph, cell=cell * scale, pbc=pbc)
        assert E.device.type == "cpu" and F.device.type == "cpu"
        E0, F0 = _eager(model, Zd, Ph.cuda(), cell=cell * scale, pbc=pbc)
        assert torch.equal(E, E0.cpu()) and torch.equal(F, F0.cpu())
    # a ragged batch with a host structure index, pageable host inputs
    m = systems.molecule_batch(8, 10, 50, seed=9)
    b = torch.as_tensor(np.repeat(np.arange(m.n_mol), np.diff(m.mol_ptr)))
    Z = torch.as_tensor(m.Z, dtype=torch.int64)
    for it in range(3):
        P = torch.as_tensor(m.pos + 0.01 * it, dtype=torch.float32)
        E, F = model.energy_and_forces(Z, P, batch=b)
        E0, F0 = _eager(model, Z.cuda(), P.cuda(), batch=b)
        assert torch.equal(E, E0.cpu()) and torch.equal(F, F0.cpu())


def test_forward_autograd_equals_engine_forces(model):
    """The reference API in inference (eval mode): E = model(Z, pos, batch),
    forces by torch.autograd.grad(E.sum(), pos) through the CUDA adjoint,
    equal to the engine's forces bit for bit; no parameter gradients."""
    from mlff_gb300 import systems
    model.eval()
    s = systems.molecule_batch(5, 10, 40, seed=14)
    Z = torch.as_tensor(s.Z, dtype=torch.int64, device="cuda")
    x = torch.as_tensor(s.pos, dtype=torch.float32, device="cuda").requires_grad_(True)
    b = torch.as_tensor(np.repeat(np.arange(s.n_mol), np.diff(s.mol_ptr)))
    E = model(Z, x, batch=b)
    assert E.shape == (s.n_mol,)
    (gx,) = torch.autograd.grad(E.sum(), x)
    E0, F0 = _eager(model, Z, x.detach(), batch=b)
    assert torch.equal(E.detach().double(), E0.to(E.dtype).double())
    assert torch.equal(-gx, F0)
    assert all(p.grad is None for p in model.parameters())
