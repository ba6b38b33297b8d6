"""Generate golden vectors from the reference implementation itself.

Run where the reference source tree is available (it is not needed at test
time):

    python tests/golden/make_golden.py /path/to/MLFF-Distiller

It imports the reference StudentForceField by file path
(src/mlff_distiller/models/student_model.py; the package __init__ needs
modules that are not in the reference tree), builds it right after
torch.manual_seed(0), and records energies, forces and edge lists for small
seeded inputs in float32 (the reference's own dtype) and float64
(model.double()).  Outputs go next to this script:

* weights_seed0.npz       -- the seed-0 state_dict (reference key names)
* bias_perturbation.npz   -- seeded non-zero biases (trained-like weights)
* golden_cases.npz        -- per case: Z, pos, mol_ptr, edge_index, E/F in
                             float32 and float64, for seed and biased weights
* golden_norm.npz         -- float32 vectors with |d| near 5 A and the
                             reference's torch.norm decision |d| <= 5
* golden_train.npz        -- one training step's parameter gradients: the
                             reference model (biased weights, float64) with
                             forces taken with create_graph=True, the
                             reference's ForceFieldLoss (training/losses.py,
                             configs/train_student.yaml weights) and
                             loss.backward(); per tensor the gradient's norm
                             and its values at seeded sample indices; and the
                             loss with mae / huber components: its value and
                             derivatives in the predicted energies and forces

* golden_metrics.npz      -- the reference's own energy-conservation and
                             force-accuracy metrics (testing/energy_metrics.py,
                             testing/force_metrics.py, pure numpy) on seeded
                             energy traces and force arrays: inputs and
                             every returned value

``--train-only`` rewrites golden_train.npz alone, ``--metrics-only``
golden_metrics.npz alone.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "mlff-distiller_gb300"))

from mlff_gb300 import systems  # noqa: E402


def load_reference(ref_root: str):
    for name in ["mlff_distiller", "mlff_distiller.models"]:
        if name not in sys.modules:
            m = types.ModuleType(name)
            m.__path__ = []
            sys.modules[name] = m
    path = os.path.join(ref_root, "src", "mlff_distiller", "models", "student_model.py")
    spec = importlib.util.spec_from_file_location("mlff_distiller.models.student_model", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_reference_losses(ref_root: str):
    path = os.path.join(ref_root, "src", "mlff_distiller", "training", "losses.py")
    spec = importlib.util.spec_from_file_location("mlff_distiller_training_losses", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


TRAIN_SAMPLES = 64   # sampled gradient entries per tensor


def sample_indices(name: str, numel: int) -> np.ndarray:
    """Seeded flat indices of the gradient entries recorded for one tensor."""
    seed = sum(ord(c) * (i + 1) for i, c in enumerate(name))
    k = min(TRAIN_SAMPLES, numel)
    return np.sort(np.random.default_rng(seed).choice(numel, size=k, replace=False))


def make_train_golden(sm, ref_root: str, sd, pert):
    losses = load_reference_losses(ref_root)
    model = sm.StudentForceField(use_torch_cluster=False)
    model.load_state_dict({k: torch.tensor(sd[k] + pert[k]) if k in pert else torch.tensor(sd[k]) for k in sd})
    model = model.double()
    model.train()
    sysm = systems.molecule_batch(3, 12, 30, seed=31)
    batch = np.repeat(np.arange(sysm.n_mol), np.diff(sysm.mol_ptr))
    pos32 = sysm.pos.astype(np.float32)
    x = torch.tensor(pos32.astype(np.float64)).requires_grad_(True)
    E = model(torch.tensor(sysm.Z, dtype=torch.long), x, batch=torch.tensor(batch, dtype=torch.long))
    F = -torch.autograd.grad(E, x, grad_outputs=torch.ones_like(E), create_graph=True)[0]
    g = np.random.default_rng(77)
    E_ref = E.detach().numpy() + g.normal(0.0, 0.5, size=E.shape)
    F_ref = F.detach().numpy() + g.normal(0.0, 0.3, size=F.shape)
    loss_fn = losses.ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=0.1, angular_weight=10.0)
    out = loss_fn({"energy": E, "forces": F}, {"energy": torch.tensor(E_ref), "forces": torch.tensor(F_ref)})
    out["total"].backward()
    rec = {"Z": sysm.Z, "pos": pos32, "mol_ptr": sysm.mol_ptr, "E_ref": E_ref, "F_ref": F_ref,
           "E": E.detach().numpy(), "F": F.detach().numpy(), "loss": np.float64(out["total"].item()),
           "loss_energy": np.float64(out["energy"].item()), "loss_force": np.float64(out["force"].item()),
           "loss_angular": np.float64(out["angular"].item())}
    # the loss alone for other component types: values and derivatives in E and F
    for kind in ("mae", "huber"):
        Ed = E.detach().clone().requires_grad_(True)
        Fd = F.detach().clone().requires_grad_(True)
        lf = losses.ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=0.1, angular_weight=10.0,
                                   energy_loss_type=kind, force_loss_type=kind, huber_delta=0.2)
        o = lf({"energy": Ed, "forces": Fd}, {"energy": torch.tensor(E_ref), "forces": torch.tensor(F_ref)})
        gE, gF = torch.autograd.grad(o["total"], [Ed, Fd])
        rec[f"{kind}/loss"] = np.float64(o["total"].item())
        rec[f"{kind}/dE"] = gE.numpy()
        rec[f"{kind}/dF"] = gF.numpy()
    for name, prm in model.named_parameters():
        gr = torch.zeros_like(prm) if prm.grad is None else prm.grad
        flat = gr.detach().reshape(-1).numpy()
        rec[f"grad/{name}/norm"] = np.float64(np.linalg.norm(flat))
        rec[f"grad/{name}/idx"] = sample_indices(name, flat.size)
        rec[f"grad/{name}/val"] = flat[rec[f"grad/{name}/idx"]]
    np.savez_compressed(os.path.join(HERE, "golden_train.npz"), **rec)


def ref_eval(model, Z, pos, batch=None, dtype=torch.float32):
    m = model.to(dtype)
    x = torch.tensor(pos, dtype=dtype).requires_grad_(True)
    Zt = torch.tensor(Z, dtype=torch.long)
    bt = None if batch is None else torch.tensor(batch, dtype=torch.long)
    E = m(Zt, x, batch=bt)
    F = -torch.autograd.grad(E, x, grad_outputs=torch.ones_like(E))[0]
    return np.atleast_1d(E.detach().numpy()).astype(np.float64), F.detach().numpy().astype(np.float64)


def main(ref_root: str, train_only: bool = False):
    sm = load_reference(ref_root)
    if train_only:
        sd = dict(np.load(os.path.join(HERE, "weights_seed0.npz")))
        pert = dict(np.load(os.path.join(HERE, "bias_perturbation.npz")))
        make_train_golden(sm, ref_root, sd, pert)
        print("wrote golden_train.npz")
        return
    torch.manual_seed(0)
    model = sm.StudentForceField(use_torch_cluster=False)
    model.eval()
    sd = {k: v.detach().numpy().copy() for k, v in model.state_dict().items()}
    np.savez_compressed(os.path.join(HERE, "weights_seed0.npz"), **sd)

    rng = np.random.default_rng(1234)
    pert = {k: (0.05 * rng.standard_normal(v.shape)).astype(np.float32)
            for k, v in sd.items() if k.endswith(".bias")}
    np.savez_compressed(os.path.join(HERE, "bias_perturbation.npz"), **pert)
    biased = sm.StudentForceField(use_torch_cluster=False)
    biased.load_state_dict({k: torch.tensor(sd[k] + pert[k]) if k in pert else torch.tensor(sd[k])
                            for k in sd})
    biased.eval()

    cases = {}

    def add_case(name, sysm: systems.System):
        pos32 = sysm.pos.astype(np.float32)
        batch = np.repeat(np.arange(sysm.n_mol), np.diff(sysm.mol_ptr))
        bt = torch.tensor(batch, dtype=torch.long) if sysm.n_mol > 1 else None
        ei = sm.radius_graph_native(torch.tensor(pos32), 5.0, bt, loop=False).numpy()
        cases[f"{name}/Z"] = sysm.Z
        cases[f"{name}/pos"] = pos32
        cases[f"{name}/mol_ptr"] = sysm.mol_ptr
        cases[f"{name}/edge_index"] = ei
        b = batch if sysm.n_mol > 1 else None
        for tag, mdl in (("seed", model), ("bias", biased)):
            E32, F32 = ref_eval(mdl, sysm.Z, pos32, b, torch.float32)
            E64, F64 = ref_eval(mdl, sysm.Z, pos32.astype(np.float64), b, torch.float64)
            mdl.float()
            cases[f"{name}/{tag}/E32"] = E32
            cases[f"{name}/{tag}/F32"] = F32
            cases[f"{name}/{tag}/E64"] = E64
            cases[f"{name}/{tag}/F64"] = F64

    add_case("molecule60", systems.lattice_molecule(60, seed=0))
    add_case("batch6", systems.molecule_batch(6, 10, 40, seed=7))
    water = systems.System(np.array([8, 1, 1]), np.array([[0.0, 0, 0], [0.96, 0, 0], [-0.24, 0.93, 0]]),
                           np.array([0, 3]), np.zeros((1, 3)), np.zeros(1, bool), "water")
    methane = systems.System(np.array([6, 1, 1, 1, 1]),
                             np.array([[0.0, 0, 0], [0.63, 0.63, 0.63], [-0.63, -0.63, 0.63],
                                       [-0.63, 0.63, -0.63], [0.63, -0.63, -0.63]]),
                             np.array([0, 5]), np.zeros((1, 3)), np.zeros(1, bool), "methane")
    add_case("water", water)
    add_case("methane", methane)
    # a pair at exactly 5.0 A (kept by <=, zero cutoff weight), an isolated
    # atom, and a pair just inside the cutoff
    edge = systems.System(np.array([6, 8, 1, 7]),
                          np.array([[0.0, 0, 0], [3.0, 4.0, 0], [40.0, 0, 0], [0.0, 0, 4.999]]),
                          np.array([0, 4]), np.zeros((1, 3)), np.zeros(1, bool), "cutoff_edge")
    add_case("cutoff_edge", edge)
    np.savez_compressed(os.path.join(HERE, "golden_cases.npz"), **cases)

    # edge decision: vectors whose float32 norm straddles the cutoff
    g = np.random.default_rng(99)
    dirs = g.standard_normal((40_000, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    radii = 5.0 + g.uniform(-4e-6, 4e-6, size=(40_000, 1))
    vec = (dirs * radii).astype(np.float32)
    dist = torch.norm(torch.tensor(vec), dim=1).numpy()
    np.savez_compressed(os.path.join(HERE, "golden_norm.npz"), vec=vec, dist=dist,
                        keep=(dist <= 5.0))
    make_train_golden(sm, ref_root, sd, pert)
    make_metrics_golden(ref_root)
    print("wrote", sorted(os.listdir(HERE)))


def load_reference_testing(ref_root: str, name: str):
    """testing/<name>.py by file path (numpy only; the package __init__
    pulls in ASE, which is not needed by these modules)."""
    path = os.path.join(ref_root, "src", "mlff_distiller", "testing", f"{name}.py")
    spec = importlib.util.spec_from_file_location(f"mlff_distiller_testing_{name}", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def metric_traces():
    """Seeded energy traces (kinetic, potential; 0.5 fs steps in ps): an
    oscillating conserved trajectory, one with a linear drift, one noisy,
    one short."""
    g = np.random.default_rng(11)
    out = []
    for n, drift, noise in ((400, 0.0, 1e-4), (400, 2e-3, 1e-4), (250, -5e-4, 3e-3), (12, 0.0, 1e-3)):
        t = np.arange(n) * 5e-4
        k = 1.2 + 0.3 * np.sin(2 * np.pi * t / 0.02) + noise * g.standard_normal(n)
        p = -40.0 - 0.3 * np.sin(2 * np.pi * t / 0.02) + drift * np.arange(n) + noise * g.standard_normal(n)
        out.append((t, k, p))
    return out


def metric_forces():
    """Seeded (predicted, reference) force arrays: [n_atoms, 3] with noise,
    [frames, atoms, 3], and one with zero and near-zero vectors."""
    g = np.random.default_rng(12)
    ref = g.standard_normal((300, 3)) * 1.5
    a = (ref + 0.05 * g.standard_normal(ref.shape), ref)
    ref3 = g.standard_normal((5, 40, 3))
    b = (ref3 + 0.2 * g.standard_normal(ref3.shape), ref3)
    ref_z = g.standard_normal((60, 3))
    pred_z = ref_z + 0.1 * g.standard_normal(ref_z.shape)
    ref_z[:5] = 0.0
    pred_z[5:8] = 1e-8
    pred_z[8] = -ref_z[8]
    c = (pred_z, ref_z)
    return [a, b, c]


def make_metrics_golden(ref_root: str):
    em = load_reference_testing(ref_root, "energy_metrics")
    fm = load_reference_testing(ref_root, "force_metrics")
    out = {}
    for i, (t, k, p) in enumerate(metric_traces()):
        e = k + p
        pre = f"e{i}/"
        out[pre + "time"], out[pre + "kinetic"], out[pre + "potential"] = t, k, p
        out[pre + "drift_relative"] = em.compute_energy_drift(e, "relative")
        out[pre + "drift_absolute"] = em.compute_energy_drift(e, "absolute")
        out[pre + "drift_max_deviation"] = em.compute_energy_drift(e, "max_deviation")
        out[pre + "conservation_ratio"] = em.compute_energy_conservation_ratio(e)
        out[pre + "conservation_ratio_w10"] = em.compute_energy_conservation_ratio(e, window=10)
        for key, v in em.compute_energy_fluctuations(e).items():
            out[pre + "fluct/" + key] = v
        for key, v in em.compute_kinetic_potential_stability(k, p).items():
            out[pre + "kp/" + key] = v
        for key, v in em.compute_time_resolved_drift(t, e).items():
            out[pre + "trd/" + key] = v
        for key, v in em.compute_time_resolved_drift(t, e, method="cumulative").items():
            out[pre + "trc/" + key] = v
        a = em.assess_energy_conservation({"time": list(t), "total_energy": list(e), "kinetic_energy": list(k),
                                           "potential_energy": list(p)}, verbose=False)
        out[pre + "assess/passed"] = a["passed"]
        for key in ("energy_drift_pct", "energy_drift_max_pct", "conservation_ratio"):
            out[pre + "assess/" + key] = a[key]
        for key, v in a["criteria"].items():
            out[pre + "assess/criteria/" + key] = v
    for i, (pred, ref) in enumerate(metric_forces()):
        pre = f"f{i}/"
        out[pre + "pred"], out[pre + "ref"] = pred, ref
        out[pre + "rmse"] = fm.compute_force_rmse(pred, ref)
        out[pre + "rmse_comp"] = fm.compute_force_rmse(pred, ref, per_component=True)
        out[pre + "mae"] = fm.compute_force_mae(pred, ref)
        out[pre + "mae_comp"] = fm.compute_force_mae(pred, ref, per_component=True)
        for key, v in fm.compute_force_magnitude_error(pred, ref).items():
            out[pre + "mag/" + key] = v
        out[pre + "angular_median"] = fm.compute_angular_error(pred, ref)
        out[pre + "angular_dist"] = fm.compute_angular_error(pred, ref, return_distribution=True)
        for key, v in fm.compute_force_correlation(pred, ref).items():
            out[pre + "corr/" + key] = v
        if pred.ndim == 2:
            for key, v in fm.compute_per_atom_force_errors(pred, ref).items():
                out[pre + "atom/" + key] = v
        a = fm.assess_force_accuracy(pred, ref, verbose=False)
        out[pre + "assess/passed"] = a["passed"]
        for key, v in a["angular_percentiles"].items():
            out[pre + "assess/pct/" + key] = v
        for key, v in a["criteria"].items():
            out[pre + "assess/criteria/" + key] = v
    np.savez_compressed(os.path.join(HERE, "golden_metrics.npz"), **{k: np.asarray(v) for k, v in out.items()})
    print("wrote golden_metrics.npz with", len(out), "arrays")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("MLFF_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference checkout> [--train-only] "
                 "(or set MLFF_REFERENCE_ROOT)")
    if "--metrics-only" in sys.argv:
        make_metrics_golden(root)
    else:
        main(root, train_only="--train-only" in sys.argv)
