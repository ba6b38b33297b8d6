"""The oracle (CPU restatement) against golden vectors written by the
reference implementation itself (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, case_names
from oracle import nbr, painn

CASES = ["batch6", "cutoff_edge", "methane", "molecule60", "water"]


def test_fixture_case_list(golden_cases):
    assert case_names(golden_cases) == CASES


@pytest.mark.parametrize("name", CASES)
def test_edge_list_bit_exact(golden_cases, name):
    """Same edges, same order as radius_graph_native (student_model.py:63-109)."""
    g = golden_cases
    src, dst, sh = nbr.radius_graph(g[f"{name}/pos"], g[f"{name}/mol_ptr"])
    ei = g[f"{name}/edge_index"]
    np.testing.assert_array_equal(src, ei[0])
    np.testing.assert_array_equal(dst, ei[1])
    assert not sh.any()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("tag", ["seed", "bias"])
def test_energy_forces_fp64(golden_cases, weights_seed0, weights_bias, name, tag):
    g = golden_cases
    W = weights_seed0 if tag == "seed" else weights_bias
    E, F = painn.energy_forces(W, g[f"{name}/Z"], g[f"{name}/pos"].astype(np.float64),
                               g[f"{name}/mol_ptr"])
    np.testing.assert_allclose(E.numpy(), g[f"{name}/{tag}/E64"], rtol=0, atol=1e-10)
    if name == "methane":
        # The carbon's vector feature is exactly zero by symmetry, where
        # |v| (PaiNNUpdate, student_model.py:437) has no derivative: forces
        # there depend on rounding noise even between the reference's own
        # float32 and float64 runs, so only the energy is pinned.
        return
    np.testing.assert_allclose(F.numpy(), g[f"{name}/{tag}/F64"], rtol=0, atol=1e-9)


def test_norm_recipe_matches_torch_norm():
    """sqrtf(fmaf(z,z,fmaf(y,y,x*x))) equals the reference's torch.norm."""
    import os
    from conftest import GOLDEN
    gn = np.load(os.path.join(GOLDEN, "golden_norm.npz"))
    d = nbr.pair_distance(gn["vec"][:5000])
    np.testing.assert_array_equal(d, gn["dist"][:5000])
    np.testing.assert_array_equal(d <= 5.0, gn["keep"][:5000])


def test_norm_recipe_matches_local_torch():
    """Re-check the recipe against this machine's torch.norm (the GPU host
    runs a different CPU architecture)."""
    import torch
    rng = np.random.default_rng(5)
    v = (rng.standard_normal((3000, 3)) * 3).astype(np.float32)
    ref = torch.norm(torch.tensor(v), dim=1).numpy()
    np.testing.assert_array_equal(nbr.pair_distance(v), ref)


def test_periodic_min_image_antisymmetric():
    """d_ij == d_ji bit for bit under the minimum-image rule, and every
    periodic edge appears in both directions with opposite image shifts."""
    from mlff_gb300 import systems
    s = systems.water_box(n_water=50, L=11.0, seed=3)
    src, dst, sh = nbr.radius_graph(s.pos.astype(np.float32), s.mol_ptr, 5.0, s.box, s.pbc)
    fwd = {(int(a), int(b)): tuple(k) for a, b, k in zip(src, dst, sh)}
    for (a, b), k in fwd.items():
        assert fwd[(b, a)] == tuple(-x for x in k)


def test_cell_list_matches_brute_force():
    from mlff_gb300 import systems
    s = systems.large_box(n_atoms=5000, seed=11)
    pos = s.pos.astype(np.float32)
    a = nbr.radius_graph(pos, s.mol_ptr, 5.0, s.box, s.pbc)  # cells (n > 4000)
    lib = nbr._load()
    cap = 80 * len(pos)
    src = np.empty(cap, np.int64); dst = np.empty(cap, np.int64); shf = np.empty((cap, 3), np.int32)
    box = s.box.astype(np.float32); pbc = np.ones(1, np.uint8); mp = s.mol_ptr.astype(np.int64)
    e = lib.oracle_radius_graph(pos.ctypes.data, len(pos), mp.ctypes.data, 1, box.ctypes.data,
                                pbc.ctypes.data, 5.0, src.ctypes.data, dst.ctypes.data,
                                shf.ctypes.data, cap)
    np.testing.assert_array_equal(a[0], src[:e])
    np.testing.assert_array_equal(a[1], dst[:e])
    np.testing.assert_array_equal(a[2], shf[:e])


def test_virial_matches_finite_difference():
    """Strain derivative of the oracle energy vs central differences."""
    import torch
    from mlff_gb300 import systems
    W = dict(np.load(__import__("os").path.join(__import__("conftest").GOLDEN, "weights_seed0.npz")))
    s = systems.water_box(n_water=40, L=10.5, d_oo=2.2, seed=4)
    E, F, V = painn.energy_forces(W, s.Z, s.pos, s.mol_ptr, box=s.box, pbc=s.pbc, virial=True)
    h = 1e-5
    for (a, b) in [(0, 0), (1, 2), (2, 1)]:
        vals = []
        for sign in (1, -1):
            eps = np.eye(3)
            eps[a, b] += sign * h
            pos = s.pos @ eps
            box = s.box * np.diag(eps)[None, :] if a == b else s.box
            if a != b:
                # off-diagonal strain of an orthorhombic box: evaluate with the
                # strained shift vectors through the autograd path instead
                continue
            Ep, _ = painn.energy_forces(W, s.Z, pos, s.mol_ptr, box=box, pbc=s.pbc)
            vals.append(float(Ep[0]))
        if vals:
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - float(V[0, a, b])) < 1e-5 * max(1.0, abs(fd))


def test_oracle_param_grads_match_finite_differences(weights_bias):
    """The oracle's parameter gradients (autograd) against central
    differences of its float64 energy, a few entries of every kind of
    tensor, on a small molecule."""
    from mlff_gb300 import systems
    s = systems.lattice_molecule(12, seed=5)
    pos = s.pos.astype(np.float32).astype(np.float64)
    w = np.array([0.7])
    _, g = painn.param_grads(weights_bias, s.Z, pos, s.mol_ptr, w)
    rng = np.random.default_rng(3)
    for key in ["embedding.weight", "interactions.0.message.rbf_to_scalar.0.weight",
                "interactions.1.message.rbf_to_scalar.2.bias", "interactions.2.update.mixing_matrix",
                "interactions.0.update.update_mlp.0.weight", "energy_head.2.weight", "energy_head.4.bias"]:
        shape = weights_bias[key].shape
        for _ in range(2):
            idx = tuple(int(rng.integers(0, n)) for n in shape)
            if key == "embedding.weight":
                idx = (int(s.Z[0]),) + idx[1:]
            h = 1e-5
            vals = []
            for sgn in (1, -1):
                W = {k: v.copy() for k, v in weights_bias.items()}
                W[key] = W[key].astype(np.float64)
                W[key][idx] += sgn * h
                E, _ = painn.energy_forces(W, s.Z, pos, s.mol_ptr)
                vals.append(float(E[0]) * w[0])
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - float(g[key][idx])) <= 1e-6 + 1e-5 * abs(fd), (key, idx, fd, float(g[key][idx]))


def test_force_loss_grads_match_reference_training_step(weights_bias):
    """One training step of the reference (its model in float64, forces
    with create_graph=True, its ForceFieldLoss with the train_student.yaml
    weights, loss.backward()) recorded in golden_train.npz, against the
    restated loss (mlff_gb300.training.ForceFieldLoss: values and the
    derivatives dL/dE, dL/dF) and the oracle's second-order parameter
    gradients for those derivatives."""
    import torch
    from mlff_gb300.training import ForceFieldLoss
    g = np.load(os.path.join(GOLDEN, "golden_train.npz"))
    E, F = torch.tensor(g["E"]), torch.tensor(g["F"])
    loss = ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=0.1, angular_weight=10.0)
    out, w, G, _ = loss.derivatives(E, F, torch.tensor(g["E_ref"]), torch.tensor(g["F_ref"]))
    for key in ["loss", "loss_energy", "loss_force", "loss_angular"]:
        name = "total" if key == "loss" else key.split("_", 1)[1]
        assert abs(float(out[name].detach()) - float(g[key])) <= 1e-12 * max(1.0, abs(float(g[key]))), key
    E0, F0, grads = painn.param_grads_forces(weights_bias, g["Z"], g["pos"].astype(np.float64), g["mol_ptr"],
                                             w.numpy(), G.double().numpy())
    assert np.abs(E0.numpy() - g["E"]).max() < 1e-10
    assert np.abs(F0.numpy() - g["F"]).max() < 1e-10
    names = sorted(k.split("/")[1] for k in g.files if k.startswith("grad/") and k.endswith("/norm"))
    assert set(names) == set(grads), set(names) ^ set(grads)
    for k in names:
        ref_norm = float(g[f"grad/{k}/norm"])
        got = grads[k].reshape(-1).numpy()
        # G is rounded to float32 (the library's input type): relative 1e-6
        assert abs(np.linalg.norm(got) - ref_norm) <= 1e-6 * ref_norm + 1e-12, k
        val = g[f"grad/{k}/val"]
        err = np.abs(got[g[f"grad/{k}/idx"]] - val).max()
        assert err <= 1e-6 * max(np.abs(val).max(), ref_norm / np.sqrt(got.size)) + 1e-12, (k, err)


def test_oracle_strain_second_order_matches_finite_differences(weights_bias):
    """The oracle's stress-loss parameter gradients sum_ab S_ab dW_ab/dtheta
    (W = dE/d(strain) taken with create_graph=True) against central
    differences of S : W over a few parameters, on a small periodic box."""
    from mlff_gb300 import systems
    s = systems.water_box(n_water=40, L=11.0, d_oo=2.2, seed=3)
    pos = s.pos.astype(np.float32).astype(np.float64)
    S = np.random.default_rng(4).normal(size=(1, 3, 3))
    _, _, g = painn.param_grads_forces(weights_bias, s.Z, pos, s.mol_ptr, np.zeros(1), None, box=s.box,
                                       pbc=s.pbc, virial_weights=S)
    rng = np.random.default_rng(5)
    for key in ["interactions.0.message.rbf_to_scalar.0.weight", "interactions.2.update.update_mlp.2.bias",
                "energy_head.0.weight"]:
        idx = tuple(int(rng.integers(0, n)) for n in weights_bias[key].shape)
        h = 1e-5
        vals = []
        for sgn in (1, -1):
            W = {k: v.copy() for k, v in weights_bias.items()}
            W[key] = W[key].astype(np.float64)
            W[key][idx] += sgn * h
            _, _, V = painn.energy_forces(W, s.Z, pos, s.mol_ptr, box=s.box, pbc=s.pbc, virial=True)
            vals.append(float((V.numpy() * S).sum()))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - float(g[key][idx])) <= 1e-6 + 1e-5 * abs(fd), (key, idx, fd, float(g[key][idx]))


@pytest.mark.parametrize("kind", ["mae", "huber"])
def test_force_field_loss_components_match_reference(kind):
    """The restated ForceFieldLoss with mae / huber components (delta 0.2)
    against the reference's own loss on the same predictions: value and the
    derivatives in the energies and forces (golden_train.npz)."""
    import torch
    from mlff_gb300.training import ForceFieldLoss
    g = np.load(os.path.join(GOLDEN, "golden_train.npz"))
    loss = ForceFieldLoss(energy_weight=1.0, force_weight=100.0, stress_weight=0.1, angular_weight=10.0,
                          energy_loss_type=kind, force_loss_type=kind, huber_delta=0.2)
    out, w, G, _ = loss.derivatives(torch.tensor(g["E"]), torch.tensor(g["F"]), torch.tensor(g["E_ref"]),
                                    torch.tensor(g["F_ref"]))
    assert abs(float(out["total"].detach()) - float(g[f"{kind}/loss"])) <= 1e-12 * abs(float(g[f"{kind}/loss"]))
    np.testing.assert_allclose(w.numpy(), g[f"{kind}/dE"], rtol=1e-12, atol=1e-15)
    # G is returned in float32 (the library's input type)
    np.testing.assert_allclose(G.numpy(), g[f"{kind}/dF"], rtol=1e-6, atol=1e-9)


def test_oracle_edge_chunks_equal_single_pass(weights_bias):
    """The oracle's checkpointed edge chunks (used for the benchmark-size
    parity tests) give the single-pass result up to float64 rounding."""
    from mlff_gb300 import systems
    s = systems.water_box(n_water=40, L=10.5, d_oo=2.2, seed=9)
    p = s.pos.astype(np.float32).astype(np.float64)
    E1, F1, V1 = painn.energy_forces(weights_bias, s.Z, p, s.mol_ptr, box=s.box, pbc=s.pbc, virial=True)
    E2, F2, V2 = painn.energy_forces(weights_bias, s.Z, p, s.mol_ptr, box=s.box, pbc=s.pbc, virial=True,
                                     edge_chunk=1000)
    assert abs(float(E1[0] - E2[0])) < 1e-10
    assert float((F1 - F2).abs().max()) < 1e-11
    assert float((V1 - V2).abs().max()) < 1e-10


def _golden_metrics():
    return np.load(os.path.join(GOLDEN, "golden_metrics.npz"))


def test_energy_metrics_oracle_pinned_to_reference():
    """oracle/energy_metrics.py against the reference's own energy_metrics
    outputs on seeded traces (golden_metrics.npz, written by make_golden.py)."""
    from oracle import energy_metrics
    g = _golden_metrics()
    for i in range(4):
        pre = f"e{i}/"
        t, k, p = g[pre + "time"], g[pre + "kinetic"], g[pre + "potential"]
        s = energy_metrics.stats(k + p, k, p, float(t[1] - t[0]))
        want = {2: "drift_relative", 3: "drift_max_deviation", 5: "fluct/std", 6: "fluct/range",
                7: "fluct/mean_abs_dev", 8: "conservation_ratio", 9: "kp/ke_mean", 10: "kp/ke_std",
                11: "kp/pe_mean", 12: "kp/pe_std", 13: "kp/ke_pe_correlation", 14: "kp/energy_partition_ratio",
                15: "trd/drift_rate", 16: "trd/r_squared", 17: "trd/drift_rate_std"}
        for j, key in want.items():
            np.testing.assert_allclose(s[j], g[pre + key], rtol=1e-9, atol=1e-12, err_msg=pre + key)
        np.testing.assert_allclose(s[1] - s[0], g[pre + "drift_absolute"], rtol=1e-9, atol=1e-12)


def test_force_metrics_oracle_pinned_to_reference():
    from oracle import force_metrics
    g = _golden_metrics()
    for i in range(3):
        pre = f"f{i}/"
        m = force_metrics.metrics(g[pre + "pred"], g[pre + "ref"])
        for key, v in m.items():
            np.testing.assert_allclose(v, g[pre + key], rtol=1e-9, atol=1e-12, err_msg=pre + key)


def test_oracle_vec_langevin_thermostat_and_fixed_centre():
    """The float64 Vanden-Eijnden-Ciccotti restatement on free particles:
    centre of mass fixed, kinetic temperature at T over 3n - 3 degrees of
    freedom."""
    from oracle.md import langevin_vec
    n = 200
    rng = np.random.default_rng(5)
    pos = rng.uniform(0, 50, (n, 3))
    masses = rng.choice([1.008, 12.011, 15.999], n)
    kT = 8.617333262e-5 * 300.0
    free = lambda r: (np.zeros(1), np.zeros_like(r))
    r, v, _, _, ek = langevin_vec(pos, np.zeros((n, 3)), masses, free, 0.05, 0.5, kT, 3, 0, 3000, np.array([0, n]))
    com = lambda x: (masses[:, None] * x).sum(0) / masses.sum()
    assert np.abs(com(r) - com(pos)).max() < 1e-9
    T = ek[1000:, 0].mean() / (0.5 * (3 * n - 3) * 8.617333262e-5)
    assert abs(T / 300.0 - 1.0) < 0.03
