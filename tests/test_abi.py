"""The C-ABI library builds, loads and exports every symbol the header
declares (no compute calls: runs without a GPU)."""
import os
import re

import pytest

from conftest import ROOT


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "mlff_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mlff_[a-z_]+)\s*\(", txt)))


def test_header_lists_all_bound_symbols():
    from mlff_gb300 import _lib
    assert sorted(_lib.EXPORTS) == header_symbols()


def test_library_loads_and_exports():
    from mlff_gb300 import _build, _lib
    _build.build()
    lib = _lib.load()
    for name in header_symbols():
        assert hasattr(lib, name), name
    assert lib.mlff_version() == 100


def test_size_queries_without_gpu():
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    d = dims_of(128, 20, 3, 119, 5.0)
    n = lib.mlff_packed_weights_size(ctypes.byref(d))
    # 429,596 parameters plus transposed copies and split-BF16 tiles
    assert n > 4 * 429_596
    ws_plain = lib.mlff_workspace_size(ctypes.byref(d), 1000, 4, 64_000, _lib.PATH_PLAIN_FP32)
    ws_tuned = lib.mlff_workspace_size(ctypes.byref(d), 1000, 4, 64_000, _lib.PATH_TUNED_TC)
    assert ws_plain > ws_tuned > 0
    ws_train = lib.mlff_workspace_size(ctypes.byref(d), 1000, 4, 64_000, _lib.PATH_TRAIN)
    ws_force = lib.mlff_workspace_size(ctypes.byref(d), 1000, 4, 64_000, _lib.PATH_TRAIN_FORCES)
    # the tangent pass keeps (value, tangent) pairs: about twice the training workspace
    assert 1.8 * ws_train < ws_force < 2.1 * ws_train


def test_unsupported_shape_is_reported():
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    d = dims_of(64, 20, 3, 119, 5.0)
    assert lib.mlff_packed_weights_size(ctypes.byref(d)) == 0
    assert b"hidden" in lib.mlff_last_error_string()


def test_invalid_arguments_rejected_on_host():
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    d = dims_of(128, 20, 3, 119, 5.0)
    s = _lib.System()
    s.n_atoms = 0
    s.n_mol = 1
    out = _lib.Outputs()
    r = lib.mlff_energy_forces(ctypes.byref(d), None, ctypes.byref(s), 0, 1, ctypes.byref(out), None, 0, None)
    assert r == _lib.ERR_INVALID
    assert b"empty" in lib.mlff_last_error_string()


def test_seeded_init_matches_reference_weights(weights_seed0):
    import numpy as np
    import torch
    from mlff_gb300.student_model import StudentForceField
    torch.manual_seed(0)
    m = StudentForceField()
    sd = m.state_dict()
    assert set(sd) == set(weights_seed0)
    for k, v in weights_seed0.items():
        np.testing.assert_array_equal(sd[k].numpy(), v)


def test_checkpoint_roundtrip(tmp_path, weights_seed0):
    import numpy as np
    import torch
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField()
    m.load_state_dict({k: torch.tensor(v) for k, v in weights_seed0.items()})
    p = tmp_path / "ckpt.pt"
    m.save(p)
    m2 = StudentForceField.load(p)
    for k, v in m2.state_dict().items():
        np.testing.assert_array_equal(v.numpy(), weights_seed0[k])
    # legacy checkpoint without config, trainer-style "model." prefix
    torch.save({"model_state_dict": {"model." + k: torch.tensor(v) for k, v in weights_seed0.items()}}, p)
    m3 = StudentForceField.load(p)
    assert m3.num_interactions == 3 and m3.hidden_dim == 128 and m3.max_z == 118


def test_model_refuses_cpu_compute(weights_seed0):
    import torch
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField()
    with pytest.raises(RuntimeError, match="CUDA"):
        m(torch.tensor([1, 1]), torch.tensor([[0.0, 0, 0], [1.0, 0, 0]]))


def test_force_loss_gradient_arguments_checked_on_host():
    """mlff_param_grads_forces validates its arguments before any device
    work: no direction (neither force nor virial weights), a NULL workspace
    and a short workspace."""
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    d = dims_of(128, 20, 3, 119, 5.0)
    pos = (ctypes.c_float * 6)()
    Z = (ctypes.c_int64 * 2)(1, 1)
    ptr = (ctypes.c_int64 * 2)(0, 2)
    s = _lib.System()
    s.n_atoms, s.n_mol = 2, 1
    s.pos = ctypes.cast(pos, ctypes.c_void_p).value
    s.Z = ctypes.cast(Z, ctypes.c_void_p).value
    s.mol_ptr = ctypes.cast(ptr, ctypes.c_void_p).value
    g = _lib.Grads()
    need = lib.mlff_workspace_size(ctypes.byref(d), 2, 1, 1024, _lib.PATH_TRAIN_FORCES)
    fake = ctypes.c_void_p(256)   # never dereferenced: every call below fails on the host
    r = lib.mlff_param_grads_forces(ctypes.byref(d), fake, ctypes.byref(s), 1024, None, None, ctypes.byref(g),
                                    fake, need, None)
    assert r == _lib.ERR_INVALID and b"force_weights" in lib.mlff_last_error_string()
    r = lib.mlff_param_grads_forces(ctypes.byref(d), fake, ctypes.byref(s), 1024, fake, None, ctypes.byref(g), None,
                                    need, None)
    assert r == _lib.ERR_INVALID and b"workspace" in lib.mlff_last_error_string()
    r = lib.mlff_param_grads_forces(ctypes.byref(d), fake, ctypes.byref(s), 1024, None, fake, ctypes.byref(g), fake,
                                    need - 1, None)
    assert r == _lib.ERR_WORKSPACE


def test_npt_arguments_checked_on_host():
    """mlff_npt_steps validates its arguments before any device work: a
    missing NPT state, missing periodic flags, a thermostat without a
    temperature and a negative pfactor."""
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    d = dims_of(128, 20, 3, 119, 5.0)
    fake = ctypes.c_void_p(256)   # never dereferenced: every call below fails on the host
    s = _lib.System()
    s.n_atoms, s.n_mol = 3, 1
    s.pos = s.Z = s.mol_ptr = fake.value
    st = _lib.MDState()
    st.pos = st.vel = st.inv_mass = st.forces = st.energy = fake.value
    npt = _lib.NPTState()
    npt.box = npt.box32 = npt.zeta = npt.eta = npt.xi = npt.virial = fake.value
    dbl = ctypes.c_double

    def call(state, flags, kT, ttime, pfactor):
        s.box = s.pbc = flags
        return lib.mlff_npt_steps(ctypes.byref(d), fake, ctypes.byref(s), 1024, _lib.PATH_TUNED_TC,
                                  ctypes.byref(st), state, dbl(0.02), dbl(kT), dbl(ttime), dbl(pfactor), dbl(0.0),
                                  1, fake, 1 << 30, None)

    assert call(None, fake.value, 0.025, 2.5, 1.0) == _lib.ERR_INVALID
    assert b"NPT state" in lib.mlff_last_error_string()
    assert call(ctypes.byref(npt), None, 0.025, 2.5, 1.0) == _lib.ERR_INVALID
    assert call(ctypes.byref(npt), fake.value, 0.0, 2.5, 1.0) == _lib.ERR_INVALID
    assert call(ctypes.byref(npt), fake.value, 0.025, 2.5, -1.0) == _lib.ERR_INVALID
    assert b"pfactor" in lib.mlff_last_error_string()


def test_autotune_cache_on_host():
    """The partition-factor cache: per (path, ceil log2 atoms, ceil log2
    structures) bucket, pinned with _set, read with _query, emptied with
    _reset; the workspace size does not depend on it."""
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    tc = _lib.PATH_TUNED_TC
    f = ctypes.c_int32()
    assert lib.mlff_autotune_reset() == _lib.OK
    d = dims_of(128, 20, 3, 119, 5.0)
    ws0 = lib.mlff_workspace_size(ctypes.byref(d), 9000, 200, 500_000, tc)
    assert lib.mlff_autotune_query(tc, 9000, 200, ctypes.byref(f)) == _lib.OK and f.value == 1
    assert lib.mlff_autotune_set(tc, 9000, 200, 4) == _lib.OK
    for n_atoms, n_mol, want in ((9000, 200, 4), (16384, 256, 4), (8193, 129, 4),   # same bucket (14, 8)
                                 (16385, 200, 1), (8192, 200, 1), (9000, 257, 1)):   # neighbouring buckets
        assert lib.mlff_autotune_query(tc, n_atoms, n_mol, ctypes.byref(f)) == _lib.OK
        assert f.value == want, (n_atoms, n_mol, f.value)
    assert lib.mlff_workspace_size(ctypes.byref(d), 9000, 200, 500_000, tc) == ws0
    # other paths have nothing to tune
    assert lib.mlff_autotune_query(_lib.PATH_PLAIN_FP32, 9000, 200, ctypes.byref(f)) == _lib.OK and f.value == 1
    assert lib.mlff_autotune_set(_lib.PATH_PLAIN_FP32, 9000, 200, 2) == _lib.ERR_INVALID
    assert lib.mlff_autotune_set(tc, 9000, 200, 3) == _lib.ERR_INVALID
    assert lib.mlff_autotune_set(tc, 9000, 200, 0) == _lib.OK
    assert lib.mlff_autotune_query(tc, 9000, 200, ctypes.byref(f)) == _lib.OK and f.value == 1
    lib.mlff_autotune_set(tc, 9000, 200, 2)
    assert lib.mlff_autotune_reset() == _lib.OK
    assert lib.mlff_autotune_query(tc, 9000, 200, ctypes.byref(f)) == _lib.OK and f.value == 1


def test_autotune_shape_cache_on_host():
    """The update-tile half of the shape cache: untuned buckets use 64-atom
    tiles, _set_shape pins (factor, tile), _set keeps a bucket's tile, other
    tile sizes and other paths are rejected, the workspace size does not
    depend on the shape."""
    import ctypes
    from mlff_gb300 import _lib
    from mlff_gb300.engine import dims_of
    lib = _lib.load()
    tc = _lib.PATH_TUNED_TC
    f, ut = ctypes.c_int32(), ctypes.c_int32()
    assert lib.mlff_autotune_reset() == _lib.OK
    d = dims_of(128, 20, 3, 119, 5.0)
    ws0 = lib.mlff_workspace_size(ctypes.byref(d), 3000, 1, 200_000, tc)
    assert lib.mlff_autotune_query_shape(tc, 3000, 1, ctypes.byref(f), ctypes.byref(ut)) == _lib.OK
    assert (f.value, ut.value) == (1, 64)
    assert lib.mlff_autotune_set_shape(tc, 3000, 1, 2, 32) == _lib.OK
    assert lib.mlff_autotune_query_shape(tc, 2049, 1, ctypes.byref(f), ctypes.byref(ut)) == _lib.OK   # same bucket
    assert (f.value, ut.value) == (2, 32)
    assert lib.mlff_autotune_query(tc, 3000, 1, ctypes.byref(f)) == _lib.OK and f.value == 2
    assert lib.mlff_autotune_set(tc, 3000, 1, 4) == _lib.OK                                          # tile kept
    assert lib.mlff_autotune_query_shape(tc, 3000, 1, ctypes.byref(f), ctypes.byref(ut)) == _lib.OK
    assert (f.value, ut.value) == (4, 32)
    assert lib.mlff_workspace_size(ctypes.byref(d), 3000, 1, 200_000, tc) == ws0
    assert lib.mlff_autotune_set_shape(tc, 3000, 1, 1, 48) == _lib.ERR_INVALID
    assert lib.mlff_autotune_set_shape(tc, 3000, 1, 3, 32) == _lib.ERR_INVALID
    assert lib.mlff_autotune_set_shape(_lib.PATH_PLAIN_FP32, 3000, 1, 1, 32) == _lib.ERR_INVALID
    assert lib.mlff_autotune_query_shape(tc, 3000, 1, None, ctypes.byref(ut)) == _lib.ERR_INVALID
    assert lib.mlff_autotune_set_shape(tc, 3000, 1, 0, 0) == _lib.OK                                  # removed
    assert lib.mlff_autotune_query_shape(tc, 3000, 1, ctypes.byref(f), ctypes.byref(ut)) == _lib.OK
    assert (f.value, ut.value) == (1, 64)
    assert lib.mlff_autotune_reset() == _lib.OK
