"""Autotuned shapes (GPU only): the tensor-core path gives the same
results, bit for bit, for every partition factor and update tile the
autotuner can choose, and mlff_autotune caches one of them for the call's
size bucket."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _model(weights):
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision="fp16x3").to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    return m.eval()


def _systems():
    from mlff_gb300 import systems
    return [systems.molecule_batch(40, 10, 120, seed=21), systems.water_box(n_water=300, L=20.8, d_oo=2.5, seed=4)]


@pytest.mark.parametrize("which", [0, 1], ids=["molecules", "water_box"])
def test_results_do_not_depend_on_the_tuned_shapes(weights_bias, which):
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    lib = _lib.load()
    s = _systems()[which]
    per = bool(s.pbc.any())
    b = make_batch(s.Z, s.pos.astype(np.float32), s.mol_ptr, s.box if per else None, s.pbc if per else None)
    eng = _model(weights_bias).engine()
    eng.auto_tune = False
    res = []
    try:
        for f, ut in ((1, 64), (2, 64), (4, 64), (1, 32), (4, 32)):
            _lib.check(lib.mlff_autotune_set_shape(_lib.PATH_TUNED_TC, b.n_atoms, b.n_mol, f, ut))
            E, F, V = eng.energy_forces(b, _lib.PATH_TUNED_TC, virial=per, graph=False)
            res.append([t.cpu().numpy() for t in (E, F) + ((V,) if per else ())])
    finally:
        lib.mlff_autotune_set(_lib.PATH_TUNED_TC, b.n_atoms, b.n_mol, 0)
    for other in res[1:]:
        for a, c in zip(res[0], other):
            np.testing.assert_array_equal(a, c)


def test_autotune_caches_a_candidate(weights_bias):
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    lib = _lib.load()
    s = _systems()[0]
    b = make_batch(s.Z, s.pos.astype(np.float32), s.mol_ptr)
    eng = _model(weights_bias).engine()
    E0, F0, _ = eng.energy_forces(b, _lib.PATH_TUNED_TC, graph=False)
    got = eng.autotune(b, _lib.PATH_TUNED_TC, repeats=2)
    assert got["partition_factor"] in (1, 2, 4) and got["update_tile_atoms"] in (32, 64)
    assert all(v > 0 for v in got["ms_per_call"].values())
    f, ut = ctypes.c_int32(), ctypes.c_int32()
    _lib.check(lib.mlff_autotune_query_shape(_lib.PATH_TUNED_TC, b.n_atoms, b.n_mol, ctypes.byref(f), ctypes.byref(ut)))
    assert (f.value, ut.value) == (got["partition_factor"], got["update_tile_atoms"])
    E1, F1, _ = eng.energy_forces(b, _lib.PATH_TUNED_TC, graph=False)
    np.testing.assert_array_equal(E0.cpu().numpy(), E1.cpu().numpy())
    np.testing.assert_array_equal(F0.cpu().numpy(), F1.cpu().numpy())
    lib.mlff_autotune_set(_lib.PATH_TUNED_TC, b.n_atoms, b.n_mol, 0)
