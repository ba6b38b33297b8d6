"""Bounded device waits (GPU only).  A wait that runs out must end the
kernel cleanly: MLFF_ERR_TIMEOUT in the status word, the kernel's own
copies and MMAs drained, tensor memory freed, the context usable.  The
timeout is forced with the library's test hook (a wait on an mbarrier that
nothing arrives at); no GPU fault, trap or hang is involved."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

WHERE_STALL_TEST = 99


def model_for(weights):
    from mlff_gb300.student_model import StudentForceField
    m = StudentForceField(precision="fp16x3").to("cuda")
    m.load_state_dict({k: torch.tensor(v) for k, v in weights.items()})
    return m.eval()


@pytest.mark.parametrize("kernels", [1, 2, 3], ids=["forward", "reverse", "both"])
def test_forced_timeout_reported_and_next_call_unaffected(golden_cases, weights_bias, kernels):
    from mlff_gb300 import _lib
    from mlff_gb300.engine import make_batch
    g = golden_cases
    b = make_batch(g["molecule60/Z"], g["molecule60/pos"], g["molecule60/mol_ptr"])
    fresh = model_for(weights_bias).engine()
    E0, F0, _ = fresh.energy_forces(b, _lib.PATH_TUNED_TC, graph=False)
    E0, F0 = E0.cpu().numpy(), F0.cpu().numpy()

    eng = model_for(weights_bias).engine()
    lib = _lib.load()
    try:
        _lib.check(lib.mlff_debug_stall_test(kernels))
        with pytest.raises(_lib.MLFFError) as ei:
            eng.energy_forces(b, _lib.PATH_TUNED_TC, graph=False)
        assert ei.value.code == _lib.ERR_TIMEOUT
        code, _, where = eng.status()
        assert code == _lib.ERR_TIMEOUT and where == WHERE_STALL_TEST
    finally:
        _lib.check(lib.mlff_debug_stall_test(0))
    torch.cuda.synchronize()                       # the context is still usable
    assert float(torch.ones(4, device="cuda").sum()) == 4.0
    E1, F1, _ = eng.energy_forces(b, _lib.PATH_TUNED_TC, graph=False)
    np.testing.assert_array_equal(E1.cpu().numpy(), E0)
    np.testing.assert_array_equal(F1.cpu().numpy(), F0)


def test_stall_hook_rejects_bad_mask():
    from mlff_gb300 import _lib
    lib = _lib.load()
    assert lib.mlff_debug_stall_test(4) == _lib.ERR_INVALID
    assert lib.mlff_debug_stall_test(-1) == _lib.ERR_INVALID
    assert lib.mlff_debug_stall_test(0) == _lib.OK
