"""GPU test of the failure path: every cross-CTA dependency of the library is a
bounded wait that records a timeout in the device status word instead of
hanging.  A kernel waits, with a short bound, on a flag that nothing sets; the
call returns AVS_ERR_TIMEOUT and the handle and the CUDA context stay usable.
No GPU fault, trap or hang is involved."""
import numpy as np
import pytest
import scipy.linalg as sl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_bounded_wait_times_out_and_context_survives(avs_mod, torch_cuda):
    h = avs_mod.Handle()
    try:
        assert avs_mod.selftest_timeout(handle=h) == 3  # AVS_ERR_TIMEOUT
        a = np.random.default_rng(2).standard_normal((128, 128)).astype(np.float32)
        s = avs_mod.my_CU_svdval(a, 32, handle=h)
        ref = sl.svdvals(a.astype(np.float64))
        assert np.max(np.abs(s - ref)) / ref[0] < 1e-5
        assert avs_mod.selftest_timeout(handle=h) == 3
    finally:
        h.close()


def test_loaded_device_code_is_sm103(avs_mod):
    """The runtime reports the library's device code as built for sm_103
    (cudaFuncAttributes.binaryVersion)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    bv, pv = avs_mod.kernel_arch(0)
    assert bv == 103, (bv, pv)
