"""GPU test of the tcgen05 GEMM behind the tensor-core trailing updates:
TF32 (1 product) and split TF32 (3 products) against an FP64 product of the
same device data, for every combination of operand major order."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def selftest(avs_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    f = avs_mod.lib().avsx_tc_gemm_selftest
    f.argtypes = [ctypes.c_int] * 6 + [ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int

    def run(M, N, K, akm, bkm, split):
        e = ctypes.c_float(-1.0)
        rc = f(M, N, K, akm, bkm, split, ctypes.byref(e))
        assert rc == 0, rc
        return e.value
    return run


@pytest.mark.parametrize("akm,bkm", [(1, 1), (0, 1), (1, 0), (0, 0)])
@pytest.mark.parametrize("shape", [(128, 128, 32), (256, 384, 256)])
def test_tc_gemm_split_tf32(selftest, akm, bkm, shape):
    err = selftest(*shape, akm, bkm, 3)
    assert 0 <= err < 1e-5, err  # FP32 accumulation over K: ~sqrt(K) * 2^-24


@pytest.mark.parametrize("shape", [(128, 128, 32), (256, 256, 256)])
def test_tc_gemm_tf32(selftest, shape):
    err = selftest(*shape, 1, 1, 1)
    assert 0 <= err < 2e-3, err
