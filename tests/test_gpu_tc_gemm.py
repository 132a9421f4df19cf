"""GPU test of the TMA-fed tcgen05 GEMM behind the tensor-core trailing
updates, against an FP64 product of the same device data, in every operand
format: TF32 and BF16 (one product), split TF32 and split BF16 (three
products), with 128- and 256-column tiles."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

FMT = {"tf32": 1, "tf32x3": 3, "bf16": 4, "bf16x3": 5}


@pytest.fixture(scope="module")
def selftest(avs_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    f = avs_mod.lib().avsx_tc_gemm_selftest
    f.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(ctypes.c_float)]
    f.restype = ctypes.c_int

    def run(M, N, K, fmt):
        e = ctypes.c_float(-1.0)
        rc = f(M, N, K, FMT[fmt], ctypes.byref(e))
        assert rc == 0, rc
        return e.value
    return run


SHAPES = [(128, 128, 64), (256, 256, 256), (256, 384, 256), (128, 512, 128)]


@pytest.mark.parametrize("shape", SHAPES)
def test_tc_gemm_split_tf32(selftest, shape):
    err = selftest(*shape, "tf32x3")
    assert 0 <= err < 1e-5, err  # FP32 accumulation over K: ~sqrt(K) * 2^-24


@pytest.mark.parametrize("shape", SHAPES)
def test_tc_gemm_tf32(selftest, shape):
    err = selftest(*shape, "tf32")
    assert 0 <= err < 2e-3, err


@pytest.mark.parametrize("shape", SHAPES)
def test_tc_gemm_split_bf16(selftest, shape):
    err = selftest(*shape, "bf16x3")
    assert 0 <= err < 1e-4, err  # two bf16 terms: ~16 significant bits


@pytest.mark.parametrize("shape", SHAPES)
def test_tc_gemm_bf16(selftest, shape):
    err = selftest(*shape, "bf16")
    assert 0 <= err < 2e-2, err
