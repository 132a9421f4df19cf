"""Orthogonality and backward error of the GPU band reduction.

``avs_blockbidiag_tau_dev`` leaves the band, the Householder vectors of every
tile factorisation and their tau; Q and P are rebuilt from them in float64
(``oracle/reflectors.py``) and the tests assert, for n <= 1024, tiles 16-256,
FP64, FP32 and the tensor-core modes:

* ||A - Q B P^T||_F / ||A||_F <= n * eps and ||Q^T Q - I||_F, ||P^T P - I||_F
  <= n * eps (eps of the tile type);
* the vectors and tau equal the oracle's (the CPU restatement of
  QRkernels.jl:3-129 on the Blockbidiag! schedule, tiledalgos.jl:17-59) to the
  tolerance of the band-parity test.

The reference's own tests pin the same factors and applies against LAPACK
(KAbasedSVD/test/test_QR_kernels.jl:16-62) and the band through its singular
values (test_tiledalgo.jl:32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,b", [(256, 16), (512, 32), (512, 64), (1024, 128), (1024, 256)])
def test_band_reduction_backward_error(avs_mod, oracle_mod, torch_cuda, dt, n, b):
    from oracle import reflectors
    a = np.random.default_rng(7 * n + b).standard_normal((n, n)).astype(dt)
    t = avs_mod.to_device(a)
    tq, tp = avs_mod.Blockbidiag_tau(t, b)
    out = avs_mod.from_device(t)
    tq, tp = tq.cpu().numpy(), tp.cpu().numpy()
    back, oq, op = reflectors.checks(a, out, tq, tp, b)
    eps = np.finfo(dt).eps
    assert back < n * eps and oq < n * eps and op < n * eps, (back, oq, op)
    ref, rq, rp = oracle_mod.blockbidiag_keep(a, b)
    tol = 1e-10 if dt == np.float64 else 2e-3
    assert rel_err(out, ref) < tol
    nt = n // b
    for k in range(nt):  # GEQRT / GELQT tau[b-1] is not a reflector
        rq[(k * nt + k) * b + b - 1] = tq[(k * nt + k) * b + b - 1]
        if k + 1 < nt:
            rp[(k * nt + k + 1) * b + b - 1] = tp[(k * nt + k + 1) * b + b - 1]
    assert rel_err(tq, rq) < tol and rel_err(tp, rp) < tol


@pytest.mark.parametrize("precision", ["bf16x3", "tf32x3", "fp32"])
@pytest.mark.parametrize("n,b", [(512, 128), (1024, 256)])
def test_band_reduction_backward_error_tensor_cores(avs_mod, torch_cuda, precision, n, b):
    """The tensor-core trailing updates (split BF16 / split TF32, FP32
    accumulation) keep A = Q B P^T to FP32-class accuracy."""
    from oracle import reflectors
    a = (np.random.default_rng(11 * n + b).standard_normal((n, n)) / np.sqrt(n)).astype(np.float32)
    t = avs_mod.to_device(a)
    r = avs_mod.Report()
    tq, tp = avs_mod.Blockbidiag_tau(t, b, precision=precision, report=r)
    assert r.precision == avs_mod.PREC[precision]
    back, oq, op = reflectors.checks(a, avs_mod.from_device(t), tq.cpu().numpy(), tp.cpu().numpy(), b)
    eps = np.finfo(np.float32).eps
    assert back < n * eps and oq < n * eps and op < n * eps, (back, oq, op)
