"""GPU parity tests: the CUDA library through the C ABI against the oracle
(the CPU restatement of the reference path) and LAPACK, on seeded inputs.

Tolerances (normwise on singular values, as Julia's isapprox in the reference
tests): FP64 path 1e-12 * sigma_max, FP32 path 1e-5 * sigma_max."""
import os

import numpy as np
import pytest
import scipy.linalg as sl

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")
TOL = {np.float64: 1e-12, np.float32: 1e-5}


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("b", [16, 32, 64, 128, 256])
def test_geqrt_tsqrt_tiles_vs_oracle(avs_mod, oracle_mod, torch_cuda, dt, b):
    """QR_unsafe_kernel! / QR_unsafe_kernel2! (QRkernels.jl:3-129) on the GPU
    match the oracle's factors and tau."""
    rng = np.random.default_rng(1000 + b)
    a = rng.random((b, b)).astype(dt)
    f_gpu, tau_gpu = avs_mod.geqrt_tile(a)
    f_ref, tau_ref = oracle_mod.geqrt(a)
    tol = 50 * np.finfo(dt).eps * b
    assert rel_err(f_gpu, f_ref) < tol
    assert rel_err(tau_gpu[: b - 1], tau_ref[: b - 1]) < tol
    a2 = rng.random((2 * b, b)).astype(dt)
    r_gpu, v_gpu, t_gpu = avs_mod.tsqrt_tile(a2[:b], a2[b:])
    r_ref, v_ref, t_ref = oracle_mod.tsqrt(a2[:b], a2[b:])
    assert rel_err(np.triu(r_gpu), np.triu(r_ref)) < tol
    assert np.array_equal(np.tril(r_gpu, -1), np.tril(a2[:b], -1))
    assert rel_err(v_gpu, v_ref) < tol
    assert rel_err(t_gpu, t_ref) < tol


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,b", [(64, 16), (96, 16), (128, 32), (256, 64), (512, 128), (512, 256)])
def test_blockbidiag_band_vs_oracle(avs_mod, oracle_mod, torch_cuda, dt, n, b):
    """Blockbidiag! on the GPU gives the oracle's band entry by entry (same flat
    tree, same reflectors) and keeps the singular values."""
    a = np.random.default_rng(n * 7 + b).standard_normal((n, n)).astype(dt)
    t = avs_mod.to_device(a)
    avs_mod.Blockbidiag(t, b)
    band_gpu = oracle_mod.extract_band(avs_mod.from_device(t), b)
    band_ref = oracle_mod.extract_band(oracle_mod.blockbidiag(a, b), b)
    tol = 1e-10 if dt == np.float64 else 2e-3
    assert rel_err(band_gpu, band_ref) < tol
    s_ref = sl.svdvals(a.astype(np.float64))
    assert rel_err(sl.svdvals(band_gpu.astype(np.float64)), s_ref) < 10 * TOL[dt]


@pytest.mark.parametrize("n,bw", [(64, 16), (100, 16), (256, 32), (512, 64), (768, 128), (1024, 256)])
def test_band_to_bidiag_vs_lapack(avs_mod, oracle_mod, torch_cuda, n, bw):
    """bidiagonalize (bulgechasing.jl:33-42) on the GPU: FP64 chase keeps the
    band's singular values (the oracle's multi-stage chase gives the same)."""
    torch = torch_cuda
    rng = np.random.default_rng(n + 3 * bw)
    band = np.triu(np.tril(rng.standard_normal((n, n)), bw))
    B = avs_mod.to_device(band)
    d, e = avs_mod.bidiagonalize(B, bw)
    d, e = d.cpu().numpy(), e.cpu().numpy()
    s_ref = sl.svdvals(band)
    s_gpu_bd = sl.svdvals(np.diag(d) + np.diag(e, 1))
    assert rel_err(s_gpu_bd, s_ref) < 1e-13
    bo = oracle_mod.bidiagonalize(band, bw)
    do, eo = oracle_mod.extract_bidiag(bo)
    assert rel_err(oracle_mod.bidiag_svals(do, eo), s_gpu_bd) < 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 17, 256, 1000])
def test_bidiag_svals_vs_lapack(avs_mod, oracle_mod, torch_cuda, n):
    """diag_lapack (bdsdc('U','N'), bulgechasing.jl:50-53): FP64 bisection on the GPU."""
    torch = torch_cuda
    rng = np.random.default_rng(n)
    d = rng.standard_normal(n)
    e = rng.standard_normal(max(n - 1, 0))
    s = avs_mod.diag_lapack(torch.from_numpy(d).cuda(), torch.from_numpy(e).cuda()).cpu().numpy()
    B = np.diag(d) + (np.diag(e, 1) if n > 1 else 0)
    ref = sl.svdvals(B)
    assert np.all(np.diff(s) <= 0)
    assert rel_err(s, ref) < 1e-14
    assert rel_err(s, oracle_mod.bidiag_svals(d, e)) < 1e-14


def test_golden_fixtures_gpu(avs_mod, torch_cuda):
    g = np.load(GOLDEN)
    names = sorted({k[: -len("_A")] for k in g.files if k.endswith("_A")})
    for name in names:
        a = g[name + "_A"]
        b = int(g[name + "_tile"])
        s = avs_mod.my_CU_svdval(a, b)
        tol = TOL[a.dtype.type]
        assert rel_err(s, g[name + "_sigma_oracle"]) < tol, name
        assert rel_err(s, g[name + "_sigma_lapack"]) < tol, name


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("b,nt", [(16, 4), (16, 7), (128, 4), (128, 7)])
def test_my_CU_svdval_reference_test(avs_mod, oracle_mod, torch_cuda, dt, b, nt):
    """CUDAbasedSVD/test.jl:6-17: integer-valued matrices, both the host
    (Matrix) and the device (CuMatrix) method, against the oracle and LAPACK."""
    n = b * nt
    a = np.random.default_rng(b * nt).integers(1, 11, size=(n, n)).astype(dt)
    a_copy = a.copy()
    ref = oracle_mod.svdvals(a, b)
    lap = sl.svdvals(a.astype(np.float64))
    s_host = avs_mod.my_CU_svdval(a, b)
    assert np.array_equal(a, a_copy)  # input not modified
    assert s_host.dtype == dt and np.all(np.diff(s_host) <= 0)
    assert rel_err(s_host, ref) < TOL[dt]
    assert rel_err(s_host, lap) < TOL[dt]
    t = avs_mod.to_device(a)
    t_copy = t.clone()
    s_dev = avs_mod.my_CU_svdval(t, b)
    assert bool((t == t_copy).all())
    assert rel_err(s_dev.cpu().numpy(), lap) < TOL[dt]


@pytest.mark.parametrize("dt,n,b", [(np.float64, 1024, 64), (np.float32, 1024, 64), (np.float64, 2048, 256),
                                    (np.float32, 2048, 128)])
def test_gaussian_vs_lapack_and_oracle(avs_mod, oracle_mod, torch_cuda, dt, n, b):
    """Config-1 shape (n=1024, tile 64, N(0,1)) and larger tiles."""
    from avs import workloads
    a = workloads.gaussian(n, 1, dtype=dt)
    s = avs_mod.my_CU_svdval(a, b)
    lap = sl.svdvals(a.astype(np.float64))
    assert rel_err(s, lap) < TOL[dt]
    if n <= 1024:
        assert rel_err(s, oracle_mod.svdvals(a, b)) < TOL[dt]


def test_geometric_spectrum_known_sigma(avs_mod, torch_cuda):
    """Config-2 distribution at n=2048: A = U diag(sigma) V^T with known sigma."""
    from avs import workloads
    a, sig = workloads.geometric_spectrum(2048, 2, 3, 1e-6)
    s = avs_mod.my_CU_svdval(a, 128)
    assert rel_err(s, sig) < 1e-12
    s32 = avs_mod.my_CU_svdval(a.astype(np.float32), 128)
    assert rel_err(s32, sig) < 1e-5


def test_not_implemented_cases_gpu(avs_mod, torch_cuda):
    a = np.ones((64, 64), dtype=np.float32)
    for b in (8, 24, 48, 128):
        with pytest.raises(NotImplementedError):
            avs_mod.my_CU_svdval(a, b)
    with pytest.raises(NotImplementedError):
        avs_mod.my_CU_svdval(np.ones((64, 32), dtype=np.float32), 16)
    t = avs_mod.to_device(np.ones((64, 32), dtype=np.float32))
    with pytest.raises(NotImplementedError):
        avs_mod.my_CU_svdval(t, 16)


def test_zero_and_degenerate_inputs(avs_mod, torch_cuda):
    """Zero columns (reference: 0/0 in the reflector) give the identity
    reflector here; rank-deficient matrices keep exact zeros."""
    n, b = 128, 16
    z = np.zeros((n, n))
    assert np.all(avs_mod.my_CU_svdval(z, b) == 0)
    a = np.random.default_rng(3).standard_normal((n, 4)) @ np.random.default_rng(4).standard_normal((4, n))
    s = avs_mod.my_CU_svdval(a, b)
    ref = sl.svdvals(a)
    assert rel_err(s, ref) < 1e-12
    d = np.diag(np.arange(1, n + 1, dtype=np.float64))
    assert rel_err(avs_mod.my_CU_svdval(d, b), np.arange(n, 0, -1)) < 1e-14


@pytest.mark.parametrize("n,b", [(512, 32), (1024, 64), (2048, 128), (2048, 256)])
def test_double_float_stages_match_fp64_stages(avs_mod, torch_cuda, n, b):
    """The element chase and bisection in double-float arithmetic agree with
    the FP64 stages on the same band (1e-9 normwise, plus one unit of the FP32
    output's rounding); on FP64 tiles the double-float
    stages stay within 1e-12 of the known spectrum.  The default FP32-class
    stage 2 (FP32 block stage to band 16, then the double-float chase) stays
    at FP32 level of the FP64 stages."""
    from avs import workloads
    a, sig = workloads.geometric_spectrum(n, 21, 22, 1e-6)
    s64 = avs_mod.my_CU_svdval(a, b, stages="fp64")
    sdf = avs_mod.my_CU_svdval(a, b, stages="df64")
    assert rel_err(s64, sig) < 1e-12
    assert rel_err(sdf, sig) < 1e-12
    a32 = a.astype(np.float32)
    s32_64 = avs_mod.my_CU_svdval(a32, b, stages="fp64")
    s32_df = avs_mod.my_CU_svdval(a32, b, flags=avs_mod.FLAGS["one_stage_chase"])
    # normwise 1e-9, plus the FP32 output's own rounding (a value on a rounding
    # boundary may land one unit apart)
    assert np.all(np.abs(s32_df - s32_64) <= 1e-9 * s32_64[0] + np.spacing(s32_64))
    assert rel_err(s32_df, sig) < 1e-5
    s32_h = avs_mod.my_CU_svdval(a32, b)  # hierarchical for tiles >= 64
    assert rel_err(s32_h, s32_64) < 1e-6
    assert rel_err(s32_h, sig) < 1e-5


@pytest.mark.parametrize("n,b", [(512, 128), (1024, 128), (1024, 256), (2048, 256)])
def test_tensor_core_modes(avs_mod, torch_cuda, n, b):
    """Trailing updates on tcgen05: split TF32 and split BF16 (3 products each)
    keep FP32-class accuracy (<= 1e-5 of sigma_max against LAPACK);
    single-pass TF32 and BF16 state their larger errors."""
    from avs import workloads
    a = workloads.gaussian(n, 31, 1.0 / np.sqrt(n), dtype=np.float32)
    lap = sl.svdvals(a.astype(np.float64))
    r = avs_mod.Report()
    s3 = avs_mod.my_CU_svdval(a, b, precision="tf32x3", report=r)
    assert r.precision == 4
    assert rel_err(s3, lap) < 1e-5
    s32 = avs_mod.my_CU_svdval(a, b, precision="fp32")
    assert rel_err(s3, s32) < 1e-5
    s1 = avs_mod.my_CU_svdval(a, b, precision="tf32")
    assert rel_err(s1, lap) < 5e-3
    sb3 = avs_mod.my_CU_svdval(a, b, precision="bf16x3")
    assert rel_err(sb3, lap) < 1e-5
    sb = avs_mod.my_CU_svdval(a, b, precision="bf16")
    assert rel_err(sb, lap) < 5e-2


@pytest.mark.parametrize("n,b", [(512, 128), (1024, 128), (1024, 256), (2048, 128), (2048, 256)])
def test_fp64x2_mode(avs_mod, torch_cuda, n, b):
    """AVS_PREC_FP64X2: FP64 tiles and panels, the full compact-WY trailing
    updates in double-float (two-term split FP32 products) and double-float
    stages 2-3 -- FP64-level accuracy: within 1e-12 (normwise) of LAPACK on
    Gaussian inputs and of the known spectrum on a graded one; the float32
    entry point with this mode computes in FP64 tiles too."""
    from avs import workloads
    a = workloads.gaussian(n, 77, 1.0 / np.sqrt(n))
    r = avs_mod.Report()
    s = avs_mod.my_CU_svdval(a, b, precision="fp64x2", report=r)
    assert r.precision == 7
    assert rel_err(s, sl.svdvals(a)) < 1e-12
    g, sig = workloads.geometric_spectrum(n, 5, 6, 1e-6)
    assert rel_err(avs_mod.my_CU_svdval(g, b, precision="fp64x2"), sig) < 1e-12
    a32 = a.astype(np.float32)
    s32 = avs_mod.my_CU_svdval(a32, b, precision="fp64x2")
    assert s32.dtype == np.float32
    assert rel_err(s32, sl.svdvals(a32.astype(np.float64))) < 1e-6


def test_fp64x2_batched_equals_single(avs_mod, torch_cuda):
    """Batched FP64 groups in AVS_PREC_FP64X2 equal the single call in that
    mode bit for bit."""
    rng = np.random.default_rng(55)
    hosts = [rng.standard_normal((n, n)) / np.sqrt(n) for n in (256, 512, 256, 512)]
    devs = [avs_mod.to_device(a) for a in hosts]
    import ctypes
    h = avs_mod.default_handle()
    cnt = len(devs)
    outs = [torch_cuda.empty(d.shape[0], dtype=torch_cuda.float64, device=d.device) for d in devs]
    nn = (ctypes.c_int64 * cnt)(*[d.shape[0] for d in devs])
    tt = (ctypes.c_int32 * cnt)(*([128] * cnt))
    pa = (ctypes.c_void_p * cnt)(*[d.data_ptr() for d in devs])
    ps = (ctypes.c_void_p * cnt)(*[o.data_ptr() for o in outs])
    o = avs_mod.Opts(7, 0, 0.0, None)
    r = avs_mod.Report()
    rc = avs_mod.lib().avs_svdvals_batched_dev_d(h.ptr, cnt, nn, nn, tt, pa, ps, ctypes.byref(o), ctypes.byref(r))
    assert rc == 0 and r.precision == 7
    for a, d, out in zip(hosts, devs, outs):
        single = avs_mod.my_CU_svdval(d, 128, precision="fp64x2").cpu().numpy()
        assert np.array_equal(out.cpu().numpy(), single)
        assert rel_err(single, sl.svdvals(a)) < 1e-12
