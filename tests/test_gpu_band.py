"""GPU hierarchical band reduction (stage2_band.cu) against the oracle's
restatement of one stage of the reference's bidiag! (BRD/src/bulgechasing2.jl:
22-45, oracle/brd.py ``stage``): the same LQ_QMUL / QR_QMUL operations on the
same seeded band, so the reduced band agrees entry by entry (FP64: 1e-12 of
the largest entry; FP32: singular values to FP32 rounding), nothing is left outside the target
width, and the singular values are kept (LAPACK).  The full pipeline through
the hierarchical stage 2 is checked against LAPACK and against the
one-stage element chase."""
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


def _band(n, bw, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    return np.triu(a) - np.triu(a, bw + 1)


CASES = [(256, 64, 16), (300, 64, 16), (512, 128, 16), (520, 128, 32), (1024, 256, 16), (1024, 256, 32),
         (1000, 256, 32), (256, 256, 16)]


@pytest.mark.parametrize("n,bw,tbw", CASES)
def test_band_stage_fp64_vs_oracle(avs_mod, torch_cuda, n, bw, tbw):
    from oracle import brd
    a = _band(n, bw, n + bw + tbw)
    ref = brd.stage(a, bw, tbw)
    B = avs_mod.to_device(a)
    avs_mod.band_reduce(B, bw, tbw)
    got = avs_mod.from_device(B)
    scale = np.abs(a).max()
    i, j = np.indices(got.shape)
    assert np.max(np.abs(got[(j - i > tbw) | (j < i)])) <= 1e-14 * scale
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale
    s = sl.svdvals(a)
    assert np.max(np.abs(sl.svdvals(got) - s)) <= 1e-12 * s[0]


@pytest.mark.parametrize("n,bw,tbw", [(512, 64, 16), (1024, 128, 16), (1024, 256, 16), (2048, 256, 32)])
def test_band_stage_fp32(avs_mod, torch_cuda, n, bw, tbw):
    a = _band(n, bw, 7 * n + bw).astype(np.float32)
    B = avs_mod.to_device(a)
    avs_mod.band_reduce(B, bw, tbw)
    got = avs_mod.from_device(B).astype(np.float64)
    i, j = np.indices(got.shape)
    assert np.max(np.abs(got[(j - i > tbw) | (j < i)])) == 0.0
    s = sl.svdvals(a.astype(np.float64))
    assert np.max(np.abs(sl.svdvals(got) - s)) <= 1e-5 * s[0]
    # the FP32 band is not compared entry by entry: a reflector whose alpha is
    # at the rounding level may take the other sign, after which the bands
    # differ by signs and rotations while the singular values agree


def test_band_stage_rejects_pairs(avs_mod, torch_cuda):
    B = avs_mod.to_device(_band(256, 64, 1))
    with pytest.raises(avs_mod.AvsError):
        avs_mod.band_reduce(B, 64, 32)
    with pytest.raises(avs_mod.AvsError):
        avs_mod.band_reduce(B, 64, 64)


@pytest.mark.parametrize("dtype,tile,prec,tol", [(np.float64, 64, "fp64", 1e-12), (np.float64, 256, "fp64", 1e-12),
                                                 (np.float32, 128, "fp32", 1e-5), (np.float32, 256, "bf16x3", 1e-5)])
def test_pipeline_hierarchical_vs_one_stage(avs_mod, torch_cuda, dtype, tile, prec, tol):
    """The hierarchical stage 2 (band 16 and band 32) and the one-stage
    element chase (AVS_FLAG_ONE_STAGE_CHASE) give the same values within the
    mode's tolerance, and all match LAPACK."""
    import ctypes
    n = 1024
    rng = np.random.default_rng(tile + n)
    a = (rng.standard_normal((n, n)) / np.sqrt(n)).astype(dtype)
    lap = sl.svdvals(a.astype(np.float64))
    dA = avs_mod.to_device(a)
    outs = []
    # FP64 stages run the hierarchy only on request (AVS_FLAG_HIER_CHASE = 32)
    hier = 32 if dtype == np.float64 else 0
    for flags in (hier, 4, hier | 8):
        torch = torch_cuda
        sig = torch.empty(n, dtype=dA.dtype, device=dA.device)
        o = avs_mod.Opts(avs_mod.PREC[prec], flags, 0.0, None)
        r = avs_mod.Report()
        fn = avs_mod.lib().avs_svdvals_dev_d if dtype == np.float64 else avs_mod.lib().avs_svdvals_dev_s
        rc = fn(avs_mod.default_handle().ptr, n, n, n, tile, ctypes.c_void_p(dA.data_ptr()),
                ctypes.c_void_p(sig.data_ptr()), ctypes.byref(o), ctypes.byref(r))
        assert rc == 0
        s = sig.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(s - lap)) < tol * lap[0]
        outs.append(s)
    assert np.max(np.abs(outs[0] - outs[1])) < tol * lap[0]


@pytest.mark.parametrize("dtype,n,tile,prec,tol", [(np.float32, 1024, 16, "fp32", 1e-5), (np.float32, 1024, 32, "fp32", 1e-5),
                                                   (np.float32, 2048, 256, "bf16x3", 1e-5),
                                                   (np.float64, 1024, 128, "fp64", 1e-12),
                                                   (np.float64, 1024, 16, "fp64", 1e-12),
                                                   (np.float64, 1024, 32, "fp64", 1e-12)])
def test_window_chase_vs_cluster_chase(avs_mod, torch_cuda, dtype, n, tile, prec, tol):
    """The narrow band's element chase in the shared-memory window (default)
    and with one cluster per sweep (AVS_FLAG_CLUSTER_CHASE) agree within the
    mode's tolerance, and both match LAPACK."""
    import ctypes
    if n % tile:
        pytest.skip("tile does not divide n")
    rng = np.random.default_rng(n + tile)
    a = (rng.standard_normal((n, n)) / np.sqrt(n)).astype(dtype)
    lap = sl.svdvals(a.astype(np.float64))
    dA = avs_mod.to_device(a)
    outs = []
    for flags in (0, 16, 0):
        torch = torch_cuda
        sig = torch.empty(n, dtype=dA.dtype, device=dA.device)
        o = avs_mod.Opts(avs_mod.PREC[prec], flags, 0.0, None)
        r = avs_mod.Report()
        fn = avs_mod.lib().avs_svdvals_dev_d if dtype == np.float64 else avs_mod.lib().avs_svdvals_dev_s
        rc = fn(avs_mod.default_handle().ptr, n, n, n, tile, ctypes.c_void_p(dA.data_ptr()),
                ctypes.c_void_p(sig.data_ptr()), ctypes.byref(o), ctypes.byref(r))
        assert rc == 0
        s = sig.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(s - lap)) < tol * lap[0]
        outs.append(s)
    assert np.max(np.abs(outs[0] - outs[1])) < tol * lap[0]
    assert np.array_equal(outs[0], outs[2])  # the window chase is deterministic
