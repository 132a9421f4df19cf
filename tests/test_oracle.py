"""CPU tests: the oracle (restatement of the reference path) against the
reference's own known-answer relations (LAPACK) and the committed golden
fixtures.  Mirrors KAbasedSVD/test/test_QR_kernels.jl, test_tiledalgo.jl and
CUDAbasedSVD/test.jl, with seeded inputs."""
import os

import numpy as np
import pytest
import scipy.linalg as sl

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


def julia_approx(x, y, rtol):
    """Julia's isapprox on arrays: norm(x - y) <= rtol * max(norm(x), norm(y))."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    return np.linalg.norm(x - y) <= rtol * max(np.linalg.norm(x), np.linalg.norm(y))


RTOL = {np.float32: np.sqrt(np.finfo(np.float32).eps), np.float64: np.sqrt(np.finfo(np.float64).eps)}


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("b", [16, 32])
def test_tile_kernels_vs_lapack(oracle_mod, dt, b):
    O = oracle_mod
    rng = np.random.default_rng(b)
    a = rng.random((b, b)).astype(dt)
    f, tau = O.geqrt(a)
    # QR_unsafe_kernel! factors == LAPACK qr(a).factors (test_QR_kernels.jl:16)
    assert julia_approx(f, sl.qr(a.astype(np.float64), mode="raw")[0][0], RTOL[dt])
    q = sl.qr(a.astype(np.float64))[0]
    bm = rng.random((b, 5 * b)).astype(dt)
    assert julia_approx(O.apply1(bm, f, tau, True), q.T @ bm, RTOL[dt])   # :20-21, :76
    assert julia_approx(O.apply1(bm, f, tau, False), q @ bm, RTOL[dt])    # :23-25
    a2 = rng.random((2 * b, b)).astype(dt)
    r, v, tau2 = O.tsqrt(a2[:b], a2[b:])
    stacked = np.vstack([np.triu(a2[:b]), a2[b:]]).astype(np.float64)
    # QR_unsafe_kernel2! == qr([triu R; B]).factors (:42)
    assert julia_approx(np.vstack([np.triu(r), v]), sl.qr(stacked, mode="raw")[0][0], RTOL[dt])
    # strictly-lower part of the top tile untouched (:41)
    assert np.array_equal(np.tril(r, -1), np.tril(a2[:b], -1))
    q2 = sl.qr(stacked)[0]
    bb = rng.random((2 * b, 5 * b)).astype(dt)
    o1, o2 = O.apply2(bb[:b], bb[b:], v, tau2, True)
    assert julia_approx(np.vstack([o1, o2]), q2.T @ bb, RTOL[dt])          # :84-85
    o1, o2 = O.apply2(bb[:b], bb[b:], v, tau2, False)
    assert julia_approx(np.vstack([o1, o2]), q2 @ bb, RTOL[dt])            # :51-52


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("b,nt", [(16, 4), (16, 6), (32, 4)])
def test_blockbidiag_preserves_svals(oracle_mod, dt, b, nt):
    """Blockbidiag! keeps the singular values and leaves an upper band (test_tiledalgo.jl:28-32)."""
    O = oracle_mod
    n = b * nt
    a = np.random.default_rng(nt * b).random((n, n)).astype(dt)
    band = O.blockbidiag(a, b)
    i, j = np.indices(band.shape)
    assert np.all(band[(j - i < 0) | (j - i > b)] == 0)
    assert julia_approx(sl.svdvals(band.astype(np.float64)), sl.svdvals(a.astype(np.float64)), RTOL[dt])


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,bw", [(64, 16), (128, 32), (200, 16), (256, 64)])
def test_bidiagonalize(oracle_mod, dt, n, bw):
    """bidiagonalize gives an exact bidiagonal with the band's singular values
    (the check of BRD/src/bulgechasing2.jl:101-116)."""
    O = oracle_mod
    rng = np.random.default_rng(n + bw)
    band = np.triu(np.tril(rng.standard_normal((n, n)), bw)).astype(dt)
    bd = O.bidiagonalize(band, bw)
    off = bd.copy()
    off[np.arange(n), np.arange(n)] = 0
    off[np.arange(n - 1), np.arange(1, n)] = 0
    assert np.all(off == 0)
    d, e = O.extract_bidiag(bd)
    assert julia_approx(O.bidiag_svals(d, e), sl.svdvals(band.astype(np.float64)), RTOL[dt])


def test_bidiag_svals_vs_lapack(oracle_mod):
    """Stage 3 (bdsdc('U','N')) restated as bisection equals LAPACK on the dense bidiagonal."""
    rng = np.random.default_rng(7)
    for n in (1, 2, 5, 64, 300):
        d = rng.standard_normal(n)
        e = rng.standard_normal(max(n - 1, 0))
        B = np.diag(d) + (np.diag(e, 1) if n > 1 else 0)
        ref = sl.svdvals(B)
        got = oracle_mod.bidiag_svals(d, e)
        assert np.all(np.diff(got) <= 0)
        assert np.max(np.abs(got - ref)) <= 1e-13 * max(ref[0], 1)
    # graded values keep high relative accuracy
    d = 10.0 ** -np.arange(0, 12)
    e = 1e-3 * d[:-1]
    got = oracle_mod.bidiag_svals(d, e, rel_tol=1e-30)
    ref = sl.svdvals(np.diag(d) + np.diag(e, 1))
    assert np.max(np.abs(got - ref) / ref) < 1e-10


@pytest.mark.parametrize("dt,b,nt", [(np.float32, 16, 4), (np.float32, 16, 7), (np.float64, 32, 4)])
def test_end_to_end_vs_lapack(oracle_mod, dt, b, nt):
    """my_CU_svdval restated ~= LAPACK svdvals (CUDAbasedSVD/test.jl:9-13, integer-valued input)."""
    n = b * nt
    a = np.random.default_rng(n).integers(1, 11, size=(n, n)).astype(dt)
    got = oracle_mod.svdvals(a, b)
    ref = sl.svdvals(a.astype(np.float64))
    assert julia_approx(got, ref, RTOL[dt])


def test_not_implemented_cases(oracle_mod):
    a = np.ones((64, 64))
    for b in (8, 24, 48):   # < 16, not a power of two, not dividing
        with pytest.raises(NotImplementedError):
            oracle_mod.svdvals(a, b)
    with pytest.raises(NotImplementedError):
        oracle_mod.svdvals(np.ones((64, 32)), 16)


def test_golden_fixtures(oracle_mod):
    """The oracle reproduces the committed fixtures (bitwise for the stage
    outputs: same code, same inputs) and stays within tolerance of LAPACK."""
    O = oracle_mod
    g = np.load(GOLDEN)
    for b, dt in ((16, "float64"), (32, "float32")):
        key = "tile_b%d_%s" % (b, dt)
        f, tau = O.geqrt(g[key + "_geqrt_in"])
        np.testing.assert_array_equal(f, g[key + "_geqrt_factors"])
        np.testing.assert_array_equal(tau, g[key + "_geqrt_tau"])
        r, v, tau2 = O.tsqrt(g[key + "_tsqrt_in"][:b], g[key + "_tsqrt_in"][b:])
        np.testing.assert_array_equal(v, g[key + "_tsqrt_v"])
        np.testing.assert_array_equal(tau2, g[key + "_tsqrt_tau"])
        rt = RTOL[np.dtype(dt).type]
        assert julia_approx(g[key + "_geqrt_factors"], g[key + "_lapack_geqrt_factors"], rt)
    names = sorted({k[: -len("_A")] for k in g.files if k.endswith("_A")})
    assert len(names) == 5
    for name in names:
        a = g[name + "_A"]
        b = int(g[name + "_tile"])
        band = O.blockbidiag(a, b)
        np.testing.assert_array_equal(O.extract_band(band, b), g[name + "_band"])
        s = O.svdvals(a, b)
        np.testing.assert_allclose(s, g[name + "_sigma_oracle"], rtol=0, atol=1e-14 * s[0])
        rt = 1e-5 if a.dtype == np.float32 else 1e-12
        assert np.max(np.abs(s - g[name + "_sigma_lapack"])) <= rt * s[0]


def test_gebd2_oracle_relations():
    """The numpy restatement of LAPACK's bidiagonal reduction, pinned by the
    relations that define it (no golden vectors exist for gebrd): the
    bidiagonal carries the singular values; with V e1 = e1, B^T B = V^T A^T A V
    has (1,1) entry ||a_1||^2 = d_1^2, and ||A^T a_1||^2 = d_1^2 (d_1^2 + e_1^2)."""
    import numpy as np
    from oracle import gebrd
    rng = np.random.default_rng(12)
    for n in (2, 7, 64):
        a = rng.standard_normal((n, n))
        d, e = gebrd.gebd2(a)
        b = np.diag(d) + np.diag(e, 1)
        np.testing.assert_allclose(np.linalg.svd(b, compute_uv=False), np.linalg.svd(a, compute_uv=False),
                                   rtol=1e-12, atol=1e-12)
        assert abs(abs(d[0]) - np.linalg.norm(a[:, 0])) < 1e-12 * np.linalg.norm(a)
        if n > 1:
            # (A^T A) e1 = V (B^T B) e1 and V e1 = e1: ||A^T a_1||^2 = d1^2 (d1^2 + e1^2)
            lhs = np.linalg.norm(a.T @ a[:, 0]) ** 2
            assert abs(lhs - d[0] ** 2 * (d[0] ** 2 + e[0] ** 2)) < 1e-10 * lhs
    # a zero column gives an identity reflector
    d, e = gebrd.gebd2(np.zeros((3, 3)))
    assert not np.any(d) and not np.any(e)


def test_rmt_oracle_statistics_shape():
    import numpy as np
    from oracle import gebrd
    rng = np.random.default_rng(1)
    x = rng.standard_normal((3, 4, 8, 8))
    m, c, times = gebrd.mou_process_covar(x + np.swapaxes(x, 2, 3), 0.05, 2)
    assert m.shape == (4,) and c.shape == (4,) and np.allclose(times, np.arange(4) * 0.0125)
    assert np.all(m > 0)


def test_oracle_bisection_vs_lapack_bdsdc(oracle_mod):
    """Stage 3 pinned to the routine the reference calls: LAPACK dbdsdc('U','N')
    (bulgechasing.jl:50-53) from the OpenBLAS scipy bundles."""
    from oracle import lapack
    if not lapack.available():
        pytest.skip("scipy's OpenBLAS LAPACKE symbols not found")
    rng = np.random.default_rng(21)
    for n in (1, 2, 7, 100, 500):
        d = rng.standard_normal(n)
        e = rng.standard_normal(max(n - 1, 0))
        ref = lapack.bdsdc(d, e)
        got = oracle_mod.bidiag_svals(d, e)
        assert np.max(np.abs(got - ref)) <= 1e-13 * max(ref[0], 1)
    # graded: both keep relative accuracy
    d = 10.0 ** -np.arange(0, 12)
    e = 1e-3 * d[:-1]
    ref = lapack.bdsdc(d, e)
    assert np.max(np.abs(oracle_mod.bidiag_svals(d, e, rel_tol=1e-30) - ref) / ref) < 1e-10


def test_gbbrd_comparator_relations():
    """LAPACK dgbbrd (the reference BRD code's comparator, bulgechasing2.jl:142-170)
    gives the Golub-Kahan bidiagonal of the band: the gebd2 oracle's up to signs."""
    from oracle import gebrd, lapack
    if not lapack.available():
        pytest.skip("scipy's OpenBLAS LAPACKE symbols not found")
    rng = np.random.default_rng(22)
    for n, bw in ((40, 4), (200, 16), (256, 64)):
        a = rng.standard_normal((n, n))
        band = np.triu(a) - np.triu(a, bw + 1)
        d, e = lapack.gbbrd(band, bw)
        dg, eg = gebrd.gebd2(band)
        k = min(20, n - 1)
        assert np.max(np.abs(np.abs(d[:k]) - np.abs(dg[:k]))) < 1e-12 * np.linalg.norm(band, 2)
        assert np.max(np.abs(np.abs(e[:k]) - np.abs(eg[:k]))) < 1e-12 * np.linalg.norm(band, 2)
        ref = np.linalg.svd(band, compute_uv=False)
        np.testing.assert_allclose(lapack.bdsdc(d, e), ref, rtol=0, atol=1e-13 * ref[0])


@pytest.mark.parametrize("n,bw", [(160, 4), (160, 16), (256, 64), (512, 16)])
def test_brd_hierarchical_reduction(n, bw):
    """The reference's hierarchical band reduction (BRD bidiag!, factor 4),
    restated: the result is exactly bidiagonal, keeps the singular values
    (its own test, bulgechasing2.jl:101-116), and its bidiagonal is the
    Golub-Kahan one (right transforms never touch column 1): |d|, |e| equal
    gebd2's."""
    from oracle import brd, gebrd
    rng = np.random.default_rng(n + bw)
    a = np.triu(np.tril(rng.random((n, n)), bw))
    s = brd.bidiag(a, bw)
    off = s.copy()
    off[np.arange(n), np.arange(n)] = 0
    off[np.arange(n - 1), np.arange(1, n)] = 0
    assert not np.any(off)
    ref = np.linalg.svd(a, compute_uv=False)
    assert np.max(np.abs(np.linalg.svd(s, compute_uv=False) - ref)) < 1e-12 * ref[0]
    dg, eg = gebrd.gebd2(a)
    k = 16
    assert np.max(np.abs(np.abs(np.diag(s)[:k]) - np.abs(dg[:k]))) < 1e-12 * ref[0]
    assert np.max(np.abs(np.abs(np.diag(s, 1)[:k]) - np.abs(eg[:k]))) < 1e-12 * ref[0]


def test_brd_short_propagation_range():
    """Documented divergence: at n = 64, bandwidth 4, the reference's
    propagation range 0:n stops the last kernels early and the values are
    wrong; running every kernel to the end (iters = 4n) gives them exactly."""
    from oracle import brd
    rng = np.random.default_rng(0)
    a = np.triu(np.tril(rng.random((64, 64)), 4))
    ref = np.linalg.svd(a, compute_uv=False)
    short = np.linalg.svd(brd.bidiag(a, 4), compute_uv=False)
    full = np.linalg.svd(brd.bidiag(a, 4, iters=4 * 64), compute_uv=False)
    assert np.max(np.abs(short - ref)) > 1e-6 * ref[0]
    assert np.max(np.abs(full - ref)) < 1e-12 * ref[0]


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,b", [(64, 16), (128, 32), (256, 64)])
def test_blockbidiag_reflectors_rebuild_q_p(oracle_mod, dt, n, b):
    """The Householder vectors and tau that the tile factorisations leave
    (QRkernels.jl:3-129 on the Blockbidiag! schedule, tiledalgos.jl:17-59)
    rebuild Q and P with A = Q B P^T: backward error and loss of
    orthogonality within n * eps of the element type.  Keeping the vectors
    does not change the band."""
    from oracle import reflectors
    a = np.random.default_rng(n + b).standard_normal((n, n)).astype(dt)
    out, tq, tp = oracle_mod.blockbidiag_keep(a, b)
    assert np.array_equal(oracle_mod.extract_band(out, b), oracle_mod.extract_band(oracle_mod.blockbidiag(a, b), b))
    back, oq, op = reflectors.checks(a, out, tq, tp, b)
    eps = np.finfo(dt).eps
    assert back < n * eps and oq < n * eps and op < n * eps, (back, oq, op)


@pytest.mark.parametrize("n,b", [(128, 32), (256, 64), (256, 128)])
def test_cpu_band_bidiagonal_restatement(oracle_mod, n, b):
    """The timed CPU baseline's stage 1 -- BandBidiagonal!(onGPU=false),
    CUDAbasedSVD/SVD_GPU.jl:176-214, LAPACK dgeqrt/dgemqrt on stacked tile
    pairs -- keeps the singular values and gives the band of Blockbidiag! up
    to the signs of rows and columns (QR and LQ factors are unique up to
    signs); the three timed stages return LAPACK's singular values."""
    from oracle import cpu_baseline, lapack
    if not lapack.available() or lapack._sym("dgeqrt") is None:
        pytest.skip("LAPACKE dgeqrt/dgemqrt not in scipy's OpenBLAS")
    a = np.random.default_rng(n + b).standard_normal((n, n))
    band = cpu_baseline.band_bidiagonal(a, b)
    i, j = np.indices(band.shape)
    assert not np.any(band[(j - i < 0) | (j - i > b)])
    ref = oracle_mod.extract_band(oracle_mod.blockbidiag(a, b), b)
    assert np.max(np.abs(np.abs(band) - np.abs(ref))) / np.max(np.abs(ref)) < 1e-12
    s = sl.svdvals(a)
    assert np.max(np.abs(sl.svdvals(band) - s)) / s[0] < 1e-13
    sig, ts = cpu_baseline.run(a.astype(np.float32), b)
    s32 = sl.svdvals(a.astype(np.float32).astype(np.float64))
    assert np.max(np.abs(sig - s32)) / s32[0] < 1e-12
    assert set(ts) == {"stage1", "stage2", "stage3"} and min(ts.values()) >= 0


@pytest.mark.parametrize("n,cbw,tbw", [(96, 32, 8), (200, 64, 16), (256, 64, 16), (300, 128, 32)])
def test_brd_stage_reduces_band(n, cbw, tbw):
    """One stage of the BRD bidiag! restatement (oracle/brd.py ``stage``, the
    parity reference of the GPU band reduction): the result is an upper band
    of width tbw exactly (zeros elsewhere), with the singular values of the
    input band (LAPACK), and running the stages cbw -> tbw -> 1 gives the
    bidiagonal of ``bidiag`` with the same values."""
    import scipy.linalg as sl
    from oracle import brd
    rng = np.random.default_rng(n + cbw)
    a = np.triu(np.tril(rng.standard_normal((n, n)), cbw))
    b = brd.stage(a, cbw, tbw)
    i, j = np.indices(b.shape)
    assert np.max(np.abs(b[(j - i > tbw) | (j < i)])) == 0.0
    s = sl.svdvals(a)
    assert np.max(np.abs(sl.svdvals(b) - s)) <= 1e-12 * s[0]
    c = brd.stage(b, tbw, 1)
    assert np.max(np.abs(c[(j - i > 1) | (j < i)])) == 0.0
    assert np.max(np.abs(sl.svdvals(c) - s)) <= 1e-12 * s[0]
