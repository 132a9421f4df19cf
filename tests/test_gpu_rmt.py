"""GPU tests of the batched bidiagonal output and of the random-matrix
sampling client built on it (RMT/rmt.jl:9-36).  The bidiagonal with V e1 = e1
is unique up to signs, so |d| and |e| are compared with a restatement of
LAPACK's Householder bidiagonalization (gebd2, FP64) on the same matrices; the
client's statistics are compared with the oracle's on the same noise."""
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


@pytest.mark.parametrize("n,tile", [(64, 16), (128, 32), (96, 32), (256, 64)])
def test_bidiag_batched_matches_gebd2(avs_mod, torch_cuda, n, tile):
    from oracle import gebrd
    rng = np.random.default_rng(n + tile)
    hosts = [rng.standard_normal((n, n)).astype(np.float32) for _ in range(5)]
    outs = avs_mod.bidiag_batched([avs_mod.to_device(a) for a in hosts], tiles=tile)
    for a, (d, e) in zip(hosts, outs):
        d, e = d.cpu().numpy(), e.cpu().numpy()
        assert e[-1] == 0.0
        dr, er = gebrd.gebd2(a)
        scale = np.linalg.norm(a.astype(np.float64), 2)
        lead = 16  # the leading entries (the ones the sampling client reads) are well determined
        assert np.max(np.abs(np.abs(d[:lead]) - np.abs(dr[:lead]))) / scale < 2e-5
        assert np.max(np.abs(np.abs(e[:lead]) - np.abs(er[:lead]))) / scale < 2e-5
        # the whole bidiagonal carries the singular values of A
        sv = np.linalg.svd(np.diag(d) + np.diag(e[:-1], 1), compute_uv=False)
        ref = sl.svdvals(a.astype(np.float64))
        assert np.max(np.abs(sv - ref)) / ref[0] < 1e-5


def test_bidiag_equals_svdvals_path(avs_mod, torch_cuda):
    """The bidiagonal form and the singular-value form share stages 1 and 2."""
    rng = np.random.default_rng(3)
    devs = [avs_mod.to_device(rng.standard_normal((128, 128)).astype(np.float32)) for _ in range(4)]
    outs = avs_mod.bidiag_batched(devs, tiles=32)
    sig = avs_mod.svdvals_batched(devs, tiles=32)
    for (d, e), s in zip(outs, sig):
        b = np.diag(d.cpu().numpy()) + np.diag(e.cpu().numpy()[:-1], 1)
        sv = np.linalg.svd(b, compute_uv=False)
        assert np.max(np.abs(sv - s.double().cpu().numpy())) / sv[0] < 1e-6


@pytest.mark.parametrize("n,k", [(25, 1), (32, 10), (48, 3)])
def test_rmt_client_matches_oracle(avs_mod, torch_cuda, n, k):
    from avs import rmt
    from oracle import gebrd
    t, nt, tl = 6, 5, 0.05
    rng = np.random.default_rng(100 + n)
    x = rng.standard_normal((t, nt, n, n)).astype(np.float32)
    noise = x + np.swapaxes(x, 2, 3)
    m_gpu, c_gpu, times = rmt.mou_process_covar(t, n, nt, tl, k, noise=noise, chunk=7, dtype="float32")
    m_ref, c_ref, times_ref = gebrd.mou_process_covar(noise, tl, k)
    np.testing.assert_allclose(times, times_ref)
    np.testing.assert_allclose(m_gpu, m_ref, rtol=1e-4)
    np.testing.assert_allclose(c_gpu, c_ref, rtol=1e-3, atol=1e-3)


def test_rmt_client_seeded(avs_mod, torch_cuda):
    from avs import rmt
    a = rmt.mou_process_covar(8, 100, 4, 0.05, 1, seed=11)
    b = rmt.mou_process_covar(8, 100, 4, 0.05, 1, seed=11)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # d_1^2 of G/sqrt(2) (G = X + X^T) is the squared norm of its first column:
    # mean about 2 (n - 1) / 2 + 2 = n + 1 for N(0,1) entries
    assert 0.5 * 101 < a[0][0] < 1.5 * 101
    with pytest.raises(ValueError):
        rmt.mou_process_covar(2, 16, 2, 0.05, 17)


@pytest.mark.parametrize("n,tile", [(64, 16), (128, 32), (256, 64)])
def test_bidiag_batched_fp64_matches_gebd2(avs_mod, torch_cuda, n, tile):
    """The Float64 batched bidiagonal (FP64 throughout, the reference's type
    for gebrd!, RMT/rmt.jl:23,28) matches gebd2 to FP64 rounding."""
    from oracle import gebrd
    rng = np.random.default_rng(7 * n + tile)
    hosts = [rng.standard_normal((n, n)) for _ in range(4)]
    outs = avs_mod.bidiag_batched([avs_mod.to_device(a) for a in hosts], tiles=tile)
    for a, (d, e) in zip(hosts, outs):
        d, e = d.cpu().numpy(), e.cpu().numpy()
        dr, er = gebrd.gebd2(a)
        scale = np.linalg.norm(a, 2)
        lead = 16
        assert np.max(np.abs(np.abs(d[:lead]) - np.abs(dr[:lead]))) / scale < 1e-12
        assert np.max(np.abs(np.abs(e[:lead]) - np.abs(er[:lead]))) / scale < 1e-12
        sv = np.linalg.svd(np.diag(d) + np.diag(e[:-1], 1), compute_uv=False)
        ref = sl.svdvals(a)
        assert np.max(np.abs(sv - ref)) / ref[0] < 1e-12


@pytest.mark.parametrize("n,k", [(25, 1), (48, 3)])
def test_rmt_client_fp64_matches_oracle(avs_mod, torch_cuda, n, k):
    """The sampling client in Float64 (its default, as the reference) against
    the oracle on the same noise."""
    from avs import rmt
    from oracle import gebrd
    t, nt, tl = 5, 4, 0.05
    rng = np.random.default_rng(300 + n)
    x = rng.standard_normal((t, nt, n, n))
    noise = x + np.swapaxes(x, 2, 3)
    m_gpu, c_gpu, _ = rmt.mou_process_covar(t, n, nt, tl, k, noise=noise, chunk=7, dtype="float64")
    m_ref, c_ref, _ = gebrd.mou_process_covar(noise, tl, k)
    np.testing.assert_allclose(m_gpu, m_ref, rtol=1e-10)
    np.testing.assert_allclose(c_gpu, c_ref, rtol=1e-8, atol=1e-10)
