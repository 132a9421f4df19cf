"""GPU tests of the out-of-core forms (OOC_Bidiag!, OOC_SVD!, OOC_QR!;
KAbasedSVD/src/tiledalgos.jl:232-260): the matrix stays in host memory and
passes through a small device budget in slabs.  The slabs run the in-core
kernels in the in-core order, so the result equals the in-core device result
bit for bit; every form is also checked against LAPACK.  Budgets are chosen with the planner so that the
runs cover one-tile slabs, uneven last slabs and the in-core tail."""
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


def budget_for(avs_mod, n, tile, dtype, slab):
    """Smallest device budget whose plan has `slab` tile rows per slab."""
    lo, hi = 1 << 10, 1 << 40
    while lo < hi:
        mid = (lo + hi) // 2
        if avs_mod.ooc_plan(n, tile, dtype, mid)[0] >= slab:
            hi = mid
        else:
            lo = mid + 1
    assert avs_mod.ooc_plan(n, tile, dtype, lo)[0] == slab
    return lo


def gaussian(n, dtype, seed):
    a = np.random.default_rng(seed).standard_normal((n, n)) / np.sqrt(n)
    return np.asfortranarray(a.astype(dtype))


def band_svals(a, tile):
    m = np.triu(a.astype(np.float64)) - np.triu(a.astype(np.float64), tile + 1)
    return np.linalg.svd(m, compute_uv=False)


@pytest.mark.parametrize("tile,slab", [(16, 1), (32, 1), (32, 3), (64, 2), (128, 2), (256, 2)])
def test_ooc_bidiag_equals_incore(avs_mod, torch_cuda, tile, slab):
    n = {128: 8, 256: 12}.get(tile, 16) * tile
    a = gaussian(n, np.float32, tile + slab)
    ref = sl.svdvals(a.astype(np.float64))
    dev = avs_mod.to_device(a)
    avs_mod.Blockbidiag(dev, tile)
    incore = avs_mod.from_device(dev)
    budget = budget_for(avs_mod, n, tile, np.float32, slab)
    _, _, tail = avs_mod.ooc_plan(n, tile, np.float32, budget)
    assert 0 < tail < n // tile  # slabs first, then the in-core tail
    r = avs_mod.OOC_Bidiag(a, tile, device_bytes=budget)
    assert r.workspace_bytes > 0
    assert np.array_equal(a, incore)
    assert np.max(np.abs(band_svals(a, tile) - ref)) / ref[0] < 1e-5


@pytest.mark.parametrize("tile,slab", [(32, 2), (128, 1)])
def test_ooc_bidiag_equals_incore_fp64(avs_mod, torch_cuda, tile, slab):
    n = 8 * tile
    a = gaussian(n, np.float64, 3 * tile)
    dev = avs_mod.to_device(a)
    avs_mod.Blockbidiag(dev, tile)
    incore = avs_mod.from_device(dev)
    avs_mod.OOC_Bidiag(a, tile, device_bytes=budget_for(avs_mod, n, tile, np.float64, slab))
    assert np.array_equal(a, incore)


@pytest.mark.parametrize("dtype,tol", [(np.float32, 1e-5), (np.float64, 1e-12)])
@pytest.mark.parametrize("tile", [32, 128, 256])
def test_ooc_svd_matches_lapack(avs_mod, torch_cuda, dtype, tol, tile):
    n = 8 * tile if tile < 256 else 1536
    a = gaussian(n, dtype, 7 * tile)
    ref = sl.svdvals(a.astype(np.float64))
    budget = budget_for(avs_mod, n, tile, dtype, 2)
    sig = avs_mod.OOC_SVD(a, tile, device_bytes=budget)
    assert sig.dtype == dtype and np.all(np.diff(sig) <= 0)
    assert np.max(np.abs(sig.astype(np.float64) - ref)) / ref[0] < tol
    # the band left in A carries the same values
    assert np.max(np.abs(band_svals(a, tile) - ref)) / ref[0] < 10 * tol


def test_ooc_svd_geometric_spectrum_fp64(avs_mod, torch_cuda):
    """Ill-conditioned FP64 input (sigma from 1 to 1e-6), normwise 1e-12."""
    from avs import workloads
    a, s = workloads.geometric_spectrum(512, 2, 3, 1e-6)
    a = np.asfortranarray(a)
    sig = avs_mod.OOC_SVD(a, 64, device_bytes=budget_for(avs_mod, 512, 64, np.float64, 1))
    assert np.max(np.abs(sig - s)) / s[0] < 1e-12


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ooc_qr_equals_incore(avs_mod, torch_cuda, dtype):
    tile, n = 32, 512
    a = gaussian(n, dtype, 99)
    dev = avs_mod.to_device(a)
    tau_in = avs_mod.tiled_QR(dev, tile).cpu().numpy()
    incore = avs_mod.from_device(dev)
    tau = avs_mod.OOC_QR(a, tile, device_bytes=budget_for(avs_mod, n, tile, dtype, 3))
    assert np.array_equal(a, incore)
    nt = n // tile
    for k in range(nt):  # tau of panel k, tile rows k.. (the rest is unused)
        seg = slice((k * nt + k) * tile, (k * nt + nt) * tile)
        assert np.array_equal(tau[seg], tau_in[seg])
    r = np.triu(a.astype(np.float64))
    d = np.sign(np.diag(r))
    ref = np.triu(sl.qr(gaussian(n, np.float64, 99), mode="r")[0])
    dr = np.sign(np.diag(ref))
    tol = 1e-12 if dtype == np.float64 else 2e-5
    assert np.max(np.abs(r * d[:, None] - ref * dr[:, None])) / np.max(np.abs(ref)) < tol


def test_ooc_whole_matrix_in_budget(avs_mod, torch_cuda):
    """A budget that holds the whole matrix runs it in core from step 0."""
    a = gaussian(256, np.float32, 5)
    ref = sl.svdvals(a.astype(np.float64))
    assert avs_mod.ooc_plan(256, 32, np.float32, 64 << 20)[2] == 0
    sig = avs_mod.OOC_SVD(a, 32, device_bytes=64 << 20)
    assert np.max(np.abs(sig - ref)) / ref[0] < 1e-5


def test_ooc_errors(avs_mod, torch_cuda):
    a = gaussian(256, np.float32, 1)
    with pytest.raises(avs_mod.AvsError):  # below one slab
        avs_mod.OOC_SVD(a, 32, device_bytes=4096)
    with pytest.raises(NotImplementedError):
        avs_mod.OOC_SVD(gaussian(96, np.float32, 1), 64)
    with pytest.raises(TypeError):  # in place needs a Fortran-ordered array
        avs_mod.OOC_SVD(np.ascontiguousarray(a), 32)
