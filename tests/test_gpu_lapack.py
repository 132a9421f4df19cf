"""GPU stages 2 and 3 against the LAPACK routines the reference uses around
them: dgbbrd (band -> bidiagonal; the reference BRD code's comparator,
BRD/src/bulgechasing2.jl:142-170) and dbdsdc('U','N') (the reference's
diag_lapack, bulgechasing.jl:50-53), both from the OpenBLAS scipy bundles.
The bidiagonal of a band with V e1 = e1 is unique up to signs, so |d| and |e|
of the GPU chase equal dgbbrd's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def lapack():
    from oracle import lapack as lp
    if not lp.available():
        pytest.skip("scipy's OpenBLAS LAPACKE symbols not found")
    return lp


@pytest.mark.parametrize("n,bw", [(256, 16), (512, 32), (1024, 64), (1024, 128), (1536, 256)])
def test_gpu_chase_vs_dgbbrd(avs_mod, torch_cuda, lapack, n, bw):
    rng = np.random.default_rng(n + bw)
    a = rng.standard_normal((n, n))
    band = np.triu(a) - np.triu(a, bw + 1)
    d, e = avs_mod.bidiagonalize(avs_mod.to_device(band), bw)
    d, e = d.cpu().numpy(), e.cpu().numpy()
    dl, el = lapack.gbbrd(band, bw)
    scale = np.linalg.norm(band, 2)
    k = 32
    assert np.max(np.abs(np.abs(d[:k]) - np.abs(dl[:k]))) < 1e-12 * scale
    assert np.max(np.abs(np.abs(e[:k]) - np.abs(el[:k]))) < 1e-12 * scale
    # the whole bidiagonal: LAPACK's singular values of the GPU bidiagonal equal those of the band
    ref = lapack.bdsdc(dl, el)
    assert np.max(np.abs(lapack.bdsdc(d, e) - ref)) < 1e-12 * ref[0]


@pytest.mark.parametrize("n", [1, 2, 33, 1000, 4096])
def test_gpu_bisection_vs_dbdsdc(avs_mod, torch_cuda, lapack, n):
    torch = torch_cuda
    rng = np.random.default_rng(n)
    d = rng.standard_normal(n)
    e = rng.standard_normal(max(n - 1, 0))
    s = avs_mod.diag_lapack(torch.from_numpy(d).cuda(), torch.from_numpy(e).cuda()).cpu().numpy()
    ref = lapack.bdsdc(d, e)
    assert np.all(np.diff(s) <= 0)
    assert np.max(np.abs(s - ref)) <= 1e-13 * max(ref[0], 1)
