"""GPU tests of the tiled QR (tiled_QR!, KAbasedSVD/src/tiledalgos.jl:6-15),
after the reference's own test (KAbasedSVD/test/test_tiledalgo.jl:19-26): R
times the signs of its diagonal equals LAPACK's R times the signs of its
diagonal, for Float32 and Float64, tile sizes 16..256 and 4 or 6 tiles per
side; the tau of the first GEQRT equals the oracle's."""
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


def signed_r(r):
    d = np.sign(np.diag(r))
    d[d == 0] = 1
    return np.triu(r) * d[:, None]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("tile", [16, 32, 64, 128, 256])
@pytest.mark.parametrize("blocks", [4, 6])
def test_tiled_qr_matches_lapack_r(avs_mod, oracle_mod, torch_cuda, dt, tile, blocks):
    n = tile * blocks
    a = np.random.default_rng(tile * 10 + blocks).random((n, n)).astype(dt)
    t = avs_mod.to_device(a)
    tau = avs_mod.tiled_QR(t, tile).cpu().numpy()
    r = signed_r(avs_mod.from_device(t).astype(np.float64))
    ref = signed_r(sl.qr(a.astype(np.float64), mode="r")[0])
    tol = 1e-12 if dt == np.float64 else 2e-5
    assert np.max(np.abs(r - ref)) / np.max(np.abs(ref)) < tol
    # the first panel's GEQRT tau is the tile kernel's
    _, tau_ref = oracle_mod.geqrt(a[:tile, :tile])
    assert np.max(np.abs(tau[: tile - 1] - tau_ref[: tile - 1])) < 50 * np.finfo(dt).eps * tile


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
@pytest.mark.parametrize("tile", [128, 256])
def test_tiled_qr_tensor_core_modes(avs_mod, torch_cuda, prec, tile):
    n = 4 * tile
    a = np.random.default_rng(tile).standard_normal((n, n)).astype(np.float32)
    t = avs_mod.to_device(a)
    r = avs_mod.Report()
    avs_mod.tiled_QR(t, tile, precision=prec, report=r)
    assert r.precision == avs_mod.PREC[prec]
    got = signed_r(avs_mod.from_device(t).astype(np.float64))
    ref = signed_r(sl.qr(a.astype(np.float64), mode="r")[0])
    tol = 2e-5 if prec == "tf32x3" else 1e-4  # split BF16: ~16 significant bits per operand
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < tol


def test_tiled_qr_not_implemented(avs_mod, torch_cuda):
    t = avs_mod.to_device(np.ones((96, 96), np.float32))
    with pytest.raises(NotImplementedError):
        avs_mod.tiled_QR(t, 64)
