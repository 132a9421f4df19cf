"""GPU tests of the batched path (many independent matrices of mixed orders in
one call): every matrix's values equal those of the single-matrix call on the
same input (same kernels, batch-invariant arithmetic), agree with LAPACK
within the FP32 tolerance, and do not depend on the other matrices of the
call.  The workload shape follows the many-small-SVDs client of the reference
(RMT/rmt.jl:9-36)."""
import numpy as np
import pytest
import scipy.linalg as sl

pytestmark = pytest.mark.gpu

TOL32 = 1e-5


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


def _mats(avs_mod, sizes, seed):
    rng = np.random.default_rng(seed)
    hosts = [(rng.standard_normal((n, n)) / np.sqrt(n)).astype(np.float32) for n in sizes]
    return hosts, [avs_mod.to_device(a) for a in hosts]


@pytest.mark.parametrize("tile", [16, 32, 64])
def test_batched_equals_single(avs_mod, torch_cuda, tile):
    sizes = [64, 128, 64, 256, 128, 64, 192, 256]
    sizes = [n for n in sizes if n % tile == 0]
    hosts, devs = _mats(avs_mod, sizes, 11 + tile)
    outs = avs_mod.svdvals_batched(devs, tiles=tile)
    for a, d, o in zip(hosts, devs, outs):
        single = avs_mod.my_CU_svdval(d, tile).cpu().numpy()
        got = o.cpu().numpy()
        assert np.array_equal(got, single), rel_err(got, single)
        ref = sl.svdvals(a.astype(np.float64))
        assert rel_err(got, ref) < TOL32
        assert np.all(np.diff(got) <= 0)


def test_batched_tile128(avs_mod, torch_cuda):
    """Tiles >= 128 take the full compact-WY update in the batch too."""
    sizes = [256, 512, 256]
    hosts, devs = _mats(avs_mod, sizes, 77)
    outs = avs_mod.svdvals_batched(devs, tiles=128)
    for a, d, o in zip(hosts, devs, outs):
        got = o.cpu().numpy()
        assert np.array_equal(got, avs_mod.my_CU_svdval(d, 128).cpu().numpy())
        assert rel_err(got, sl.svdvals(a.astype(np.float64))) < TOL32


@pytest.mark.parametrize("n,tile,count", [(512, 32, 64), (512, 64, 64), (1024, 128, 40)])
def test_batched_large_batch_copies(avs_mod, torch_cuda, n, tile, count):
    """Many copies of one matrix in one call: every copy gives the single
    call's values bit for bit.  With this many CTAs the panel kernels of
    different matrices share SMs, so warps of one CTA drift apart in time."""
    hosts, devs = _mats(avs_mod, [n], 300 + tile)
    copies = [devs[0].clone() for _ in range(count)]
    outs = avs_mod.svdvals_batched(copies, tiles=tile)
    single = avs_mod.my_CU_svdval(devs[0], tile).cpu().numpy()
    for o in outs:
        assert np.array_equal(o.cpu().numpy(), single), rel_err(o.cpu().numpy(), single)
    assert rel_err(single, sl.svdvals(hosts[0].astype(np.float64))) < TOL32


@pytest.mark.parametrize("tile,count", [(32, 160), (64, 320)])
def test_batched_wide_batch_equals_single(avs_mod, torch_cuda, tile, count):
    """A batch wide enough for the small-CTA chase (many sweeps per SM) gives
    each matrix the single call's values bit for bit."""
    hosts, devs = _mats(avs_mod, [256] * 4, 900 + tile)
    mats = [devs[i % 4].clone() for i in range(count)]
    outs = avs_mod.svdvals_batched(mats, tiles=tile)
    for i in range(4):
        single = avs_mod.my_CU_svdval(devs[i], tile).cpu().numpy()
        for o in outs[i::4]:
            assert np.array_equal(o.cpu().numpy(), single), rel_err(o.cpu().numpy(), single)
        assert rel_err(single, sl.svdvals(hosts[i].astype(np.float64))) < TOL32


def test_batched_large_batch_distinct(avs_mod, torch_cuda):
    """48 distinct matrices of order 512, tile 64: each within the FP32
    tolerance of LAPACK."""
    hosts, devs = _mats(avs_mod, [512] * 48, 404)
    outs = avs_mod.svdvals_batched(devs, tiles=64)
    for a, o in zip(hosts, outs):
        assert rel_err(o.cpu().numpy(), sl.svdvals(a.astype(np.float64))) < TOL32


def test_batched_solo_vs_mix(avs_mod, torch_cuda):
    """A matrix gives bit-identical values alone and inside a mixed batch."""
    hosts, devs = _mats(avs_mod, [128, 64, 128, 256, 128, 64], 5)
    mix = avs_mod.svdvals_batched(devs, tiles=[32, 32, 64, 32, 32, 16])
    for i, d in enumerate(devs):
        tile = [32, 32, 64, 32, 32, 16][i]
        solo = avs_mod.svdvals_batched([d], tiles=tile)[0]
        assert torch_cuda.equal(solo, mix[i])


def test_batched_autotune(avs_mod, torch_cuda):
    h = avs_mod.Handle()
    try:
        t = avs_mod.autotune_tile(256, sample=8, handle=h)
        assert t in (32, 64, 128)
        hosts, devs = _mats(avs_mod, [256, 128, 256], 9)
        outs = avs_mod.svdvals_batched(devs, tiles=None, handle=h)
        for a, o in zip(hosts, outs):
            assert rel_err(o.cpu().numpy(), sl.svdvals(a.astype(np.float64))) < TOL32
    finally:
        h.close()


def test_batched_graph_replay_and_report(avs_mod, torch_cuda):
    """Repeated calls replay the captured graphs and give the same values; the
    report counts the kernels of every group."""
    hosts, devs = _mats(avs_mod, [64, 128, 64], 3)
    r = avs_mod.Report()
    first = avs_mod.svdvals_batched(devs, tiles=32, report=r)
    assert r.kernel_launches > 0 and r.t_total_ms > 0
    second = avs_mod.svdvals_batched(devs, tiles=32)
    for x, y in zip(first, second):
        assert torch_cuda.equal(x, y)


def test_batched_edge_cases(avs_mod, torch_cuda):
    assert avs_mod.svdvals_batched([]) == []
    _, devs = _mats(avs_mod, [96], 1)
    with pytest.raises(NotImplementedError):
        avs_mod.svdvals_batched(devs, tiles=64)  # 64 does not divide 96
    with pytest.raises(NotImplementedError):
        avs_mod.svdvals_batched(devs, tiles=24)  # not a power of two
    rect = torch_cuda.zeros((64, 32), device="cuda", dtype=torch_cuda.float32)
    with pytest.raises(NotImplementedError):
        avs_mod.svdvals_batched([rect], tiles=16)
    z = torch_cuda.zeros((64, 64), device="cuda", dtype=torch_cuda.float32)
    out = avs_mod.svdvals_batched([z], tiles=16)[0]
    assert torch_cuda.count_nonzero(out).item() == 0


@pytest.mark.parametrize("tile,count", [(32, 8), (32, 140), (32, 160), (64, 8), (64, 290), (64, 320)])
def test_batched_chase_branches_repeat(avs_mod, torch_cuda, tile, count):
    """Order 256 at bands 32 and 64 with batch sizes on both sides of the
    threshold at which the batched chase switches to small CTAs (batch x
    (n / bw) / 2 >= 4 x SMs): both branches, called three times, give every
    matrix the single call's values bit for bit."""
    hosts, devs = _mats(avs_mod, [256] * 4, 1200 + tile + count)
    singles = [avs_mod.my_CU_svdval(d, tile).cpu().numpy() for d in devs]
    for rep in range(3):
        mats = [devs[i % 4].clone() for i in range(count)]
        outs = avs_mod.svdvals_batched(mats, tiles=tile)
        for i, o in enumerate(outs):
            got = o.cpu().numpy()
            assert np.array_equal(got, singles[i % 4]), (rep, i, rel_err(got, singles[i % 4]))
    for a, s in zip(hosts, singles):
        assert rel_err(s, sl.svdvals(a.astype(np.float64))) < TOL32


@pytest.mark.parametrize("tile", [16, 32, 64, 128])
def test_batched_fp64_equals_single(avs_mod, torch_cuda, tile):
    """Float64 batches run FP64 throughout: every matrix's values equal the
    single FP64 call's bit for bit and LAPACK's within 1e-12 (normwise)."""
    sizes = [n for n in [64, 128, 256, 128, 512, 256, 64] if n % tile == 0 and n // tile >= 1]
    rng = np.random.default_rng(2000 + tile)
    hosts = [rng.standard_normal((n, n)) / np.sqrt(n) for n in sizes]
    devs = [avs_mod.to_device(a) for a in hosts]
    r = avs_mod.Report()
    outs = avs_mod.svdvals_batched(devs, tiles=tile, report=r)
    assert r.precision == 1  # AVS_PREC_FP64
    for a, d, o in zip(hosts, devs, outs):
        assert o.dtype == torch_cuda.float64
        got = o.cpu().numpy()
        single = avs_mod.my_CU_svdval(d, tile).cpu().numpy()
        assert np.array_equal(got, single), rel_err(got, single)
        assert rel_err(got, sl.svdvals(a)) < 1e-12


@pytest.mark.parametrize("tile,count", [(32, 4), (32, 160), (64, 320)])
def test_batched_fp64_chase_branches(avs_mod, torch_cuda, tile, count):
    """FP64 batches on both sides of the small-CTA threshold equal the single
    call bit for bit."""
    rng = np.random.default_rng(3000 + tile + count)
    hosts = [rng.standard_normal((256, 256)) / 16.0 for _ in range(4)]
    devs = [avs_mod.to_device(a) for a in hosts]
    singles = [avs_mod.my_CU_svdval(d, tile).cpu().numpy() for d in devs]
    outs = avs_mod.svdvals_batched([devs[i % 4].clone() for i in range(count)], tiles=tile)
    for i, o in enumerate(outs):
        assert np.array_equal(o.cpu().numpy(), singles[i % 4])


def test_batched_rejects_mixed_dtypes(avs_mod, torch_cuda):
    a = avs_mod.to_device(np.eye(64, dtype=np.float32))
    b = avs_mod.to_device(np.eye(64))
    with pytest.raises(TypeError):
        avs_mod.svdvals_batched([a, b], tiles=16)
