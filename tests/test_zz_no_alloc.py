"""GPU test of avs_bidiag_svals_noalloc, the entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc when they need singular
values -- a host whose device memory is owned by its own pool allocator (Julia's
CUDA.jl, PyTorch's caching allocator) or a latency-critical loop that must not
pay cudaMalloc's implicit synchronisation.  Its scratch is a static device
array inside the library, shared by every call.  This test calls it through the
C ABI twice in a row (a larger problem, then a smaller one, so stale scratch
from the first call would show) and compares each result with the allocating
entry point avs_bidiag_svals_dev, within the bisection tolerance the other GPU
tests use (1e-14 relative to sigma_max)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(avs_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = avs_mod.lib()
    h = avs_mod.Handle(0)
    rng = np.random.default_rng(2024)
    for n in (1000, 300):
        d = torch.from_numpy(rng.standard_normal(n)).cuda()
        e = torch.from_numpy(rng.standard_normal(n - 1)).cuda()
        s_ref = torch.empty(n, dtype=torch.float64, device="cuda")
        s_new = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.avs_bidiag_svals_dev(h.ptr, n, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(e.data_ptr()),
                                      ctypes.c_void_p(s_ref.data_ptr()), 0.0, None)
        assert rc == 0
        torch.cuda.synchronize()
        rc = lib.avs_bidiag_svals_noalloc(n, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(e.data_ptr()),
                                          ctypes.c_void_p(s_new.data_ptr()), 0.0, None)
        assert rc == 0
        a, b = s_new.cpu().numpy(), s_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert np.max(np.abs(a - b)) <= 1e-14 * b[0]
    h.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(avs_mod):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = avs_mod.lib()
    rc = lib.avs_bidiag_svals_noalloc(65537, None, None, None, 0.0, None)
    assert rc == 8  # AVS_ERR_TOO_LARGE
    assert b"static scratch" in lib.avs_strerror(rc)
