"""CPU tests of the C ABI: the library builds for sm_103a, loads, and exports
every function include/avs.h declares; host-side argument logic.  No compute
call is made here (there is no GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(REPO, "include", "avs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(avs_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_expected(avs_mod):
    decl = declared_functions()
    assert set(avs_mod.EXPORTED_SYMBOLS) == set(decl), set(decl) ^ set(avs_mod.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(avs_mod):
    lib = avs_mod.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert ctypes.cast(getattr(lib, name), ctypes.c_void_p).value


def test_build_targets_sm103a_only(avs_mod):
    """The build recipe compiles every translation unit for sm_103a alone."""
    from avs import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_library_needs_no_torch(avs_mod):
    """The C-ABI library's dynamic dependencies (ELF DT_NEEDED, as readelf
    prints them) include no PyTorch library."""
    import shutil
    import subprocess
    if not shutil.which("readelf"):
        pytest.skip("readelf not installed")
    out = subprocess.run(["readelf", "-d", avs_mod.library_path()], capture_output=True, text=True).stdout
    needed = re.findall(r"\(NEEDED\)\s+Shared library: \[([^\]]+)\]", out)
    assert needed, out
    assert not any(("torch" in x) or ("c10" in x) for x in needed), needed


def test_kernel_arch_without_device(avs_mod):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    bv, pv = ctypes.c_int32(0), ctypes.c_int32(0)
    assert avs_mod.lib().avs_kernel_arch(0, ctypes.byref(bv), ctypes.byref(pv)) == 5  # AVS_ERR_NO_DEVICE


def test_strerror_and_version(avs_mod):
    lib = avs_mod.lib()
    assert lib.avs_strerror(avs_mod.NOT_IMPLEMENTED) == b"Not implemented"
    assert lib.avs_strerror(0) == b"success"
    assert lib.avs_version() >= 1


def test_argument_checks_without_device(avs_mod):
    """Invalid arguments are rejected before any device work (LAPACK info style)."""
    lib = avs_mod.lib()
    r = lib.avs_svdvals_s(None, 64, 64, 64, 16, None, None, None, None)
    assert r == -1


def test_create_without_gpu_reports_no_device(avs_mod):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    rc = avs_mod.lib().avs_create(ctypes.byref(h), 0)
    assert rc == 5  # AVS_ERR_NO_DEVICE


def test_workloads_are_seeded():
    import numpy as np
    from avs import workloads
    a1 = workloads.gaussian(32, 4, 1 / np.sqrt(32))
    a2 = workloads.gaussian(32, 4, 1 / np.sqrt(32))
    assert np.array_equal(a1, a2) and a1.flags.f_contiguous
    a, s = workloads.geometric_spectrum(64, 2, 3, 1e-6)
    np.testing.assert_allclose(np.linalg.svd(a, compute_uv=False), s, rtol=1e-9, atol=1e-14)
    sz = workloads.batch_sizes(4096, 5)
    assert set(np.unique(sz)) <= {64, 128, 256, 512, 1024}


def test_estimate_bytes_host_logic(avs_mod):
    """Workspace estimates are pure host arithmetic: monotone in n and in the
    group size, and the reference's "Not implemented" rules apply."""
    e1 = avs_mod.estimate_bytes(1024, 64, "fp32", 0)
    e2 = avs_mod.estimate_bytes(2048, 64, "fp32", 0)
    assert 0 < e1 < e2
    g1 = avs_mod.estimate_bytes(256, 32, "fp32", 1)
    g8 = avs_mod.estimate_bytes(256, 32, "fp32", 8)
    assert 0 < g1 < g8 and g8 >= 8 * 256 * 256 * 4
    assert avs_mod.estimate_bytes(1024, 64, "fp64", 0) > e1
    with pytest.raises(NotImplementedError):
        avs_mod.estimate_bytes(96, 64, "fp32", 0)
    with pytest.raises(NotImplementedError):
        avs_mod.estimate_bytes(96, 24, "fp32", 0)


def test_serve_and_batched_without_gpu(avs_mod):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    lib = avs_mod.lib()
    p = ctypes.c_void_p()
    assert lib.avs_serve_create(ctypes.byref(p), None) == 5  # AVS_ERR_NO_DEVICE
    assert lib.avs_serve_submit(None, 64, 64, 0, 0, None, None, None) == -1
    assert lib.avs_svdvals_batched_dev_s(None, 1, None, None, None, None, None, None, None) == -1
    with pytest.raises(avs_mod.AvsError):
        avs_mod.Server()


def test_ooc_plan_host_logic(avs_mod):
    """The out-of-core slab plan is host arithmetic: more device memory gives
    larger slabs and an earlier in-core tail; too little gives slab 0, and the
    reference's "Not implemented" rules apply."""
    s1, b1, f1 = avs_mod.ooc_plan(4096, 64, "float32", 64 << 20)
    s2, b2, f2 = avs_mod.ooc_plan(4096, 64, "float32", 256 << 20)
    assert 1 <= s1 < s2 and b1 <= (64 << 20) and b2 <= (256 << 20)
    assert f2 <= f1 <= 4096 // 64
    assert avs_mod.ooc_plan(4096, 64, "float32", 1 << 20)[0] == 0
    s8, _, _ = avs_mod.ooc_plan(4096, 64, "float64", 64 << 20)
    assert s8 < s1
    # the whole matrix in budget: in core from the first step
    assert avs_mod.ooc_plan(1024, 64, "float32", 64 << 20)[2] == 0
    with pytest.raises(NotImplementedError):
        avs_mod.ooc_plan(96, 64, "float32", 1 << 20)
    lib = avs_mod.lib()
    assert lib.avs_ooc_plan(1024, 64, 4, 0, None, None, None) == -4
    assert lib.avs_ooc_plan(1024, 64, 2, 1 << 20, None, None, None) == -3
    assert lib.avs_blockbidiag_ooc_s(None, 64, 64, 16, None, 0, None) == -1


def test_selftest_timeout_argument_check(avs_mod):
    assert avs_mod.lib().avs_selftest_timeout(None) == -1
    assert b"CUDA runtime error" in avs_mod.lib().avs_strerror(1)


def test_serve_plan_host_logic(avs_mod):
    """The serving plan is host arithmetic: FP64 requests share batched calls
    in the double-float FP64X2 mode; FP32 requests of order >= 2048 run alone
    with the split-BF16 tensor-core update (tile 128); smaller FP32 requests
    share batched FP32 calls, tile 32 up to order 256 and 64 up to 1024."""
    assert avs_mod.serve_plan(4096, np.float64) == (128, "fp64x2", True)
    assert avs_mod.serve_plan(8192, np.float32) == (128, "bf16x3", False)
    assert avs_mod.serve_plan(2048, np.float32) == (128, "bf16x3", False)
    assert avs_mod.serve_plan(1024, np.float32) == (64, "fp32", True)
    assert avs_mod.serve_plan(256, np.float32) == (32, "fp32", True)
    assert avs_mod.serve_plan(96, np.float32)[0] == 32
    # an explicit tile is kept
    assert avs_mod.serve_plan(1024, np.float32, 128) == (128, "fp32", True)
