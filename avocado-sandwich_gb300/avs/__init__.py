"""Python host mirror of the reference's tiled singular-value entry point.

Binds ``libavs.so`` (the C-ABI library built from ``../csrc``) with ctypes and
mirrors the reference's Julia interface for this path
(evelyne-ringoot/Avocado-sandwich):

* ``my_CU_svdval(A, block_size)`` -- CUDAbasedSVD/SVD_GPU.jl:257-283: host
  (numpy) or device (CUDA torch tensor) matrix in, singular values out
  (descending).  Raises ``NotImplementedError("Not implemented")`` exactly where
  the reference calls ``error("Not implemented")`` (non-square, tile not a
  power of two, tile < 16, tile not dividing n).
* ``Blockbidiag(A, tile)`` -- Blockbidiag! on a TiledMatrix
  (KAbasedSVD/src/tiledalgos.jl:17-34, TiledMatrix.jl:41-67), in place on a
  device matrix.
* ``bidiagonalize(band, bw)`` -- KAbasedSVD/src/bulgechasing.jl:33-42 on the GPU.
* ``diag_lapack(d, e)`` -- bulgechasing.jl:50-53 (bdsdc('U','N')), by FP64
  bisection on the GPU.
* ``geqrt_tile`` / ``tsqrt_tile`` -- the tile kernels of
  KAbasedSVD/src/QRkernels.jl:3-129.

Device matrices are column-major like Julia's: a torch tensor ``t`` of shape
(n, n) stores the column-major matrix ``t.T``.  ``to_device`` / ``from_device``
convert numpy arrays.  There is no CPU fallback: every call runs the CUDA
library, and a missing library raises at import of the binding.
"""
import ctypes
import os

import numpy as np

__all__ = [
    "AvsError", "Handle", "lib", "library_path", "my_CU_svdval", "svdvals", "Blockbidiag", "extract_band",
    "bidiagonalize", "band_reduce", "diag_lapack", "geqrt_tile", "tsqrt_tile", "to_device", "from_device", "PREC",
    "NOT_IMPLEMENTED", "EXPORTED_SYMBOLS", "Report", "svdvals_batched", "autotune_tile", "Server", "tiled_QR",
    "estimate_bytes",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_HANDLES = {}

NOT_IMPLEMENTED = -100
PREC = {"default": 0, "fp64": 1, "fp32": 2, "tf32": 3, "tf32x3": 4, "bf16": 5, "bf16x3": 6, "fp64x2": 7}

EXPORTED_SYMBOLS = [
    "avs_create", "avs_destroy", "avs_reserve", "avs_strerror", "avs_version",
    "avs_svdvals_s", "avs_svdvals_d", "avs_svdvals_dev_s", "avs_svdvals_dev_d",
    "avs_blockbidiag_dev_s", "avs_blockbidiag_dev_d", "avs_blockbidiag_tau_dev_s", "avs_blockbidiag_tau_dev_d",
    "avs_extract_band_dev_s", "avs_extract_band_dev_d",
    "avs_band_to_bidiag_dev", "avs_bidiag_svals_dev", "avs_bidiag_svals_noalloc",
    "avs_band_reduce_dev_s", "avs_band_reduce_dev_d",
    "avs_geqrt_tile_dev_s", "avs_geqrt_tile_dev_d", "avs_tsqrt_tile_dev_s", "avs_tsqrt_tile_dev_d",
    "avs_svdvals_batched_dev_s", "avs_bidiag_batched_dev_s", "avs_svdvals_batched_dev_d", "avs_bidiag_batched_dev_d", "avs_autotune_tile", "avs_trim", "avs_workspace_bytes", "avs_estimate_bytes",
    "avs_geqrf_dev_s", "avs_geqrf_dev_d",
    "avs_blockbidiag_ooc_s", "avs_blockbidiag_ooc_d", "avs_svdvals_ooc_s", "avs_svdvals_ooc_d",
    "avs_geqrf_ooc_s", "avs_geqrf_ooc_d", "avs_ooc_plan", "avs_selftest_timeout", "avs_kernel_arch",
    "avs_measure_chase_rate",
    "avs_serve_create", "avs_serve_submit", "avs_serve_wait", "avs_serve_stats_get", "avs_serve_destroy",
    "avs_serve_plan",
]


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("flags", ctypes.c_int32), ("bisect_rel_tol", ctypes.c_double),
                ("stream", ctypes.c_void_p)]


class Report(ctypes.Structure):
    _fields_ = [("t_total_ms", ctypes.c_double), ("t_stage1_ms", ctypes.c_double), ("t_stage2_ms", ctypes.c_double),
                ("t_stage3_ms", ctypes.c_double), ("t_h2d_ms", ctypes.c_double), ("t_d2h_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("workspace_bytes", ctypes.c_int64),
                ("precision", ctypes.c_int32), ("status", ctypes.c_int32), ("t_update_ms", ctypes.c_double),
                ("t_band_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("workers", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("autotune", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64)]


class ServeStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("queued", ctypes.c_int64), ("batches", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("throughput_rps", ctypes.c_double), ("mean_batch", ctypes.c_double),
                ("peak_bytes", ctypes.c_int64), ("budget_bytes", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AvsError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = lib().avs_strerror(status).decode() if _LIB is not None else str(status)
        super().__init__("%s: %s (status %d)" % (what, msg, status) if what else "%s (status %d)" % (msg, status))


def library_path():
    return os.path.join(_HERE, "libavs.so")


def lib():
    """Load libavs.so (raises OSError if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise OSError("libavs.so not built: run __graft_entry__.build() (or avs/build.py)")
        L = ctypes.CDLL(path)
        P, I64, I32, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int
        OP, RP = ctypes.POINTER(Opts), ctypes.POINTER(Report)
        L.avs_create.argtypes = [ctypes.POINTER(P), I]
        L.avs_destroy.argtypes = [P]
        L.avs_reserve.argtypes = [P, I64, I32, I32]
        L.avs_strerror.argtypes = [I]
        L.avs_strerror.restype = ctypes.c_char_p
        L.avs_version.restype = I
        for nm in ("avs_svdvals_s", "avs_svdvals_d", "avs_svdvals_dev_s", "avs_svdvals_dev_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I64, I32, P, P, OP, RP]
        for nm in ("avs_blockbidiag_dev_s", "avs_blockbidiag_dev_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, OP, RP]
        for nm in ("avs_blockbidiag_tau_dev_s", "avs_blockbidiag_tau_dev_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, P, P, OP, RP]
        for nm in ("avs_extract_band_dev_s", "avs_extract_band_dev_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, P, I64]
        L.avs_band_to_bidiag_dev.argtypes = [P, I64, I32, P, I64, P, P, RP]
        for nm in ("avs_band_reduce_dev_s", "avs_band_reduce_dev_d"):
            getattr(L, nm).argtypes = [P, I64, I32, I32, P, I64, RP]
        L.avs_bidiag_svals_dev.argtypes = [P, I64, P, P, P, ctypes.c_double, RP]
        L.avs_bidiag_svals_noalloc.argtypes = [I64, P, P, P, ctypes.c_double, P]
        for sfx in ("s", "d"):
            getattr(L, "avs_svdvals_batched_dev_" + sfx).argtypes = [P, I32, P, P, P, P, P, OP, RP]
            getattr(L, "avs_bidiag_batched_dev_" + sfx).argtypes = [P, I32, P, P, P, P, P, P, OP, RP]
        L.avs_autotune_tile.argtypes = [P, I64, I32, ctypes.POINTER(ctypes.c_int32)]
        for nm in ("avs_geqrf_dev_s", "avs_geqrf_dev_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, P, OP, RP]
        for nm in ("avs_blockbidiag_ooc_s", "avs_blockbidiag_ooc_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, I64, RP]
        for nm in ("avs_svdvals_ooc_s", "avs_svdvals_ooc_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, P, I64, OP, RP]
        for nm in ("avs_geqrf_ooc_s", "avs_geqrf_ooc_d"):
            getattr(L, nm).argtypes = [P, I64, I64, I32, P, P, I64, RP]
        L.avs_ooc_plan.argtypes = [I64, I32, I32, I64, ctypes.POINTER(I32), ctypes.POINTER(I64),
                                   ctypes.POINTER(I32)]
        L.avs_trim.argtypes = [P]
        L.avs_selftest_timeout.argtypes = [P]
        L.avs_kernel_arch.argtypes = [I, ctypes.POINTER(I32), ctypes.POINTER(I32)]
        L.avs_measure_chase_rate.argtypes = [I, I32, ctypes.POINTER(ctypes.c_double)]
        L.avs_workspace_bytes.argtypes = [P, ctypes.POINTER(I64), ctypes.POINTER(I64)]
        L.avs_estimate_bytes.argtypes = [I64, I32, I32, I32, ctypes.POINTER(I64)]
        L.avs_serve_create.argtypes = [ctypes.POINTER(P), ctypes.POINTER(ServeConfig)]
        L.avs_serve_submit.argtypes = [P, I64, I64, I32, I32, P, P, ctypes.POINTER(I64)]
        L.avs_serve_wait.argtypes = [P, I64, ctypes.c_double, ctypes.POINTER(I32), ctypes.POINTER(ctypes.c_double)]
        L.avs_serve_stats_get.argtypes = [P, ctypes.POINTER(ServeStats)]
        L.avs_serve_destroy.argtypes = [P]
        L.avs_serve_plan.argtypes = [I64, I32, I32, ctypes.POINTER(I32), ctypes.POINTER(I32), ctypes.POINTER(I32)]
        for nm in ("avs_geqrt_tile_dev_s", "avs_geqrt_tile_dev_d"):
            getattr(L, nm).argtypes = [P, I32, P, P]
        for nm in ("avs_tsqrt_tile_dev_s", "avs_tsqrt_tile_dev_d"):
            getattr(L, nm).argtypes = [P, I32, P, P, P]
        for nm in EXPORTED_SYMBOLS:
            if nm not in ("avs_strerror",):
                getattr(L, nm).restype = I
        _LIB = L
    return _LIB


class Handle:
    """One avs_handle (CUDA stream + grow-only workspace) on one device."""

    def __init__(self, device=0):
        self.ptr = ctypes.c_void_p()
        rc = lib().avs_create(ctypes.byref(self.ptr), int(device))
        if rc != 0:
            raise AvsError(rc, "avs_create")
        self.device = device

    def close(self):
        if self.ptr:
            lib().avs_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, n, tile, precision="default"):
        rc = lib().avs_reserve(self.ptr, int(n), int(tile), _prec(precision))
        _check(rc, "avs_reserve")


def default_handle(device=0):
    h = _HANDLES.get(device)
    if h is None:
        h = _HANDLES[device] = Handle(device)
    return h


def _prec(p):
    if p is None:
        return 0
    if isinstance(p, str):
        return PREC[p.lower()]
    return int(p)


def _check(rc, what):
    if rc == NOT_IMPLEMENTED:
        raise NotImplementedError("Not implemented")
    if rc != 0:
        raise AvsError(rc, what)


def _is_torch_cuda(x):
    return hasattr(x, "is_cuda") and getattr(x, "is_cuda")


def to_device(a, device=0):
    """numpy (n x m) -> CUDA torch tensor holding the same matrix column-major."""
    import torch
    a = np.asarray(a)
    return torch.from_numpy(np.ascontiguousarray(a.T)).to("cuda:%d" % device)


def from_device(t):
    """Inverse of to_device: CUDA tensor holding a column-major matrix -> numpy."""
    return t.detach().cpu().numpy().T.copy()


STAGES = {"auto": 0, "fp64": 1, "df64": 2}


FLAGS = {"one_stage_chase": 4, "band32": 8, "cluster_chase": 16, "hier_chase": 32}


def my_CU_svdval(A, block_size, precision=None, report=None, handle=None, rel_tol=0.0, stages="auto", flags=0):
    """Singular values (descending) of the square matrix A with tile ``block_size``.

    ``A`` is a numpy array (the ``Matrix{Float32}`` method, host copies inside
    the call) or a CUDA torch tensor holding the matrix column-major (the
    ``CuMatrix{Float32}`` method, result returned as a CUDA tensor).  float32
    and float64 are supported; the input is never modified.  ``stages``
    selects the arithmetic of the bulge chase and the bisection: "auto" (FP64
    for the plain FP64 mode, double-float for the FP32-class modes), "fp64" or
    "df64" (AVS_FLAG_FP64_STAGES / AVS_FLAG_DF64_STAGES).
    """
    h = handle or default_handle()
    o = Opts(_prec(precision), STAGES[stages] | int(flags), float(rel_tol), None)
    r = report if report is not None else Report()
    if _is_torch_cuda(A):
        import torch
        if A.dim() != 2:
            raise NotImplementedError("Not implemented")
        if A.dtype not in (torch.float32, torch.float64):
            raise TypeError("float32 / float64 only")
        # tensor (c, r) row-major = column-major r x c matrix with ld = stride(0)
        n_rows, n_cols = A.shape[1], A.shape[0]
        if A.stride(1) != 1:
            A = A.contiguous()
        lda = max(A.stride(0), 1)
        out = torch.empty(n_cols, dtype=A.dtype, device=A.device)
        fn = lib().avs_svdvals_dev_d if A.dtype == torch.float64 else lib().avs_svdvals_dev_s
        o.stream = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
        rc = fn(h.ptr, n_rows, n_cols, lda, int(block_size), ctypes.c_void_p(A.data_ptr()),
                ctypes.c_void_p(out.data_ptr()), ctypes.byref(o), ctypes.byref(r))
        _check(rc, "avs_svdvals_dev")
        return out
    a = np.asarray(A)
    if a.ndim != 2:
        raise NotImplementedError("Not implemented")
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float32)
    a = np.asfortranarray(a)
    m, n = a.shape
    out = np.empty(n, dtype=a.dtype)
    fn = lib().avs_svdvals_d if a.dtype == np.float64 else lib().avs_svdvals_s
    rc = fn(h.ptr, m, n, max(m, 1), int(block_size), ctypes.c_void_p(a.ctypes.data),
            ctypes.c_void_p(out.ctypes.data), ctypes.byref(o), ctypes.byref(r))
    _check(rc, "avs_svdvals")
    return out


svdvals = my_CU_svdval


def svdvals_batched(mats, tiles=None, report=None, handle=None, rel_tol=0.0):
    """Singular values of many independent square matrices in one call.

    ``mats`` is a list of CUDA torch tensors, all float32 or all float64, each
    holding an n_i x n_i matrix column-major (see ``to_device``); orders may
    differ.  ``tiles`` is None (the autotuner picks a tile per order), an int
    for all, or a list.  Returns a list of CUDA tensors (the input dtype) of n_i
    values each (descending).  This is the batching client of the
    many-small-SVDs workload (RMT/rmt.jl:9-36), which the reference serves one
    LAPACK call at a time.  float32: FP32 tiles, double-float stages 2-3;
    float64: FP64 throughout.
    """
    import torch
    h = handle or default_handle()
    cnt = len(mats)
    if cnt == 0:
        return []
    if isinstance(tiles, int):
        tiles = [tiles] * cnt
    n = (ctypes.c_int64 * cnt)()
    ld = (ctypes.c_int64 * cnt)()
    tt = (ctypes.c_int32 * cnt)()
    pa = (ctypes.c_void_p * cnt)()
    ps = (ctypes.c_void_p * cnt)()
    outs = []
    dev = None
    dt = mats[0].dtype if _is_torch_cuda(mats[0]) else None
    if dt not in (torch.float32, torch.float64):
        raise TypeError("svdvals_batched takes 2-D float32 or float64 CUDA tensors")
    for i, A in enumerate(mats):
        if not _is_torch_cuda(A) or A.dim() != 2 or A.dtype != dt:
            raise TypeError("svdvals_batched takes 2-D CUDA tensors of one dtype (float32 or float64)")
        if A.shape[0] != A.shape[1]:
            raise NotImplementedError("Not implemented")
        if A.stride(1) != 1:
            A = A.contiguous()
            mats[i] = A
        dev = A.device
        n[i] = A.shape[0]
        ld[i] = max(A.stride(0), 1)
        tt[i] = 0 if tiles is None else int(tiles[i])
        pa[i] = A.data_ptr()
        o = torch.empty(A.shape[0], dtype=dt, device=A.device)
        ps[i] = o.data_ptr()
        outs.append(o)
    opt = Opts(0, 0, float(rel_tol), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    r = report if report is not None else Report()
    fn = lib().avs_svdvals_batched_dev_d if dt == torch.float64 else lib().avs_svdvals_batched_dev_s
    rc = fn(h.ptr, cnt, n, ld, None if tiles is None else tt, pa, ps, ctypes.byref(opt), ctypes.byref(r))
    _check(rc, "avs_svdvals_batched_dev")
    return outs


def bidiag_batched(mats, tiles=None, report=None, handle=None):
    """The batched pipeline up to the bidiagonal: for each square CUDA matrix
    (float32, or float64 computed in FP64 throughout; column-major, see
    ``to_device``) the diagonal d and superdiagonal e
    (FP64 CUDA tensors of n values; e[n-1] = 0) of a bidiagonal B with
    A = U B V^T, V e1 = e1 -- unique up to signs, so |d| and |e| are those of
    LAPACK gebrd (the quantity RMT/rmt.jl:24-31 reads)."""
    import torch
    h = handle or default_handle()
    cnt = len(mats)
    if cnt == 0:
        return []
    if isinstance(tiles, int):
        tiles = [tiles] * cnt
    n = (ctypes.c_int64 * cnt)()
    ld = (ctypes.c_int64 * cnt)()
    tt = (ctypes.c_int32 * cnt)()
    pa = (ctypes.c_void_p * cnt)()
    pd = (ctypes.c_void_p * cnt)()
    pe = (ctypes.c_void_p * cnt)()
    outs = []
    dev = None
    dt = mats[0].dtype if _is_torch_cuda(mats[0]) else None
    if dt not in (torch.float32, torch.float64):
        raise TypeError("bidiag_batched takes 2-D float32 or float64 CUDA tensors")
    for i, A in enumerate(mats):
        if not _is_torch_cuda(A) or A.dim() != 2 or A.dtype != dt:
            raise TypeError("bidiag_batched takes 2-D CUDA tensors of one dtype (float32 or float64)")
        if A.shape[0] != A.shape[1]:
            raise NotImplementedError("Not implemented")
        if A.stride(1) != 1:
            A = A.contiguous()
            mats[i] = A
        dev = A.device
        n[i] = A.shape[0]
        ld[i] = max(A.stride(0), 1)
        tt[i] = 0 if tiles is None else int(tiles[i])
        pa[i] = A.data_ptr()
        d = torch.empty(A.shape[0], dtype=torch.float64, device=A.device)
        e = torch.empty(A.shape[0], dtype=torch.float64, device=A.device)
        pd[i], pe[i] = d.data_ptr(), e.data_ptr()
        outs.append((d, e))
    opt = Opts(0, 0, 0.0, ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    r = report if report is not None else Report()
    fn = lib().avs_bidiag_batched_dev_d if dt == torch.float64 else lib().avs_bidiag_batched_dev_s
    rc = fn(h.ptr, cnt, n, ld, None if tiles is None else tt, pa, pd, pe, ctypes.byref(opt), ctypes.byref(r))
    _check(rc, "avs_bidiag_batched_dev")
    return outs


def selftest_timeout(handle=None):
    """Status of the bounded-wait check (AVS_ERR_TIMEOUT = 3 when the failure path works)."""
    h = handle or default_handle()
    return lib().avs_selftest_timeout(h.ptr)


def kernel_arch(device=0):
    """(binaryVersion, ptxVersion) of the library's device code as loaded on
    ``device`` (103 = sm_103a)."""
    bv, pv = ctypes.c_int32(0), ctypes.c_int32(0)
    _check(lib().avs_kernel_arch(int(device), ctypes.byref(bv), ctypes.byref(pv)), "avs_kernel_arch")
    return bv.value, pv.value


def chase_rate(device=0, fp64=False, arith=None):
    """Measured compute roof of the chase arithmetic (flops/s, 4 per element
    step): double-float by default, FP64 with fp64=True, or arith in
    {"df64", "fp64", "fp32"} (fp32: the blocked band reduction's arithmetic)."""
    mode = {"df64": 0, "fp64": 1, "fp32": 2}[arith] if arith else (1 if fp64 else 0)
    r = ctypes.c_double(0.0)
    _check(lib().avs_measure_chase_rate(int(device), mode, ctypes.byref(r)), "avs_measure_chase_rate")
    return r.value


def autotune_tile(n, sample=16, handle=None):
    """Tile the batched path uses for order n (timed on the device, cached on the handle)."""
    h = handle or default_handle()
    best = ctypes.c_int32(0)
    _check(lib().avs_autotune_tile(h.ptr, int(n), int(sample), ctypes.byref(best)), "avs_autotune_tile")
    return best.value


def tiled_QR(A, tile, precision=None, handle=None, report=None):
    """tiled_QR! (KAbasedSVD/src/tiledalgos.jl:6-15) in place on a CUDA tensor
    holding a column-major n x n matrix: R in the upper triangle, the
    Householder vectors below.  Returns the tau values as a CUDA tensor of
    nt * nt * tile elements (panel k, tile row r, reflector l at
    (k * nt + r) * tile + l)."""
    import torch
    h = handle or default_handle()
    if A.dim() != 2 or A.shape[0] != A.shape[1]:
        raise NotImplementedError("Not implemented")
    n = A.shape[0]
    nt = n // tile if tile > 0 else 0
    tau = torch.zeros(max(nt * nt * max(tile, 1), 1), dtype=A.dtype, device=A.device)
    o = Opts(_prec(precision), 0, 0.0, ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream))
    r = report if report is not None else Report()
    fn = lib().avs_geqrf_dev_d if A.dtype == torch.float64 else lib().avs_geqrf_dev_s
    rc = fn(h.ptr, n, max(A.stride(0), 1), int(tile), ctypes.c_void_p(A.data_ptr()),
            ctypes.c_void_p(tau.data_ptr()), ctypes.byref(o), ctypes.byref(r))
    _check(rc, "avs_geqrf_dev")
    return tau


def Blockbidiag(A, tile, handle=None):
    """Blockbidiag! in place on a CUDA tensor holding a column-major n x n matrix."""
    import torch
    h = handle or default_handle()
    n = A.shape[0]
    if A.dim() != 2 or A.shape[0] != A.shape[1] or not A.is_contiguous():
        raise NotImplementedError("Not implemented")
    fn = lib().avs_blockbidiag_dev_d if A.dtype == torch.float64 else lib().avs_blockbidiag_dev_s
    r = Report()
    rc = fn(h.ptr, n, n, int(tile), ctypes.c_void_p(A.data_ptr()), None, ctypes.byref(r))
    _check(rc, "avs_blockbidiag_dev")
    return r


def Blockbidiag_tau(A, tile, precision=None, handle=None, report=None):
    """Blockbidiag! in place on a CUDA tensor holding a column-major n x n
    matrix, keeping the tau of every reflector: returns (tau_q, tau_p), CUDA
    tensors of nt * nt * tile elements laid out as avs_blockbidiag_tau_dev
    documents (QR half-step k, tile row r at (k * nt + r) * tile; LQ half-step
    k, tile column c at (k * nt + c) * tile).  With the Householder vectors left
    in A they give Q and P of A = Q B P^T."""
    import torch
    h = handle or default_handle()
    if A.dim() != 2 or A.shape[0] != A.shape[1]:
        raise NotImplementedError("Not implemented")
    n = A.shape[0]
    nt = n // tile if tile > 0 else 0
    tq = torch.zeros(max(nt * nt * max(tile, 1), 1), dtype=A.dtype, device=A.device)
    tp = torch.zeros_like(tq)
    o = Opts(_prec(precision), 0, 0.0, ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream))
    r = report if report is not None else Report()
    fn = lib().avs_blockbidiag_tau_dev_d if A.dtype == torch.float64 else lib().avs_blockbidiag_tau_dev_s
    rc = fn(h.ptr, n, max(A.stride(0), 1), int(tile), ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(tq.data_ptr()),
            ctypes.c_void_p(tp.data_ptr()), ctypes.byref(o), ctypes.byref(r))
    _check(rc, "avs_blockbidiag_tau_dev")
    return tq, tp


def _ooc_matrix(A):
    a = A
    if not isinstance(a, np.ndarray) or a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise NotImplementedError("Not implemented")
    if a.dtype not in (np.float32, np.float64) or not a.flags.f_contiguous or not a.flags.writeable:
        raise TypeError("out-of-core calls work in place on a writeable Fortran-ordered float32/float64 array")
    return a


def ooc_plan(n, tile, dtype=np.float32, device_bytes=0):
    """(slab, device bytes, in-core step) of the out-of-core calls for this device budget."""
    slab, nb, frm = ctypes.c_int32(0), ctypes.c_int64(0), ctypes.c_int32(0)
    rc = lib().avs_ooc_plan(int(n), int(tile), np.dtype(dtype).itemsize, int(device_bytes), ctypes.byref(slab),
                            ctypes.byref(nb), ctypes.byref(frm))
    _check(rc, "avs_ooc_plan")
    return slab.value, nb.value, frm.value


def OOC_Bidiag(A, tile, device_bytes=0, handle=None, report=None):
    """OOC_Bidiag! (KAbasedSVD/src/tiledalgos.jl:248) in place on a host matrix
    (numpy, Fortran order): the band reduction streams the matrix through at
    most ``device_bytes`` of device memory (0: 90% of the free memory)."""
    h = handle or default_handle()
    a = _ooc_matrix(A)
    fn = lib().avs_blockbidiag_ooc_d if a.dtype == np.float64 else lib().avs_blockbidiag_ooc_s
    r = report if report is not None else Report()
    rc = fn(h.ptr, a.shape[0], max(a.shape[0], 1), int(tile), ctypes.c_void_p(a.ctypes.data), int(device_bytes),
            ctypes.byref(r))
    _check(rc, "avs_blockbidiag_ooc")
    return r


def OOC_SVD(A, tile, device_bytes=0, handle=None, report=None, rel_tol=0.0):
    """OOC_SVD! (KAbasedSVD/src/tiledalgos.jl:253-260) in place on a host matrix
    (numpy, Fortran order); returns the singular values (descending)."""
    h = handle or default_handle()
    a = _ooc_matrix(A)
    out = np.empty(a.shape[0], dtype=a.dtype)
    fn = lib().avs_svdvals_ooc_d if a.dtype == np.float64 else lib().avs_svdvals_ooc_s
    o = Opts(0, 0, float(rel_tol), None)
    r = report if report is not None else Report()
    rc = fn(h.ptr, a.shape[0], max(a.shape[0], 1), int(tile), ctypes.c_void_p(a.ctypes.data),
            ctypes.c_void_p(out.ctypes.data), int(device_bytes), ctypes.byref(o), ctypes.byref(r))
    _check(rc, "avs_svdvals_ooc")
    return out


def OOC_QR(A, tile, device_bytes=0, handle=None, report=None):
    """OOC_QR! (KAbasedSVD/src/tiledalgos.jl:247) in place on a host matrix
    (numpy, Fortran order); returns tau (nt * nt * tile, layout of tiled_QR)."""
    h = handle or default_handle()
    a = _ooc_matrix(A)
    n = a.shape[0]
    nt = n // int(tile) if tile else 0
    tau = np.zeros(max(nt * nt * int(tile), 1), dtype=a.dtype)
    fn = lib().avs_geqrf_ooc_d if a.dtype == np.float64 else lib().avs_geqrf_ooc_s
    r = report if report is not None else Report()
    rc = fn(h.ptr, n, max(n, 1), int(tile), ctypes.c_void_p(a.ctypes.data), ctypes.c_void_p(tau.ctypes.data),
            int(device_bytes), ctypes.byref(r))
    _check(rc, "avs_geqrf_ooc")
    return tau


def extract_band(A, bw, handle=None):
    """Upper band (0 <= j - i <= bw) of a device column-major matrix -> dense FP64 device matrix."""
    import torch
    h = handle or default_handle()
    n = A.shape[0]
    B = torch.empty((n, n), dtype=torch.float64, device=A.device)
    fn = lib().avs_extract_band_dev_d if A.dtype == torch.float64 else lib().avs_extract_band_dev_s
    rc = fn(h.ptr, n, n, int(bw), ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()), n)
    _check(rc, "avs_extract_band_dev")
    return B


def bidiagonalize(B, bw, handle=None):
    """Dense FP64 device band matrix (column-major) -> (d, e) FP64 device vectors."""
    import torch
    h = handle or default_handle()
    n = B.shape[0]
    d = torch.empty(n, dtype=torch.float64, device=B.device)
    e = torch.empty(max(n - 1, 1), dtype=torch.float64, device=B.device)
    r = Report()
    rc = lib().avs_band_to_bidiag_dev(h.ptr, n, int(bw), ctypes.c_void_p(B.data_ptr()), n,
                                      ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(e.data_ptr()), ctypes.byref(r))
    _check(rc, "avs_band_to_bidiag_dev")
    return d, e[: max(n - 1, 0)]


def band_reduce(B, bw, tbw, handle=None):
    """One stage of the hierarchical band reduction (the reference's bidiag!
    with factor bw / tbw, BRD/src/bulgechasing2.jl:22-45) in place on a CUDA
    tensor holding a dense column-major n x n upper band matrix of width bw
    (FP32 or FP64; the arithmetic follows the type): on return it holds a band
    of width tbw with the same singular values.  Returns the report."""
    import torch
    h = handle or default_handle()
    n = B.shape[0]
    if B.dim() != 2 or B.shape[0] != B.shape[1] or not B.is_contiguous():
        raise ValueError("a contiguous square matrix is needed")
    fn = lib().avs_band_reduce_dev_d if B.dtype == torch.float64 else lib().avs_band_reduce_dev_s
    r = Report()
    rc = fn(h.ptr, n, int(bw), int(tbw), ctypes.c_void_p(B.data_ptr()), n, ctypes.byref(r))
    _check(rc, "avs_band_reduce_dev")
    return r


def diag_lapack(d, e, rel_tol=0.0, handle=None):
    """Singular values (descending) of the upper bidiagonal (d, e) on the GPU."""
    import torch
    h = handle or default_handle()
    n = d.shape[0]
    s = torch.empty(n, dtype=torch.float64, device=d.device)
    rc = lib().avs_bidiag_svals_dev(h.ptr, n, ctypes.c_void_p(d.data_ptr()),
                                    ctypes.c_void_p(e.data_ptr()) if e.numel() else None,
                                    ctypes.c_void_p(s.data_ptr()), float(rel_tol), None)
    _check(rc, "avs_bidiag_svals_dev")
    return s


def geqrt_tile(a, handle=None):
    """GEQRT of one b x b tile (numpy in, numpy factors + tau out), on the GPU."""
    import torch
    h = handle or default_handle()
    a = np.asarray(a)
    b = a.shape[0]
    t = to_device(a)
    tau = torch.zeros(b, dtype=t.dtype, device=t.device)
    fn = lib().avs_geqrt_tile_dev_d if a.dtype == np.float64 else lib().avs_geqrt_tile_dev_s
    _check(fn(h.ptr, b, ctypes.c_void_p(t.data_ptr()), ctypes.c_void_p(tau.data_ptr())), "avs_geqrt_tile_dev")
    return from_device(t), tau.cpu().numpy()


def tsqrt_tile(r, bt, handle=None):
    """TSQRT of [triu(r); bt] (numpy in) -> (r', V, tau), on the GPU."""
    import torch
    h = handle or default_handle()
    r = np.asarray(r)
    b = r.shape[0]
    tr, tb = to_device(r), to_device(np.asarray(bt, dtype=r.dtype))
    tau = torch.zeros(b, dtype=tr.dtype, device=tr.device)
    fn = lib().avs_tsqrt_tile_dev_d if r.dtype == np.float64 else lib().avs_tsqrt_tile_dev_s
    _check(fn(h.ptr, b, ctypes.c_void_p(tr.data_ptr()), ctypes.c_void_p(tb.data_ptr()),
              ctypes.c_void_p(tau.data_ptr())), "avs_tsqrt_tile_dev")
    return from_device(tr), from_device(tb), tau.cpu().numpy()


def estimate_bytes(n, tile, precision="fp32", count=0):
    """Device workspace of one call (count 0) or of one batched FP32 group of ``count``."""
    b = ctypes.c_int64(0)
    _check(lib().avs_estimate_bytes(int(n), int(tile), _prec(precision), int(count), ctypes.byref(b)),
           "avs_estimate_bytes")
    return b.value


def serve_plan(n, dtype, tile=0):
    """(tile, precision mode name, batched) the serving loop uses for a request
    of order n and numpy dtype (float32 / float64); a served result equals
    my_CU_svdval(A, tile, precision=mode) bit for bit."""
    t, p, bt = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
    dt = 1 if np.dtype(dtype) == np.float64 else 0
    _check(lib().avs_serve_plan(int(n), dt, int(tile), ctypes.byref(t), ctypes.byref(p), ctypes.byref(bt)),
           "avs_serve_plan")
    name = {v: k for k, v in PREC.items()}[p.value]
    return t.value, name, bool(bt.value)


class Server:
    """SVD request server with continuous batching (``avs_serve_*`` in avs.h).

    ``submit(A)`` queues a host matrix (numpy float32 / float64, square) and
    returns a request id; ``wait(id)`` blocks until its values are ready and
    returns ``(sigma, latency_ms)``.  Several execution slots run groups
    concurrently on the GPU; requests of the same order and type that are
    queued together run as one batched call.  ``stats()`` gives p50/p99 latency,
    throughput and the device memory held against the admission budget.
    """

    def __init__(self, device=0, workers=4, max_batch=512, autotune=False, hbm_budget_bytes=0):
        cfg = ServeConfig(device, workers, max_batch, 1 if autotune else 0, int(hbm_budget_bytes))
        p = ctypes.c_void_p()
        _check(lib().avs_serve_create(ctypes.byref(p), ctypes.byref(cfg)), "avs_serve_create")
        self.ptr = p
        self._live = {}

    def submit(self, A, tile=0):
        a = np.asfortranarray(A)
        if a.ndim != 2 or a.shape[0] != a.shape[1]:
            raise NotImplementedError("Not implemented")
        if a.dtype not in (np.float32, np.float64):
            raise TypeError("float32 / float64 only")
        out = np.empty(a.shape[0], dtype=a.dtype)
        rid = ctypes.c_int64(0)
        dt = 1 if a.dtype == np.float64 else 0
        rc = lib().avs_serve_submit(self.ptr, a.shape[0], max(a.shape[0], 1), dt, int(tile),
                                    ctypes.c_void_p(a.ctypes.data), ctypes.c_void_p(out.ctypes.data),
                                    ctypes.byref(rid))
        _check(rc, "avs_serve_submit")
        self._live[rid.value] = (a, out)
        return rid.value

    def wait(self, rid, timeout_ms=-1.0):
        st = ctypes.c_int32(0)
        lat = ctypes.c_double(0.0)
        rc = lib().avs_serve_wait(self.ptr, int(rid), float(timeout_ms), ctypes.byref(st), ctypes.byref(lat))
        a, out = self._live.pop(rid, (None, None)) if rc != 3 else self._live.get(rid, (None, None))
        _check(rc, "avs_serve_wait")
        return out, lat.value

    def stats(self):
        s = ServeStats()
        _check(lib().avs_serve_stats_get(self.ptr, ctypes.byref(s)), "avs_serve_stats_get")
        return s.as_dict()

    def close(self):
        if self.ptr:
            lib().avs_serve_destroy(self.ptr)
            self.ptr = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
