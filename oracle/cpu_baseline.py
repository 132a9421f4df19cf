"""The reference's CPU path of the tiled SVD, stage by stage, for timing.

TEST AND BENCHMARK INFRASTRUCTURE ONLY: the timed CPU baseline beside the GPU
numbers (never part of the product).  Paths are inside
evelyne-ringoot/Avocado-sandwich.

* Stage 1, ``band_bidiagonal``: BandBidiagonal!(A, b, b, nt, nt, onGPU=false)
  (CUDAbasedSVD/SVD_GPU.jl:176-214, with QR! at :67-160).  Each QR half-step
  stacks the pivot tile and one tile below it as a dense 2b x b block, factors
  it with Julia's qr! -- LAPACK dgeqrt with block size min(36, b), Julia's
  QRCompactWY -- and applies Q' to the stacked tile pairs of the row panel with
  lmul! (LAPACK dgemqrt 'L','T'); the LQ half-step does the same on adjoint
  copies and applies Q from the right with rmul! (dgemqrt 'R','N').  The
  reference's CPU temporaries are Float64 (``zeros``), so this runs in float64.
  LAPACK comes from the OpenBLAS that scipy bundles (the reference's is
  OpenBLAS_jll 0.3.27 through libblastrampoline).
* Stage 2: ``bidiagonalize`` (KAbasedSVD/src/bulgechasing.jl:33-42), the
  oracle's C restatement (OpenMP).
* Stage 3: ``diag_lapack`` = LAPACK dbdsdc('U', 'N') (bulgechasing.jl:50-53).

``run(a, b)`` times the three stages separately (wall clock) and returns the
singular values with the times.
"""
import ctypes
import time

import numpy as np

from . import lapack

COL_MAJOR = 102


def _f(name):
    f = lapack._sym(name)
    if f is None:
        raise RuntimeError("LAPACKE %s not found in scipy's OpenBLAS" % name)
    return f


def _setup():
    P, I, C = ctypes.c_void_p, ctypes.c_int, ctypes.c_char
    geqrt = _f("dgeqrt")
    geqrt.restype = I
    geqrt.argtypes = [I, I, I, I, P, I, P, I]
    gemqrt = _f("dgemqrt")
    gemqrt.restype = I
    gemqrt.argtypes = [I, C, C, I, I, I, I, P, I, P, I, P, I]
    return geqrt, gemqrt


def blas_threads(n=None):
    """Get (n is None) or set the thread count of scipy's OpenBLAS."""
    lib = lapack._lib()
    if lib is None:
        return 1
    if n is None:
        f = getattr(lib, "scipy_openblas_get_num_threads", None)
        return int(f()) if f else 1
    f = getattr(lib, "scipy_openblas_set_num_threads", None)
    if f:
        f.argtypes = [ctypes.c_int]
        f(int(n))
    return int(n)


def _ptr(x):
    return ctypes.c_void_p(x.ctypes.data)


def band_bidiagonal(A, b):
    """BandBidiagonal!(A, b, b, nt, nt, onGPU=false) on a float64 copy of A:
    returns the upper band (0 <= j - i <= b; everything else exactly zero)."""
    geqrt, gemqrt = _setup()
    a = np.array(A, dtype=np.float64, order="F")
    n = a.shape[0]
    nt = n // b
    nb = min(36, b)
    t = np.zeros((nb, b), order="F")
    b2 = 2 * b

    def qr(blk, m):
        info = geqrt(COL_MAJOR, m, b, nb, _ptr(blk), blk.shape[0], _ptr(t), nb)
        if info != 0:
            raise RuntimeError("dgeqrt info %d" % info)

    def apply(side, trans, v, m_v, c, m, ncols):
        info = gemqrt(COL_MAJOR, side, trans, m, ncols, b, nb, _ptr(v), v.shape[0], _ptr(t), nb, _ptr(c),
                      c.shape[0])
        if info != 0:
            raise RuntimeError("dgemqrt info %d" % info)

    for k in range(nt):
        # ---- QR sweep (SVD_GPU.jl:183-195): cached 2b x b blocks of the row panel
        cache = [np.zeros((b2, b), order="F") for _ in range(nt - k)]
        for j in range(nt - k):
            cache[j][:b] = a[k * b:(k + 1) * b, (k + j) * b:(k + j + 1) * b]
        top = np.array(cache[0][:b], order="F")  # QR_single_col!
        qr(top, b)
        for j in range(1, nt - k):
            c = np.array(cache[j][:b], order="F")
            apply(b"L", b"T", top, b, c, b, b)
            cache[j][:b] = c
        cache[0][:b] = np.triu(top)
        for row in range(k + 1, nt):  # QR_double_col!
            for j in range(nt - k):
                cache[j][b:] = a[row * b:(row + 1) * b, (k + j) * b:(k + j + 1) * b]
            blk = np.array(cache[0], order="F")
            qr(blk, b2)
            for j in range(1, nt - k):
                c = np.array(cache[j], order="F")
                apply(b"L", b"T", blk, b2, c, b2, b)
                cache[j][:] = c
            cache[0][:] = np.triu(blk)
            for j in range(nt - k):
                a[row * b:(row + 1) * b, (k + j) * b:(k + j + 1) * b] = cache[j][b:]
        for j in range(nt - k):
            a[k * b:(k + 1) * b, (k + j) * b:(k + j + 1) * b] = cache[j][:b]
        if k == nt - 1:
            break
        # ---- LQ sweep (SVD_GPU.jl:197-210): QR of adjoint copies, rmul! on the column panels
        k1 = slice((k + 1) * b, (k + 2) * b)
        rows = slice((k + 1) * b, n)
        top = np.array(a[k * b:(k + 1) * b, k1].T, order="F")  # QR_single_row!
        qr(top, b)
        c = np.array(a[rows, k1], order="F")
        apply(b"R", b"N", top, b, c, c.shape[0], b)
        a[rows, k1] = c
        lower = np.tril(top.T)
        for col in range(k + 2, nt):  # QR_double_row!
            blk = np.zeros((b2, b), order="F")
            blk[:b] = lower.T
            blk[b:] = a[k * b:(k + 1) * b, col * b:(col + 1) * b].T
            qr(blk, b2)
            c = np.zeros((n - (k + 1) * b, b2), order="F")
            c[:, :b] = a[rows, k1]
            c[:, b:] = a[rows, col * b:(col + 1) * b]
            apply(b"R", b"N", blk, b2, c, c.shape[0], b2)
            a[rows, k1] = c[:, :b]
            a[rows, col * b:(col + 1) * b] = c[:, b:]
            lower = np.tril(np.triu(blk[:b]).T)
            a[k * b:(k + 1) * b, col * b:(col + 1) * b] = 0.0
        a[k * b:(k + 1) * b, k1] = lower
    i, j = np.indices(a.shape)
    a[(j - i < 0) | (j - i > b)] = 0.0
    return a


def run(A, b, threads=None):
    """The three stages on A (float64 arithmetic), timed separately:
    (sigma descending, {"stage1": s, "stage2": s, "stage3": s})."""
    from . import oracle as O
    if threads is not None:
        blas_threads(threads)
        O.set_threads(threads)
    t0 = time.perf_counter()
    band = band_bidiagonal(A, b)
    t1 = time.perf_counter()
    bd = O.bidiagonalize(band, b)
    t2 = time.perf_counter()
    d, e = O.extract_bidiag(bd)
    s = np.sort(np.abs(lapack.bdsdc(d, e)))[::-1]
    t3 = time.perf_counter()
    return s, {"stage1": t1 - t0, "stage2": t2 - t1, "stage3": t3 - t2}
