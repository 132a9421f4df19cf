"""ctypes wrapper around ``liboracle.so`` (built from ``oracle.c`` by ``make``).

TEST INFRASTRUCTURE ONLY -- the parity reference for the CUDA library.

Functions mirror the reference building blocks (paths inside
evelyne-ringoot/Avocado-sandwich):

* ``geqrt`` / ``tsqrt`` / ``apply1`` / ``apply2``: KAbasedSVD/src/QRkernels.jl:3-197
* ``blockbidiag``: Blockbidiag! (KAbasedSVD/src/tiledalgos.jl:17-59)
* ``bidiagonalize``: KAbasedSVD/src/bulgechasing.jl:33-42
* ``bidiag_svals``: the quantity of LAPACK bdsdc('U','N') (bulgechasing.jl:50-53),
  by bisection on the Golub-Kahan tridiagonal
* ``svdvals``: my_CU_svdval (CUDAbasedSVD/SVD_GPU.jl:257-283) end to end

Arrays are numpy, column-major (Fortran order), float32 or float64.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

__all__ = [
    "build", "lib", "geqrt", "tsqrt", "apply1", "apply2", "blockbidiag", "blockbidiag_keep", "bidiagonalize",
    "bidiag_svals", "svdvals", "set_threads", "num_threads", "extract_bidiag", "extract_band",
]


def build(force=False):
    """Compile liboracle.so with make (gcc, OpenMP)."""
    so = os.path.join(_HERE, "liboracle.so")
    if force or not os.path.exists(so) or os.path.getmtime(so) < max(
            os.path.getmtime(os.path.join(_HERE, f)) for f in ("oracle.c", "oracle_impl.h")):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"] + (["-B"] if force else []))
    return so


def lib():
    global _LIB
    if _LIB is None:
        so = build()
        L = ctypes.CDLL(so)
        P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        for suf in ("_s", "_d"):
            getattr(L, "oracle_geqrt" + suf).argtypes = [P, I64, I, P]
            getattr(L, "oracle_tsqrt" + suf).argtypes = [P, I64, P, I64, I, P]
            getattr(L, "oracle_apply1" + suf).argtypes = [P, I64, I64, P, I64, P, I, I]
            getattr(L, "oracle_apply2" + suf).argtypes = [P, I64, P, I64, I64, P, I64, P, I, I]
            getattr(L, "oracle_blockbidiag" + suf).argtypes = [P, I64, I64, I]
            getattr(L, "oracle_blockbidiag_keep" + suf).argtypes = [P, I64, I64, I, P, P]
            getattr(L, "oracle_bidiagonalize" + suf).argtypes = [P, I64, I64, I64]
            getattr(L, "oracle_svdvals" + suf).argtypes = [P, I64, I64, I, P, ctypes.c_double]
            getattr(L, "oracle_svdvals" + suf).restype = I
        L.oracle_bidiag_svals.argtypes = [P, P, I64, P, ctypes.c_double]
        L.oracle_set_threads.argtypes = [I]
        L.oracle_num_threads.restype = I
        _LIB = L
    return _LIB


def _suf(a):
    if a.dtype == np.float32:
        return "_s"
    if a.dtype == np.float64:
        return "_d"
    raise TypeError("oracle supports float32 / float64 only")


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _fortran(a, dtype=None):
    a = np.asarray(a, dtype=dtype)
    return np.array(a, order="F", copy=True)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def num_threads():
    return int(lib().oracle_num_threads())


def geqrt(a):
    """GEQRT of one b x b tile -> (factors, tau) as QR_unsafe_kernel! leaves them."""
    a = _fortran(a)
    b = a.shape[0]
    tau = np.zeros(b, dtype=a.dtype)
    getattr(lib(), "oracle_geqrt" + _suf(a))(_ptr(a), b, b, _ptr(tau))
    return a, tau


def tsqrt(r, bt):
    """TSQRT of [triu(r); bt] -> (r', V, tau) as QR_unsafe_kernel2! leaves them."""
    r = _fortran(r)
    bt = _fortran(bt, r.dtype)
    b = r.shape[0]
    tau = np.zeros(b, dtype=r.dtype)
    getattr(lib(), "oracle_tsqrt" + _suf(r))(_ptr(r), b, _ptr(bt), b, b, _ptr(tau))
    return r, bt, tau


def apply1(bm, v, tau, trans=True):
    """Apply Q^T (trans) or Q of a GEQRT tile to a b x m block."""
    bm = _fortran(bm)
    v = _fortran(v, bm.dtype)
    tau = np.ascontiguousarray(tau, dtype=bm.dtype)
    b = v.shape[0]
    getattr(lib(), "oracle_apply1" + _suf(bm))(_ptr(bm), b, bm.shape[1], _ptr(v), b, _ptr(tau), b, int(trans))
    return bm


def apply2(am, bm, v, tau, trans=True):
    """Apply Q^T (trans) or Q of a TSQRT pair to [am; bm] (each b x m)."""
    am = _fortran(am)
    bm = _fortran(bm, am.dtype)
    v = _fortran(v, am.dtype)
    tau = np.ascontiguousarray(tau, dtype=am.dtype)
    b = v.shape[0]
    getattr(lib(), "oracle_apply2" + _suf(am))(_ptr(am), b, _ptr(bm), b, am.shape[1], _ptr(v), b, _ptr(tau), b,
                                              int(trans))
    return am, bm


def blockbidiag(a, b):
    """Blockbidiag! on a copy of the square matrix a with tile b -> upper band (dense array)."""
    a = _fortran(a)
    n = a.shape[0]
    getattr(lib(), "oracle_blockbidiag" + _suf(a))(_ptr(a), n, n, int(b))
    return a


def blockbidiag_keep(a, b):
    """Blockbidiag! on a copy of a, keeping the Householder vectors in the
    tiles and every tau -> (matrix, tau_q, tau_p), tau layout of
    avs_blockbidiag_tau_dev (QR half-step k, tile row r at (k*nt + r)*b; LQ
    half-step k, tile column c at (k*nt + c)*b).  The band equals blockbidiag's."""
    a = _fortran(a)
    n = a.shape[0]
    nt = n // int(b)
    tq = np.zeros(max(nt * nt * int(b), 1), dtype=a.dtype)
    tp = np.zeros_like(tq)
    getattr(lib(), "oracle_blockbidiag_keep" + _suf(a))(_ptr(a), n, n, int(b), _ptr(tq), _ptr(tp))
    return a, tq, tp


def bidiagonalize(a, bw):
    """bidiagonalize(A, bw) on a copy of the dense banded matrix a."""
    a = _fortran(a)
    n = a.shape[0]
    getattr(lib(), "oracle_bidiagonalize" + _suf(a))(_ptr(a), n, n, int(bw))
    return a


def extract_bidiag(a):
    a = np.asarray(a)
    return np.ascontiguousarray(np.diag(a), dtype=np.float64), np.ascontiguousarray(np.diag(a, 1), dtype=np.float64)


def extract_band(a, bw):
    """Upper band 0 <= j - i <= bw of a dense matrix, zeros elsewhere."""
    a = np.asarray(a)
    i, j = np.indices(a.shape)
    return np.where((j - i >= 0) & (j - i <= bw), a, 0).astype(a.dtype)


def bidiag_svals(d, e, rel_tol=1e-15):
    """Singular values (descending) of the upper bidiagonal (d, e), bisection in float64."""
    d = np.ascontiguousarray(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    n = d.shape[0]
    if e.shape[0] < max(n - 1, 0):
        raise ValueError("e must have n-1 entries")
    if e.shape[0] == 0:
        e = np.zeros(1)
    s = np.zeros(n, dtype=np.float64)
    lib().oracle_bidiag_svals(_ptr(d), _ptr(e), n, _ptr(s), float(rel_tol))
    return s


def svdvals(a, b, rel_tol=1e-15):
    """my_CU_svdval(a, b) restated on the CPU: float64 singular values, descending.

    Raises NotImplementedError on the reference's "Not implemented" cases
    (CUDAbasedSVD/SVD_GPU.jl:261-262, 275-276).
    """
    a = np.asarray(a)
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise NotImplementedError("Not implemented")
    a = _fortran(a)
    n = a.shape[0]
    s = np.zeros(n, dtype=np.float64)
    rc = getattr(lib(), "oracle_svdvals" + _suf(a))(_ptr(a), n, n, int(b), _ptr(s), float(rel_tol))
    if rc == -1:
        raise NotImplementedError("Not implemented")
    if rc != 0:
        raise MemoryError("oracle_svdvals failed (%d)" % rc)
    return s
