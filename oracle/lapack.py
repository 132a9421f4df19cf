"""LAPACK band-to-bidiagonal reduction (xGBBRD) and bidiagonal SVD (xBDSDC)
from the OpenBLAS that scipy bundles, through its LAPACKE C interface.

TEST INFRASTRUCTURE ONLY -- third-party comparators, never part of the product.

* ``gbbrd(band, bw)``: LAPACK dgbbrd on an upper band matrix (kl = 0, ku = bw),
  vect = 'N'.  The reference's BRD code compares its hierarchical band
  reduction with it (``gbbrd!``, BRD/src/bulgechasing2.jl:142-170).  dgbbrd's
  right rotations never touch column 1, so its bidiagonal is the Golub-Kahan
  bidiagonal of the band (V e1 = e1): equal to the GPU chase's up to signs.
* ``bdsdc(d, e)``: LAPACK dbdsdc('U', 'N'), the bidiagonal singular values
  the reference computes with ``LAPACK.bdsdc!`` (bulgechasing.jl:50-53;
  SVD_GPU.jl:267,281).  The GPU bisection is checked against it.

The library is located in scipy's wheel (``scipy.libs``, or next to the
package); ``available()`` is False where it, or the symbols, are missing.
"""
import ctypes
import glob
import os

import numpy as np

_LIB = None
_TRIED = False
_PREFIXES = ("scipy_LAPACKE_", "LAPACKE_")
LAPACK_COL_MAJOR = 102


def _find():
    try:
        import scipy
    except ImportError:
        return None
    root = os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__)))
    cands = sorted(glob.glob(os.path.join(root, "scipy.libs", "libscipy_openblas*.so*")))
    cands += sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), ".libs", "lib*openblas*.so*")))
    return cands[0] if cands else None


def _lib():
    global _LIB, _TRIED
    if not _TRIED:
        _TRIED = True
        path = _find()
        if path:
            try:
                _LIB = ctypes.CDLL(path)
            except OSError:
                _LIB = None
    return _LIB


def _sym(name):
    lib = _lib()
    if lib is None:
        return None
    for pre in _PREFIXES:
        f = getattr(lib, pre + name, None)
        if f is not None:
            return f
    return None


def available():
    return _sym("dgbbrd") is not None and _sym("dbdsdc") is not None


def gbbrd(band, bw):
    """(d, e) of LAPACK dgbbrd on the upper band (0 <= j - i <= bw) of a dense
    square matrix (only the band is read)."""
    f = _sym("dgbbrd")
    if f is None:
        raise RuntimeError("LAPACKE dgbbrd not found")
    a = np.asarray(band, dtype=np.float64)
    n = a.shape[0]
    ldab = bw + 1
    ab = np.zeros((n, ldab))  # column-major (ldab x n): ab[c, bw + r - c] = A[r, c]
    for k in range(bw + 1):  # diagonal k above the main one
        if k < n:
            ab[k:, bw - k] = np.diagonal(a, k)
    ab = np.ascontiguousarray(ab)
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 1))
    dummy = np.zeros(1)
    P, I = ctypes.c_void_p, ctypes.c_int
    f.restype = I
    f.argtypes = [I, ctypes.c_char, I, I, I, I, I, P, I, P, P, P, I, P, I, P, I]
    info = f(LAPACK_COL_MAJOR, b"N", n, n, 0, 0, bw, ab.ctypes.data, ldab, d.ctypes.data, e.ctypes.data,
             dummy.ctypes.data, 1, dummy.ctypes.data, 1, dummy.ctypes.data, 1)
    if info != 0:
        raise RuntimeError("dgbbrd info %d" % info)
    return d, e[: max(n - 1, 0)]


def bdsdc(d, e):
    """Singular values (descending) of the upper bidiagonal (d, e), LAPACK dbdsdc('U', 'N')."""
    f = _sym("dbdsdc")
    if f is None:
        raise RuntimeError("LAPACKE dbdsdc not found")
    dd = np.array(d, dtype=np.float64)
    n = dd.shape[0]
    ee = np.zeros(max(n, 1))
    ee[: n - 1] = np.asarray(e, dtype=np.float64)[: n - 1]
    dummy = np.zeros(1)
    idummy = np.zeros(1, dtype=np.int64)
    P, I = ctypes.c_void_p, ctypes.c_int
    f.restype = I
    f.argtypes = [I, ctypes.c_char, ctypes.c_char, I, P, P, P, I, P, I, P, P]
    info = f(LAPACK_COL_MAJOR, b"U", b"N", n, dd.ctypes.data, ee.ctypes.data, dummy.ctypes.data, 1,
             dummy.ctypes.data, 1, dummy.ctypes.data, idummy.ctypes.data)
    if info != 0:
        raise RuntimeError("dbdsdc info %d" % info)
    return dd
