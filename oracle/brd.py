"""Hierarchical band reduction of the reference's BRD code, in numpy.

TEST INFRASTRUCTURE ONLY -- the parity reference for an alternative stage-2
schedule; nothing in the product library imports it.

``bidiag(A, bandwidth, factor=4, kernelsizeinit=32)`` restates ``bidiag!``
(BRD/src/bulgechasing2.jl:22-45): the band is reduced in stages cbw -> tbw =
cbw // factor until it is bidiagonal.  Within a stage, sweeps start every
``kernelsize * ts`` rows (ts = tbw); at propagation index ``iter`` the
``kernelsize`` kernels of a sweep each run

* ``LQ_QMUL`` (:13-20): LQ of the ts rows starting at ``rowstart`` over the
  column window [row + cbw, row + 2cbw); the rows below, up to row + 2cbw - 1,
  are multiplied by Q^T; the ts rows become lower triangular in the window;
* ``QR_QMUL`` (:4-11): QR of the rows [row + cbw, row + 2cbw) over the first ts
  columns of [row + cbw, row + 3cbw); Q^T is applied to the rest of the column
  window; the ts columns become upper triangular;

with ``row = sweeprow + kernelidx * ts + cbw * (iter + 1 - 2 * kernelidx)``
and ``rowstart = row + cbw - tbw`` on a kernel's first step.  Index ranges are
the reference's 1-based inclusive ones, clipped to [1, n] as there.  The
Householder QR/LQ come from LAPACK through numpy (the reference calls Julia's
``qr!`` / ``lq!``, also LAPACK).
"""
import math

import numpy as np


def _clip(start, stop, n):
    return max(1, start), min(n, stop)


def _qr_qmul(a, r0, r1, c0, c1, n, ts):
    r0, r1 = _clip(r0, r1, n)
    c0, c1 = _clip(c0, c1, n)
    if r0 > r1 or c0 > c1:
        return
    ce = min(c0 + ts - 1, n)
    blk = a[r0 - 1:r1, c0 - 1:ce]
    q, r = np.linalg.qr(blk, mode="complete")
    if ce < c1:
        a[r0 - 1:r1, ce:c1] = q.T @ a[r0 - 1:r1, ce:c1]
    rr = np.zeros_like(blk)
    k = min(r.shape)
    rr[:k, :] = np.triu(r[:k, :])
    a[r0 - 1:r1, c0 - 1:ce] = rr


def _lq_qmul(a, r0, r1, c0, c1, n, ts):
    r0, r1 = _clip(r0, r1, n)
    c0, c1 = _clip(c0, c1, n)
    if r0 > r1 or c0 > c1:
        return
    re = min(r0 + ts - 1, n)
    blk = a[r0 - 1:re, c0 - 1:c1]
    # LQ of blk = (QR of blk^T)^T: blk = L Q with L = R^T, Q = Q1^T
    q1, r = np.linalg.qr(blk.T, mode="complete")
    if re < r1:
        a[re:r1, c0 - 1:c1] = a[re:r1, c0 - 1:c1] @ q1
    ll = np.zeros_like(blk)
    k = min(r.shape)
    ll[:, :k] = np.tril(r[:k, :].T)
    a[r0 - 1:re, c0 - 1:c1] = ll


def stage(a, cbw, tbw, kernelsizeinit=32, iters=None):
    """One stage of bidiag! (the body of its ``while cbw > 1`` loop) on a copy
    of the dense upper band matrix a (FP64): band cbw -> band tbw with ts =
    tbw; returns the copy.  ``iters`` as in ``bidiag``; None runs every kernel
    to the end (4 n)."""
    a = np.array(a, dtype=np.float64)
    n = a.shape[1]
    last = 4 * n if iters is None else int(iters)
    ts = tbw
    kernelsize = max(4, math.ceil(kernelsizeinit / tbw))
    for sweeprow in range(1, n - 1 - ts + 1, kernelsize * ts):
        for it in range(0, last + 1):
            active = False
            for kernelidx in range(1, kernelsize + 1):
                row = sweeprow + kernelidx * ts + cbw * (it + 1 - 2 * kernelidx)
                if it >= 2 * kernelidx - 2 and row < n:
                    active = True
                    rowstart = row + cbw - tbw if it == 2 * kernelidx - 2 else row
                    _lq_qmul(a, rowstart, row + 2 * cbw - 1, row + cbw, row + 2 * cbw - 1, n, ts)
                    _qr_qmul(a, row + cbw, row + 2 * cbw - 1, row + cbw, row + 3 * cbw - 1, n, ts)
            if not active and it > 2 * kernelsize:
                break
    return a


def bidiag(a, bandwidth, factor=4, kernelsizeinit=32, iters=None):
    """bidiag! on a copy of the dense upper band matrix a (FP64); returns it.

    ``iters`` is the last propagation index (the reference's ``0:n``).  That
    range is too short when n is small against the kernel count: the last
    kernels of a sweep stop before their bulge leaves the matrix (n = 64,
    bandwidth 4: kernel 32 starts at index 62 and needs about 70), and the
    result is not orthogonally equivalent to the input; ``iters = 4 n`` runs
    every kernel to the end."""
    a = np.array(a, dtype=np.float64)
    n = a.shape[1]
    last = n if iters is None else int(iters)
    cbw = int(bandwidth)
    while cbw > 1:
        tbw = max(1, cbw // factor)
        ts = tbw
        kernelsize = max(4, math.ceil(kernelsizeinit / tbw))
        for sweeprow in range(1, n - 1 - ts + 1, kernelsize * ts):
            for it in range(0, last + 1):
                for kernelidx in range(1, kernelsize + 1):
                    row = sweeprow + kernelidx * ts + cbw * (it + 1 - 2 * kernelidx)
                    if it >= 2 * kernelidx - 2 and row < n:
                        rowstart = row + cbw - tbw if it == 2 * kernelidx - 2 else row
                        _lq_qmul(a, rowstart, row + 2 * cbw - 1, row + cbw, row + 2 * cbw - 1, n, ts)
                        _qr_qmul(a, row + cbw, row + 2 * cbw - 1, row + cbw, row + 3 * cbw - 1, n, ts)
        cbw = tbw
    return a
