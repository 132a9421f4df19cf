"""Householder bidiagonalization and the RMT sampling statistics, in numpy.

TEST INFRASTRUCTURE ONLY -- the parity reference for the batched bidiagonal
output and for the random-matrix sampling client.  Nothing in the product
library imports it.

* ``gebd2``: the unblocked LAPACK bidiagonal reduction xGEBD2 (the kernel of
  xGEBRD, which the reference's RMT script calls as LAPACK.gebrd!,
  RMT/rmt.jl:24,29; LAPACK from OpenBLAS_jll 0.3.27, pinned in the reference's
  Manifest.toml): for i = 1..n a left reflector H(i) zeroes A(i+1:m, i), then a
  right reflector G(i) zeroes A(i, i+2:n); reflectors in the xLARFG convention
  beta = -sign(alpha) ||(alpha, x)||, tau = (beta - alpha) / beta,
  v = (1, x / (alpha - beta)).  Returns the diagonal d and superdiagonal e.
* ``mou_process_covar``: generate_MOUprocess_covar (RMT/rmt.jl:9-36) on given
  symmetric noise matrices G[trial, step] with gebd2 in FP64.
"""
import math

import numpy as np


def _larfg(x):
    """(beta, tau, v) of the reflector mapping x to beta e1 (v[0] = 1)."""
    alpha = x[0]
    xnorm = np.linalg.norm(x[1:])
    v = np.zeros_like(x)
    v[0] = 1.0
    if xnorm == 0.0:
        return alpha, 0.0, v
    beta = -math.copysign(math.hypot(alpha, xnorm), alpha)
    tau = (beta - alpha) / beta
    v[1:] = x[1:] / (alpha - beta)
    return beta, tau, v


def gebd2(a):
    """d (n) and e (n - 1) of the upper bidiagonal of a square matrix (FP64)."""
    a = np.array(a, dtype=np.float64)
    n = a.shape[0]
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 0))
    for i in range(n):
        beta, tau, v = _larfg(a[i:, i].copy())
        d[i] = beta
        if i + 1 < n and tau != 0.0:
            blk = a[i:, i + 1:]
            blk -= tau * np.outer(v, v @ blk)
        if i + 1 < n:
            beta, tau, v = _larfg(a[i, i + 1:].copy())
            e[i] = beta
            if i + 1 < n and tau != 0.0:
                blk = a[i + 1:, i + 1:]
                blk -= tau * np.outer(blk @ v, v)
    return d, e


def mou_process_covar(noise, timelength, k):
    """Statistics of RMT/rmt.jl:9-36 for noise[trial, step] (n x n symmetric)."""
    t, nt, n = noise.shape[0], noise.shape[1], noise.shape[2]
    dt = timelength / nt
    vals = np.zeros((nt, t))
    for j in range(t):
        m = noise[j, 0].astype(np.float64) / math.sqrt(2.0)
        vals[0, j] = gebd2(m)[0][k - 1]
        for i in range(1, nt):
            m = m * (1.0 - dt) + noise[j, i].astype(np.float64) * math.sqrt(dt)
            vals[i, j] = gebd2(m)[0][k - 1]
    vals = vals ** 2
    z = (vals - (n - k + 1)) / math.sqrt(n - k + 1)
    covar = z * z[0:1, :]
    return vals.mean(axis=1), covar.mean(axis=1), np.arange(nt) * dt
