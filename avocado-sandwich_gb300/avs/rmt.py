"""Random-matrix sampling client of the batched path.

The reference's RMT study (RMT/rmt.jl:9-36) follows a matrix Ornstein-Uhlenbeck
process: for each trial, M_1 = G_1 / sqrt(2) and M_i = (1 - dt) M_{i-1} +
sqrt(dt) G_i (i = 2..nt), with G_i = X + X^T for a Gaussian X (rmt.jl:3-7).
Each M_i goes through LAPACK gebrd! one at a time and the k-th diagonal entry
d_k of its bidiagonal is recorded; the outputs are the trial means of d_k^2
and of the standardised products c_i = z_i z_1, z = (d_k^2 - (n-k+1)) /
sqrt(n-k+1), per time step (rmt.jl:32-35).

Here all matrices of a time step (one per trial) -- and several time steps at
once, up to ``chunk`` matrices -- go through one batched call
(``avs.bidiag_batched``), and the process itself is stepped on the GPU.  The
bidiagonal with V e1 = e1 is unique up to signs, so d_k^2 is gebrd's d_k^2.
Orders that no tile of at least 16 divides are zero-padded to the next
multiple of 16: the bidiagonal of [M 0; 0 0] is that of M followed by zeros.
``dtype`` selects the arithmetic: float64 (the reference's, LAPACK gebrd! in
Float64, rmt.jl:23,28) runs the FP64 batched path throughout; float32 the FP32
path (double-float stages).
"""
import math

import numpy as np

import avs


def padded_order(n, tile=16):
    return ((n + tile - 1) // tile) * tile


def mou_process_covar(numtrials, matrixsize, numtimestep, timelength, kthsvdval, seed=0, tile=None,
                      chunk=4096, noise=None, handle=None, dtype="float64"):
    """generate_MOUprocess_covar (RMT/rmt.jl:9-36) on the GPU.

    Returns (mean of d_k^2 per time step, mean of the standardised products per
    time step, time grid), as the reference.  ``noise`` (optional) is a
    (numtrials, numtimestep, n, n) array of the symmetric G_i to use
    instead of the seeded generator (for tests against the oracle)."""
    import torch
    n, nt, t, k = int(matrixsize), int(numtimestep), int(numtrials), int(kthsvdval)
    if not (1 <= k <= n):
        raise ValueError("kthsvdval must be in 1..matrixsize")
    dt = timelength / nt
    npad = padded_order(n)
    if not tile:  # the largest power of two <= 64 dividing npad with at least two tiles
        tile = 64
        while tile > 16 and (npad % tile or npad // tile < 2):
            tile //= 2
    dev = torch.device("cuda", torch.cuda.current_device())
    tdt = {"float64": torch.float64, "float32": torch.float32}[str(np.dtype(dtype))]
    gen = torch.Generator(device=dev).manual_seed(int(seed))
    h = handle or avs.default_handle()

    def draw(i):
        if noise is not None:
            g = torch.as_tensor(np.asarray(noise[:, i]), device=dev).to(tdt)
        else:
            x = torch.randn((t, n, n), generator=gen, device=dev, dtype=tdt)
            g = x + x.transpose(1, 2)
        return g

    vals = np.zeros((nt, t))
    pending, slots = [], []

    def flush():
        if not pending:
            return
        outs = avs.bidiag_batched(pending, tiles=tile, handle=h)
        dk = torch.stack([d[k - 1] for d, _ in outs]).cpu().numpy()
        for (i, j), v in zip(slots, dk):
            vals[i, j] = float(v) ** 2
        pending.clear()
        slots.clear()

    m = None
    for i in range(nt):
        g = draw(i)
        m = g / math.sqrt(2.0) if i == 0 else m * (1.0 - dt) + g * math.sqrt(dt)
        padded = torch.zeros((t, npad, npad), dtype=tdt, device=dev)
        padded[:, :n, :n] = m  # symmetric: row- and column-major views agree
        for j in range(t):
            pending.append(padded[j])
            slots.append((i, j))
        if len(pending) >= chunk:
            flush()
    flush()
    z = (vals - (n - k + 1)) / math.sqrt(n - k + 1)
    covar = z * z[0:1, :]
    return vals.mean(axis=1), covar.mean(axis=1), np.arange(nt) * dt
