"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (no dataset is involved; numpy PCG64 generators).

* ``gaussian(n, seed, scale)``: i.i.d. N(0, scale^2) entries (config 1:
  n=1024, seed 1, scale 1; config 3: n=16384, seed 4, scale 1/sqrt(n)).
* ``geometric_spectrum(n, seed_u, seed_v, lo)``: A = U diag(sigma) V^T with
  Haar-random orthogonal U, V (QR of seeded Gaussians, columns sign-fixed by
  diag(R)) and sigma_i = lo^((i-1)/(n-1)) (config 2: n=8192, seeds 2, 3,
  lo = 1e-6).  The exact singular values are returned with the matrix.
* ``integer_valued(n, seed)``: entries drawn from 1..10, as in the reference's
  end-to-end test (CUDAbasedSVD/test.jl:9).
* ``batch_sizes(count, seed, choices)``: matrix sizes for the batching config.
"""
import numpy as np


def gaussian(n, seed, scale=1.0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    if scale != 1.0:
        a *= scale
    return np.asfortranarray(a.astype(dtype, copy=False))


def _haar(n, seed, device=None):
    if device is not None:
        import torch
        g = torch.Generator(device="cpu").manual_seed(seed)
        z = torch.randn((n, n), generator=g, dtype=torch.float64).to(device)
        q, r = torch.linalg.qr(z)
        return q * torch.sign(torch.diagonal(r))[None, :]
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))[None, :]


def geometric_sigma(n, lo=1e-6):
    if n == 1:
        return np.ones(1)
    return lo ** (np.arange(n) / (n - 1.0))


def geometric_spectrum(n, seed_u=2, seed_v=3, lo=1e-6, dtype=np.float64, device=None):
    """(A, sigma): A = U diag(sigma) V^T.  With ``device`` (a torch device) the
    product is formed there and A is returned as a CUDA tensor holding the
    column-major matrix; otherwise as a Fortran-ordered numpy array."""
    sig = geometric_sigma(n, lo)
    if device is not None:
        import torch
        u = _haar(n, seed_u, device)
        v = _haar(n, seed_v, device)
        s = torch.from_numpy(sig).to(device)
        a = (u * s[None, :]) @ v.T
        tdt = torch.float64 if dtype == np.float64 else torch.float32
        return a.T.contiguous().to(tdt), sig
    u = _haar(n, seed_u)
    v = _haar(n, seed_v)
    a = (u * sig[None, :]) @ v.T
    return np.asfortranarray(a.astype(dtype)), sig


def integer_valued(n, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.integers(1, 11, size=(n, n)).astype(dtype))


def batch_sizes(count=4096, seed=5, choices=(64, 128, 256, 512, 1024)):
    rng = np.random.default_rng(seed)
    return rng.choice(np.asarray(choices), size=count)
