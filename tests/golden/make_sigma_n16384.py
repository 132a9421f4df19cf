"""Fixture: FP64 LAPACK singular values of the n = 16384 headline matrix.

The matrix is ``avs.workloads.gaussian(16384, 4, 1/sqrt(n), float32)`` -- numpy
PCG64 seed 4, N(0, 1/n) entries rounded to float32 -- the input of the
precision configuration (n = 16384, tile 256).  Its singular values are
computed by LAPACK dgesdd (scipy, values only) on the float32 entries widened
to float64, so they are exact for the matrix the GPU receives.  The fixture
also stores a SHA-256 of the float32 bytes, so that a test on another machine
checks that numpy generated the same matrix there before it compares.

    python tests/golden/make_sigma_n16384.py   # ~30-60 min on 8 cores
"""
import hashlib
import os
import sys
import time

import numpy as np
import scipy.linalg as sl

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "avocado-sandwich_gb300"))

N, SEED = 16384, 4
OUT = os.path.join(HERE, "sigma_n16384_seed4.npz")


def matrix():
    from avs import workloads
    return workloads.gaussian(N, SEED, 1.0 / np.sqrt(N), dtype=np.float32)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes(order="F")).hexdigest()


def main():
    a = matrix()
    h = digest(a)
    t0 = time.time()
    s = sl.svdvals(a.astype(np.float64), check_finite=False)
    dt = time.time() - t0
    np.savez_compressed(OUT, sigma=s, sha256=np.array(h), n=N, seed=SEED, seconds=dt)
    print("wrote", OUT, "sha256", h, "%.0f s" % dt)


if __name__ == "__main__":
    main()
