"""Generates tests/golden/golden.npz: seeded inputs with the oracle's outputs
and LAPACK's (scipy) singular values.

The reference ships no stored vectors (its tests draw unseeded random inputs
and compare against LAPACK / cuSOLVER, KAbasedSVD/test/test_QR_kernels.jl,
test_tiledalgo.jl, CUDAbasedSVD/test.jl), so these fixtures pin the oracle
with the same known-answer relations on fixed seeds:
  * GEQRT / TSQRT factors and tau of the oracle (QRkernels.jl restatement),
  * the band after Blockbidiag!, the bidiagonal after bidiagonalize,
  * the oracle's singular values and LAPACK gesdd's on the original matrix.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
import scipy.linalg as sl

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "avocado-sandwich_gb300"))

import oracle  # noqa: E402
from avs import workloads  # noqa: E402

CASES = [
    # name, n, tile, dtype, generator
    ("gauss_n64_b16_f64", 64, 16, np.float64, lambda n: workloads.gaussian(n, 11)),
    ("gauss_n128_b32_f64", 128, 32, np.float64, lambda n: workloads.gaussian(n, 12)),
    ("gauss_n128_b16_f32", 128, 16, np.float32, lambda n: workloads.gaussian(n, 13, dtype=np.float32)),
    ("int_n64_b16_f32", 64, 16, np.float32, lambda n: workloads.integer_valued(n, 14)),
    ("geom_n128_b64_f64", 128, 64, np.float64, lambda n: workloads.geometric_spectrum(n, 15, 16, 1e-6)[0]),
]


def main():
    out = {}
    rng = np.random.default_rng(100)
    for b, dt in ((16, np.float64), (32, np.float32)):
        a = rng.random((b, b)).astype(dt)
        f, tau = oracle.geqrt(a)
        a2 = rng.random((2 * b, b)).astype(dt)
        r, v, tau2 = oracle.tsqrt(a2[:b], a2[b:])
        key = "tile_b%d_%s" % (b, np.dtype(dt).name)
        out[key + "_geqrt_in"] = a
        out[key + "_geqrt_factors"] = f
        out[key + "_geqrt_tau"] = tau
        out[key + "_tsqrt_in"] = a2
        out[key + "_tsqrt_r"] = r
        out[key + "_tsqrt_v"] = v
        out[key + "_tsqrt_tau"] = tau2
        out[key + "_lapack_geqrt_factors"] = sl.qr(a.astype(np.float64), mode="raw")[0][0]
    for name, n, b, dt, gen in CASES:
        a = np.asarray(gen(n), dtype=dt)
        band = oracle.blockbidiag(a, b)
        bd = oracle.bidiagonalize(band, b)
        d, e = oracle.extract_bidiag(bd)
        out[name + "_A"] = a
        out[name + "_band"] = oracle.extract_band(band, b)
        out[name + "_d"] = d
        out[name + "_e"] = e
        out[name + "_sigma_oracle"] = oracle.svdvals(a, b)
        out[name + "_sigma_lapack"] = sl.svd(a.astype(np.float64), compute_uv=False, lapack_driver="gesdd")
        out[name + "_tile"] = np.array(b)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
