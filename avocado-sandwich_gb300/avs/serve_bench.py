"""Serving benchmark: a Poisson stream of SVD requests through ``avs.Server``.

Request mix (the serving workload of the reference's benchmark plan): square
orders log-uniform in [128, 8192] rounded to a power of two, 70% float32 / 30%
float64, half Gaussian N(0, 1/n) and half with a prescribed geometric spectrum
(sigma_i from 1 down to 1e-6).  Inputs come from a seeded pool (a few matrices
per order and kind, generated once on the GPU and kept in host memory), so the
stream itself costs no generation time.  Arrivals are Poisson at ``rate``
requests/s; one thread submits at the arrival times, the server batches and
overlaps, and the script waits for all results.

Prints one JSON object: SVDs/s, p50/p99 latency, the mix, the max normwise
singular-value error of every checked request against an FP64 LAPACK
reference (``check`` requests, the smallest orders), and the one-at-a-time
SVDs/s of the same request list through blocking calls, each in its own
precision and all through the plain FP64 path.

    python -m avs.serve_bench --requests 200 --rate 2.0
"""
import argparse
import json
import threading
import time

import numpy as np

import avs
from avs import workloads

ORDERS = (128, 256, 512, 1024, 2048, 4096, 8192)


def request_list(count, seed, max_order=8192):
    rng = np.random.default_rng(seed)
    lo, hi = np.log(128), np.log(max_order)
    n = np.exp(rng.uniform(lo, hi, size=count))
    n = (2 ** np.round(np.log2(n))).astype(np.int64)
    f64 = rng.random(count) < 0.3
    geo = rng.random(count) < 0.5
    variant = rng.integers(0, 2, size=count)
    return [(int(a), bool(b), bool(c), int(d)) for a, b, c, d in zip(n, f64, geo, variant)]


def make_pool(reqs, device="cuda"):
    """(n, f64, geometric, variant) -> host matrix (Fortran order)."""
    import torch
    pool = {}
    for key in sorted(set(reqs)):
        n, f64, geo, var = key
        dt = np.float64 if f64 else np.float32
        if geo:
            a, _ = workloads.geometric_spectrum(n, 20 + var, 40 + var, 1e-6, dtype=dt, device=device)
            pool[key] = np.asfortranarray(a.cpu().numpy().T)
        else:
            g = torch.Generator(device="cpu").manual_seed(1000 * n + var)
            a = torch.randn((n, n), generator=g, dtype=torch.float64) / np.sqrt(n)
            pool[key] = np.asfortranarray(a.numpy().astype(dt))
    return pool


def rule_tile(n):
    t = 32 if n <= 256 else (64 if n <= 1024 else 128)
    while t > 16 and (n % t or t > n):
        t //= 2
    return t


def run(requests=200, rate=2.0, seed=7, workers=4, check=16, one_at_a_time=True, max_order=8192,
        baseline_every=1):
    reqs = request_list(requests, seed, max_order)
    pool = make_pool(reqs)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(reqs)))
    ids = [None] * len(reqs)
    srv = avs.Server(workers=workers)
    # warm the slots (module load, first kernel launches) outside the measured stream
    for key in sorted(pool)[:2]:
        srv.wait(srv.submit(pool[key]))

    def submitter():
        t0 = time.perf_counter()
        for i, key in enumerate(reqs):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids[i] = srv.submit(pool[key])

    t_start = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    outs, lats = [], []
    for i in ids:
        s, lat = srv.wait(i)
        outs.append(s)
        lats.append(lat)
    wall = time.perf_counter() - t_start
    st = srv.stats()
    srv.close()
    lats = np.sort(np.asarray(lats))
    res = {
        "requests": len(reqs), "offered_rate_rps": rate, "workers": workers,
        "svds_per_s": len(reqs) / wall, "wall_s": wall,
        "p50_ms": float(np.percentile(lats, 50, method="higher")),
        "p99_ms": float(np.percentile(lats, 99, method="higher")),
        "server": st,
        "mix": {"f32": sum(1 for r in reqs if not r[1]), "f64": sum(1 for r in reqs if r[1]),
                "orders": {int(n): sum(1 for r in reqs if r[0] == n) for n in ORDERS if n <= max_order}},
    }
    # accuracy of the smallest requests against FP64 LAPACK
    import scipy.linalg as sl
    order = np.argsort([r[0] for r in reqs], kind="stable")[:check]
    err = {"f32": 0.0, "f64": 0.0}
    for i in order:
        key = reqs[i]
        ref = sl.svdvals(pool[key].astype(np.float64))
        e = float(np.max(np.abs(outs[i].astype(np.float64) - ref)) / ref[0])
        k = "f64" if key[1] else "f32"
        err[k] = max(err[k], e)
    res["max_rel_sigma_err"] = err
    if one_at_a_time:
        # the same request list, one blocking call at a time (no overlap, no batching):
        # (1) each request in its own precision, (2) every request through the
        # plain FP64 path (FP32 inputs widened on the host, outside the timing)
        # (every baseline_every-th request of the list, scaled to the list)
        sub = reqs[::max(1, baseline_every)]
        h = avs.Handle()
        for key in sorted(set(sub))[:2]:
            avs.my_CU_svdval(pool[key], rule_tile(key[0]), handle=h)
        t0 = time.perf_counter()
        for key in sub:
            avs.my_CU_svdval(pool[key], rule_tile(key[0]), handle=h)
        res["one_at_a_time_svds_per_s"] = len(sub) / (time.perf_counter() - t0)
        wide = {k: np.asfortranarray(v.astype(np.float64)) for k, v in pool.items() if k in set(sub)}
        t_sum = 0.0
        for key in sub:
            t0 = time.perf_counter()
            avs.my_CU_svdval(wide[key], rule_tile(key[0]), handle=h)
            t_sum += time.perf_counter() - t0
        res["one_at_a_time_plain_fp64_svds_per_s"] = len(sub) / t_sum
        res["one_at_a_time_sample"] = "%d of the %d requests" % (len(sub), len(reqs))
        res["speedup_vs_one_at_a_time_plain_fp64"] = res["svds_per_s"] / res["one_at_a_time_plain_fp64_svds_per_s"]
        h.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=2.0)
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--max-order", type=int, default=8192)
    ap.add_argument("--no-baseline", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.requests, a.rate, a.seed, a.workers, one_at_a_time=not a.no_baseline,
                         max_order=a.max_order)))


if __name__ == "__main__":
    main()
