"""Serving benchmark: Poisson streams of SVD requests through ``avs.Server``.

Request mix (the serving workload of the reference's benchmark plan): square
orders log-uniform in [128, 8192] rounded to a power of two, 70% float32 / 30%
float64, half Gaussian N(0, 1/n) and half with a prescribed geometric spectrum
(sigma_i from 1 down to 1e-6).  Inputs come from a seeded pool (a few matrices
per order and kind, generated once and kept in host memory), so the stream
itself costs no generation time.

1. Capacity: the whole request list submitted at once; SVDs/s of the server
   saturated.
2. Load-latency curve: Poisson arrivals at fractions of that capacity (50% and
   80% by default, sustainable loads), p50/p99 latency per load.
3. Parity of every request of every stream: bit-identical to the single-matrix
   call on the same matrix (the server's tile and precision mode for it,
   avs_serve_plan), and within tolerance
   (FP32 1e-5, FP64 1e-12, normwise) of an FP64 reference for that matrix --
   LAPACK dgesdd for n <= 2048, the prescribed spectrum for the geometric
   matrices, and the plain FP64 GPU path (itself held to 1e-12 of known spectra
   in the tests) for the larger Gaussian ones.
4. One-at-a-time baselines: the same request list through blocking calls, in
   each request's precision (the server's mode for it) and through the plain
   FP64 path.

    python -m avs.serve_bench --requests 200
"""
import argparse
import json
import threading
import time

import numpy as np

import avs
from avs import workloads

ORDERS = (128, 256, 512, 1024, 2048, 4096, 8192)
TOL = {"f32": 1e-5, "f64": 1e-12}
FLOOR = 1e-3


class ParityError(AssertionError):
    pass


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
    """(n, f64, geometric, variant) -> (host matrix in Fortran order, exact sigma
    or None)."""
    pool = {}
    for key in sorted(set(reqs)):
        n, f64, geo, var = key
        dt = np.float64 if f64 else np.float32
        if geo:
            a, sig = workloads.geometric_spectrum(n, 20 + var, 40 + var, 1e-6, dtype=dt, device=device)
            pool[key] = (np.asfortranarray(a.cpu().numpy().T), sig)
        else:
            pool[key] = (workloads.gaussian(n, 1000 * n + var, 1.0 / np.sqrt(n), dtype=dt), None)
    return pool


def single_call(a, handle):
    """The single-matrix call a served request equals: the server's tile and
    precision mode for its order and type (avs_serve_plan)."""
    tile, mode, _ = avs.serve_plan(a.shape[0], a.dtype)
    return avs.my_CU_svdval(a, tile, precision=mode, handle=handle)


def errors(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    m = ref >= FLOOR * ref[0]
    return float(np.max(np.abs(got - ref)) / ref[0]), float(np.max(np.abs(got[m] - ref[m]) / ref[m]))


def stream(srv, reqs, pool, arrivals):
    """Submit reqs at the given arrival times (s from the start); wait for all."""
    ids = [None] * len(reqs)

    def submitter():
        t0 = time.perf_counter()
        for i, key in enumerate(reqs):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids[i] = srv.submit(pool[key][0])

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
    lats = np.sort(np.asarray(lats))
    return outs, {"svds_per_s": len(reqs) / wall, "wall_s": wall,
                  "p50_ms": float(np.percentile(lats, 50, method="higher")),
                  "p99_ms": float(np.percentile(lats, 99, method="higher")),
                  "mean_ms": float(np.mean(lats)), "max_ms": float(lats[-1])}


def references(pool):
    """Single-matrix call and FP64 reference sigma per pool key."""
    import scipy.linalg as sl
    single, ref, src = {}, {}, {}
    h = avs.Handle()
    for key, (a, exact) in pool.items():
        n = key[0]
        single[key] = single_call(a, h)
        if exact is not None:
            ref[key], src[key] = exact, "prescribed spectrum"
        elif n <= 2048:
            ref[key], src[key] = sl.svdvals(a.astype(np.float64), check_finite=False), "LAPACK dgesdd"
        else:
            ref[key] = avs.my_CU_svdval(np.asfortranarray(a.astype(np.float64)), avs.serve_plan(n, np.float64)[0],
                                        precision="fp64", handle=h)
            src[key] = "plain FP64 GPU path"
    h.close()
    return single, ref, src


def check(reqs, results, single, ref):
    """Every request of every stream against its single call (bitwise) and its
    reference (tolerance)."""
    worst = {"f32": [0.0, 0.0], "f64": [0.0, 0.0]}
    mismatches, breaches = 0, 0
    for outs in results:
        for key, s in zip(reqs, outs):
            k = "f64" if key[1] else "f32"
            mismatches += int(not np.array_equal(s, single[key]))
            e, p = errors(s, ref[key])
            breaches += int(e >= TOL[k])
            worst[k] = [max(worst[k][0], e), max(worst[k][1], p)]
    return {"requests_checked": sum(len(o) for o in results), "bitwise_mismatches_vs_single_call": mismatches,
            "tolerance_breaches": breaches, "tolerance": TOL,
            "max_err_normwise": {k: v[0] for k, v in worst.items()},
            "max_err_per_value": {k: v[1] for k, v in worst.items()}, "per_value_floor": FLOOR,
            "ok": mismatches == 0 and breaches == 0}


def run(requests=120, rate=None, seed=7, workers=4, one_at_a_time=True, max_order=8192, baseline_every=1,
        strict=True, loads=(0.5, 0.8)):
    reqs = request_list(requests, seed, max_order)
    pool = make_pool(reqs)
    rng = np.random.default_rng(seed + 1)
    srv = avs.Server(workers=workers)
    # warm the slots (module load, first launches, graph captures of the group shapes)
    for key in sorted(pool):
        srv.wait(srv.submit(pool[key][0]))
    results = []
    outs, sat = stream(srv, reqs, pool, np.zeros(len(reqs)))
    results.append(outs)
    capacity = sat["svds_per_s"]
    curve = []
    for r in ([rate] if rate else [f * capacity for f in loads]):
        arrivals = np.cumsum(rng.exponential(1.0 / r, size=len(reqs)))
        outs, st = stream(srv, reqs, pool, arrivals)
        results.append(outs)
        curve.append(dict(st, offered_rps=r, load_fraction=r / capacity))
    stats = srv.stats()
    srv.close()
    single, ref, src = references(pool)
    parity = check(reqs, results, single, ref)
    head = curve[-1] if curve else sat
    res = {
        "requests": len(reqs), "workers": workers, "svds_per_s": capacity, "capacity": sat,
        "load_curve": curve, "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"],
        "latency_at": "offered %.2f req/s (%.0f%% of capacity)" % (head.get("offered_rps", capacity),
                                                                  100 * head.get("load_fraction", 1.0)),
        "server": stats, "parity": parity,
        "reference_sources": sorted(set(src.values())),
        "mix": {"f32": sum(1 for r in reqs if not r[1]), "f64": sum(1 for r in reqs if r[1]),
                "orders": {int(n): sum(1 for r in reqs if r[0] == n) for n in ORDERS if n <= max_order}},
    }
    if one_at_a_time:
        # the same request list, one blocking call at a time (no overlap, no batching):
        # (1) each request in its own precision, (2) every request through the
        # plain FP64 path (FP32 inputs widened on the host, outside the timing)
        # (every baseline_every-th request of the list, scaled to the list)
        sub = reqs[::max(1, baseline_every)]
        h = avs.Handle()
        for key in sorted(set(sub)):
            single_call(pool[key][0], h)
        t0 = time.perf_counter()
        for key in sub:
            single_call(pool[key][0], h)
        res["one_at_a_time_svds_per_s"] = len(sub) / (time.perf_counter() - t0)
        wide = {k: np.asfortranarray(v[0].astype(np.float64)) for k, v in pool.items() if k in set(sub)}
        t_sum = 0.0
        for key in sub:
            t0 = time.perf_counter()
            avs.my_CU_svdval(wide[key], avs.serve_plan(key[0], np.float64)[0], precision="fp64", handle=h)
            t_sum += time.perf_counter() - t0
        res["one_at_a_time_plain_fp64_svds_per_s"] = len(sub) / t_sum
        res["one_at_a_time_sample"] = "%d of the %d requests" % (len(sub), len(reqs))
        res["speedup_vs_one_at_a_time_plain_fp64"] = capacity / res["one_at_a_time_plain_fp64_svds_per_s"]
        h.close()
    if strict and not parity["ok"]:
        raise ParityError(json.dumps(parity))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=120)
    ap.add_argument("--rate", type=float, default=0.0, help="one offered rate (req/s) instead of the load curve")
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--max-order", type=int, default=8192)
    ap.add_argument("--no-baseline", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.requests, a.rate or None, a.seed, a.workers, one_at_a_time=not a.no_baseline,
                         max_order=a.max_order)))


if __name__ == "__main__":
    main()
