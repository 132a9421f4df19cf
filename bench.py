"""Benchmark: seconds per singular-value decomposition of one n x n matrix.

Headline workload (the precision configuration of the tiled SVD): n = 16384,
tile 256, i.i.d. N(0, 1/n) entries from a seeded generator, FP32 tiles with
the trailing compact-WY updates on the tensor cores in split BF16 (three BF16
products per product, FP32 accumulation: FP32-class accuracy, stated against
the plain FP64 GPU path).  Every timed step runs the whole path -- copy of the
input into the workspace, GE2BND, bulge chase, bisection -- on an input
already resident in HBM (1 GiB per matrix, larger than L2).  ``e2e`` times the
same call through the host C-ABI entry point (avs_svdvals_s: host matrix in,
host singular values out, copies inside the timed region).

Also reported (single GPU): ``modes`` -- the other precision modes (split
TF32, TF32, BF16, FP32 SIMT) with their singular-value errors; ``plain_fp64``
-- the plain FP64 GPU path on the same matrix; ``batched`` -- 4096 FP32
matrices of orders drawn from {64..1024} in one batched call against one call
per matrix; ``serving`` -- a bounded Poisson request stream through the
serving loop (avs.Server) with p50/p99 latency; ``cpu_baseline`` -- the oracle
(a C restatement of the reference's CPU path) on a bounded sample.

``--impl reference`` times the reference's path on the host CPU instead: the
oracle (Blockbidiag! + bidiagonalize + the bidiagonal singular values, OpenMP
on all host threads) on a bounded sample of the same workload (n = 2048, same
tile), scaled to n by n^3.

One JSON line is printed by rank 0.  Several GPUs: one process per GPU, each
running independent SVDs (the path does not shard: replicas only).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "avocado-sandwich_gb300"))
sys.path.insert(0, REPO)

METRIC = "s_per_svd"
UNIT = "s/SVD"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--tile", type=int, default=256)
    p.add_argument("--precision", default="bf16x3")
    p.add_argument("--e2e-steps", type=int, default=1)
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    p.add_argument("--no-modes", action="store_true", help="skip the other precision modes")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-ooc", action="store_true", help="skip the out-of-core run")
    p.add_argument("--ooc-budget-mb", type=int, default=512)
    p.add_argument("--batch-count", type=int, default=4096)
    p.add_argument("--serve-requests", type=int, default=120)
    p.add_argument("--serve-rate", type=float, default=12.0)
    p.add_argument("--cpu-sample-n", type=int, default=2048)
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_desc(args):
    return {"workload": "svdvals n=%d tile=%d N(0,1/n) seed 4" % (args.n, args.tile), "n": args.n,
            "tile": args.tile, "precision": args.precision, "matrices_per_step": 1,
            "l2": "inputs larger than L2 (%.2f GiB per matrix)" % (args.n * args.n * 4 / 2**30)}


def cpu_sample(args, steps=1):
    """Oracle on n = cpu_sample_n (same tile, same distribution), scaled by n^3."""
    import oracle
    from avs import workloads
    ns = min(args.cpu_sample_n, args.n)
    b = min(args.tile, ns)
    a = workloads.gaussian(ns, 4, 1.0 / np.sqrt(ns), dtype=np.float32)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        oracle.svdvals(a, b, rel_tol=1e-12)
        times.append(time.perf_counter() - t0)
    scale = (args.n / ns) ** 3
    t = float(np.median(times))
    out = {"value": t * scale, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
           "sample": "oracle (C restatement of Blockbidiag! + bidiagonalize + bidiagonal singular values), "
                     "n=%d tile %d float32, %d run(s), median %.2f s, scaled by (%d/%d)^3 (extrapolated)"
                     % (ns, b, steps, t, args.n, ns)}
    # stage-2 comparator: LAPACK dgbbrd (the reference BRD code's, bulgechasing2.jl:142-170)
    from oracle import lapack
    if lapack.available():
        rng = np.random.default_rng(4)
        full = rng.standard_normal((ns, ns))
        band = np.triu(full) - np.triu(full, b + 1)
        t0 = time.perf_counter()
        lapack.gbbrd(band, b)
        tg = time.perf_counter() - t0
        out["stage2_lapack_dgbbrd"] = {"n": ns, "bw": b, "s": tg, "s_scaled_to_n": tg * (args.n / ns) ** 2,
                                       "note": "OpenBLAS (scipy's) dgbbrd, one thread of the host; band reduction "
                                               "is O(n^2 b), scaled by (n/%d)^2 (extrapolated)" % ns}
    return out


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def load_traffic():
    p = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return {}
    return {}


def update_flops(n, b):
    """Flops of the tensor-core trailing updates of one GE2BND (all half-steps):
    S_p = Y_p^T A_p and A_p -= Y_p W_p (2 b^2 ntr each per tile), the chain
    products T_p^T Z (b^2 ntr, triangular) and Y0 W0 (b^2 ntr, triangular)."""
    nt = n // b
    total = 0
    for k in range(nt - 1):
        ntr = n - (k + 1) * b
        for P in (nt - k, nt - k - 1):  # QR half-step k, LQ half-step k
            total += 2 * b * b * ntr * P + 2 * b * b * ntr * (P - 1) + b * b * ntr * (P + 1)
    return float(total)


def roofline(args, stage_ms, update_ms):
    """Roofline of the dominant kernel of the step.  Stage times are CUDA-event
    durations on the launching stream, averaged over the timed steps: stage 2
    is one launch of the bulge-chase kernel (plus two copy kernels under 0.5%
    of it), stage 3 one bisection launch, stage 1 the GE2BND launch sequence."""
    n, b = args.n, args.tile
    hbm, bf16, src = load_peaks()
    traffic = load_traffic()
    dom = max(stage_ms, key=stage_ms.get)
    t = stage_ms[dom] / 1e3
    if dom == "stage1":
        flops = 8.0 / 3.0 * n ** 3
        ach = flops / t / 1e12
        return {"bound": "tensor", "kernel": "ge2bnd (panels + trailing WY updates)", "achieved": ach,
                "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16, "traffic": traffic.get("stage1"),
                "algorithmic": "(8/3) n^3 flops per SVD", "peak_source": src + " bf16 dense (burst), of measured"}
    if dom == "stage2":
        byts = n * (b + 1) * 8.0 + 2 * n * 8.0
        ach = byts / t / 1e9
        return {"bound": "hbm", "kernel": "chase_cluster_kernel (band -> bidiagonal, double-float)",
                "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "traffic": traffic.get("stage2"),
                "algorithmic": "n(b+1)*8 band bytes read + 16n bidiagonal bytes written per launch (one launch "
                               "per SVD)", "peak_source": src + " HBM copy, of measured",
                "note": "the chase is latency-bound (sweep wavefront, dependent reflector steps); its band "
                        "(n*3b*8 bytes) stays in L2"}
    byts = 2 * n * 8.0
    ach = byts / t / 1e9
    return {"bound": "hbm", "kernel": "bisect_df_kernel (Sturm counts)", "achieved": ach, "peak": hbm,
            "unit": "GB/s", "frac": ach / hbm, "traffic": traffic.get("stage3"),
            "algorithmic": "2n*8 bytes per launch", "peak_source": src + " HBM copy, of measured"}


def tensor_roofline(args, update_ms):
    """Achieved rate of the tensor-core trailing updates (TMA-fed tcgen05 GEMMs
    + chain) against the measured dense bf16 peak; split modes run three
    products per product, so their tensor work is 3x the algorithmic flops."""
    if not update_ms:
        return None
    hbm, bf16, src = load_peaks()
    flops = update_flops(args.n, args.tile)
    mult = 3.0 if args.precision in ("tf32x3", "bf16x3") else 1.0
    ach = flops / (update_ms / 1e3) / 1e12
    return {"kernels": "ycopy + gemm_kernel (S = Y^T A) + chain_tc_kernel + gemm_kernel (A -= Y W), per half-step",
            "algorithmic_tflop": flops / 1e12, "ms": update_ms, "achieved": ach, "tensor_products": mult,
            "tensor_rate": ach * mult, "peak": bf16, "unit": "TFLOP/s", "frac": ach * mult / bf16,
            "peak_source": src + " bf16 dense (burst), of measured; TF32 runs at half the bf16 rate"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    for _ in range(args.warmup):
        pass  # the CPU path has no warm-up state; each step is a fresh oracle run
    t0 = time.perf_counter()
    cb = cpu_sample(args, steps=args.steps)
    total = time.perf_counter() - t0
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / max(args.steps, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic N(0,1/n), PCG64 seed 4",
            "config": workload_desc(args), "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_modes(args, A, h, s64):
    """The other precision modes on the same matrix: one warm-up, one timed call."""
    import avs
    out = {}
    for p in ("tf32x3", "tf32", "bf16x3", "bf16", "fp32"):
        if p == args.precision:
            continue
        r = avs.Report()
        avs.my_CU_svdval(A, args.tile, precision=p, report=r, handle=h)
        s = avs.my_CU_svdval(A, args.tile, precision=p, report=r, handle=h).double().cpu().numpy()
        d = {"s_per_svd": r.t_total_ms / 1e3,
             "stage_ms": {"stage1": r.t_stage1_ms, "stage2": r.t_stage2_ms, "stage3": r.t_stage3_ms}}
        if s64 is not None:
            d["max_abs_err_over_sigma_max_vs_fp64"] = float(np.max(np.abs(s - s64)) / s64[0])
        out[p] = d
    return out


def run_batched(args, h):
    """Many-matrices workload: `count` FP32 N(0, 1/n) matrices, orders drawn
    uniformly from {64, 128, 256, 512, 1024} (seed 5), tiles from the autotuner,
    one batched call; against one call per matrix (a seeded sample, scaled)."""
    import torch
    import avs
    from avs import workloads
    sizes = workloads.batch_sizes(args.batch_count, 5)
    g = torch.Generator(device="cuda").manual_seed(5)
    mats = [torch.randn((int(m), int(m)), generator=g, device="cuda") / np.sqrt(m) for m in sizes]
    tiles = {int(m): avs.autotune_tile(int(m), handle=h) for m in sorted(set(int(x) for x in sizes))}
    r = avs.Report()
    avs.svdvals_batched(mats, tiles=[tiles[int(m)] for m in sizes], report=r, handle=h)  # graph capture
    torch.cuda.synchronize()
    times, dev = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        outs = avs.svdvals_batched(mats, tiles=[tiles[int(m)] for m in sizes], report=r, handle=h)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        dev.append(r.t_total_ms / 1e3)
    wall = float(np.median(times))
    # one call per matrix, FP32 and plain FP64, on a seeded sample of the same list
    rng = np.random.default_rng(6)
    idx = rng.choice(len(mats), size=min(256, len(mats)), replace=False)
    for i in idx[:4]:
        avs.my_CU_svdval(mats[i], tiles[int(sizes[i])], handle=h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in idx:
        avs.my_CU_svdval(mats[i], tiles[int(sizes[i])], handle=h)
    torch.cuda.synchronize()
    one32 = (time.perf_counter() - t0) / len(idx) * len(mats)
    idx64 = idx[:64]
    m64 = {int(i): mats[i].double() for i in idx64}
    t0 = time.perf_counter()
    for i in idx64:
        avs.my_CU_svdval(m64[int(i)], tiles[int(sizes[i])], handle=h)
    torch.cuda.synchronize()
    one64 = (time.perf_counter() - t0) / len(idx64) * len(mats)
    err = 0.0
    for i in idx[:16]:
        ref = np.linalg.svd(mats[i].double().cpu().numpy(), compute_uv=False)
        err = max(err, float(np.max(np.abs(outs[i].double().cpu().numpy() - ref)) / ref[0]))
    return {"workload": "%d FP32 matrices, orders uniform over {64,128,256,512,1024} (seed 5), N(0,1/n)"
                        % len(mats),
            "tiles": tiles, "svds_per_s": len(mats) / wall, "wall_s": wall, "device_s": float(np.median(dev)),
            "stage_s": {"stage1": r.t_stage1_ms / 1e3, "stage2": r.t_stage2_ms / 1e3, "stage3": r.t_stage3_ms / 1e3},
            "kernel_launches": int(r.kernel_launches),
            "one_at_a_time_fp32_svds_per_s": len(mats) / one32,
            "one_at_a_time_plain_fp64_svds_per_s": len(mats) / one64,
            "one_at_a_time_sample": "%d (FP32) and %d (FP64) matrices of the list, scaled" % (len(idx), len(idx64)),
            "speedup_vs_one_at_a_time_plain_fp64": one64 / wall,
            "max_rel_sigma_err_vs_lapack_fp64": err, "checked": 16}


def run_ooc(args, a_host, s64, h):
    """Out-of-core form (OOC_SVD!) on the same matrix, kept in host memory and
    streamed through a device budget smaller than the matrix."""
    import avs
    budget = args.ooc_budget_mb << 20
    slab, used, incore_from = avs.ooc_plan(args.n, args.tile, np.float32, budget)
    a = np.asfortranarray(a_host.T)  # the headline's column-major matrix, host copy (overwritten)
    r = avs.Report()
    t0 = time.perf_counter()
    sig = avs.OOC_SVD(a, args.tile, device_bytes=budget, report=r, handle=h)
    wall = time.perf_counter() - t0
    out = {"workload": "OOC_SVD! of the headline matrix (FP32, host resident, %d MiB of device memory for a "
                       "%d MiB matrix)" % (args.ooc_budget_mb, args.n * args.n * 4 >> 20),
           "s_per_svd": wall, "stage_ms": {"stage1": r.t_stage1_ms, "stage2": r.t_stage2_ms,
                                           "stage3": r.t_stage3_ms},
           "slab_tile_rows": slab, "device_bytes": used, "in_core_from_step": incore_from,
           "n_steps": args.n // args.tile}
    if s64 is not None:
        out["max_abs_err_over_sigma_max_vs_fp64"] = float(np.max(np.abs(sig.astype(np.float64) - s64)) / s64[0])
    return out


def run_serving(args):
    from avs import serve_bench
    res = serve_bench.run(requests=args.serve_requests, rate=args.serve_rate, seed=7, workers=4, check=8,
                          one_at_a_time=True, baseline_every=3)
    res["note"] = ("bounded sample of the serving stream (orders log-uniform in [128, 8192], 70% FP32 / 30% "
                   "FP64, half Gaussian, half geometric spectrum); latency = completion - submission")
    return res


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    import avs
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    h = avs.Handle(local)
    n, b = args.n, args.tile
    h.reserve(n, b, args.precision)
    g = torch.Generator(device="cpu").manual_seed(4 + 1000 * rank)
    a_host = (torch.randn((n, n), generator=g, dtype=torch.float32) / np.sqrt(n)).numpy()
    A = torch.from_numpy(a_host).to(dev)  # the column-major matrix a_host.T (same singular values)
    rep = avs.Report()

    def step():
        return avs.my_CU_svdval(A, b, precision=args.precision, report=rep, handle=h)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    stage = {"stage1": 0.0, "stage2": 0.0, "stage3": 0.0}
    update_ms = 0.0
    launches = 0
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        start.record()
        for _ in range(args.steps):
            s = step()
            stage["stage1"] += rep.t_stage1_ms
            stage["stage2"] += rep.t_stage2_ms
            stage["stage3"] += rep.t_stage3_ms
            update_ms += rep.t_update_ms
            launches += rep.kernel_launches
        end.record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = start.elapsed_time(end)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    sigma = s.double().cpu().numpy()
    stage = {k: v / args.steps for k, v in stage.items()}
    update_ms /= args.steps

    # e2e: host matrix in, host sigma out, through avs_svdvals_s
    a_cm = np.asfortranarray(a_host.T)
    e2e_times = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        s_host = avs.my_CU_svdval(a_cm, b, precision=args.precision, handle=h)
        e2e_times.append(time.perf_counter() - t0)
    e2e = {"value": float(np.mean(e2e_times)) if e2e_times else None, "unit": UNIT,
           "h2d_bytes_per_step": int(n * n * 4), "d2h_bytes_per_step": int(n * 4), "steps": args.e2e_steps,
           "entry_point": "avs_svdvals_s (host pointers; copies inside)"}

    line = {"metric": METRIC, "value": ms / 1e3 / (args.steps * world), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision != "fp64" else "f64",
            "data": "synthetic N(0,1/n), PCG64-seeded torch generator (seed 4 + 1000*rank)",
            "config": dict(workload_desc(args), parallelism="replicas" if world > 1 else "single"),
            "stage_ms": stage, "roofline": roofline(args, stage, update_ms),
            "roofline_tensor_updates": tensor_roofline(args, update_ms), "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk.summary()}

    extras = rank == 0 and world == 1
    s64 = None
    if extras and not args.no_plain and args.precision != "fp64":
        # the plain FP64 GPU path on the same matrix: the accuracy reference of
        # the FP32-class modes (its own parity with LAPACK gesdd is in the tests)
        A64 = A.double()
        r64 = avs.Report()
        t0 = time.perf_counter()
        s64 = avs.my_CU_svdval(A64, b, precision="fp64", report=r64, handle=h).cpu().numpy()
        line["plain_fp64"] = {
            "s_per_svd": r64.t_total_ms / 1e3, "wall_s": time.perf_counter() - t0,
            "stage_ms": {"stage1": r64.t_stage1_ms, "stage2": r64.t_stage2_ms, "stage3": r64.t_stage3_ms},
            "speedup_of_headline_mode": (r64.t_total_ms / 1e3) / (ms / 1e3 / args.steps)}
        line["accuracy"] = {
            "vs": "plain FP64 GPU path", "mode": args.precision,
            "max_abs_err_over_sigma_max": float(np.max(np.abs(sigma - s64)) / s64[0]),
            "tolerance": 1e-5,
            "host_vs_device_max_diff": float(np.max(np.abs(s_host.astype(np.float64) - sigma)))}
        del A64
    if extras and not args.no_modes:
        line["modes"] = run_modes(args, A, h, s64)
    del A
    if extras and not args.no_ooc:
        line["out_of_core"] = run_ooc(args, a_host, s64, h)
    if extras and not args.no_batched:
        line["batched"] = run_batched(args, h)
    h.close()
    if extras and not args.no_serving:
        line["serving"] = run_serving(args)
    if extras and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(args, steps=1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
