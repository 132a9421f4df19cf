"""Benchmark: seconds per singular-value decomposition of one n x n matrix.

Workload (default): n = 16384, tile 256, i.i.d. N(0, 1/n) entries from a
seeded PCG64 generator (the precision configuration of the tiled SVD), FP32
tiles with the fastest precision mode that meets FP32-class accuracy.  Every
timed step runs the whole path -- copy of the input into the workspace,
GE2BND, bulge chase, bisection -- on an input already resident in HBM (1 GiB,
larger than L2).  ``e2e`` times the same call through the host C-ABI entry
point (avs_svdvals_s: host matrix in, host singular values out, copies inside
the timed region).

``--impl reference`` times the reference's path on the host CPU instead: the
oracle (a C restatement of the reference's Blockbidiag! + bidiagonalize + the
bidiagonal singular values, OpenMP on all host threads) on a bounded sample
of the same workload (n = 2048, same tile), scaled to n by n^3.

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
    p.add_argument("--precision", default="fp32")
    p.add_argument("--e2e-steps", type=int, default=1)
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
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
    return {"value": t * scale, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": "oracle (C restatement of Blockbidiag! + bidiagonalize + bidiagonal singular values), "
                      "n=%d tile %d float32, %d run(s), median %.2f s, scaled by (%d/%d)^3 (extrapolated)"
                      % (ns, b, steps, t, args.n, ns)}


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


def roofline(args, stage_ms):
    """Roofline of the dominant kernel of the step (stage times are CUDA-event
    durations on the launching stream, averaged over the timed steps)."""
    n, b = args.n, args.tile
    hbm, bf16, src = load_peaks()
    traffic = load_traffic()
    dom = max(stage_ms, key=stage_ms.get)
    t = stage_ms[dom] / 1e3
    if dom == "stage1":
        # GE2BND: (8/3) n^3 flops; the trailing compact-WY updates are the tensor-shaped work
        flops = 8.0 / 3.0 * n ** 3
        ach = flops / t / 1e12
        return {"bound": "tensor", "kernel": "ge2bnd (panel + trailing WY update)", "achieved": ach,
                "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16, "traffic": traffic.get("stage1"),
                "algorithmic": "(8/3) n^3 flops per SVD", "peak_source": src + " bf16 dense"}
    if dom == "stage2":
        # bulge chase: the band (n x (b+1) FP64) read once and the bidiagonal written once
        byts = n * (b + 1) * 8.0 + 2 * n * 8.0
        ach = byts / t / 1e9
        return {"bound": "hbm", "kernel": "chase_kernel (band -> bidiagonal, FP64)", "achieved": ach, "peak": hbm,
                "unit": "GB/s", "frac": ach / hbm, "traffic": traffic.get("stage2"),
                "algorithmic": "n(b+1)*8 + 16n bytes per SVD", "peak_source": src + " HBM copy",
                "note": "the chase is bound by FP64 issue and the sweep wavefront, not by bytes"}
    byts = 2 * n * 8.0
    ach = byts / t / 1e9
    return {"bound": "hbm", "kernel": "bisect_kernel (FP64 Sturm counts)", "achieved": ach, "peak": hbm,
            "unit": "GB/s", "frac": ach / hbm, "traffic": traffic.get("stage3"),
            "algorithmic": "2n*8 bytes per SVD", "peak_source": src + " HBM copy"}


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
            launches += rep.kernel_launches
        end.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    sigma = s.double().cpu().numpy()
    stage = {k: v / args.steps for k, v in stage.items()}

    # e2e: host matrix in, host sigma out, through avs_svdvals_s
    a_cm = np.asfortranarray(a_host.T)
    e2e_times = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        s_host = avs.my_CU_svdval(a_cm, b, precision=args.precision, handle=h)
        e2e_times.append(time.perf_counter() - t0)
    e2e = {"value": float(np.mean(e2e_times)) if e2e_times else None, "unit": UNIT, "h2d_bytes_per_step": int(n * n * 4),
           "d2h_bytes_per_step": int(n * 4), "steps": args.e2e_steps}

    # accuracy of this mode against the plain FP64 GPU path (whose parity with
    # LAPACK gesdd is covered by the tests)
    accuracy = None
    plain = None
    if not args.no_plain and args.precision != "fp64":
        A64 = A.double()
        r64 = avs.Report()
        t0 = time.perf_counter()
        s64 = avs.my_CU_svdval(A64, b, precision="fp64", report=r64, handle=h).cpu().numpy()
        plain = {"s_per_svd": r64.t_total_ms / 1e3, "wall_s": time.perf_counter() - t0,
                 "stage_ms": {"stage1": r64.t_stage1_ms, "stage2": r64.t_stage2_ms, "stage3": r64.t_stage3_ms},
                 "speedup_of_this_mode": (r64.t_total_ms / 1e3) / (ms / 1e3 / args.steps)}
        accuracy = {"vs": "plain FP64 GPU path", "max_abs_err_over_sigma_max":
                    float(np.max(np.abs(sigma - s64)) / s64[0]),
                    "host_vs_device_max_diff": float(np.max(np.abs(s_host.astype(np.float64) - sigma)))}
        del A64

    line = {"metric": METRIC, "value": ms / 1e3 / (args.steps * world), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision != "fp64" else "f64",
            "data": "synthetic N(0,1/n), PCG64-seeded torch generator (seed 4 + 1000*rank)",
            "config": dict(workload_desc(args), parallelism="replicas" if world > 1 else "single"),
            "stage_ms": stage, "roofline": roofline(args, stage), "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk.summary(), "accuracy": accuracy, "plain_fp64": plain}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(args, steps=1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    h.close()


if __name__ == "__main__":
    main()
