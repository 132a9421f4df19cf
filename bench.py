"""Benchmark: seconds per singular-value decomposition of one n x n matrix.

Headline workload (the precision configuration of the tiled SVD): n = 16384,
tile 256, i.i.d. N(0, 1/n) entries from numpy's PCG64 generator (seed 4,
rounded to float32; the CPU arm draws the same bytes), FP32 tiles with the
trailing compact-WY updates on the tensor cores in split BF16 (three BF16
products per product, FP32 accumulation: FP32-class accuracy, stated against
FP64 LAPACK dgesdd on the same matrix and against the plain FP64 GPU path).
Every timed step runs the whole path -- copy of the input into the workspace,
GE2BND, bulge chase, bisection -- on an input already resident in HBM (1 GiB
per matrix, larger than L2).  ``e2e`` times the same call through the host
C-ABI entry point (avs_svdvals_s: host matrix in, host singular values out,
copies inside the timed region).

Also reported (single GPU): ``modes`` -- the other precision modes with their
singular-value errors, and the headline mode with FP64 stages 2 and 3;
``plain_fp64`` -- the plain FP64 GPU path on the same matrix; ``batched`` --
4096 FP32 matrices of orders drawn from {64..1024} in one batched call against
one call per matrix; ``serving`` -- a bounded Poisson request stream through
the serving loop (avs.Server) with p50/p99 latency, every result checked;
``cpu_baseline`` -- the reference's CPU path (BandBidiagonal! with LAPACK on
stacked tile pairs, bidiagonalize, LAPACK dbdsdc) timed stage by stage on a
bounded sample and extrapolated per stage.

``--impl reference`` times that CPU path alone (one bounded sample per step).

One JSON line is printed by rank 0.  Several GPUs: one process per GPU, each
running independent SVDs (the path does not shard: replicas only).
"""
import argparse
import hashlib
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
FLOOR = 1e-3  # per-value relative errors are stated for sigma_i >= FLOOR * sigma_max
FIXTURE = os.path.join(REPO, "tests", "golden", "sigma_n16384_seed4.npz")
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (nominal; no measured figure on this machine)


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
    p.add_argument("--serve-rate", type=float, default=0.0, help="offered rate (req/s); 0 = 80%% of capacity")
    p.add_argument("--cpu-sample-n", type=int, default=2048)
    p.add_argument("--cpu-1core-n", type=int, default=1024)
    p.add_argument("--ref-sample-n", type=int, default=1024)
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_desc(args):
    return {"workload": "svdvals n=%d tile=%d N(0,1/n) numpy PCG64 seed 4, float32" % (args.n, args.tile),
            "n": args.n, "tile": args.tile, "precision": args.precision, "matrices_per_step": 1,
            "l2": "inputs larger than L2 (%.2f GiB per matrix)" % (args.n * args.n * 4 / 2**30)}


def errors(got, ref, floor=FLOOR):
    """Normwise max|d sigma| / sigma_max and the max per-value relative error
    over sigma_i >= floor * sigma_max."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if ref.size == 0 or ref[0] == 0:
        return {"normwise": float(np.max(np.abs(got - ref))) if ref.size else 0.0, "per_value": 0.0,
                "floor": floor}
    m = ref >= floor * ref[0]
    return {"normwise": float(np.max(np.abs(got - ref)) / ref[0]),
            "per_value": float(np.max(np.abs(got[m] - ref[m]) / ref[m])), "floor": floor}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's CPU path, stage by stage.

def cpu_stage_sample(n, b, threads, seed=4):
    from avs import workloads
    from oracle import cpu_baseline
    a = workloads.gaussian(n, seed, 1.0 / np.sqrt(n), dtype=np.float32)
    _, ts = cpu_baseline.run(a, b, threads=threads)
    return ts


def extrapolate(ts, ns, n):
    """Per-stage extrapolation from order ns to n at the same tile: stage 1
    (band reduction, (8/3) n^3 class) by (n/ns)^3, stages 2 (chase, n^2 b
    class) and 3 (dbdsdc, values only) by (n/ns)^2."""
    r = n / ns
    return {"stage1": ts["stage1"] * r ** 3, "stage2": ts["stage2"] * r ** 2, "stage3": ts["stage3"] * r ** 2}


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline(args):
    """The reference's CPU path on all host cores (median of 3 at n = cpu_sample_n,
    after one warm-up at a small size) and on one core (n = cpu_1core_n),
    extrapolated per stage to the headline n."""
    cores = host_cores()
    b = args.tile
    ns = min(args.cpu_sample_n, args.n)
    cpu_stage_sample(min(512, ns), min(b, 512), cores)  # warm-up (library load, threads)
    runs = [cpu_stage_sample(ns, min(b, ns), cores) for _ in range(3)]
    med = {k: float(np.median([r[k] for r in runs])) for k in runs[0]}
    ext = extrapolate(med, ns, args.n)
    total = sum(ext.values())
    n1 = min(args.cpu_1core_n, args.n)
    one = cpu_stage_sample(n1, min(b, n1), 1)
    one_ext = extrapolate(one, n1, args.n)
    from oracle import cpu_baseline as cbm
    cbm.blas_threads(cores)
    return {"value": total, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "reference CPU path restated: BandBidiagonal!(onGPU=false) (LAPACK dgeqrt/dgemqrt on stacked "
                      "2b x b tile pairs, scipy's OpenBLAS, float64) + bidiagonalize (C restatement, OpenMP) + "
                      "LAPACK dbdsdc; n=%d tile %d float32 input, median of 3 runs on %d threads, extrapolated per "
                      "stage to n=%d (stage 1 by n^3, stages 2-3 by n^2)" % (ns, min(b, ns), cores, args.n),
            "stage_s_sample": med, "stage_s_extrapolated": ext, "sample_n": ns, "extrapolated": True,
            "one_core": {"value": sum(one_ext.values()), "sample_n": n1, "stage_s_sample": one,
                         "stage_s_extrapolated": one_ext}}


def run_reference(args):
    """Reference arm: the reference's CPU path on this machine's host cores, one
    bounded sample (n = ref_sample_n, same tile) per step, extrapolated per
    stage to the headline n."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = host_cores()
    ns = min(args.ref_sample_n, args.n)
    b = min(args.tile, ns)
    for _ in range(args.warmup):
        cpu_stage_sample(ns, b, cores)
    t0 = time.perf_counter()
    vals, stages = [], []
    for _ in range(args.steps):
        ts = cpu_stage_sample(ns, b, cores)
        stages.append(ts)
        vals.append(sum(extrapolate(ts, ns, args.n).values()))
    total = time.perf_counter() - t0
    v = float(np.median(vals))
    med = {k: float(np.median([s[k] for s in stages])) for k in stages[0]}
    cb = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
          "sample": "reference CPU path restated (BandBidiagonal!(onGPU=false) with LAPACK, bidiagonalize, "
                    "dbdsdc), n=%d tile %d per step, median over steps, extrapolated per stage to n=%d "
                    "(stage 1 by n^3, stages 2-3 by n^2)" % (ns, b, args.n),
          "stage_s_sample": med, "stage_s_extrapolated": extrapolate(med, ns, args.n), "extrapolated": True}
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / max(args.steps, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic N(0,1/n), numpy PCG64 seed 4 (the GPU arm's bytes at the sample size)",
            "config": workload_desc(args), "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Clocks, peaks, rooflines.

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


def chase_flops(n, bw):
    """Exact flop count of the bulge chase (chase_cluster_kernel) on an n x n
    band of width bw.  Sweep j, step m: pivot row rho (j, then j + 1 + (m-1) bw),
    columns c0 = j + 1 + m bw .. c1 = min(c0 + bw - 1, n - 1), L = c1 - c0 + 1.
    R op: the reflector (3L) and, for each row rho+1 .. c1, a dot product and
    an update over L columns (4L); L op: the reflector (3L) and, for each
    column c0+1 .. min(c0 + 2 bw - 1, n - 1), 4L.  Sum over j, m with L >= 2
    of 4L (rows + cols) + 6L (~ 8 n^2 bw)."""
    total = 0
    for j in range(n - 1):
        nsteps = (n - j - 2) // bw + 1
        m = np.arange(nsteps)
        rho = np.where(m == 0, j, j + 1 + (m - 1) * bw)
        c0 = j + 1 + m * bw
        c1 = np.minimum(c0 + bw - 1, n - 1)
        L = c1 - c0 + 1
        rows = c1 - rho
        cols = np.minimum(c0 + 2 * bw - 1, n - 1) - c0
        total += int(np.sum(np.where(L >= 2, 4 * L * (rows + cols) + 6 * L, 0)))
    return float(total)


def _panel_qr_flops(m, t):
    """Householder QR of an m x t panel (m rows, t reflectors): per reflector k
    the norm (2(m-k)), its application to the t-k-1 columns right of it
    (4(m-k) each) and the Gram column v_j^T v_k of the compact-WY factor (2(m-k)
    for each j < k), plus the factor's recurrence (k^2)."""
    k = np.arange(min(t, max(m - 1, 0)))
    mk = m - k
    return float(np.sum(2 * mk + 4 * mk * (t - k - 1) + 2 * mk * k + k * k))


def band_stage_flops(n, bw, tbw):
    """Algorithmic flops of the blocked band reduction bw -> tbw (stage2_band.cu,
    the reference's bidiag! stage): per sweep s (rows p = s tbw ..) and step m
    (c0 = p + tbw + m bw), the R op -- QR of the L x tbw panel (L = min(bw, n -
    c0)) and the compact-WY apply to its Mr = min(c0 + bw, n) - rho - tbw rows:
    W = A V (2 Mr L tbw), Y = W T (Mr tbw^2), A -= Y V^T (2 Mr L tbw) -- and the
    L op -- QR of the L x tbw panel and the apply to Mc = min(c0 + 2bw, n) - c0 -
    tbw columns (4 L Mc tbw + Mc tbw^2).  About 8 n^2 bw."""
    total = 0.0
    nsw = (n - 2 - tbw) // tbw + 1 if n - 2 - tbw >= 0 else 0
    panel = {}
    for sw in range(nsw):
        p = sw * tbw
        nsteps = (n - 2 - p - tbw) // bw + 1
        m = np.arange(nsteps)
        c0 = p + tbw + m * bw
        L = np.minimum(bw, n - c0)
        rho = np.where(m == 0, p, c0 - bw)
        mr = np.minimum(c0 + bw, n) - rho - tbw
        mc = np.maximum(np.minimum(c0 + 2 * bw, n) - c0 - tbw, 0)
        total += float(np.sum(4.0 * mr * L * tbw + mr * tbw * tbw + 4.0 * L * mc * tbw + mc * tbw * tbw))
        for l_ in L:
            l_ = int(l_)
            if l_ not in panel:
                panel[l_] = _panel_qr_flops(l_, tbw)
            total += 2 * panel[l_]
    return total


NARROW_BAND = 16  # the hierarchical stage 2 reduces the band to this width, then chases it


def chase_roofline(args, chase_ms, bw, fp64_stages=False, kernel="chase_win_kernel (band 16 -> bidiagonal)"):
    """Roofline of the element bulge chase against its measured compute roof:
    the chase's arithmetic (double-float compensated dots and updates) from
    registers on every SM (avs_measure_chase_rate).  Its band (n x 3 bw x 8
    bytes) stays in L2 and shared memory, so HBM bytes are reported beside it,
    not as the bound."""
    import avs
    hbm, _, src = load_peaks()
    n = args.n
    flops = chase_flops(n, bw)
    peak = avs.chase_rate(0, fp64=fp64_stages) / 1e12
    t = chase_ms / 1e3
    ach = flops / t / 1e12
    byts = n * (bw + 1) * 8.0 + 2 * n * 8.0
    return {"bound": "compute (double-float on the FP32 pipe)" if not fp64_stages else "compute (FP64)",
            "kernel": kernel, "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "traffic": load_traffic().get("chase"), "ms": chase_ms,
            "algorithmic": "chase_flops(n, bw) = sum over sweeps j and steps m of 4L(rows + cols) + 6L = %.4e flops "
                           "per launch (n=%d, band %d), one launch per SVD, over the chase's event time"
                           % (flops, n, bw),
            "peak_source": "measured: avs_measure_chase_rate (the chase's df64 arithmetic from registers, all SMs)",
            "hbm": {"algorithmic_bytes": byts, "achieved_gbs": byts / t / 1e9, "peak_gbs": hbm,
                    "frac": byts / t / 1e9 / hbm, "peak_source": src + " HBM copy",
                    "note": "band stays in L2 / shared memory; HBM is not the bound"}}


def band_roofline(args, band_ms, tbw=NARROW_BAND):
    """Roofline of the blocked band reduction tile -> tbw (band_stage_kernel,
    FP32 SIMT compact-WY applies) against the measured FP32 rate."""
    import avs
    flops = band_stage_flops(args.n, args.tile, tbw)
    peak = avs.chase_rate(0, arith="fp32") / 1e12
    ach = flops / (band_ms / 1e3) / 1e12
    return {"bound": "compute (FP32 pipe)", "kernel": "band_stage_kernel (band %d -> %d)" % (args.tile, tbw),
            "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak, "ms": band_ms,
            "traffic": load_traffic().get("band_stage"),
            "algorithmic": "band_stage_flops(n, %d, %d) = %.4e flops per launch (panels, compact-WY factors, "
                           "W = A V, Y = W T, A -= Y V^T per op; about 8 n^2 b)" % (args.tile, tbw, flops),
            "peak_source": "measured: avs_measure_chase_rate(fp32) (FP32 FMA steps from registers, all SMs)"}


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


def gflops_report(args, seconds):
    """The usual convention for a bidiagonal reduction: (8/3) n^3 flops per SVD
    over the whole SVD's time, against the FP64 and TF32 compute roofs."""
    _, bf16, src = load_peaks()
    f = 8.0 / 3.0 * float(args.n) ** 3
    g = f / seconds / 1e9
    return {"gflops": g, "convention": "(8/3) n^3 flops per SVD / time per SVD",
            "frac_fp64_roof": g / (FP64_NOMINAL_TFLOPS * 1e3), "fp64_roof": "%.2f TFLOP/s nominal" % FP64_NOMINAL_TFLOPS,
            "frac_tf32_roof": g / (bf16 / 2 * 1e3),
            "tf32_roof": "%.0f TFLOP/s = half the %s bf16 dense rate" % (bf16 / 2, src)}


# ---------------------------------------------------------------------------
# Other legs.

def run_modes(args, A, h, s64, lapack):
    """The other precision modes on the same matrix (one warm-up, one timed call),
    and the headline mode with FP64 stages 2 and 3 (the bulge chase and the
    bisection in FP64 arithmetic)."""
    import avs
    out = {}
    legs = [(p, "auto") for p in ("tf32x3", "tf32", "bf16x3", "bf16", "fp32") if p != args.precision]
    legs.append((args.precision, "fp64"))
    for p, stages in legs:
        r = avs.Report()
        avs.my_CU_svdval(A, args.tile, precision=p, report=r, handle=h, stages=stages)
        s = avs.my_CU_svdval(A, args.tile, precision=p, report=r, handle=h, stages=stages).double().cpu().numpy()
        d = {"s_per_svd": r.t_total_ms / 1e3,
             "stage_ms": {"stage1": r.t_stage1_ms, "stage2": r.t_stage2_ms, "stage3": r.t_stage3_ms}}
        if s64 is not None:
            d["err_vs_plain_fp64_gpu"] = errors(s, s64)
        if lapack is not None:
            d["err_vs_lapack_dgesdd"] = errors(s, lapack)
        out[p if stages == "auto" else p + "+fp64_stages"] = d
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
    singles = {}
    for i in idx:
        singles[int(i)] = avs.my_CU_svdval(mats[i], tiles[int(sizes[i])], handle=h)
    torch.cuda.synchronize()
    one32 = (time.perf_counter() - t0) / len(idx) * len(mats)
    idx64 = idx[:64]
    m64 = {int(i): mats[i].double() for i in idx64}
    t0 = time.perf_counter()
    for i in idx64:
        avs.my_CU_svdval(m64[int(i)], tiles[int(sizes[i])], handle=h)
    torch.cuda.synchronize()
    one64 = (time.perf_counter() - t0) / len(idx64) * len(mats)
    # every sampled result: bit-identical to its single call, and within tolerance of LAPACK
    worst = {"normwise": 0.0, "per_value": 0.0, "floor": FLOOR}
    mismatch = 0
    for i in idx:
        got = outs[i].double().cpu().numpy()
        mismatch += int(not np.array_equal(outs[i].cpu().numpy(), singles[int(i)].cpu().numpy()))
        ref = np.linalg.svd(mats[i].double().cpu().numpy(), compute_uv=False)
        e = errors(got, ref)
        worst["normwise"] = max(worst["normwise"], e["normwise"])
        worst["per_value"] = max(worst["per_value"], e["per_value"])
    return {"workload": "%d FP32 matrices, orders uniform over {64,128,256,512,1024} (seed 5), N(0,1/n)"
                        % len(mats),
            "tiles": tiles, "svds_per_s": len(mats) / wall, "wall_s": wall, "device_s": float(np.median(dev)),
            "stage_s": {"stage1": r.t_stage1_ms / 1e3, "stage2": r.t_stage2_ms / 1e3, "stage3": r.t_stage3_ms / 1e3},
            "kernel_launches": int(r.kernel_launches),
            "one_at_a_time_fp32_svds_per_s": len(mats) / one32,
            "one_at_a_time_plain_fp64_svds_per_s": len(mats) / one64,
            "one_at_a_time_sample": "%d (FP32) and %d (FP64) matrices of the list, scaled" % (len(idx), len(idx64)),
            "speedup_vs_one_at_a_time_plain_fp64": one64 / wall,
            "err_vs_lapack_fp64": worst, "checked": int(len(idx)),
            "bitwise_vs_single_call_mismatches": mismatch}


def run_ooc(args, a_host, s64, h):
    """Out-of-core form (OOC_SVD!) on the same matrix, kept in host memory and
    streamed through a device budget smaller than the matrix."""
    import avs
    budget = args.ooc_budget_mb << 20
    slab, used, incore_from = avs.ooc_plan(args.n, args.tile, np.float32, budget)
    a = np.array(a_host, order="F")  # host copy of the headline matrix (overwritten in place)
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
        out["err_vs_plain_fp64_gpu"] = errors(sig, s64)
    return out


def run_serving(args):
    from avs import serve_bench
    res = serve_bench.run(requests=args.serve_requests, rate=args.serve_rate or None, seed=7, workers=4,
                          one_at_a_time=True, baseline_every=3, strict=False)
    res["note"] = ("bounded sample of the serving stream (orders log-uniform in [128, 8192], 70% FP32 / 30% "
                   "FP64, half Gaussian, half geometric spectrum); latency = completion - submission")
    return res


def lapack_reference(args, a):
    """FP64 LAPACK dgesdd singular values of the headline matrix, from the
    committed fixture, when this is that matrix (n, seed, SHA-256 of the bytes)."""
    if args.n != 16384 or not os.path.exists(FIXTURE):
        return None
    fx = np.load(FIXTURE)
    h = hashlib.sha256(np.ascontiguousarray(a).tobytes(order="F")).hexdigest()
    return fx["sigma"] if h == str(fx["sha256"]) else None


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    import avs
    from avs import workloads
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    h = avs.Handle(local)
    n, b = args.n, args.tile
    h.reserve(n, b, args.precision)
    a_host = workloads.gaussian(n, 4 + 1000 * rank, 1.0 / np.sqrt(n), dtype=np.float32)  # Fortran order
    A = avs.to_device(a_host, local)  # the column-major matrix a_host on the device
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
    band_ms = 0.0
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
            band_ms += rep.t_band_ms
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
    band_ms /= args.steps
    per_svd = ms / 1e3 / args.steps

    # e2e: host matrix in, host sigma out, through avs_svdvals_s
    e2e_times = []
    s_host = None
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        s_host = avs.my_CU_svdval(a_host, b, precision=args.precision, handle=h)
        e2e_times.append(time.perf_counter() - t0)
    e2e = {"value": float(np.mean(e2e_times)) if e2e_times else None, "unit": UNIT,
           "h2d_bytes_per_step": int(n * n * 4), "d2h_bytes_per_step": int(n * 4), "steps": args.e2e_steps,
           "entry_point": "avs_svdvals_s (host pointers; copies inside)"}

    line = {"metric": METRIC, "value": per_svd / world, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision != "fp64" else "f64",
            "data": "synthetic N(0,1/n), numpy PCG64 seed 4 + 1000*rank, rounded to float32",
            "config": dict(workload_desc(args), parallelism="replicas" if world > 1 else "single"),
            "stage_ms": stage, "gpu_launches": int(launches), "clocks": clk.summary(), "e2e": e2e}
    hier = band_ms > 0.0
    chase_ms = stage["stage2"] - band_ms
    if rank == 0:
        chase = chase_roofline(args, chase_ms, NARROW_BAND if hier else args.tile,
                               kernel="chase_win_kernel (band %d -> bidiagonal)" % NARROW_BAND if hier
                               else "chase_cluster_kernel (band %d -> bidiagonal)" % args.tile)
        line["roofline"] = chase
        if hier:
            line["roofline_band_stage"] = band_roofline(args, band_ms)
    line["dominant_stage"] = max(stage, key=stage.get)
    line["stage2_split_ms"] = {"band_reduction": band_ms, "element_chase": chase_ms}
    line["roofline_tensor_updates"] = tensor_roofline(args, update_ms)
    line["gflops"] = gflops_report(args, per_svd)

    extras = rank == 0 and world == 1
    s64 = None
    lapack = lapack_reference(args, a_host) if extras else None
    acc = {"mode": args.precision, "tolerance_normwise": 1e-5,
           "host_vs_device_max_diff": (float(np.max(np.abs(s_host.astype(np.float64) - sigma)))
                                       if s_host is not None else None)}
    if lapack is not None:
        acc["vs_lapack_dgesdd"] = errors(sigma, lapack)
        acc["lapack_source"] = "tests/golden/sigma_n16384_seed4.npz (dgesdd on the same float32 matrix, SHA-256 checked)"
    if extras and not args.no_plain and args.precision != "fp64":
        # the plain FP64 GPU path on the same matrix (its own parity with LAPACK
        # gesdd is in the tests, and against the fixture here)
        A64 = A.double()
        r64 = avs.Report()
        t0 = time.perf_counter()
        s64 = avs.my_CU_svdval(A64, b, precision="fp64", report=r64, handle=h).cpu().numpy()
        line["plain_fp64"] = {
            "s_per_svd": r64.t_total_ms / 1e3, "wall_s": time.perf_counter() - t0,
            "stage_ms": {"stage1": r64.t_stage1_ms, "stage2": r64.t_stage2_ms, "stage3": r64.t_stage3_ms},
            "speedup_of_headline_mode": (r64.t_total_ms / 1e3) / per_svd}
        if lapack is not None:
            line["plain_fp64"]["err_vs_lapack_dgesdd"] = errors(s64, lapack)
        acc["vs_plain_fp64_gpu"] = errors(sigma, s64)
        del A64
    line["accuracy"] = acc
    if extras and not args.no_modes:
        line["modes"] = run_modes(args, A, h, s64, lapack)
    del A
    if extras and not args.no_ooc:
        line["out_of_core"] = run_ooc(args, a_host, s64, h)
    if extras and not args.no_batched:
        line["batched"] = run_batched(args, h)
    h.close()
    if extras and not args.no_serving:
        line["serving"] = run_serving(args)
    if extras and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
