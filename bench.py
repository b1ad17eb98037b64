#!/usr/bin/env python3
"""Benchmark: phase-linked pixels per second on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): a synthetic
2048 x 2048 scene, N = 30 dates, half-window 5 x 10 (11 x 21 = 231 taps),
coherence gamma(dt) = 0.7 exp(-dt/24 d) + 0.2 on a 12-day grid, 8 amplitude
classes on seeded Voronoi cells, nmap = same-class neighbours (SHP counts
20..231), MLE with the reference evd semantics.  One step phase-links the
whole scene.

Forms: the headline form is the mixed-precision one (tensor-core BF16
hi/lo Gamma + FP32 eigen-solves, FP64 only where an FP32 decision is
ambiguous); the plain FP32 form is timed beside it in the same run
(``other_form``, ``mixed_over_fp32``).

value : px/s with the stack and nmap resident in HBM (device pointers, no
        copies in the timed region).  The 1 GB stack exceeds the 129 MB L2,
        so no L2 flush is needed between steps.
e2e   : px/s through the C ABI with pinned HOST buffers: every step copies the
        stack + nmap to the device and phase + tcorr + compressed SLC back.
kernels / roofline : per-kernel CUDA-event times on the launching stream;
        the roofline object describes the kernel with the largest share.
accuracy_vs_fp64 : phase RMS and temporal-coherence error of each form
        against the FP64 form of the same kernels over the whole scene, with
        validity-code mismatches counted separately.
cpu_baseline : the oracle port (CPU restatement of the reference loop) on the
        host cores, on a bounded row sample of the same scene.

Under torchrun each rank phase-links its own scene (weak scaling, no
data-path collective); value = all ranks' pixels / max-over-ranks time.
``--impl reference`` times the reference's CPU implementation of the path
(the oracle port; the reference's own LAPACK-linked build needs the reference
tree) on rank 0 only.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# LAPACK single-threaded inside the OpenMP pixel loop, as the reference's
# module scripts set it (src/evd/evd.py:43)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

NB, ROWS, COLS, NY, NX = 30, 2048, 2048, 5, 10
SEED = 1002
METRIC = "phase-linked px/s (N=30, 11x21)"


# what the ncu captures under profiles/ show for each kernel
# what the ncu captures under profiles/ show for each kernel
BOUND_NOTES = {
    "solve": "instruction issue (one warp per pixel; per-pixel FP32 factorisations, sweep inverse and "
             "triangular solves); DRAM and tensor pipe idle",
    "gram": "operand build on the CUDA cores with 8 warps/SM and a barrier per chunk; tensor pipe partly idle",
    "fp32": "per-pixel FP32 gather, Gamma and eigen-solves: latency/issue-bound",
}
# FP32 flops of the MLE eigen-solves per pixel as implemented, for n dates and
# `solves` pairs of triangular solves: the Cholesky test of C - 1e-6 I and the
# Cholesky of M - sigma I (n^3/6 complex multiply-adds each, 8 flops), the
# sweep inverse of the real |C| (n^3 multiply-adds, 2 flops), the start
# vector and Rayleigh quotient (5 complex matrix-vector products) and the
# inverse-iteration solves (n^2 complex multiply-adds per pair).
def solve_flops_per_px(n, solves):
    return 2 * (n ** 3 / 6.0) * 8 + n ** 3 * 2 + 5 * n * n * 8 + solves * n * n * 8


def kernel_counters():
    p = os.path.join(ROOT, "profiles", "kernel_counters.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--method", default="MLE", choices=["MLE", "EVD", "STBAS"])
    ap.add_argument("--precision", default="mixed", choices=["fp32", "mixed"],
                    help="headline form (the other form is timed beside it)")
    ap.add_argument("--no-compare", action="store_true", help="skip the other form")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the error statistics against the FP64 form")
    ap.add_argument("--rows", type=int, default=ROWS)
    ap.add_argument("--cols", type=int, default=COLS)
    ap.add_argument("--cpu-rows", type=int, default=0,
                    help="rows of the CPU-baseline sample (0 = auto)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the serving-loop measurement")
    ap.add_argument("--serve-jobs", type=int, default=24)
    ap.add_argument("--no-nmap", action="store_true", help="skip the SHP-map measurement")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched-ministack and ill-conditioned measurements")
    return ap.parse_args()


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def popcount_words(nmap):
    cnt = np.zeros(nmap.shape[:2], np.int64)
    for w in range(nmap.shape[2]):
        v = nmap[..., w].astype(np.uint64)
        c = v - ((v >> 1) & 0x55555555)
        c = (c & 0x33333333) + ((c >> 2) & 0x33333333)
        c = (((c + (c >> 4)) & 0x0F0F0F0F) * 0x01010101) >> 24
        cnt += (c & 0xFF).astype(np.int64)
    return cnt


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = str(device_index)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-i", self.idx, "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(stack, nmap, method, rows):
    """Oracle port on the host cores over rows [0, rows) of the scene; also
    returns the oracle's result for those rows (the parity check)."""
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    res = oracle.run(stack, nmap, NY, NX, method=method, rows=(0, rows), nthreads=threads)
    dt = time.perf_counter() - t0
    px = rows * stack.shape[2]
    return {"value": px / dt, "unit": "px/s", "cores": threads, "kind": "port",
            "sample": "rows 0..%d of the %dx%d scene (%d px), %s, evd semantics, %.1f s"
                      % (rows, stack.shape[1], stack.shape[2], px, method, dt)}, res


def parity_vs_oracle(gpu_out, ora, rows, tol):
    """Parity of one GPU form against the oracle over rows [0, rows) of the
    same scene: phase RMS / max (wrapped, over pixels valid in both), max
    |dtcorr|, validity-code mismatches, compressed-SLC error (in units of the
    oracle's mean |comp|) and whether each is within the stated tolerance."""
    sys.path.insert(0, ROOT)
    from tests.parity import COMP_RMS_TOL, compare
    g = {k: gpu_out[k][..., :rows, :].cpu().numpy() for k in ("phase", "tcorr", "comp")}
    o = {k: ora[k][..., :rows, :] for k in ("phase", "tcorr", "comp")}
    m = compare(g, o)
    tol = dict(tol, comp_rms=min(tol["phase_rms"], COMP_RMS_TOL))
    ok = (m["code_mismatch"] == 0 and m["phase_rms"] <= tol["phase_rms"] and m["tcorr_max"] <= tol["tcorr_max"]
          and m["comp_rms"] <= tol["comp_rms"] and m["zero_mismatch"] == 0 and m["comp_zero_mismatch"] == 0)
    return {"pixels_compared": m["valid_both"], "rows": "0..%d" % rows, "phase_rms_rad": m["phase_rms"],
            "phase_max_rad": m["phase_max"], "tcorr_max_abs": m["tcorr_max"],
            "code_mismatch_px": m["code_mismatch"], "comp_rms": m["comp_rms"], "comp_max": m["comp_max"],
            "skipped_not_zero_px": m["zero_mismatch"] + m["comp_zero_mismatch"],
            "tolerance": tol, "within_tolerance": bool(ok)}


def cpu_baseline_detail(stack, nmap, rows):
    """Oracle port on the host cores for both methods: the CPU-runnable
    configuration in full (200x200, N = 10, half-window 5x5, all-ones SHP
    map) in EVD and MLE, and EVD over rows [0, rows) of the headline scene
    (its MLE sample is the main cpu_baseline).  A few seconds in all."""
    import oracle
    from fringe_gb300 import synth
    threads = os.cpu_count() or 1
    res = {"cores": threads, "kind": "port"}
    st1, nm1 = synth.scene("uniform", 200, 200, 10, 5, 5, seed=1001)
    for method in ("EVD", "MLE"):
        t0 = time.perf_counter()
        oracle.run(st1, nm1, 5, 5, method=method, nthreads=threads)
        dt = time.perf_counter() - t0
        res["uniform200_n10_%s" % method.lower()] = {"value": 200 * 200 / dt, "unit": "px/s",
                                                     "sample": "whole 200x200 scene, %.2f s" % dt}
    t0 = time.perf_counter()
    oracle.run(stack, nmap, NY, NX, method="EVD", rows=(0, rows), nthreads=threads)
    dt = time.perf_counter() - t0
    res["voronoi_n30_evd"] = {"value": rows * stack.shape[2] / dt, "unit": "px/s",
                              "sample": "rows 0..%d of the %dx%d scene, %.1f s" % (rows, stack.shape[1],
                                                                                    stack.shape[2], dt)}
    return res


def serving_measurement(njobs, seed=5):
    """Serving loop on a mix of jobs: tiles 256^2..2048^2, N in 10..60,
    half-windows 3x3..5x10, MLE/EVD, in the mixed-precision form and in the
    plain FP32 form.  Per form: (1) all jobs submitted at once (saturating
    load): throughput and p50/p99 latency; (2) Poisson arrivals at 30, 50, 70
    and 90% of the saturated job rate: p50/p99 latency, overall and per tile
    size."""
    from fringe_gb300 import synth
    from fringe_gb300.serve import Server
    shapes = [(256, 10, (3, 3)), (512, 30, (5, 10)), (1024, 20, (3, 5)), (512, 60, (5, 10)),
              (256, 45, (4, 8)), (1024, 30, (5, 10)), (2048, 30, (5, 10)), (2048, 15, (3, 3))]
    import torch

    def pinned(a):
        return torch.from_numpy(a).pin_memory().numpy()

    pool = []
    for k, (r, n, hw) in enumerate(shapes):
        st, nm = synth.scene("voronoi", r, r, n, hw[0], hw[1], seed=100 + k)
        pool.append((pinned(st), pinned(nm.view(np.int32)).view(np.uint32), hw))

    def outputs(p):
        nb, R, C = pool[p][0].shape
        return {"phase": torch.zeros((nb, R, C), dtype=torch.complex64).pin_memory().numpy(),
                "tcorr": torch.zeros((R, C), dtype=torch.float32).pin_memory().numpy(),
                "comp": torch.zeros((R, C), dtype=torch.complex64).pin_memory().numpy()}

    result = {"jobs": int(njobs),
              "mix": "tiles 256^2..2048^2, N 10..60, half-windows 3x3..5x10, MLE/EVD, 80 GB budget"}

    def by_size(picks, lat):
        out = {}
        for size in sorted({pool[p][0].shape[1] for p in picks}):
            sel = np.array([pool[p][0].shape[1] == size for p in picks])
            out["%dx%d" % (size, size)] = {"jobs": int(sel.sum()),
                                           "p50_ms": float(np.percentile(lat[sel], 50)),
                                           "p99_ms": float(np.percentile(lat[sel], 99))}
        return out
    for prec in ("mixed", "fp32"):
        rng = np.random.Generator(np.random.PCG64(seed))
        picks = rng.integers(0, len(pool), njobs)
        outs = [outputs(p) for p in picks]
        methods = rng.choice(["MLE", "EVD"], njobs)
        srv = Server(memory_budget=80 << 30, wave_pixels=1 << 20)
        # warm-up (kernel loading, allocator)
        st, nm, hw = pool[0]
        srv.wait(srv.submit(st, nm, hw, precision=prec))

        def run(arrivals):
            t0 = time.perf_counter()
            tickets = []
            for k in range(njobs):
                if arrivals is not None:
                    dt = arrivals[k] - (time.perf_counter() - t0)
                    if dt > 0:
                        time.sleep(dt)
                st, nm, hw = pool[picks[k]]
                tickets.append(srv.submit(st, nm, hw, method=str(methods[k]), out=outs[k], precision=prec))
            lat = [srv.wait(t)["total_ms"] for t in tickets]
            wall = time.perf_counter() - t0
            for t in tickets:
                srv.result(t)
            return wall, np.array(lat)

        px = float(sum(pool[p][0].shape[1] * pool[p][0].shape[2] for p in picks))
        wall, lat = run(None)
        rate_sat = njobs / wall
        sweep = []
        for frac in (0.3, 0.5, 0.7, 0.9):
            rate = frac * rate_sat
            arrivals = np.cumsum(rng.exponential(1.0 / rate, njobs))
            w, lat_p = run(arrivals)
            sweep.append({"load": frac, "rate_jobs_per_s": rate, "throughput_px_s": px / w,
                          "p50_ms": float(np.percentile(lat_p, 50)), "p99_ms": float(np.percentile(lat_p, 99)),
                          "by_tile": by_size(picks, lat_p)})
        srv.close()
        result["pixels"] = px
        result[prec] = {
            "saturated": {"throughput_px_s": px / wall, "jobs_per_s": rate_sat,
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "by_tile": by_size(picks, lat)},
            "poisson": sweep}
    return result


def run_reference(args, rank):
    """The reference's CPU implementation of the path on the host cores: the
    oracle loop linked to the reference's own EVWorker + LAPACK where that
    build exists (oracle/_ref), else the oracle port; each step phase-links
    a band of rows of the same scene (rank 0 only)."""
    if rank != 0:
        return
    from fringe_gb300 import synth
    stack, nmap = synth.scene("voronoi", args.rows, args.cols, NB, NY, NX, seed=SEED)
    import oracle
    kind = "port"
    try:
        oracle.load("reference")
        kind = "reference"
    except (FileNotFoundError, OSError):
        pass
    threads = os.cpu_count() or 1
    rows = args.cpu_rows or 16
    rows = min(rows, args.rows)
    for _ in range(args.warmup):
        oracle.run(stack, nmap, NY, NX, method=args.method, rows=(0, 2), nthreads=threads, kind=kind)
    t0 = time.perf_counter()
    for s in range(args.steps):
        r0 = (s * rows) % max(1, args.rows - rows)
        oracle.run(stack, nmap, NY, NX, method=args.method, rows=(r0, r0 + rows), nthreads=threads, kind=kind)
    dt = time.perf_counter() - t0
    px = args.steps * rows * args.cols
    v = px / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "px/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.rows, args.cols, args.method),
                   "sample_rows_per_step": rows},
        "cpu_baseline": {"value": v, "unit": "px/s", "cores": threads, "kind": kind,
                         "sample": "%d rows x %d cols per step" % (rows, args.cols)},
        "e2e": {"value": v, "unit": "px/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_name(rows, cols, method):
    return "voronoi %dx%d N=%d half-window %dx%d %s evd-semantics" % (rows, cols, NB, NY, NX, method)


def device_form(phase_link, d_stack, d_nmap, ctx, precision, method, steps, warmup, dist, local):
    """Times `steps` device-resident runs of one form; returns its figures
    and its outputs (kept on the device for the accuracy comparison)."""
    import torch
    nb, R, C = d_stack.shape
    out = {"phase": torch.zeros((nb, R, C), dtype=torch.complex64, device="cuda"),
           "tcorr": torch.zeros((R, C), dtype=torch.float32, device="cuda"),
           "comp": torch.zeros((R, C), dtype=torch.complex64, device="cuda")}
    kw = dict(method=method, precision=precision, ctx=ctx, out=out)
    for _ in range(max(3, warmup)):
        phase_link(d_stack, d_nmap, (NY, NX), **kw)
    torch.cuda.synchronize()
    ctx.set_profiling(True)
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        phase_link(d_stack, d_nmap, (NY, NX), **kw)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    _, _, runs = ctx.profile()
    kms = {k: v / max(runs, 1) for k, v in ctx.profile_kernels().items()}
    ctx.set_profiling(False)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    # kernels of one step: FP32 pixel kernel + FP64 settle, or per chunk of
    # rows (<= 2^20 pixels) the Gamma and solve kernels, then the FP64 settle
    if precision == "mixed":
        rows_per_chunk = max(1, max(C, 1 << 20) // C)
        launches = 2 * (-(-R // rows_per_chunk)) + 1
    else:
        launches = 2
    return {"ms": ms, "kernel_ms": kms, "clocks": clk, "launches_per_step": launches}, out


def nmap_measurement(stack, d_stack, ctx, steps, cpu_rows):
    """The SHP map producer (fpl_nmap, KS2 and AD2 tests) on the same scene:
    device-resident px/s over `steps` runs (each call ends with a stream
    sync), and the oracle's restatement of the nmap module on the host cores
    over a row sample."""
    import torch
    from fringe_gb300 import nmap
    nb, R, C = stack.shape
    res = {}
    for method in ("KS2", "AD2"):
        out = None
        for _ in range(2):
            out = nmap(d_stack, (NY, NX), ctx=ctx, out=out, method=method)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            nmap(d_stack, (NY, NX), ctx=ctx, out=out, method=method)
        dt = (time.perf_counter() - t0) / steps
        r = {"value": R * C / dt, "unit": "px/s", "ms_per_step": dt * 1e3,
             "mean_count": float(out["count"].float().mean().item()),
             "workload": "%s threshold 0.05 on the same %dx%d N=%d scene, half-window %dx%d"
                         % (method, R, C, nb, NY, NX)}
        if cpu_rows:
            import oracle
            rows = min(cpu_rows, R - 2 * NY)
            t0 = time.perf_counter()
            oracle.nmap(stack[:, :rows + 2 * NY], NY, NX, 0.05, nthreads=os.cpu_count() or 1, method=method)
            dt = time.perf_counter() - t0
            r["cpu_baseline"] = {"value": rows * C / dt, "unit": "px/s", "cores": os.cpu_count() or 1,
                                 "kind": "port", "sample": "%d rows (+%d apron rows) of the scene, %.1f s"
                                                            % (rows, 2 * NY, dt)}
        res[method.lower()] = r
    res["value"] = res["ks2"]["value"]
    return res


def integrate_ps_measurement(d_stack, ctx, steps, hbm_peak, seed=5):
    """The PS/DS merge downstream of phase linking (fpl_integrate_ps,
    python/integratePS.py) on the same scene: the stack serves as both the
    phase-linked and the SLC stack, 10% of the pixels are PS.  HBM-bound:
    per pixel the PS flag, tcorr and one stack (8N bytes) are read and the
    N-1 interferograms and tcorr written, 16N + 1 bytes; timed with CUDA
    events on the launching stream over `steps` launches."""
    import torch
    from fringe_gb300 import integrate_ps
    nb, R, C = d_stack.shape
    g = torch.Generator(device="cuda").manual_seed(seed)
    ps = (torch.rand((R, C), generator=g, device="cuda") < 0.1).to(torch.uint8)
    tc = torch.rand((R, C), generator=g, device="cuda")
    for _ in range(3):
        integrate_ps(d_stack, d_stack, tc, ps, ctx=ctx)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(steps):
        integrate_ps(d_stack, d_stack, tc, ps, ctx=ctx)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    alg = float(R * C * (16 * nb + 1))
    return {"workload": "single-master PS/DS merge of the %dx%d N=%d scene, 10%% PS pixels" % (R, C, nb),
            "value": R * C / (ms / 1e3), "unit": "px/s", "ms_per_step": ms,
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": hbm_peak,
                         "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / hbm_peak,
                         "work": "16N+1 bytes per pixel"}}


def batch_measurement(stack, nmap, seed=7):
    """Uneven ministacks in one batched launch sequence (replayed CUDA graph):
    16 tiles of 512^2..2048^2 pixels cut from the scene, ministacks of
    N in {10, 15, 20, 30} dates of it and N = 45 from a second 1024^2
    45-date scene, half-window 5x10, EVD and MLE alternating.  Per form: the
    batch's px/s, against the same jobs run one after another."""
    import torch
    from fringe_gb300 import synth
    from fringe_gb300.linker import PhaseLinkBatch, phase_link
    rng = np.random.Generator(np.random.PCG64(seed))
    st45, nm45 = synth.scene("voronoi", 1024, 1024, 45, NY, NX, seed=1045)
    d_main = torch.from_numpy(stack).cuda()
    d_nm = torch.from_numpy(nmap.view(np.int32)).cuda()
    d45 = torch.from_numpy(st45).cuda()
    d_nm45 = torch.from_numpy(nm45.view(np.int32)).cuda()
    R = stack.shape[1]
    jobs, px = [], 0
    for k in range(16):
        if k % 5 == 4:
            size, n, src, snm = int(rng.choice([512, 1024])), 45, d45, d_nm45
        else:
            size, n, src, snm = int(rng.choice([512, 1024, 1536, 2048])), int(rng.choice([10, 15, 20, 30])), d_main, d_nm
        size = min(size, src.shape[1])
        r0 = int(rng.integers(0, src.shape[1] - size + 1))
        c0 = int(rng.integers(0, src.shape[2] - size + 1))
        jobs.append({"stack": src[:n, r0:r0 + size, c0:c0 + size].contiguous(),
                     "nmap": snm[r0:r0 + size, c0:c0 + size].contiguous(),
                     "half_window": (NY, NX), "method": "MLE" if k % 2 else "EVD",
                     "mini_stack_count": 1 + k % 3})
        px += size * size
    res = {"jobs": len(jobs), "pixels": px,
           "mix": "16 tiles 512^2..2048^2, N in {10,15,20,30,45}, half-window 5x10, EVD/MLE, miniStackCount 1..3"}
    for prec in ("mixed", "fp32"):
        b = PhaseLinkBatch(jobs, graph=True, autotune=True, precision=prec)
        for _ in range(2):
            b.run()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            b.run()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        b.close()
        # the same jobs one after another (fpl_run_async each)
        outs = [None] * len(jobs)
        for k, j in enumerate(jobs):
            outs[k] = phase_link(j["stack"], j["nmap"], j["half_window"], method=j["method"],
                                 mini_stack_count=j["mini_stack_count"], precision=prec, out=outs[k])
        torch.cuda.synchronize()
        e0.record()
        for k, j in enumerate(jobs):
            phase_link(j["stack"], j["nmap"], j["half_window"], method=j["method"],
                       mini_stack_count=j["mini_stack_count"], precision=prec, out=outs[k])
        e1.record()
        torch.cuda.synchronize()
        ms1 = e0.elapsed_time(e1)
        res[prec] = {"batch_px_s": px / ms * 1e3, "batch_ms": ms,
                     "one_by_one_px_s": px / ms1 * 1e3, "one_by_one_ms": ms1}
    del d45, d_nm45
    return res


def illcond_measurement(ctx, cpu_rows=24, size=1024):
    """Ill-conditioned MLE stress (gamma0 ~ U(0.05, 0.9), 10% of pixels with
    gamma_inf = 0): N = 64, the configuration's full 1024^2 pixels,
    half-window 5x10: px/s of the mixed form, the share of pixels settled in
    FP64, its error against the FP64 form over the whole scene, and parity of
    both forms against the oracle over a row sample."""
    import torch
    from fringe_gb300 import phase_link, synth
    st, nm = synth.scene("illcond", size, size, 64, NY, NX, seed=1003)
    d, dn = torch.from_numpy(st).cuda(), torch.from_numpy(nm.view(np.int32)).cuda()
    res = {"workload": "illcond %dx%d N=64 half-window 5x10 MLE evd-semantics" % (size, size)}
    outs = {}
    for prec in ("mixed", "fp32"):
        # one host-memory run (synchronous fpl_run) for the FP64-settled count
        phase_link(st, nm, (NY, NX), method="MLE", precision=prec, ctx=ctx)
        fp64_px = ctx.stats()["fp64_pixels"]
        out = None
        for _ in range(2):
            out = phase_link(d, dn, (NY, NX), method="MLE", precision=prec, ctx=ctx, out=out)
        torch.cuda.synchronize()
        ctx.set_profiling(True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            phase_link(d, dn, (NY, NX), method="MLE", precision=prec, ctx=ctx, out=out)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        _, _, runs = ctx.profile()
        kms = {k: v / max(runs, 1) for k, v in ctx.profile_kernels().items() if v > 0}
        ctx.set_profiling(False)
        outs[prec] = out
        res[prec] = {"value": size * size / ms * 1e3, "unit": "px/s", "ms": ms,
                     "kernel_ms": kms,
                     "fp64_settled_px": int(fp64_px), "fp64_settled_share": fp64_px / float(size * size)}
    ref = {k: torch.zeros_like(v) for k, v in outs["mixed"].items()}
    ctx.set_tuning(force_fp64=True)
    phase_link(d, dn, (NY, NX), method="MLE", ctx=ctx, out=ref)
    torch.cuda.synchronize()
    ctx.set_tuning(force_fp64=False)
    for prec in ("mixed", "fp32"):
        res[prec]["accuracy_vs_fp64"] = accuracy(outs[prec], ref, ref["tcorr"] > 0)
    del ref
    if cpu_rows:
        import oracle
        t0 = time.perf_counter()
        ora = oracle.run(st, nm, NY, NX, method="MLE", rows=(0, cpu_rows), nthreads=os.cpu_count() or 1)
        dt = time.perf_counter() - t0
        tol = {"phase_rms": 1e-3, "tcorr_max": 2e-4}
        res["parity_vs_oracle"] = {p: parity_vs_oracle(outs[p], ora, cpu_rows, tol) for p in ("mixed", "fp32")}
        res["cpu_baseline"] = {"value": cpu_rows * size / dt, "unit": "px/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": "rows 0..%d (%.1f s)" % (cpu_rows, dt)}
    res["value"] = res["mixed"]["value"]
    return res


def accuracy(out, ref, valid_ref):
    """Phase and coherence error of one form against the FP64 form, over the
    pixels valid in both; validity-code mismatches counted separately."""
    import torch
    tc, tr = out["tcorr"], ref["tcorr"]
    code_a = torch.where(tc < 0, tc, torch.zeros_like(tc))
    code_b = torch.where(tr < 0, tr, torch.zeros_like(tr))
    mism = int((code_a != code_b).sum().item())
    both = (tc > 0) & valid_ref
    d = torch.angle(out["phase"][:, both] * torch.conj(ref["phase"][:, both]))
    rms = float(torch.sqrt(torch.mean(d.double() ** 2)).item()) if d.numel() else 0.0
    per_px = torch.sqrt(torch.mean(d.double() ** 2, dim=0)) if d.numel() else torch.zeros(1)
    dt = (tc[both] - tr[both]).abs()
    return {"phase_rms_rad": rms, "phase_rms_p999_rad": float(torch.quantile(per_px.float()[:1 << 24], 0.999).item()),
            "phase_max_abs_rad": float(d.abs().max().item()) if d.numel() else 0.0,
            "tcorr_max_abs": float(dt.max().item()) if dt.numel() else 0.0,
            "tcorr_rms": float(torch.sqrt(torch.mean(dt.double() ** 2)).item()) if dt.numel() else 0.0,
            "code_mismatch_px": mism, "compared_px": int(both.sum().item())}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from fringe_gb300 import _lib, build, phase_link, synth
    build.build()
    ctx = _lib.Context(local)

    stack, nmap = synth.scene("voronoi", args.rows, args.cols, NB, NY, NX, seed=SEED + rank)
    R, C = args.rows, args.cols
    npx = R * C
    shp = popcount_words(nmap)
    sbar = float(shp.mean())

    # ---- device-resident runs (value): the headline form, then the other -----
    d_stack = torch.from_numpy(stack).cuda()
    d_nmap = torch.from_numpy(nmap.view(np.int32)).cuda()
    other = "fp32" if args.precision == "mixed" else "mixed"
    forms = [args.precision] + ([] if args.no_compare else [other])
    res, outs = {}, {}
    for prec in forms:
        res[prec], outs[prec] = device_form(phase_link, d_stack, d_nmap, ctx, prec, args.method,
                                            args.steps, args.warmup, dist, local)
    head = res[args.precision]
    ms = head["ms"]
    value = world * npx * args.steps / (ms / 1e3)
    tc = outs[args.precision]["tcorr"].cpu().numpy()
    valid = int((tc > 0).sum())

    # ---- accuracy of both forms against the FP64 form (whole scene) -----------
    acc = None
    if not args.no_accuracy:
        ref = {"phase": torch.zeros_like(outs[args.precision]["phase"]),
               "tcorr": torch.zeros_like(outs[args.precision]["tcorr"]),
               "comp": torch.zeros_like(outs[args.precision]["comp"])}
        ctx.set_tuning(force_fp64=True)
        t0 = time.perf_counter()
        phase_link(d_stack, d_nmap, (NY, NX), method=args.method, ctx=ctx, out=ref)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        ctx.set_tuning(force_fp64=False)
        vref = ref["tcorr"] > 0
        acc = {p: accuracy(outs[p], ref, vref) for p in forms}
        acc["fp64_form_s"] = t64
        acc["reference"] = "FP64 form of the same kernels (all pixels FP64, pinned to the oracle)"
        del ref

    # ---- end to end through the C ABI with pinned host buffers ---------------
    e2e = None
    fp64_px = None
    if not args.no_e2e:
        h_stack = torch.from_numpy(stack).pin_memory()
        h_nmap = torch.from_numpy(nmap.view(np.int32)).pin_memory()
        h_out = {"phase": torch.zeros((NB, R, C), dtype=torch.complex64).pin_memory(),
                 "tcorr": torch.zeros((R, C), dtype=torch.float32).pin_memory(),
                 "comp": torch.zeros((R, C), dtype=torch.complex64).pin_memory()}
        np_out = {k: v.numpy() for k, v in h_out.items()}
        hs, hn = h_stack.numpy(), h_nmap.numpy().view(np.uint32)
        for _ in range(max(3, args.warmup)):
            phase_link(hs, hn, (NY, NX), method=args.method, precision=args.precision,
                       ctx=ctx, out=np_out)
        st = ctx.stats()
        fp64_px = st["fp64_pixels"]
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            phase_link(hs, hn, (NY, NX), method=args.method, precision=args.precision,
                       ctx=ctx, out=np_out)
        dt = time.perf_counter() - t0
        if dist:
            t = torch.tensor([dt], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        h2d = stack.nbytes + nmap.nbytes
        d2h = sum(v.nbytes for v in np_out.values())
        e2e = {"value": world * npx * args.steps / dt, "unit": "px/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
        assert np.array_equal(np_out["tcorr"], tc), "host and device paths differ"

    if rank != 0:
        return
    hbm_peak, tf_peak, peak_src = load_peaks()
    centre = shp > 0
    flops = float((4.0 * NB * (NB + 1) * shp[centre]).sum())     # Gamma, Hermitian half
    alg_bytes = npx * (16 * NB + 4 * nmap.shape[2] + 12)
    km = head["kernel_ms"]
    if args.precision == "mixed":
        # dominant kernel of the mixed form by device time
        dom = "solve" if km["solve"] >= km["gram"] else "gram"
    else:
        dom = "fp32"
    names = {"fp32": "k_pixels<float> (FP32 SIMT gather + Gamma + eigen-solves)",
             "gram": "k_gram_box (tcgen05 bf16 hi/lo Gamma, TMEM accumulate)",
             "solve": "k_solve (warp eigen-solves from the Gamma records)"}
    k_ms = km[dom]
    kc = kernel_counters()
    ent = kc.get(dom) or {}
    traffic = ent["dram_bytes_per_px"] * npx if ent.get("dram_bytes_per_px") else None
    clk_mhz = head["clocks"].get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    issue_peak = sms * 4 * clk_mhz * 1e6 / 1e9          # warp instructions per second, G
    fp32_peak = sms * 128 * 2 * clk_mhz * 1e6 / 1e12     # FP32 FMA pipe, TFLOP/s
    gamma_tf = flops / (km["gram"] / 1e3) / 1e12 if km.get("gram", 0) > 0 else None
    if dom in ("solve", "fp32") and ent.get("warp_inst_per_px"):
        inst = ent["warp_inst_per_px"] * npx / (k_ms / 1e3) / 1e9
        sflops = float(solve_flops_per_px(NB, ent.get("solve_pairs_per_px") or 4.6)) * valid / (k_ms / 1e3) / 1e12
        roof = {"bound": "issue", "achieved": inst, "peak": issue_peak, "unit": "Gwarp-inst/s",
                "frac": inst / issue_peak, "traffic": traffic, "kernel": names[dom], "kernel_ms": k_ms,
                "work": "ncu warp instructions per pixel x pixels, per step",
                "peak_source": "%d SMs x 4 issue slots x %.0f MHz (median SM clock of the timed region)"
                               % (sms, clk_mhz),
                "fp32": {"achieved_tflops": sflops, "peak_tflops": fp32_peak, "frac": sflops / fp32_peak,
                         "work": "eigen-solve FP32 flops per valid pixel as implemented (solve_flops_per_px)"},
                "ncu": {k: ent.get(k) for k in ("issue_active", "fma_pipe_active", "tensor_pipe_active",
                                                 "warp_inst_per_px", "dram_bytes_per_px", "source")},
                "hbm_achieved_gbs": alg_bytes / (k_ms / 1e3) / 1e9, "hbm_peak_gbs": hbm_peak,
                "what_bounds_it": BOUND_NOTES.get(dom, "")}
    else:
        achieved_tf = flops / (k_ms / 1e3) / 1e12
        roof = {"bound": "tensor", "achieved": achieved_tf, "peak": tf_peak, "unit": "TFLOP/s",
                "frac": achieved_tf / tf_peak, "traffic": traffic, "peak_source": peak_src,
                "kernel": names[dom], "work": "Gamma flops 4N(N+1)S summed over pixels, per step",
                "kernel_ms": k_ms, "what_bounds_it": BOUND_NOTES.get(dom, "")}
    gram_line = None
    if gamma_tf:
        g = kc.get("gram") or {}
        gram_line = {"bound": "tensor", "kernel": names["gram"], "kernel_ms": km["gram"],
                     "achieved": gamma_tf, "peak": tf_peak, "unit": "TFLOP/s", "frac": gamma_tf / tf_peak,
                     "peak_source": peak_src + " bf16 burst",
                     "work": "Gamma flops 4N(N+1)S summed over pixels (hi/lo passes and masked-out products "
                             "not credited)",
                     "traffic": g["dram_bytes_per_px"] * npx if g.get("dram_bytes_per_px") else None,
                     "ncu_tensor_pipe_active": g.get("tensor_pipe_active")}
    per_kernel = {}
    for k, v in km.items():
        if v <= 0:
            continue
        e = {"ms_per_step": v}
        if k in ("fp32", "gram"):
            e["gamma_tflops"] = flops / (v / 1e3) / 1e12
            e["frac_of_bf16_peak"] = e["gamma_tflops"] / tf_peak
        e["path_bytes_gbs"] = alg_bytes / (v / 1e3) / 1e9
        per_kernel[k] = e
    line = {
        "metric": METRIC, "value": value, "unit": "px/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "bf16x2-split/f32",
        "data": "synthetic (seeded Voronoi scene, coherence model of tests/evd/test_evd.py)",
        "config": {"workload": workload_name(R, C, args.method),
                   "precision": args.precision, "mean_shp": sbar,
                   "l2": "inputs (%.2f GB stack) exceed the 129 MB L2; no flush needed" % (stack.nbytes / 1e9),
                   "valid_px": valid, "fp64_settled_px": fp64_px},
        "e2e": e2e,
        "gpu_launches": head["launches_per_step"] * args.steps,
        "clocks": head["clocks"],
        "roofline": roof,
        "roofline_gamma": gram_line,
        "kernels": per_kernel,
    }
    if not args.no_compare:
        o = res[other]
        line["other_form"] = {"precision": other, "value": world * npx * args.steps / (o["ms"] / 1e3),
                              "ms_per_step": o["ms"] / args.steps, "kernel_ms": o["kernel_ms"]}
        line["mixed_over_fp32"] = (res["fp32"]["ms"] / res["mixed"]["ms"])
    if acc is not None:
        line["accuracy_vs_fp64"] = acc
    if not args.no_serve and world == 1:
        line["serving"] = serving_measurement(args.serve_jobs)
    if not args.no_batch and world == 1:
        line["batch"] = batch_measurement(stack, nmap)
        line["illconditioned"] = illcond_measurement(ctx, 0 if args.no_cpu else 24)
    if not args.no_nmap and world == 1:
        line["nmap"] = nmap_measurement(stack, d_stack, ctx, max(1, args.steps), 0 if args.no_cpu else 384)
        line["integrate_ps"] = integrate_ps_measurement(d_stack, ctx, max(3, args.steps), hbm_peak)
    if not args.no_cpu:
        rows = min(args.cpu_rows or 480, R)          # about 15 s on 16 host cores
        line["cpu_baseline"], ora = cpu_baseline(stack, nmap, args.method, rows)
        tols = {"fp32": {"phase_rms": 1e-3, "tcorr_max": 1e-4}, "mixed": {"phase_rms": 1e-3, "tcorr_max": 2e-4}}
        line["parity_vs_oracle"] = {p: parity_vs_oracle(outs[p], ora, rows, tols[p]) for p in forms}
        line["parity_vs_oracle"]["oracle"] = "oracle port (FP64 restatement of the reference loop), same scene"
        del ora
        line["cpu_baseline_detail"] = cpu_baseline_detail(stack, nmap, min(rows // 4, R))
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
