#!/usr/bin/env python3
"""Throughput of the GB300 X-BACH difference-imaging path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--mode mixed|plain] [--cpu-runs R] [--config 2|4] [--files N --io T]

Workload: a 2048x2048 FP32 template/science pair
(seeded synthetic field: 20k sources, FWHM varying across the field, 1 %
cosmic-ray pixels, 40 saturated stars, detector saturation 6e4), 16x16 stamps,
49 basis functions, spatial kernel order 2, background order 1.  One step is
one difference image: init (mask) -> sss -> cmv -> cd -> ksc -> conv -> sub.

value: difference images per second with T and S already resident in HBM,
timed with CUDA events on the library's stream, L2 flushed (256 MB write)
before every step, max over ranks.  e2e: the same through xb_run() with the
host->device copy of both FP32 inputs from pinned memory and the
device->host read of the conv and diff images inside the timed region.

The headline runs 24 frame pairs per step on 24 worker contexts (--batch,
--workers), each frame replayed as one captured CUDA graph (--graph 1), with
the learned substamp order (--rank 1: policy 1 with the shipped weights,
xbach/ranker_preset5.npy).  The process asks for 32 hardware work queues
(CUDA_DEVICE_MAX_CONNECTIONS, set before CUDA starts): with the default 8,
the workers' streams share queues and their graphs serialise.

roofline: the kernel with the most device time per frame (single-frame
kernel timers) against the roof of the unit that bounds it, with the
reference's algorithmic work (not the extra operations issued here for
precision); rooflines: every hot kernel's views (conv+sub: HBM at 20 B/px and
FP32 at 2 x 441 FLOP/px; fused fill + Gram: FP32 passes and tensor Gram per
substamp; global solve: FP64 at 2/3 n^3).  Peaks: MEASURED_PEAKS.json for HBM
and bf16, the FP32/FP64 FMA peaks measured in this run.  cpu_baseline: the
median of --cpu-runs FP64 oracle runs on all host threads over the batch's
first pairs, and one single-threaded run.

Beside the headline (ranked, frame graphs): chosen_unranked (the same batch
without the learned ranking), plain_gpu_batched (the plain FP64 pipeline
through the same batch API, pairs and workers; chosen_over_plain divides by
it) and plain_gpu_single; accuracy gives the chosen image against the plain
one with the same ranking and without it, the unranked chosen image against
the unranked plain one, and names the gate.

--config 4: 64 pairs of mixed sizes per step (preset 4).  --files N: N
2048^2 pairs per step streamed as FITS files through xb_pipeline.

N > 1 (torchrun): replicas - every rank runs its own frame pairs on its own
GPU; the only cross-rank traffic is the barrier and the max of the timings.

--impl reference: the reference's CPU path.  The reference cannot be built
here (OpenCL and CCfits are absent), so this arm times the repository's FP64
C++ restatement of it (oracle/, OpenMP over all host threads) on the same
frame pair; rank 0 only.
"""
import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

# concurrent frame graphs need their own hardware queues (read when the CUDA
# context is created, so before torch touches the device)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = pathlib.Path(__file__).resolve().parent
PKG = REPO / "thesis-emx-bach_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(REPO / "tests"))

METRIC = "difference-images/s at 2048², chosen vs plain GPU at ≤1e-3σ; % HBM/TC peak"
UNIT = "difference-images/s"
WORKLOAD = ("2048x2048 FP32 template/science pair, 20k sources, FWHM 2.2-3.2/3.0-4.2 px, "
            "1% cosmic-ray pixels, 40 saturated stars, saturation 6e4 (threshHigh), 16x16 stamps, "
            "49 basis functions (3 Gaussians, degrees 6/4/2), kernel order 2, background order 1")


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


# ---- replicas (N > 1): every rank runs its own pairs; no data-path traffic ----
def rank_frames(rank, batch):
    """Seeds (frame indices) of the pairs one rank runs: disjoint across ranks."""
    return [rank * batch + i for i in range(batch)]


def max_over_ranks(ms, world, device):
    """The slowest rank's time (the job's time), via one all-reduce."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, pairs_per_rank, steps, ms):
    """Whole-job throughput: every rank's pairs over the slowest rank's time."""
    return world * pairs_per_rank * steps / (ms / 1000.0)


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def frame_params(xbach_or_oracle, info, mode=None):
    kw = dict(stampsx=info["stamps"], stampsy=info["stamps"], threshHigh=info["threshHigh"])
    if mode is not None:
        kw["mode"] = mode
    return xbach_or_oracle.default_params(**kw)


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi sampling during the timed region (200 ms period)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        for line in pathlib.Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------ CPU baseline --
def cpu_frames_per_s(T, S, info, runs, threads=None, params_kw=None):
    import build_native
    build_native.build_oracle()
    from xbach_testlib import Oracle
    o = Oracle()
    p = frame_params(o, info)
    for k, v in (params_kw or {}).items():
        if k in ("dg", "bg"):
            for i, x in enumerate(v):
                getattr(p, k)[i] = x
        else:
            setattr(p, k, v)
    T64, S64 = T.astype("float64"), S.astype("float64")
    threads = threads or os.cpu_count() or 1
    times = []
    last = None
    for _ in range(runs):
        last = None
        t0 = time.perf_counter()
        r = o.run(p, T64, S64, nthreads=threads)
        times.append(time.perf_counter() - t0)
        assert r.status == 0, r.status
        last = r
    return runs / sum(times), threads, times, last


def run_reference(args):
    """The reference's CPU path on the GPU arm's frames: step k runs the
    frame pairs of seeds k*f .. k*f+f-1 (mod --batch), f = ceil(batch /
    steps), so the timed steps cover every seed the GPU arm runs."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import build_native
    build_native.build_oracle()
    from xbach_testlib import Oracle
    from xbach.synth import make_pair
    B = max(1, args.batch)
    per = -(-B // max(1, args.steps))
    o = Oracle()
    threads = os.cpu_count() or 1
    frames = {}

    def frame(seed):
        if seed not in frames:
            T, S, info = make_pair(2, frame=seed)
            frames[seed] = (T.astype("float64"), S.astype("float64"), frame_params(o, info))
        return frames[seed]

    def step(k):
        seeds = [(k * per + i) % B for i in range(per)]
        for sd in seeds:
            frame(sd)  # generated outside the timed region
        t0 = time.perf_counter()
        for sd in seeds:
            T64, S64, p = frames[sd]
            r = o.run(p, T64, S64, nthreads=threads)
            assert r.status == 0, r.status
        return time.perf_counter() - t0
    for k in range(args.warmup):
        step(k)
    times = [step(k) for k in range(args.steps)]
    total = sum(times)
    fps = per * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": fps, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 2048x2048 crowded fields, one seed per frame pair)",
        "config": {"workload": WORKLOAD, "frames_per_step": per,
                   "seeds": f"0..{B - 1} (the GPU arm's batch), {per} per step",
                   "implementation": "FP64 C++ restatement of the reference "
                   "CPU path (the reference needs OpenCL + CCfits, absent here)"},
        "cpu_baseline": {"value": fps, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{per * args.steps} full 2048x2048 frame pairs, {per} per step, "
                                   f"seeds cycling over the GPU arm's {B}"},
        "e2e": {"value": fps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- roofline --
# Algorithmic work per unit (the reference's operations, not the extra ones
# this implementation issues for precision):
#   conv+sub: 2 x 441 FLOP and 20 B of HBM per pixel (T, S read FP32; conv
#     and diff written FP32; mask 2 B read and written);
#   cmv fill of one substamp: Y pass 15 filters x 1581 x 21 + X pass
#     49 x 961 x 21 MAC (2.97 MFLOP, FP32 in mixed mode) and the Gram
#     1275 x 961 + B 50 x 961 MAC (2.45 MFLOP, tensor cores);
#   global solve: the reference's LU, 2/3 n^3 FLOP (n = 292); the LDL^T here
#     executes n^3 / 3 of them;
#   sss (stamp statistics, substamp search): 6 B of HBM per pixel and image
#     (the pixel and its mask bits), the stamps tiling the frame.
FILL_PASS_FLOP = 2.0 * (15 * 1581 * 21 + 49 * 961 * 21)
FILL_GRAM_FLOP = 2.0 * (1275 * 961 + 50 * 961)
CONV_BYTES_PER_PX = 20


def rooflines(kernels, params, n_pix, mode, stamps, peaks):
    """Per-kernel rooflines from the single-frame kernel timers (CUDA events
    around each launch on the library's stream).  peaks: measured HBM GB/s
    and bf16 TFLOP/s (MEASURED_PEAKS.json) and the FP32/FP64 FMA peaks
    measured in this run (xb_measure_fma_peaks; MEASURED_PEAKS.json has no
    CUDA-core entries)."""
    from xbach.accuracy import layout
    out = {}
    fk = 2 * params.hKernelWidth + 1

    def view(bound, work, ms, peak, unit, scale, **kw):
        ach = work / (ms * 1e-3) / scale
        d = {"bound": bound, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak,
             "ms_per_launch": ms}
        d.update(kw)
        return d
    if "conv_sub" in kernels:
        k = kernels["conv_sub"]
        ms = k["ms_total"] / k["launches"]
        byt = CONV_BYTES_PER_PX * n_pix + (16 * n_pix if mode == "plain" else 0)
        flop = 2.0 * fk * fk * n_pix
        out["conv_sub"] = {
            "hbm": view("hbm", byt, ms, peaks["hbm"], "GB/s", 1e9, bytes_per_launch=byt,
                        peak_source=peaks["hbm_source"]),
            "cuda_cores": view("fp32" if mode == "mixed" else "fp64", flop, ms,
                               peaks["fp32"] if mode == "mixed" else peaks["fp64"], "TFLOP/s",
                               1e12, flop_per_launch=flop, peak_source=peaks["fma_source"])}
    if "fill_gram" in kernels:
        k = kernels["fill_gram"]
        ms = k["ms_total"]
        out["fill_gram"] = {
            "fp32_passes": view("fp32", FILL_PASS_FLOP * stamps, ms, peaks["fp32"], "TFLOP/s", 1e12,
                                flop_per_substamp=FILL_PASS_FLOP, substamps_per_frame=stamps,
                                ms_per_frame=ms, peak_source=peaks["fma_source"]),
            "tensor_gram": view("tensor", FILL_GRAM_FLOP * stamps, ms, peaks["bf16"], "TFLOP/s",
                                1e12, flop_per_substamp=FILL_GRAM_FLOP,
                                mma_flop_per_substamp=16 * 4 * 2 * 128 * (256 + 64 + 192) * 16,
                                substamps_per_frame=stamps, ms_per_frame=ms,
                                peak_source=peaks["bf16_source"])}
        for v in out["fill_gram"].values():
            v.pop("ms_per_launch")
    # sss: every stamp pixel and its mask bits once per pass, both images
    # (the stamps tile the frame): 2 x 6 B per pixel
    for name in ("stamp_stats", "find_substamps"):
        if name in kernels:
            k = kernels[name]
            byt = 2 * 6 * n_pix
            out[name] = view("hbm", byt, k["ms_total"], peaks["hbm"], "GB/s", 1e9,
                             bytes_per_frame=byt, ms_per_frame=k["ms_total"],
                             peak_source=peaks["hbm_source"])
            out[name].pop("ms_per_launch")
    if "global_ldl" in kernels:
        k = kernels["global_ldl"]
        ms = k["ms_total"] / k["launches"]
        n_comp, n_bg = layout(params)
        n = n_comp + n_bg + 1
        out["global_ldl"] = view("fp64", 2.0 * n ** 3 / 3.0, ms, peaks["fp64"], "TFLOP/s", 1e12,
                                 n=n, flop_per_launch=2.0 * n ** 3 / 3.0,
                                 flop_executed_per_launch=n ** 3 / 3.0,
                                 peak_source=peaks["fma_source"])
    return out


def run_result(xbach, cx):
    return {"diff": cx.image(xbach.XB_IMG_DIFF), "conv": cx.image(xbach.XB_IMG_CONV),
            "solution": cx.solution(), "kernSum": cx.scalar("kernSum"),
            "convTemplate": cx.scalar("convTemplate")}


SIGMA_BAR = 1e-3


def accuracy(xbach, ctx, pctx, oracle_res, T, S, params, prctx=None, uctx=None):
    """Chosen vs plain GPU (acceptance: diff within 1e-3 sigma) and against
    the FP64 oracle on the same frame pair.

    ctx: the chosen pipeline (mixed, ranked when prctx is given); pctx: the
    plain FP64 GPU pipeline without ranking (the reference's semantics);
    prctx: the plain pipeline with the same learned ranking (the same
    substamp picks, so the difference is the precision error alone); uctx:
    the mixed pipeline without ranking.  The gate is named in the result."""
    from xbach import accuracy as acc
    n_comp, n_bg = acc.layout(params)
    chosen, plain = run_result(xbach, ctx), run_result(xbach, pctx)
    out = {"sigma_definition": "sqrt(|target| + |conv| + 2*5^2) ADU, gain 1"}
    if prctx is None:
        out["chosen_vs_plain"] = acc.compare(chosen, plain, T, S, n_comp, n_bg)
        m = out["chosen_vs_plain"]["diff"]["max_sigma"]
        out["gate"] = {"uses": "chosen_vs_plain", "max_sigma": m, "bar": SIGMA_BAR,
                       "pass": bool(m <= SIGMA_BAR)}
    else:
        plain_same = run_result(xbach, prctx)
        unranked = run_result(xbach, uctx)
        out["chosen_vs_plain_same_ranking"] = acc.compare(chosen, plain_same, T, S, n_comp, n_bg)
        out["chosen_vs_plain_same_ranking"]["reference"] = (
            "plain FP64 GPU pipeline with the same learned ranking (same substamp picks)")
        out["chosen_vs_plain_unranked"] = acc.compare(chosen, plain, T, S, n_comp, n_bg)
        out["chosen_vs_plain_unranked"]["reference"] = (
            "plain FP64 GPU pipeline without ranking (the reference's picks): another fit, "
            "not a precision figure")
        out["unranked_chosen_vs_plain_unranked"] = acc.compare(unranked, plain, T, S, n_comp, n_bg)
        m_same = out["chosen_vs_plain_same_ranking"]["diff"]["max_sigma"]
        m_unr = out["unranked_chosen_vs_plain_unranked"]["diff"]["max_sigma"]
        out["gate"] = {
            "uses": "chosen_vs_plain_same_ranking (ranked headline) and "
                    "unranked_chosen_vs_plain_unranked (chosen_unranked throughput)",
            "max_sigma_same_ranking": m_same, "max_sigma_unranked": m_unr, "bar": SIGMA_BAR,
            "pass": bool(m_same <= SIGMA_BAR and m_unr <= SIGMA_BAR),
            "note": "the ranking picks other substamps, so the ranked chosen image is another "
                    "valid fit; against the unranked plain image it is compared in "
                    "chosen_vs_plain_unranked and ranking_effect, not gated"}
        out["ranking_effect"] = acc.compare(chosen, unranked, T, S, n_comp, n_bg)
        out["ranking_effect"]["ksc_refills"] = [int(uctx.scalar("ksc_refills")),
                                                int(ctx.scalar("ksc_refills"))]
        out["ranking_effect"]["ksc_iterations"] = [int(uctx.scalar("ksc_iterations")),
                                                   int(ctx.scalar("ksc_iterations"))]
        q = acc.residual_noise([unranked, chosen], T, S)
        out["ranking_effect"]["residual_noise"] = {"unranked": q[0], "ranked": q[1]}
    if oracle_res is not None:
        ref = {"diff": oracle_res.image("diff"), "conv": oracle_res.image("conv"),
               "solution": oracle_res.array("solution", "float64"),
               "kernSum": oracle_res.scalar("kernSum"),
               "convTemplate": oracle_res.scalar("convTemplate")}
        mixed = run_result(xbach, uctx) if uctx is not None else chosen
        key = "mixed_unranked_vs_fp64_oracle" if uctx is not None else "chosen_vs_fp64_oracle"
        out[key] = acc.compare(mixed, ref, T, S, n_comp, n_bg)
        out["plain_vs_fp64_oracle"] = acc.compare(plain, ref, T, S, n_comp, n_bg)
    return out


def _make_pair4(frame):
    sys.path.insert(0, str(PKG))
    from xbach.synth import make_pair4
    return make_pair4(frame)


def run_config4(args):
    """64 pairs of sizes 512^2..4096^2, each with its own stamp grid, source
    density and FWHM ratio (preset 4), in one batch per step: frame graphs on
    `workers` contexts, per-pair parameters, fixed schedule."""
    import concurrent.futures
    import multiprocessing
    n_pairs = args.pairs
    # host generation in a spawned pool, before CUDA starts in this process
    with concurrent.futures.ProcessPoolExecutor(
            max_workers=min(16, os.cpu_count() or 1),
            mp_context=multiprocessing.get_context("spawn")) as ex:
        frames = list(ex.map(_make_pair4, range(n_pairs)))
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    import xbach
    mode = xbach.XB_MODE_PLAIN if args.mode == "plain" else xbach.XB_MODE_MIXED
    params = [frame_params(xbach, f[2], mode) for f in frames]
    dT = [torch.from_numpy(f[0]).cuda() for f in frames]
    dS = [torch.from_numpy(f[1]).cuda() for f in frames]
    dC = [torch.empty_like(t) for t in dT]
    dD = [torch.empty_like(t) for t in dT]
    ws = [t.shape[1] for t in dT]
    hs = [t.shape[0] for t in dT]
    pix = sum(w * h for w, h in zip(ws, hs))
    batch = xbach.Batch(params[0], workers=args.workers)
    batch.set_params(params)
    use_graph = bool(args.graph) and args.mode == "mixed"
    use_rank = bool(args.rank) and args.mode == "mixed"
    if use_rank:
        from xbach import ranker
        w_rank = ranker.preset5_weights()
        for i in range(batch.n_workers):
            ranker.enable(batch.worker(i), w_rank, policy=1, tau=args.rank_tau)
    if use_graph:
        batch.set_option("graph", 1)
    st = torch.cuda.Stream()
    batch.set_stream(st.cuda_stream)

    def run():
        batch.run_ptrs([t.data_ptr() for t in dT], [t.data_ptr() for t in dS], ws, hs,
                       [t.data_ptr() for t in dC], [t.data_ptr() for t in dD], device=True)
    t0 = time.time()
    run()  # first pass: every worker captures the graphs of its pairs
    torch.cuda.synchronize()
    capture_s = time.time() - t0
    for _ in range(max(args.warmup - 1, 1)):
        run()
    torch.cuda.synchronize()
    workers = [batch.worker(i) for i in range(batch.n_workers)]
    l0 = sum(wk.launches() for wk in workers)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ms = 0.0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run()
            e1.record(st)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
    launches = sum(wk.launches() for wk in workers) - l0
    # end to end: pinned host frames in, host images out, the same batch
    hT = [torch.from_numpy(f[0]).pin_memory() for f in frames]
    hS = [torch.from_numpy(f[1]).pin_memory() for f in frames]
    hC = [torch.empty_like(t).pin_memory() for t in hT]
    hD = [torch.empty_like(t).pin_memory() for t in hT]

    def run_e2e():
        batch.run_ptrs([t.data_ptr() for t in hT], [t.data_ptr() for t in hS], ws, hs,
                       [t.data_ptr() for t in hC], [t.data_ptr() for t in hD])
    run_e2e()
    e2e_ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        run_e2e()
        e1.record(st)
        e1.synchronize()
        e2e_ms += e0.elapsed_time(e1)
    e2e = {"value": n_pairs * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
           "h2d_bytes_per_step": 2 * 4 * pix, "d2h_bytes_per_step": 2 * 4 * pix}
    # rooflines from the largest pair, one frame with the kernel timers on
    big = max(range(n_pairs), key=lambda i: ws[i] * hs[i])
    kctx = xbach.Context(params[big])
    if use_rank:
        ranker.enable(kctx, w_rank, policy=1, tau=args.rank_tau)

    def one_big():
        kctx.init_device(dT[big].data_ptr(), dS[big].data_ptr(), ws[big], hs[big])
        for stage in (kctx.sss, kctx.cmv, kctx.cd, kctx.ksc, kctx.conv, kctx.sub):
            stage()
    one_big()
    torch.cuda.synchronize()
    kctx.set_option("time_kernels", 1)
    one_big()
    torch.cuda.synchronize()
    kernels = {}
    for name in ("stamp_stats", "find_substamps", "fill_gram", "stamp_test_fit", "sigs",
                 "global_ldl", "global_solve", "mx_build", "conv_sub", "rank_score"):
        kms, kn = kctx.kernel_time(name)
        if kn:
            kernels[name] = {"ms_total": kms, "launches": kn}
    kctx.set_option("time_kernels", 0)
    hbm_peak, bf16_peak, peak_src = measured_peaks()
    fp32_peak, fp64_peak = xbach.measure_fma_peaks(0)
    stamps = kctx.scalar("nstamps0") + kctx.scalar("nstamps1") + kctx.scalar("ksc_refills")
    peaks = {"hbm": hbm_peak, "bf16": bf16_peak, "fp32": fp32_peak, "fp64": fp64_peak,
             "hbm_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
             "bf16_source": f"{peak_src} (MEASURED_PEAKS.json bf16_tflops)",
             "fma_source": "measured in this run by xb_measure_fma_peaks"}
    roofs = rooflines(kernels, params[big], ws[big] * hs[big], args.mode, stamps, peaks)
    dominant = max(kernels, key=lambda k: kernels[k]["ms_total"]) if kernels else None
    roof = dict(roofs[dominant]) if dominant in roofs else None
    if roof is not None and "bound" not in roof:
        roof = dict(next(iter(roof.values())))
    if roof is not None:
        roof.update({"kernel": dominant, "traffic": None,
                     "pair": f"{ws[big]}x{hs[big]} (the batch's largest)"})
    kctx.close()
    # a sample of pairs against single contexts run stage by stage
    check = sorted(range(n_pairs), key=lambda i: ws[i] * hs[i])
    check = check[:2] + check[-1:]
    same = []
    for i in check:
        ctx = xbach.Context(params[i])
        if use_rank:
            ranker.enable(ctx, w_rank, policy=1, tau=args.rank_tau)
        ctx.init_device(dT[i].data_ptr(), dS[i].data_ptr(), ws[i], hs[i])
        for stage in (ctx.sss, ctx.cmv, ctx.cd, ctx.ksc, ctx.conv, ctx.sub):
            stage()
        ref = torch.from_numpy(ctx.image(xbach.XB_IMG_DIFF, f64=False))
        same.append(bool(torch.equal(ref, dD[i].cpu())))
        ctx.close()
    sizes = {}
    for w in ws:
        sizes[f"{w}^2"] = sizes.get(f"{w}^2", 0) + 1
    line = {
        "metric": "difference-images/s, 64 pairs of mixed size (preset 4)",
        "value": n_pairs * args.steps / (ms / 1000.0), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.mode == "plain" else "f32",
        "data": "synthetic (preset 4: size, stamp grid, density, FWHM ratio per pair from its seed)",
        "config": {"workload": f"{n_pairs} pairs, sizes {sizes}, stamp grids "
                               f"{min(p.stampsx for p in params)}-{max(p.stampsx for p in params)}, "
                               "49 basis functions, kernel order 2, background order 1",
                   "mode": args.mode, "frames_per_step": n_pairs, "workers": args.workers,
                   "frame_graphs": use_graph, "schedule": "fixed, largest first" if use_graph
                   else "shared queue",
                   "learned_ranking": f"policy 1, tau {args.rank_tau}, xbach/ranker_preset5.npy" if use_rank
                   else None,
                   "hw_queues": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                   "l2": "flushed before every step; inputs exceed L2",
                   "inputs": "device-resident FP32 T,S"},
        "megapixels_per_s": pix * args.steps / (ms / 1000.0) / 1e6,
        "gpu_launches": launches, "clocks": clk.summary(), "roofline": roof, "rooflines": roofs,
        "kernels_largest_pair": kernels, "e2e": e2e,
        "first_pass_s": capture_s,
        "check_vs_stage_by_stage": {"pairs": check, "identical": same},
    }
    print(json.dumps(line), flush=True)
    return 0


def _make_pair3(frame):
    sys.path.insert(0, str(PKG))
    from xbach.synth import make_pair
    return make_pair(3, frame=frame)


def run_config3(args):
    """Config 3: 3072^2 crowded fields with 4 Gaussians (59 basis functions
    by the reference's counting rule), kernel order 3, background order 2
    (587 unknowns), 20x20 stamps.  --pairs3 pairs per step on as many worker
    contexts, frame graphs, no ranking; the plain FP64 pipeline through the
    same batch API; accuracy of frame 0 against the plain GPU result and the
    FP64 oracle; rooflines from one frame with the kernel timers on."""
    import concurrent.futures
    import multiprocessing
    B = max(1, args.pairs3)
    with concurrent.futures.ProcessPoolExecutor(
            max_workers=min(16, os.cpu_count() or 1),
            mp_context=multiprocessing.get_context("spawn")) as ex:
        frames = list(ex.map(_make_pair3, range(B)))
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    import xbach
    from xbach.synth import PARAMS_3
    T, S, info = frames[0]
    h, w = T.shape
    n_pix = w * h

    def params_for(mode):
        return xbach.default_params(stampsx=info["stamps"], stampsy=info["stamps"],
                                    threshHigh=info["threshHigh"], mode=mode, **PARAMS_3)
    params = params_for(xbach.XB_MODE_MIXED)
    dT = [torch.from_numpy(f[0]).cuda() for f in frames]
    dS = [torch.from_numpy(f[1]).cuda() for f in frames]
    dC = [torch.empty_like(t) for t in dT]
    dD = [torch.empty_like(t) for t in dT]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    st = torch.cuda.Stream()

    def timed(run, steps):
        ms = 0.0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run()
            e1.record(st)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
        return ms

    def batch_for(bparams, graphs):
        bt = xbach.Batch(bparams, workers=B)
        bt.set_stream(st.cuda_stream)
        if graphs:
            bt.set_option("graph", 1)
            for i in range(bt.n_workers):
                bt.worker(i).run_device(dT[0].data_ptr(), dS[0].data_ptr(), w, h,
                                        dC[0].data_ptr(), dD[0].data_ptr())
            torch.cuda.synchronize()

        def run():
            bt.run_ptrs([t.data_ptr() for t in dT], [t.data_ptr() for t in dS], [w] * B, [h] * B,
                        [t.data_ptr() for t in dC], [t.data_ptr() for t in dD], device=True)
        return bt, run

    # one frame, stage by stage with the kernel timers: rooflines
    ctx = xbach.Context(params)
    cst = torch.cuda.ExternalStream(ctx.stream())

    def single():
        ctx.init_device(dT[0].data_ptr(), dS[0].data_ptr(), w, h)
        for stage in (ctx.sss, ctx.cmv, ctx.cd, ctx.ksc, ctx.conv, ctx.sub):
            stage()
    for _ in range(2):
        single()
    torch.cuda.synchronize()
    ctx.set_option("time_kernels", 1)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(cst)
    single()
    e1.record(cst)
    e1.synchronize()
    single_ms = e0.elapsed_time(e1)
    kernels = {}
    for name in ("stamp_stats", "find_substamps", "fill_w", "fill_finish", "gram", "fill_gram",
                 "stamp_test_fit", "sigs", "global_ldl", "global_solve", "mx_build",
                 "mx_scatter", "conv_sub", "ksc_check", "kernel_sum"):
        ms, n = ctx.kernel_time(name)
        if n:
            kernels[name] = {"ms_total": ms, "launches": n}
    ctx.set_option("time_kernels", 0)
    stamps = ctx.scalar("nstamps0") + ctx.scalar("nstamps1") + ctx.scalar("ksc_refills")
    hbm_peak, bf16_peak, peak_src = measured_peaks()
    fp32_peak, fp64_peak = xbach.measure_fma_peaks(0)
    peaks = {"hbm": hbm_peak, "bf16": bf16_peak, "fp32": fp32_peak, "fp64": fp64_peak,
             "hbm_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
             "bf16_source": f"{peak_src} (MEASURED_PEAKS.json bf16_tflops)",
             "fma_source": "measured in this run by xb_measure_fma_peaks"}
    roofs = rooflines(kernels, params, n_pix, "mixed", stamps, peaks)
    dominant = max(kernels, key=lambda k: kernels[k]["ms_total"]) if kernels else None

    # the batch: mixed with graphs, then the plain pipeline
    batch, run = batch_for(params, True)
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    wks = [batch.worker(i) for i in range(batch.n_workers)]
    l0 = sum(wk.launches() for wk in wks)
    with ClockSampler(0) as clk:
        ms = timed(run, args.steps)
    launches = sum(wk.launches() for wk in wks) - l0
    d0 = dD[0].clone()
    hT = [torch.from_numpy(f[0]).pin_memory() for f in frames]
    hS = [torch.from_numpy(f[1]).pin_memory() for f in frames]
    hC = [torch.empty((h, w), dtype=torch.float32).pin_memory() for _ in range(B)]
    hD = [torch.empty((h, w), dtype=torch.float32).pin_memory() for _ in range(B)]

    def run_e2e():
        batch.run_ptrs([t.data_ptr() for t in hT], [t.data_ptr() for t in hS], [w] * B, [h] * B,
                       [t.data_ptr() for t in hC], [t.data_ptr() for t in hD])
    run_e2e()
    e2e_ms = timed(run_e2e, args.steps)
    batch.close()
    pbatch, prun = batch_for(params_for(xbach.XB_MODE_PLAIN), False)
    prun()
    torch.cuda.synchronize()
    p_steps = max(1, min(args.steps, 2))
    p_ms = timed(prun, p_steps)
    pbatch.close()

    # accuracy of frame 0: mixed (stage run = the batch's frame 0) against
    # the plain GPU result and the FP64 oracle
    from xbach import accuracy as acc
    pctx = xbach.Context(params_for(xbach.XB_MODE_PLAIN))
    pctx.init_device(dT[0].data_ptr(), dS[0].data_ptr(), w, h)
    for stage in (pctx.sss, pctx.cmv, pctx.cd, pctx.ksc, pctx.conv, pctx.sub):
        stage()
    single()
    torch.cuda.synchronize()
    _, threads, times, ores = cpu_frames_per_s(T, S, info, 1, params_kw=PARAMS_3)
    ref = {"diff": ores.image("diff"), "conv": ores.image("conv"),
           "solution": ores.array("solution", "float64"), "kernSum": ores.scalar("kernSum"),
           "convTemplate": ores.scalar("convTemplate")}
    n_comp, n_bg = acc.layout(params)
    mixed_r, plain_r = run_result(xbach, ctx), run_result(xbach, pctx)
    accuracy = {"chosen_vs_plain": acc.compare(mixed_r, plain_r, T, S, n_comp, n_bg),
                "chosen_vs_fp64_oracle": acc.compare(mixed_r, ref, T, S, n_comp, n_bg),
                "plain_vs_fp64_oracle": acc.compare(plain_r, ref, T, S, n_comp, n_bg),
                "kernel_sum": {"chosen": ctx.scalar("kernSum"), "plain": pctx.scalar("kernSum"),
                               "oracle": ores.scalar("kernSum"), "generator_flux_ratio": 1.1},
                "batch_frame0_equals_single": bool(torch.equal(
                    d0.cpu(), torch.from_numpy(ctx.image(xbach.XB_IMG_DIFF, f64=False))))}
    m = accuracy["chosen_vs_plain"]["diff"]["max_sigma"]
    accuracy["gate"] = {"uses": "chosen_vs_plain", "max_sigma": m, "bar": SIGMA_BAR,
                        "pass": bool(m <= SIGMA_BAR)}
    value = B * args.steps / (ms / 1000.0)
    plain_v = B * p_steps / (p_ms / 1000.0)
    roof = dict(roofs[dominant]) if dominant in roofs else None
    if roof is not None and "bound" not in roof:
        roof = dict(next(iter(roof.values())))
    if roof is not None:
        roof["kernel"] = dominant
        roof["traffic"] = None
    line = {
        "metric": "difference-images/s at 3072² (config 3), chosen vs plain GPU at ≤1e-3σ",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (preset 3: seeded 3072x3072 crowded fields, one seed per pair)",
        "config": {"workload": "3072x3072 FP32 pairs, 80k sources, 4 Gaussians (degrees 6/4/3/2, "
                               "59 basis functions), kernel order 3, background order 2 (587 "
                               "unknowns), 20x20 stamps",
                   "mode": "mixed", "frames_per_step": B, "workers": B, "frame_graphs": True,
                   "learned_ranking": None, "l2": "flushed before every step; inputs exceed L2",
                   "inputs": "device-resident FP32 T,S"},
        "e2e": {"value": B * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": B * 2 * 4 * n_pix, "d2h_bytes_per_step": B * 2 * 4 * n_pix},
        "gpu_launches": launches, "clocks": clk.summary(), "roofline": roof, "rooflines": roofs,
        "single_frame": {"value": 1000.0 / single_ms, "unit": UNIT, "ms_per_step": single_ms,
                         "path": "stages, host-driven (per-kernel timers on)"},
        "dominant_kernel": dominant, "kernels": kernels,
        "plain_gpu_batched": {"value": plain_v, "unit": UNIT, "ms_per_step": p_ms / p_steps,
                              "steps": p_steps, "frames_per_step": B},
        "chosen_over_plain": value / plain_v,
        "cpu_baseline": {"value": 1.0 / times[0], "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "frame pair 0, one full 3072x3072 pair (FP64 oracle, OpenMP "
                                   f"over {threads} host threads)"},
        "accuracy": accuracy,
    }
    print(json.dumps(line), flush=True)
    return 0


def _make_pair2(frame):
    sys.path.insert(0, str(PKG))
    from xbach.synth import make_pair
    return make_pair(2, frame=frame)


def run_files(args):
    """FITS in, FITS out: `--files` pairs per step stream through
    xb_pipeline (reader threads decode into pinned slots, `workers` contexts
    replay frame graphs, writer threads encode conv and sub).  The inputs are
    the headline's 2048^2 pairs written once as BITPIX -32 files to a
    RAM-backed directory (page cache: the figure is the pipeline's, not a
    disk's)."""
    import concurrent.futures
    import multiprocessing
    B = max(1, args.batch)
    with concurrent.futures.ProcessPoolExecutor(
            max_workers=min(16, os.cpu_count() or 1),
            mp_context=multiprocessing.get_context("spawn")) as ex:
        frames = list(ex.map(_make_pair2, range(B)))
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    import xbach
    from xbach_testlib import write_fits
    root = pathlib.Path("/dev/shm") if pathlib.Path("/dev/shm").is_dir() else None
    tmp = pathlib.Path(tempfile.mkdtemp(prefix="xbach_files_", dir=root))
    try:
        tps, sps = [], []
        for i, (T, S, _) in enumerate(frames):
            tps.append(tmp / f"t{i}.fits")
            sps.append(tmp / f"s{i}.fits")
            write_fits(tps[-1], T)
            write_fits(sps[-1], S)
        n = args.files
        T_list = [tps[i % B] for i in range(n)]
        S_list = [sps[i % B] for i in range(n)]
        convs = [tmp / f"conv{i}.fits" for i in range(n)]
        diffs = [tmp / f"sub{i}.fits" for i in range(n)]
        mode = xbach.XB_MODE_PLAIN if args.mode == "plain" else xbach.XB_MODE_MIXED
        params = frame_params(xbach, frames[0][2], mode)
        use_graph = bool(args.graph) and args.mode == "mixed"
        use_rank = bool(args.rank) and args.mode == "mixed"
        pl = xbach.Pipeline(params, workers=args.workers, io=args.io)
        if use_rank:
            from xbach import ranker
            w_rank = ranker.preset5_weights()
            for i in range(pl.n_workers):
                ranker.enable(pl.worker(i), w_rank, policy=1, tau=args.rank_tau)
        if use_graph:
            pl.set_option("graph", 1)
        for _ in range(max(args.warmup, 1)):
            pl.run_files(T_list, S_list, convs, diffs)
        launches0 = sum(pl.worker(i).launches() for i in range(pl.n_workers))
        wall, parts = [], []
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                t0 = time.perf_counter()
                pl.run_files(T_list, S_list, convs, diffs)
                wall.append(time.perf_counter() - t0)
                parts.append(pl.stats())
        launches = sum(pl.worker(i).launches() for i in range(pl.n_workers)) - launches0
        # every output of the last step against a single context's xb_run
        from xbach_testlib import read_fits
        same = []
        for i in range(min(B, n)):
            ctx = xbach.Context(params)
            if use_rank:
                ranker.enable(ctx, w_rank, policy=1, tau=args.rank_tau)
            ctx.run(frames[i][0], frames[i][1])
            same.append(bool(np.array_equal(read_fits(diffs[i]),
                                            ctx.image(xbach.XB_IMG_DIFF, f64=False).astype(np.float64))))
            ctx.close()
        pl.close()
    finally:
        import shutil
        shutil.rmtree(tmp, ignore_errors=True)
    total = sum(wall)
    per = {k: sum(p[k] for p in parts) / len(parts) for k in ("read_ms", "compute_ms", "write_ms")}
    line = {
        "metric": "difference-images/s at 2048², FITS files in and out (streaming pipeline)",
        "value": n * args.steps / total, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.mode == "plain" else "f32",
        "data": "synthetic (the headline's seeded 2048^2 fields as BITPIX -32 FITS files)",
        "config": {"workload": WORKLOAD, "mode": args.mode, "pairs_per_step": n,
                   "distinct_pairs": B, "workers": args.workers, "io_threads": args.io,
                   "frame_graphs": use_graph,
                   "learned_ranking": f"policy 1, tau {args.rank_tau}" if use_rank else None,
                   "files": "RAM-backed directory (page cache)",
                   "timing": "host wall clock around xb_pipeline_run_files"},
        "thread_ms_per_step": per,
        "fits_bytes_per_step": {"read": parts[-1]["bytes_read"], "written": parts[-1]["bytes_written"]},
        "gpu_launches": launches, "clocks": clk.summary(),
        "check_vs_single_context": {"pairs": min(B, n), "identical": same},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="mixed", choices=["plain", "mixed"],
                    help="mixed = the chosen pipeline (headline); plain = the FP64 path alone")
    ap.add_argument("--batch", type=int, default=24,
                    help="frame pairs per step, run concurrently (1 = one pair per step)")
    ap.add_argument("--workers", type=int, default=24, help="concurrent frames of a batch")
    ap.add_argument("--cpu-runs", type=int, default=6,
                    help="CPU baseline: oracle runs (median reported)")
    ap.add_argument("--cpu-single", type=int, default=1,
                    help="CPU baseline: also time one single-threaded oracle run")
    ap.add_argument("--config", type=int, default=2, choices=[2, 3, 4],
                    help="2: the headline 2048^2 workload; 3: 3072^2 with 59 basis functions, "
                         "kernel order 3, background order 2; 4: 64 pairs of mixed size")
    ap.add_argument("--pairs3", type=int, default=8, help="--config 3: pairs per step")
    ap.add_argument("--pairs", type=int, default=64, help="--config 4: pairs per step")
    ap.add_argument("--rank", type=int, default=1,
                    help="mixed mode: learned substamp order (policy 1, shipped weights) on (1) "
                         "or off (0)")
    ap.add_argument("--rank-tau", type=float, default=0.3,
                    help="learned ranking: accept-probability threshold of policy 1 (0.3 was "
                         "chosen on validation frames 100-111 of the workload, not the timed ones)")
    ap.add_argument("--graph", type=int, default=1,
                    help="mixed mode: replay every frame as one captured CUDA graph (1) or run "
                         "the stages host-driven (0)")
    ap.add_argument("--files", type=int, default=0,
                    help="> 0: stream this many 2048^2 FITS pairs per step through xb_pipeline "
                         "(FITS in and out) instead of the device-resident batch")
    ap.add_argument("--io", type=int, default=6, help="--files: reader and writer threads each")
    ap.add_argument("--ldl-cluster", type=int, default=16, choices=[8, 16],
                    help="batch workers: CTAs of the LDL^T cluster (identical factors)")
    args = ap.parse_args()
    use_graph = bool(args.graph) and args.mode == "mixed"
    use_rank = bool(args.rank) and args.mode == "mixed"
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 4:
        return run_config4(args)
    if args.config == 3:
        return run_config3(args)
    if args.files > 0:
        return run_files(args)

    rank, world, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__
    if rank == 0 or world == 1:
        __graft_entry__.build()
    if world > 1:
        dist.barrier()
        __graft_entry__._paths()
    import xbach
    from xbach import ranker
    from xbach.synth import make_pair
    rank_w = ranker.preset5_weights() if use_rank else None

    def with_rank(cx):
        if use_rank:
            ranker.enable(cx, rank_w, policy=1, tau=args.rank_tau)
        return cx

    B = max(1, args.batch)
    frames = [make_pair(2, frame=f) for f in rank_frames(rank, B)]
    T, S, info = frames[0]
    h, w = T.shape
    n_pix = w * h
    mode = xbach.XB_MODE_PLAIN if args.mode == "plain" else xbach.XB_MODE_MIXED
    params = frame_params(xbach, info, mode)
    dT = [torch.from_numpy(f[0]).cuda() for f in frames]
    dS = [torch.from_numpy(f[1]).cuda() for f in frames]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def make_pipeline(cx, i=0):
        def pipeline():
            cx.init_device(dT[i].data_ptr(), dS[i].data_ptr(), w, h)
            cx.sss()
            cx.cmv()
            cx.cd()
            cx.ksc()
            cx.conv()
            cx.sub()
        return pipeline

    def timed(run, st, steps):
        ms = 0.0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            if world > 1:
                dist.barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            run()
            e1.record(st)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
        torch.cuda.synchronize()
        return ms

    def max_ranks(ms):
        return max_over_ranks(ms, world, "cuda")

    # ---- one frame pair per step: per-kernel breakdown ----
    ctx = with_rank(xbach.Context(params, device=local))
    cst = torch.cuda.ExternalStream(ctx.stream())
    single = make_pipeline(ctx)
    for _ in range(args.warmup):
        single()
    torch.cuda.synchronize()
    ctx.set_option("time_kernels", 1)
    launches_single0 = ctx.launches()
    single_ms = max_ranks(timed(single, cst, args.steps))
    launches_single = ctx.launches() - launches_single0
    kernels = {}
    for name in ("mask_input", "spread_mask", "stamp_stats", "find_substamps", "compact_stamps",
                 "fill_w", "fill_finish", "gram_qb", "stamp_test_fit", "cd_select", "weights",
                 "stamp_dots", "build_matrix", "build_rhs", "global_lu", "global_lubksb",
                 "kernel_sum", "sigs", "cd_merit", "ksc_check", "conv_sub", "gram",
                 "fill_gram", "gram_scatter", "global_ldl", "lu_fallback", "global_solve",
                 "mx_build", "mx_scatter", "rank_score"):
        ms, n = ctx.kernel_time(name)
        if n:
            kernels[name] = {"ms_total": ms / args.steps, "launches": n / args.steps}
    ctx.set_option("time_kernels", 0)
    single_value = world * args.steps / (single_ms / 1000.0)
    single_graph = None
    if use_graph:
        # the same frame as a replayed graph (one launch, one synchronisation)
        gctx = with_rank(xbach.Context(params, device=local))
        gctx.set_option("graph", 1)
        gC = torch.empty((h, w), dtype=torch.float32, device="cuda")
        gD = torch.empty((h, w), dtype=torch.float32, device="cuda")

        def single_g():
            gctx.run_device(dT[0].data_ptr(), dS[0].data_ptr(), w, h, gC.data_ptr(),
                            gD.data_ptr())
        for _ in range(max(args.warmup, 2)):
            single_g()
        torch.cuda.synchronize()
        gl0 = gctx.launches()
        g_ms = max_ranks(timed(single_g, torch.cuda.ExternalStream(gctx.stream()),
                                    args.steps))
        single_graph = {"value": world * args.steps / (g_ms / 1000.0), "unit": UNIT,
                        "ms_per_step": g_ms / args.steps,
                        "gpu_launches": (gctx.launches() - gl0) / args.steps}

    # ---- the headline: B frame pairs per step through the batch API ----
    jst = torch.cuda.Stream()
    dC = [torch.empty((h, w), dtype=torch.float32, device="cuda") for _ in range(B)]
    dD = [torch.empty((h, w), dtype=torch.float32, device="cuda") for _ in range(B)]

    def make_batch(bparams, ranked, graphs):
        bt = xbach.Batch(bparams, device=local, workers=max(1, min(args.workers, B)))
        bt.set_stream(jst.cuda_stream)
        if ranked:
            for i in range(bt.n_workers):
                ranker.enable(bt.worker(i), rank_w, policy=1, tau=args.rank_tau)
        if bparams.mode == xbach.XB_MODE_MIXED:
            bt.set_option("ldl_cluster", args.ldl_cluster)
        if graphs:
            # every worker captures its graph before the timed steps
            bt.set_option("graph", 1)
            for i in range(bt.n_workers):
                bt.worker(i).run_device(dT[0].data_ptr(), dS[0].data_ptr(), w, h,
                                        dC[0].data_ptr(), dD[0].data_ptr())
            torch.cuda.synchronize()

        def run():
            bt.run_ptrs([t.data_ptr() for t in dT], [t.data_ptr() for t in dS], [w] * B,
                        [h] * B, [t.data_ptr() for t in dC], [t.data_ptr() for t in dD],
                        device=True)
        return bt, run

    def time_batch(bt, run, steps, warmup):
        for _ in range(warmup):
            run()
        torch.cuda.synchronize()
        wks = [bt.worker(i) for i in range(bt.n_workers)]
        l0 = sum(wk.launches() for wk in wks)
        with ClockSampler(local) as clk:
            tm = max_ranks(timed(run, jst, steps))
        return tm, sum(wk.launches() for wk in wks) - l0, clk.summary()

    if B > 1:
        batch, run_batch = make_batch(params, use_rank, use_graph)
        t_max, launches, clocks = time_batch(batch, run_batch, args.steps, args.warmup)
    else:
        with ClockSampler(local) as clk:
            t_max = max_ranks(timed(single, cst, args.steps))
        launches = launches_single
        clocks = clk.summary()
    value = job_value(world, B, args.steps, t_max)
    d0_headline = dD[0].clone() if B > 1 else None  # later batches reuse the output buffers

    # ---- end to end: host frames (pinned) in, host images out ----
    hT = [torch.from_numpy(f[0]).pin_memory() for f in frames]
    hS = [torch.from_numpy(f[1]).pin_memory() for f in frames]
    hC = [torch.empty((h, w), dtype=torch.float32).pin_memory() for _ in range(B)]
    hD = [torch.empty((h, w), dtype=torch.float32).pin_memory() for _ in range(B)]
    if B > 1:
        def run_e2e():
            batch.run_ptrs([t.data_ptr() for t in hT], [t.data_ptr() for t in hS], [w] * B,
                           [h] * B, [t.data_ptr() for t in hC], [t.data_ptr() for t in hD])
        est = jst
    else:
        L = xbach.lib()

        def run_e2e():
            rc = L.xb_run(ctx.h, ctypes.c_void_p(hT[0].data_ptr()), ctypes.c_void_p(hS[0].data_ptr()),
                          w, h, ctypes.c_void_p(hC[0].data_ptr()), ctypes.c_void_p(hD[0].data_ptr()))
            if rc:
                raise RuntimeError(L.xb_last_error(ctx.h).decode())
        est = cst
    run_e2e()
    e2e_ms = max_ranks(timed(run_e2e, est, args.steps))
    e2e = {"value": world * B * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
           "h2d_bytes_per_step": B * 2 * 4 * n_pix, "d2h_bytes_per_step": B * 2 * 4 * n_pix}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0
    hbm_peak, bf16_peak, peak_src = measured_peaks()
    dominant = max(kernels, key=lambda k: kernels[k]["ms_total"]) if kernels else None
    fp32_peak, fp64_peak = xbach.measure_fma_peaks(local)
    stamps = ctx.scalar("nstamps0") + ctx.scalar("nstamps1") + ctx.scalar("ksc_refills")
    peaks = {"hbm": hbm_peak, "bf16": bf16_peak, "fp32": fp32_peak, "fp64": fp64_peak,
             "hbm_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
             "bf16_source": f"{peak_src} (MEASURED_PEAKS.json bf16_tflops)",
             "fma_source": "measured in this run by xb_measure_fma_peaks (MEASURED_PEAKS.json "
                           "has no FP32/FP64 CUDA-core entry)"}
    roofs = rooflines(kernels, params, n_pix, args.mode, stamps, peaks)
    # the contract's object: the kernel with the most device time per frame
    roof = dict(roofs.get(dominant, {})) if dominant in roofs else None
    if roof is not None and "bound" not in roof:
        roof = dict(next(iter(roof.values())))
    if roof is not None:
        roof["kernel"] = dominant
        roof["traffic"] = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.mode == "plain" else "f32",
        "data": "synthetic (seeded 2048x2048 crowded fields, one seed per frame pair)",
        "config": {"workload": WORKLOAD, "mode": args.mode,
                   "frames_per_step": B, "concurrent_frames": min(args.workers, B) if B > 1 else 1,
                   "parallelism": f"replicas x{world}",
                   "l2": "flushed before every step (256 MB write); each step's inputs exceed L2",
                   "inputs": "device-resident FP32 T,S",
                   "frame_graphs": use_graph,
                   "learned_ranking": f"policy 1, tau {args.rank_tau}, xbach/ranker_preset5.npy "
                                      "(BF16 weights)" if use_rank else None,
                   "hw_queues": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                   "ldl_cluster": args.ldl_cluster if args.mode == "mixed" else None},
        "e2e": e2e, "gpu_launches": launches, "clocks": clocks, "roofline": roof,
        "rooflines": roofs,
        "single_frame": {"value": single_value, "unit": UNIT,
                         "ms_per_step": single_ms / args.steps, "gpu_launches": launches_single,
                         "path": "stages, host-driven (per-kernel timers on)"},
        "single_frame_graph": single_graph,
        "dominant_kernel": dominant, "kernels": kernels,
    }
    oracle_res = None
    if world == 1 and args.cpu_runs > 0:
        # the first --cpu-runs frame pairs of the batch, one oracle run each
        times = []
        threads = os.cpu_count() or 1
        for i in range(args.cpu_runs):
            Ti, Si, infoi = frames[i % B]
            _, threads, ti, res = cpu_frames_per_s(Ti, Si, infoi, 1)
            times.append(ti[0])
            if i == 0:
                oracle_res = res
        med = statistics.median(times)
        line["cpu_baseline"] = {"value": 1.0 / med, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"median over the batch's first {args.cpu_runs} frame "
                                          f"pairs, one full 2048x2048 pair each (FP64 oracle, "
                                          f"OpenMP over {threads} host threads)",
                                "seconds_per_frame": times}
        if args.cpu_single:
            _, _, t1, _ = cpu_frames_per_s(T, S, info, 1, threads=1)
            line["cpu_baseline"]["single_thread"] = {"value": 1.0 / t1[0], "unit": UNIT,
                                                     "cores": 1, "seconds_per_frame": t1[0]}
    if args.mode == "mixed" and world == 1:
        if B > 1:
            batch.close()
            # the chosen pipeline without the learned ranking, same batch
            if use_rank:
                ubatch, run_u = make_batch(params, False, use_graph)
                u_ms, _, u_clk = time_batch(ubatch, run_u, args.steps, args.warmup)
                line["chosen_unranked"] = {"value": B * args.steps / (u_ms / 1000.0), "unit": UNIT,
                                           "ms_per_step": u_ms / args.steps, "clocks": u_clk,
                                           "config": "same batch, frame graphs, no ranking"}
                ubatch.close()
            # the plain FP64 GPU pipeline through the same batch API: same
            # pairs, same workers, stages host-driven (plain mode has no graphs)
            pparams = frame_params(xbach, info, xbach.XB_MODE_PLAIN)
            pbatch, run_p = make_batch(pparams, False, False)
            p_steps = max(1, min(args.steps, 3))
            p_ms, _, p_clk = time_batch(pbatch, run_p, p_steps, 1)
            line["plain_gpu_batched"] = {"value": B * p_steps / (p_ms / 1000.0), "unit": UNIT,
                                         "ms_per_step": p_ms / p_steps, "steps": p_steps,
                                         "frames_per_step": B, "workers": min(args.workers, B),
                                         "clocks": p_clk}
            pbatch.close()
        # the plain pipeline one pair at a time, and the acceptance reference
        pctx = xbach.Context(frame_params(xbach, info, xbach.XB_MODE_PLAIN), device=local)
        make_pipeline(pctx)()
        p_steps = max(1, min(args.steps, 3))
        p_ms = timed(make_pipeline(pctx), torch.cuda.ExternalStream(pctx.stream()), p_steps)
        line["plain_gpu_single"] = {"value": p_steps / (p_ms / 1000.0), "unit": UNIT,
                                    "ms_per_step": p_ms / p_steps, "steps": p_steps}
        plain_ref = line.get("plain_gpu_batched", line["plain_gpu_single"])
        line["chosen_over_plain"] = value / plain_ref["value"]
        line["chosen_over_plain_basis"] = ("plain_gpu_batched (same batch API, pairs and workers)"
                                           if "plain_gpu_batched" in line else "plain_gpu_single")
        line["chosen_over_plain_single"] = value / line["plain_gpu_single"]["value"]
        make_pipeline(ctx)()
        prctx = uctx = None
        if use_rank:
            prctx = with_rank(xbach.Context(frame_params(xbach, info, xbach.XB_MODE_PLAIN),
                                            device=local))
            make_pipeline(prctx)()
            uctx = xbach.Context(params, device=local)
            make_pipeline(uctx)()
        torch.cuda.synchronize()
        line["accuracy"] = accuracy(xbach, ctx, pctx, oracle_res, T, S, params, prctx, uctx)
        if B > 1:
            same = bool(torch.equal(d0_headline.cpu(),
                                    torch.from_numpy(ctx.image(xbach.XB_IMG_DIFF, f64=False))))
            line["accuracy"]["batch_frame0_equals_single"] = same
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
