"""Benchmark: input frames/s of the hologram pipeline on one GB300 (replicas on N GPUs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload cfg1]

A step is one batch of B raw frames pushed through the Pipe (convert + spatial propagation +
ring + time transform + view + render + uint16). Prints ONE JSON line (rank 0):
  value      whole-job input frames/s, inputs resident in HBM, timed with CUDA events on the
             pipe's stream (max over ranks), inputs larger than L2 (the time ring and the
             cycled input batches exceed the 129 MB L2)
  e2e        the same through the public API from pinned host memory: every step copies its
             raw batch host->device and reads its uint16 hologram device->host
  latency_ms p50 / p99 frame-to-hologram latency of the e2e steps (push start -> output on host)
  roofline   dominant kernel: algorithmic bytes / CUDA-event duration vs MEASURED_PEAKS.json
  cpu_baseline the FP64 numpy oracle (the reference has no CPU path) on a bounded sample
The path does not shard (one stream per GPU): N GPUs run N independent replicas ("replicas only").
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DEFAULT_WORKLOAD = "cfg1"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--server-mode", default="stream", choices=["bucket", "stream", "eager"],
                    help="serving workloads: one CUDA graph per stream on its own CUDA stream (default), one "
                         "graph per shape bucket, or no graphs")
    return ap.parse_args()


# ------------------------------------------------------------------------------------ helpers
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_throughput(ms_local: float, frames_per_rank: int, world: int, device: str = "cuda"):
    """Replicas (one independent pipe per GPU, no collective on the data path): the slowest
    rank's time (max over ranks) and the whole job's frames / that time. (ms, frames/s)."""
    import torch

    ms = ms_local
    if world > 1:
        t = torch.tensor([ms_local], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, frames_per_rank * world / (ms * 1e-3)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


# ------------------------------------------------------------------------------------ workloads
def make_workload(name: str):
    import holovibes_gb300 as hv
    from holovibes_gb300.synthetic import CONFIGS, generator, settings_for

    c = CONFIGS[name]
    fd = hv.FrameDescriptor(c["width"], c["height"], c["depth"])
    s = settings_for(name).validate(fd)
    return c, fd, s, generator(name, seed=1234)


def unique_batches(gen, B: int, nbatches: int, frames_cap: int):
    """nbatches distinct batches built from at most frames_cap generated frames (cyclic reuse)."""
    nf = min(frames_cap, B * nbatches)
    frames = gen.frames(0, nf)
    idx = np.arange(B * nbatches) % nf
    return frames[idx].reshape(nbatches, B, *frames.shape[1:])


def algorithmic_bytes_per_frame(fd, s):
    """B_alg = HW * (b + 8 + 8*T/S + 2/S): raw read, ring write, T/S ring reads, uint16 output."""
    HW = fd.width * fd.height
    T, S = s.time_transformation_size, s.time_stride
    return HW * (fd.depth + 8 + 8.0 * T / S + 2.0 / S)


# ------------------------------------------------------------------------------------ CPU oracle
def cpu_oracle_run(c, fd, s, gen, budget_s: float, max_batches: int | None = None):
    """Times the FP64 numpy oracle (OraclePipe) on whole batches of the same workload until the
    budget is spent; returns (frames/s, frames, seconds, batches)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import holovibes_oracle as O

    names = ({0: "NONE", 1: "FRESNELTR", 2: "ANGULARSP"}, {0: "NONE", 1: "STFT", 2: "PCA"},
             {0: "MODULUS", 1: "SQUARED_MODULUS", 2: "ARGUMENT"})
    os_ = O.OracleSettings(
        width=fd.width, height=fd.height, depth=fd.depth, space_transformation=names[0][s.space_transformation],
        time_transformation=names[1][s.time_transformation], time_transformation_size=s.time_transformation_size,
        time_stride=s.time_stride, batch_size=s.batch_size, lam=s.lambda_, z=s.z_distance, pixel_size=s.pixel_size,
        image_type=names[2][s.image_type], p_start=s.p_start, p_width=s.p_width, fft_shift=bool(s.fft_shift),
        renorm=bool(s.renorm), renorm_constant=s.renorm_constant, accumulation=s.accumulation,
        contrast_enabled=bool(s.contrast_enabled), contrast_lower=s.contrast_lower, contrast_upper=s.contrast_upper,
        unwrap_2d=bool(s.unwrap_2d))
    pipe = O.OraclePipe(os_)
    B = s.batch_size
    batch = gen.frames(0, B)
    # fill the ring untimed so every timed batch renders like the steady state
    fill = max(0, s.time_transformation_size // max(1, B) - 1) * (s.time_stride // B)
    for _ in range(fill):
        pipe.process_batch(batch)
    n = 0
    t0 = time.perf_counter()
    while True:
        pipe.process_batch(batch)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (max_batches and n >= max_batches):
            break
    return n * B / el, n * B, el, n


# ------------------------------------------------------------------------------------ reference arm
def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    c, fd, s, gen = make_workload(args.workload)
    cores = os.cpu_count() or 1
    budget = max(5.0, min(120.0, 2.0 * args.steps))  # bounded: the run ends within a few minutes
    fps, frames, el, nb = cpu_oracle_run(c, fd, s, gen, budget_s=min(budget, 60.0), max_batches=args.steps)
    line = {
        "metric": "input frames/s", "value": fps, "unit": "frames/s", "n_gpus": args.gpus, "steps": nb,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / nb, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded interferograms)", "impl": "reference",
        "config": {"workload": f"{args.workload}: {c['desc']}", "width": fd.width, "height": fd.height,
                   "batch": s.batch_size, "time_transformation_size": s.time_transformation_size},
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": f"{nb} batches of {s.batch_size} frames through the FP64 numpy oracle "
                                   f"(scipy.fft with {cores} workers; FFTW unavailable)"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------ our arm
def time_kernel(fn, stream, n=20):
    import torch

    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(n):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / n  # ms


def steps_for(hv, fd, s, dev_batch, stream):
    """Single-kernel launches of the workload's hot path on `stream`, each with its algorithmic
    bytes per launch (minimal DRAM traffic of that kernel: inputs read once, outputs written once)."""
    import torch

    L = hv.lib()
    W, H, B, T = fd.width, fd.height, s.batch_size, s.time_transformation_size
    HW = W * H
    buf = lambda n: torch.empty(max(int(n), 16), dtype=torch.uint8, device="cuda")
    lens, work, ring = buf(HW * 8), buf(B * HW * 8), buf(T * HW * 8)
    # the FFT timings below fill only B of the T ring frames: start from finite sample values so
    # that no kernel reads uninitialised memory
    gen = torch.Generator(device="cuda").manual_seed(0)
    ring.view(torch.float32).normal_(0.0, 1000.0, generator=gen)
    work.view(torch.float32).normal_(0.0, 1000.0, generator=gen)
    if s.space_transformation == hv.SPACE_FRESNELTR:
        L.hv_fresnel_lens(lens.data_ptr(), W, H, s.lambda_, s.z_distance, s.pixel_size, s.lens_mode, stream)
    else:
        L.hv_angular_spectrum_lens(lens.data_ptr(), W, H, s.lambda_, s.z_distance, s.pixel_size, s.lens_mode, stream)
    raw = dev_batch.data_ptr()
    out = []
    if s.space_transformation == hv.SPACE_FRESNELTR:
        out.append(("fft_rows(convert*lens)", lambda: L.hv_fft_rows(raw, fd.depth, 0, work.data_ptr(), W, H, B,
                                                                    lens.data_ptr(), 0, 1.0, 0, B, stream),
                    B * HW * (fd.depth + 8)))
        out.append(("fft_cols(->ring)", lambda: L.hv_fft_cols(work.data_ptr(), ring.data_ptr(), W, H, B, None, 0, 1.0,
                                                              0, T, stream), B * HW * 16))
    elif s.space_transformation == hv.SPACE_ANGULARSP:
        out.append(("fft_rows(convert)", lambda: L.hv_fft_rows(raw, fd.depth, 0, work.data_ptr(), W, H, B, None, 0,
                                                               1.0, 0, B, stream), B * HW * (fd.depth + 8)))
        # out of place (the pipe runs it in place): repeated in-place launches would scale the
        # unnormalised forward * G * inverse by H W per launch into Inf / NaN, and the views'
        # atan2 is slower on non-finite and all-zero samples than on image data
        work2 = buf(B * HW * 8)
        out.append(("fft_cols(fwd*G,inv)", lambda: L.hv_fft_cols(work.data_ptr(), work2.data_ptr(), W, H, B,
                                                                 lens.data_ptr(), 2, 1.0, 0, B, stream), B * HW * 16))
        out.append(("fft_rows(inv->ring)", lambda: L.hv_fft_rows(work2.data_ptr(), 8, 0, ring.data_ptr(), W, H, B,
                                                                 None, 1, 1.0 / HW, 0, T, stream), B * HW * 16))
    pmin = s.p_start
    pmax = min(s.p_start + s.p_width, T) if s.p_width else s.p_start
    pmax = min(pmax, T - 1)
    K = pmax - pmin + 1
    wts = buf(K * T * 8)
    L.hv_stft_weights(wts.data_ptr(), T, pmin, pmax, stream)
    view = buf(HW * 4)
    tc_ws = L.hv_time_view_tc_workspace(K, T)
    if K >= 8 and tc_ws and HW % 2 == 0:
        # the pipe's automatic engine for K >= 8 bins: tcgen05; the weights are split once (as the
        # pipe does per settings refresh) and only the contraction kernel is timed
        vw = buf(tc_ws)
        hv.check(L.hv_time_view_tc_prepare(wts.data_ptr(), K, T, vw.data_ptr(), stream), "view_tc prepare")
        out.append(("time_view_tc", lambda: L.hv_time_view_tc_run(ring.data_ptr(), T, W, H, K, s.image_type, 1.0,
                                                                  s.fft_shift, view.data_ptr(), None, vw.data_ptr(),
                                                                  stream), T * HW * 8 + HW * 4))
    else:
        out.append(("time_view", lambda: L.hv_time_view(ring.data_ptr(), T, W, H, wts.data_ptr(), K, s.image_type,
                                                        1.0, s.fft_shift, view.data_ptr(), None, stream),
                    T * HW * 8 + HW * 4))
    if s.time_transformation == hv.TIME_PCA:
        cov, cw = buf(T * T * 16), buf(L.hv_pca_cov_workspace(T, HW))
        out.append(("pca_covariance", lambda: L.hv_pca_covariance(ring.data_ptr(), T, HW, cov.data_ptr(),
                                                                  cw.data_ptr(), stream), T * HW * 8))
    return out


# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the dominant kernel, from the ncu
# captures of the same launch summarised in profiles/ (k_fft_cols_w32_tma_1024x1024.md,
# launches_cfg2_768x768_u16_as_stft_T256_K33.md, launches_cfg0_512x512_u16_as_stft_T16.md)
NCU_TRAFFIC = {
    ("cfg0", "fft_cols(fwd*G,inv)"): 35712256 + 1280,
    ("cfg1", "fft_cols(->ring)"): 268523520 + 214097664,
    ("cfg2", "time_view_tc"): 1208223232 + 5527808,
    ("cfg2", "fft_cols(fwd*G,inv)"): 307309312 + 245959936,
}


def roofline(hv, fd, s, dev_batch, peak_gbs, peak_src, workload=""):
    """Dominant kernel measured alone with CUDA events on its launching stream."""
    import torch

    stream = torch.cuda.Stream()
    kernels = steps_for(hv, fd, s, dev_batch, stream.cuda_stream)
    rows = []
    with torch.cuda.stream(stream):
        for name, fn, alg_bytes in kernels:
            ms = time_kernel(lambda: hv.check(fn(), name), stream)
            rows.append((name, ms, alg_bytes))
    name, ms, alg = max(rows, key=lambda r: r[1])
    achieved = alg / (ms * 1e-3) / 1e9
    traffic = NCU_TRAFFIC.get((workload, name))
    return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
            "frac": achieved / peak_gbs, "traffic": traffic, "peak_source": peak_src,
            "per_launch_bytes": alg, "ms_per_launch": ms,
            "all": {n: {"ms": round(m, 5), "GB/s": round(b / (m * 1e-3) / 1e9, 1)} for n, m, b in rows}}


def run_ours(args):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    import holovibes_gb300 as hv

    hv.lib()
    c, fd, s, gen = make_workload(args.workload)
    B = s.batch_size
    HW = fd.width * fd.height
    nb_unique = 4
    batches = unique_batches(gen, B, nb_unique, frames_cap=2 * B)
    dev_batches = torch.from_numpy(batches.reshape(nb_unique, -1).view(np.uint8)).cuda()
    frame_bytes = HW * fd.depth
    pipe = hv.Pipe(fd, s)
    stream = torch.cuda.ExternalStream(pipe.stream)

    def step(i):
        pipe.enqueue_ptr(dev_batches[i % nb_unique].data_ptr(), B, hv.MEM_DEVICE)

    # fill the ring and warm up
    fill = max(0, s.time_transformation_size // B - 1) * (s.time_stride // B)
    for i in range(fill + args.warmup):
        step(i)
    pipe.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = pipe.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for i in range(args.steps):
            step(i)
        pipe.join()  # the rendering stream joins the pipe stream before the closing event
        e1.record(stream)
        torch.cuda.synchronize()
    launches = pipe.kernel_launches() - launches0
    ms, value = replica_throughput(e0.elapsed_time(e1), args.steps * B, world)

    # e2e through the public API from pinned host memory, with per-step latency
    host_in = torch.from_numpy(batches.reshape(nb_unique, -1).view(np.uint8)).pin_memory()
    host_out = torch.empty(HW * 2, dtype=torch.uint8).pin_memory()
    while pipe.output_count():
        pipe.pull_into(host_out.data_ptr(), hv.MEM_HOST)
    # acquisition-style loop with one batch in flight: push batch i (its H2D copy), then read the
    # hologram of batch i-1 back to the host (D2H); latency = push start -> hologram on the host
    lat = []
    e2e_steps = args.steps
    if world > 1:
        torch.distributed.barrier()
    pushed = []
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        pushed.append(time.perf_counter())
        pipe.enqueue_ptr(host_in[i % nb_unique].data_ptr(), B, hv.MEM_HOST)
        while pipe.output_count() > 1:
            pipe.pull_into(host_out.data_ptr(), hv.MEM_HOST)
            lat.append(time.perf_counter() - pushed.pop(0))
    while pipe.output_count():
        pipe.pull_into(host_out.data_ptr(), hv.MEM_HOST)
        lat.append(time.perf_counter() - pushed.pop(0))
    pipe.sync()
    t_e2e_ms, e2e_value = replica_throughput((time.perf_counter() - t0) * 1e3, e2e_steps * B, world)
    lat_ms = np.array(lat) * 1e3 if lat else np.array([float("nan")])

    peak_gbs, _, peak_src = measured_peaks()
    rl = roofline(hv, fd, s, dev_batches[0], peak_gbs, peak_src, args.workload) if rank == 0 else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        fps, frames, el, nb = cpu_oracle_run(c, fd, s, gen, budget_s=args.cpu_budget_s)
        cpu = {"value": fps, "unit": "frames/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{nb} batches of {B} frames ({frames} frames, {el:.1f} s) through the FP64 numpy "
                         f"oracle, scipy.fft workers={os.cpu_count()} (FFTW unavailable)"}
    pipe.close()
    if rank == 0:
        balg = algorithmic_bytes_per_frame(fd, s)
        line = {
            "metric": "input frames/s", "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FFT, views), bf16x3/f32 (PCA covariance), f64 (eigensolve)",
            "data": "synthetic (seeded interferograms, generator in holovibes_gb300/synthetic.py)",
            "config": {"workload": f"{args.workload}: {c['desc']}", "width": fd.width, "height": fd.height,
                       "depth_bytes": fd.depth, "batch": B, "time_stride": s.time_stride,
                       "time_transformation_size": s.time_transformation_size,
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2: time ring %d MB + %d cycled input batches of %d MB" % (
                           HW * 8 * s.time_transformation_size >> 20, nb_unique, B * frame_bytes >> 20),
                       "B_alg_bytes_per_frame": balg},
            "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": B * frame_bytes,
                    "d2h_bytes_per_step": HW * 2},
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99))},
            "pipeline_hbm_frac": value / world * balg / (peak_gbs * 1e9),
            "gpu_launches": int(launches),
            "roofline": rl,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0



# ------------------------------------------------------------------------------------ serving
SERVE_WORKLOADS = {
    "serve512": "12 streams of 512x512 u16, angular spectrum + STFT T=32, B=S=8, modulus p=1, per-stream z/lambda",
    "cfg4": "12 streams, {256x256, 512x512, 1024x768, 1024x1024} x {u8, u16}, STFT or PCA, T in {16,32,64,128}, "
            "B=S=T/4 (>= 4), z in [0.2, 0.6] m, lambda in {785, 852} nm",
}


def serve_streams(name: str, only: int | None = None):
    """(fd, settings, batches[nb][B*frame_bytes] uint8) per stream, seeded; `only` keeps one stream
    (the same one as in the full list)."""
    import holovibes_gb300 as hv
    from holovibes_gb300.synthetic import Interferogram

    rng = np.random.default_rng(4242)
    out = []
    for i in range(12):
        if name == "serve512":
            W, H, depth, tt, T = 512, 512, 2, 1, 32
        else:
            W, H = [(256, 256), (512, 512), (1024, 768), (1024, 1024)][i % 4]
            depth = 1 + (i // 4) % 2
            tt = 1 if i % 3 else 2
            T = [16, 32, 64, 128][int(rng.integers(0, 4))]
        B = 8 if name == "serve512" else max(4, T // 4)
        z = float(rng.uniform(0.2, 0.6))
        lam = [785e-9, 852e-9][int(rng.integers(0, 2))]
        fd = hv.FrameDescriptor(W, H, depth)
        over = dict(space_transformation=2, time_transformation=tt, time_transformation_size=T, time_stride=B,
                    batch_size=B, z_distance=z, lambda_=lam, pixel_size=20.0, p_start=1, fft_shift=1, renorm=1,
                    contrast_enabled=1, contrast_lower=0.5, contrast_upper=99.5)
        if tt == 2:
            over.update(p_start=T - 4, p_width=3, image_type=1)
        s = hv.Settings.defaults().update(**over).validate(fd)
        if only is not None and i != only:
            continue
        g = Interferogram(width=W, height=H, seed=100 + i, dtype=np.uint8 if depth == 1 else np.uint16,
                          max_value=255 if depth == 1 else 4095, z=z, lam=lam, modes=6 if tt == 2 else 0)
        frames = g.frames(0, 2 * B)
        out.append((fd, s, frames.reshape(2, -1).view(np.uint8)))
    return out


def _plain_process(idx: int, workload: str, steps: int, warmup: int, barrier, queue) -> None:
    """One stream on one hv_pipe in its own process (one CUDA context), as the reference is run:
    one Holovibes instance, one compute pipeline, per stream. Same client loop as the in-process
    arms: push one batch from pinned memory, read back the holograms."""
    import torch

    import holovibes_gb300 as hv

    try:
        torch.cuda.set_device(0)
        (fd, s, b), = serve_streams(workload, only=idx)
        pinned = torch.from_numpy(b.copy()).pin_memory()
        out = torch.empty(fd.width * fd.height * 2, dtype=torch.uint8).pin_memory()
        pipe = hv.Pipe(fd, s)
        B = s.batch_size
        for k in range(s.time_transformation_size // B + warmup):
            pipe.enqueue_ptr(pinned[k % 2].data_ptr(), B, hv.MEM_HOST)
            while pipe.output_count():
                pipe.pull_into(out.data_ptr(), hv.MEM_HOST)
        pipe.sync()
        while pipe.output_count():
            pipe.pull_into(out.data_ptr(), hv.MEM_HOST)
        barrier.wait(timeout=600)
        lat, pushed = [], []
        t0 = time.perf_counter()
        for k in range(steps):
            pushed.append(time.perf_counter())
            pipe.enqueue_ptr(pinned[k % 2].data_ptr(), B, hv.MEM_HOST)
            while pipe.output_count():
                pipe.pull_into(out.data_ptr(), hv.MEM_HOST)
                if pushed:
                    lat.append(time.perf_counter() - pushed.pop(0))
        pipe.sync()
        while pipe.output_count():
            pipe.pull_into(out.data_ptr(), hv.MEM_HOST)
            if pushed:
                lat.append(time.perf_counter() - pushed.pop(0))
        t1 = time.perf_counter()
        pipe.close()
        queue.put((idx, steps * B, t0, t1, lat))
    except Exception as e:  # reported to the parent, which fails the arm
        queue.put((idx, -1, 0.0, 0.0, repr(e)))


def run_plain_processes(args, nstreams: int, steps: int) -> dict:
    """Aggregate input frames/s of one plain pipe per process over all streams (wall clock from
    the first timed push to the last hologram of any process)."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nstreams)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_plain_process, args=(i, args.workload, steps, args.warmup, barrier, queue))
             for i in range(nstreams)]
    for p in procs:
        p.start()
    res = [queue.get(timeout=900) for _ in procs]
    for p in procs:
        p.join(60)
    bad = [r for r in res if r[1] < 0]
    if bad:
        raise RuntimeError(f"plain process failed: {bad[0][4]}")
    t0 = min(r[2] for r in res)
    t1 = max(r[3] for r in res)
    lat = np.array([x for r in res for x in r[4]]) * 1e3
    return {"frames_per_s": sum(r[1] for r in res) / (t1 - t0), "processes": nstreams,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}}


def run_serving(args):
    """Served (hv_server: engine thread, shape buckets, CUDA graphs) vs plain (one hv_pipe per
    stream) on the same streams, from pinned host memory with holograms read back: one client
    thread pushes one batch per stream per step and reads back the holograms of the previous step."""
    import torch

    import holovibes_gb300 as hv

    torch.cuda.set_device(0)
    hv.lib()
    streams = serve_streams(args.workload)
    steps = max(20, min(args.steps, 400))
    pinned = [torch.from_numpy(b.copy()).pin_memory() for (_, _, b) in streams]
    outs = [torch.empty(fd.width * fd.height * 2, dtype=torch.uint8).pin_memory() for (fd, _, _) in streams]
    frames_per_step = sum(s.batch_size for (_, s, _) in streams)

    def drive(push, count, pull, nsteps, lat):
        pushed = [[] for _ in streams]
        t0 = time.perf_counter()
        for k in range(nsteps):
            for i, (fd, s, _) in enumerate(streams):
                pushed[i].append(time.perf_counter())
                push(i, pinned[i][k % 2].data_ptr(), s.batch_size)
            for i in range(len(streams)):
                while count(i) > 0:
                    pull(i, outs[i].data_ptr())
                    if pushed[i]:
                        lat.append(time.perf_counter() - pushed[i].pop(0))
        return t0

    results = {}
    with ClockSampler(0) as clk:
        # ---- plain: one Pipe per stream, driven by the client thread
        pipes = [hv.Pipe(fd, s) for (fd, s, _) in streams]
        push = lambda i, ptr, n: pipes[i].enqueue_ptr(ptr, n, hv.MEM_HOST)
        count = lambda i: pipes[i].output_count()
        pull = lambda i, ptr: pipes[i].pull_into(ptr, hv.MEM_HOST)
        warm = max(s.time_transformation_size // s.batch_size for (_, s, _) in streams) + args.warmup
        drive(push, count, pull, warm, [])
        for p in pipes:
            p.sync()
        lat = []
        t0 = drive(push, count, pull, steps, lat)
        for i, p in enumerate(pipes):
            p.sync()
            while p.output_count():
                p.pull_into(outs[i].data_ptr(), hv.MEM_HOST)
        el = time.perf_counter() - t0
        launches = sum(p.kernel_launches() for p in pipes)
        for p in pipes:
            p.close()
        results["plain"] = {"frames_per_s": steps * frames_per_step / el,
                            "latency_ms": {"p50": float(np.percentile(np.array(lat) * 1e3, 50)),
                                           "p99": float(np.percentile(np.array(lat) * 1e3, 99))}}
        # ---- served
        flags = {"bucket": 0, "stream": hv.SERVER_STREAM_GRAPHS, "eager": hv.SERVER_NO_GRAPHS}[args.server_mode]
        srv = hv.Server(flags=flags)
        sts = [srv.open_stream(fd, s) for (fd, s, _) in streams]
        push = lambda i, ptr, n: sts[i].enqueue_ptr(ptr, n, hv.MEM_HOST)
        count = lambda i: sts[i].output_count()
        pull = lambda i, ptr: sts[i].pull_into(ptr, hv.MEM_HOST)
        drive(push, count, pull, warm, [])
        srv.sync()
        for i, st in enumerate(sts):
            while st.output_count():
                st.pull_into(outs[i].data_ptr(), hv.MEM_HOST)
        srv.reset_stats()
        g0 = srv.stats()
        k0 = hv.kernel_launches()
        lat = []
        t0 = drive(push, count, pull, steps, lat)
        srv.sync()
        for i, st in enumerate(sts):
            while st.output_count():
                st.pull_into(outs[i].data_ptr(), hv.MEM_HOST)
        el = time.perf_counter() - t0
        g1 = srv.stats()
        eager_kernels = hv.kernel_launches() - k0
        srv.close()
        results["served"] = {"frames_per_s": steps * frames_per_step / el,
                             "latency_ms": {"p50": float(np.percentile(np.array(lat) * 1e3, 50)),
                                            "p99": float(np.percentile(np.array(lat) * 1e3, 99))},
                             "device_latency_ms": {"p50": g1["latency_p50_us"] / 1e3,
                                                   "p99": g1["latency_p99_us"] / 1e3},
                             "graph_launches": g1["graph_launches"] - g0["graph_launches"],
                             "graph_kernels": g1["graph_kernels"] - g0["graph_kernels"],
                             "eager_cycles": g1["eager_cycles"] - g0["eager_cycles"],
                             "eager_kernels": eager_kernels,
                             "buckets": g1["buckets"]}
    # one plain pipe per process (the reference's deployment: one instance per stream); outside
    # the clock sampler's window so the processes' start-up is not sampled
    results["plain_per_process"] = run_plain_processes(args, len(streams), steps)
    window_ms = min(1e3 * s.time_transformation_size / (results["served"]["frames_per_s"] / len(streams))
                    for (_, s, _) in streams)
    v = results["served"]["frames_per_s"]
    h2d = sum(b.shape[1] for (_, _, b) in streams)
    d2h = sum(fd.width * fd.height * 2 // s.time_stride * s.batch_size for (fd, s, _) in streams)
    line = {
        "metric": "input frames/s", "value": v, "unit": "frames/s", "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * frames_per_step / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FFT, views), bf16x3/f32 (PCA covariance)",
        "data": "synthetic (seeded interferograms, one seed per stream)",
        "config": {"workload": f"{args.workload}: {SERVE_WORKLOADS[args.workload]}", "streams": len(streams),
                   "server_mode": args.server_mode,
                   "frames_per_step": frames_per_step, "parallelism": "one GPU, streams overlapped",
                   "l2": "time rings of all streams exceed L2"},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "serving": {"served": results["served"], "plain": results["plain"],
                    "served_over_plain": v / results["plain"]["frames_per_s"],
                    "plain_per_process": results["plain_per_process"],
                    "served_over_plain_per_process": v / results["plain_per_process"]["frames_per_s"],
                    "shortest_window_ms_at_served_rate": window_ms},
        "gpu_launches": int(results["served"]["graph_kernels"] + results["served"]["eager_kernels"]),
        "roofline": None, "cpu_baseline": None, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in SERVE_WORKLOADS:
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
