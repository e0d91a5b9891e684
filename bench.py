"""Benchmark: input frames/s of the hologram pipeline on one GB300 (replicas on N GPUs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload cfg1]

A step is one batch of B raw frames pushed through the Pipe (convert + spatial propagation +
ring + time transform + view + render + uint16). Prints ONE JSON line (rank 0):
  value      whole-job input frames/s, inputs resident in HBM, timed with CUDA events on the
             pipe's stream (max over ranks), inputs larger than L2 (the time ring and the
             cycled input batches exceed the 129 MB L2)
  e2e        the same through the public API from pinned host memory: every step copies its
             raw batch host->device and reads its uint16 hologram device->host
  latency_ms p50 / p99 frame-to-hologram latency (push start -> hologram on the host), measured
             with batches pushed at 80% of the e2e rate (no queue in front of the pipe)
  roofline   the slowest hot kernel timed alone with CUDA events on its stream: algorithmic bytes
             (and tensor-core flops where it contracts) per launch over its duration, against
             MEASURED_PEAKS.json; `bound` is the roof it is closer to
  cpu_baseline the FP64 numpy oracle (and its FP32 twin) on a bounded sample of the workload; the
             same leg reports `parity`: the GPU Pipe's output on the sampled window against it
  serving    (default run) the served engine against plain pipes on 512x512 STFT-32 streams
  clocks     NVML SM clock and clock-event reasons sampled every 10 ms over the whole run
`--impl reference` times the CPU restatement of the path (the reference has no CPU
implementation; its own GPU build is timed beside it in `reference_gpu_build`).
The path does not shard (one stream per GPU): N GPUs run N independent replicas ("replicas only").
"""

from __future__ import annotations

import argparse
import ctypes
import hashlib
import importlib.util
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
SPACE_NAMES = {0: "NONE", 1: "FRESNELTR", 2: "ANGULARSP"}
TIME_NAMES = {0: "NONE", 1: "STFT", 2: "PCA", 3: "SSA_STFT"}
IMG_NAMES = {0: "MODULUS", 1: "SQUARED_MODULUS", 2: "ARGUMENT"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving comparison of the default run")
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


def load_synthetic():
    """holovibes_gb300/synthetic.py loaded on its own (plain numpy): the generator and the workload
    table, without importing the package, so the CPU arm never maps the product library."""
    name = "_hv_synthetic_standalone"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, ROOT / "holovibes_gb300" / "synthetic.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def load_oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import holovibes_oracle as O

    return O


class ClockSampler:
    """SM clock, maximum SM clock and clock-event reasons of one GPU, read every 10 ms through NVML
    (read-only queries of the driver's management library) from start to stop; nvidia-smi at
    100 ms when NVML cannot be loaded."""

    # NVML clock-event reason bits (nvmlClocksEventReason*)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}
    IDLE = 0x1

    def __init__(self, index: int, uuid: str | None = None, period_s: float = 0.01):
        self.index, self.uuid, self.period = index, uuid, period_s
        self.samples = []  # (sm_mhz, reasons bitmask)
        self.max_mhz = None
        self.source = None
        self._stop = threading.Event()
        self._thread = None
        self._proc = None

    def _nvml(self):
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = ctypes.c_void_p()
        rc = 1
        if self.uuid:
            rc = nv.nvmlDeviceGetHandleByUUID(self.uuid.encode(), ctypes.byref(h))
        if rc != 0:
            rc = nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h))
        if rc != 0:
            raise OSError("no NVML handle")
        reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        return nv, h, reasons_fn

    def start(self):
        try:
            nv, h, reasons_fn = self._nvml()
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:  # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            self.source = "nvml"

            def run():
                clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
                while not self._stop.is_set():
                    if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and \
                            reasons_fn(h, ctypes.byref(rs)) == 0:
                        self.samples.append((float(clk.value), int(rs.value)))
                    self._stop.wait(self.period)
                nv.nvmlShutdown()

            self._thread = threading.Thread(target=run, daemon=True)
            self._thread.start()
        except (OSError, AttributeError):
            self._start_smi()
        return self

    def _start_smi(self):
        query = "clocks.sm,clocks.max.sm,clocks_event_reasons.active"
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={query}",
                                           "--format=csv,noheader,nounits", "-lms", "100"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            return
        self.source = "nvidia-smi"

        def read():
            for line in self._proc.stdout:
                parts = [p.strip() for p in line.split(",")]
                try:
                    self.max_mhz = float(parts[1])
                    self.samples.append((float(parts[0]), int(parts[2], 16)))
                except (ValueError, IndexError):
                    continue

        self._thread = threading.Thread(target=read, daemon=True)
        self._thread.start()

    def stop(self):
        self._stop.set()
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._thread is not None:
            self._thread.join(timeout=5)

    def summary(self):
        busy = [(c, r) for c, r in self.samples if not r & self.IDLE]
        use = busy or self.samples
        reasons = sorted({n for _, r in use for bit, n in self.REASONS.items() if r & bit})
        return {"sm_mhz": float(np.median([c for c, _ in use])) if use else None, "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.samples), "samples_not_idle": len(busy),
                "source": self.source}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


# ------------------------------------------------------------------------------------ workloads
def workload_config(name: str, world: int = 1) -> tuple[dict, dict]:
    """(the workload's table entry, the `config` object both arms print)."""
    c = load_synthetic().CONFIGS[name]
    st = c["settings"]
    HW = c["width"] * c["height"]
    T, S, B = st["time_transformation_size"], st["time_stride"], st["batch_size"]
    cfg = {"workload": f"{name}: {c['desc']}", "width": c["width"], "height": c["height"], "depth_bytes": c["depth"],
           "batch": B, "time_stride": S, "time_transformation_size": T, "parallelism": f"replicas x{world}",
           "l2": "inputs larger than L2: time ring %d MB + 4 cycled input batches of %d MB" % (
               HW * 8 * T >> 20, B * HW * c["depth"] >> 20),
           "B_alg_bytes_per_frame": HW * (c["depth"] + 8 + 8.0 * T / S + 2.0 / S)}
    return c, cfg


def oracle_settings_for(c: dict, O, precision: str = "fp64"):
    """The oracle's settings for a workload-table entry (the library's defaults elsewhere)."""
    st = c["settings"]
    return O.OracleSettings(
        width=c["width"], height=c["height"], depth=c["depth"],
        space_transformation=SPACE_NAMES[st["space_transformation"]],
        time_transformation=TIME_NAMES[st["time_transformation"]],
        time_transformation_size=st["time_transformation_size"], time_stride=st["time_stride"],
        batch_size=st["batch_size"], lam=st["lambda_"], z=st["z_distance"], pixel_size=st["pixel_size"],
        image_type=IMG_NAMES[st["image_type"]], p_start=st["p_start"], p_width=st["p_width"],
        fft_shift=bool(st["fft_shift"]), renorm=bool(st["renorm"]), accumulation=st["accumulation"],
        contrast_enabled=bool(st["contrast_enabled"]), contrast_auto_refresh=bool(st["contrast_auto_refresh"]),
        contrast_lower=st["contrast_lower"], contrast_upper=st["contrast_upper"],
        unwrap_2d=bool(st.get("unwrap_2d", 0)), precision=precision)


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


def window_frames(gen, st: dict) -> list:
    """The raw batches up to and including the first rendered window (T / B batches)."""
    B, T, S = st["batch_size"], st["time_transformation_size"], st["time_stride"]
    n = max(1, (T + B - 1) // B) * (S // B)
    return [gen.frames(i * B, B) for i in range(n)]


# ------------------------------------------------------------------------------------ CPU legs
def cpu_oracle_run(c, batches, budget_s: float, precision: str = "fp64", max_batches: int | None = None):
    """Times the numpy oracle (OraclePipe, FP64 or its FP32 twin) on whole batches of the workload:
    the ring is filled untimed, then the window's last batch is pushed until the budget is spent.
    Returns (frames/s, frames, seconds, batches, the first timed output)."""
    O = load_oracle()
    pipe = O.OraclePipe(oracle_settings_for(c, O, precision))
    B = c["settings"]["batch_size"]
    for b in batches[:-1]:
        pipe.process_batch(b)
    n = 0
    first = None
    t0 = time.perf_counter()
    while True:
        out = pipe.process_batch(batches[-1])
        if first is None:
            first = out
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (max_batches and n >= max_batches):
            break
    return n * B / el, n * B, el, n, first


def parity_against(hv, O, fd, s, batches, ref_out) -> dict:
    """A fresh Pipe on the same window as the oracle's first timed output: rel-L2 of the float
    frame fed to the contrast stage (argument views: wrapped differences, branch-cut pixels
    counted apart), uint16 mismatches against the oracle's contrast stage on the GPU's own float
    frame, and for PCA the relative error of the kept eigenvalues."""
    pipe = hv.Pipe(fd, s)
    for b in batches[:-1]:
        pipe.enqueue(b)
    pipe.enqueue(batches[-1])
    got_u16 = pipe.pull()
    got_f = pipe.float_frame()
    lo, hi = pipe.contrast_range()
    ring = pipe.ring()[0] if s.time_transformation == hv.TIME_PCA else None
    pipe.close()
    ref = ref_out.float_frame
    res = {"output": "first rendered window of the sample"}
    if s.image_type == hv.IMG_ARGUMENT and not s.unwrap_2d:
        wd = (got_f - ref + np.pi) % (2 * np.pi) - np.pi
        cut = np.abs(wd) > 1e-3
        res["rel_l2"] = float(np.linalg.norm(wd[~cut]) / np.linalg.norm(ref[~cut]))
        res["branch_cut_fraction"] = float(np.mean(cut))
    else:
        res["rel_l2"] = float(np.linalg.norm(got_f - ref) / np.linalg.norm(ref))
    res["u16_mismatch"] = int(np.count_nonzero(got_u16 != O.float_to_ushort(O.apply_contrast(got_f, lo, hi))))
    if ring is not None:
        import torch

        T = s.time_transformation_size
        L = hv.lib()
        npix = fd.width * fd.height
        rd = torch.from_numpy(ring.view(np.float32)).cuda()
        cov = torch.empty(T * T * 2, dtype=torch.float64, device="cuda")
        cw = torch.empty(max(16, L.hv_pca_cov_workspace(T, npix)), dtype=torch.uint8, device="cuda")
        hv.check(L.hv_pca_covariance(rd.data_ptr(), T, npix, cov.data_ptr(), cw.data_ptr(), None), "covariance")
        ev = torch.empty(T, dtype=torch.float64, device="cuda")
        vec = torch.empty(T * T * 2, dtype=torch.float64, device="cuda")
        ew = torch.empty(max(16, L.hv_pca_eigh_workspace(T)), dtype=torch.uint8, device="cuda")
        hv.check(L.hv_pca_eigh(cov.data_ptr(), T, ev.data_ptr(), vec.data_ptr(), 0, 0, None, ew.data_ptr(), None),
                 "eigh")
        got_w = ev.cpu().numpy()
        ref_w, _ = O.pca_eigh(O.pca_covariance(ring.astype(np.complex128)))
        pmin, pmax = O.p_range(s.p_start, s.p_width, T)
        k = slice(pmin, pmax + 1)
        res["eig_rel_err_kept"] = float(np.max(np.abs(got_w[k] - ref_w[k]) / np.abs(ref_w[k])))
    return res


# ------------------------------------------------------------------------------------ reference arm
def reference_gpu_build(c, batches, steps: int, warmup: int) -> dict:
    """The reference's own GPU build (unmodified cuFFT / cuBLAS / cuSOLVER translation units, one
    Pipe cycle per batch with its stream synchronisations) on device-resident batches."""
    sys.path.insert(0, str(ROOT / "oracle"))
    try:
        import ref_pipe
        import torch

        if not ref_pipe.available():
            return {"unavailable": "reference sources not staged (oracle/ref_build.py stages them from the "
                                   "reference tree)"}
        O = load_oracle()
        rp = ref_pipe.RefPipe.from_oracle_settings(oracle_settings_for(c, O), keep_float_frame=False)
        dev = [torch.from_numpy(np.ascontiguousarray(b).reshape(-1).view(np.uint8)).cuda() for b in batches]
        ptrs = [d.data_ptr() for d in dev]
        B, T = c["settings"]["batch_size"], c["settings"]["time_transformation_size"]
        rp.run_device_batches(ptrs, max(1, T // B) + warmup)
        ms = rp.run_device_batches(ptrs, steps)
        rp.close()
        return {"value": steps * B / (ms * 1e-3), "unit": "frames/s", "ms_per_step": ms / steps, "steps": steps,
                "inputs": "device-resident raw batches (the BatchInputQueue's device slots)",
                "what": "the reference's hot-path translation units compiled unmodified for sm_103a, one Pipe "
                        "cycle per batch in Pipe::refresh order with its host synchronisations"}
    except Exception as e:  # reported, the CPU line stands
        return {"unavailable": f"{type(e).__name__}: {e}"}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    if args.workload in SERVE_WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": "the reference runs one pipeline per process and has "
                                                              "no serving engine; serving is compared against "
                                                              "plain pipes by the default arm"}), flush=True)
        return 0
    c, cfg = workload_config(args.workload, world)
    cfg["parallelism"] = f"replicas x{world}"
    gen = load_synthetic().generator(args.workload, seed=1234)
    st = c["settings"]
    cores = os.cpu_count() or 1
    batches = window_frames(gen, st)
    budget = max(5.0, min(60.0, 2.0 * args.steps))  # bounded: the run ends within a few minutes
    fps, frames, el, nb, _ = cpu_oracle_run(c, batches, budget_s=budget, max_batches=args.steps)
    line = {
        "metric": "input frames/s", "value": fps, "unit": "frames/s", "n_gpus": args.gpus, "steps": nb,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / nb, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded interferograms)", "impl": "reference",
        "config": cfg,
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": f"{nb} batches of {st['batch_size']} frames through the FP64 numpy oracle "
                                   f"(scipy.fft with {cores} workers; FFTW unavailable); the reference has no CPU "
                                   f"implementation of this path"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_cpu_baseline:
        line["reference_gpu_build"] = reference_gpu_build(c, batches, steps=max(args.steps, 20), warmup=args.warmup)
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------ our arm
def time_kernel(fn, stream, n=20, reps=3):
    """Device time of one call of `fn` (ms) and how it was taken. The n calls are captured in a CUDA
    graph and replayed, so that the host's enqueue rate (a ctypes call and its launches take tens of
    microseconds on the host cores) does not set the figure for kernels of 50-100 us; calls that
    cannot be captured are timed as n eager launches."""
    import torch

    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            for _ in range(n):
                fn()
        g.replay()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            g.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / (n * reps), "graph"
    except Exception:
        torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(n):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / n, "eager"


def steps_for(hv, fd, s, dev_batch, stream):
    """Single-kernel launches of the workload's hot path on `stream`, each with its algorithmic
    bytes per launch (minimal DRAM traffic: inputs read once, outputs written once) and, for the
    tensor-core contractions, its tensor flops per launch (split-BF16: 3 BF16 products per FP32
    product)."""
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
                    B * HW * (fd.depth + 8), 0))
        out.append(("fft_cols(->ring)", lambda: L.hv_fft_cols(work.data_ptr(), ring.data_ptr(), W, H, B, None, 0, 1.0,
                                                              0, T, stream), B * HW * 16, 0))
    elif s.space_transformation == hv.SPACE_ANGULARSP:
        out.append(("fft_rows(convert)", lambda: L.hv_fft_rows(raw, fd.depth, 0, work.data_ptr(), W, H, B, None, 0,
                                                               1.0, 0, B, stream), B * HW * (fd.depth + 8), 0))
        # out of place (the pipe runs it in place): repeated in-place launches would scale the
        # unnormalised forward * G * inverse by H W per launch into Inf / NaN, and the views'
        # atan2 is slower on non-finite and all-zero samples than on image data
        work2 = buf(B * HW * 8)
        out.append(("fft_cols(fwd*G,inv)", lambda: L.hv_fft_cols(work.data_ptr(), work2.data_ptr(), W, H, B,
                                                                 lens.data_ptr(), 2, 1.0, 0, B, stream), B * HW * 16,
                    0))
        out.append(("fft_rows(inv->ring)", lambda: L.hv_fft_rows(work2.data_ptr(), 8, 0, ring.data_ptr(), W, H, B,
                                                                 None, 1, 1.0 / HW, 0, T, stream), B * HW * 16, 0))
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
                                                                  stream), T * HW * 8 + HW * 4, 3 * 8 * HW * T * K))
    else:
        out.append(("time_view", lambda: L.hv_time_view(ring.data_ptr(), T, W, H, wts.data_ptr(), K, s.image_type,
                                                        1.0, s.fft_shift, view.data_ptr(), None, stream),
                    T * HW * 8 + HW * 4, 0))
    if s.time_transformation == hv.TIME_PCA:
        cov, cw = buf(T * T * 16), buf(L.hv_pca_cov_workspace(T, HW))
        real = 1 if s.space_transformation == hv.SPACE_NONE and not s.filter2d_enabled else 0
        pb = L.hv_pca_planes_bytes(T, HW, real)
        S = s.time_stride
        if pb and S < T:
            # the pipe's path for T > 64: each window's S new frames are split into BF16 planes (real
            # parts only for a real ring), and the covariance rows and columns of the slot blocks they
            # land in (64 frames, 128 for real planes; one window: slots 0 .. S-1) are recomputed from
            # the planes: every frame of the ring is read once, the tiles touching those blocks are
            # multiplied
            if real:
                # the pipe's ring without a spatial transform: imaginary parts 0
                ring.view(torch.float32).view(-1, 2)[:, 1].zero_()
            planes = buf(pb)
            hv.check(L.hv_pca_split_planes(ring.data_ptr(), T, HW, 0, T, real, planes.data_ptr(), stream), "split")
            fb = 128 if real else 64
            nb = (T + fb - 1) // fb
            blocks = 0
            for sl in range(S):
                blocks |= 1 << (sl // fb)
            tiles = sum(1 for bm in range(nb) for bn in range(bm, nb) if (blocks >> bm) & 1 or (blocks >> bn) & 1)
            out.append(("ring_split", lambda: L.hv_pca_split_planes(ring.data_ptr(), T, HW, 0, S, real,
                                                                    planes.data_ptr(), stream),
                        S * HW * (12 if real else 16), 0))
            out.append(("pca_covariance", lambda: L.hv_pca_covariance_planes(planes.data_ptr(), T, HW, real, blocks,
                                                                             cov.data_ptr(), cw.data_ptr(), stream),
                        T * HW * (4 if real else 8), tiles * 3 * 2 * 128 * 128 * HW))
            if real and T >= 2 * B and fd.depth <= 2:
                # the pipe's view of a real ring pipelined over streams: the planes, except the B
                # slots the next batch overwrites, which come from the ring
                out = [r for r in out if r[0] != "time_view"]
                out.append(("time_view_planes", lambda: L.hv_time_view_planes(
                    planes.data_ptr(), ring.data_ptr(), S % T, B, T, W, H, wts.data_ptr(), K, s.image_type, 1.0,
                    s.fft_shift, view.data_ptr(), None, stream), (T - B) * HW * 4 + B * HW * 8 + HW * 4, 0))
        else:
            # tensor flops: the 128 x 128 tiles of the 2T x 2T real Gram matrix on or above its
            # diagonal, three BF16 products each (T <= 32: one packed 128 x 128 product)
            nb = (T + 63) // 64
            flops = 2 * 128 * 128 * HW if 2 * T <= 64 else nb * (nb + 1) // 2 * 3 * 2 * 128 * 128 * HW
            out.append(("pca_covariance", lambda: L.hv_pca_covariance(ring.data_ptr(), T, HW, cov.data_ptr(),
                                                                      cw.data_ptr(), stream), T * HW * 8, flops))
    return out


def ncu_traffic(workload: str, kernel: str):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu capture summary
    (profiles/ncu_traffic.json), used only when the capture was taken on the same kernel sources
    as this build (its digest matches); otherwise None."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None, None
    d = json.loads(p.read_text())
    e = d.get("captures", {}).get(f"{workload}/{kernel}")
    if not e or e.get("kernel_sources_sha256") != kernel_sources_digest():
        return None, e.get("kernel_sources_sha256") if e else None
    return e["dram_bytes"], e.get("command")


def kernel_sources_digest() -> str:
    h = hashlib.sha256()
    for f in sorted((ROOT / "holovibes_gb300" / "csrc").glob("*")):
        if f.suffix in (".cu", ".cuh", ".cpp", ".h"):
            h.update(f.name.encode())
            h.update(f.read_bytes())
    return h.hexdigest()


def roofline(hv, fd, s, dev_batch, peaks, workload=""):
    """Every hot kernel measured alone with CUDA events on its launching stream; the slowest is
    reported against the roof it is closer to (HBM bytes, or tensor flops for the contractions)."""
    import torch

    peak_gbs, peak_tf, peak_src = peaks
    stream = torch.cuda.Stream()
    kernels = steps_for(hv, fd, s, dev_batch, stream.cuda_stream)
    rows = []
    timing = {}
    with torch.cuda.stream(stream):
        for name, fn, alg_bytes, flops in kernels:
            ms, timing[name] = time_kernel(lambda: hv.check(fn(), name), stream)
            rows.append((name, ms, alg_bytes, flops))
    name, ms, alg, flops = max(rows, key=lambda r: r[1])
    gbs = alg / (ms * 1e-3) / 1e9
    tfs = flops / (ms * 1e-3) / 1e12
    hbm_frac, tc_frac = gbs / peak_gbs, tfs / peak_tf
    traffic, cmd = ncu_traffic(workload, name)
    out = {"kernel": name, "peak_source": peak_src, "per_launch_bytes": alg, "per_launch_tensor_flops": flops,
           "ms_per_launch": ms, "traffic": traffic,
           "traffic_source": cmd if traffic else "no ncu capture of these kernel sources (profiles/ncu_traffic.json)",
           "all": {n: {"ms": round(m, 5), "GB/s": round(b / (m * 1e-3) / 1e9, 1),
                       **({"TFLOP/s": round(f / (m * 1e-3) / 1e12, 1)} if f else {}), "timing": timing[n]}
                   for n, m, b, f in rows}}
    if tc_frac > hbm_frac:
        out.update(bound="tensor", achieved=tfs, peak=peak_tf, unit="TFLOP/s", frac=tc_frac, hbm_frac=hbm_frac)
    else:
        out.update(bound="hbm", achieved=gbs, peak=peak_gbs, unit="GB/s", frac=hbm_frac,
                   **({"tensor_frac": tc_frac} if flops else {}))
    return out


def dtype_of(hv, s) -> str:
    parts = ["f32 (convert, FFT passes, views, render)"]
    if s.time_transformation == hv.TIME_PCA:
        # the library's default eigensolver precision: FP32 iterations, the viewed (kept) eigenvectors
        # corrected in FP64 against the FP64 covariance; FP64 sweeps above T = 512
        T = s.time_transformation_size
        top = s.p_start >= T - 16
        if T > 512:
            eig = "f64 Jacobi sweeps"
        elif T > 64 and top:
            eig = "f32 block subspace iteration (32 vectors) + Rayleigh-Ritz, f64 correction of the kept eigenvectors"
        else:
            eig = "f32 Jacobi sweeps, f64 correction of the kept eigenvectors"
        parts.append("bf16x3 on tcgen05 with f32 accumulation, f64 reduce (covariance)")
        parts.append(f"{eig} (eigensolve)")
    elif s.time_transformation in (hv.TIME_STFT, hv.TIME_SSA_STFT):
        parts.append("f64-built weights; bf16x3 tcgen05 contraction for >= 8 bins, else f32 (STFT bins)")
    return ", ".join(parts)


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
    clk = ClockSampler(local, uuid=f"GPU-{torch.cuda.get_device_properties(torch.cuda.current_device()).uuid}")
    clk.start()
    c, fd, s, gen = make_workload(args.workload)
    _, cfg = workload_config(args.workload, world)
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
    # acquisition-style loop: the caller's thread pushes every batch from pinned memory (its H2D
    # copy) as the camera would deliver it, and a consumer thread reads each hologram back to the
    # host (D2H) as soon as it is ready; latency = push start -> hologram on the host. With
    # stride == batch every batch renders one window, so there are as many holograms as batches.
    lat = []
    e2e_steps = args.steps
    pushed = [0.0] * e2e_steps
    if world > 1:
        torch.distributed.barrier()
    errors = []

    def consume():
        try:
            deadline = time.perf_counter() + 60.0
            for k in range(e2e_steps):
                while pipe.output_count() == 0:  # not yet enqueued by the pushing thread
                    if time.perf_counter() > deadline:
                        raise TimeoutError("no hologram within 60 s")
                    time.sleep(0)
                pipe.pull_into(host_out.data_ptr(), hv.MEM_HOST, timeout_us=30_000_000)
                lat.append(time.perf_counter() - pushed[k])
        except Exception as e:  # reported after the join
            errors.append(e)

    consumer = threading.Thread(target=consume)
    t0 = time.perf_counter()
    consumer.start()
    for i in range(e2e_steps):
        pushed[i] = time.perf_counter()
        pipe.enqueue_ptr(host_in[i % nb_unique].data_ptr(), B, hv.MEM_HOST)
    consumer.join()
    if errors:
        raise errors[0]
    pipe.sync()
    t_e2e_ms, e2e_value = replica_throughput((time.perf_counter() - t0) * 1e3, e2e_steps * B, world)
    # latency at a sustainable rate: the same loop with batches pushed at 80% of the e2e rate (a
    # camera delivering frames at that rate), so that no queue builds up in front of the pipe
    period = B / (0.8 * e2e_value / world)
    lat.clear()
    consumer = threading.Thread(target=consume)
    t1 = time.perf_counter()
    consumer.start()
    for i in range(e2e_steps):
        due = t1 + i * period
        while time.perf_counter() < due:
            time.sleep(0)
        pushed[i] = time.perf_counter()
        pipe.enqueue_ptr(host_in[i % nb_unique].data_ptr(), B, hv.MEM_HOST)
    consumer.join()
    if errors:
        raise errors[0]
    pipe.sync()
    lat_ms = np.array(lat) * 1e3 if lat else np.array([float("nan")])
    pipe.close()

    peaks = measured_peaks()
    rl = roofline(hv, fd, s, dev_batches[0], peaks, args.workload) if rank == 0 else None
    serving = None
    if rank == 0 and world == 1 and not args.no_serving and args.workload == DEFAULT_WORKLOAD:
        try:
            serving = serving_comparison(args, "serve512", steps=max(50, min(args.steps, 200)))
        except Exception as e:  # reported in the line; the headline measurement stands
            serving = {"error": f"{type(e).__name__}: {e}"}
    clk.stop()
    cpu = parity = None
    if rank == 0 and not args.no_cpu_baseline:
        O = load_oracle()
        win = window_frames(gen, c["settings"])
        fps, frames, el, nb, first = cpu_oracle_run(c, win, budget_s=args.cpu_budget_s)
        fps32, frames32, el32, nb32, _ = cpu_oracle_run(c, win, budget_s=args.cpu_budget_s / 2, precision="fp32")
        cores = os.cpu_count() or 1
        cpu = {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
               "sample": f"{nb} batches of {B} frames ({frames} frames, {el:.1f} s) through the FP64 numpy oracle "
                         f"after an untimed ring fill, scipy.fft workers={cores} (FFTW unavailable)",
               "fp32": {"value": fps32, "unit": "frames/s", "cores": cores,
                        "sample": f"{nb32} batches ({frames32} frames, {el32:.1f} s), same equations in "
                                  f"complex64 / float32"}}
        # the GPU Pipe's output on the sampled window against the oracle's (the checker's use)
        parity = parity_against(hv, O, fd, s, win, first)
    if rank == 0:
        balg = cfg["B_alg_bytes_per_frame"]
        line = {
            "metric": "input frames/s", "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype_of(hv, s),
            "data": "synthetic (seeded interferograms, generator in holovibes_gb300/synthetic.py)",
            "config": cfg,
            "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": B * frame_bytes,
                    "d2h_bytes_per_step": HW * 2},
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                           "at_input_frames_per_s": 0.8 * e2e_value / world,
                           "window_ms_at_that_rate": 1e3 * s.time_transformation_size / (0.8 * e2e_value / world)},
            "pipeline_hbm_frac": value / world * balg / (peaks[0] * 1e9),
            "gpu_launches": int(launches),
            "roofline": rl,
            "cpu_baseline": cpu,
            "parity": parity,
            "serving": serving,
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


def run_plain_processes(args, nstreams: int, steps: int, workload: str) -> dict:
    """Aggregate input frames/s of one plain pipe per process over all streams (wall clock from
    the first timed push to the last hologram of any process)."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nstreams)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_plain_process, args=(i, workload, steps, args.warmup, barrier, queue))
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


def serving_comparison(args, workload: str, steps: int) -> dict:
    """Served (hv_server: engine thread, shape buckets, CUDA graphs) against plain in-process pipes
    (one hv_pipe per stream, each on its own CUDA stream) and one plain pipe per process, on the
    same streams, from pinned host memory with holograms read back: one client thread pushes one
    batch per stream per step and reads back the holograms of the previous step."""
    import torch

    import holovibes_gb300 as hv

    streams = serve_streams(workload)
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

    def pct(lat):
        a = np.array(lat) * 1e3
        return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99))}

    results = {}
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
    plain_launches = sum(p.kernel_launches() for p in pipes)
    for p in pipes:
        p.close()
    results["plain"] = {"frames_per_s": steps * frames_per_step / el, "latency_ms": pct(lat),
                        "kernel_launches_total": plain_launches}
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
    results["served"] = {"frames_per_s": steps * frames_per_step / el, "latency_ms": pct(lat),
                         "device_latency_ms": {"p50": g1["latency_p50_us"] / 1e3, "p99": g1["latency_p99_us"] / 1e3},
                         "graph_launches": g1["graph_launches"] - g0["graph_launches"],
                         "graph_kernels": g1["graph_kernels"] - g0["graph_kernels"],
                         "eager_cycles": g1["eager_cycles"] - g0["eager_cycles"],
                         "eager_kernels": eager_kernels,
                         "buckets": g1["buckets"], "server_mode": args.server_mode}
    # one plain pipe per process (one Holovibes instance and one compute pipeline per stream)
    results["plain_per_process"] = run_plain_processes(args, len(streams), steps, workload)
    v = results["served"]["frames_per_s"]
    window_ms = min(1e3 * s.time_transformation_size / (v / len(streams)) for (_, s, _) in streams)
    results.update(
        workload=f"{workload}: {SERVE_WORKLOADS[workload]}", streams=len(streams), frames_per_step=frames_per_step,
        steps=steps, served_over_plain=v / results["plain"]["frames_per_s"],
        served_over_plain_per_process=v / results["plain_per_process"]["frames_per_s"],
        shortest_window_ms_at_served_rate=window_ms,
        p99_under_one_window=results["served"]["latency_ms"]["p99"] < window_ms,
        h2d_bytes_per_step=sum(b.shape[1] for (_, _, b) in streams),
        d2h_bytes_per_step=sum(fd.width * fd.height * 2 // s.time_stride * s.batch_size for (fd, s, _) in streams))
    return results


def run_serving(args):
    import torch

    import holovibes_gb300 as hv

    torch.cuda.set_device(0)
    hv.lib()
    clk = ClockSampler(0, uuid=f"GPU-{torch.cuda.get_device_properties(0).uuid}").start()
    steps = max(20, min(args.steps, 400))
    res = serving_comparison(args, args.workload, steps)
    clk.stop()
    v = res["served"]["frames_per_s"]
    line = {
        "metric": "input frames/s", "value": v, "unit": "frames/s", "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * res["frames_per_step"] / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FFT, views), bf16x3/f32 (PCA covariance)",
        "data": "synthetic (seeded interferograms, one seed per stream)",
        "config": {"workload": res["workload"], "streams": res["streams"], "server_mode": args.server_mode,
                   "frames_per_step": res["frames_per_step"], "parallelism": "one GPU, streams overlapped",
                   "l2": "time rings of all streams exceed L2"},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": res["h2d_bytes_per_step"],
                "d2h_bytes_per_step": res["d2h_bytes_per_step"]},
        "serving": res,
        "gpu_launches": int(res["served"]["graph_kernels"] + res["served"]["eager_kernels"]),
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
