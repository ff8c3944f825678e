"""Benchmark: 1080p stabilized frames/s, the chosen form against the plain
FP32 GPU path (and the quality of its output against the plain path's).

Workload (one step = one frame): a 1920x1080 synthetic stream of 120 frames
(seeded Gaussian blobs advected by a smooth flow re-drawn every 30 frames,
processed frames with colour shift and flicker; RGBA8 in and out); the timed
steps cycle through it.  Per frame: load the next frame (RGBA8 -> float,
flow features), compute the forward and backward flow through the
Correlation (81 displacements) and Warp kernels, then the stabilization pass
(five warps, adaptive combination, consistency weights, 2-level pyramid
solve with 75 + 150 iterations) and the RGBA8 output —
VideoStabilizer::doOneStep with its defaults.

Forms (--form, default bf16_ds2_fma): "plain" computes the flow with FP32
correlations at full resolution and solves with kernel_consist_out's exact
arithmetic, as the reference does; "bf16" / "fp16" run the flow estimator's
correlations on the tensor cores; "bf16_ds2" also computes the flow at half
resolution (FLOWDOWNSCALE=2, bilinear upsampling); the "_fma" forms solve
with the FMA form of the same iteration (within 1e-6 of the exact one).
Warps, mask and blend are FP32 in every form.

value : frames/s of the chosen form with every input frame already resident
        in HBM (RGBA8); "plain" holds the plain path's figure, timed the same
        way, and "quality_vs_plain" the PSNR of the chosen form's output
        frames, its flow error and its mask disagreement against the plain
        path's.
e2e   : the chosen form (and, under "plain", the plain path) through the
        public C ABI with host buffers: each step copies the next frame pair
        from pinned host memory and reads the stabilized frame back, inside
        the timed region; the median of three consecutive windows of
        --steps steps (listed under "windows").
Every stabilizer first runs six untimed steps that capture its step graphs
(GRAPH_CAPTURE_STEPS), then the --warmup steps, then the --steps timed ones.
The per-step working set (~0.6 GB) is far larger than L2, so no flush is
needed between steps.  The default line also carries the Correlation's
BF16/FP16 error against the FP64 restatement, the full-resolution BF16 form's
quality, and the 16-stream workload (--no-extras skips them).

--impl reference: the reference's CPU path on the host cores (the CPU
restatement in oracle/, which for the two custom ops is bit-identical to the
reference's correlation.cc / warp.cc; the reference has no CPU code for the
stabilization pass).

Multi-GPU: the path does not shard within a stream (frame t needs the
stabilized frame t-1), so N ranks run N independent replica streams (weak
scaling); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "video-stream-consistency_gb300"
W, H = 1920, 1080
N_FRAMES = 120  # the 1080p stream's length; the timed steps cycle through it
METRIC = "1080p stabilized frames/s, chosen form vs plain GPU at PSNR>=40 dB; HBM GB/s"
# Solver Jacobi step, per pixel: reads O, U, lap(P), A, consWt (5 x 12 B),
# writes O, U (2 x 12 B); the kernel performs vsc_solver_steps_per_launch()
# steps per launch (temporal blocking), so its algorithmic bytes per launch
# are that many steps' worth ("effective" bandwidth can exceed the HBM peak).
SOLVER_BYTES_PER_PX = 84


def import_pkg():
    if "vsc_gb300" in sys.modules:
        return sys.modules["vsc_gb300"]
    spec = importlib.util.spec_from_file_location("vsc_gb300", PKG / "__init__.py",
                                                  submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["vsc_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


GATE_CYCLES = 40_000_000  # ~19 ms at 2.07 GHz


def device_ms(stream, call, n):
    """Device time per call of n back-to-back calls (call(k), k = 0 .. n-1):
    a spin kernel holds the stream while the host enqueues them, so the CUDA
    events bracket device work only, not the API's host-side cost (for
    kernels of a few microseconds that cost would otherwise dominate).
    Returns (ms per call, host enqueue ms); the gate covers the enqueue when
    the latter stays below the gate's ~19 ms."""
    import time

    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        torch.cuda._sleep(GATE_CYCLES)
    t0 = time.perf_counter()
    e0.record(stream)
    for k in range(n):
        call(k)
    e1.record(stream)
    host_ms = (time.perf_counter() - t0) * 1000.0
    e1.synchronize()
    return e0.elapsed_time(e1) / n, host_ms


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (burst copy)"
    return 6800.0, "fallback 6.8 TB/s"


class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled every 20 ms during
    the timed region, through NVML (libnvidia-ml, the library nvidia-smi
    reads), on a background thread.  The device is found by UUID so the
    sample is of the GPU the benchmark runs on whatever CUDA_VISIBLE_DEVICES
    says.  Falls back to `nvidia-smi -lms 20` when NVML cannot be loaded.
    Reading clocks changes nothing on the GPU."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40,
            "hw_power_brake_slowdown": 0x80}
    PERIOD_S = 0.02

    def __init__(self, device_index: int):
        import torch

        self.uuid = None
        try:
            self.uuid = "GPU-" + str(torch.cuda.get_device_properties(device_index).uuid)
        except Exception:  # noqa: BLE001 - older torch without .uuid
            pass
        self.samples = []  # (sm_mhz, max_mhz, reasons bitmask, source)
        self.thread = None
        self.stop_flag = False
        self.proc = None
        self.file = None

    # ---- NVML -----------------------------------------------------------------
    def _nvml(self):
        import ctypes as C

        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = C.c_void_p()
        if self.uuid is None or lib.nvmlDeviceGetHandleByUUID(self.uuid.encode(), C.byref(h)) != 0:
            raise OSError("device not found by UUID")
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        return lib, h, reasons

    def _loop(self, lib, h, reasons_fn):
        import ctypes as C

        clk, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self.stop_flag:
            if (lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and  # NVML_CLOCK_SM
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 and reasons_fn(h, C.byref(rs)) == 0):
                self.samples.append((float(clk.value), float(mx.value), int(rs.value)))
            time.sleep(self.PERIOD_S)

    def start(self):
        import threading

        try:
            lib, h, fn = self._nvml()
        except (OSError, AttributeError):
            return self._start_smi()
        self.stop_flag = False
        self.thread = threading.Thread(target=self._loop, args=(lib, h, fn), daemon=True)
        self.thread.start()
        t0 = time.perf_counter()
        while not self.samples and time.perf_counter() - t0 < 2.0:  # first sample before the region opens
            time.sleep(0.001)

    # ---- nvidia-smi fallback -------------------------------------------------------
    def _start_smi(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.uuid or 0}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.5)
        except (OSError, FileNotFoundError):
            self.proc = None

    def _stop_smi(self):
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                bits = sum(self.BITS[n] for n, v in zip(names, r[5:9]) if v.strip().lower() == "active")
                self.samples.append((float(r[1]), float(r[2]), bits))
            except (ValueError, IndexError):
                continue

    def stop(self):
        source = "nvml"
        if self.thread is not None:
            self.stop_flag = True
            self.thread.join(timeout=5)
        elif self.proc is not None:
            self._stop_smi()
            source = "nvidia-smi"
        else:
            return None
        if not self.samples:
            return None
        sm = [s[0] for s in self.samples]
        reasons = sorted({n for s in self.samples for n, b in self.BITS.items() if s[2] & b})
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": max(s[1] for s in self.samples),
                "samples": len(sm), "period_ms": int(self.PERIOD_S * 1000), "source": source, "reasons": reasons}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(value: float, ws: int, device=None) -> float:
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def make_frames(n: int, seed: int, device: str):
    vsc = import_pkg()
    from vsc_gb300 import synth

    s = synth.SyntheticStream(W, H, seed=seed, device=device)
    return [s.frame(i) for i in range(n)]


# ---------------------------------------------------------------------------
def cpu_baseline_sample(frames, threads: int, n_frames: int = 10):
    """The CPU path timed on a bounded sample: n_frames full 1080p steps."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    O.set_threads(threads)
    n_frames = max(1, min(n_frames, len(frames) - 2))
    orig = [O.rgba_to_float(o) for o, _ in frames[: n_frames + 2]]
    proc = [O.rgba_to_float(p) for _, p in frames[: n_frames + 2]]
    last = proc[2]
    t0 = time.perf_counter()
    for t in range(1, n_frames + 1):
        ff = O.flow_estimate(orig[t], orig[t + 1])
        fb = O.flow_estimate(orig[t + 1], orig[t])
        last, _ = O.stab_pass(orig[t - 1:t + 2], proc[t - 1:t + 2], ff, fb, last)
    dt = time.perf_counter() - t0
    return {"value": n_frames / dt, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{n_frames} consecutive 1920x1080 frames of the same stream: flow (fwd+bwd, the "
                      f"restated Correlation/Warp ops) + stabilization pass + RGBA8 output, OpenMP over "
                      f"{threads} host threads",
            "seconds": dt}


def reference_gpu_timing(frames, reps: int = 5):
    """The reference's own CUDA kernels (compiled in place for sm_103a with
    nvcc's default flags, launched with the reference's geometry and host
    schedule by oracle/ref_gpu) timed on this GPU at 1920x1080: one
    stabilization pass (videostabilizer.cpp:178-247, synchronising after every
    launcher and allocating inside get_consist_out and copyToQImage as the
    reference does) and its Correlation / Warp op calls over the five flow
    levels of one direction.  Host wall time, since the reference schedule
    synchronises inside.  None when no GPU or no cubin is present."""
    try:
        import torch
    except ImportError:
        return None
    if not torch.cuda.is_available():
        return None
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    import ref_gpu as RG

    O.build(ref=False)
    if not RG.available("default"):
        return None
    L = RG.load("default")
    dev = torch.device("cuda", 0)
    f = lambda a: torch.from_numpy(O.rgba_to_float(a)).to(dev)  # noqa: E731
    orig = [f(o) for o, _ in frames[:3]]
    proc = [f(p) for _, p in frames[:3]]
    g = torch.Generator(device=dev).manual_seed(2)
    flows = [torch.randn((H, W, 3), device=dev, generator=g) * 2 for _ in range(2)]
    for fl in flows:
        fl[..., 2] = 0
    last = proc[2].clone()
    e = lambda c=3, w=W, h=H: torch.empty((h, w, c), dtype=torch.float32, device=dev)  # noqa: E731
    ins = [*orig, *proc, flows[0], flows[1], last]
    scratch = [e() for _ in range(11)]
    lvl0 = [e() for _ in range(4)]
    lvl1 = [e(3, W // 2, H // 2) for _ in range(4)]
    host = torch.empty((H, W, 4), dtype=torch.uint8).pin_memory()
    arr = lambda ts: (RG.Img * len(ts))(*[RG.img(t) for t in ts])  # noqa: E731
    a_in, a_s, a_0, a_1 = arr(ins), arr(scratch), arr(lvl0), arr(lvl1)

    def stab():
        RG.check(L, L.rg_stab_pass(a_in, a_s, a_0, a_1, 2, 150, 6800.0, 6800.0, 2.0, 0.15, 0.15, host.data_ptr()))

    stab()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        stab()
    torch.cuda.synchronize()
    stab_ms = 1000 * (time.perf_counter() - t0) / reps
    # the ops of one flow direction over the PWC pyramid of a 1920x1088 frame
    levels = [(480, 272, 32), (240, 136, 64), (120, 68, 96), (60, 34, 128), (30, 17, 196)]
    bufs = []
    for lw, lh, lc in levels:
        a = torch.randn((1, lc, lh, lw), device=dev, generator=g)
        b = torch.randn((1, lc, lh, lw), device=dev, generator=g)
        fl = torch.randn((1, 2, lh, lw), device=dev, generator=g)
        bufs.append((a, b, fl, torch.empty((1, 81, lh, lw), device=dev), torch.empty_like(a), lw, lh, lc))

    def ops(kind):
        for a, b, fl, cv, wo, lw, lh, lc in bufs:
            if kind == "corr":
                RG.check(L, L.rg_correlation(a.data_ptr(), b.data_ptr(), cv.data_ptr(), 1, lc, lh, lw, 4, None))
            else:
                RG.check(L, L.rg_warp_op(b.data_ptr(), fl.data_ptr(), wo.data_ptr(), 1, lc, lh, lw, None))
        torch.cuda.synchronize()

    res = {"stab_pass_ms": stab_ms}
    for kind in ("corr", "warp"):
        ops(kind)
        t0 = time.perf_counter()
        for _ in range(reps):
            ops(kind)
        res[f"{kind}_pyramid_one_direction_ms"] = 1000 * (time.perf_counter() - t0) / reps
    res["source"] = ("the reference's CUDA kernels (flowconsistency.cu, gpuimage.cu, correlation_cuda.cu, "
                     "warp_cuda.cu) compiled in place for sm_103a with nvcc defaults, launched with the "
                     "reference's geometry and host schedule; 1920x1080, host wall time")
    return res


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    O.build(ref=False)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    n = min(args.steps + args.warmup + 2, 120)
    frames = make_frames(n, seed=0, device="cpu")
    orig = [O.rgba_to_float(o) for o, _ in frames]
    proc = [O.rgba_to_float(p) for _, p in frames]
    last = proc[2]

    def step(t):
        nonlocal last
        i = 1 + (t % (n - 2))
        ff = O.flow_estimate(orig[i], orig[i + 1])
        fb = O.flow_estimate(orig[i + 1], orig[i])
        last, rgba = O.stab_pass(orig[i - 1:i + 2], proc[i - 1:i + 2], ff, fb, last)
        return rgba

    for t in range(args.warmup):
        step(t)
    t0 = time.perf_counter()
    for t in range(args.steps):
        step(args.warmup + t)
    dt = time.perf_counter() - t0
    v = args.steps / dt
    ref_gpu = reference_gpu_timing(frames)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "1920x1080 synthetic stream, plain method (flow at full resolution, 2-level "
                               "pyramid, 150 iterations), RGBA8 in/out", "width": W, "height": H},
        "cpu_baseline": {"value": v, "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"each step one 1920x1080 frame on {threads} host threads (OpenMP): the CPU "
                                   "restatement, bit-identical to the reference's CPU Correlation/Warp ops; the "
                                   "reference has no CPU stabilization pass"},
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if ref_gpu:
        line["reference_gpu"] = ref_gpu
    print(json.dumps(line))


def solver_roofline(vsc, dev, stream, iters: int = 144, form: str = "exact"):
    """Times the dominant kernel — the full-resolution solver in the given
    form — with CUDA events on its stream: the time of one Jacobi step from
    an 8-step and an (8 + iters)-step solve of the same size (both whole
    numbers of 8-step rounds), reported per round."""
    import torch

    peak, peak_src = peaks()
    g = torch.Generator(device=dev).manual_seed(1)
    P = torch.rand((H, W, 3), device=dev, generator=g)
    A = torch.rand((H, W, 3), device=dev, generator=g)
    Wt = torch.rand((H, W, 3), device=dev, generator=g) * 2
    O = P.clone()
    wsp = torch.empty(vsc.consist_out_workspace_size(W, H, form=form) // 4, dtype=torch.float32, device=dev)
    T = int(vsc.load().vsc_solver_steps_per_launch())
    torch.cuda.synchronize()
    for _ in range(2):
        vsc.get_consist_out(P, A, Wt, iters, 0.15, 0.15, O, workspace=wsp, stream=stream, form=form)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    vsc.get_consist_out(P, A, Wt, 8, 0.15, 0.15, O, workspace=wsp, stream=stream, form=form)
    ev[1].record(stream)
    ev[2].record(stream)
    vsc.get_consist_out(P, A, Wt, 8 + iters, 0.15, 0.15, O, workspace=wsp, stream=stream, form=form)
    ev[3].record(stream)
    ev[3].synchronize()
    step_ms = (ev[2].elapsed_time(ev[3]) - ev[0].elapsed_time(ev[1])) / iters
    round_ms = step_ms * T
    kname, round_bpp = SOLVER_KERNELS[form]
    alg_bytes = round_bpp * W * H  # each input image read once, O and U written once, per round
    achieved = alg_bytes / (round_ms / 1000.0) / 1e9
    eff = SOLVER_BYTES_PER_PX * W * H * T / (round_ms / 1000.0) / 1e9
    traffic = SOLVER_TRAFFIC_BYTES.get(kname)
    if form == "fma":
        desc = (f"{kname} (one persistent launch per solve: rounds of {T} Jacobi steps on 128x72 tiles of one "
                "channel plane, tiles taken in round order, each waiting for its neighbours' previous round; "
                "1920x1080)")
    else:
        desc = f"{kname} (one launch per round of {T} Jacobi steps on 64x48 tiles of three channels; 1920x1080)"
    line = {"bound": "hbm", "kernel": desc,
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "algorithmic_bytes_per_round": alg_bytes,
            "algorithmic_bytes_rule": f"{round_bpp} B/px per {T}-step round: each input image read once and O, U "
                                      "written once (a round's compulsory bytes)",
            "effective_gbs": eff, "frac_effective": eff / peak,
            "effective_rule": f"{SOLVER_BYTES_PER_PX} B/px per Jacobi step x {T} steps per round (the reference's "
                              "one launch per step would move these bytes)",
            "steps_per_round": T, "round_ms": round_ms, "ms_per_jacobi_step": step_ms,
            "timing_rule": f"CUDA events on the solver's stream: (time of an ({T} + {iters})-step solve - time of "
                           f"a {T}-step solve) / {iters} per step, x {T} per round",
            "peak_source": peak_src}
    if traffic:
        line["frac_dram"] = traffic / (round_ms / 1000.0) / 1e9 / peak
        line["traffic_source"] = SOLVER_TRAFFIC_SOURCE[kname]
    line["pipe_counters"] = SOLVER_PIPE.get(kname)
    return line


MULTI_STREAMS = [(640, 360)] * 4 + [(1280, 720)] * 6 + [(1920, 1080)] * 4 + [(3840, 2160)] * 2


def multistream_forms(form):
    """Per-stream (flow_downscale, corr_dtype) of a form on the 16-stream
    workload; a form with the learned upsampler uses it on the 1920x1080 and
    3840x2160 streams only (flow at half size there, full size below)."""
    kw, _ = FORMS[form]
    out = []
    for w, h in MULTI_STREAMS:
        if kw.get("upsampler"):
            out.append((2 if h >= 1080 else 1, kw["corr_dtype"]))
        else:
            out.append((kw["flow_downscale"], kw["corr_dtype"]))
    return out


def multistream_measure(vsc, dev, form: str, steps: int, warmup: int, grouped: bool, n_unique: int = 4):
    """16 concurrent synthetic streams of mixed resolution (4x 640x360, 6x
    1280x720, 4x 1920x1080, 2x 3840x2160; 31,334,400 px per step) stabilized
    in lockstep, one CUDA graph launch per frame step (vsc_multistream),
    the solves of all 16 grouped: per pyramid level, each launch of the
    persistent solver kernel (8 Jacobi steps) walks the tiles of all 16
    images (grouped=False: each stream's solve on its own CUDA stream).  A
    step is one frame of every stream; each stream cycles through n_unique
    generated frames (the work per step does not depend on which).  Value:
    stream-frames/s and Mpx/s, CUDA events on the multistream's stream."""
    import torch

    from vsc_gb300 import synth

    kw, form_desc = FORMS[form]
    forms = multistream_forms(form)
    stream = torch.cuda.Stream(device=dev)
    frames = []
    for i, (w, h) in enumerate(MULTI_STREAMS):
        s_ = synth.SyntheticStream(w, h, seed=100 + i, device=str(dev))
        frames.append([tuple(torch.from_numpy(a).to(dev) for a in s_.frame(t)) for t in range(n_unique)])
    torch.cuda.synchronize()
    ms = vsc.MultiStream(MULTI_STREAMS, flow_downscale=[f[0] for f in forms], corr_dtype=[f[1] for f in forms],
                         stream=stream)
    ms.set_fused(grouped)
    if kw.get("solver_form", "exact") != "exact":
        ms.set_solver_form(kw["solver_form"])
    up = None
    if kw.get("upsampler"):
        up = vsc.Upsampler(kw["upsampler"])
        ms.set_upsampler(up)
    outs = [torch.empty((h, w, 4), dtype=torch.uint8, device=dev) for w, h in MULTI_STREAMS]
    state = {"t": 0}

    def load():
        t = state["t"] % n_unique
        ms.load_frames([f[t][0] for f in frames], [f[t][1] for f in frames])
        state["t"] += 1

    for _ in range(3):
        load()

    def step():
        with torch.cuda.stream(stream):
            ms.step(outs)
        load()

    for _ in range(GRAPH_CAPTURE_STEPS + warmup):
        step()
    stream.synchronize()
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    px = sum(w * h for w, h in MULTI_STREAMS)
    is_grouped = ms.fused
    res = {
        "value": len(MULTI_STREAMS) * steps / (ms_total / 1000), "unit": "stream-frames/s",
        "mpx_per_s": px * steps / (ms_total / 1000) / 1e6, "steps": steps, "warmup": warmup,
        "ms_per_step": ms_total / steps,
        "config": {"workload": f"16 streams: 4x 640x360, 6x 1280x720, 4x 1920x1080, 2x 3840x2160; form "
                               f"'{form}': {form_desc}" + ("; learned upsampler on the 1080p and 4K streams only"
                                                         if kw.get("upsampler") else ""),
                   "px_per_step": px, "form": form,
                   "per_stream": [{"size": [w, h], "flow_downscale": d, "corr_dtype": c}
                                  for (w, h), (d, c) in zip(MULTI_STREAMS, forms)],
                   "solves": "grouped: one persistent-kernel launch per 8 Jacobi steps covers all 16 images"
                             if is_grouped else "per stream, each on its own CUDA stream"},
        "grouped_solves": is_grouped, "gpu_launches_per_step": ms.last_launches, "clocks": clk,
    }
    ms.close()
    if up is not None:
        up.close()
    return res


def run_multistream(args):
    """--workload multistream: the 16-stream workload as its own line (see
    multistream_measure); default form BF16 correlations, the learned
    upsampler on the 1080p and 4K streams, the solver in its FMA form."""
    import torch

    vsc = import_pkg()
    vsc.build()
    vsc.load()
    dev = torch.device("cuda", 0)
    form = args.form or DEFAULT_MS_FORM
    res = multistream_measure(vsc, dev, form, args.steps, args.warmup, args.ms_grouped == "on", n_unique=8)
    kw = FORMS[form][0]
    line = {"metric": "multi-stream stabilized stream-frames/s (16 mixed-resolution streams, one graph launch per "
                      "step)", "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": kw["corr_dtype"], "data": "synthetic", **res,
            "gpu_launches": res["gpu_launches_per_step"] * args.steps}
    print(json.dumps(line))


PWC_LEVELS_1080P = [(480, 272, 32), (240, 136, 64), (120, 68, 96), (60, 34, 128), (30, 17, 196)]


def run_corr_only(args):
    """--kernel corr: the Correlation op over the five PWC levels of a
    1920x1088 frame (one direction), FP32 CUDA-core kernel against the BF16 /
    FP16 tensor-core one (the latter including its per-level scaling and
    16-bit conversion launches); CUDA events on the launching stream.
    Algorithmic bytes of the FP32 contract: 4 (2 C H W + 81 H W)."""
    import torch

    vsc = import_pkg()
    vsc.build()
    vsc.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    g = torch.Generator(device=dev).manual_seed(3)
    peak, peak_src = peaks()
    res = {}
    for lw, lh, lc in PWC_LEVELS_1080P:
        f1 = torch.randn((1, lc, lh, lw), device=dev, generator=g)
        f2 = torch.randn((1, lc, lh, lw), device=dev, generator=g)
        out = torch.empty((1, 9, 9, lh, lw), device=dev)
        ws = torch.empty(vsc.load().vsc_correlation_lowp_workspace_size(1, lc, lh, lw), dtype=torch.uint8,
                         device=dev)
        calls = {"f32": lambda: vsc.correlation(f1, f2, 4, out=out, stream=stream),
                 "bf16": lambda: vsc.correlation_lowp(f1, f2, 4, "bf16", out=out, workspace=ws, stream=stream),
                 "fp16": lambda: vsc.correlation_lowp(f1, f2, 4, "fp16", out=out, workspace=ws, stream=stream)}
        alg = 4 * (2 * lc * lh * lw + 81 * lh * lw)
        lev = {"shape": [lc, lh, lw], "algorithmic_bytes": alg}
        for name, fn in calls.items():
            for _ in range(max(args.warmup, 3)):
                fn()
            ms, host_ms = device_ms(stream, lambda k: fn(), args.steps)
            lev[name] = {"ms": ms, "gbs": alg / (ms / 1000) / 1e9, "host_enqueue_ms": host_ms}
        res[f"{lw}x{lh}"] = lev
    tot = {k: sum(v[k]["ms"] for v in res.values()) for k in ("f32", "bf16", "fp16")}
    print(json.dumps({"kernel": "correlation, PWC pyramid of one 1920x1088 direction", "levels": res,
                      "total_ms": tot, "peak_gbs": peak, "peak_source": peak_src}))


def run_front_only(args):
    """--kernel front: the fused front pass (five warps + adaptive combination
    + consistency weights in one pass) at 1920x1080, CUDA events on its
    stream, in both forms: vsc_stab_front on float frames (124 B/px: two
    3-channel flows 24 B, five warped sources 60 B, the current original and
    processed frames 24 B, two outputs 24 B; the stabilizer's form) and
    vsc_stab_front_rgba on RGBA8 frames (84 B/px: flows 24 B, four warped
    RGBA8 sources 16 B, the warped last stabilized frame 12 B, the current
    RGBA8 frames 8 B, outputs 24 B).  The inputs exceed L2 (258 / 174 MB),
    so no flush is needed."""
    import torch

    vsc = import_pkg()
    vsc.build()
    vsc.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    g = torch.Generator(device=dev).manual_seed(5)
    rgba = [torch.randint(0, 256, (H, W, 4), device=dev, generator=g, dtype=torch.uint8) for _ in range(6)]
    with torch.cuda.stream(stream):
        ims = [vsc.char_to_float_image(r, stream=stream) for r in rgba]
    stream.synchronize()
    ims.append(torch.rand((H, W, 3), device=dev, generator=g))
    yy, xx = torch.meshgrid(torch.arange(H, device=dev), torch.arange(W, device=dev), indexing="ij")
    ff = torch.stack([3 * torch.sin(xx / 97.0), 2 * torch.cos(yy / 83.0), torch.zeros_like(xx, dtype=torch.float32)],
                     -1).float().contiguous()
    fb = (-ff).contiguous()
    apr, wt = torch.empty_like(ims[0]), torch.empty_like(ims[0])
    peak, peak_src = peaks()
    forms = {
        "fused_front_kernel (vsc_stab_front, float frames)": (124, lambda: vsc.stab_front(
            ims[0:3], ims[3:6], ims[6], ff, fb, 6800.0, 6800.0, 2.0, out=(apr, wt), stream=stream)),
        # |gamma| > 1e30 selects the general form (64-bit taps, the full expf_cw)
        "fused_front_kernel general form (vsc_stab_front, gamma 2e30)": (124, lambda: vsc.stab_front(
            ims[0:3], ims[3:6], ims[6], ff, fb, 6800.0, 6800.0, 2e30, out=(apr, wt), stream=stream)),
        "fused_front_rgba_kernel (vsc_stab_front_rgba, RGBA8 frames)": (84, lambda: (
            vsc.stab_front_rgba(rgba[0:3], rgba[3:6], ims[6], ff, fb, 6800.0, 6800.0, 2.0, out=(apr, wt),
                                stream=stream))),
    }
    res = []
    for name, (bpp, call) in forms.items():
        for _ in range(max(args.warmup, 3)):
            call()
        ms, host_ms = device_ms(stream, lambda k: call(), args.steps)
        alg = bpp * W * H
        res.append({"kernel": name + " 1920x1080", "ms": ms, "bytes_per_px": bpp,
                    "achieved_gbs": alg / (ms / 1000) / 1e9, "frac": alg / (ms / 1000) / 1e9 / peak,
                    "algorithmic_bytes": alg, "host_enqueue_ms": host_ms})
    print(json.dumps({"forms": res, "peak_gbs": peak, "peak_source": peak_src}))


def run_solver_only(args):
    """--kernel solver: only the 1920x1080 solver (for profiler captures)."""
    import torch

    vsc = import_pkg()
    vsc.build()
    vsc.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    for form in ("exact", "fma"):
        rows = vsc.solver_autotune(W, H, stream=stream, form=form)
        print(json.dumps({"form": form, "tile_rows": rows,
                          **solver_roofline(vsc, dev, stream, iters=args.steps * 8, form=form)}))


def run_warpblend(args):
    """--kernel warpblend: the warp, mask and blend kernels one by one at
    1920x1080 (float HWC3 images, 3-channel flows), each against its
    algorithmic bytes (every input tensor read once, every output written
    once, in the layout the kernel uses): kernel_warp 36 B/px (source 12,
    flow 12, out 12), adap_comb 108 B/px (seven images in, two out),
    consist_wt 36 B/px, the fused front pass 124 B/px, bilinear 12 B per
    input and output pixel, the Warp op 4 (2 C + 2) B per pixel (a batch of
    8 at the 480x272, 32-channel PWC level), RGBA8 <-> float 16 B/px.
    K calls back to back between two CUDA events on the kernels' stream,
    enqueued while a spin kernel holds the stream (device_ms), each call on
    the next of four input sets, so that consecutive calls never find their
    inputs in L2 (every case's four sets exceed 129 MB)."""
    import torch

    vsc = import_pkg()
    vsc.build()
    vsc.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    g = torch.Generator(device=dev).manual_seed(6)
    nsets = 4
    yy, xx = torch.meshgrid(torch.arange(H, device=dev), torch.arange(W, device=dev), indexing="ij")

    def img(h=H, w=W):
        return torch.rand((h, w, 3), device=dev, generator=g)

    def flow(k):
        return torch.stack([3 * torch.sin(xx / (97.0 + k)), 2 * torch.cos(yy / (83.0 + k)),
                            torch.zeros_like(xx, dtype=torch.float32)], -1).float().contiguous()

    def smooth_flow(n, w, h, k):  # N x 2 x h x w, |v| <= 3 px, smooth like an upsampled estimate
        yy2, xx2 = torch.meshgrid(torch.arange(h, device=dev), torch.arange(w, device=dev), indexing="ij")
        f = torch.stack([3 * torch.sin(xx2 / (31.0 + k)), 3 * torch.cos(yy2 / (23.0 + k))], 0).float()
        return f.unsqueeze(0).repeat(n, 1, 1, 1).contiguous()

    sets = []
    for k in range(nsets):
        ims = [img() for _ in range(7)]
        ff = flow(k)
        outs = [torch.empty_like(ims[0]) for _ in range(2)]
        sets.append({
            "ims": ims, "ff": ff, "fb": (-ff).contiguous(), "outs": outs, "small": img(H // 2, W // 2),
            "rgba": torch.randint(0, 256, (H, W, 4), device=dev, generator=g, dtype=torch.uint8),
            "x32": torch.randn((8, 32, 272, 480), device=dev, generator=g),
            "fl32": smooth_flow(8, 480, 272, k),
            "x3": ims[0].permute(2, 0, 1).unsqueeze(0).contiguous(),
            "fl3": ff[..., :2].permute(2, 0, 1).unsqueeze(0).contiguous(),
        })
    torch.cuda.synchronize()
    peak, peak_src = peaks()
    px, spx = W * H, (W // 2) * (H // 2)
    cases = [
        ("stab_warp_kernel (get_warp_result)", 36 * px, lambda d: vsc.get_warp_result(d["ims"][0], d["ff"], stream=stream)),
        ("adap_comb_kernel (get_adap_comb)", 108 * px, lambda d: vsc.get_adap_comb(*d["ims"][0:7], 6800.0, stream=stream)),
        ("consist_wt_kernel (get_consist_wt)", 36 * px,
         lambda d: vsc.get_consist_wt(d["ims"][0], d["ims"][1], 6800.0, 2.0, stream=stream)),
        ("fused_front_kernel (stab_front)", 124 * px, lambda d: vsc.stab_front(
            d["ims"][0:3], d["ims"][3:6], d["ims"][6], d["ff"], d["fb"], 6800.0, 6800.0, 2.0, out=d["outs"],
            stream=stream)),
        ("bilinear 1920x1080 -> 960x540", 12 * (px + spx), lambda d: vsc.get_bilinear(d["ims"][0], W // 2, H // 2,
                                                                                      stream=stream)),
        ("bilinear 960x540 -> 1920x1080", 12 * (px + spx), lambda d: vsc.get_bilinear(d["small"], W, H, stream=stream)),
        ("warp_op_kernel (Warp op, C=3, 1920x1080)", 4 * (2 * 3 + 2) * px,
         lambda d: vsc.warp(d["x3"], d["fl3"], stream=stream)),
        ("warp_op_kernel (Warp op, 8 x C=32, 480x272)", 8 * 4 * (2 * 32 + 2) * 480 * 272,
         lambda d: vsc.warp(d["x32"], d["fl32"], stream=stream)),
        ("rgba_to_float (char_to_float_image)", 16 * px, lambda d: vsc.char_to_float_image(d["rgba"], stream=stream)),
        ("float_to_rgba (float_to_char_image)", 16 * px, lambda d: vsc.float_to_char_image(d["ims"][0], stream=stream)),
    ]
    res = []
    for name, alg, call in cases:
        for k in range(max(args.warmup, 3)):
            call(sets[k % nsets])
        ms, host_ms = device_ms(stream, lambda k: call(sets[k % nsets]), args.steps)
        res.append({"kernel": name, "ms": ms, "algorithmic_bytes": alg, "achieved_gbs": alg / (ms / 1000) / 1e9,
                    "frac": alg / (ms / 1000) / 1e9 / peak, "host_enqueue_ms": host_ms})
    print(json.dumps({"kernels": res, "peak_gbs": peak, "peak_source": peak_src}))


def run_upsampler_only(args):
    """--kernel upsampler: the learned 2x upsampler's inference on one
    1920x1080 flow (vsc_upsampler_apply: input preparation, FP16 conversion,
    the four tensor-core convolutions with the fallback test fused into the
    last), CUDA events on its stream.  Algorithmic bytes per pixel: prepare
    12 in (frame; the coarse flow is a quarter of the pixels, 3 B) + 12 out,
    conversion 12 in + 16 out, layer 1 16 in + 64 out, layers 2-3 64 in + 64
    out each, layer 4 64 + 12 in + 12 out: 423 B/px.  Tensor work: 2 x 9 x
    (16 x 32 + 32 x 32 + 32 x 32 + 32 x 16) FLOP per pixel as issued
    (channels padded to the MMA shape; 39,744 FLOP/px useful)."""
    import torch

    vsc = import_pkg()
    vsc.build()
    vsc.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    g = torch.Generator(device=dev).manual_seed(9)
    coarse = (torch.randn((H // 2, W // 2, 3), device=dev, generator=g) * 2).contiguous()
    frame = torch.rand((H, W, 3), device=dev, generator=g)
    up = vsc.Upsampler("default")
    out = torch.empty_like(frame)
    for _ in range(max(args.warmup, 3)):
        vsc.load().vsc_upsampler_apply(up._h, *(vsc.C.byref(vsc.image(t)) for t in (coarse, frame, out)),
                                      vsc._stream(stream))
    ms, _ = device_ms(stream, lambda k: vsc._check(vsc.load().vsc_upsampler_apply(
        up._h, *(vsc.C.byref(vsc.image(t)) for t in (coarse, frame, out)), vsc._stream(stream))), args.steps)
    peak, peak_src = peaks()
    alg = 423 * W * H
    flops = 2 * 9 * (16 * 32 + 32 * 32 + 32 * 32 + 32 * 16) * W * H
    print(json.dumps({"kernel": "learned upsampler inference (vsc_upsampler_apply) 1920x1080", "ms": ms,
                      "algorithmic_bytes": alg, "achieved_gbs": alg / (ms / 1000) / 1e9,
                      "frac_hbm": alg / (ms / 1000) / 1e9 / peak, "tensor_tflops_issued": flops / (ms / 1000) / 1e12,
                      "peak_gbs": peak, "peak_source": peak_src}))
    up.close()


# ---------------------------------------------------------------------------
# Forms of the per-frame path.  "plain" is the method as the reference runs
# it (FP32 correlations, flow at full resolution); the others change only the
# flow estimator's arithmetic or resolution, never the warps, mask and blend.
FORMS = {
    "plain": ({"corr_dtype": "f32", "flow_downscale": 1},
              "plain FP32 path: flow at full resolution (Correlation md=4 + Warp, FP32)"),
    "bf16": ({"corr_dtype": "bf16", "flow_downscale": 1},
             "flow at full resolution with the Correlations on the tensor cores (BF16 operands, FP32 "
             "accumulation); warps, mask and blend FP32"),
    "fp16": ({"corr_dtype": "fp16", "flow_downscale": 1},
             "flow at full resolution with the Correlations on the tensor cores (FP16 operands with a per-level "
             "scale, FP32 accumulation); warps, mask and blend FP32"),
    "bf16_ds2": ({"corr_dtype": "bf16", "flow_downscale": 2},
                 "FLOWDOWNSCALE=2 (flow at 960x540, bilinear upsampling) with BF16 tensor-core Correlations"),
    "bf16_ds2_learned": ({"corr_dtype": "bf16", "flow_downscale": 2, "upsampler": "default"},
                         "FLOWDOWNSCALE=2 with BF16 tensor-core Correlations and the learned 2x flow upsampler "
                         "(weights shipped with the package; bilinear fallback where its residual exceeds 0.5 px)"),
    "plain_fma": ({"corr_dtype": "f32", "flow_downscale": 1, "solver_form": "fma"},
                  "plain flow (FP32 correlations at full resolution) with the solver in its FMA form"),
    "bf16_ds2_fma": ({"corr_dtype": "bf16", "flow_downscale": 2, "solver_form": "fma"},
                     "FLOWDOWNSCALE=2 (flow at 960x540, bilinear upsampling) with BF16 tensor-core Correlations "
                     "and the solver in its FMA form (fused multiply-adds around per-solve constants; within 1e-6 "
                     "of the exact form)"),
    "bf16_ds2_learned_fma": ({"corr_dtype": "bf16", "flow_downscale": 2, "upsampler": "default",
                              "solver_form": "fma"},
                             "FLOWDOWNSCALE=2 with BF16 tensor-core Correlations, the learned 2x flow upsampler and "
                             "the solver in its FMA form"),
}
DEFAULT_FORM = "bf16_ds2_fma"
DEFAULT_MS_FORM = "bf16_ds2_learned_fma"
# Untimed steps run right after a stabilizer is made: its step CUDA graph is
# captured once per window position (3) and feedback buffer (2), so six steps
# keep every capture out of the warm-up and timed steps.
GRAPH_CAPTURE_STEPS = 6


def make_stabilizer(vsc, kw, stream):
    """A Stabilizer for a form; the learned upsampler, when the form has one,
    is attached (and kept alive by the stabilizer)."""
    args = {k: v for k, v in kw.items() if k != "upsampler"}
    st = vsc.Stabilizer(W, H, stream=stream, **args)
    if kw.get("upsampler"):
        st.set_upsampler(vsc.Upsampler(kw["upsampler"]))
    return st


def time_form(vsc, kw, dev_frames, stream, steps, warmup, ws, dev, clocks=None):
    """K device-resident steps of one form, CUDA events on the stabilizer's
    stream; returns (ms over ranks, launches per step, stabilizer)."""
    import torch

    n_frames = len(dev_frames)
    out_dev = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    st = make_stabilizer(vsc, kw, stream)
    for i in range(3):
        st.load_frame(*dev_frames[i])
    state = {"nxt": 3, "launches": 0}

    def step():
        st.step(out_dev)
        n = st.last_launches
        st.load_frame(*dev_frames[state["nxt"] % n_frames])
        state["launches"] = n + st.last_launches
        state["nxt"] += 1

    with torch.cuda.stream(stream):
        for _ in range(GRAPH_CAPTURE_STEPS + warmup):
            step()
    stream.synchronize()
    if clocks:
        clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    ms = reduce_max(e0.elapsed_time(e1), ws, dev)
    st.step_fn = step
    return ms, state["launches"], st


def e2e_form(vsc, kw, pinned, stream, steps, warmup, ws, dev):
    """The same metric through the public API with pinned host frames: each
    step uploads the next frame pair (vsc_stabilizer_load_frame: a copy on
    the stabilizer's copy stream, overlapping the step before it) and reads
    the stabilized frame back into pinned host memory (VSC_OUT_HOST_ASYNC:
    the copy is enqueued behind the step).  The host waits for step k's
    result before it enqueues step k + 2, so every result is on the host
    inside the timed region and the host runs at most two steps ahead.
    Three consecutive windows of `steps` steps, each opened on an idle
    stream and closed when its last result is on the host; the value is
    their median (all three are listed): a host thread that is descheduled
    for a few milliseconds stalls the two-step pipeline, and on a shared
    host that happens in some windows of ~30 ms and not in others."""
    import torch

    n_frames = len(pinned)
    outs = [torch.empty((H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(2)]
    st = make_stabilizer(vsc, kw, stream)
    for i in range(3):
        st.load_frame(pinned[i][0].numpy(), pinned[i][1].numpy())
    state = {"nxt": 3, "k": 0, "checksum": 0, "wait_s": 0.0, "enq_s": []}

    def step():
        k = state["k"]
        if k >= 2:
            t = time.perf_counter()
            st.wait_output(1)  # step k - 2's frame is on the host
            state["wait_s"] += time.perf_counter() - t
            state["checksum"] += int(outs[k % 2][0, 0, 0])
        t = time.perf_counter()
        st.step(outs[k % 2], asynchronous=True)
        o, p = pinned[state["nxt"] % n_frames]
        st.load_frame(o.numpy(), p.numpy())
        state["enq_s"].append(time.perf_counter() - t)
        state["nxt"] += 1
        state["k"] += 1

    for _ in range(GRAPH_CAPTURE_STEPS + warmup):
        step()
    windows, host = [], []
    for _ in range(3):
        st.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        state["wait_s"], state["enq_s"] = 0.0, []
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        st.synchronize()  # the last two results
        t = time.perf_counter() - t0
        windows.append(ws * steps / reduce_max(t, ws, dev))
        # where the host's time went: blocked on results (GPU-bound) or
        # enqueueing a step and its upload (host-bound when it nears a step)
        host.append({"wait_frac": round(state["wait_s"] / t, 3),
                     "enqueue_us_median": round(1e6 * statistics.median(state["enq_s"]), 1),
                     "enqueue_us_max": round(1e6 * max(state["enq_s"]), 1)})
    st.close()
    # the copy bandwidths of this run's pinned buffers (a slow host link shows
    # here, not in the kernels): one frame pair up, one frame down, CUDA events
    pair = torch.empty((2, H, W, 4), dtype=torch.uint8, device=dev)
    src = torch.stack([pinned[0][0], pinned[0][1]]).pin_memory()
    gbs = {"h2d": [], "d2h": []}
    with torch.cuda.stream(stream):
        for _ in range(5):
            for kind, dst_t, src_t in (("h2d", pair, src), ("d2h", outs[0], pair[0])):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                dst_t.copy_(src_t, non_blocking=True)
                e1.record(stream)
                e1.synchronize()
                gbs[kind].append(dst_t.numel() / (e0.elapsed_time(e1) * 1e6))
    return {"value": statistics.median(windows), "unit": "frames/s", "windows": windows, "host": host,
            "copy_gbs": {k: round(statistics.median(v), 1) for k, v in gbs.items()},
            "h2d_bytes_per_step": 2 * W * H * 4, "d2h_bytes_per_step": W * H * 4,
            "pipelining": "results read back asynchronously into pinned memory on the stabilizer's download "
                          "stream, the host at most two steps ahead; uploads on its copy stream"}


def quality_vs_plain(vsc, kw, dev_frames, stream, n_steps: int = 12):
    """The form against the plain path on the same frames, step by step:
    PSNR of the stabilized RGB output; the forward flow's error (px, max-abs
    and RMS over both components; the flow estimator has no FP64
    restatement, so the plain path's FP32 flow is the reference); and the
    consistency mask's disagreement rate — the fraction of consWt values
    whose zero / non-zero decision (the 1e-3 clamp, flowconsistency.cu:
    181-186) differs from the plain path's."""
    import torch

    sts = [make_stabilizer(vsc, FORMS["plain"][0], stream), make_stabilizer(vsc, kw, stream)]
    for st in sts:
        for i in range(3):
            st.load_frame(*dev_frames[i])
    psnr, fmax, fsq, dis = [], 0.0, [], []
    for t in range(n_steps):
        outs, flows, wts = [], [], []
        for st in sts:
            with torch.cuda.stream(stream):
                outs.append(st.step()[..., :3].float())
                flows.append(st.buffer(1)[..., :2].clone())
                wts.append(st.buffer(4).clone())
        stream.synchronize()
        mse = float(torch.mean((outs[0] - outs[1]) ** 2)) / 255.0 ** 2
        psnr.append(99.0 if mse == 0 else 10 * math.log10(1.0 / mse))
        d = (flows[1] - flows[0]).abs()
        fmax = max(fmax, float(d.max()))
        fsq.append(float(torch.mean(d.double() ** 2)))
        dis.append(float(torch.mean(((wts[0] == 0) != (wts[1] == 0)).double())))
        for st in sts:
            st.load_frame(*dev_frames[(t + 3) % len(dev_frames)])
    for st in sts:
        st.close()
    return {"psnr_min_db": min(psnr), "psnr_mean_db": statistics.mean(psnr), "frames": n_steps,
            "flow_err_vs_plain_px": {"max_abs": fmax, "rms": math.sqrt(statistics.mean(fsq))},
            "mask_disagreement_vs_plain": statistics.mean(dis),
            "note": "PSNR 99 = identical frames; flow error and mask disagreement against the plain FP32 path"}


def correlation_precision(vsc, dev, seed: int = 7):
    """The Correlation op's error in BF16 and FP16 (tensor cores, FP32
    accumulation) and in FP32 (CUDA cores) against the FP64 restatement, on
    N(0, 1) feature pyramids of a 1920x1088 frame pair (the five PWC levels,
    md 4): max-abs and RMS per level, and the error relative to the largest
    |value| of the level."""
    import numpy as np
    import torch

    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    from vsc_gb300 import synth

    O.build(ref=False)
    O.set_threads(os.cpu_count() or 1)
    out = {}
    for (f1, f2), (lw, lh, lc) in zip(synth.feature_pyramid(W, H, seed), PWC_LEVELS_1080P):
        ref = O.correlation(f1.astype(np.float64), f2.astype(np.float64), 4)
        d1, d2 = torch.from_numpy(f1).to(dev), torch.from_numpy(f2).to(dev)
        lev = {"shape": [lc, lh, lw], "max_abs_value": float(np.abs(ref).max())}
        for name, call in (("f32", lambda: vsc.correlation(d1, d2, 4)),
                           ("bf16", lambda: vsc.correlation_lowp(d1, d2, 4, "bf16")),
                           ("fp16", lambda: vsc.correlation_lowp(d1, d2, 4, "fp16"))):
            e = call().cpu().numpy().astype(np.float64) - ref
            lev[name] = {"max_abs": float(np.abs(e).max()), "rms": float(np.sqrt(np.mean(e * e))),
                         "max_rel_to_level_max": float(np.abs(e).max() / lev["max_abs_value"])}
        out[f"{lw}x{lh}"] = lev
    return {"levels": out, "reference": "FP64 restatement of correlation.cc (oracle/), N(0,1) features"}


def run_gpu(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    vsc = import_pkg()
    vsc.build()
    vsc.load()

    n_frames = N_FRAMES
    frames = make_frames(n_frames, seed=rank, device=str(dev))
    stream = torch.cuda.Stream(device=dev)
    dev_frames = [(torch.from_numpy(o).to(dev), torch.from_numpy(p).to(dev)) for o, p in frames]
    torch.cuda.synchronize()
    form = args.form or DEFAULT_FORM
    kw, form_desc = FORMS[form]

    # ---- device-resident: the chosen form, then plain; clocks sampled from the
    # first timed region to the last end-to-end one ------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    ms_max, launches_per_step, st = time_form(vsc, kw, dev_frames, stream, args.steps, args.warmup, ws, dev)
    value = ws * args.steps / (ms_max / 1000.0)
    plain = None
    if form != "plain":
        pms, pl, pst = time_form(vsc, FORMS["plain"][0], dev_frames, stream, args.steps, args.warmup, ws, dev)
        pst.close()
        plain = {"value": ws * args.steps / (pms / 1000.0), "unit": "frames/s", "ms_per_step": pms / args.steps,
                 "gpu_launches_per_step": pl}

    # ---- end to end through the public API with pinned host buffers ------------
    pinned = [(torch.from_numpy(o).pin_memory(), torch.from_numpy(p).pin_memory()) for o, p in frames]
    e2e = e2e_form(vsc, kw, pinned, stream, args.steps, args.warmup, ws, dev)
    if plain:
        plain["e2e"] = e2e_form(vsc, FORMS["plain"][0], pinned, stream, args.steps, args.warmup, ws, dev)
    clk = clocks.stop()

    # ---- per-stage device time (separate pass; stage events synchronise) -------
    st.enable_timing(True)
    stages = []
    for _ in range(5):
        st.step_fn()
        stages.append(st.stage_ms())
    st.enable_timing(False)
    stages_ms = {k: statistics.median(d[k] for d in stages) for k in stages[0]}
    st.close()

    roofline = solver_roofline(vsc, dev, stream, form=kw.get("solver_form", "exact"))
    line = {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if kw["corr_dtype"] == "f32" else f"f32 ({kw['corr_dtype']} correlation)",
        "data": "synthetic",
        "config": {"workload": f"1920x1080 synthetic stream of {n_frames} frames (flow re-drawn every 30), form "
                               f"'{form}': {form_desc}; 2-level pyramid, 75+150 solver iterations, RGBA8 in/out",
                   "form": form, "width": W, "height": H, "frames_generated": n_frames,
                   "graph_capture_steps": GRAPH_CAPTURE_STEPS,
                   "l2": "per-step working set ~0.6 GB > 129 MB L2; no flush",
                   "parallelism": f"replicas x{ws}"},
        "e2e": e2e, "gpu_launches": launches_per_step * args.steps, "roofline": roofline, "clocks": clk,
        "stages_ms": stages_ms,
    }
    if plain:
        plain["roofline"] = solver_roofline(vsc, dev, stream, form="exact")
        line["plain"] = plain
        line["speedup_vs_plain"] = value / plain["value"]
        line["e2e_speedup_vs_plain"] = e2e["value"] / plain["e2e"]["value"]
        line["quality_vs_plain"] = quality_vs_plain(vsc, kw, dev_frames, stream)
    if rank == 0 and ws == 1 and not args.no_extras:
        line["precision_bf16_fullres"] = quality_vs_plain(vsc, FORMS["bf16"][0], dev_frames, stream)
        line["correlation_precision"] = correlation_precision(vsc, dev)
        line["multistream"] = multistream_measure(vsc, dev, args.ms_form or DEFAULT_MS_FORM, 12, 3, True)
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample(frames, os.cpu_count() or 1)
        line["cpu_baseline"]["one_core"] = cpu_baseline_sample(frames, 1, n_frames=1)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


# The full-resolution solver kernel of each form and its compulsory bytes per
# 8-step round (per pixel): exact form O, U, A, consWt, lap P in (60) + O, U
# out (24); FMA form O, U, nK, Cs in (48) + O, U out (24).
SOLVER_KERNELS = {"exact": ("solver_tall_kernel", 84), "fma": ("solver_fma_solve_kernel", 72)}
# dram__bytes_read.sum + dram__bytes_write.sum of one 8-step round at
# 1920x1080 from the ncu captures summarised in profiles/, and where each
# comes from.
SOLVER_TRAFFIC_BYTES = {"solver_tall_kernel": 144_198_912, "solver_fma_solve_kernel": 140_631_616}
SOLVER_TRAFFIC_SOURCE = {
    "solver_tall_kernel": "profiles/solver_tall_1080p.md (one launch per round; mean of two launches: "
                          "124,613,888 + 21,037,568 and 124,601,600 + 18,144,768 bytes)",
    "solver_fma_solve_kernel": "profiles/solver_fma_solve_1080p.md (one launch per solve; per round, the "
                               "difference of a 40-step and an 8-step solve over 4 rounds: (466,624,512 - "
                               "99,649,280) read + (212,874,752 - 17,323,520) written, / 4)",
}
# What bounds each solver kernel, from the same captures: the FP32 pipe and
# its latency, not HBM (the time steps stay on chip): the FMA pipe's active
# cycles per sub-partition cycle (sm__pipe_fma_cycles_active / 4 /
# sm__cycles_active) and smsp__issue_active.
SOLVER_PIPE = {
    "solver_tall_kernel": {"fma_pipe_active": None, "issue_active": 0.585},
    "solver_fma_solve_kernel": {"fma_pipe_active": 0.647, "issue_active": 0.448},
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the precision report and the 16-stream measurement of the default line")
    ap.add_argument("--ms-form", choices=sorted(FORMS), default=None,
                    help="form of the 16-stream measurement inside the default line")
    ap.add_argument("--workload", choices=["1080p", "multistream"], default="1080p",
                    help="multistream: the 16-stream mixed-resolution workload (a separate line)")
    ap.add_argument("--form", choices=sorted(FORMS), default=None,
                    help="the chosen form reported as value (the plain path is timed beside it); default "
                         f"{DEFAULT_FORM} (1080p) or {DEFAULT_MS_FORM} (multistream)")
    ap.add_argument("--ms-grouped", choices=["on", "off"], default="on",
                    help="multistream: group every stream's solve into shared solver launches")
    ap.add_argument("--kernel", choices=["step", "solver", "corr", "front", "upsampler", "warpblend"], default="step",
                    help="solver / corr: time only the 1920x1080 solver or the correlation pyramid "
                         "(profiler targets)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "multistream":
        run_multistream(args)
    elif args.kernel == "solver":
        run_solver_only(args)
    elif args.kernel == "corr":
        run_corr_only(args)
    elif args.kernel == "front":
        run_front_only(args)
    elif args.kernel == "upsampler":
        run_upsampler_only(args)
    elif args.kernel == "warpblend":
        run_warpblend(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
