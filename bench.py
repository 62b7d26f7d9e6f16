"""Benchmark of the headline workload: full development of 5760x3240 RGGB
12-bit frames -- VST + NLM 1.0 (7x7 search, 3x3 patch) + RCD + matrix to
ACES AP1 float32 RGB (with the ACES 1.3 gamut compression) + the AWB
histogram -- on one GB300 per process. The frame is written as RGB32F
(three floats a pixel, the config's "float32 RGB"; an extension format of
this library) by default; ``--out-format rgba32f`` writes the reference's
RGBA32F (alpha 1), which the side runs also measure.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fused|plain|reference]
                    [--storage fp32|fp16]

One JSON line on rank 0. A step develops one frame through
craw_pipeline_record() (libcraw.so). ``value`` is frames/s with the mosaic
resident in device memory, from CUDA events around every step on the
recording stream, L2 flushed (a 256 MB write) between steps; ``e2e`` is
the same metric through the same call with the mosaic copied in from and
the developed frame copied out to pinned host memory inside the timed
region. ``roofline`` is the dominant kernel's (the denoise) HBM view and
``roofline_fp32`` its FP32-pipe view; ``cpu_baseline`` is the CPU oracle
(a port of the reference's lib/ref) on the host cores.

Under torchrun every rank develops its own frames (replicas: the path has
no exchange step); ``value`` is all ranks' frames over the slowest rank's
time.

``--impl reference`` times the reference's CPU implementation of the path
(the oracle port of lib/ref; the reference's own compiled code is only
available where its source tree is) with all host threads, on the same
config, and prints the same kind of line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import ctypes as C
import errno
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "5760x3240 frames/s full develop; p50/p99 frame latency at <=1e-3 rel err"
WORKLOAD = "5760x3240 RGGB 12-bit: VST + NLM 1.0 + RCD + ACES AP1 (RGC) float32 + AWB histogram"
#: Pipelines the end-to-end leg rotates over (`--e2e-lanes`).
E2E_LANES = 3
#: Denoise tile shapes by craw_pipeline_get_kernel_config() index.
DN_SHAPES = ["2x8", "2x4", "2x8 f32x2", "2x4 f32x2"]
#: dram__bytes_read.sum + dram__bytes_write.sum of one launch of the stage's
#: kernel at 5760x3240 (ncu captures summarised in profiles/denoise_nlm_5760x3240.md).
DRAM_BYTES_5760x3240 = {
    ("denoise_nlm", "2x8 f32x2"): 37.365e6 + 1.070e6,
    ("denoise_nlm", "2x8"): 37.37e6 + 0.66e6,
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="fused", choices=["fused", "plain", "reference"])
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16"])
    ap.add_argument("--rounding", default="exact", choices=["exact", "float"],
                    help="exact: the denoised codes as an FP64 evaluation rounds them "
                         "(CRAW_PIPELINE_FLAG_EXACT_ROUNDING), which the metric's 1e-3 bound needs; "
                         "float: the reference's float rounding")
    ap.add_argument("--no-extras", action="store_true", help="skip the plain/fp16/cpu side runs")
    ap.add_argument("--extras", default="plain,fp16,rgba32f,batch,temporal,serve,target,config1,highlights,"
                                        "noise,cpu",
                    help="comma list of side runs: plain, fp16, rgba32f, batch, temporal, serve, "
                         "highlights, noise, cpu")
    ap.add_argument("--force-shape", type=int, default=-1,
                    help="denoise tile shape index instead of the autotuner's (profiling)")
    ap.add_argument("--rcd", default="auto", choices=["auto", "tiles", "strips"],
                    help="RCD interior by 64x16 tiles or by strips instead of the library's choice "
                         "(profiling)")
    ap.add_argument("--e2e-lanes", type=int, default=0,
                    help="pipelines the end-to-end leg rotates over (0: the default)")
    ap.add_argument("--width", type=int, default=None, help="frame width (default: the workload's)")
    ap.add_argument("--height", type=int, default=None, help="frame height (default: the workload's)")
    ap.add_argument("--out-format", default="rgb32f", choices=["rgb32f", "rgba32f"],
                    help="the developed frame's layout: three floats a pixel (the config's float32 "
                         "RGB) or the reference's four (alpha 1)")
    ap.add_argument("--workload", default="nlm_rcd_ap1",
                    choices=["nlm_rcd_ap1", "batch_rcd_bt2020", "bilinear_bt709_1080p"],
                    help="the timed single-frame workload: the headline (5760x3240 VST + NLM + RCD + "
                         "ACES AP1 with the gamut compression), one frame of the batch (the same with "
                         "BT.2020 output), or 1920x1080 bilinear BT.709; for profiling runs")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- helpers

def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


def dist_init(backend: str = "nccl"):
    """Rank, world size and local rank from the torchrun environment; joins
    the process group (NCCL on the GPUs; gloo for the CPU tests of this
    logic). Replicas: no collective touches the data path, only a barrier
    around the timed region and the max of the timings."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if backend == "nccl":
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist.init_process_group(backend)
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(base: int, rank: int, i: int) -> int:
    """Seed of frame `i` of a rank: every replica develops frames of its own."""
    return base + 7919 * rank + i


def whole_job_rate(units_per_rank: int, ws: int, seconds_per_rank: float) -> float:
    """Units all ranks processed over the slowest rank's time (weak scaling:
    per-rank work is fixed, so the job is as fast as its slowest rank)."""
    slowest = max_over_ranks(seconds_per_rank, ws)
    return ws * units_per_rank / slowest


# ------------------------------------------------------------- CPU baseline

def cpu_oracle_fps(frame: np.ndarray, params, fp, rows_frac: float = 0.25, single: bool = True) -> dict:
    """The CPU oracle (float restatement of the reference's lib/ref) on
    `rows_frac` of a frame, split into one strip per host thread, each strip
    developed as a frame of its own: frames/s = rows_frac / wall time.
    `single`: also time one strip alone on one thread (outside that wall
    time) for the single-threaded milliseconds a frame."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle import Oracle
    import libcraw_gb300 as L

    orc = Oracle()
    cores = os.cpu_count() or 1
    h, w = frame.shape
    rows = max(16, int(h * rows_frac) // cores // 2 * 2)
    strips = [np.ascontiguousarray(frame[i * rows:(i + 1) * rows]) for i in range(cores)]
    pps = [L.pipeline_params(w, rows, debayer=params.debayer, out_space=params.out_space,
                             flags=params.flags, out_format=L.FORMAT_RGBA32F) for _ in strips]
    outs = [None] * cores

    def work(i):
        outs[i] = orc.process(strips[i], pps[i], fp, "f32")

    threads = [threading.Thread(target=work, args=(i,)) for i in range(cores)]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    dt = time.perf_counter() - t0
    done = rows * cores / h
    res = {"value": done / dt, "unit": "frames/s", "cores": cores, "kind": "port",
           "sample": f"{cores} strips of {w}x{rows} ({done:.3f} of a frame) through the float "
                     f"oracle (lib/ref restated), one strip per host thread, {dt:.2f} s wall",
           "nproc": cores, "cpu_model": cpu_model()}
    if single:
        t1 = time.perf_counter()
        work(0)
        res["single_thread_ms_per_frame"] = (time.perf_counter() - t1) * 1e3 * h / rows
    return res


def cpu_model() -> str:
    """The host CPU's name as /proc/cpuinfo gives it (x86: "model name";
    Arm: implementer and part numbers), else the machine type."""
    import platform
    try:
        info = open("/proc/cpuinfo").read().splitlines()
    except OSError:
        return platform.machine()
    fields = {}
    for line in info:
        k, _, v = line.partition(":")
        fields.setdefault(k.strip(), v.strip())
    if "model name" in fields:
        return fields["model name"]
    if "CPU part" in fields:
        # Arm Ltd (implementer 0x41) cores by part number.
        arm = {"0xd0c": "Neoverse-N1", "0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2",
               "0xd4f": "Neoverse-V2", "0xd84": "Neoverse-V3"}
        part = fields["CPU part"].lower()
        if fields.get("CPU implementer", "").lower() == "0x41" and part in arm:
            return f"Arm {arm[part]}"
        return (f"{platform.machine()} implementer {fields.get('CPU implementer', '?')} "
                f"part {fields['CPU part']}")
    return platform.machine()


def out_image(L, w, h, fmt):
    """A device image for the developed frame: (tensor, craw image). RGB32F
    rows are w * 12 bytes rounded up to 16 (the tensor a view of them)."""
    import torch
    if fmt == L.FORMAT_RGB32F:
        pitch = (w * 12 + 15) // 16 * 16
        buf = torch.empty((h, pitch // 4), dtype=torch.float32, device="cuda")
        return buf[:, : 3 * w].view(h, w, 3), L.Image(buf.data_ptr(), pitch, fmt, w, h)
    t = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    return t, L.Image(t.data_ptr(), w * 16, fmt, w, h)


def run_reference(args):
    # Rank 0 alone runs the CPU baseline; the other ranks have no work.
    if int(os.environ.get("RANK", "0")) != 0:
        return
    ws = 1
    import libcraw_gb300 as L
    from libcraw_gb300 import build as B
    from libcraw_gb300 import workloads as W
    B.build()
    c = W.workload("nlm_rcd_ap1", args.width, args.height)
    frame = c.frame()
    prof = W.make_profile()
    pp = L.pipeline_params(c.width, c.height, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                           out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, **c.frame_kwargs())
    frac = 0.5
    for _ in range(args.warmup):
        cpu_oracle_fps(frame, pp, fp, frac, single=False)
    times = []
    last = None
    for i in range(args.steps):
        last = cpu_oracle_fps(frame, pp, fp, frac, single=i == args.steps - 1)
        times.append(frac / last["value"])
    total = sum(times)
    value = args.steps * frac / total
    lat = sorted(t / frac * 1000 for t in times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1000, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: the seeded generator's 5760x3240 frames",
        "config": {"workload": WORKLOAD, "width": c.width, "height": c.height},
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "cpu_baseline": {**last, "value": value},
        "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(ws)


# --------------------------------------------------------------- GPU arm

def run_gpu(args):
    import torch

    global E2E_LANES
    if args.e2e_lanes > 0:
        E2E_LANES = args.e2e_lanes
    rank, ws, local = dist_init()
    import libcraw_gb300 as L
    from libcraw_gb300 import build as B
    from libcraw_gb300 import workloads as W
    if rank == 0 or ws == 1:
        B.build()
    barrier(ws)
    torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    props = torch.cuda.get_device_properties(dev)

    c = W.workload(args.workload, args.width, args.height)
    w, h = c.width, c.height
    label = WORKLOAD if args.workload == "nlm_rcd_ap1" and (w, h) == (5760, 3240) else f"{w}x{h} {c.name}"
    prof = W.make_profile()
    fp = L.frame_params(prof, **c.frame_kwargs())
    storage = L.STORAGE_FP16 if args.storage == "fp16" else L.STORAGE_FP32
    impl = L.IMPL_PLAIN if args.impl == "plain" else L.IMPL_FUSED

    # Four distinct frames in rotation (different seeds), 16-byte rows.
    nfr = 4
    host_frames = [W.synth_frame(w, h, replica_seed(c.seed, rank, i), rects=c.rects, zone_plates=c.zone_plates,
                                 noise_a_dn=c.noise_a_dn, noise_b_dn=c.noise_b_dn) for i in range(nfr)]
    dev_frames = [torch.from_numpy(f.view(np.int16)).cuda() for f in host_frames]
    srcs = [L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h) for t in dev_frames]
    out_fmt = L.FORMAT_RGB32F if args.out_format == "rgb32f" else L.FORMAT_RGBA32F
    out, dst = out_image(L, w, h, out_fmt)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    ctx = L.Context(dev)
    if args.force_shape >= 0:
        # A fixed denoise shape and no autotuner launches, for profiling runs.
        L.debug_force_denoise_shape(args.force_shape)
    if args.rcd != "auto":
        # The RCD interior by tiles or by strips whatever the colour stage.
        L.debug_rcd_strips(0 if args.rcd == "tiles" else 2)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream

    exact = args.rounding == "exact" and impl == L.IMPL_FUSED

    def make_pipe(impl_, storage_, profile=True, exact_=None, fmt=None):
        exact_ = exact if exact_ is None else exact_
        flags = c.flags | (L.FLAG_PROFILE if profile else 0) | (L.FLAG_EXACT_ROUNDING if exact_ else 0)
        return L.Pipeline(ctx, L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space,
                                                 flags=flags, out_format=fmt or out_fmt,
                                                 storage=storage_, impl=impl_, nb_awb_slots=2))

    def timed(pipe, steps, warmup, collect=True, dst=dst):
        with torch.cuda.stream(stream):
            for i in range(warmup):
                pipe.record(sptr, srcs[i % nfr], dst, fp)
            torch.cuda.synchronize()
            barrier(ws)
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(steps)]
            stage: dict[str, list[float]] = {}
            t0 = time.perf_counter()
            for i in range(steps):
                flush.zero_()
                evs[i][0].record(stream)
                pipe.record(sptr, srcs[i % nfr], dst, fp)
                evs[i][1].record(stream)
                if collect:
                    evs[i][1].synchronize()
                    for name, cnt, ms in pipe.stage_times():
                        stage.setdefault(name, []).append(ms)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        barrier(ws)
        ms = [a.elapsed_time(b) for a, b in evs]
        return ms, stage, wall

    pipe = make_pipe(impl, storage)
    kcfg = pipe.kernel_config()
    with ClockSampler(dev) as clk:
        ms, stage, wall = timed(pipe, args.steps, max(3, args.warmup))
    total_s = sum(ms) / 1000.0
    value = whole_job_rate(args.steps, ws, total_s)
    lat = sorted(ms)
    hist = pipe.awb_histogram()

    # The roofline of the dominant kernel, from its own events in the timed region.
    dom = max(stage, key=lambda k: sum(stage[k])) if stage else None
    dom_ms = statistics.mean(stage[dom]) if dom else None
    n_px = w * h
    pk = peaks()
    roof = roof32 = None
    if dom:
        # Algorithmic bytes per launch of the denoise: mosaic in (2 B/px), denoised
        # mosaic out (2 B/px); of the develop: mosaic in (2) + RGBA32F out (16)
        # + AWB records (8 per 64 px).
        bpp = {"denoise_nlm": 4.0, "develop": 18.0 + 8.0 / 64, "plain_denoise": 4.0,
               "plain_develop": 18.0}.get(dom, 4.0)
        achieved = bpp * n_px / (dom_ms / 1000.0) / 1e9
        # DRAM bytes (read + write) of one launch from an ncu capture at
        # 5760x3240 (profiles/), scaled by the pixels of this run.
        traffic = DRAM_BYTES_5760x3240.get((dom, DN_SHAPES[kcfg[0]]))
        if traffic is not None:
            traffic = traffic * n_px / (5760 * 3240)
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                "peak_src": pk["src"], "bytes_per_px": bpp, "ms_per_launch": dom_ms}
        if dom.endswith("denoise_nlm") or dom == "plain_denoise":
            clk_s = clk.summary()
            mhz = clk_s["sm_mhz"] or 2070.0
            peak_lane_ops = props.multi_processor_count * 128 * mhz * 1e6 / 1e12
            ops = n_px * 49 * 13 / (dom_ms / 1000.0) / 1e12
            roof32 = {"bound": "fp32", "achieved": ops, "peak": peak_lane_ops, "unit": "Tlane-op/s",
                      "frac": ops / peak_lane_ops,
                      "model": "N*49*13 FP32 lane-ops per frame (7x7 search, 13 ops an offset); "
                               "peak = SMs x 128 FP32 lanes x median SM clock"}
            # The HBM fraction is small by nature: the NLM does 637 FP32
            # operations per 4 bytes moved. The binding roofline is the FP32 pipe.
            roof["binding"] = "fp32"
            roof["binding_frac"] = roof32["frac"]
            roof["note"] = ("the denoise is bound by the FP32 pipe, not by HBM: "
                            f"{roof32['frac']:.2f} of the FP32 lane rate (roofline_fp32), "
                            f"{roof['frac']:.3f} of HBM")

    # End to end through the same call: pinned host mosaic in, the frame
    # out. E2E_LANES lanes (pipeline + CUDA stream + device buffers each)
    # take the steps in turn, so one frame's copy in, another's kernels and
    # others' copies out overlap, as a caller streaming frames would.
    pinned_in = [torch.from_numpy(f.view(np.int16)).pin_memory() for f in host_frames]

    def run_e2e(fmt):
        lanes = []
        for _ in range(E2E_LANES):
            ls = torch.cuda.Stream()
            d_in = torch.empty((h, w), dtype=torch.int16, device="cuda")
            d_out, d_img = out_image(L, w, h, fmt)
            lanes.append(dict(stream=ls, d_in=d_in, d_buf=d_out._base if d_out._base is not None else d_out,
                              src=L.Image(d_in.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h), dst=d_img,
                              pipe=make_pipe(impl, storage, profile=False, fmt=fmt)))
            ln = lanes[-1]
            ln["h_buf"] = torch.empty(ln["d_buf"].shape, dtype=ln["d_buf"].dtype).pin_memory()

        def e2e_step(i, nl):
            ln = lanes[i % nl]
            with torch.cuda.stream(ln["stream"]):
                ln["d_in"].copy_(pinned_in[i % nfr], non_blocking=True)
                ln["pipe"].record(ln["stream"].cuda_stream, ln["src"], ln["dst"], fp)
                ln["h_buf"].copy_(ln["d_buf"], non_blocking=True)

        def e2e_run(nl):
            for i in range(3 * nl):
                e2e_step(i, nl)
            torch.cuda.synchronize()
            barrier(ws)
            t0 = time.perf_counter()
            for i in range(args.steps):
                e2e_step(i, nl)
            torch.cuda.synchronize()
            return max_over_ranks(time.perf_counter() - t0, ws)

        e2e_s1 = e2e_run(1)
        e2e_s = e2e_run(len(lanes))
        name = "RGB32F" if fmt == L.FORMAT_RGB32F else "RGBA32F"
        res = {"value": ws * args.steps / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": w * h * 2,
               "d2h_bytes_per_step": lanes[0]["h_buf"].numel() * 4,
               "one_stream_value": ws * args.steps / e2e_s1,
               "how": "per step: H2D of the mosaic from pinned memory, craw_pipeline_record, D2H of "
                      f"the {name} frame to pinned memory, on one of {E2E_LANES} streams in turn (each with "
                      "its own pipeline and buffers); wall clock over all steps; one_stream_value: all "
                      "steps on one stream"}
        for ln in lanes:
            ln["pipe"].close()
        return res

    e2e = run_e2e(out_fmt)

    extras = {}
    want = set() if args.no_extras else set(args.extras.split(","))
    if want and rank == 0:
        if "serve" in want:
            # The serving workload first, right after the headline: after
            # the plain, FP16 and RGBA32F side runs in the same process its
            # requests' device time rose by half or more (p99 22-28 ms
            # against 6-7 ms), without throttling, for a reason not found.
            extras["serve"] = run_serve(ctx)
        for name, (im, st) in {"plain_fp32": (L.IMPL_PLAIN, L.STORAGE_FP32),
                               "fused_fp16": (L.IMPL_FUSED, L.STORAGE_FP16),
                               "fused_fp32": (L.IMPL_FUSED, L.STORAGE_FP32)}.items():
            if im == impl and st == storage:
                continue
            if ("plain" if im == L.IMPL_PLAIN else "fp16") not in want:
                continue
            with make_pipe(im, st, profile=False) as p2:
                m2, _, _ = timed(p2, max(5, args.steps // 3), 3, collect=False)
            extras[name] = {"fps": 1000.0 / statistics.mean(m2), "ms_per_frame": statistics.mean(m2)}
        if "rgba32f" in want and out_fmt != L.FORMAT_RGBA32F:
            # The reference's output layout, four floats a pixel (alpha 1):
            # a quarter more bytes written, and copied to the host.
            o4, d4 = out_image(L, w, h, L.FORMAT_RGBA32F)
            with make_pipe(impl, storage, profile=False, fmt=L.FORMAT_RGBA32F) as p2:
                m2, _, _ = timed(p2, max(5, args.steps // 3), 3, collect=False, dst=d4)
            del o4
            extras["rgba32f_output"] = {"fps": 1000.0 / statistics.mean(m2), "ms_per_frame": statistics.mean(m2),
                                        "e2e": run_e2e(L.FORMAT_RGBA32F)}
        if exact:
            # The same pipeline with the reference's float rounding of the
            # denoised codes (about 0.03 % of them one code from an FP64
            # evaluation's; the frame up to a few 1e-3 from FP64).
            with make_pipe(impl, storage, profile=False, exact_=False) as p2:
                m2, _, _ = timed(p2, max(5, args.steps // 3), 3, collect=False)
            extras["float_rounding"] = {"fps": 1000.0 / statistics.mean(m2), "ms_per_frame": statistics.mean(m2)}
        base = extras.get("plain_fp32", {}).get("fps")
        if base:
            extras["speedup_vs_plain_fp32"] = (args.steps / total_s) / base
        if "batch" in want:
            extras["batch"] = run_batch_mix(ctx, stream, max(5, args.steps // 3), 3)
            small = [W.BatchFrame(640, 360, 41000 + i, 4.0, 40.0) for i in range(64)]
            extras["batch_small"] = run_batch_mix(
                ctx, stream, max(5, args.steps // 3), 3, small,
                "64 frames of 640x360 (previews), NLM 1.0 + RCD + BT.2020 float32")
            if base:
                extras["batch"]["eq_speedup_vs_plain_fp32"] = (
                    extras["batch"]["split_default"]["eq_5760x3240_fps"] / base)
                extras["batch"]["persistent_eq_speedup_vs_plain_fp32"] = (
                    extras["batch"]["unfused_graph"]["eq_5760x3240_fps"] / base)
        if "temporal" in want:
            extras["temporal_seq"] = run_temporal_seq(ctx, stream)
        if "serve" in want and base:
            extras["serve"]["eq_speedup_vs_plain_fp32"] = (
                extras["serve"]["saturated"]["eq_5760x3240_fps"] / base)
        if "target" in want:
            extras["target"] = run_target(ctx, stream)
        if "config1" in want:
            extras["config1"] = run_config1(ctx, stream, max(10, args.steps), 3)
        if "highlights" in want:
            extras["highlights"] = run_highlights(ctx, stream)
        if "noise" in want:
            extras["noise_estimate"] = run_noise_estimate(cpu="cpu" in want)

    cpu = None
    if rank == 0 and "cpu" in want:
        cpu = cpu_oracle_fps(host_frames[0], L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space,
                                                              flags=c.flags), fp, 1.0)

    if rank == 0:
        clk_s = clk.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": sum(ms) / len(ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded generator (gradient + 256 rectangles + 4 zone plates, "
                    "Poisson-Gaussian noise a=4 DN, b=40 DN^2), 4 frames in rotation",
            "config": {"workload": label, "width": w, "height": h, "impl": args.impl,
                       "output": "RGB32F (three floats a pixel)" if out_fmt == L.FORMAT_RGB32F
                                 else "RGBA32F (four floats a pixel, alpha 1)",
                       "storage": args.storage, "l2": "flushed between steps (256 MB write)",
                       "rounding": ("exact: denoised codes as an FP64 evaluation rounds them"
                                    if exact else "float (the reference's)"),
                       "parallelism": f"replicas x{ws}",
                       "denoise_tile": DN_SHAPES[kcfg[0]] + " (autotuned)"},
            "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                           "max": lat[-1]},
            "stage_ms": {k: statistics.mean(v) for k, v in stage.items()},
            "roofline": roof, "roofline_fp32": roof32,
            "e2e": e2e,
            # Our kernels per step: fused = denoise, [the rounding's compaction,
            # decision and double-float kernels,] RCD interior (tiles or strips),
            # RCD border tiles, awb_reduce; plain = vst + nlm, prep + 8 RCD
            # sweeps + awb + colour.
            "gpu_launches": args.steps * ((7 if exact else 4) if impl == L.IMPL_FUSED else 13),
            "clocks": {k: clk_s[k] for k in ("sm_mhz", "sm_max_mhz", "reasons")},
            "awb_samples": int(hist.count.sum()),
            "wall_s_timed": wall,
            "extras": extras,
            "cpu_baseline": cpu,
            "device": props.name,
        }
        print(json.dumps(line), flush=True)
    pipe.close()
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_batch_mix(ctx, stream, steps: int, warmup: int, mix=None, label: str | None = None) -> dict:
    """The batched workload (16 frames of four sizes, NLM 1.0 + RCD + BT.2020
    float32) as one recording of the batch API: a persistent fused launch
    replayed from a captured CUDA graph; beside it the unfused and
    graph-less variants and the same 16 frames through the single-frame
    pipeline one after another. Inputs (336 MB) are larger than L2.
    `mix` / `label` run another list of frames the same way."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    mix = mix or W.batch_mix()
    prof = W.make_profile()
    mw, mh = max(f.width for f in mix), max(f.height for f in mix)
    srcs, dsts, fps, keep = [], [], [], []
    for f in mix:
        t = torch.from_numpy(f.frame().view(np.int16)).cuda()
        o = torch.empty((f.height, f.width, 4), dtype=torch.float32, device="cuda")
        keep += [t, o]
        srcs.append(L.Image(t.data_ptr(), f.width * 2, L.FORMAT_R16_UNORM, f.width, f.height))
        dsts.append(L.Image(o.data_ptr(), f.width * 16, L.FORMAT_RGBA32F, f.width, f.height))
        fps.append(L.frame_params(prof, denoise_strength=1.0,
                                  noise_override=W.noise_model(f.noise_a_dn, f.noise_b_dn)))
    n_px = sum(f.width * f.height for f in mix)
    sptr = stream.cuda_stream

    def timed(record):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                record()
            torch.cuda.synchronize()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(steps)]
            for e0, e1 in evs:
                e0.record(stream)
                record()
                e1.record(stream)
            torch.cuda.synchronize()
        ms = sorted(a.elapsed_time(b) for a, b in evs)
        return {"ms_per_batch": statistics.mean(ms), "p50_ms": ms[len(ms) // 2], "max_ms": ms[-1],
                "frames_per_s": len(mix) * 1000.0 / statistics.mean(ms),
                "mpx_per_s": n_px / 1e3 / statistics.mean(ms),
                "eq_5760x3240_fps": n_px / (5760 * 3240) * 1000.0 / statistics.mean(ms)}

    res = {"workload": label or ("16 frames: 6x1920x1080, 4x3840x2160, 4x5760x3240, 2x6000x4000; "
                                 "NLM 1.0 + RCD + BT.2020 float32; noise a~U[1,8], b~U[10,80] per frame"),
           "mpx": n_px / 1e6}
    # Every frame in the persistent launch (one fused launch with a grid
    # barrier, two launches, without a graph), then the default plan: two
    # persistent launches from a graph for the frames under 4 Mpx, the
    # larger ones through the single-frame kernels after them.
    for name, flags, direct in (("fused_graph", L.BATCH_FLAG_FUSED, L.BATCH_ALL_PERSISTENT),
                                ("unfused_graph", L.BATCH_FLAG_UNFUSED, L.BATCH_ALL_PERSISTENT),
                                ("fused_no_graph", L.BATCH_FLAG_FUSED | L.BATCH_FLAG_NO_GRAPH,
                                 L.BATCH_ALL_PERSISTENT),
                                ("split_default", 0, 0)):
        bp = L.batch_params(mw, mh, max_frames=len(mix), debayer=L.DEBAYER_RCD,
                            out_space=L.CS_BT2020, flags=L.FLAG_DENOISE | flags, direct_pixels=direct)
        with L.Batch(ctx, bp) as b:
            res[name] = timed(lambda: b.record(sptr, srcs, dsts, fps))
            info = b.info()
            res[name]["denoise_tile"] = ["2x4", "2x8"][info["denoise_shape"]]
            if info["direct_frames"]:
                res[name]["direct_frames_per_batch"] = sum(
                    1 for f in mix if f.width * f.height >= L.BATCH_DIRECT_PIXELS)
                res[name]["direct_denoise_tile"] = L.DN_SHAPES[info["direct_shape"]]
    pipes = {}
    for f in mix:
        if (f.width, f.height) not in pipes:
            pipes[(f.width, f.height)] = L.Pipeline(ctx, L.pipeline_params(
                f.width, f.height, debayer=L.DEBAYER_RCD, out_space=L.CS_BT2020,
                flags=L.FLAG_DENOISE, out_format=L.FORMAT_RGBA32F))

    def singles():
        for f, s_, d_, fp_ in zip(mix, srcs, dsts, fps):
            pipes[(f.width, f.height)].record(sptr, s_, d_, fp_)
    res["single_frame_pipeline"] = timed(singles)
    for p_ in pipes.values():
        p_.close()
    res["speedup_vs_single_frames"] = (res["unfused_graph"]["frames_per_s"] /
                                       res["single_frame_pipeline"]["frames_per_s"])
    res["split_speedup_vs_single_frames"] = (res["split_default"]["frames_per_s"] /
                                             res["single_frame_pipeline"]["frames_per_s"])
    return res


def run_highlights(ctx, stream, nsteps: int = 20) -> dict:
    """The headline chain (VST + NLM 1.0 + RCD + ACES AP1 + AWB) with the
    highlight reconstruction on, at 5760x3240, on the benchmark scene and
    on a scene whose highlights clip (2.5x under three lamps: 30 % of sites
    near or at the clip): frames/s from CUDA events around each record and
    the per-stage device times."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    c = W.workload("nlm_rcd_ap1")
    w, h = c.width, c.height
    prof = W.make_profile()
    fp = L.frame_params(prof, flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION, **c.frame_kwargs())
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    dst = L.Image(out.data_ptr(), w * 16, L.FORMAT_RGBA32F, w, h)
    pp = L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space,
                           flags=c.flags | L.FLAG_PROFILE | L.FLAG_HIGHLIGHT_RECONSTRUCTION,
                           out_format=L.FORMAT_RGBA32F)
    res = {"workload": f"{w}x{h}: VST + NLM 1.0 + highlight reconstruction + RCD + ACES AP1 f32 + AWB"}
    for scene, frame in (("benchmark_scene", c.frame(0)), ("clipped_scene", W.highlight_frame(w, h, 7))):
        t = torch.from_numpy(frame.view(np.int16)).cuda()
        src = L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h)
        with L.Pipeline(ctx, pp) as pipe, torch.cuda.stream(stream):
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(nsteps + 3)]
            stage: dict[str, list[float]] = {}
            for i, (e0, e1) in enumerate(evs):
                e0.record(stream)
                pipe.record(stream.cuda_stream, src, dst, fp)
                e1.record(stream)
                e1.synchronize()
                if i >= 3:
                    for sname, _, ms in pipe.stage_times():
                        stage.setdefault(sname, []).append(ms)
            torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in evs[3:]]
        res[scene] = {"fps": 1000.0 * len(ms) / sum(ms), "ms_per_frame": statistics.mean(ms),
                      "stage_ms": {k: statistics.mean(v) for k, v in stage.items()}}
    return res


def run_noise_estimate(nsteps: int = 10, cpu: bool = True) -> dict:
    """craw_noise_estimate_cuda() on a 5760x3240 frame of the benchmark
    scene already on the device (wall time of the call, which ends with
    the estimate on the host), craw_noise_estimate() from host memory, and
    the CPU oracle (the reference's algorithm restated, one host thread,
    as the reference runs it) on the same frame."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    c = W.workload("nlm_rcd_ap1")
    w, h = c.width, c.height
    prof = W.make_profile()
    frame = c.frame(0)
    t = torch.from_numpy(frame.view(np.int16)).cuda()
    img = L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h)
    s = torch.cuda.Stream()
    for _ in range(3):
        est = L.noise_estimate_cuda(img, prof, stream=s.cuda_stream)
    dev = []
    for _ in range(nsteps):
        t0 = time.perf_counter()
        est = L.noise_estimate_cuda(img, prof, stream=s.cuda_stream)
        dev.append(1e3 * (time.perf_counter() - t0))
    host = []
    for _ in range(3):
        t0 = time.perf_counter()
        L.noise_estimate(frame, prof)
        host.append(1e3 * (time.perf_counter() - t0))
    res = {"workload": f"{w}x{h} benchmark scene, default options (128 bins, 20000 samples a bin)",
           "device_ms": statistics.median(dev), "host_frame_ms": statistics.median(host),
           "estimate": {"a": est.model.a, "b": est.model.b, "bins": est.nb_bins,
                        "inliers": est.nb_inliers, "fit_rms": est.fit_rms},
           "true_model": list(W.noise_model(4.0, 40.0))}
    if cpu:
        sys.path.insert(0, str(ROOT / "tests"))
        from oracle import Oracle
        t0 = time.perf_counter()
        ret, ref = Oracle().noise_estimate(frame, prof)
        res["cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t0)
        res["cpu_oracle_cores"] = 1
        res["same_as_oracle"] = ret == 0 and ref.as_tuple() == est.as_tuple()
    return res


def run_config1(ctx, stream, steps: int, warmup: int) -> dict:
    """The plain-method configuration: one 1920x1080 frame, bilinear, no
    denoise, BT.709 linear float32 + AWB histogram, from device memory, L2
    flushed between steps (the frame and its output fit in it)."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    c = W.workload("bilinear_bt709_1080p")
    w, h = c.width, c.height
    fp = L.frame_params(W.make_profile())
    frames = [torch.from_numpy(W.synth_frame(w, h, c.seed + i, rects=c.rects, zone_plates=c.zone_plates,
                                             noise_a_dn=c.noise_a_dn, noise_b_dn=c.noise_b_dn).view(np.int16)).cuda()
              for i in range(4)]
    srcs = [L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h) for t in frames]
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    dst = L.Image(out.data_ptr(), w * 16, L.FORMAT_RGBA32F, w, h)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    pp = L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                           out_format=L.FORMAT_RGBA32F)
    sptr = stream.cuda_stream
    with L.Pipeline(ctx, pp) as pipe, torch.cuda.stream(stream):
        for i in range(warmup):
            pipe.record(sptr, srcs[i % 4], dst, fp)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        # A frame this small takes the device less time than the host takes
        # to record it, so the device is held (torch's bounded sleep kernel,
        # 0.4 ms a step at the maximum clock) while every step is enqueued:
        # the events then bracket the device's work alone, and the host's
        # recording time is reported beside it.
        torch.cuda._sleep(int(steps * 0.4e-3 * 2.07e9))
        t0 = time.perf_counter()
        for i, (e0, e1) in enumerate(evs):
            flush.zero_()
            e0.record(stream)
            pipe.record(sptr, srcs[i % 4], dst, fp)
            e1.record(stream)
        host_s = time.perf_counter() - t0
        torch.cuda.synchronize()
        # The same steps without the hold: the host's recording paces them.
        paced = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(steps)]
        for i, (e0, e1) in enumerate(paced):
            flush.zero_()
            e0.record(stream)
            pipe.record(sptr, srcs[i % 4], dst, fp)
            e1.record(stream)
        torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in evs]
    ms_paced = [a.elapsed_time(b) for a, b in paced]
    # Algorithmic bytes: mosaic in 2 B/px, RGBA32F out 16 B/px, AWB records 8 B per 64 px.
    gbs = (18.0 + 8.0 / 64) * w * h / (statistics.mean(ms) / 1000.0) / 1e9
    return {"workload": "1920x1080 RGGB 12-bit (var = 2 s + 16 DN^2): bilinear, no denoise, BT.709 f32 + AWB",
            "fps": 1000.0 / statistics.mean(ms), "ms_per_frame": statistics.mean(ms),
            "hbm_gbs": gbs, "hbm_frac": gbs / peaks()["hbm_gbs"],
            "host_record_ms_per_step": 1000.0 * host_s / steps,
            "ms_per_frame_host_paced": statistics.mean(ms_paced),
            "how": "device time of each step's recording (events around craw_pipeline_record, L2 flushed "
                   "before each), the steps enqueued while a bounded sleep kernel held the device; "
                   "host_paced: the same with each step enqueued as the device reaches it"}


def run_temporal_seq(ctx, stream, nsteps: int = 60, distinct: int = 12) -> dict:
    """The temporal sequence (60 frames of 5760x3240, rectangles moving 2, 8
    and 24 px/frame, temporal 0.8 + NLM 1.0 + chroma 0.5 + MHC + P3-D65
    float32 + AWB) through one pipeline, FP32 and FP16 storage: frames/s
    from CUDA events around each record, and how far the FP16 output lies
    from the FP32 one on the last frame. `distinct` seeded frames are
    generated and cycled (the work does not depend on the content)."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    c = W.workload("temporal_mhc_p3")
    w, h = c.width, c.height
    prof = W.make_profile()
    fp = L.frame_params(prof, **c.frame_kwargs())
    dev = [torch.from_numpy(c.frame(i).view(np.int16)).cuda() for i in range(distinct)]
    srcs = [L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h) for t in dev]
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    dst = L.Image(out.data_ptr(), w * 16, L.FORMAT_RGBA32F, w, h)
    sptr = stream.cuda_stream
    res, last = {}, {}
    for name, storage in (("fp32", L.STORAGE_FP32), ("fp16", L.STORAGE_FP16)):
        pp = L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space,
                               flags=c.flags | L.FLAG_PROFILE, out_format=L.FORMAT_RGBA32F,
                               storage=storage, nb_awb_slots=2)
        with L.Pipeline(ctx, pp) as pipe, torch.cuda.stream(stream):
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(nsteps)]
            stage: dict[str, list[float]] = {}
            for i, (e0, e1) in enumerate(evs):
                e0.record(stream)
                pipe.record(sptr, srcs[i % distinct], dst, fp)
                e1.record(stream)
                if i >= 3:
                    e1.synchronize()
                    for sname, _, ms in pipe.stage_times():
                        stage.setdefault(sname, []).append(ms)
            torch.cuda.synchronize()
            last[name] = out.clone()
        ms = sorted(a.elapsed_time(b) for a, b in evs[3:])
        res[name] = {"fps": 1000.0 * len(ms) / sum(ms), "p50_ms": ms[len(ms) // 2],
                     "p99_ms": ms[min(len(ms) - 1, int(0.99 * len(ms)))],
                     "stage_ms": {k: statistics.mean(v) for k, v in stage.items()}}
    a, b = last["fp16"].float(), last["fp32"].float()
    peak = float(b[..., :3].abs().max())
    den = torch.maximum(b[..., :3].abs(), torch.tensor(0.01 * peak, device=b.device))
    rel = ((a[..., :3] - b[..., :3]).abs() / den)
    mse = float(((a[..., :3] - b[..., :3]) ** 2).mean())
    res["fp16_vs_fp32_last_frame"] = {"max_rel": float(rel.max()), "mean_rel": float(rel.mean()),
                                      "psnr_db": 10 * np.log10(peak * peak / max(mse, 1e-30))}
    res["workload"] = (f"{w}x{h} x{nsteps} (12 distinct seeded frames cycled), movers 2/8/24 px: "
                       "temporal 0.8 + NLM 1.0 + chroma 0.5 + MHC + P3-D65 f32 + AWB")
    return res


def run_target(ctx, stream, nframes: int = 24, plain_frames: int = 6, streams: int = 4) -> dict:
    """The headline target's chain: 5760x3240 frames through temporal 0.8 +
    NLM 1.0 + RCD + matrix (ACES AP1, RGC) float32, FP16 storage, against
    the plain FP32 single-frame pipeline on the same chain, temporal
    included. Frames/s of: the plain FP32 pipeline; the fused FP16 pipeline
    (device-resident frames, CUDA events); the frame server developing
    `streams` such clips at once from pinned host memory to pinned host
    memory, RGB32F out (saturated). The batch (one persistent launch for
    many frames) takes spatial frames only, so it does not run this chain.
    And the fused output's error against the FP64 oracle on a 256x128 window in the
    middle of a frame with a history (the oracle fed the state the GPU
    left: the crop of frame 1's mosaic developed from frame 0's state)."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    c = W.workload("serve_rcd_ap0")
    w, h = c.width, c.height
    prof = W.make_profile()
    model = W.noise_model(c.noise_a_dn, c.noise_b_dn)
    fp = L.frame_params(prof, denoise_strength=1.0, denoise_temporal_strength=0.8, noise_override=model,
                        out_space=L.CS_ACES_AP1, out_space_set=1)
    flags = L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE
    movers = [(2.0, 0.5), (8.0, 2.0), (24.0, 10.0)]
    host = [W.synth_frame(w, h, 60060 + i, frame=i, rects=256, zone_plates=4, noise_a_dn=c.noise_a_dn,
                          noise_b_dn=c.noise_b_dn, movers=movers) for i in range(4)]
    dev = [torch.from_numpy(f.view(np.int16)).cuda() for f in host]
    srcs = [L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h) for t in dev]
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    dst = L.Image(out.data_ptr(), w * 16, L.FORMAT_RGBA32F, w, h)
    sptr = stream.cuda_stream
    res = {"chain": f"{w}x{h} temporal 0.8 + NLM 1.0 + RCD + ACES AP1 (RGC) float32"}

    def seq(impl, storage, n, keep=False):
        pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                               flags=flags | (L.FLAG_KEEP_INTERMEDIATE if keep else 0),
                               out_format=L.FORMAT_RGBA32F, storage=storage, impl=impl)
        with L.Pipeline(ctx, pp) as pipe, torch.cuda.stream(stream):
            for i in range(2):
                pipe.record(sptr, srcs[i % 4], dst, fp)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(n):
                pipe.record(sptr, srcs[i % 4], dst, fp)
            e1.record(stream)
            torch.cuda.synchronize()
            return 1000.0 * n / e0.elapsed_time(e1)

    res["plain_fp32_fps"] = seq(L.IMPL_PLAIN, L.STORAGE_FP32, plain_frames)
    res["fused_fp16_fps"] = seq(L.IMPL_FUSED, L.STORAGE_FP16, nframes)
    res["fused_fp32_fps"] = seq(L.IMPL_FUSED, L.STORAGE_FP32, nframes)

    # Served: `streams` clips at once, every frame submitted up front.
    pin_in = [torch.from_numpy(f.view(np.int16)).pin_memory() for f in host]
    outs = [torch.empty((h, w, 3), dtype=torch.float32).pin_memory() for _ in range(2 * streams)]
    pp16 = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1, flags=flags,
                             out_format=L.FORMAT_RGB32F, storage=L.STORAGE_FP16)
    with L.Server(ctx, L.server_params(hbm_budget=60 << 30, max_inflight=2 * streams,
                                       slots_per_stream=2)) as srv:
        sids = [srv.open(L.server_stream_params(pp16)) for _ in range(streams)]
        t0 = time.perf_counter()
        for i in range(nframes):
            for k, sid in enumerate(sids):
                o = outs[(i % 2) * streams + k]
                srv.submit(sid, pin_in[(i + k) % 4].data_ptr(), w * 2, o.data_ptr(), w * 12, fp, i / 24.0,
                           (k << 32) | i)
        srv.drain()
        wall = time.perf_counter() - t0
        got = []
        while True:
            r = srv.poll(256, 0)
            if not r:
                break
            got += r
    res["served_fp16"] = {"streams": streams, "frames": len(got), "fps": len(got) / wall,
                          "device_ms_mean": float(np.mean([r.device_ms for r in got])),
                          "how": "host to host: pinned mosaic in, pinned RGB32F out, inside the timing"}
    base = res["plain_fp32_fps"]
    res["fused_fp16_vs_plain_fp32"] = res["fused_fp16_fps"] / base
    res["served_fp16_vs_plain_fp32"] = res["served_fp16"]["fps"] / base
    res["batch"] = "not run: the persistent batch launch carries spatial frames only"

    # The error against FP64 on a central window of frame 1 (history from frame 0).
    sys.path.insert(0, str(ROOT / "tests"))
    from gpu_util import download_image
    from oracle import Oracle, max_rel, psnr
    orc = Oracle()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                           flags=flags | L.FLAG_KEEP_INTERMEDIATE, out_format=L.FORMAT_RGBA32F,
                           storage=L.STORAGE_FP16)
    x, y, ww, hh, mg = 2816, 1568, 256, 128, 32
    x0, y0, x1, y1 = x - mg, y - mg, x + ww + mg, y + hh + mg
    with L.Pipeline(ctx, pp) as pipe, torch.cuda.stream(stream):
        pipe.record(sptr, srcs[0], dst, fp)
        torch.cuda.synchronize()
        lvl, var = pipe.temporal_state()
        prev = np.stack([download_image(lvl, "r32f")[y0:y1, x0:x1].astype(np.float64),
                         (download_image(var, "r8")[y0:y1, x0:x1].astype(np.float64) / 255.0) ** 2])
        pipe.record(sptr, srcs[1], dst, fp)
        torch.cuda.synchronize()
        got = out[y:y + hh, x:x + ww].cpu().numpy()
    crop = np.ascontiguousarray(host[1][y0:y1, x0:x1])
    mos64, _ = orc.denoise_temporal(crop, prof, model, 1.0, 0.8, prev=np.ascontiguousarray(prev), s="f64")
    pp0 = L.pipeline_params(x1 - x0, y1 - y0, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                            out_format=L.FORMAT_RGBA32F)
    fp0 = L.frame_params(prof, out_space=L.CS_ACES_AP1, out_space_set=1)
    ref = orc.process(mos64, pp0, fp0, "f64")[mg:mg + hh, mg:mg + ww]
    res["fused_fp16_vs_fp64_window"] = {"max_rel": max_rel(got, ref), "psnr_db": psnr(got, ref),
                                        "window": [x, y, ww, hh]}
    return res


SERVE_STREAMS = ([(1920, 1080, 60.0, "clip")] * 2 + [(3840, 2160, 30.0, "clip")] * 3 +
                 [(5760, 3240, 24.0, "clip")] * 2 + [(6000, 4000, 2.0, "stills")])


def run_serve(ctx, seconds: float = 5.0, frames_per_clip: int = 120) -> dict:
    """The serving workload through the frame server (craw_server_*): 8
    streams - 2 x 1920x1080 at 60 fps, 3 x 3840x2160 at 30, 2 x 5760x3240 at
    24 and one of 6000x4000 stills arriving as a Poisson process at 2/s -
    admitted under a 60 GB budget; clips run temporal 0.8 + NLM 1.0 + RCD +
    ACES AP0 float32 (stills the same without the temporal stage, each
    still being a new scene), from pinned host memory to pinned host
    memory, out as RGB32F (three floats a pixel). Paced: frames are
    submitted at their arrival times for `seconds` (at most
    frames_per_clip per clip); latency is submission to the result in host
    memory. Saturated: every frame of the same schedule submitted at once,
    for the aggregate throughput."""
    import torch
    import libcraw_gb300 as L
    from libcraw_gb300 import workloads as W

    prof = W.make_profile()
    rng = np.random.default_rng(5005)
    movers = [(2.0, 0.5), (8.0, 2.0), (24.0, 10.0)]
    streams = []
    for k, (w, h, rate, kind) in enumerate(SERVE_STREAMS):
        clip = kind == "clip"
        a_dn, b_dn = float(rng.uniform(2.0, 6.0)), float(rng.uniform(20.0, 60.0))
        src = [torch.from_numpy(W.synth_frame(w, h, 50050 + 97 * k + i, frame=i, rects=64, zone_plates=2,
                                              noise_a_dn=a_dn, noise_b_dn=b_dn,
                                              movers=movers if clip else []).view(np.int16)).pin_memory()
               for i in range(4)]
        dst = [torch.empty((h, w, 3), dtype=torch.float32).pin_memory() for _ in range(3)]
        kw = dict(denoise_strength=1.0, noise_override=W.noise_model(a_dn, b_dn))
        if clip:
            kw["denoise_temporal_strength"] = 0.8
        flags = L.FLAG_DENOISE | (L.FLAG_TEMPORAL_DENOISE if clip else 0)
        pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP0, flags=flags,
                               out_format=L.FORMAT_RGB32F)
        if clip:
            times = [i / rate for i in range(min(frames_per_clip, int(seconds * rate)))]
        else:
            times, t = [], float(rng.exponential(1.0 / rate))
            while t < seconds:
                times.append(t)
                t += float(rng.exponential(1.0 / rate))
        streams.append(dict(w=w, h=h, rate=rate, kind=kind, src=src, dst=dst,
                            fp=L.frame_params(prof, **kw), pp=pp, times=times))

    def run(paced: bool) -> dict:
        # Clips carry their frame interval as their deadline (earliest
        # deadline first); stills none.
        # Saturated, the producer meets backpressure: at most 2 frames of a
        # stream wait in the server, a submit beyond that is refused
        # (EAGAIN) and made again after a poll.
        max_queued = 0 if paced else 2
        with L.Server(ctx, L.server_params(hbm_budget=60 << 30, max_inflight=16,
                                           slots_per_stream=2, max_queued=max_queued)) as srv:
            for s in streams:
                dl = 1000.0 / s["rate"] if s["kind"] == "clip" else 0.0
                s["sid"] = srv.open(L.server_stream_params(s["pp"], deadline_ms=dl))
            resident = srv.stats().hbm_resident
            sched = sorted((t, k, i) for k, s in enumerate(streams) for i, t in enumerate(s["times"]))
            res = []
            t0 = time.perf_counter()
            for t, k, i in sched:
                if paced:
                    while time.perf_counter() - t0 < t:
                        res += srv.poll(64, 0)
                        time.sleep(0.0002)
                s = streams[k]
                srcb, dstb = s["src"][i % 4], s["dst"][i % 3]
                while True:
                    try:
                        srv.submit(s["sid"], srcb.data_ptr(), s["w"] * 2, dstb.data_ptr(), s["w"] * 12,
                                   s["fp"], t, (k << 32) | i)
                        break
                    except L.CrawError as e:
                        if e.errno != errno.EAGAIN:
                            raise
                        res += srv.poll(64, 1)
            srv.drain()
            wall = time.perf_counter() - t0
            while True:
                got = srv.poll(256, 0)
                if not got:
                    break
                res += got
            st = srv.stats()
        lat = np.array([r.latency_ms for r in res])
        px = sum(streams[r.user >> 32]["w"] * streams[r.user >> 32]["h"] for r in res)
        out = {"frames": len(res), "failed": int(st.failed), "wall_s": wall, "max_queued": max_queued,
               "submits_refused": int(st.submits_refused),
               "fps": len(res) / wall, "eq_5760x3240_fps": px / (5760 * 3240) / wall,
               "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
               "max_ms": float(lat.max()), "hbm_resident_gb": resident / 1e9,
               "device_ms_mean": float(np.mean([r.device_ms for r in res]))}
        per = {}
        for k, s in enumerate(streams):
            key = f"{s['w']}x{s['h']}@{s['rate']:g}"
            lk = [r.latency_ms for r in res if r.user >> 32 == k]
            per.setdefault(key, []).extend(lk)
        out["per_class"] = {k: {"frames": len(v), "p50_ms": float(np.percentile(v, 50)),
                                "p99_ms": float(np.percentile(v, 99))} for k, v in per.items() if v}
        return out

    paced = run(True)
    saturated = run(False)
    return {"workload": "8 streams: 2x1920x1080@60, 3x3840x2160@30, 2x5760x3240@24 (temporal 0.8 + "
                        "NLM 1.0 + RCD + ACES AP0 f32), 1x6000x4000 stills Poisson 2/s (NLM + RCD + "
                        "AP0); pinned host in, pinned RGB32F out; 60 GB budget; clips' deadline = their frame "
                        "interval",
            "seconds": seconds, "paced": paced, "saturated": saturated,
            "p99_under_60fps_interval": paced["p99_ms"] < 1000.0 / 60}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
