"""Command-line front end, modelled on the reference's `cineraw` tool
(tools/cineraw.c): develop a raw mosaic dump to a PFM image, time the
pipeline on frames of a given size (`cineraw --bench`, tools/cineraw.c:
1217-1290), and write synthetic mosaic dumps.

    python -m libcraw_gb300.cli develop IN.raw OUT.pfm --width W --height H [options]
    python -m libcraw_gb300.cli bench --width W --height H [--frames N] [options]
    python -m libcraw_gb300.cli synth OUT.raw --width W --height H [--seed S]
    python -m libcraw_gb300.cli noise --width W --height H [--input IN.raw] [--frames N]

Options include the stages (--denoise, --temporal, --chroma strengths,
--highlights) and, for synthetic frames, --scene highlights: the scene at
2.5x exposure under three lamps, a third of its sites near the clip.

A mosaic dump is W x H native-endian uint16 samples, rows top to bottom,
no header (the reference's test frames, tests/test_pipeline.c:5519-5562).
A PFM file is "PF\\n<w> <h>\\n-1.0\\n" followed by little-endian float32
RGB rows bottom to top (tools/cineraw.c:532-568). The camera is described
by --black, --white and --wb (the defaults are the synthetic camera of the
benchmarks); every frame goes through craw_pipeline_record() on the GPU.
"""
from __future__ import annotations

import argparse
import statistics
import sys
import time
from pathlib import Path

import numpy as np

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W

DEBAYERS = {"bilinear": L.DEBAYER_BILINEAR, "mhc": L.DEBAYER_MHC, "rcd": L.DEBAYER_RCD}
SPACES = {"xyz": L.CS_XYZ_D65, "bt709": L.CS_BT709, "bt2020": L.CS_BT2020, "p3": L.CS_P3D65,
          "vgamut": L.CS_V_GAMUT, "ap0": L.CS_ACES_AP0, "ap1": L.CS_ACES_AP1}


def read_raw(path: str | Path, width: int, height: int) -> np.ndarray:
    """A W x H uint16 mosaic dump."""
    data = np.fromfile(path, dtype=np.uint16)
    if data.size != width * height:
        raise ValueError(f"{path}: {data.size} samples, not a {width}x{height} uint16 frame")
    return data.reshape(height, width)


def write_pfm(path: str | Path, rgba: np.ndarray) -> None:
    """RGB of an (h, w, 3 or 4) float image as a little-endian PFM."""
    h, w = rgba.shape[:2]
    rows = np.ascontiguousarray(rgba[::-1, :, :3], dtype="<f4")
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode("ascii"))
        f.write(rows.tobytes())


def read_pfm(path: str | Path) -> np.ndarray:
    """A PFM as an (h, w, 3) float32 image, top row first."""
    with open(path, "rb") as f:
        kind = f.readline().strip()
        if kind not in (b"PF", b"Pf"):
            raise ValueError(f"{path}: not a PFM file")
        w, h = (int(v) for v in f.readline().split())
        scale = float(f.readline())
        ch = 3 if kind == b"PF" else 1
        data = np.frombuffer(f.read(w * h * ch * 4), dtype="<f4" if scale < 0 else ">f4")
    return data.reshape(h, w, ch)[::-1].astype(np.float32)


def camera(args) -> L.Profile:
    p = W.make_profile()
    for s in range(4):
        p.black_level[s] = args.black / 65535.0
        p.white_level[s] = args.white / 65535.0
    for c in range(3):
        p.as_shot_wb[c] = args.wb[c]
    return p


def params(args, width: int, height: int) -> tuple[L.PipelineParams, L.FrameParams, L.Profile]:
    prof = camera(args)
    flags = L.FLAG_PROFILE
    kw = {"exposure_stops": args.exposure}
    if args.denoise > 0:
        flags |= L.FLAG_DENOISE
        kw["denoise_strength"] = args.denoise
    if args.temporal > 0:
        flags |= L.FLAG_TEMPORAL_DENOISE
        kw["denoise_temporal_strength"] = args.temporal
    if args.chroma > 0:
        flags |= L.FLAG_CHROMA_DENOISE
        kw["denoise_chroma_strength"] = args.chroma
    if args.denoise > 0 or args.temporal > 0:
        rng = args.white - args.black
        kw["noise_override"] = (args.noise[0] / rng, args.noise[1] / (rng * rng))
    if args.highlights:
        flags |= L.FLAG_HIGHLIGHT_RECONSTRUCTION
        kw["flags"] = L.FRAME_HIGHLIGHT_RECONSTRUCTION
    pp = L.pipeline_params(width, height, debayer=DEBAYERS[args.debayer], out_space=SPACES[args.space],
                           flags=flags, out_format=L.FORMAT_RGBA32F,
                           storage=L.STORAGE_FP16 if args.fp16 else L.STORAGE_FP32)
    return pp, L.frame_params(prof, **kw), prof


def develop_frames(frames: list[np.ndarray], args, stream=None):
    """Develops mosaics through one pipeline; yields (RGBA float32, stage
    times) per frame."""
    import torch

    h, w = frames[0].shape
    pp, fp, prof = params(args, w, h)
    ctx = L.Context(args.device)
    try:
        with L.Pipeline(ctx, pp) as pipe:
            s = stream or torch.cuda.Stream(device=args.device)
            out = torch.empty((h, w, 4), dtype=torch.float32, device=f"cuda:{args.device}")
            dst = L.Image(out.data_ptr(), w * 16, L.FORMAT_RGBA32F, w, h)
            for m in frames:
                t = torch.from_numpy(np.ascontiguousarray(m).view(np.int16)).to(f"cuda:{args.device}")
                src = L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h)
                pipe.record(s.cuda_stream, src, dst, fp)
                s.synchronize()
                yield out.cpu().numpy(), pipe.stage_times()
    finally:
        ctx.close()


def cmd_develop(args) -> int:
    m = read_raw(args.input, args.width, args.height)
    for rgba, stages in develop_frames([m], args):
        write_pfm(args.output, rgba)
        print(" ".join(f"{n} {ms:.3f} ms" for n, _, ms in stages))
    return 0


def cmd_bench(args) -> int:
    """Develops `frames` frames (a dump cycled, or seeded synthetic frames)
    and prints the frame rate and the per-stage device time, as
    `cineraw --bench` does."""
    import torch

    if args.input:
        src = [read_raw(args.input, args.width, args.height)]
    else:
        src = [scene(args, 4242 + i) for i in range(4)]
    h, w = src[0].shape
    pp, fp, _ = params(args, w, h)
    ctx = L.Context(args.device)
    try:
        dev = [torch.from_numpy(m.view(np.int16)).to(f"cuda:{args.device}") for m in src]
        srcs = [L.Image(t.data_ptr(), w * 2, L.FORMAT_R16_UNORM, w, h) for t in dev]
        out = torch.empty((h, w, 4), dtype=torch.float32, device=f"cuda:{args.device}")
        dst = L.Image(out.data_ptr(), w * 16, L.FORMAT_RGBA32F, w, h)
        s = torch.cuda.Stream(device=args.device)
        stages: dict[str, list[float]] = {}
        with L.Pipeline(ctx, pp) as pipe:
            for i in range(3):
                pipe.record(s.cuda_stream, srcs[i % len(srcs)], dst, fp)
            s.synchronize()
            t0 = time.perf_counter()
            for i in range(args.frames):
                pipe.record(s.cuda_stream, srcs[i % len(srcs)], dst, fp)
                s.synchronize()
                for n, _, ms in pipe.stage_times():
                    stages.setdefault(n, []).append(ms)
            wall = time.perf_counter() - t0
    finally:
        ctx.close()
    print(f"{w}x{h}: {args.frames} frames in {wall:.3f} s, {args.frames / wall:.1f} frames/s "
          "(each frame waited for)")
    for n, v in stages.items():
        print(f"  {n:18s} {statistics.mean(v):8.3f} ms  (min {min(v):.3f})")
    return 0


def scene(args, seed: int) -> np.ndarray:
    """A seeded synthetic mosaic: the benchmark scene, or with --scene
    highlights the scene at 2.5x exposure under three lamps (a third of
    the sites near or at the clip)."""
    if args.scene == "highlights":
        return W.highlight_frame(args.width, args.height, seed)
    return W.synth_frame(args.width, args.height, seed, noise_a_dn=args.noise[0], noise_b_dn=args.noise[1])


def cmd_noise(args) -> int:
    """Fits the noise model of each frame (`cineraw --noise-estimate`,
    tools/cineraw.c:2705-2730): a dump, or seeded synthetic frames, with
    the time of each estimate."""
    prof = camera(args)
    params = L.noise_estimate_params()
    if args.bins:
        params.nb_bins = args.bins
    if args.min_samples:
        params.min_bin_samples = args.min_samples
    frames = ([read_raw(args.input, args.width, args.height)] if args.input else
              [scene(args, 4242 + i) for i in range(args.frames)])
    for i, m in enumerate(frames):
        t0 = time.perf_counter()
        try:
            est = L.noise_estimate(m, prof, params)
        except L.CrawError as e:
            if e.code == -61:
                print(f"frame {i:5d}: too few levels in this frame to fit anything", file=sys.stderr)
                return 1
            raise
        ms = 1e3 * (time.perf_counter() - t0)
        print(f"frame {i:5d}: a {est.model.a:.4e} b {est.model.b:.4e}   {est.nb_bins} bins, "
              f"{est.nb_inliers} fitted, fit error {100 * est.fit_rms:.1f}%, read noise "
              f"{est.read_noise_lsb:.2f} code values  ({ms:.2f} ms)")
    return 0


def cmd_synth(args) -> int:
    scene(args, args.seed).astype(np.uint16).tofile(args.output)
    return 0


def parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="python -m libcraw_gb300.cli", description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)

    def common(p, need_io=True):
        p.add_argument("--width", type=int, required=True)
        p.add_argument("--height", type=int, required=True)
        p.add_argument("--noise", type=float, nargs=2, default=(4.0, 40.0), metavar=("A_DN", "B_DN"),
                       help="noise model var = a*signal + b in DN (synthesis and the denoise)")
        p.add_argument("--scene", choices=("plain", "highlights"), default="plain",
                       help="synthetic frames: the benchmark scene, or one whose highlights clip")
        if not need_io:
            return
        p.add_argument("--device", type=int, default=0)
        p.add_argument("--debayer", choices=sorted(DEBAYERS), default="rcd")
        p.add_argument("--space", choices=sorted(SPACES), default="ap1")
        p.add_argument("--denoise", type=float, default=0.0, help="NLM strength (0: off)")
        p.add_argument("--temporal", type=float, default=0.0, help="temporal strength (0: off)")
        p.add_argument("--chroma", type=float, default=0.0, help="chroma denoise strength (0: off)")
        p.add_argument("--exposure", type=float, default=0.0, help="stops")
        p.add_argument("--fp16", action="store_true", help="FP16 intermediate storage")
        p.add_argument("--highlights", action="store_true",
                       help="rebuild clipped highlights before the debayer")
        p.add_argument("--black", type=float, default=W.BLACK_DN, help="black level, 16-bit code")
        p.add_argument("--white", type=float, default=W.WHITE_DN, help="white level, 16-bit code")
        p.add_argument("--wb", type=float, nargs=3, default=W.WB, metavar=("R", "G", "B"),
                       help="as-shot white balance gains")

    p = sub.add_parser("develop", help="develop a mosaic dump to a PFM image")
    p.add_argument("input")
    p.add_argument("output")
    common(p)
    p.set_defaults(fn=cmd_develop)
    p = sub.add_parser("bench", help="frames/s and per-stage times")
    p.add_argument("--input", default=None, help="a mosaic dump (default: synthetic frames)")
    p.add_argument("--frames", type=int, default=30)
    common(p)
    p.set_defaults(fn=cmd_bench)
    p = sub.add_parser("synth", help="write a synthetic mosaic dump")
    p.add_argument("output")
    p.add_argument("--seed", type=int, default=1)
    common(p, need_io=False)
    p.set_defaults(fn=cmd_synth)
    p = sub.add_parser("noise", help="fit the sensor noise model of frames (on the GPU)")
    p.add_argument("--input", default=None, help="a mosaic dump (default: synthetic frames)")
    p.add_argument("--frames", type=int, default=3, help="synthetic frames to fit")
    p.add_argument("--bins", type=int, default=0, help="intensity bins (0: 128)")
    p.add_argument("--min-samples", type=int, default=0, help="samples a bin needs (0: 20000)")
    common(p)
    p.set_defaults(fn=cmd_noise)
    return ap


def main(argv: list[str] | None = None) -> int:
    args = parser().parse_args(argv)
    return args.fn(args)


if __name__ == "__main__":
    sys.exit(main())
