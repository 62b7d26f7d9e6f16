"""Frames developed through whichever build of libcraw.so this process
loaded (CRAW_LIBRARY): the cases the bounds-checked build is run on, from
the reference's minimum sizes to frames whose tiles, strips and segments
end short, over every kernel the checks cover (develop, denoise, chroma,
highlight reconstruction). `python bounds_cases.py
OUT.npz` writes each case's output and the kernel error bits of its
pipeline."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import libcraw_gb300 as L  # noqa: E402
from libcraw_gb300 import workloads as W  # noqa: E402
from gpu_util import develop  # noqa: E402

# (name, w, h, debayer, out space, pipeline flags, frame kwargs, frames)
CASES = [
    ("min_bilinear", 8, 8, L.DEBAYER_BILINEAR, L.CS_BT709, L.FLAG_AWB_HISTOGRAM, {}, 1),
    ("thin_rcd", 1030, 18, L.DEBAYER_RCD, L.CS_ACES_AP1, L.FLAG_AWB_HISTOGRAM, {}, 1),
    ("tall_rcd", 18, 1030, L.DEBAYER_RCD, L.CS_BT709, L.FLAG_AWB_HISTOGRAM, {}, 1),
    ("ref_nlm_rcd_ap1", 256, 160, L.DEBAYER_RCD, L.CS_ACES_AP1, L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM,
     dict(denoise_strength=1.0), 1),
    ("strips_exact", 1000, 700, L.DEBAYER_RCD, L.CS_BT709,
     L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM | L.FLAG_EXACT_ROUNDING, dict(denoise_strength=1.0), 1),
    ("tiles_ap1", 1286, 718, L.DEBAYER_RCD, L.CS_ACES_AP1, L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM,
     dict(denoise_strength=1.0), 1),
    ("temporal_mhc_chroma", 390, 262, L.DEBAYER_MHC, L.CS_P3D65,
     L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE | L.FLAG_CHROMA_DENOISE | L.FLAG_AWB_HISTOGRAM,
     dict(denoise_strength=1.0, denoise_temporal_strength=0.8, denoise_chroma_strength=0.5), 3),
    ("highlights_rcd", 704, 398, L.DEBAYER_RCD, L.CS_BT709,
     L.FLAG_HIGHLIGHT_RECONSTRUCTION | L.FLAG_AWB_HISTOGRAM, dict(flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION), 1),
    ("fp16_keep", 642, 386, L.DEBAYER_RCD, L.CS_BT2020, L.FLAG_AWB_HISTOGRAM | L.FLAG_KEEP_INTERMEDIATE,
     {}, 1),
]


def run_cases() -> dict[str, np.ndarray]:
    """Each case's frames, histogram counts and kernel error bits. The
    denoise shape is fixed (packed 2x4, which every mode has), since the
    autotuner's timing-based pick could differ between two processes."""
    out: dict[str, np.ndarray] = {}
    prof = W.make_profile()
    L.debug_force_denoise_shape(L.DN_SHAPES.index("2x4 f32x2"))
    with L.Context(0) as ctx:
        for name, w, h, deb, cs, flags, kw, nfr in CASES:
            storage = L.STORAGE_FP16 if name.startswith("fp16") else L.STORAGE_FP32
            pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, out_format=L.FORMAT_RGBA32F,
                                   flags=flags, storage=storage)
            fp = L.frame_params(prof, noise_override=W.noise_model(4.0, 40.0), **kw)
            with L.Pipeline(ctx, pp) as pipe:
                for f in range(nfr):
                    m = (W.highlight_frame(w, h, 55 + f) if name.startswith("highlights") else
                         W.synth_frame(w, h, 17 * w + h + f, noise_a_dn=4.0, noise_b_dn=40.0))
                    out[f"{name}/{f}"] = develop(pipe, m, fp)
                out[f"{name}/hist"] = pipe.awb_histogram().count
                out[f"{name}/errors"] = np.array([pipe.kernel_errors()], np.uint32)
    L.debug_force_denoise_shape(-1)
    return out


if __name__ == "__main__":
    np.savez(sys.argv[1], **run_cases())
