"""Seeded synthetic workloads of the benchmark configurations.

Each configuration is a frame (or a sequence, a batch or a set of streams)
of RGGB uint16 mosaics with 12-bit values, black 256 and white 4095, made
by ``_lib/libcraw_synth.so`` from a seed, plus the camera profile and the
frame parameters it is developed with. The profile uses a fixed camera
matrix of this project (rows summing to the XYZ of D65 white) and the
as-shot gains R 2.0, G 1, B 1.5 the scene was divided by. No public
dataset is involved; these stand in for real camera frames.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import (CS_ACES_AP0, CS_ACES_AP1, CS_BT2020, CS_BT709, CS_P3D65, DEBAYER_BILINEAR,
               DEBAYER_MHC, DEBAYER_RCD, FLAG_AWB_HISTOGRAM, FLAG_CHROMA_DENOISE, FLAG_DENOISE,
               FLAG_TEMPORAL_DENOISE, LIB_DIR, Profile, profile_init)

BLACK_DN, WHITE_DN = 256, 4095
WB = (2.0, 1.0, 1.5)
RANGE_DN = WHITE_DN - BLACK_DN
#: Balanced camera RGB -> XYZ (D65); rows sum to (0.9505, 1.0, 1.089).
CAMERA_MATRIX = ((0.6850, 0.1640, 0.1015),
                 (0.2950, 0.7700, -0.0650),
                 (0.0100, 0.0400, 1.0390))


class SynthParams(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("seed", C.c_uint64), ("frame", C.c_uint32),
        ("nb_rects", C.c_uint32), ("nb_zone_plates", C.c_uint32), ("noise_a_dn", C.c_float),
        ("noise_b_dn", C.c_float), ("wb", C.c_float * 3), ("black_dn", C.c_uint32),
        ("white_dn", C.c_uint32), ("nb_movers", C.c_uint32), ("mover_speed", C.c_float * 4),
        ("mover_contrast", C.c_float * 4),
    ]


_synth = None


def _lib():
    global _synth
    if _synth is None:
        path = LIB_DIR / "libcraw_synth.so"
        if not path.exists():
            raise ImportError(f"{path} is missing: run libcraw_gb300.build.build() first")
        _synth = C.CDLL(str(path))
        _synth.craw_synth_frame.restype = C.c_int
        _synth.craw_synth_frame.argtypes = [C.POINTER(SynthParams), C.c_void_p, C.c_size_t]
    return _synth


def synth_frame(width: int, height: int, seed: int, *, frame: int = 0, rects: int = 64,
                zone_plates: int = 1, noise_a_dn: float = 2.0, noise_b_dn: float = 16.0,
                movers: list[tuple[float, float]] | None = None, out: np.ndarray | None = None) -> np.ndarray:
    """One (height, width) uint16 mosaic."""
    p = SynthParams()
    p.width, p.height, p.seed, p.frame = width, height, seed, frame
    p.nb_rects, p.nb_zone_plates = rects, zone_plates
    p.noise_a_dn, p.noise_b_dn = noise_a_dn, noise_b_dn
    for i, g in enumerate(WB):
        p.wb[i] = g
    p.black_dn, p.white_dn = BLACK_DN, WHITE_DN
    movers = movers or []
    p.nb_movers = len(movers)
    for i, (speed, contrast) in enumerate(movers):
        p.mover_speed[i], p.mover_contrast[i] = speed, contrast
    if out is None:
        out = np.empty((height, width), np.uint16)
    assert out.flags.c_contiguous and out.dtype == np.uint16
    ret = _lib().craw_synth_frame(C.byref(p), out.ctypes.data, width)
    if ret < 0:
        raise ValueError(f"craw_synth_frame failed ({ret})")
    return out


def make_profile() -> Profile:
    p = profile_init()
    for s in range(4):
        p.black_level[s] = BLACK_DN / 65535.0
        p.white_level[s] = WHITE_DN / 65535.0
    for c in range(3):
        p.as_shot_wb[c] = WB[c]
        for j in range(3):
            p.as_shot_matrix[c][j] = CAMERA_MATRIX[c][j]
    p.as_shot_cct = 5500.0
    p.gain = 1.0
    p.name = b"craw-gb300 synthetic camera"
    return p


def noise_model(a_dn: float, b_dn: float) -> tuple[float, float]:
    """(a, b) of the pipeline's normalised model for a model in DN."""
    return a_dn / RANGE_DN, b_dn / (RANGE_DN * RANGE_DN)


@dataclass
class Config:
    name: str
    width: int
    height: int
    seed: int
    rects: int
    zone_plates: int
    noise_a_dn: float
    noise_b_dn: float
    debayer: int
    out_space: int
    flags: int
    denoise_strength: float = 0.0
    temporal_strength: float = 0.0
    chroma_strength: float = 0.0
    frames: int = 1
    movers: list = field(default_factory=list)

    def frame(self, i: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        return synth_frame(self.width, self.height, self.seed, frame=i, rects=self.rects,
                           zone_plates=self.zone_plates, noise_a_dn=self.noise_a_dn,
                           noise_b_dn=self.noise_b_dn, movers=self.movers, out=out)

    def frame_kwargs(self) -> dict:
        kw = dict(noise_override=noise_model(self.noise_a_dn, self.noise_b_dn))
        if self.denoise_strength:
            kw["denoise_strength"] = self.denoise_strength
        if self.temporal_strength:
            kw["denoise_temporal_strength"] = self.temporal_strength
        if self.chroma_strength:
            kw["denoise_chroma_strength"] = self.chroma_strength
        return kw


#: The benchmark workloads by name.
WORKLOADS = ("bilinear_bt709_1080p", "nlm_rcd_ap1", "temporal_mhc_p3", "batch_rcd_bt2020",
             "serve_rcd_ap0")


def workload(name: str, width: int | None = None, height: int | None = None) -> Config:
    """Benchmark workload `name` (one of WORKLOADS), optionally at another
    size (the tests run them small)."""
    if name == "bilinear_bt709_1080p":   # bilinear, no denoise, BT.709
        c = Config("1920x1080 bilinear BT.709", 1920, 1080, 1001, 64, 1, 2.0, 16.0,
                   DEBAYER_BILINEAR, CS_BT709, FLAG_AWB_HISTOGRAM)
    elif name == "nlm_rcd_ap1":          # the full chain on one frame
        c = Config("5760x3240 VST+NLM1.0+RCD+AP1+AWB", 5760, 3240, 2002, 256, 4, 4.0, 40.0,
                   DEBAYER_RCD, CS_ACES_AP1, FLAG_AWB_HISTOGRAM | FLAG_DENOISE,
                   denoise_strength=1.0)
    elif name == "temporal_mhc_p3":      # a temporal sequence with movers
        c = Config("5760x3240 x60 temporal0.8+NLM1.0+chroma0.5+MHC+P3", 5760, 3240, 3003, 256, 4,
                   4.0, 40.0, DEBAYER_MHC, CS_P3D65,
                   FLAG_AWB_HISTOGRAM | FLAG_DENOISE | FLAG_TEMPORAL_DENOISE | FLAG_CHROMA_DENOISE,
                   denoise_strength=1.0, temporal_strength=0.8, chroma_strength=0.5, frames=60,
                   movers=[(2.0, 0.5), (8.0, 2.0), (24.0, 10.0)])
    elif name == "batch_rcd_bt2020":     # one frame of the uneven batch
        c = Config("batch NLM1.0+RCD+BT.2020", 5760, 3240, 4004, 256, 4, 4.0, 40.0,
                   DEBAYER_RCD, CS_BT2020, FLAG_AWB_HISTOGRAM | FLAG_DENOISE, denoise_strength=1.0)
    elif name == "serve_rcd_ap0":        # one frame of a served clip
        c = Config("serve temporal0.8+NLM+RCD+AP0", 5760, 3240, 5005, 256, 4, 4.0, 40.0,
                   DEBAYER_RCD, CS_ACES_AP0,
                   FLAG_AWB_HISTOGRAM | FLAG_DENOISE | FLAG_TEMPORAL_DENOISE,
                   denoise_strength=1.0, temporal_strength=0.8)
    else:
        raise ValueError(name)
    if width:
        c.width = width
    if height:
        c.height = height
    return c


@dataclass
class BatchFrame:
    width: int
    height: int
    seed: int
    noise_a_dn: float
    noise_b_dn: float

    def frame(self, out: np.ndarray | None = None) -> np.ndarray:
        return synth_frame(self.width, self.height, self.seed, rects=256, zone_plates=4,
                           noise_a_dn=self.noise_a_dn, noise_b_dn=self.noise_b_dn, out=out)


def batch_mix(scale: int = 1) -> list[BatchFrame]:
    """The batched workload: 6 x 1920x1080, 4 x 3840x2160, 4 x 5760x3240 and
    2 x 6000x4000 frames, independent seeds, noise a ~ U[1, 8] DN and
    b ~ U[10, 80] DN^2 per frame; ``scale`` divides every side (rounded to
    even) for tests."""
    rng = np.random.default_rng(4004)
    sizes = [(1920, 1080)] * 6 + [(3840, 2160)] * 4 + [(5760, 3240)] * 4 + [(6000, 4000)] * 2
    out = []
    for i, (w, h) in enumerate(sizes):
        a, b = float(rng.uniform(1.0, 8.0)), float(rng.uniform(10.0, 80.0))
        out.append(BatchFrame(max(12, w // scale // 2 * 2), max(12, h // scale // 2 * 2),
                              40040 + i, a, b))
    return out



def highlight_frame(width: int, height: int, seed: int, gain: float = 2.5,
                    lamps: int = 3) -> np.ndarray:
    """A synthetic mosaic whose highlights clip: the seeded scene's signal
    above black raised by `gain`, plus `lamps` bright discs, clipped at the
    white level (the input of the highlight reconstruction)."""
    m = synth_frame(width, height, seed, rects=16, zone_plates=1, noise_a_dn=2.0, noise_b_dn=16.0)
    v = (m.astype(np.float32) - BLACK_DN) * gain
    rng = np.random.default_rng(seed + 17)
    yy, xx = np.mgrid[0:height, 0:width]
    for _ in range(lamps):
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        r = rng.uniform(0.03, 0.12) * min(width, height)
        d = np.hypot(xx - cx, yy - cy)
        v += np.clip(1.0 - d / r, 0.0, 1.0) * RANGE_DN * rng.uniform(1.0, 3.0)
    return np.clip(np.rint(v + BLACK_DN), 0, WHITE_DN).astype(np.uint16)


def noise_ramp(width: int, height: int, seed: int, a_dn: float = 4.0, b_dn: float = 40.0,
               lo: float = 0.01, hi: float = 0.95) -> np.ndarray:
    """A mosaic whose signal is a horizontal ramp from `lo` to `hi` of the
    range above black, the same on every site, with Poisson-Gaussian noise
    of variance a_dn * signal + b_dn (12-bit DN), rounded and clipped: a
    frame whose every bin holds nothing but noise (a ramp is locally
    linear, which the estimator's high-pass removes), so the noise-model
    estimate should recover (a_dn, b_dn) / (range, range^2)."""
    rng = np.random.default_rng(seed)
    sig = np.broadcast_to(np.linspace(lo, hi, width) * RANGE_DN, (height, width))
    v = BLACK_DN + sig + rng.standard_normal((height, width)) * np.sqrt(a_dn * sig + b_dn)
    return np.clip(np.rint(v), 0, 65535).astype(np.uint16)
