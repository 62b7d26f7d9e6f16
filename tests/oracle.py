"""ctypes bindings of the CPU oracle (oracle/_build/liboracle.so, float and
double) and of the reference's own CPU code (oracle/_ref/libcraw_ref.so,
present only where the reference tree was available to build it).

Test infrastructure: the oracle, never the thing measured. The structs
are those of libcraw_gb300, byte compatible with the reference's.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

import libcraw_gb300 as L

ROOT = Path(__file__).resolve().parent.parent
ORACLE_SO = ROOT / "oracle" / "_build" / "liboracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libcraw_ref.so"

P = C.POINTER
vp, u32, i32, f32, sz = C.c_void_p, C.c_uint32, C.c_int, C.c_float, C.c_size_t


class GamutParams(C.Structure):
    _fields_ = [("thr", C.c_float * 3), ("scl", C.c_float * 3), ("pwr", C.c_float),
                ("inv_pwr", C.c_float)]


def _sig(lib, name, res, args):
    fn = getattr(lib, name)
    fn.restype, fn.argtypes = res, args
    return fn


def _noise_estimate(fn, bayer, profile, params):
    bayer = np.ascontiguousarray(bayer, np.uint16)
    h, w = bayer.shape
    out = L.NoiseEstimate()
    ret = fn(bayer.ctypes.data, w, h, w, C.byref(profile), None if params is None else C.byref(params),
             C.byref(out))
    return ret, out


class Oracle:
    """The restatement (float: ``f32``, double: ``f64``)."""

    def __init__(self, path: Path = ORACLE_SO):
        self.lib = C.CDLL(str(path))
        lib = self.lib
        for s in ("f32", "f64"):
            _sig(lib, f"orc_process_{s}", i32, [vp, u32, u32, sz, P(L.PipelineParams), P(L.FrameParams), vp])
            _sig(lib, f"orc_denoise_temporal_{s}", i32,
                 [vp, u32, u32, sz, P(L.Profile), P(L.NoiseModel), f32, f32, vp, vp, vp, sz])
            _sig(lib, f"orc_debayer_wb_{s}", i32, [vp, u32, u32, sz, P(L.Profile), P(C.c_float * 3), i32, vp])
            _sig(lib, f"orc_debayer_mosaic_{s}", i32, [vp, u32, u32, i32, vp])
            _sig(lib, f"orc_chroma_denoise_{s}", i32, [vp, u32, u32, f32])
            _sig(lib, f"orc_color_{s}", i32, [vp, u32, u32, P(L.FrameParams), i32])
            _sig(lib, f"orc_highlights_{s}", i32, [vp, u32, u32, sz, P(L.Profile), P(C.c_float * 3), vp])
        _sig(lib, "orc_awb_histogram", i32, [vp, u32, u32, sz, i32, P(C.c_float * 3), vp, vp, vp])
        _sig(lib, "orc_profile_eval", i32, [P(L.Profile), i32, P(L.Illuminant), P(L.ColorParams)])
        _sig(lib, "orc_colorspace_from_xyz_f", i32, [i32, P(C.c_float * 9)])
        _sig(lib, "orc_gamut_params", None, [P(GamutParams)])
        _sig(lib, "orc_noise_model_eval", i32, [P(L.NoiseKnot), u32, f32, P(L.NoiseModel)])
        _sig(lib, "orc_noise_estimate", i32, [vp, u32, u32, sz, P(L.Profile), P(L.NoiseEstimateParams),
                                              P(L.NoiseEstimate)])
        self.prefix = "orc_"

    def noise_estimate(self, bayer, profile, params=None):
        """(return code, estimate) of the restated craw_noise_estimate."""
        return _noise_estimate(self.lib.orc_noise_estimate, bayer, profile, params)

    def _dt(self, s):
        return np.float32 if s == "f32" else np.float64

    def process(self, bayer: np.ndarray, params: L.PipelineParams, fp: L.FrameParams, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w, 4), self._dt(s))
        ret = getattr(self.lib, f"orc_process_{s}")(bayer.ctypes.data, w, h, bayer.strides[0] // 2,
                                                   C.byref(params), C.byref(fp), out.ctypes.data)
        assert ret == 0, ret
        return out

    def denoise_temporal(self, bayer, profile, model, strength, alpha, prev=None, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w), np.uint16)
        nxt = np.zeros((2, h, w), self._dt(s)) if alpha > 0 else None
        ret = getattr(self.lib, f"orc_denoise_temporal_{s}")(
            bayer.ctypes.data, w, h, w, C.byref(profile), C.byref(L.NoiseModel(*model)), strength,
            alpha, None if prev is None else prev.ctypes.data,
            None if nxt is None else nxt.ctypes.data, out.ctypes.data, w)
        assert ret == 0, ret
        return out, nxt

    def debayer_wb(self, bayer, profile, wb, method, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w, 4), self._dt(s))
        ret = getattr(self.lib, f"orc_debayer_wb_{s}")(bayer.ctypes.data, w, h, w, C.byref(profile),
                                                      C.byref((C.c_float * 3)(*wb)), method, out.ctypes.data)
        assert ret == 0, ret
        return out

    def chroma_denoise(self, rgba, strength, s="f32"):
        out = np.ascontiguousarray(rgba, self._dt(s)).copy()
        h, w, _ = out.shape
        ret = getattr(self.lib, f"orc_chroma_denoise_{s}")(out.ctypes.data, w, h, strength)
        assert ret == 0, ret
        return out

    def highlights(self, bayer, profile, wb, s="f32"):
        """The rebuilt, balanced mosaic (values rounded to fp16)."""
        h, w = bayer.shape
        out = np.zeros((h, w), self._dt(s))
        ret = getattr(self.lib, f"orc_highlights_{s}")(bayer.ctypes.data, w, h, bayer.strides[0] // 2,
                                                      C.byref(profile), C.byref((C.c_float * 3)(*wb)),
                                                      out.ctypes.data)
        assert ret == 0, ret
        return out

    def color(self, rgba, fp, out_space, s="f32"):
        out = np.ascontiguousarray(rgba, self._dt(s)).copy()
        h, w, _ = out.shape
        ret = getattr(self.lib, f"orc_color_{s}")(out.ctypes.data, w, h, C.byref(fp), out_space)
        assert ret == 0, ret
        return out

    def awb_histogram(self, rgba: np.ndarray, wb):
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w, ch = rgba.shape
        out = [np.zeros(128 * 128, np.uint32) for _ in range(3)]
        ret = self.lib.orc_awb_histogram(rgba.ctypes.data, w, h, w * ch, ch, C.byref((C.c_float * 3)(*wb)),
                                         *[o.ctypes.data for o in out])
        assert ret == 0, ret
        return tuple(o.reshape(128, 128) for o in out)


class Reference:
    """The reference's lib/ref and host code, compiled from its own sources
    (oracle/build_ref.sh). Same call shapes as :class:`Oracle` (float only)."""

    def __init__(self, path: Path = REF_SO):
        self.lib = C.CDLL(str(path))
        lib = self.lib
        _sig(lib, "craw_ref_process", i32, [vp, u32, u32, sz, P(L.PipelineParams), P(L.FrameParams), vp])
        _sig(lib, "craw_ref_denoise_temporal", i32,
             [vp, u32, u32, sz, P(L.Profile), P(L.NoiseModel), f32, f32, vp, vp, vp, sz])
        _sig(lib, "craw_ref_debayer_wb", i32, [vp, u32, u32, sz, P(L.Profile), P(C.c_float * 3), i32, vp])
        _sig(lib, "craw_ref_chroma_denoise", i32, [vp, u32, u32, f32])
        _sig(lib, "craw_ref_color", i32, [vp, u32, u32, P(L.FrameParams), i32])
        _sig(lib, "craw_awb_histogram_from_rgb", i32, [vp, u32, u32, sz, i32, P(C.c_float * 3), vp, vp, vp])
        _sig(lib, "craw_profile_eval", i32, [P(L.Profile), i32, P(L.Illuminant), P(L.ColorParams)])
        _sig(lib, "craw_colorspace_from_xyz_d65", i32, [i32, P(C.c_float * 9)])
        _sig(lib, "craw_colorspace_to_xyz_d65", i32, [i32, P(C.c_float * 9)])
        _sig(lib, "craw_gamut_compress_params", None, [P(GamutParams)])
        _sig(lib, "craw_noise_model_eval", i32, [P(L.NoiseKnot), u32, f32, P(L.NoiseModel)])
        _sig(lib, "craw_planckian_xy", i32, [f32, P(C.c_float * 2)])
        _sig(lib, "craw_bradford_adaptation", i32, [P(C.c_float * 2), P(C.c_float * 2), P(C.c_float * 9)])

    def process(self, bayer, params, fp, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w, 4), np.float32)
        ret = self.lib.craw_ref_process(bayer.ctypes.data, w, h, bayer.strides[0] // 2, C.byref(params),
                                        C.byref(fp), out.ctypes.data)
        assert ret == 0, ret
        return out

    def denoise_temporal(self, bayer, profile, model, strength, alpha, prev=None, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w), np.uint16)
        nxt = np.zeros((2, h, w), np.float32) if alpha > 0 else None
        ret = self.lib.craw_ref_denoise_temporal(
            bayer.ctypes.data, w, h, w, C.byref(profile), C.byref(L.NoiseModel(*model)), strength, alpha,
            None if prev is None else prev.ctypes.data, None if nxt is None else nxt.ctypes.data,
            out.ctypes.data, w)
        assert ret == 0, ret
        return out, nxt

    def debayer_wb(self, bayer, profile, wb, method, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w, 4), np.float32)
        ret = self.lib.craw_ref_debayer_wb(bayer.ctypes.data, w, h, w, C.byref(profile),
                                           C.byref((C.c_float * 3)(*wb)), method, out.ctypes.data)
        assert ret == 0, ret
        return out

    def chroma_denoise(self, rgba, strength, s="f32"):
        out = np.ascontiguousarray(rgba, np.float32).copy()
        h, w, _ = out.shape
        assert self.lib.craw_ref_chroma_denoise(out.ctypes.data, w, h, strength) == 0
        return out

    def highlights(self, bayer, profile, wb, s="f32"):
        h, w = bayer.shape
        out = np.zeros((h, w), np.float32)
        _sig(self.lib, "craw_ref_highlights", i32, [vp, u32, u32, sz, P(L.Profile), P(C.c_float * 3), vp])
        assert self.lib.craw_ref_highlights(bayer.ctypes.data, w, h, bayer.strides[0] // 2, C.byref(profile),
                                            C.byref((C.c_float * 3)(*wb)), out.ctypes.data) == 0
        return out

    def color(self, rgba, fp, out_space, s="f32"):
        out = np.ascontiguousarray(rgba, np.float32).copy()
        h, w, _ = out.shape
        assert self.lib.craw_ref_color(out.ctypes.data, w, h, C.byref(fp), out_space) == 0
        return out

    def noise_estimate(self, bayer, profile, params=None):
        _sig(self.lib, "craw_noise_estimate", i32, [vp, u32, u32, sz, P(L.Profile), P(L.NoiseEstimateParams),
                                                    P(L.NoiseEstimate)])
        return _noise_estimate(self.lib.craw_noise_estimate, bayer, profile, params)

    def awb_histogram(self, rgba, wb):
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w, ch = rgba.shape
        out = [np.zeros(128 * 128, np.uint32) for _ in range(3)]
        assert self.lib.craw_awb_histogram_from_rgb(rgba.ctypes.data, w, h, w * ch, ch,
                                                    C.byref((C.c_float * 3)(*wb)),
                                                    *[o.ctypes.data for o in out]) == 0
        return tuple(o.reshape(128, 128) for o in out)


def reference_available() -> bool:
    return REF_SO.exists()


# --------------------------------------------------------------- metrics

def max_abs(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.max(np.abs(a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64))))


def max_rel(test: np.ndarray, ref: np.ndarray) -> float:
    """Largest error relative to the pixel's magnitude (the largest of its
    three components), the scale floored at 1% of the frame's peak: the
    metric of reference tests/test_pipeline.c:321-359."""
    t = test[..., :3].astype(np.float64)
    r = ref[..., :3].astype(np.float64)
    a = np.abs(r)
    floor = max(1e-9, 0.01 * float(a.max()))
    scale = np.maximum(a.max(axis=-1, keepdims=True), floor)
    return float(np.max(np.abs(t - r) / scale))


def rel_map(test: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """The per-pixel error of max_rel()."""
    t = test[..., :3].astype(np.float64)
    r = ref[..., :3].astype(np.float64)
    a = np.abs(r)
    floor = max(1e-9, 0.01 * float(a.max()))
    scale = np.maximum(a.max(axis=-1), floor)
    return np.abs(t - r).max(axis=-1) / scale


def denoised_chain_ok(test: np.ndarray, ref: np.ndarray) -> tuple[bool, dict]:
    """The bound for a chain that includes the denoise. Its output mosaic
    is re-encoded to 16-bit codes (reference lib/ref/ref_denoise.c:318-323),
    so any two float evaluations differ by one code at the samples whose
    value lies within rounding of a code boundary -- the reference's own
    float code does against its double run (tests/test_oracle_pin.py) --
    and a one-code step is up to ~1e-2 of a dark pixel. Bound: max_rel
    under 1.5e-2, at most 0.1% of pixels above 1e-3, PSNR above 80 dB."""
    r = rel_map(test, ref)
    st = {"max_rel": float(r.max()), "frac_over_1e-3": float((r > 1e-3).mean()),
          "psnr": psnr(test, ref)}
    return (st["max_rel"] < 1.5e-2 and st["frac_over_1e-3"] < 1e-3 and st["psnr"] > 80), st


def psnr(test: np.ndarray, ref: np.ndarray) -> float:
    t = test[..., :3].astype(np.float64)
    r = ref[..., :3].astype(np.float64)
    mse = float(np.mean((t - r) ** 2))
    peak = float(np.abs(r).max())
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def hist_nonlocal(gpu: np.ndarray, ref: np.ndarray) -> int:
    """Samples in a bin not adjacent to the reference's (reference
    tests/test_pipeline.c:370-407): each +1 is cancelled against a -1 in
    one of its eight neighbours, and what is left is counted."""
    n = gpu.shape[0]
    d = gpu.astype(np.int64) - ref.astype(np.int64)
    for y in range(n):
        for x in range(n):
            if d[y, x] <= 0:
                continue
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if d[y, x] <= 0:
                        break
                    ny, nx = y + dy, x + dx
                    if 0 <= ny < n and 0 <= nx < n and d[ny, nx] < 0:
                        t = min(d[y, x], -d[ny, nx])
                        d[y, x] -= t
                        d[ny, nx] += t
    return int(np.abs(d).sum() // 2)
