"""craw-gb300: libcraw's frame-development path on one NVIDIA GB300.

This module is the Python host mirror of the ``craw_*`` C ABI
(``include/craw/*.h``) that ``_lib/libcraw.so`` exports: the same structs
(byte compatible, checked at import), the same functions, the same
negative-errno error behaviour (raised here as :class:`CrawError`). It is
plumbing over the C library; every frame goes through the sm_103a kernels
in ``libcraw.so`` and there is no other implementation to fall back to.

The reference's entry points and what replaces them (reference files):

====================================  =====================================
reference (include/craw/*.h)          here
====================================  =====================================
craw_context_create(VkDevice ...)     :class:`Context` (CUDA device ordinal)
craw_pipeline_create                  :class:`Pipeline`
craw_pipeline_record(VkCommandBuffer) :meth:`Pipeline.record` (cudaStream_t)
craw_pipeline_get_awb_histogram[_n]   :meth:`Pipeline.awb_histogram`
craw_pipeline_get_stage_times[_n]     :meth:`Pipeline.stage_times`
craw_profile_eval / colorspace ...    module functions of the same names
====================================  =====================================
"""
from __future__ import annotations

import ctypes as C
import errno as _errno
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_DIR = _HERE / "_lib"

# --------------------------------------------------------------- constants

CFA_RGGB = 0
DEBAYER_BILINEAR, DEBAYER_MHC, DEBAYER_RCD = 0, 1, 2
(CS_XYZ_D65, CS_BT709, CS_BT2020, CS_P3D65, CS_V_GAMUT, CS_ACES_AP0,
 CS_ACES_AP1) = range(7)
FORMAT_R16_UNORM, FORMAT_RGBA16F, FORMAT_RGBA32F = 70, 97, 109
FORMAT_R16F = 76
#: Three floats a pixel, no alpha (an extension of this library).
FORMAT_RGB32F = 106
WB_AS_SHOT, WB_REBALANCE = 0, 1
STORAGE_FP32, STORAGE_FP16 = 0, 1
IMPL_FUSED, IMPL_PLAIN = 0, 1

FLAG_AWB_HISTOGRAM = 1 << 0
FLAG_DENOISE = 1 << 1
FLAG_LENS = 1 << 2
FLAG_FALSE_COLOR = 1 << 3
FLAG_CHROMA_DENOISE = 1 << 4
FLAG_HIGHLIGHT_RECONSTRUCTION = 1 << 5
FLAG_DEFRINGE = 1 << 6
FLAG_TEMPORAL_DENOISE = 1 << 7
FLAG_SHARPEN = 1 << 8
FLAG_PROFILE = 1 << 9
FLAG_KEEP_INTERMEDIATE = 1 << 16
FLAG_NO_AUTOTUNE = 1 << 17
FLAG_EXACT_ROUNDING = 1 << 18
BATCH_FLAG_UNFUSED = 1 << 20
BATCH_FLAG_NO_GRAPH = 1 << 21
BATCH_FLAG_FUSED = 1 << 22

FRAME_CLAMP_NEGATIVE = 1 << 0
FRAME_NO_GAMUT_COMPRESSION = 1 << 2
FRAME_HIGHLIGHT_RECONSTRUCTION = 1 << 3
FRAME_TEMPORAL_RESET = 1 << 4

AWB_BINS = 128
AWB_NOALLOC_MAX_BLOCKS = 1 << 18
PROFILE_SLOTS = 4

# ----------------------------------------------------------------- structs


class WbKnot(C.Structure):
    _fields_ = [("cct", C.c_float), ("wb", C.c_float * 3)]


class MatrixKnot(C.Structure):
    _fields_ = [("cct", C.c_float), ("m", (C.c_float * 3) * 3)]


class NoiseKnot(C.Structure):
    _fields_ = [("iso", C.c_float), ("a", C.c_float), ("b", C.c_float)]


class NoiseModel(C.Structure):
    _fields_ = [("a", C.c_float), ("b", C.c_float)]


class NoiseEstimateParams(C.Structure):
    _fields_ = [("nb_bins", C.c_uint32), ("min_bin_samples", C.c_uint32), ("max_level", C.c_float),
                ("padding", C.c_uint8 * 52)]


class NoiseEstimate(C.Structure):
    _fields_ = [("model", NoiseModel), ("nb_bins", C.c_uint32), ("nb_inliers", C.c_uint32),
                ("fit_rms", C.c_float), ("read_noise_lsb", C.c_float), ("padding", C.c_uint8 * 40)]

    def as_tuple(self):
        return (self.model.a, self.model.b, self.nb_bins, self.nb_inliers, self.fit_rms,
                self.read_noise_lsb)


class Illuminant(C.Structure):
    _fields_ = [("cct", C.c_float), ("tint", C.c_float)]


class Profile(C.Structure):
    _fields_ = [
        ("cfa", C.c_int),
        ("black_level", C.c_float * 4),
        ("white_level", C.c_float * 4),
        ("as_shot_wb", C.c_float * 3),
        ("as_shot_matrix", (C.c_float * 3) * 3),
        ("as_shot_cct", C.c_float),
        ("gain", C.c_float),
        ("as_shot_ei", C.c_float),
        ("exposure_index", C.c_float),
        ("wb_knots", WbKnot * 16),
        ("nb_wb_knots", C.c_uint32),
        ("matrix_knots", MatrixKnot * 16),
        ("nb_matrix_knots", C.c_uint32),
        ("name", C.c_char * 64),
        ("noise_knots", NoiseKnot * 16),
        ("nb_noise_knots", C.c_uint32),
    ]


class ColorParams(C.Structure):
    _fields_ = [("wb", C.c_float * 3), ("cam_to_xyz", (C.c_float * 3) * 3), ("gain", C.c_float)]


class LensCorrection(C.Structure):
    _fields_ = [("k", (C.c_float * 4) * 3), ("centre", C.c_float * 2), ("valid", C.c_bool),
                ("reserved", C.c_uint8 * 7)]


class FrameParams(C.Structure):
    _fields_ = [
        ("profile", C.POINTER(Profile)),
        ("wb_mode", C.c_int),
        ("illuminant", Illuminant),
        ("exposure_stops", C.c_float),
        ("flags", C.c_uint32),
        ("out_space", C.c_int),
        ("out_space_set", C.c_bool),
        ("denoise_strength", C.c_float),
        ("noise_override", NoiseModel),
        ("false_color_passes", C.c_uint32),
        ("denoise_chroma_strength", C.c_float),
        ("lens", LensCorrection),
        ("defringe_strength", C.c_float),
        ("denoise_temporal_strength", C.c_float),
        ("denoise_temporal_replay", C.c_bool),
        ("sharpen_radius", C.c_float),
        ("sharpen_iterations", C.c_uint32),
        ("sharpen_contrast", C.c_float),
        ("rotation", C.c_float),
        ("padding", C.c_uint8 * 112),
    ]


class PipelineParams(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("cfa", C.c_int), ("debayer", C.c_int),
        ("out_space", C.c_int), ("out_format", C.c_int), ("flags", C.c_uint32),
        ("nb_awb_slots", C.c_uint32), ("storage", C.c_int), ("impl", C.c_int),
        ("padding", C.c_uint8 * 216),
    ]


class CudaInitParams(C.Structure):
    _fields_ = [("device", C.c_int), ("mem_pool", C.c_void_p), ("padding", C.c_uint8 * 48)]


LOG_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_char_p, C.c_void_p)


class ContextOptions(C.Structure):
    _fields_ = [("log_opaque", C.c_void_p), ("log_cb", C.c_void_p), ("log_level", C.c_int),
                ("padding", C.c_uint8 * 1004)]


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("pitch", C.c_size_t), ("format", C.c_int),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class AwbHistogramC(C.Structure):
    _fields_ = [("bins", C.c_uint32), ("log_min", C.c_float), ("log_max", C.c_float),
                ("count", C.POINTER(C.c_uint32)), ("weight", C.POINTER(C.c_uint32)),
                ("weight_bright", C.POINTER(C.c_uint32))]


class StageTime(C.Structure):
    _fields_ = [("name", C.c_char_p), ("count", C.c_uint32), ("ms", C.c_double)]


class AwbParams(C.Structure):
    _fields_ = [("band", C.c_float), ("sigma", C.c_float), ("min_zone_fraction", C.c_float),
                ("ambience", C.c_float), ("ambience_knee_cct", C.c_float), ("cct_min", C.c_float),
                ("cct_max", C.c_float), ("prefer_bright", C.c_bool),
                ("bright_max_spread_mired", C.c_float)]


class AwbCandidate(C.Structure):
    _fields_ = [("valid", C.c_bool), ("illuminant", Illuminant), ("in_zone_fraction", C.c_float),
                ("spread_mired", C.c_float)]


class AwbEstimate(C.Structure):
    _fields_ = [("valid", C.c_bool), ("illuminant", Illuminant), ("confidence", C.c_float),
                ("in_zone_fraction", C.c_float), ("spread_mired", C.c_float), ("source", C.c_int),
                ("zone", AwbCandidate), ("bright", AwbCandidate)]


class AwbSmootherParams(C.Structure):
    _fields_ = [("time_constant", C.c_float), ("hysteresis_mired", C.c_float),
                ("max_slew_mired_per_s", C.c_float), ("min_confidence", C.c_float)]


class ServerParams(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_inflight", C.c_uint32),
                ("slots_per_stream", C.c_uint32), ("idle_timeout_ms", C.c_uint32),
                ("max_queued", C.c_uint32), ("padding", C.c_uint8 * 40)]


class ServerStreamParams(C.Structure):
    _fields_ = [("pipeline", PipelineParams), ("flags", C.c_uint32), ("awb", AwbParams),
                ("smoother", AwbSmootherParams), ("deadline_ms", C.c_float), ("padding", C.c_uint8 * 60)]


class ServerResult(C.Structure):
    _fields_ = [("user", C.c_uint64), ("stream", C.c_uint32), ("status", C.c_int),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double), ("device_ms", C.c_double),
                ("awb_valid", C.c_bool), ("awb", Illuminant), ("estimate", AwbEstimate),
                ("noise_valid", C.c_bool), ("noise", NoiseEstimate)]


class ServerStats(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("hbm_resident", C.c_uint64), ("streams", C.c_uint32),
                ("queued", C.c_uint32), ("inflight", C.c_uint32), ("submitted", C.c_uint64),
                ("completed", C.c_uint64), ("failed", C.c_uint64), ("streams_admitted", C.c_uint64),
                ("streams_refused", C.c_uint64), ("streams_reclaimed", C.c_uint64),
                ("submits_refused", C.c_uint64)]


SERVER_STREAM_AUTO_WB = 1 << 0
SERVER_STREAM_ESTIMATE_NOISE = 1 << 1


class BatchParams(C.Structure):
    _fields_ = [("max_frames", C.c_uint32), ("max_width", C.c_uint32), ("max_height", C.c_uint32),
                ("debayer", C.c_int), ("out_space", C.c_int), ("out_format", C.c_int),
                ("flags", C.c_uint32), ("direct_pixels", C.c_uint32), ("padding", C.c_uint8 * 32)]


#: Frames of a batch with at least this many pixels go to the single-frame
#: kernels (BatchParams.direct_pixels = 0); BATCH_ALL_PERSISTENT keeps every
#: frame in the persistent launch.
BATCH_DIRECT_PIXELS = 4000000
BATCH_ALL_PERSISTENT = 0xFFFFFFFF


class BatchInfo(C.Structure):
    _fields_ = [("denoise_shape", C.c_int), ("fused", C.c_int), ("graph", C.c_int),
                ("captures", C.c_uint64), ("replays", C.c_uint64), ("direct_shape", C.c_int),
                ("direct_frames", C.c_uint64)]


for _s, _n in ((Profile, 1264), (FrameParams, 264), (PipelineParams, 256), (CudaInitParams, 64),
               (ContextOptions, 1024), (LensCorrection, 64), (BatchParams, 64), (AwbParams, 36),
               (AwbCandidate, 20), (AwbEstimate, 68), (AwbSmootherParams, 16), (ServerParams, 64),
               (ServerStreamParams, 376), (ServerResult, 192), (NoiseEstimateParams, 64),
               (NoiseEstimate, 64)):
    assert C.sizeof(_s) == _n, (_s.__name__, C.sizeof(_s), _n)

# ----------------------------------------------------------------- library

#: Every symbol the C ABI exports (include/craw/*.h).
EXPORTS = (
    "craw_version_int", "craw_log", "craw_context_create", "craw_context_free",
    "craw_cuda_check_device", "craw_debug_fail_alloc", "craw_debug_force_denoise_shape",
    "craw_debug_rcd_tma", "craw_debug_rcd_strips", "craw_debug_denoise_tma", "craw_debug_kernel_errors", "craw_debug_denoise_round",
    "craw_debug_denoise_round_decide", "craw_debug_denoise_round_stats",
    "craw_pipeline_params_init", "craw_frame_params_init", "craw_pipeline_create",
    "craw_pipeline_free", "craw_pipeline_record", "craw_pipeline_get_awb_histogram",
    "craw_pipeline_get_awb_histogram_n", "craw_pipeline_get_stage_times",
    "craw_pipeline_get_stage_times_n", "craw_pipeline_get_intermediate",
    "craw_pipeline_get_temporal_state", "craw_pipeline_get_kernel_config",
    "craw_profile_init", "craw_profile_validate", "craw_profile_eval",
    "craw_profile_noise_eval", "craw_noise_model_eval", "craw_colorspace_from_xyz_d65",
    "craw_colorspace_to_xyz_d65", "craw_planckian_xy", "craw_bradford_adaptation",
    "craw_awb_histogram_from_rgb",
    "craw_batch_params_init", "craw_batch_create", "craw_batch_record", "craw_batch_get_info",
    "craw_batch_free", "craw_awb_histogram_from_rgb_cuda_noalloc",
    "craw_profile_neutral_to_illuminant", "craw_profile_illuminant_to_neutral",
    "craw_awb_params_init", "craw_awb_estimate", "craw_awb_smoother_params_init",
    "craw_awb_smoother_create", "craw_awb_smoother_free", "craw_awb_smoother_reset",
    "craw_awb_smoother_set", "craw_awb_smoother_push",
    "craw_server_params_init", "craw_server_stream_params_init", "craw_server_create",
    "craw_server_free", "craw_server_stream_open", "craw_server_stream_close",
    "craw_server_submit", "craw_server_poll", "craw_server_drain", "craw_server_get_stats",
    "craw_noise_estimate_params_init", "craw_noise_estimate", "craw_noise_estimate_cuda",
)


class CrawError(RuntimeError):
    """A negative errno returned by the C library."""

    def __init__(self, code: int, what: str = ""):
        self.code = code
        self.errno = -code
        name = _errno.errorcode.get(-code, str(-code))
        super().__init__(f"{what or 'craw'} failed: {name} ({code})")


def _check(ret: int, what: str) -> int:
    if ret < 0:
        raise CrawError(ret, what)
    return ret


_lib = None


def awb_signatures() -> dict:
    """ctypes signatures of the locus, AWB estimator and smoother functions
    (the same in the reference's build, which the tests load beside)."""
    vp, i32, f32, f64 = C.c_void_p, C.c_int, C.c_float, C.c_double
    return {
        "craw_profile_neutral_to_illuminant": (i32, [C.POINTER(Profile), f32, f32, C.POINTER(Illuminant)]),
        "craw_profile_illuminant_to_neutral": (i32, [C.POINTER(Profile), C.POINTER(Illuminant),
                                                     C.POINTER(f32), C.POINTER(f32)]),
        "craw_awb_params_init": (None, [C.POINTER(AwbParams)]),
        "craw_awb_estimate": (i32, [C.POINTER(Profile), C.POINTER(AwbHistogramC), C.POINTER(AwbParams),
                                    C.POINTER(AwbEstimate)]),
        "craw_awb_smoother_params_init": (None, [C.POINTER(AwbSmootherParams)]),
        "craw_awb_smoother_create": (i32, [C.POINTER(AwbSmootherParams), C.POINTER(vp)]),
        "craw_awb_smoother_free": (None, [C.POINTER(vp)]),
        "craw_awb_smoother_reset": (None, [vp]),
        "craw_awb_smoother_set": (None, [vp, f64, C.POINTER(Illuminant)]),
        "craw_awb_smoother_push": (i32, [vp, f64, C.POINTER(AwbEstimate), C.c_bool, C.POINTER(Illuminant)]),
    }


def lib() -> C.CDLL:
    """Loads ``_lib/libcraw.so`` (built by ``libcraw_gb300.build``); raises if
    it is missing: there is no fallback implementation. ``CRAW_LIBRARY``
    names another build of the same library to load instead (the
    bounds-checked ``_lib/libcraw_bounds.so``)."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ["CRAW_LIBRARY"]) if os.environ.get("CRAW_LIBRARY") else LIB_DIR / "libcraw.so"
    if not path.exists():
        raise ImportError(f"{path} is missing: run libcraw_gb300.build.build() first")
    L = C.CDLL(str(path))
    vp, u32, i32, f32 = C.c_void_p, C.c_uint32, C.c_int, C.c_float
    sig = {
        "craw_version_int": (u32, []),
        "craw_context_create": (i32, [C.POINTER(vp), C.POINTER(CudaInitParams), C.POINTER(ContextOptions)]),
        "craw_context_free": (None, [C.POINTER(vp)]),
        "craw_cuda_check_device": (i32, [i32, C.POINTER(C.c_char_p)]),
        "craw_debug_fail_alloc": (None, [i32]),
        "craw_debug_force_denoise_shape": (i32, [i32]),
        "craw_debug_rcd_tma": (i32, [i32]),
        "craw_debug_rcd_strips": (i32, [i32]),
        "craw_debug_denoise_tma": (i32, [i32]),
        "craw_debug_kernel_errors": (i32, [vp]),
        "craw_debug_denoise_round": (C.c_float, [C.c_float]),
        "craw_debug_denoise_round_decide": (i32, [i32]),
        "craw_debug_denoise_round_stats": (i32, [vp, C.POINTER(C.c_uint32), vp, C.c_uint32]),
        "craw_pipeline_params_init": (None, [C.POINTER(PipelineParams)]),
        "craw_frame_params_init": (None, [C.POINTER(FrameParams)]),
        "craw_pipeline_create": (i32, [vp, C.POINTER(PipelineParams), C.POINTER(vp)]),
        "craw_pipeline_free": (None, [C.POINTER(vp)]),
        "craw_pipeline_record": (i32, [vp, vp, C.POINTER(Image), C.POINTER(Image), C.POINTER(FrameParams)]),
        "craw_pipeline_get_awb_histogram_n": (i32, [vp, u32, C.POINTER(AwbHistogramC)]),
        "craw_pipeline_get_stage_times_n": (i32, [vp, u32, C.POINTER(StageTime), u32]),
        "craw_pipeline_get_intermediate": (i32, [vp, C.POINTER(Image), C.POINTER(Image)]),
        "craw_pipeline_get_temporal_state": (i32, [vp, C.POINTER(Image), C.POINTER(Image)]),
        "craw_pipeline_get_kernel_config": (i32, [vp, C.POINTER(i32), C.POINTER(i32)]),
        "craw_profile_init": (None, [C.POINTER(Profile)]),
        "craw_profile_validate": (i32, [C.POINTER(Profile)]),
        "craw_profile_eval": (i32, [C.POINTER(Profile), i32, C.POINTER(Illuminant), C.POINTER(ColorParams)]),
        "craw_profile_noise_eval": (i32, [C.POINTER(Profile), f32, C.POINTER(NoiseModel)]),
        "craw_noise_model_eval": (i32, [C.POINTER(NoiseKnot), u32, f32, C.POINTER(NoiseModel)]),
        "craw_colorspace_from_xyz_d65": (i32, [i32, C.POINTER(C.c_float * 9)]),
        "craw_colorspace_to_xyz_d65": (i32, [i32, C.POINTER(C.c_float * 9)]),
        "craw_planckian_xy": (i32, [f32, C.POINTER(C.c_float * 2)]),
        "craw_bradford_adaptation": (i32, [C.POINTER(C.c_float * 2), C.POINTER(C.c_float * 2),
                                           C.POINTER(C.c_float * 9)]),
        "craw_awb_histogram_from_rgb": (i32, [vp, u32, u32, C.c_size_t, i32, C.POINTER(C.c_float * 3),
                                              vp, vp, vp]),
        "craw_batch_params_init": (None, [C.POINTER(BatchParams)]),
        "craw_batch_create": (i32, [vp, C.POINTER(BatchParams), C.POINTER(vp)]),
        "craw_batch_record": (i32, [vp, vp, u32, C.POINTER(Image), C.POINTER(Image), C.POINTER(FrameParams)]),
        "craw_batch_get_info": (i32, [vp, C.POINTER(BatchInfo)]),
        "craw_batch_free": (None, [C.POINTER(vp)]),
        "craw_awb_histogram_from_rgb_cuda_noalloc": (i32, [vp, u32, u32, C.c_size_t, i32,
                                                           C.POINTER(C.c_float * 3), vp, vp, vp, vp]),
        **awb_signatures(),
        "craw_server_params_init": (None, [C.POINTER(ServerParams)]),
        "craw_server_stream_params_init": (None, [C.POINTER(ServerStreamParams)]),
        "craw_server_create": (i32, [vp, C.POINTER(ServerParams), C.POINTER(vp)]),
        "craw_server_free": (None, [C.POINTER(vp)]),
        "craw_server_stream_open": (i32, [vp, C.POINTER(ServerStreamParams), C.POINTER(u32)]),
        "craw_server_stream_close": (i32, [vp, u32]),
        "craw_server_submit": (i32, [vp, u32, vp, C.c_size_t, vp, C.c_size_t, C.POINTER(FrameParams),
                                     C.c_double, C.c_uint64]),
        "craw_server_poll": (i32, [vp, C.POINTER(ServerResult), u32, i32]),
        "craw_server_drain": (i32, [vp]),
        "craw_server_get_stats": (i32, [vp, C.POINTER(ServerStats)]),
        "craw_noise_estimate_params_init": (None, [C.POINTER(NoiseEstimateParams)]),
        "craw_noise_estimate": (i32, [vp, u32, u32, C.c_size_t, C.POINTER(Profile),
                                      C.POINTER(NoiseEstimateParams), C.POINTER(NoiseEstimate)]),
        "craw_noise_estimate_cuda": (i32, [C.POINTER(Image), C.POINTER(Profile), C.POINTER(NoiseEstimateParams),
                                           C.POINTER(NoiseEstimate), vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def version() -> tuple[int, int, int]:
    v = lib().craw_version_int()
    return (v >> 16) & 0xFF, (v >> 8) & 0xFF, v & 0xFF


# ------------------------------------------------------------ host helpers

def profile_init() -> Profile:
    p = Profile()
    lib().craw_profile_init(C.byref(p))
    return p


def profile_validate(p: Profile) -> None:
    _check(lib().craw_profile_validate(C.byref(p)), "craw_profile_validate")


def profile_eval(p: Profile, mode: int = WB_AS_SHOT, illum: Illuminant | None = None) -> ColorParams:
    out = ColorParams()
    _check(lib().craw_profile_eval(C.byref(p), mode, C.byref(illum) if illum else None, C.byref(out)),
           "craw_profile_eval")
    return out


def profile_noise_eval(p: Profile, iso: float = 0.0) -> NoiseModel:
    out = NoiseModel()
    _check(lib().craw_profile_noise_eval(C.byref(p), iso, C.byref(out)), "craw_profile_noise_eval")
    return out


def noise_model_eval(knots: list[tuple[float, float, float]], iso: float) -> NoiseModel:
    arr = (NoiseKnot * max(1, len(knots)))(*[NoiseKnot(*k) for k in knots])
    out = NoiseModel()
    _check(lib().craw_noise_model_eval(arr, len(knots), iso, C.byref(out)), "craw_noise_model_eval")
    return out


def noise_estimate_params(**kw) -> NoiseEstimateParams:
    p = NoiseEstimateParams()
    lib().craw_noise_estimate_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def noise_estimate(bayer: np.ndarray, profile: Profile,
                   params: NoiseEstimateParams | None = None) -> NoiseEstimate:
    """craw_noise_estimate() of an (h, w) uint16 host mosaic."""
    bayer = np.asarray(bayer)
    if bayer.dtype != np.uint16 or bayer.ndim != 2 or bayer.strides[1] != 2:
        raise ValueError("an (h, w) uint16 mosaic with contiguous rows")
    h, w = bayer.shape
    out = NoiseEstimate()
    _check(lib().craw_noise_estimate(bayer.ctypes.data, w, h, bayer.strides[0] // 2, C.byref(profile),
                                     None if params is None else C.byref(params), C.byref(out)),
           "craw_noise_estimate")
    return out


def noise_estimate_cuda(mosaic: Image, profile: Profile, params: NoiseEstimateParams | None = None,
                        stream: int = 0) -> NoiseEstimate:
    """craw_noise_estimate_cuda() of a device R16 image, on `stream`."""
    out = NoiseEstimate()
    _check(lib().craw_noise_estimate_cuda(C.byref(mosaic), C.byref(profile),
                                          None if params is None else C.byref(params), C.byref(out),
                                          stream or None), "craw_noise_estimate_cuda")
    return out


def colorspace_from_xyz_d65(cs: int) -> np.ndarray:
    m = (C.c_float * 9)()
    _check(lib().craw_colorspace_from_xyz_d65(cs, C.byref(m)), "craw_colorspace_from_xyz_d65")
    return np.frombuffer(m, dtype=np.float32).reshape(3, 3).copy()


def colorspace_to_xyz_d65(cs: int) -> np.ndarray:
    m = (C.c_float * 9)()
    _check(lib().craw_colorspace_to_xyz_d65(cs, C.byref(m)), "craw_colorspace_to_xyz_d65")
    return np.frombuffer(m, dtype=np.float32).reshape(3, 3).copy()


def planckian_xy(cct: float) -> tuple[float, float]:
    xy = (C.c_float * 2)()
    _check(lib().craw_planckian_xy(cct, C.byref(xy)), "craw_planckian_xy")
    return xy[0], xy[1]


def bradford_adaptation(src, dst) -> np.ndarray:
    s, d, m = (C.c_float * 2)(*src), (C.c_float * 2)(*dst), (C.c_float * 9)()
    _check(lib().craw_bradford_adaptation(C.byref(s), C.byref(d), C.byref(m)), "craw_bradford_adaptation")
    return np.frombuffer(m, dtype=np.float32).reshape(3, 3).copy()


def awb_histogram_from_rgb(rgb: np.ndarray, wb_applied) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """CPU builder over an (h, w, 3|4) float32 array."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w, ch = rgb.shape
    out = [np.zeros(AWB_BINS * AWB_BINS, np.uint32) for _ in range(3)]
    wb = (C.c_float * 3)(*wb_applied)
    _check(lib().craw_awb_histogram_from_rgb(rgb.ctypes.data, w, h, w * ch, ch, C.byref(wb),
                                             *[o.ctypes.data for o in out]),
           "craw_awb_histogram_from_rgb")
    return tuple(o.reshape(AWB_BINS, AWB_BINS) for o in out)


def pipeline_params(width: int, height: int, **kw) -> PipelineParams:
    p = PipelineParams()
    lib().craw_pipeline_params_init(C.byref(p))
    p.width, p.height = width, height
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def frame_params(profile: Profile, **kw) -> FrameParams:
    fp = FrameParams()
    lib().craw_frame_params_init(C.byref(fp))
    fp.profile = C.pointer(profile)
    for k, v in kw.items():
        if k == "noise_override":
            v = NoiseModel(*v)
        elif k == "illuminant":
            v = Illuminant(*v)
        setattr(fp, k, v)
    return fp


def image(data_ptr: int, pitch: int, fmt: int, width: int, height: int) -> Image:
    return Image(data_ptr, pitch, fmt, width, height)


def image_from_tensor(t, fmt: int) -> Image:
    """A CRAWImage over a CUDA tensor: (h, w) uint16/int16 for R16_UNORM,
    (h, w, 4) float32/float16 for RGBA32F/RGBA16F, rows contiguous."""
    h, w = t.shape[0], t.shape[1]
    return Image(t.data_ptr(), t.stride(0) * t.element_size(), fmt, w, h)


# ---------------------------------------------------------------- objects

class Context:
    """A craw context on one CUDA device (craw_context_create)."""

    def __init__(self, device: int = 0, log_level: int | None = None):
        self._h = C.c_void_p()
        params = CudaInitParams(device, None)
        opts = ContextOptions()
        opts.log_level = 2 if log_level is None else log_level
        self._children = []
        _check(lib().craw_context_create(C.byref(self._h), C.byref(params), C.byref(opts)),
               "craw_context_create")
        self.device = device

    @property
    def handle(self):
        return self._h

    def _own(self, handle: C.c_void_p, free: str) -> None:
        """Records the handle box of a pipeline, server or batch created on
        this context and the name of its free function. The box itself is
        kept (not the Python object): the garbage collector clears weak
        references before it finalises a reference cycle, and may finalise
        the context before the objects that refer to it."""
        self._children = [(h, f) for h, f in self._children if h] + [(handle, free)]

    def close(self) -> None:
        """Frees the context, and first every pipeline, server and batch
        still open on it (they hold its device memory and stream). Each
        shares its handle box with its object, so the object's own close
        then finds it freed."""
        for h, free in reversed(getattr(self, "_children", ())):
            if h:
                getattr(lib(), free)(C.byref(h))
        self._children = []
        if self._h:
            lib().craw_context_free(C.byref(self._h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AwbHistogram:
    def __init__(self, count: np.ndarray, weight: np.ndarray, weight_bright: np.ndarray):
        self.count, self.weight, self.weight_bright = count, weight, weight_bright


class Pipeline:
    """craw_pipeline_create / record / free over a :class:`Context`."""

    def __init__(self, ctx: Context, params: PipelineParams):
        self.ctx = ctx
        self.params = params
        self._h = C.c_void_p()
        ctx._own(self._h, "craw_pipeline_free")
        _check(lib().craw_pipeline_create(ctx.handle, C.byref(params), C.byref(self._h)),
               "craw_pipeline_create")

    def record(self, stream: int, src: Image, dst: Image, fp: FrameParams) -> None:
        """Enqueues one frame on ``stream`` (a cudaStream_t as an int, e.g.
        ``torch.cuda.current_stream().cuda_stream``)."""
        _check(lib().craw_pipeline_record(self._h, C.c_void_p(stream), C.byref(src), C.byref(dst),
                                          C.byref(fp)), "craw_pipeline_record")

    def awb_histogram(self, frames_back: int = 0) -> AwbHistogram:
        h = AwbHistogramC()
        _check(lib().craw_pipeline_get_awb_histogram_n(self._h, frames_back, C.byref(h)),
               "craw_pipeline_get_awb_histogram_n")
        n = h.bins * h.bins

        def arr(p):
            return np.ctypeslib.as_array(p, shape=(n,)).reshape(h.bins, h.bins).copy()
        return AwbHistogram(arr(h.count), arr(h.weight), arr(h.weight_bright))

    def stage_times(self, frames_back: int = 0) -> list[tuple[str, int, float]]:
        buf = (StageTime * 16)()
        n = _check(lib().craw_pipeline_get_stage_times_n(self._h, frames_back, buf, 16),
                   "craw_pipeline_get_stage_times_n")
        return [(buf[i].name.decode(), buf[i].count, buf[i].ms) for i in range(n)]

    def intermediate(self) -> tuple[Image, Image]:
        rgb, mosaic = Image(), Image()
        _check(lib().craw_pipeline_get_intermediate(self._h, C.byref(rgb), C.byref(mosaic)),
               "craw_pipeline_get_intermediate")
        return rgb, mosaic

    def kernel_config(self) -> tuple[int, int]:
        """The denoise tile shapes the autotuner chose (no history, history)."""
        a, b = C.c_int(), C.c_int()
        _check(lib().craw_pipeline_get_kernel_config(self._h, C.byref(a), C.byref(b)),
               "craw_pipeline_get_kernel_config")
        return a.value, b.value

    def kernel_errors(self) -> int:
        """Waits for the device and returns (and clears) the error bits the
        pipeline's kernels set: 0 when all is well."""
        return _check(lib().craw_debug_kernel_errors(self._h), "craw_debug_kernel_errors")

    def round_stats(self, max_records: int = 4096):
        """Waits for the device and returns (and clears) the exact rounding's
        statistics: (samples re-evaluated, codes changed, records, samples
        evaluated in double-float), records an (n, 4) float32 array of (t,
        x, distance of the exact x from its rounding boundary, plane) per
        changed code."""
        import numpy as np
        counts = (C.c_uint32 * 3)()
        rec = np.zeros((max_records, 4), np.float32)
        n = _check(lib().craw_debug_denoise_round_stats(self._h, counts, rec.ctypes.data, max_records),
                   "craw_debug_denoise_round_stats")
        return int(counts[0]), int(counts[1]), rec[:n], int(counts[2])

    def temporal_state(self) -> tuple[Image, Image]:
        lvl, var = Image(), Image()
        _check(lib().craw_pipeline_get_temporal_state(self._h, C.byref(lvl), C.byref(var)),
               "craw_pipeline_get_temporal_state")
        return lvl, var

    def close(self) -> None:
        if self._h:
            lib().craw_pipeline_free(C.byref(self._h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def awb_params(**kw) -> AwbParams:
    p = AwbParams()
    lib().craw_awb_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def awb_estimate(profile: Profile, count: np.ndarray, weight: np.ndarray,
                 weight_bright: np.ndarray | None, params: AwbParams | None = None,
                 bins: int = AWB_BINS, log_min: float = -2.5, log_max: float = 1.0,
                 library: C.CDLL | None = None) -> AwbEstimate:
    """craw_awb_estimate over three (bins, bins) uint32 arrays."""
    L_ = library or lib()
    arrs = [np.ascontiguousarray(a, dtype=np.uint32) if a is not None else None
            for a in (count, weight, weight_bright)]
    P32 = C.POINTER(C.c_uint32)
    h = AwbHistogramC(bins, log_min, log_max, *[a.ctypes.data_as(P32) if a is not None else P32()
                                                for a in arrs])
    out = AwbEstimate()
    _check(L_.craw_awb_estimate(C.byref(profile), C.byref(h), C.byref(params) if params else None,
                                C.byref(out)), "craw_awb_estimate")
    return out


class AwbSmoother:
    """craw_awb_smoother_*: one stream's illuminant track."""

    def __init__(self, params: AwbSmootherParams | None = None, library: C.CDLL | None = None):
        self._L = library or lib()
        self._h = C.c_void_p()
        _check(self._L.craw_awb_smoother_create(C.byref(params) if params else None,
                                                C.byref(self._h)), "craw_awb_smoother_create")

    def push(self, pts: float, est: AwbEstimate, scene_cut: bool = False) -> tuple[int, Illuminant]:
        out = Illuminant(-1.0, -1.0)
        ret = self._L.craw_awb_smoother_push(self._h, pts, C.byref(est), scene_cut, C.byref(out))
        return ret, out

    def set(self, pts: float, il: Illuminant) -> None:
        self._L.craw_awb_smoother_set(self._h, pts, C.byref(il))

    def reset(self) -> None:
        self._L.craw_awb_smoother_reset(self._h)

    def close(self) -> None:
        if self._h:
            self._L.craw_awb_smoother_free(C.byref(self._h))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def server_params(**kw) -> ServerParams:
    p = ServerParams()
    lib().craw_server_params_init(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def server_stream_params(pipeline: PipelineParams, flags: int = 0,
                         deadline_ms: float = 0.0) -> ServerStreamParams:
    p = ServerStreamParams()
    lib().craw_server_stream_params_init(C.byref(p))
    p.pipeline = pipeline
    p.flags = flags
    p.deadline_ms = deadline_ms
    return p


class Server:
    """craw_server_*: streams admitted under a device-memory budget, frames
    from host memory developed as they arrive."""

    def __init__(self, ctx: Context, params: ServerParams):
        self.ctx = ctx
        self._h = C.c_void_p()
        ctx._own(self._h, "craw_server_free")
        _check(lib().craw_server_create(ctx.handle, C.byref(params), C.byref(self._h)),
               "craw_server_create")

    def open(self, params: ServerStreamParams) -> int:
        sid = C.c_uint32()
        _check(lib().craw_server_stream_open(self._h, C.byref(params), C.byref(sid)),
               "craw_server_stream_open")
        return sid.value

    def close_stream(self, sid: int) -> None:
        _check(lib().craw_server_stream_close(self._h, sid), "craw_server_stream_close")

    def submit(self, sid: int, src: int, src_pitch: int, dst: int, dst_pitch: int,
               fp: FrameParams, pts: float = 0.0, user: int = 0) -> None:
        _check(lib().craw_server_submit(self._h, sid, C.c_void_p(src), src_pitch, C.c_void_p(dst),
                                        dst_pitch, C.byref(fp), pts, user), "craw_server_submit")

    def poll(self, max_results: int = 64, timeout_ms: int = 0) -> list[ServerResult]:
        buf = (ServerResult * max_results)()
        n = _check(lib().craw_server_poll(self._h, buf, max_results, timeout_ms), "craw_server_poll")
        return [buf[i] for i in range(n)]

    def drain(self) -> None:
        _check(lib().craw_server_drain(self._h), "craw_server_drain")

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(lib().craw_server_get_stats(self._h, C.byref(st)), "craw_server_get_stats")
        return st

    def close(self) -> None:
        if self._h:
            lib().craw_server_free(C.byref(self._h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_params(max_width: int, max_height: int, **kw) -> BatchParams:
    p = BatchParams()
    lib().craw_batch_params_init(C.byref(p))
    p.max_width, p.max_height = max_width, max_height
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Batch:
    """craw_batch_create / record / free: many frames of uneven sizes in
    one persistent launch replayed from a CUDA graph."""

    def __init__(self, ctx: Context, params: BatchParams):
        self.ctx = ctx
        self.params = params
        self._h = C.c_void_p()
        ctx._own(self._h, "craw_batch_free")
        _check(lib().craw_batch_create(ctx.handle, C.byref(params), C.byref(self._h)),
               "craw_batch_create")

    def record(self, stream: int, src: list[Image], dst: list[Image], fp: list[FrameParams]) -> None:
        n = len(src)
        if len(dst) != n or len(fp) != n:
            raise ValueError("src, dst and fp differ in length")
        S, D, P = (Image * n)(*src), (Image * n)(*dst), (FrameParams * n)(*fp)
        _check(lib().craw_batch_record(self._h, C.c_void_p(stream), n, S, D, P), "craw_batch_record")

    def info(self) -> dict:
        i = BatchInfo()
        _check(lib().craw_batch_get_info(self._h, C.byref(i)), "craw_batch_get_info")
        return {"denoise_shape": i.denoise_shape, "fused": bool(i.fused), "graph": bool(i.graph),
                "captures": i.captures, "replays": i.replays, "direct_shape": i.direct_shape,
                "direct_frames": i.direct_frames}

    def close(self) -> None:
        if self._h:
            lib().craw_batch_free(C.byref(self._h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def debug_fail_alloc(k: int) -> None:
    lib().craw_debug_fail_alloc(k)


#: Denoise tile shapes by craw_pipeline_get_kernel_config() index.
DN_SHAPES = ("2x8", "2x4", "2x8 f32x2", "2x4 f32x2")


def debug_force_denoise_shape(shape: int) -> None:
    """Every pipeline created from now uses denoise shape `shape` (-1: the
    autotuner's)."""
    _check(lib().craw_debug_force_denoise_shape(shape), "craw_debug_force_denoise_shape")


def debug_denoise_round(scale: float) -> float:
    """Width of the exact rounding's band in units of the float error bound
    (default 2; 0: off; 1e6: every sample); a negative scale only reads.
    Returns the previous scale."""
    return float(lib().craw_debug_denoise_round(scale))


def debug_denoise_round_decide(on: int) -> int:
    """1 (default): the float decision stage settles what it can of the
    marked samples; 0: all of them in double-float; -1 only reads."""
    return int(lib().craw_debug_denoise_round_decide(on))


def debug_rcd_tma(on: bool) -> bool:
    """RCD interior tiles by one TMA tile copy (True, the default) or by
    plain loads; returns the previous setting."""
    return bool(lib().craw_debug_rcd_tma(1 if on else 0))


def debug_rcd_strips(mode: int) -> int:
    """RCD interior by 64x16 tiles (0), by strips unless the colour stage
    has the gamut compression (1, the default), or by strips wherever they
    apply (2); -1 only reads. Returns the previous setting."""
    return int(lib().craw_debug_rcd_strips(int(mode)))


def debug_denoise_tma(on: bool) -> bool:
    """Denoise interior tiles (packed kernels, spatial filtering) by one
    TMA tile copy (True, the default) or by plain loads; returns the
    previous setting."""
    return bool(lib().craw_debug_denoise_tma(1 if on else 0))
