"""Frames and options of the noise-model estimation fixtures (reference
lib/noise.c:338-504, craw_noise_estimate), shared by make_golden.py and the
tests. Small frames with small min_bin_samples so that the fixtures stay
small; the estimator's steps do not depend on the frame's size."""
from __future__ import annotations

import numpy as np

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W


def params(nb_bins=0, min_bin_samples=0, max_level=0.0) -> L.NoiseEstimateParams:
    return L.NoiseEstimateParams(nb_bins=nb_bins, min_bin_samples=min_bin_samples, max_level=max_level)


def cases():
    """(name, mosaic, params) of every fixture."""
    flat = np.full((64, 64), W.BLACK_DN + 1000, np.uint16)
    return [
        ("ramp_32bins", W.noise_ramp(256, 192, 11), params(32, 100)),
        ("ramp_8bins_dark", W.noise_ramp(192, 128, 12, a_dn=2.0, b_dn=90.0, lo=0.0, hi=0.3), params(8, 200)),
        ("scene_16bins", W.synth_frame(192, 128, 13, noise_a_dn=4.0, noise_b_dn=40.0), params(16, 50)),
        ("highlights_maxlevel", W.highlight_frame(160, 96, 14), params(16, 10, 0.9)),
        ("scene_defaults", W.synth_frame(64, 64, 15, noise_a_dn=4.0, noise_b_dn=40.0), None),
        ("flat", flat, params(32, 10)),
        ("ramp_512bins", W.noise_ramp(256, 160, 16), params(512, 20)),
    ]


def row(ret: int, est: L.NoiseEstimate) -> np.ndarray:
    """A fixture row: return code, a, b, bins, inliers, fit error, read noise."""
    if ret < 0:
        return np.array([ret, 0, 0, 0, 0, 0, 0], np.float64)
    return np.array([ret, *est.as_tuple()], np.float64)
