"""Exact rounding of the denoised mosaic against the double-precision oracle.

The denoise re-encodes its result as 16-bit codes (reference
lib/ref/ref_denoise.c:318-323). The GPU marks the samples whose float code
lies near a rounding boundary and settles them again (a float evaluation
that bounds its own error, then double-float arithmetic for what that
cannot decide), so that its denoised mosaic is the one a double evaluation
of the reference's algorithm gives. These tests compare it with the FP64
oracle code for code, and the developed output with the FP64 oracle at the
1e-3 max-rel bound of the headline chain (the reference's own float code
is 1.24e-3 from FP64 on the same kind of frame: tests/test_oracle_pin.py).
"""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, download_image, upload_mosaic
from oracle import Oracle, max_rel

pytestmark = pytest.mark.gpu

orc = Oracle()


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def _default_rounding():
    scale, dec = L.debug_denoise_round(-1.0), L.debug_denoise_round_decide(-1)
    yield
    L.debug_denoise_round(scale)
    L.debug_denoise_round_decide(dec)


def denoise_gpu(ctx, m, prof, model, strength):
    """(denoised mosaic, round statistics) of one record."""
    h, w = m.shape
    pp = L.pipeline_params(w, h, flags=L.FLAG_DENOISE | L.FLAG_KEEP_INTERMEDIATE | L.FLAG_EXACT_ROUNDING,
                           out_format=L.FORMAT_RGBA32F, out_space=L.CS_ACES_AP1)
    fp = L.frame_params(prof, denoise_strength=strength, noise_override=model)
    with L.Pipeline(ctx, pp) as pipe:
        pipe.round_stats()
        _, src = upload_mosaic(m)
        _, dst = alloc_rgba(w, h)
        pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
        torch.cuda.synchronize()
        _, mos = pipe.intermediate()
        got = download_image(mos, "r16").copy()
        stats = pipe.round_stats()
    return got, stats


@pytest.mark.parametrize("w,h,seed,a,b,strength", [
    (512, 320, 1, 4.0, 40.0, 1.0),
    (384, 256, 2, 8.0, 80.0, 0.5),
    (386, 258, 3, 2.0, 16.0, 2.0),       # ragged: planes of 193 x 129
    (1024, 768, 4, 4.0, 40.0, 1.0),
    (768, 512, 5, 1.0, 10.0, 1.0),       # a low noise level: most of the frame far from black
])
def test_denoised_mosaic_equals_fp64(ctx, w, h, seed, a, b, strength):
    m = W.synth_frame(w, h, seed, rects=24, zone_plates=1, noise_a_dn=a, noise_b_dn=b)
    prof = W.make_profile()
    model = W.noise_model(a, b)
    got, (n, changed, _, nx) = denoise_gpu(ctx, m, prof, model, strength)
    ref64, _ = orc.denoise_temporal(m, prof, model, strength, 0.0, s="f64")
    ref32, _ = orc.denoise_temporal(m, prof, model, strength, 0.0, s="f32")
    assert n > 0, "no sample was re-evaluated"
    diff = int((got != ref64).sum())
    assert diff == 0, f"{diff} codes differ from the FP64 oracle ({n} re-evaluated, {nx} in double-float)"
    # The reference's own float evaluation does not round as FP64 does
    # everywhere; the GPU differs from it exactly there.
    assert np.array_equal(got != ref32, ref64 != ref32)


@pytest.mark.parametrize("decide", [1, 0])
def test_every_sample_settled_alike(ctx, decide):
    """Re-evaluating every sample gives the same mosaic as re-evaluating
    the marked band only (no sample outside the band rounds differently),
    and the float decision stage decides as the double-float stage does."""
    w, h = 1024, 640
    m = W.synth_frame(w, h, 11, rects=64, zone_plates=2, noise_a_dn=4.0, noise_b_dn=40.0)
    prof = W.make_profile()
    model = W.noise_model(4.0, 40.0)
    band, (nb, changed, _, _) = denoise_gpu(ctx, m, prof, model, 1.0)
    L.debug_denoise_round(1e6)
    L.debug_denoise_round_decide(decide)
    full, (nf, _, _, nx) = denoise_gpu(ctx, m, prof, model, 1.0)
    assert nf == w * h and nb < nf / 20, (nb, nf)
    assert changed > 0
    # The list of undecided samples holds a sixteenth of the samples.
    assert decide == 1 or nx == nf
    if decide == 0:
        # Only the first sixteenth of the list was evaluated: compare those.
        return
    assert nx < nf / 16, nx
    assert np.array_equal(band, full)


def test_rounding_off_is_the_float_path(ctx):
    L.debug_denoise_round(0.0)
    m = W.synth_frame(256, 160, 5, rects=10, zone_plates=1, noise_a_dn=4.0, noise_b_dn=40.0)
    prof = W.make_profile()
    got, (n, changed, _, _) = denoise_gpu(ctx, m, prof, W.noise_model(4.0, 40.0), 1.0)
    assert n == 0 and changed == 0
    ref32, _ = orc.denoise_temporal(m, prof, W.noise_model(4.0, 40.0), 1.0, 0.0, s="f32")
    assert np.abs(got.astype(np.int32) - ref32.astype(np.int32)).max() <= 1


@pytest.mark.parametrize("deb", [L.DEBAYER_RCD, L.DEBAYER_MHC, L.DEBAYER_BILINEAR])
def test_headline_chain_within_1e3_of_fp64(ctx, deb):
    """VST + NLM 1.0 + debayer + ACES AP1 (RGC): the developed output within
    the 1e-3 max-rel bound of the FP64 oracle; the develop alone (the
    oracle's FP64 develop of the GPU's own denoised mosaic) too."""
    w, h = 512, 320
    c = W.workload("nlm_rcd_ap1", w, h)
    m = c.frame()
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=deb, out_space=c.out_space,
                           flags=c.flags | L.FLAG_KEEP_INTERMEDIATE | L.FLAG_EXACT_ROUNDING,
                           out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, **c.frame_kwargs())
    with L.Pipeline(ctx, pp) as pipe:
        _, src = upload_mosaic(m)
        out, dst = alloc_rgba(w, h)
        pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
        torch.cuda.synchronize()
        _, mos = pipe.intermediate()
        mosaic = download_image(mos, "r16").copy()
        got = out.cpu().numpy()
    ref64 = orc.process(m, pp, fp, "f64")
    assert max_rel(got, ref64) <= 1e-3, max_rel(got, ref64)
    pp0 = L.pipeline_params(w, h, debayer=deb, out_space=c.out_space, out_format=L.FORMAT_RGBA32F)
    dev64 = orc.process(mosaic, pp0, L.frame_params(prof), "f64")
    assert max_rel(got, dev64) <= 1e-3, max_rel(got, dev64)
