"""The reference's behavioural checks of the denoise, on the GPU (its
known answers, reference tests/test_pipeline.c:700-730 and 1195-1395, and
the noise trajectory its design notes publish): the spatial filter takes a
flat patch's noise down to at most 60 % and keeps at least 70 % of a 2x2
checkerboard at the sampling limit; over an eight-frame sequence whose
noise is the model's own, the temporal average makes every frame quieter
than the first and the last less than half as noisy, keeps the static
detail, and leaves no more than 0.25 sigma of a strong bar (0.6 of a
faint one) behind it; on top of the spatial filter it takes away at least
a quarter of what that one leaves, without taking more of the faint
detail. The scenes are restated in tests/kat_scenes.py; the flat patch's
noise over the sequence is the oracle's (the reference restated) to 0.3
count, and the oracle's is the reference's published 71.7, 60.0, 50.2,
43.2, 40.0, 36.3, 34.8, 31.9 counts."""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
import kat_scenes as K
from gpu_util import alloc_rgba, download_image, upload_mosaic
from oracle import Oracle

pytestmark = pytest.mark.gpu

orc = Oracle()


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def denoised(pipe, m, fp):
    _, src = upload_mosaic(m)
    _, dst = alloc_rgba(K.W_, K.H_)
    pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
    torch.cuda.synchronize()
    rgb, mos = pipe.intermediate()
    return download_image(mos, "r16").copy(), download_image(rgb, "rgba32f").copy()


@pytest.mark.parametrize("strength", [1.0, 2.0])
def test_still_noise_and_detail(ctx, strength):
    m = K.still()
    pp = L.pipeline_params(K.W_, K.H_, debayer=L.DEBAYER_MHC, out_space=L.CS_XYZ_D65,
                           flags=L.FLAG_DENOISE | L.FLAG_KEEP_INTERMEDIATE, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(K.profile(), denoise_strength=strength, noise_override=K.model())
    with L.Pipeline(ctx, pp) as pipe:
        clean, _ = denoised(pipe, m, fp)
    flat0, flat1 = K.plane_noise(m, K.FLAT_NEUTRAL), K.plane_noise(clean, K.FLAT_NEUTRAL)
    ck0, ck1 = K.plane_noise(m, K.CHECKER), K.plane_noise(clean, K.CHECKER)
    print(f"strength {strength}: flat patch {flat0:.2f} -> {flat1:.2f}, checkerboard {ck0:.0f} -> {ck1:.0f}")
    assert flat1 <= 0.60 * flat0, (flat0, flat1)
    assert ck1 >= 0.70 * ck0, (ck0, ck1)
    ref, _ = orc.denoise_temporal(m, K.profile(), K.model(), strength, 0.0)
    assert abs(K.plane_noise(ref, K.FLAT_NEUTRAL) - flat1) <= 0.05 * flat0


def sequence(ctx, strength):
    """Per frame of the sequence through one pipeline: the flat patch's
    noise, and the trails behind the bars (on the denoised mosaic and on
    the camera RGB); then the static detail and the faint checkerboard kept
    on the last frame."""
    pp = L.pipeline_params(K.W_, K.H_, debayer=L.DEBAYER_MHC, out_space=L.CS_XYZ_D65,
                           flags=L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE | L.FLAG_KEEP_INTERMEDIATE,
                           out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(K.profile(), denoise_strength=strength, denoise_temporal_strength=K.TN_ALPHA,
                        noise_override=K.model())
    truth = K.tn_frame(K.TN_FRAMES - 1, noisy=False)
    res = dict(noise=[], strong=0.0, faint=0.0, gpu_strong=0.0)
    with L.Pipeline(ctx, pp) as pipe:
        for f in range(K.TN_FRAMES):
            clean, rgb = denoised(pipe, K.tn_frame(f), fp)
            res["noise"].append(K.plane_noise(clean, K.TN_FLAT))
            if f == 0:
                res["detail0"] = K.plane_noise(clean, K.TN_DETAIL)
            else:
                x0, x1 = K.tn_bar_x(f - 1), K.tn_bar_x(f) - 1
                res["strong"] = max(res["strong"], abs(K.tn_bias(clean, x0, K.TN_STRONG[0], x1, K.TN_STRONG[1], K.TN_BG)))
                res["faint"] = max(res["faint"], abs(K.tn_bias(clean, x0, K.TN_FAINT[0], x1, K.TN_FAINT[1], K.TN_BG)))
                res["gpu_strong"] = max(res["gpu_strong"], abs(K.tn_bias_rgb(
                    rgb, x0 + 3, K.TN_STRONG[0] + 3, x1 - 3, K.TN_STRONG[1] - 3, K.TN_BG)))
    res["detail"] = K.plane_noise(clean, K.TN_DETAIL)
    res["faint_kept"] = K.tn_detail(clean, truth, K.TN_FAINT_CHECKER)
    return res


def test_temporal_alone(ctx):
    r = sequence(ctx, 0.0)
    print("temporal alone: flat patch", [round(n, 1) for n in r["noise"]], "trails", r["strong"], r["faint"],
          r["gpu_strong"], "detail", r["detail0"], r["detail"], "faint kept", r["faint_kept"])
    n = r["noise"]
    assert all(n[f] < n[0] for f in range(1, K.TN_FRAMES)), n
    assert n[-1] <= 0.5 * n[0], n
    assert r["detail"] >= 0.95 * r["detail0"] and r["faint_kept"] >= 0.95, r
    assert r["strong"] <= 0.25 and r["gpu_strong"] <= 0.25 and r["faint"] <= 0.6, r
    # The oracle (the reference restated) on the same frames.
    prev, ref = None, []
    for f in range(K.TN_FRAMES):
        clean, prev = orc.denoise_temporal(K.tn_frame(f), K.profile(), K.model(), 0.0, K.TN_ALPHA, prev=prev)
        ref.append(K.plane_noise(clean, K.TN_FLAT))
    assert np.allclose(n, ref, atol=0.3), (n, ref)
    assert np.allclose(ref, [71.7, 60.0, 50.2, 43.2, 40.0, 36.3, 34.8, 31.9], atol=0.06), ref


def test_temporal_with_spatial(ctx):
    r = sequence(ctx, 1.0)
    pp = L.pipeline_params(K.W_, K.H_, debayer=L.DEBAYER_MHC, out_space=L.CS_XYZ_D65,
                           flags=L.FLAG_DENOISE | L.FLAG_KEEP_INTERMEDIATE, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(K.profile(), denoise_strength=1.0, noise_override=K.model())
    with L.Pipeline(ctx, pp) as pipe:
        single, _ = denoised(pipe, K.tn_frame(K.TN_FRAMES - 1), fp)
    truth = K.tn_frame(K.TN_FRAMES - 1, noisy=False)
    spatial_noise = K.plane_noise(single, K.TN_FLAT)
    spatial_kept = K.tn_detail(single, truth, K.TN_FAINT_CHECKER)
    print("temporal + spatial 1.0: flat patch", [round(n, 1) for n in r["noise"]], f"(spatial alone {spatial_noise:.1f})",
          "faint kept", round(r["faint_kept"], 2), f"(spatial alone {spatial_kept:.2f})",
          "trails", r["strong"], r["faint"], r["gpu_strong"])
    assert r["noise"][-1] <= 0.75 * spatial_noise, (r["noise"][-1], spatial_noise)
    assert r["faint_kept"] >= spatial_kept, (r["faint_kept"], spatial_kept)
    assert r["strong"] <= 0.25 and r["gpu_strong"] <= 0.25 and r["faint"] <= 0.6, r
