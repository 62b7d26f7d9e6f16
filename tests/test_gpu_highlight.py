"""GPU: the highlight reconstruction (kernels/highlight.cu) against the
oracle's restatement of the reference's lib/ref/ref_highlight.c.

The rebuilt mosaic is fp16; the device's logf/expf differ from the host's
by an ulp or two, so a sample may round to the neighbouring half: the
tolerance is one half-float step (2^-10 relative) on at most 1 % of the
samples, the rest equal. A sample one half step off moves the debayered
pixels around it by up to the stencil's weights times that step (MHC's
reach 6/8 and 1.5/8 of neighbours on top of the centre): the developed
frame is held to 5e-3 against the float oracle and the double one."""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, download_image, upload_mosaic
from oracle import Oracle, max_rel
import golden.make_golden as MG

pytestmark = pytest.mark.gpu

orc = Oracle()


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def run(ctx, m, prof, deb=L.DEBAYER_RCD, cs=L.CS_ACES_AP1, flags=0, fflags=L.FRAME_HIGHLIGHT_RECONSTRUCTION,
        **kw):
    h, w = m.shape
    pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, out_format=L.FORMAT_RGBA32F,
                           flags=L.FLAG_HIGHLIGHT_RECONSTRUCTION | L.FLAG_KEEP_INTERMEDIATE | flags)
    fp = L.frame_params(prof, flags=fflags, **kw)
    with L.Pipeline(ctx, pp) as pipe:
        _, src = upload_mosaic(m)
        out, dst = alloc_rgba(w, h)
        pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
        _, mos = pipe.intermediate()
        rebuilt = download_image(mos, "r16f").astype(np.float32) if mos.format == L.FORMAT_R16F else None
        torch.cuda.synchronize()
        return out.cpu().numpy(), rebuilt, pp, fp


def close_in_half_steps(got, ref):
    d = np.abs(got.astype(np.float64) - ref)
    step = np.maximum(np.abs(ref), 2.0 ** -14) * 2.0 ** -10
    return d.max() <= 1.01 * step.max() and (d <= 1.01 * step).all() and (d > 0).mean() < 0.01, \
        dict(max_abs=float(d.max()), frac=float((d > 0).mean()))


@pytest.mark.parametrize("wh,seed", [((96, 64), 401), ((200, 136), 402), ((518, 262), 403), ((12, 12), 404)])
def test_rebuilt_mosaic_vs_oracle(ctx, wh, seed):
    w, h = wh
    prof = MG.golden_profile()
    m = W.highlight_frame(w, h, seed)
    _, rebuilt, pp, fp = run(ctx, m, prof)
    assert rebuilt is not None
    ref = orc.highlights(m, prof, (2.0, 1.0, 1.5), "f32")
    ok, st = close_in_half_steps(rebuilt, ref)
    assert ok, st
    # Above the balanced clip point where the channels clipped.
    if w > 12:
        assert rebuilt.max() > 1.2


@pytest.mark.parametrize("deb", [L.DEBAYER_BILINEAR, L.DEBAYER_MHC, L.DEBAYER_RCD])
def test_developed_frame_vs_oracle(ctx, deb):
    prof = MG.golden_profile()
    m = W.highlight_frame(160, 120, 410 + deb)
    got, _, pp, fp = run(ctx, m, prof, deb=deb, cs=L.CS_BT709)
    ref = orc.process(m, pp, fp, "f32")
    assert max_rel(got, ref) < 5e-3, max_rel(got, ref)
    assert max_rel(got, orc.process(m, pp, fp, "f64")) < 5e-3


def test_frame_flag_switches_the_pass(ctx):
    """Without the frame flag the frame is clipped at the balanced clip
    point exactly as on a pipeline built without the stage."""
    prof = MG.golden_profile()
    m = W.highlight_frame(128, 96, 420)
    got, rebuilt, pp, fp = run(ctx, m, prof, fflags=0)
    assert rebuilt is None
    pp0 = L.pipeline_params(128, 96, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                            out_format=L.FORMAT_RGBA32F)
    with L.Pipeline(ctx, pp0) as pipe:
        from gpu_util import develop
        plain = develop(pipe, m, fp)
    assert np.array_equal(got, plain)
    on, _, _, _ = run(ctx, m, prof)
    assert not np.array_equal(on, plain)


def test_with_denoise_and_awb(ctx):
    """After the denoise (the pass reads the denoised mosaic) and with the
    AWB histogram, against the oracle's chain."""
    prof = MG.golden_profile()
    m = W.highlight_frame(192, 128, 430)
    got, _, pp, fp = run(ctx, m, prof, flags=L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM,
                         denoise_strength=1.0, noise_override=W.noise_model(2.0, 16.0))
    from oracle import denoised_chain_ok
    ok, st = denoised_chain_ok(got, orc.process(m, pp, fp, "f32"))
    assert ok, st
