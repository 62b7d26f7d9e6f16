"""GPU: the RCD's and the denoise's interior tiles loaded by one TMA tile
copy each against the same tiles by plain loads (the arithmetic after the
load is the same, so the frames are equal bit for bit), including frames
whose last interior RCD tile's box reaches past the right edge (columns
read as zeros, unused), the rebuilt-highlight mosaic (fp16) and the
denoised mosaic as sources, frames with no interior denoise tile, and the
exact rounding's marking kernel; and no kernel error bits."""
import numpy as np
import pytest

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import develop

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    L.debug_rcd_tma(True)
    L.debug_denoise_tma(True)
    c.close()


def both(ctx, m, pp, fp):
    """The RCD interior by tiles (whatever the output space would pick),
    with plain loads, then with the TMA copy."""
    out = []
    mode = L.debug_rcd_strips(0)
    for on in (False, True):
        L.debug_rcd_tma(on)
        with L.Pipeline(ctx, pp) as pipe:
            out.append(develop(pipe, m, fp))
            assert pipe.kernel_errors() == 0
    L.debug_rcd_tma(True)
    L.debug_rcd_strips(mode)
    return out


@pytest.mark.parametrize("w,h", [(198, 92), (199 * 2, 120), (1000, 700), (5760, 3240)])
def test_tma_equals_plain_loads(ctx, w, h):
    m = W.synth_frame(w, h, w + h, noise_a_dn=4.0, noise_b_dn=40.0)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1, out_format=L.FORMAT_RGBA32F,
                           flags=L.FLAG_AWB_HISTOGRAM)
    a, b = both(ctx, m, pp, L.frame_params(prof))
    assert np.array_equal(a, b)


def test_tma_with_denoise_and_highlights(ctx):
    w, h = 704, 398
    m = W.highlight_frame(w, h, 55)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_BT709, out_format=L.FORMAT_RGBA32F,
                           flags=L.FLAG_DENOISE | L.FLAG_HIGHLIGHT_RECONSTRUCTION)
    fp = L.frame_params(prof, flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION, denoise_strength=1.0,
                        noise_override=W.noise_model(2.0, 16.0))
    a, b = both(ctx, m, pp, fp)
    assert np.array_equal(a, b)


def both_denoise(ctx, m, pp, fp):
    out = []
    for on in (False, True):
        L.debug_denoise_tma(on)
        with L.Pipeline(ctx, pp) as pipe:
            out.append(develop(pipe, m, fp))
            assert pipe.kernel_errors() == 0
    L.debug_denoise_tma(True)
    return out


@pytest.mark.parametrize("w,h", [(64, 48), (198, 92), (1000, 700), (2050, 1030), (5760, 3240)])
@pytest.mark.parametrize("exact", [False, True])
def test_denoise_tma_equals_plain_loads(ctx, w, h, exact):
    m = W.synth_frame(w, h, 3 * w + h, noise_a_dn=4.0, noise_b_dn=40.0)
    prof = W.make_profile()
    flags = L.FLAG_DENOISE | (L.FLAG_EXACT_ROUNDING if exact else 0)
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1, out_format=L.FORMAT_RGBA32F,
                           flags=flags)
    fp = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4.0, 40.0))
    a, b = both_denoise(ctx, m, pp, fp)
    assert np.array_equal(a, b)
