"""GPU: the RCD's interior by strips (a thread a quad column walking down a
segment) against the same interior by 64x16 tiles. The two evaluate the
same formulas with the same explicit roundings, so every output is equal
bit for bit: the developed frame, the camera-RGB intermediate, the AWB
histogram; over frame sizes whose strips and segments end short, with
FP16 storage, a half-float output, a denoised source and a rebuilt
highlight mosaic (fp16 source); and no kernel error bits. The strips are
forced where the default would take the tiles (the gamut compression's
output space)."""
import numpy as np
import pytest

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import develop, download_image

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    L.debug_rcd_strips(1)
    c.close()


def both(ctx, m, pp, fp, fmt=L.FORMAT_RGBA32F, keep=False):
    """(output, histogram counters, intermediate or None) by tiles, then by
    strips."""
    out = []
    for mode in (0, 2):
        L.debug_rcd_strips(mode)
        with L.Pipeline(ctx, pp) as pipe:
            img = develop(pipe, m, fp, fmt)
            hist = pipe.awb_histogram() if pp.flags & L.FLAG_AWB_HISTOGRAM else None
            inter = None
            if keep:
                rgb, _ = pipe.intermediate()
                inter = download_image(rgb, "rgba16f" if pp.storage == L.STORAGE_FP16 else "rgba32f")
            assert pipe.kernel_errors() == 0
            out.append((img, hist, inter))
    L.debug_rcd_strips(1)
    return out


def same(a, b):
    (ia, ha, ka), (ib, hb, kb) = a, b
    assert np.array_equal(ia.view(np.uint8), ib.view(np.uint8))
    if ha is not None:
        assert np.array_equal(ha.count, hb.count)
        assert np.array_equal(ha.weight, hb.weight)
        assert np.array_equal(ha.weight_bright, hb.weight_bright)
    if ka is not None:
        assert np.array_equal(ka.view(np.uint8), kb.view(np.uint8))


@pytest.mark.parametrize("w,h", [(140, 40), (198, 92), (1000, 700), (1030, 614), (2050, 1030),
                                 (3840, 2160), (5760, 3240), (6000, 4000)])
def test_strips_equal_tiles(ctx, w, h):
    m = W.synth_frame(w, h, 7 * w + h, noise_a_dn=4.0, noise_b_dn=40.0)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1, out_format=L.FORMAT_RGBA32F,
                           flags=L.FLAG_AWB_HISTOGRAM)
    a, b = both(ctx, m, pp, L.frame_params(prof))
    same(a, b)


@pytest.mark.parametrize("storage", [L.STORAGE_FP32, L.STORAGE_FP16])
def test_strips_equal_tiles_kept_intermediate(ctx, storage):
    w, h = 1286, 718
    m = W.synth_frame(w, h, 91, noise_a_dn=2.0, noise_b_dn=16.0)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_BT2020, out_format=L.FORMAT_RGBA32F,
                           flags=L.FLAG_AWB_HISTOGRAM | L.FLAG_KEEP_INTERMEDIATE, storage=storage)
    a, b = both(ctx, m, pp, L.frame_params(prof), keep=True)
    same(a, b)


def test_strips_equal_tiles_half_output_denoised(ctx):
    w, h = 2304, 1296
    m = W.synth_frame(w, h, 5, noise_a_dn=4.0, noise_b_dn=40.0)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP0, out_format=L.FORMAT_RGBA16F,
                           flags=L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM)
    fp = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4.0, 40.0))
    a, b = both(ctx, m, pp, fp, fmt=L.FORMAT_RGBA16F)
    same(a, b)


def test_strips_equal_tiles_highlights(ctx):
    w, h = 1408, 796
    m = W.highlight_frame(w, h, 55)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_BT709, out_format=L.FORMAT_RGBA32F,
                           flags=L.FLAG_HIGHLIGHT_RECONSTRUCTION | L.FLAG_AWB_HISTOGRAM)
    fp = L.frame_params(prof, flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION)
    a, b = both(ctx, m, pp, fp)
    same(a, b)
