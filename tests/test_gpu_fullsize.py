"""The headline chain at its full size, 5760x3240 (VST + NLM 1.0 + RCD +
ACES AP1 with RGC + AWB), through the C ABI, checked by properties that
do not need the oracle to develop the whole frame:

  * windows of the GPU frame against the oracle run on a crop of the
    mosaic around each window: every stage of this chain reads a bounded
    neighbourhood (the denoise 8 mosaic samples, the RCD 6), so with a
    32-sample margin the crop's own mirrored edges do not reach the
    compared interior, and where a window touches the frame's edge the
    crop mirrors at the same edge;
  * the frame's AWB histogram, bit for bit, against the CPU builder run on
    the whole intermediate the GPU produced;
  * the same frame recorded twice gives the same bytes.
"""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, download_image, upload_mosaic
from oracle import Oracle, denoised_chain_ok

pytestmark = pytest.mark.gpu

orc = Oracle()
WIDTH, HEIGHT = 5760, 3240
MARGIN = 32
#: (x, y, w, h) windows of the frame: the four corners, two edges, the centre.
WINDOWS = [(0, 0, 256, 128), (WIDTH - 256, 0, 256, 128), (0, HEIGHT - 128, 256, 128),
           (WIDTH - 256, HEIGHT - 128, 256, 128), (2880, 0, 192, 96), (0, 1600, 192, 96),
           (2816, 1568, 256, 128)]


@pytest.fixture(scope="module")
def developed():
    """The frame through the headline pipeline, recorded twice (output and
    histogram), and through a second pipeline that also keeps the camera-RGB
    intermediate (its histogram and intermediate)."""
    c = W.workload("nlm_rcd_ap1")
    assert (c.width, c.height) == (WIDTH, HEIGHT)
    assert c.flags & L.FLAG_AWB_HISTOGRAM
    m = c.frame()
    prof = W.make_profile()
    fp = L.frame_params(prof, **c.frame_kwargs())
    s = torch.cuda.current_stream().cuda_stream
    res = dict(c=c, m=m, fp=fp)
    with L.Context(0) as ctx:
        _, src = upload_mosaic(m)
        pp = L.pipeline_params(WIDTH, HEIGHT, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                               out_format=L.FORMAT_RGBA32F)
        with L.Pipeline(ctx, pp) as pipe:
            out, dst = alloc_rgba(WIDTH, HEIGHT)
            pipe.record(s, src, dst, fp)
            torch.cuda.synchronize()
            res["hist"] = pipe.awb_histogram()
            again, dst2 = alloc_rgba(WIDTH, HEIGHT)
            pipe.record(s, src, dst2, fp)
            torch.cuda.synchronize()
            res["same"] = bool(torch.equal(out, again))
            del again
            res["got"] = out.cpu().numpy()
            del out
        pp.flags |= L.FLAG_KEEP_INTERMEDIATE
        with L.Pipeline(ctx, pp) as pipe:
            out, dst = alloc_rgba(WIDTH, HEIGHT)
            pipe.record(s, src, dst, fp)
            torch.cuda.synchronize()
            rgb_img, _ = pipe.intermediate()
            res["rgb"] = download_image(rgb_img, "rgba32f").astype(np.float32)
            res["hist_keep"] = pipe.awb_histogram()
            res["same_keep"] = bool(np.array_equal(out.cpu().numpy(), res["got"]))
    return res


@pytest.mark.parametrize("win", WINDOWS, ids=[f"{x}_{y}" for x, y, _, _ in WINDOWS])
def test_windows_vs_oracle(developed, win):
    x, y, w, h = win
    c, m = developed["c"], developed["m"]
    x0, y0 = max(0, x - MARGIN), max(0, y - MARGIN)
    x1, y1 = min(WIDTH, x + w + MARGIN), min(HEIGHT, y + h + MARGIN)
    assert x0 % 2 == 0 and y0 % 2 == 0, "the crop keeps the CFA phase"
    crop = np.ascontiguousarray(m[y0:y1, x0:x1])
    pp = L.pipeline_params(x1 - x0, y1 - y0, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                           out_format=L.FORMAT_RGBA32F)
    ref = orc.process(crop, pp, developed["fp"], "f32")[y - y0:y - y0 + h, x - x0:x - x0 + w]
    got = developed["got"][y:y + h, x:x + w]
    assert not np.isnan(got).any()
    assert np.all(got[..., 3] == 1.0)
    ok, st = denoised_chain_ok(got, ref)
    assert ok, (win, st)


def test_awb_histogram_full_frame(developed):
    cnt, wgt, brt = L.awb_histogram_from_rgb(developed["rgb"], W.WB)
    assert cnt.sum() > 0.5 * (WIDTH // 8) * (HEIGHT // 8)
    for hist in (developed["hist"], developed["hist_keep"]):
        assert np.array_equal(hist.count, cnt)
        assert np.array_equal(hist.weight, wgt)
        assert np.array_equal(hist.weight_bright, brt)


def test_recording_is_deterministic(developed):
    assert developed["same"]
    assert developed["same_keep"], "keeping the intermediate changes the output"
