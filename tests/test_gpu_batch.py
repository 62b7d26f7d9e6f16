"""GPU: the batch API (craw_batch_*) against the single-frame pipeline and
the oracle, frames of uneven sizes in one persistent launch.

The batch runs the same tile bodies as the single-frame kernels, so frames
without the denoise are bit-identical to craw_pipeline_record()'s; with the
denoise the denoise tile shape may differ, and the outputs agree within the
bound of the denoised chain (a re-encoded 16-bit sample may flip by one
code)."""
import errno

import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, develop, upload_mosaic
from oracle import Oracle, denoised_chain_ok, max_rel

pytestmark = pytest.mark.gpu

orc = Oracle()
SIZES = [(640, 352), (518, 262), (256, 160), (62, 46), (1030, 18), (12, 12)]


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def frames(seed):
    return [W.synth_frame(w, h, seed + i, rects=6, zone_plates=1, noise_a_dn=4.0, noise_b_dn=40.0)
            for i, (w, h) in enumerate(SIZES)]


def params(prof, i, denoise, shift=0):
    kw = dict(exposure_stops=0.25 * ((i + shift) % 3))
    if denoise and i % 2 == 0:
        kw.update(denoise_strength=1.0, noise_override=W.noise_model(4, 40))
    return L.frame_params(prof, **kw)


def run_batch(b, ms, fps, fmt=L.FORMAT_RGBA32F):
    keep, src, dst, outs = [], [], [], []
    for m in ms:
        t, s = upload_mosaic(m)
        o, d = alloc_rgba(m.shape[1], m.shape[0], fmt)
        keep.append(t)
        src.append(s)
        dst.append(d)
        outs.append(o)
    b.record(torch.cuda.current_stream().cuda_stream, src, dst, fps)
    torch.cuda.synchronize()
    return [o.float().cpu().numpy() for o in outs]


def single(ctx, m, fp, deb, flags, fmt=L.FORMAT_RGBA32F):
    h, w = m.shape
    pp = L.pipeline_params(w, h, debayer=deb, out_space=L.CS_ACES_AP1, out_format=fmt, flags=flags)
    with L.Pipeline(ctx, pp) as pipe:
        return develop(pipe, m, fp, fmt)


def check_against_single(ctx, got, ms, fps, deb, flags, fmt=L.FORMAT_RGBA32F):
    for i, (g, m, fp) in enumerate(zip(got, ms, fps)):
        ref = single(ctx, m, fp, deb, flags, fmt)
        assert not np.isnan(g).any(), i
        if fp.denoise_strength > 0:
            ok, st = denoised_chain_ok(g, ref)
            assert ok, (i, SIZES[i], st)
        else:
            assert np.array_equal(g, ref), (i, SIZES[i], np.abs(g - ref).max())


@pytest.mark.parametrize("deb", [L.DEBAYER_BILINEAR, L.DEBAYER_MHC, L.DEBAYER_RCD])
def test_batch_matches_single_frames(ctx, deb):
    prof = W.make_profile()
    ms = frames(100 + deb)
    fps = [params(prof, i, True) for i in range(len(ms))]
    bp = L.batch_params(1030, 352, max_frames=8, debayer=deb, out_space=L.CS_ACES_AP1,
                        flags=L.FLAG_DENOISE)
    with L.Batch(ctx, bp) as b:
        got = run_batch(b, ms, fps)
        assert b.info()["captures"] == 1
    check_against_single(ctx, got, ms, fps, deb, L.FLAG_DENOISE)


def test_split_plan_matches_single_frames(ctx):
    """With a low direct_pixels the larger frames go to the single-frame
    kernels after the persistent launch of the others: the results are the
    single-frame pipeline's all the same, and a replay repeats them."""
    prof = W.make_profile()
    ms = frames(300)
    fps = [params(prof, i, True) for i in range(len(ms))]
    bp = L.batch_params(1030, 352, max_frames=8, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                        flags=L.FLAG_DENOISE, direct_pixels=100000)
    with L.Batch(ctx, bp) as b:
        got = run_batch(b, ms, fps)
        info = b.info()
        assert info["direct_frames"] == sum(1 for w, h in SIZES if w * h >= 100000) == 2
        assert 0 <= info["direct_shape"] < len(L.DN_SHAPES)
        again = run_batch(b, ms, fps)
        assert all(np.array_equal(a, c) for a, c in zip(got, again))
        assert b.info()["captures"] == 1
    check_against_single(ctx, got, ms, fps, L.DEBAYER_RCD, L.FLAG_DENOISE)


def test_batch_vs_oracle(ctx):
    """The transitive check made direct: batch frames against the oracle."""
    prof = W.make_profile()
    ms = frames(200)
    fps = [params(prof, i, True) for i in range(len(ms))]
    bp = L.batch_params(1030, 352, max_frames=8, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                        flags=L.FLAG_DENOISE)
    with L.Batch(ctx, bp) as b:
        got = run_batch(b, ms, fps)
    for i, (g, m, fp) in enumerate(zip(got, ms, fps)):
        h, w = m.shape
        pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                               out_format=L.FORMAT_RGBA32F,
                               flags=L.FLAG_DENOISE if fp.denoise_strength > 0 else 0)
        ref = orc.process(m, pp, fp, "f32")
        if fp.denoise_strength > 0:
            ok, st = denoised_chain_ok(g, ref)
            assert ok, (i, st)
        else:
            assert max_rel(g, ref) < 1e-3, (i, max_rel(g, ref))


def test_graph_replay_and_recapture(ctx):
    prof = W.make_profile()
    bp = L.batch_params(1030, 352, max_frames=8, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                        flags=L.FLAG_DENOISE)
    with L.Batch(ctx, bp) as b:
        ms = frames(300)
        fps = [params(prof, i, True) for i in range(len(ms))]
        run_batch(b, ms, fps)
        # Same shapes, new data and settings: a replay of the same graph.
        ms2 = frames(400)
        fps2 = [params(prof, i, True, shift=1) for i in range(len(ms2))]
        got2 = run_batch(b, ms2, fps2)
        info = b.info()
        assert info["graph"] and info["captures"] == 1 and info["replays"] == 2, info
        check_against_single(ctx, got2, ms2, fps2, L.DEBAYER_RCD, L.FLAG_DENOISE)
        # Another shape set (fewer frames, and the denoise moved): a new capture.
        fps3 = [params(prof, i + 1, True) for i in range(3)]
        assert [f.denoise_strength > 0 for f in fps3] == [False, True, False]
        got3 = run_batch(b, ms2[:3], fps3)
        assert b.info()["captures"] == 2
        check_against_single(ctx, got3, ms2[:3], fps3, L.DEBAYER_RCD, L.FLAG_DENOISE)


def test_fused_unfused_graph_agree(ctx):
    prof = W.make_profile()
    ms = frames(500)
    fps = [params(prof, i, True) for i in range(len(ms))]
    outs = []
    for flags in (L.BATCH_FLAG_FUSED, L.BATCH_FLAG_UNFUSED, L.BATCH_FLAG_NO_GRAPH,
                  L.BATCH_FLAG_FUSED | L.BATCH_FLAG_NO_GRAPH):
        bp = L.batch_params(1030, 352, max_frames=8, debayer=L.DEBAYER_RCD,
                            out_space=L.CS_ACES_AP1, flags=L.FLAG_DENOISE | flags)
        with L.Batch(ctx, bp) as b:
            outs.append((run_batch(b, ms, fps), b.info()))
    assert [o[1]["fused"] for o in outs] == [True, False, False, True]
    for o, info in outs[1:]:
        for a, c in zip(outs[0][0], o):
            if info["denoise_shape"] == outs[0][1]["denoise_shape"]:
                assert np.array_equal(a, c)
            else:
                assert denoised_chain_ok(a, c)[0]
    assert not outs[2][1]["graph"] and outs[2][1]["captures"] == 0


def test_batch_rgba16f(ctx):
    prof = W.make_profile()
    ms = frames(600)[:4]
    fps = [params(prof, i, False) for i in range(len(ms))]
    bp = L.batch_params(1030, 352, max_frames=4, debayer=L.DEBAYER_MHC, out_space=L.CS_ACES_AP1,
                        out_format=L.FORMAT_RGBA16F)
    with L.Batch(ctx, bp) as b:
        got = run_batch(b, ms, fps, L.FORMAT_RGBA16F)
    check_against_single(ctx, got, ms, fps, L.DEBAYER_MHC, 0, L.FORMAT_RGBA16F)


def test_batch_errors(ctx):
    prof = W.make_profile()
    with pytest.raises(L.CrawError) as e:
        L.Batch(ctx, L.batch_params(640, 352, flags=L.FLAG_AWB_HISTOGRAM))
    assert e.value.errno == errno.ENOTSUP
    for bad in (dict(max_frames=0), dict(max_frames=65)):
        with pytest.raises(L.CrawError) as e:
            L.Batch(ctx, L.batch_params(640, 352, **bad))
        assert e.value.errno == errno.EINVAL
    with pytest.raises(L.CrawError):
        L.Batch(ctx, L.batch_params(641, 352))
    bp = L.batch_params(256, 160, max_frames=2, debayer=L.DEBAYER_BILINEAR, out_space=L.CS_ACES_AP1)
    with L.Batch(ctx, bp) as b:
        m = W.synth_frame(256, 160, 1)
        big = W.synth_frame(258, 160, 2)
        fp = L.frame_params(prof)
        s = torch.cuda.current_stream().cuda_stream
        t1, src1 = upload_mosaic(m)
        o1, dst1 = alloc_rgba(256, 160)
        t2, src2 = upload_mosaic(big)
        o2, dst2 = alloc_rgba(258, 160)
        cases = [
            ([src1] * 3, [dst1] * 3, [fp] * 3),              # more frames than the batch holds
            ([src2], [dst2], [fp]),                          # larger than max_width
            ([src1, src1], [dst1, dst1], [fp, fp]),          # destinations alias
            ([src1], [L.Image(dst1.data, dst1.pitch, L.FORMAT_RGBA16F, 256, 160)], [fp]),
        ]
        for src, dst, fps in cases:
            with pytest.raises(L.CrawError) as e:
                b.record(s, src, dst, fps)
            assert e.value.errno == errno.EINVAL
        # Nothing was enqueued by the failed recordings, nothing captured.
        assert b.info()["captures"] == 0
        # The batch still works after the errors.
        got = run_batch(b, [m], [fp])
        check_against_single(ctx, got, [m], [fp], L.DEBAYER_BILINEAR, 0)
