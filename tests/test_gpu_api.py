"""GPU tests of the API's semantics: argument errors, the temporal-state
rules (bit for bit, GPU against GPU), histogram slots, profiling, and
allocation failure."""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, download_image, upload_mosaic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def stream():
    return torch.cuda.current_stream().cuda_stream


def test_check_device():
    import ctypes as C
    missing = C.c_char_p()
    assert L.lib().craw_cuda_check_device(0, C.byref(missing)) == 0
    assert L.lib().craw_cuda_check_device(97, C.byref(missing)) < 0


def test_create_errors(ctx):
    bad = [
        dict(width=7, height=8), dict(width=6, height=8), dict(width=0, height=8),
        dict(width=64, height=48, out_format=L.FORMAT_R16_UNORM),
        dict(width=64, height=48, debayer=3), dict(width=64, height=48, out_space=9),
        dict(width=8, height=8, flags=L.FLAG_DENOISE),
        dict(width=10, height=12, flags=L.FLAG_TEMPORAL_DENOISE),
    ]
    for kw in bad:
        w, h = kw.pop("width"), kw.pop("height")
        with pytest.raises(L.CrawError) as e:
            L.Pipeline(ctx, L.pipeline_params(w, h, **kw))
        assert e.value.errno == 22, (w, h, kw)
    for flag in (L.FLAG_LENS, L.FLAG_FALSE_COLOR, L.FLAG_DEFRINGE, L.FLAG_SHARPEN):
        with pytest.raises(L.CrawError) as e:
            L.Pipeline(ctx, L.pipeline_params(64, 48, flags=flag))
        assert e.value.errno == 95
    # The highlight reconstruction is built for the fused path only.
    with pytest.raises(L.CrawError) as e:
        L.Pipeline(ctx, L.pipeline_params(64, 48, flags=L.FLAG_HIGHLIGHT_RECONSTRUCTION, impl=L.IMPL_PLAIN))
    assert e.value.errno == 95
    with pytest.raises(L.CrawError) as e:
        L.Pipeline(ctx, L.pipeline_params(64, 48, cfa=1))
    assert e.value.errno == 95


def test_record_errors(ctx):
    w, h = 64, 48
    m = W.synth_frame(w, h, 1)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, flags=L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE | L.FLAG_CHROMA_DENOISE,
                           out_format=L.FORMAT_RGBA32F)
    with L.Pipeline(ctx, pp) as pipe:
        t, src = upload_mosaic(m)
        out, dst = alloc_rgba(w, h)
        fp = L.frame_params(prof)
        s = stream()
        cases = []
        d2 = L.Image(dst.data, dst.pitch, L.FORMAT_RGBA16F, w, h)
        cases.append((src, d2, fp, 22))                       # wrong dst format
        s2 = L.Image(src.data, src.pitch, L.FORMAT_RGBA32F, w, h)
        cases.append((s2, dst, fp, 22))                       # wrong src format
        cases.append((L.Image(src.data, src.pitch, src.format, w - 2, h), dst, fp, 22))
        cases.append((L.Image(src.data + 2, src.pitch, src.format, w, h), dst, fp, 22))  # misaligned
        alias = L.Image(src.data, dst.pitch, dst.format, w, h)
        cases.append((src, alias, fp, 22))                    # src and dst alias
        cases.append((src, dst, L.frame_params(prof, denoise_strength=1.0), 95))  # no noise model
        cases.append((src, dst, L.frame_params(prof, denoise_temporal_strength=1.5,
                                               noise_override=(1e-3, 1e-6)), 22))
        cases.append((src, dst, L.frame_params(prof, denoise_chroma_strength=1.5), 22))
        cases.append((src, dst, L.frame_params(prof, out_space=11, out_space_set=True), 22))
        bad_prof = W.make_profile()
        bad_prof.white_level[1] = bad_prof.black_level[1]
        cases.append((src, dst, L.frame_params(bad_prof), 22))
        cases.append((src, dst, L.frame_params(prof, wb_mode=L.WB_REBALANCE, illuminant=(5000, 0)), 95))
        for a, b, f, err in cases:
            with pytest.raises(L.CrawError) as e:
                pipe.record(s, a, b, f)
            assert e.value.errno == err
        # Nothing above touched the output or the state.
        torch.cuda.synchronize()
        assert torch.isnan(out).all()
        with pytest.raises(L.CrawError) as e:
            pipe.temporal_state()
        assert e.value.errno == 11  # EAGAIN: still no state
        pipe.record(s, src, dst, fp)
        torch.cuda.synchronize()
        assert not torch.isnan(out).any()


def temporal_run(ctx, frames, plan, w=96, h=64):
    """Runs `plan` (a list of (frame index, frame kwargs)) through one
    temporal pipeline and returns every output."""
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, flags=L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE,
                           out_format=L.FORMAT_RGBA32F)
    outs = []
    with L.Pipeline(ctx, pp) as pipe:
        srcs = [upload_mosaic(f) for f in frames]
        for i, kw in plan:
            base = dict(denoise_strength=1.0, denoise_temporal_strength=0.8,
                        noise_override=W.noise_model(4, 40))
            base.update(kw)
            fp = L.frame_params(prof, **base)
            o, dst = alloc_rgba(w, h)
            pipe.record(stream(), srcs[i][1], dst, fp)
            torch.cuda.synchronize()
            outs.append(o.cpu().numpy())
    return outs


def test_temporal_rules(ctx):
    w, h = 96, 64
    frames = [W.synth_frame(w, h, 5, frame=i, movers=[(8.0, 2.0)]) for i in range(4)]
    base = temporal_run(ctx, frames, [(0, {}), (1, {}), (2, {})])
    # Replay: develops the last frame again, bit for bit, however often.
    rep = temporal_run(ctx, frames, [(0, {}), (1, {}), (1, {"denoise_temporal_replay": True}),
                                     (1, {"denoise_temporal_replay": True}), (2, {})])
    assert np.array_equal(rep[2], base[1]) and np.array_equal(rep[3], base[1])
    assert np.array_equal(rep[4], base[2])
    # A replay with other parameters changes that frame only.
    rep2 = temporal_run(ctx, frames, [(0, {}), (1, {}), (1, {"denoise_temporal_replay": True,
                                                             "exposure_stops": 1.0}), (2, {})])
    assert not np.array_equal(rep2[2], base[1])
    assert np.array_equal(rep2[3], base[2])
    # Reset: the frame is developed as a first frame.
    first = temporal_run(ctx, frames, [(2, {})])
    rst = temporal_run(ctx, frames, [(0, {}), (1, {}), (2, {"flags": L.FRAME_TEMPORAL_RESET})])
    assert np.array_equal(rst[2], first[0])
    # A next frame with the pass off leaves no state: the one after restarts.
    off = temporal_run(ctx, frames, [(0, {}), (1, {"denoise_temporal_strength": 0.0}), (2, {})])
    assert np.array_equal(off[2], first[0])
    # A replay with the pass off leaves the state alone.
    roff = temporal_run(ctx, frames, [(0, {}), (1, {}), (1, {"denoise_temporal_replay": True,
                                                             "denoise_temporal_strength": 0.0}), (2, {})])
    assert np.array_equal(roff[3], base[2])
    # The average changes the picture versus the spatial filter alone.
    assert not np.array_equal(base[2], first[0])


def test_recordings_in_flight(ctx):
    """Four recordings queued on one stream before any is waited for give
    the same frames as four recorded one at a time."""
    w, h = 96, 64
    frames = [W.synth_frame(w, h, 9, frame=i) for i in range(4)]
    one = temporal_run(ctx, frames, [(i, {}) for i in range(4)])
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, flags=L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE | L.FLAG_AWB_HISTOGRAM,
                           out_format=L.FORMAT_RGBA32F, nb_awb_slots=4)
    with L.Pipeline(ctx, pp) as pipe:
        srcs = [upload_mosaic(f) for f in frames]
        outs = [alloc_rgba(w, h) for _ in frames]
        fp = L.frame_params(prof, denoise_strength=1.0, denoise_temporal_strength=0.8,
                            noise_override=W.noise_model(4, 40))
        for i in range(4):
            pipe.record(stream(), srcs[i][1], outs[i][1], fp)
        torch.cuda.synchronize()
        for i in range(4):
            assert np.array_equal(outs[i][0].cpu().numpy(), one[i])
        # All four histograms are readable, newest first.
        for back in range(4):
            assert pipe.awb_histogram(back).count.sum() > 0
        with pytest.raises(L.CrawError):
            pipe.awb_histogram(4)


def test_determinism(ctx):
    w, h = 200, 120
    c = W.workload("nlm_rcd_ap1", w, h)
    m = c.frame()
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, flags=c.flags, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, **c.frame_kwargs())
    from gpu_util import develop
    with L.Pipeline(ctx, pp) as pipe:
        a = develop(pipe, m, fp)
        b = develop(pipe, m, fp)
        ha = pipe.awb_histogram().count
    assert np.array_equal(a, b)
    assert ha.sum() > 0


def test_stage_times(ctx):
    w, h = 128, 96
    m = W.synth_frame(w, h, 3)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, flags=L.FLAG_PROFILE | L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM,
                           out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4, 40))
    with L.Pipeline(ctx, pp) as pipe:
        with pytest.raises(L.CrawError):
            pipe.stage_times()
        from gpu_util import develop
        develop(pipe, m, fp)
        st = pipe.stage_times()
        names = [s[0] for s in st]
        assert names == ["denoise_nlm", "develop", "awb_reduce"], names
        assert all(s[1] == 1 and s[2] > 0 for s in st)
    with L.Pipeline(ctx, L.pipeline_params(w, h)) as pipe:
        with pytest.raises(L.CrawError) as e:
            pipe.stage_times()
        assert e.value.errno == 22


def test_alloc_failure_leaves_nothing(ctx):
    pp = L.pipeline_params(256, 160, flags=L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE |
                           L.FLAG_AWB_HISTOGRAM | L.FLAG_CHROMA_DENOISE)
    for k in range(1, 8):
        L.debug_fail_alloc(k)
        with pytest.raises(L.CrawError) as e:
            L.Pipeline(ctx, pp)
        assert e.value.errno == 12
    L.debug_fail_alloc(0)
    with L.Pipeline(ctx, pp):
        pass


def test_awb_requires_flag(ctx):
    with L.Pipeline(ctx, L.pipeline_params(64, 48)) as pipe:
        with pytest.raises(L.CrawError) as e:
            pipe.awb_histogram()
        assert e.value.errno == 22


def test_context_closes_its_pipelines_first():
    """Closing a context frees the pipelines still open on it first, so
    that a later close (or the garbage collector finalising the two in
    either order) never touches freed memory."""
    import gc
    c = L.Context(0)
    p = L.Pipeline(c, L.pipeline_params(64, 48, flags=L.FLAG_DENOISE))
    c.close()
    assert not p._h
    p.close()
    # A reference cycle holding both: collected in whatever order.
    c2 = L.Context(0)
    p2 = L.Pipeline(c2, L.pipeline_params(64, 48))
    cyc = [c2, p2]
    cyc.append(cyc)
    del c2, p2, cyc
    gc.collect()
