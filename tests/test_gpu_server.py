"""GPU: the frame server (craw_server_*): a stream's results are the same
alone and in a mix of streams of other sizes and deadlines (bit for bit,
and the same as craw_pipeline_record() driven directly), backpressure on
submit, admission under the device-memory budget, a dead producer's
stream reclaimed, and the closed AWB loop."""
import errno
import threading
import time

import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, upload_mosaic
import golden.make_golden as MG

pytestmark = pytest.mark.gpu

MOVERS = [(2.0, 0.5), (8.0, 2.0), (24.0, 10.0)]


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def pipeline_params(w, h, temporal=True, awb=False, fmt=L.FORMAT_RGBA32F):
    flags = L.FLAG_DENOISE | (L.FLAG_TEMPORAL_DENOISE if temporal else 0) | (L.FLAG_AWB_HISTOGRAM if awb else 0)
    return L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP0, flags=flags,
                             out_format=fmt)


def frames(w, h, seed, n):
    return [W.synth_frame(w, h, seed, frame=i, rects=8, zone_plates=1, noise_a_dn=4.0,
                          noise_b_dn=40.0, movers=MOVERS) for i in range(n)]


def fparams(prof, temporal=True):
    kw = dict(denoise_strength=1.0, noise_override=W.noise_model(4.0, 40.0))
    if temporal:
        kw["denoise_temporal_strength"] = 0.8
    return L.frame_params(prof, **kw)


class Feed:
    """Pinned host inputs and outputs of one stream's frames."""

    def __init__(self, ms, fmt=L.FORMAT_RGBA32F):
        self.h, self.w = ms[0].shape
        self.src = [torch.from_numpy(m.view(np.int16)).pin_memory() for m in ms]
        dt = torch.float32 if fmt == L.FORMAT_RGBA32F else torch.float16
        self.dst = [torch.full((self.h, self.w, 4), float("nan"), dtype=dt).pin_memory() for _ in ms]

    def submit(self, srv, sid, i, fp, pts=0.0):
        s, d = self.src[i], self.dst[i]
        srv.submit(sid, s.data_ptr(), s.stride(0) * 2, d.data_ptr(), d.stride(0) * d.element_size(),
                   fp, pts, user=(sid << 32) | i)


def direct(ctx, ms, pp, fp):
    """The same frames through craw_pipeline_record(), one after another."""
    outs = []
    with L.Pipeline(ctx, pp) as pipe:
        for m in ms:
            _, src = upload_mosaic(m)
            o, dst = alloc_rgba(m.shape[1], m.shape[0])
            pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
            torch.cuda.synchronize()
            outs.append(o.cpu().numpy())
    return outs


def test_same_alone_and_in_the_mix(ctx):
    prof = W.make_profile()
    fp = fparams(prof)
    ms = frames(256, 160, 501, 6)
    pp = pipeline_params(256, 160)
    # Alone.
    with L.Server(ctx, L.server_params(hbm_budget=4 << 30)) as srv:
        a = Feed(ms)
        sid = srv.open(L.server_stream_params(pp))
        for i in range(len(ms)):
            a.submit(srv, sid, i, fp)
        srv.drain()
        res = srv.poll(64)
        assert len(res) == len(ms) and all(r.status == 0 for r in res)
        alone = [d.numpy().copy() for d in a.dst]
    # In the mix: three other streams of other sizes and settings, their
    # frames interleaved with ours and submitted while ours are in flight;
    # the streams have deadlines (earliest-deadline-first launches) or none.
    others = [(512, 288, 601, True, 33.3), (96, 64, 602, True, 0.0), (640, 352, 603, False, 41.7)]
    with L.Server(ctx, L.server_params(hbm_budget=4 << 30, max_inflight=8)) as srv:
        b = Feed(ms)
        sid = srv.open(L.server_stream_params(pp, deadline_ms=16.7))
        feeds = []
        for w, h, seed, temporal, dl in others:
            f = Feed(frames(w, h, seed, 6))
            feeds.append((srv.open(L.server_stream_params(pipeline_params(w, h, temporal), deadline_ms=dl)), f,
                          fparams(prof, temporal)))
        for i in range(len(ms)):
            for osid, f, ofp in feeds:
                f.submit(srv, osid, i, ofp)
            b.submit(srv, sid, i, fp)
        srv.drain()
        res = []
        while True:
            got = srv.poll(64)
            if not got:
                break
            res += got
        assert len(res) == 4 * len(ms) and all(r.status == 0 for r in res)
        # Each stream's frames finished in submission order.
        for s_ in {r.stream for r in res}:
            order = [r.user & 0xFFFFFFFF for r in res if r.stream == s_]
            assert order == sorted(order)
        mixed = [d.numpy() for d in b.dst]
        st = srv.stats()
        assert st.completed == 4 * len(ms) and st.failed == 0 and st.streams == 4
    for i, (x, y) in enumerate(zip(alone, mixed)):
        assert np.array_equal(x, y), (i, np.nanmax(np.abs(x - y)))
    # And both are craw_pipeline_record's own results.
    for i, (x, y) in enumerate(zip(alone, direct(ctx, ms, pp, fp))):
        assert np.array_equal(x, y), i


def test_backpressure(ctx):
    """With max_queued, a stream's waiting frames stay bounded: a submit
    beyond the bound returns EAGAIN at once and queues nothing; the
    producer polls and submits the same frame again, and the results are
    the sequence's own, in order."""
    prof = W.make_profile()
    fp = fparams(prof)
    w, h = 5760, 3240
    ms = frames(w, h, 701, 4)
    pp = pipeline_params(w, h)
    with L.Server(ctx, L.server_params(hbm_budget=8 << 30, max_inflight=1, slots_per_stream=1,
                                       max_queued=1)) as srv:
        f = Feed(ms)
        sid = srv.open(L.server_stream_params(pp, deadline_ms=41.7))
        refused, res = 0, []
        for i in range(len(ms)):
            while True:
                try:
                    f.submit(srv, sid, i, fp)
                    break
                except L.CrawError as e:
                    assert e.errno == errno.EAGAIN
                    refused += 1
                    assert srv.stats().queued <= 1
                    res += srv.poll(8, 1)
            assert srv.stats().queued <= 1
        srv.drain()
        while True:
            got = srv.poll(8)
            if not got:
                break
            res += got
        st = srv.stats()
        assert refused > 0 and st.submits_refused == refused
        assert st.completed == len(ms) and st.failed == 0
        assert [r.user & 0xFFFFFFFF for r in res] == list(range(len(ms)))
        got_frames = [d.numpy().copy() for d in f.dst]
    for i, (x, y) in enumerate(zip(got_frames, direct(ctx, ms, pp, fp))):
        assert np.array_equal(x, y), i


def test_admission_under_budget(ctx):
    pp = pipeline_params(640, 352)
    with L.Server(ctx, L.server_params(hbm_budget=1 << 40)) as probe:
        sid = probe.open(L.server_stream_params(pp))
        one = probe.stats().hbm_resident
        probe.close_stream(sid)
        assert probe.stats().hbm_resident == 0
    assert one > 640 * 352 * (2 + 16) * 2    # at least the two staging slots
    with L.Server(ctx, L.server_params(hbm_budget=int(one * 1.5))) as srv:
        a = srv.open(L.server_stream_params(pp))
        with pytest.raises(L.CrawError) as e:
            srv.open(L.server_stream_params(pp))
        assert e.value.errno == errno.EAGAIN
        with pytest.raises(L.CrawError) as e:
            srv.open(L.server_stream_params(pipeline_params(1280, 704)))
        assert e.value.errno == errno.ENOSPC
        st = srv.stats()
        assert st.streams == 1 and st.streams_refused == 2 and st.hbm_resident == one
        srv.close_stream(a)
        b = srv.open(L.server_stream_params(pp))    # the freed memory admits it
        assert srv.stats().hbm_resident == one
        srv.close_stream(b)
        with pytest.raises(L.CrawError) as e:
            srv.close_stream(b)
        assert e.value.errno == errno.ENOENT


def test_dead_producer_is_reclaimed(ctx):
    """A producer thread dies (an exception) after submitting two frames,
    without closing its stream: the server closes the stream once it has
    been idle for idle_timeout_ms and its memory admits another stream."""
    prof = W.make_profile()
    pp = pipeline_params(320, 192)
    with L.Server(ctx, L.server_params(hbm_budget=1 << 40)) as probe:
        probe.close_stream(probe.open(L.server_stream_params(pp)))
    with L.Server(ctx, L.server_params(hbm_budget=1 << 40)) as probe:
        sid = probe.open(L.server_stream_params(pp))
        one = probe.stats().hbm_resident
    with L.Server(ctx, L.server_params(hbm_budget=int(one * 1.5), idle_timeout_ms=300)) as srv:
        feed = Feed(frames(320, 192, 701, 2))
        died = []

        def producer():
            sid = srv.open(L.server_stream_params(pp))
            feed.submit(srv, sid, 0, fparams(prof))
            feed.submit(srv, sid, 1, fparams(prof))
            raise RuntimeError("producer died")

        t = threading.Thread(target=lambda: died.append(pytest.raises(RuntimeError, producer)))
        t.start()
        t.join()
        assert died
        # Its frames still finish and are reported.
        got = []
        t0 = time.time()
        while len(got) < 2 and time.time() - t0 < 10:
            got += srv.poll(8, 200)
        assert len(got) == 2 and all(r.status == 0 for r in got)
        # Meanwhile the budget has no room for another stream.
        with pytest.raises(L.CrawError) as e:
            srv.open(L.server_stream_params(pp))
        assert e.value.errno == errno.EAGAIN
        t0 = time.time()
        while srv.stats().streams_reclaimed < 1 and time.time() - t0 < 10:
            time.sleep(0.05)
        st = srv.stats()
        assert st.streams_reclaimed == 1 and st.streams == 0 and st.hbm_resident == 0
        sid = srv.open(L.server_stream_params(pp))
        assert srv.stats().streams == 1


def test_auto_wb_closed_loop(ctx):
    """With AUTO_WB each frame's histogram is read into an estimate and the
    stream's track, and the next frame is developed at the track: the same
    as developing that frame directly with CRAW_WB_REBALANCE there."""
    prof = MG.golden_profile()
    pp = pipeline_params(256, 160, temporal=False, awb=True)
    ms = [W.synth_frame(256, 160, 801 + i, rects=4, zone_plates=0, noise_a_dn=2.0, noise_b_dn=16.0)
          for i in range(4)]
    fp = fparams(prof, temporal=False)
    with L.Server(ctx, L.server_params(hbm_budget=4 << 30)) as srv:
        sp = L.server_stream_params(pp, L.SERVER_STREAM_AUTO_WB)
        # A band that takes every bin, so that each frame gives a reading.
        sp.awb.min_zone_fraction = 0.0
        sp.awb.band = 4.0
        sp.awb.sigma = 4.0
        sid = srv.open(sp)
        feed = Feed(ms)
        for i in range(len(ms)):
            feed.submit(srv, sid, i, fp, pts=i / 24.0)
        srv.drain()
        res = sorted(srv.poll(16), key=lambda r: r.user)
    assert len(res) == 4 and all(r.status == 0 for r in res)
    assert all(r.awb_valid for r in res), [(r.estimate.valid, r.estimate.source) for r in res]
    # Frame 0 used the as-shot balance; frame i > 0 the track after frame i-1.
    for i in range(1, len(ms)):
        il = res[i - 1].awb
        fpi = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4.0, 40.0),
                             wb_mode=L.WB_REBALANCE, illuminant=(il.cct, il.tint))
        want = direct(ctx, [ms[i]], pipeline_params(256, 160, temporal=False, awb=True), fpi)[0]
        assert np.array_equal(feed.dst[i].numpy(), want), i


def test_estimate_noise_for_a_stream_without_a_model(ctx):
    """With ESTIMATE_NOISE the first frame's model is measured on the
    device (equal to craw_noise_estimate of that frame) and every frame
    without an override is developed with it: the same as developing it
    directly with that model. A stream of frames too flat to fit fails its
    frame with ENODATA and tries again on the next."""
    prof = W.make_profile()
    w, h = 2560, 1440            # enough samples for the default 20000 a bin
    ms = [W.noise_ramp(w, h, 900 + i, lo=0.0) for i in range(3)]
    pp = pipeline_params(w, h, temporal=False)
    fp = L.frame_params(prof, denoise_strength=1.0)          # no model: estimated
    est0 = L.noise_estimate(ms[0], prof)
    with L.Server(ctx, L.server_params(hbm_budget=8 << 30)) as srv:
        sid = srv.open(L.server_stream_params(pp, L.SERVER_STREAM_ESTIMATE_NOISE))
        feed = Feed(ms)
        for i in range(len(ms)):
            feed.submit(srv, sid, i, fp)
        srv.drain()
        res = sorted(srv.poll(16), key=lambda r: r.user)
        assert [r.status for r in res] == [0, 0, 0]
        assert [r.noise_valid for r in res] == [True, False, False]
        assert res[0].noise.as_tuple() == est0.as_tuple()
        fpm = L.frame_params(prof, denoise_strength=1.0, noise_override=(est0.model.a, est0.model.b))
        want = direct(ctx, ms, pp, fpm)
        for i in range(len(ms)):
            assert np.array_equal(feed.dst[i].numpy(), want[i]), i

        flat = [np.full((h, w), W.BLACK_DN + 900, np.uint16)] + ms[:1]
        sid2 = srv.open(L.server_stream_params(pp, L.SERVER_STREAM_ESTIMATE_NOISE))
        feed2 = Feed(flat)
        for i in range(2):
            feed2.submit(srv, sid2, i, fp)
        srv.drain()
        res2 = sorted(srv.poll(16), key=lambda r: r.user)
        assert res2[0].status == -errno.ENODATA and not res2[0].noise_valid
        assert res2[1].status == 0 and res2[1].noise_valid
    with L.Server(ctx, L.server_params(hbm_budget=8 << 30)) as srv:
        with pytest.raises(L.CrawError):
            srv.open(L.server_stream_params(L.pipeline_params(w, h), L.SERVER_STREAM_ESTIMATE_NOISE))


def test_server_errors(ctx):
    prof = W.make_profile()
    with L.Server(ctx, L.server_params(hbm_budget=1 << 30)) as srv:
        with pytest.raises(L.CrawError) as e:
            srv.open(L.server_stream_params(pipeline_params(256, 160), L.SERVER_STREAM_AUTO_WB))
        assert e.value.errno == errno.EINVAL
        with pytest.raises(L.CrawError) as e:
            srv.submit(12345, 1, 512, 1, 4096, fparams(prof))
        assert e.value.errno == errno.ENOENT
        sid = srv.open(L.server_stream_params(pipeline_params(256, 160)))
        with pytest.raises(L.CrawError) as e:
            srv.submit(sid, 1, 100, 1, 4096, fparams(prof))     # pitch below the row
        assert e.value.errno == errno.EINVAL
        # A frame whose recording fails (no profile) reports its error and
        # leaves the stream working.
        feed = Feed(frames(256, 160, 901, 2))
        bad = fparams(prof)
        bad.profile = None
        feed.submit(srv, sid, 0, bad)
        feed.submit(srv, sid, 1, fparams(prof))
        srv.drain()
        res = sorted(srv.poll(8), key=lambda r: r.user)
        assert res[0].status == -errno.EINVAL and res[1].status == 0
        assert srv.stats().failed == 1
