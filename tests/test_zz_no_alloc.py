"""GPU: craw_awb_histogram_from_rgb_cuda_noalloc, the AWB histogram of a
device RGB image built in a fixed static scratch with no allocation, against
craw_awb_histogram_from_rgb (the CPU builder) on the same image: the three
histograms must be equal bit for bit, on two calls in a row, and while
another thread holds a global-mode stream capture (whose graph must still
capture and replay). The file is named to be collected last, so that it
also runs after every other GPU test in the same process; it passes alone
as well."""
import ctypes as C
import errno

import numpy as np
import pytest
import torch

import libcraw_gb300 as L

pytestmark = pytest.mark.gpu

N = L.AWB_BINS * L.AWB_BINS


def rgb_image(w, h, ch, seed):
    """Blocky camera RGB in [0, 1.1): a smooth field, flat 8x8 blocks whose
    ratios sit exactly on bin edges (the host bins those), clipped and dark
    blocks, and a few negative samples."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    img = np.empty((h, w, ch), np.float32)
    img[..., 0] = 0.15 + 0.5 * xx / w + 0.05 * rng.standard_normal((h, w))
    img[..., 1] = 0.25 + 0.4 * yy / h + 0.05 * rng.standard_normal((h, w))
    img[..., 2] = 0.2 + 0.3 * (xx + yy) / (w + h) + 0.05 * rng.standard_normal((h, w))
    if ch == 4:
        img[..., 3] = 1.0
    wb = np.array([2.0, 1.0, 1.5], np.float32)
    # Flat blocks on bin edges: ln(rr) = -2.5 + k * 3.5 / 128.
    for i, k in enumerate(range(20, 100, 7)):
        by, bx = (2 * i) % (h // 8), (3 * i) % (w // 8)
        g = 0.4
        rr = np.float32(np.exp(-2.5 + k * 3.5 / 128))
        img[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8, 0] = rr * g * wb[0]
        img[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8, 1] = g
        img[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8, 2] = 0.3 * g * wb[2]
    img[:8, -16:, :3] = 1.05      # clipped
    img[-8:, :16, 1] = 0.001      # dark
    img[16:18, 16:18, 0] = -0.2   # negative samples
    return np.ascontiguousarray(img), wb


def cpu_hist(img, wb):
    h, w, ch = img.shape
    out = [np.zeros(N, np.uint32) for _ in range(3)]
    wbc = (C.c_float * 3)(*wb)
    ret = L.lib().craw_awb_histogram_from_rgb(img.ctypes.data, w, h, w * ch, ch, wbc,
                                              *[o.ctypes.data for o in out])
    assert ret == 0
    return out


def gpu_hist(dev, w, h, stride, ch, wb, stream):
    out = [np.full(N, 0xDEADBEEF, np.uint32) for _ in range(3)]
    wbc = (C.c_float * 3)(*wb)
    ret = L.lib().craw_awb_histogram_from_rgb_cuda_noalloc(
        dev.data_ptr(), w, h, stride, ch, wbc, *[o.ctypes.data for o in out], stream)
    return ret, out


@pytest.mark.parametrize("w,h,ch", [(640, 352, 4), (517, 263, 3)])
def test_noalloc_matches_cpu_builder_twice(w, h, ch):
    stream = torch.cuda.Stream()
    for call, seed in enumerate((1, 2)):
        img, wb = rgb_image(w, h, ch, seed + 10 * ch)
        dev = torch.from_numpy(img).cuda()
        torch.cuda.synchronize()
        ret, got = gpu_hist(dev, w, h, w * ch, ch, wb, stream.cuda_stream)
        assert ret == 0, (call, ret)
        ref = cpu_hist(img, wb)
        for name, g, r in zip(("count", "weight", "weight_bright"), got, ref):
            assert np.array_equal(g, r), (call, name, int(np.abs(g.astype(np.int64) - r).max()))
        assert ref[0].sum() > 0


def test_noalloc_rejects_beyond_scratch():
    limit = L.AWB_NOALLOC_MAX_BLOCKS
    dev = torch.zeros(16, dtype=torch.float32, device="cuda")
    # One row of blocks more than the scratch holds: rejected before any work.
    w = 8 * 4096
    h = 8 * (limit // 4096 + 1)
    ret, _ = gpu_hist(dev, w, h, w * 4, 4, [1.0, 1.0, 1.0], 0)
    assert ret == -errno.EINVAL
    # Exactly at the limit (a 4096 x 4096 image) is accepted, even when every
    # block sits on a bin edge and goes to the host: the worst case of the
    # scratch's deferred list.
    wb = np.array([2.0, 1.0, 1.5], np.float32)
    g = np.float32(0.4)
    px = np.array([np.float32(np.exp(-0.75)) * g * wb[0], g, 0.3 * g * wb[2], 1.0], np.float32)
    img = np.broadcast_to(px, (4096, 4096, 4)).copy()
    ret, got = gpu_hist(torch.from_numpy(img).cuda(), 4096, 4096, 4096 * 4, 4, wb, 0)
    assert ret == 0
    ref = cpu_hist(img, wb)
    assert int(ref[0].sum()) == limit
    for g_, r_ in zip(got, ref):
        assert np.array_equal(g_, r_)


def test_noalloc_while_another_thread_captures():
    """After its set-up call on the device, the entry point runs while
    another thread holds a global-mode stream capture (the case it exists
    for: the caller cannot allocate then). The call returns 0 with the CPU
    builder's histograms, and the other thread's capture still ends and
    its graph replays."""
    import threading

    w, h, ch = 256, 160, 4
    img, wb = rgb_image(w, h, ch, 7)
    dev = torch.from_numpy(img).cuda()
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    ret, _ = gpu_hist(dev, w, h, w * ch, ch, wb, stream.cuda_stream)   # the set-up call
    assert ret == 0
    x = torch.arange(1024, dtype=torch.float32, device="cuda")
    y = torch.zeros_like(x)
    cap_stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    started, release = threading.Event(), threading.Event()
    errors = []

    def capture():
        try:
            torch.cuda.set_device(dev.device)
            with torch.cuda.stream(cap_stream):
                graph.capture_begin(capture_error_mode="global")
                try:
                    torch.mul(x, 2.0, out=y)
                    started.set()
                    release.wait(30)
                finally:
                    graph.capture_end()
        except Exception as e:   # reported by the main thread
            errors.append(e)
            started.set()

    t = threading.Thread(target=capture)
    t.start()
    try:
        assert started.wait(30)
        ret, got = gpu_hist(dev, w, h, w * ch, ch, wb, stream.cuda_stream)
    finally:
        release.set()
        t.join(60)
    assert ret == 0 and not errors, (ret, errors)
    ref = cpu_hist(img, wb)
    for name, g, r in zip(("count", "weight", "weight_bright"), got, ref):
        assert np.array_equal(g, r), name
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, x * 2.0)
