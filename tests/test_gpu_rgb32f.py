"""GPU: the RGB32F output (three floats a pixel, no alpha; an extension of
this library) carries exactly the first three channels of the RGBA32F
output, bit for bit: through the tile and strip RCD kernels, the chroma
path with a temporal sequence, FP16 storage, the plain pipeline, a batch
of uneven frames and the frame server."""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from gpu_util import alloc_rgba, develop, upload_mosaic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


CASES = [
    # (name, w, h, debayer, space, flags, storage, impl, frame kwargs, frames)
    ("rcd_ap1_tiles", 1030, 614, L.DEBAYER_RCD, L.CS_ACES_AP1, L.FLAG_DENOISE | L.FLAG_AWB_HISTOGRAM,
     L.STORAGE_FP32, L.IMPL_FUSED, dict(denoise_strength=1.0), 1),
    ("rcd_bt2020_strips", 1030, 614, L.DEBAYER_RCD, L.CS_BT2020, L.FLAG_AWB_HISTOGRAM,
     L.STORAGE_FP32, L.IMPL_FUSED, {}, 1),
    ("mhc_chroma_temporal", 390, 262, L.DEBAYER_MHC, L.CS_P3D65,
     L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE | L.FLAG_CHROMA_DENOISE,
     L.STORAGE_FP32, L.IMPL_FUSED, dict(denoise_strength=1.0, denoise_temporal_strength=0.8,
                                        denoise_chroma_strength=0.5), 3),
    ("bilinear_fp16", 200, 136, L.DEBAYER_BILINEAR, L.CS_BT709, L.FLAG_AWB_HISTOGRAM,
     L.STORAGE_FP16, L.IMPL_FUSED, {}, 1),
    ("plain_rcd", 256, 160, L.DEBAYER_RCD, L.CS_ACES_AP1, L.FLAG_DENOISE, L.STORAGE_FP32, L.IMPL_PLAIN,
     dict(denoise_strength=1.0), 1),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_rgb32f_is_rgba32f_without_alpha(ctx, case):
    name, w, h, deb, cs, flags, storage, impl, kw, nfr = case
    prof = W.make_profile()
    fp = L.frame_params(prof, noise_override=W.noise_model(4.0, 40.0), **kw)
    ms = [W.synth_frame(w, h, 31 * w + f, noise_a_dn=4.0, noise_b_dn=40.0) for f in range(nfr)]
    outs = {}
    for fmt in (L.FORMAT_RGBA32F, L.FORMAT_RGB32F):
        pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, out_format=fmt, flags=flags, storage=storage,
                               impl=impl)
        with L.Pipeline(ctx, pp) as pipe:
            outs[fmt] = [develop(pipe, m, fp, fmt) for m in ms]
    for a, b in zip(outs[L.FORMAT_RGBA32F], outs[L.FORMAT_RGB32F]):
        assert b.shape == (h, w, 3)
        assert np.array_equal(a[..., :3].view(np.uint32), b.view(np.uint32))


def test_rgb32f_batch(ctx):
    prof = W.make_profile()
    sizes = [(640, 352), (256, 160), (62, 46)]
    ms = [W.synth_frame(w, h, 900 + i, noise_a_dn=4.0, noise_b_dn=40.0) for i, (w, h) in enumerate(sizes)]
    fps = [L.frame_params(prof) for _ in ms]
    got = {}
    for fmt in (L.FORMAT_RGBA32F, L.FORMAT_RGB32F):
        with L.Batch(ctx, L.batch_params(640, 352, max_frames=4, out_format=fmt)) as b:
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
            got[fmt] = [o.cpu().numpy() for o in outs]
    for a, b in zip(got[L.FORMAT_RGBA32F], got[L.FORMAT_RGB32F]):
        assert np.array_equal(a[..., :3].view(np.uint32), b.view(np.uint32))


def test_rgb32f_server(ctx):
    prof = W.make_profile()
    w, h = 512, 288
    m = W.synth_frame(w, h, 77, noise_a_dn=4.0, noise_b_dn=40.0)
    fp = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4.0, 40.0))
    src = torch.from_numpy(m.view(np.int16)).pin_memory()
    got = {}
    for fmt, ch in ((L.FORMAT_RGBA32F, 4), (L.FORMAT_RGB32F, 3)):
        pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP0, flags=L.FLAG_DENOISE,
                               out_format=fmt)
        dst = torch.full((h, w, ch), float("nan"), dtype=torch.float32).pin_memory()
        with L.Server(ctx, L.server_params(hbm_budget=2 << 30)) as srv:
            sid = srv.open(L.server_stream_params(pp))
            srv.submit(sid, src.data_ptr(), w * 2, dst.data_ptr(), w * 4 * ch, fp)
            srv.drain()
            res = srv.poll(4)
            assert len(res) == 1 and res[0].status == 0
        got[fmt] = dst.numpy().copy()
    assert np.array_equal(got[L.FORMAT_RGBA32F][..., :3].view(np.uint32), got[L.FORMAT_RGB32F].view(np.uint32))
