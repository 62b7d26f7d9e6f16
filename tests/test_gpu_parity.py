"""GPU parity: every stage of the path through the C ABI (libcraw.so) against
the CPU oracle on the same seeded inputs, at sizes the oracle finishes in
seconds.

Tolerances (the metric of reference tests/test_pipeline.c:321-359,
per-pixel magnitude-relative error floored at 1% of the frame peak):
  * FP32 storage vs the float oracle: 2e-4 (bilinear, MHC), 1e-3 (RCD),
    the differences being fused multiply-adds and division order;
  * FP16 storage vs the float oracle: 2e-3 (one half-float rounding of the
    intermediate, 4.9e-4 relative, carried through the 3x3 matrix);
  * with the denoise: the denoised mosaic within one 16-bit code of the
    oracle's, and the output within 2e-3;
  * against the double oracle: 1e-3 for FP32 storage (the target).
AWB histograms are compared for exact equality with the CPU builder run on
the intermediate the GPU produced.
"""
import numpy as np
import pytest
import torch

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from oracle import Oracle, denoised_chain_ok, max_abs, max_rel, psnr

pytestmark = pytest.mark.gpu

orc = Oracle()
TOL_FP32 = {L.DEBAYER_BILINEAR: 2e-4, L.DEBAYER_MHC: 2e-4, L.DEBAYER_RCD: 1e-3}
TOL_FP16 = 2e-3


@pytest.fixture(scope="module")
def ctx():
    c = L.Context(0)
    yield c
    c.close()


def run(ctx, m, pp, fp, fmt=L.FORMAT_RGBA32F):
    from gpu_util import develop
    with L.Pipeline(ctx, pp) as pipe:
        return develop(pipe, m, fp, fmt)


def frame(w, h, seed, a=4.0, b=40.0, **kw):
    return W.synth_frame(w, h, seed, rects=10, zone_plates=1, noise_a_dn=a, noise_b_dn=b, **kw)


@pytest.mark.parametrize("storage", [L.STORAGE_FP32, L.STORAGE_FP16])
@pytest.mark.parametrize("deb", [L.DEBAYER_BILINEAR, L.DEBAYER_MHC, L.DEBAYER_RCD])
@pytest.mark.parametrize("cs", [L.CS_BT709, L.CS_ACES_AP1])
def test_develop_vs_oracle(ctx, deb, cs, storage):
    w, h = 200, 136
    m = frame(w, h, 10 + deb)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, out_format=L.FORMAT_RGBA32F,
                           storage=storage)
    fp = L.frame_params(prof)
    got = run(ctx, m, pp, fp)
    ref = orc.process(m, pp, fp, "f32")
    assert not np.isnan(got).any()
    assert np.all(got[..., 3] == 1.0)
    tol = TOL_FP32[deb] if storage == L.STORAGE_FP32 else TOL_FP16
    assert max_rel(got, ref) < tol, (max_rel(got, ref), max_abs(got, ref))
    if storage == L.STORAGE_FP32:
        assert max_rel(got, orc.process(m, pp, fp, "f64")) < 1e-3


@pytest.mark.parametrize("storage", [L.STORAGE_FP32, L.STORAGE_FP16])
def test_config1_at_its_size(ctx, storage):
    """The plain-method configuration at its stated size and noise: one
    1920x1080 frame (12-bit, black 256, white 4095, 64 rectangles and a zone
    plate, var = 2 s + 16 DN^2), bilinear debayer, no denoise, BT.709 linear
    float32, AWB histogram. FP32 storage within 2e-4 of the float oracle and
    1e-3 of the double one (the reference's debayer checks,
    tests/test_pipeline.c:6019-6111, hold their GPU output to the same
    kind of bound); FP16 storage (the debayered values rounded to half)
    within 2e-3 of both."""
    c = W.workload("bilinear_bt709_1080p")
    assert (c.width, c.height, c.noise_a_dn, c.noise_b_dn) == (1920, 1080, 2.0, 16.0)
    assert c.debayer == L.DEBAYER_BILINEAR and c.out_space == L.CS_BT709
    m = c.frame()
    prof = W.make_profile()
    pp = L.pipeline_params(c.width, c.height, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                           out_format=L.FORMAT_RGBA32F, storage=storage)
    fp = L.frame_params(prof)
    got = run(ctx, m, pp, fp)
    assert not np.isnan(got).any() and np.all(got[..., 3] == 1.0)
    r32, r64 = max_rel(got, orc.process(m, pp, fp, "f32")), max_rel(got, orc.process(m, pp, fp, "f64"))
    if storage == L.STORAGE_FP32:
        assert r32 < 2e-4 and r64 < 1e-3, (r32, r64)
    else:
        assert r32 < TOL_FP16 and r64 < TOL_FP16, (r32, r64)


@pytest.mark.parametrize("impl", [L.IMPL_FUSED, L.IMPL_PLAIN])
def test_full_chain_vs_oracle(ctx, impl):
    """The single-frame chain of the headline workload at a small size:
    VST + NLM 1.0 + RCD + ACES AP1 (with RGC) + AWB."""
    w, h = 256, 160
    c = W.workload("nlm_rcd_ap1", w, h)
    m = c.frame()
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                           out_format=L.FORMAT_RGBA32F, impl=impl)
    fp = L.frame_params(prof, **c.frame_kwargs())
    got = run(ctx, m, pp, fp)
    ok, st = denoised_chain_ok(got, orc.process(m, pp, fp, "f32"))
    assert ok, st
    ok, st = denoised_chain_ok(got, orc.process(m, pp, fp, "f64"))
    assert ok, st


def test_denoise_mosaic_vs_oracle(ctx):
    from gpu_util import download_image, upload_mosaic, alloc_rgba
    w, h = 192, 128
    m = frame(w, h, 31, a=8.0, b=80.0)
    prof = W.make_profile()
    model = W.noise_model(8.0, 80.0)
    for strength in (0.5, 1.0, 2.0):
        pp = L.pipeline_params(w, h, flags=L.FLAG_DENOISE | L.FLAG_KEEP_INTERMEDIATE,
                               out_format=L.FORMAT_RGBA32F)
        fp = L.frame_params(prof, denoise_strength=strength, noise_override=model)
        with L.Pipeline(ctx, pp) as pipe:
            _, src = upload_mosaic(m)
            _, dst = alloc_rgba(w, h)
            pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
            _, mos = pipe.intermediate()
            got = download_image(mos, "r16")
        ref, _ = orc.denoise_temporal(m, prof, model, strength, 0.0)
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 1, (strength, d.max())
        assert (d > 0).mean() < 0.01, (strength, (d > 0).mean())
        # The filter did something.
        assert np.abs(got.astype(np.int32) - m.astype(np.int32)).mean() > 0.5


@pytest.mark.parametrize("shape", range(len(L.DN_SHAPES)), ids=list(L.DN_SHAPES))
@pytest.mark.parametrize("temporal", [False, True])
def test_every_denoise_shape_vs_oracle(ctx, shape, temporal):
    """Each denoise tile shape (the scalar and the packed f32x2 searches),
    forced past the autotuner, on a ragged frame: the denoised mosaic within
    one 16-bit code of the oracle's, over a three-frame temporal sequence
    when `temporal` (the first frame has no history, the others have)."""
    from gpu_util import download_image, upload_mosaic, alloc_rgba
    w, h = 202, 134
    prof = W.make_profile()
    model = W.noise_model(8.0, 80.0)
    flags = L.FLAG_DENOISE | L.FLAG_KEEP_INTERMEDIATE | (L.FLAG_TEMPORAL_DENOISE if temporal else 0)
    kw = dict(denoise_strength=1.0, noise_override=model)
    if temporal:
        kw["denoise_temporal_strength"] = 0.8
    fp = L.frame_params(prof, **kw)
    frames = [W.synth_frame(w, h, 41, frame=i, rects=10, zone_plates=1, noise_a_dn=8.0,
                            noise_b_dn=80.0, movers=[(2.0, 0.5), (8.0, 2.0)]) for i in range(3 if temporal else 1)]
    L.debug_force_denoise_shape(shape)
    try:
        with L.Pipeline(ctx, L.pipeline_params(w, h, flags=flags, out_format=L.FORMAT_RGBA32F)) as pipe:
            assert pipe.kernel_config() == (shape, shape)
            prev = None
            for m in frames:
                _, src = upload_mosaic(m)
                _, dst = alloc_rgba(w, h)
                pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
                _, mos = pipe.intermediate()
                got = download_image(mos, "r16")
                ref, _ = orc.denoise_temporal(m, prof, model, 1.0, 0.8 if temporal else 0.0, prev)
                d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
                limit = 2 if prev is not None else 1
                assert d.max() <= limit, d.max()
                assert (d > 0).mean() < 0.02, (d > 0).mean()
                if temporal:
                    # Follow the GPU's own state so the comparison does not drift.
                    lvl, var = pipe.temporal_state()
                    qv = (download_image(var, "r8").astype(np.float32) / 255.0) ** 2
                    prev = np.stack([download_image(lvl, "r32f"), qv]).astype(np.float32)
    finally:
        L.debug_force_denoise_shape(-1)


def test_autotuned_shapes_agree_per_size(ctx):
    """Pipelines of one size get the same denoise shapes whatever mix of
    stages they were created with (the tuner's picks are kept per size and
    per kind), so that they give the same results."""
    w, h = 1206, 610
    seen = []
    for flags in (L.FLAG_DENOISE, L.FLAG_DENOISE, L.FLAG_TEMPORAL_DENOISE,
                  L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE, L.FLAG_DENOISE):
        with L.Pipeline(ctx, L.pipeline_params(w, h, flags=flags)) as pipe:
            a, b = pipe.kernel_config()
            seen.append((a if flags & L.FLAG_DENOISE else None,
                         b if flags & L.FLAG_TEMPORAL_DENOISE else None))
    spatial = {s[0] for s in seen if s[0] is not None}
    temporal = {s[1] for s in seen if s[1] is not None}
    assert len(spatial) == 1 and len(temporal) == 1, seen


def test_autotuned_shapes_survive_many_sizes(ctx):
    """A size's shapes stay those of its live pipelines however many other
    sizes are tuned meanwhile (the tuner's table keeps an entry while a
    pipeline of its size exists), and a later pipeline of the size after
    the others finds them too."""
    w, h = 1030, 614
    flags = L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE
    with L.Pipeline(ctx, L.pipeline_params(w, h, flags=flags)) as held:
        first = held.kernel_config()
        for i in range(48):
            with L.Pipeline(ctx, L.pipeline_params(64 + 2 * i, 34, flags=flags)):
                pass
        with L.Pipeline(ctx, L.pipeline_params(w, h, flags=flags)) as again:
            assert again.kernel_config() == first
    with L.Pipeline(ctx, L.pipeline_params(w, h, flags=flags)) as later:
        assert later.kernel_config() == first


@pytest.mark.parametrize("storage", [L.STORAGE_FP32, L.STORAGE_FP16])
@pytest.mark.parametrize("deb", [L.DEBAYER_BILINEAR, L.DEBAYER_RCD])
@pytest.mark.parametrize("chroma", [False, True])
def test_awb_bit_exact(ctx, deb, storage, chroma):
    """The GPU histogram equals the CPU builder's on the intermediate the
    GPU produced, in all three counters, bit for bit."""
    from gpu_util import download_image
    w, h = 320, 200
    m = frame(w, h, 41 + deb)
    prof = W.make_profile()
    flags = L.FLAG_AWB_HISTOGRAM | L.FLAG_KEEP_INTERMEDIATE | (L.FLAG_CHROMA_DENOISE if chroma else 0)
    pp = L.pipeline_params(w, h, debayer=deb, flags=flags, out_format=L.FORMAT_RGBA32F,
                           storage=storage, nb_awb_slots=2)
    fp = L.frame_params(prof, denoise_chroma_strength=0.5 if chroma else 0.0)
    from gpu_util import upload_mosaic, alloc_rgba
    with L.Pipeline(ctx, pp) as pipe:
        _, src = upload_mosaic(m)
        _, dst = alloc_rgba(w, h)
        pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
        torch.cuda.synchronize()
        rgb_img, _ = pipe.intermediate()
        rgb = download_image(rgb_img, "rgba16f" if storage == L.STORAGE_FP16 else "rgba32f").astype(np.float32)
        hist = pipe.awb_histogram()
    cnt, wgt, brt = L.awb_histogram_from_rgb(rgb, W.WB)
    assert cnt.sum() > 0.5 * (w // 8) * (h // 8)
    assert np.array_equal(hist.count, cnt)
    assert np.array_equal(hist.weight, wgt)
    assert np.array_equal(hist.weight_bright, brt)
    ocnt, _, _ = orc.awb_histogram(rgb, W.WB)
    assert np.array_equal(ocnt, cnt)


def test_awb_many_edge_blocks(ctx):
    """More blocks on AWB bin edges than a slot carries to the host (4096):
    flat 64x64 regions of two colours whose R/G ratio puts ln(R/G) on a bin
    edge to within 1e-6 of a bin, 1024x1024 pixels (16384 blocks). The
    device defers every such block; the histogram is still the CPU
    builder's on the GPU's intermediate, bit for bit (the blocks past the
    slot's 4096 are read from its device list)."""
    from gpu_util import download_image, upload_mosaic, alloc_rgba
    w = h = 1024
    codes = [(519, 1029, 700), (1073, 977, 1300)]   # (R, G, B) raw codes
    m = np.empty((h, w), np.uint16)
    for ry in range(0, h, 64):
        for rx in range(0, w, 64):
            r, g, b = codes[((rx // 64) + (ry // 64)) & 1]
            blk = m[ry:ry + 64, rx:rx + 64]
            blk[0::2, 0::2] = r
            blk[0::2, 1::2] = g
            blk[1::2, 0::2] = g
            blk[1::2, 1::2] = b
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, flags=L.FLAG_AWB_HISTOGRAM | L.FLAG_KEEP_INTERMEDIATE, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof)
    with L.Pipeline(ctx, pp) as pipe:
        _, src = upload_mosaic(m)
        _, dst = alloc_rgba(w, h)
        pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
        torch.cuda.synchronize()
        rgb_img, _ = pipe.intermediate()
        rgb = download_image(rgb_img, "rgba32f").astype(np.float32)
        hist = pipe.awb_histogram()
    # How many blocks lie within the device's deferral margin of a bin edge.
    means = rgb[..., :3].reshape(h // 8, 8, w // 8, 8, 3).astype(np.float64).mean(axis=(1, 3))
    with np.errstate(divide="ignore", invalid="ignore"):
        fx = (np.log(means[..., 0] / W.WB[0] / means[..., 1]) + 2.5) / 3.5 * 128
    near = np.abs(fx - np.rint(fx)) < 2e-4
    assert near.sum() > 4096, near.sum()
    cnt, wgt, brt = L.awb_histogram_from_rgb(rgb, W.WB)
    assert np.array_equal(hist.count, cnt)
    assert np.array_equal(hist.weight, wgt)
    assert np.array_equal(hist.weight_bright, brt)


def test_chroma_vs_oracle(ctx):
    w, h = 240, 160
    c = W.workload("temporal_mhc_p3", w, h)
    m = c.frame()
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_MHC, out_space=L.CS_P3D65,
                           flags=L.FLAG_CHROMA_DENOISE, out_format=L.FORMAT_RGBA32F)
    for s in (0.5, 1.0):
        fp = L.frame_params(prof, denoise_chroma_strength=s)
        got = run(ctx, m, pp, fp)
        ref = orc.process(m, pp, fp, "f32")
        assert max_rel(got, ref) < 2e-4, (s, max_rel(got, ref))


def test_temporal_sequence_vs_oracle(ctx):
    """Five frames with moving rectangles: temporal 0.8 + NLM 1.0; the
    denoised mosaic, the state and the output follow the oracle's chain."""
    from gpu_util import download_image, upload_mosaic, alloc_rgba
    w, h = 160, 112
    c = W.workload("temporal_mhc_p3", w, h)
    prof = W.make_profile()
    model = W.noise_model(c.noise_a_dn, c.noise_b_dn)
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_MHC, out_space=L.CS_P3D65,
                           flags=L.FLAG_DENOISE | L.FLAG_TEMPORAL_DENOISE | L.FLAG_KEEP_INTERMEDIATE,
                           out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, denoise_strength=1.0, denoise_temporal_strength=0.8, noise_override=model)
    prev = None
    with L.Pipeline(ctx, pp) as pipe:
        for f in range(5):
            m = c.frame(f)
            _, src = upload_mosaic(m)
            _, dst = alloc_rgba(w, h)
            pipe.record(torch.cuda.current_stream().cuda_stream, src, dst, fp)
            _, mos = pipe.intermediate()
            got = download_image(mos, "r16")
            lvl, var = pipe.temporal_state()
            glvl = download_image(lvl, "r32f")
            gvar = download_image(var, "r8")
            clean, nxt = orc.denoise_temporal(m, prof, model, 1.0, 0.8, prev)
            d = np.abs(got.astype(np.int32) - clean.astype(np.int32))
            assert d.max() <= 2 and (d > 0).mean() < 0.02, (f, d.max(), (d > 0).mean())
            assert np.max(np.abs(glvl - nxt[0])) < 1e-4, f
            qv = (gvar.astype(np.float32) / 255.0) ** 2
            assert np.max(np.abs(qv - nxt[1])) < 0.01, f
            # Follow the GPU's own state so the comparison does not drift.
            prev = np.stack([glvl, qv]).astype(np.float32)


def test_plain_and_fused_agree(ctx):
    w, h = 256, 144
    c = W.workload("nlm_rcd_ap1", w, h)
    m = c.frame()
    prof = W.make_profile()
    fp = L.frame_params(prof, **c.frame_kwargs())
    outs = []
    for impl in (L.IMPL_FUSED, L.IMPL_PLAIN):
        pp = L.pipeline_params(w, h, debayer=c.debayer, out_space=c.out_space, flags=c.flags,
                               out_format=L.FORMAT_RGBA32F, impl=impl)
        outs.append(run(ctx, m, pp, fp))
    ok, st = denoised_chain_ok(outs[0], outs[1])
    assert ok, st


def test_rgba16f_output(ctx):
    w, h = 128, 96
    m = frame(w, h, 51)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_BT2020,
                           out_format=L.FORMAT_RGBA16F)
    fp = L.frame_params(prof)
    got = run(ctx, m, pp, fp, L.FORMAT_RGBA16F)
    ref = orc.process(m, pp, fp, "f32")
    assert max_rel(got, ref) < 3e-3


def test_frame_options_vs_oracle(ctx):
    """Rebalance to an illuminant, exposure, clamp, the output-space
    override and the RGC veto."""
    import golden.make_golden as MG
    w, h = 128, 96
    m = frame(w, h, 61)
    prof = MG.golden_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_MHC, out_space=L.CS_XYZ_D65,
                           out_format=L.FORMAT_RGBA32F)
    cases = [
        dict(wb_mode=L.WB_REBALANCE, illuminant=(3200.0, 0.02)),
        dict(exposure_stops=1.5, flags=L.FRAME_CLAMP_NEGATIVE),
        dict(out_space=L.CS_ACES_AP1, out_space_set=True),
        dict(out_space=L.CS_ACES_AP1, out_space_set=True, flags=L.FRAME_NO_GAMUT_COMPRESSION),
        dict(out_space=L.CS_V_GAMUT, out_space_set=True),
    ]
    for kw in cases:
        fp = L.frame_params(prof, **kw)
        got = run(ctx, m, pp, fp)
        ref = orc.process(m, pp, fp, "f32")
        assert max_rel(got, ref) < 2e-4, (kw, max_rel(got, ref))


@pytest.mark.parametrize("wh", [(8, 8), (16, 10), (24, 24), (62, 46), (1030, 18)])
def test_edge_sizes(ctx, wh):
    """Frames smaller than a tile or an apron, and ragged last tiles."""
    w, h = wh
    m = frame(w, h, 71)
    prof = W.make_profile()
    for deb in (0, 1, 2):
        pp = L.pipeline_params(w, h, debayer=deb, out_space=L.CS_BT709, out_format=L.FORMAT_RGBA32F,
                               flags=L.FLAG_AWB_HISTOGRAM)
        fp = L.frame_params(prof)
        got = run(ctx, m, pp, fp)
        ref = orc.process(m, pp, fp, "f32")
        assert max_rel(got, ref) < TOL_FP32[deb], (wh, deb, max_rel(got, ref))
    if w >= 12 and h >= 12:
        pp = L.pipeline_params(w, h, debayer=2, flags=L.FLAG_DENOISE, out_format=L.FORMAT_RGBA32F)
        fp = L.frame_params(prof, denoise_strength=1.0, noise_override=W.noise_model(4, 40))
        got = run(ctx, m, pp, fp)
        ok, st = denoised_chain_ok(got, orc.process(m, pp, fp, "f32"))
        assert ok, (wh, st)


@pytest.mark.parametrize("wh", [(640, 352), (518, 262)])
def test_rcd_quad_tiles_vs_oracle(ctx, wh):
    """Frames where most RCD tiles are interior (the quad kernel) and the
    rest, including ragged last tiles, go through the per-pixel kernel."""
    w, h = wh
    m = frame(w, h, 81)
    prof = W.make_profile()
    pp = L.pipeline_params(w, h, debayer=L.DEBAYER_RCD, out_space=L.CS_XYZ_D65,
                           out_format=L.FORMAT_RGBA32F, flags=L.FLAG_AWB_HISTOGRAM)
    fp = L.frame_params(prof)
    got = run(ctx, m, pp, fp)
    ref = orc.process(m, pp, fp, "f32")
    assert max_rel(got, ref) < TOL_FP32[L.DEBAYER_RCD], max_rel(got, ref)
    assert max_rel(got, orc.process(m, pp, fp, "f64")) < 1e-3
