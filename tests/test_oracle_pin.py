"""Pins the CPU oracle: its float instantiation must reproduce the
reference's own CPU implementation bit for bit, against the committed
golden fixtures (tests/golden/reference_outputs.npz, made by
tests/golden/make_golden.py from oracle/_ref) and, where the reference was
built here, against oracle/_ref directly on more seeded cases. Its double
instantiation must agree with the float one to float accuracy.
Also checks the product's host constants (libcraw.so) against the same
fixtures."""
from pathlib import Path

import numpy as np
import pytest

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from oracle import Oracle, Reference, reference_available, max_rel

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_outputs.npz")
import golden.make_golden as MG  # noqa: E402

orc = Oracle()
needs_ref = pytest.mark.skipif(not reference_available(), reason="reference build absent")


@pytest.mark.parametrize("case", MG.PROCESS_CASES, ids=[c[0] for c in MG.PROCESS_CASES])
def test_process_golden(case):
    name, w, h, seed, deb, cs, flags, kw = case
    prof = MG.golden_profile()
    m = GOLD[f"process/{name}/in"]
    pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, flags=flags, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, noise_override=W.noise_model(4.0, 40.0), **kw)
    got = orc.process(m, pp, fp, "f32")
    assert np.array_equal(got, GOLD[f"process/{name}/out"])
    # The double run is the same algorithm: float-level agreement.
    assert max_rel(orc.process(m, pp, fp, "f64"), got) < 2e-3


def test_temporal_golden():
    prof = MG.golden_profile()
    model = W.noise_model(4.0, 40.0)
    prev = None
    for f in range(3):
        clean, nxt = orc.denoise_temporal(GOLD[f"temporal/{f}/in"], prof, model, 1.0, 0.8, prev)
        assert np.array_equal(clean, GOLD[f"temporal/{f}/clean"])
        assert np.array_equal(nxt, GOLD[f"temporal/{f}/state"])
        prev = nxt
    clean, _ = orc.denoise_temporal(GOLD["temporal_only/in"], prof, model, 0.0, 0.6, None)
    assert np.array_equal(clean, GOLD["temporal_only/clean"])


@pytest.mark.parametrize("case", MG.HL_CASES, ids=[c[0] for c in MG.HL_CASES])
def test_highlights_golden(case):
    """The highlight reconstruction restated (lib/ref/ref_highlight.c): the
    rebuilt fp16 mosaic bit for bit, and the double run within fp16
    rounding of it."""
    name, w, h, seed, wb = case
    prof = MG.golden_profile()
    m = GOLD[f"highlights/{name}/in"]
    got = orc.highlights(m, prof, wb, "f32")
    assert np.array_equal(got, GOLD[f"highlights/{name}/out"])
    # The frame is clipped and the pass lifted it past the clip point.
    assert (m == W.WHITE_DN).mean() > 0.05 and got.max() > 1.2
    d = orc.highlights(m, prof, wb, "f64")
    assert np.max(np.abs(d - got) / np.maximum(np.abs(got), 1e-3)) < 2e-3


def test_highlights_process_golden():
    prof = MG.golden_profile()
    m = GOLD["highlights/process/in"]
    pp = L.pipeline_params(64, 48, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                           flags=L.FLAG_HIGHLIGHT_RECONSTRUCTION, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION)
    assert np.array_equal(orc.process(m, pp, fp, "f32"), GOLD["highlights/process/out"])
    # The frame flag alone switches the pass: without it, the plain prep.
    fp0 = L.frame_params(prof)
    assert not np.array_equal(orc.process(m, pp, fp0, "f32"), GOLD["highlights/process/out"])


@needs_ref
def test_highlights_against_reference_build():
    prof = MG.golden_profile()
    ref = Reference()
    for seed, (w, h) in enumerate([(64, 48), (98, 66), (160, 120), (8, 8)]):
        m = W.highlight_frame(w, h, 500 + seed)
        for wb in ((2.0, 1.0, 1.5), (1.3, 1.0, 2.6)):
            assert np.array_equal(orc.highlights(m, prof, wb, "f32"), ref.highlights(m, prof, wb)), (w, h, wb)


def test_awb_golden():
    rgb = GOLD["awb/rgb"]
    for impl in (orc.awb_histogram(rgb, W.WB), L.awb_histogram_from_rgb(rgb, W.WB)):
        for got, key in zip(impl, ("count", "weight", "weight_bright")):
            assert np.array_equal(got, GOLD[f"awb/{key}"]), key
    assert GOLD["awb/count"].sum() == (64 // 8) * (48 // 8) - 0 or GOLD["awb/count"].sum() > 0


def test_host_constants_golden():
    """The product's host math (libcraw.so) against the reference's."""
    for cs in range(7):
        assert np.array_equal(L.colorspace_from_xyz_d65(cs), GOLD[f"cs/{cs}/from"]), cs
        assert np.array_equal(L.colorspace_to_xyz_d65(cs), GOLD[f"cs/{cs}/to"]), cs
    knots = MG.NOISE_KNOTS
    for iso, (a, b) in zip(GOLD["noise/iso"], GOLD["noise/model"]):
        nm = L.noise_model_eval(knots, float(iso))
        assert (np.float32(nm.a), np.float32(nm.b)) == (a, b), iso
    prof = MG.golden_profile()
    for (cct, tint), ev in zip(GOLD["profile/illuminants"], GOLD["profile/eval"]):
        cp = L.profile_eval(prof, L.WB_REBALANCE, L.Illuminant(float(cct), float(tint)))
        got = np.array(list(cp.wb) + [x for row in cp.cam_to_xyz for x in row] + [cp.gain], np.float32)
        assert np.array_equal(got, ev), (cct, tint)
    for t, xy in zip(GOLD["planck/cct"], GOLD["planck/xy"]):
        assert np.array_equal(np.array(L.planckian_xy(float(t)), np.float32), xy)
    assert np.array_equal(L.bradford_adaptation((0.3457, 0.3585), (0.3127, 0.3290)),
                          GOLD["bradford/d50_d65"])


def test_oracle_gamut_constants_golden():
    import ctypes as C
    from oracle import GamutParams
    g = GamutParams()
    orc.lib.orc_gamut_params(C.byref(g))
    got = np.array(list(g.thr) + list(g.scl) + [g.pwr, g.inv_pwr], np.float32)
    assert np.array_equal(got, GOLD["gamut"])


def test_profile_errors():
    p = L.profile_init()
    L.profile_validate(p)
    with pytest.raises(L.CrawError) as e:
        L.profile_eval(p, L.WB_REBALANCE, L.Illuminant(5000.0, 0.0))
    assert e.value.errno == 95  # ENOTSUP: no white balance table
    p.white_level[2] = 0.0
    with pytest.raises(L.CrawError):
        L.profile_validate(p)
    with pytest.raises(L.CrawError):
        L.profile_noise_eval(L.profile_init())


# ------------------------------------------------ against the reference build

@needs_ref
@pytest.mark.parametrize("deb", [L.DEBAYER_BILINEAR, L.DEBAYER_MHC, L.DEBAYER_RCD])
@pytest.mark.parametrize("cs", [L.CS_XYZ_D65, L.CS_BT709, L.CS_V_GAMUT, L.CS_ACES_AP1])
def test_process_vs_reference(deb, cs):
    ref = Reference()
    prof = W.make_profile()
    rng = np.random.default_rng(deb * 10 + cs)
    w, h = 2 * int(rng.integers(10, 40)), 2 * int(rng.integers(10, 30))
    m = W.synth_frame(w, h, 1000 + deb * 10 + cs, rects=6, zone_plates=1, noise_a_dn=6, noise_b_dn=60)
    flags = L.FLAG_DENOISE | L.FLAG_CHROMA_DENOISE
    pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, flags=flags, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, noise_override=W.noise_model(6, 60), denoise_strength=0.7,
                        denoise_chroma_strength=0.8, exposure_stops=-0.5)
    assert np.array_equal(orc.process(m, pp, fp), ref.process(m, pp, fp))


@needs_ref
def test_tiny_and_odd_stencil_frames_vs_reference():
    """Frames smaller than the RCD apron exercise the repeated mirror."""
    ref = Reference()
    prof = W.make_profile()
    for w, h in ((8, 8), (10, 12), (16, 8)):
        m = W.synth_frame(w, h, 7, rects=1, zone_plates=0)
        for deb in (0, 1, 2):
            pp = L.pipeline_params(w, h, debayer=deb, out_space=L.CS_BT709, out_format=L.FORMAT_RGBA32F)
            fp = L.frame_params(prof)
            assert np.array_equal(orc.process(m, pp, fp), ref.process(m, pp, fp)), (w, h, deb)


@needs_ref
def test_temporal_vs_reference_reset_and_strengths():
    ref = Reference()
    prof = W.make_profile()
    model = W.noise_model(8, 80)
    pa = pb = None
    for f, (s, a) in enumerate([(1.0, 0.8), (1.0, 0.8), (0.0, 0.5), (2.0, 1.0), (1.0, 0.8)]):
        m = W.synth_frame(40, 36, 77, frame=f, rects=4, noise_a_dn=8, noise_b_dn=80,
                          movers=[(2, 0.5), (8, 2.0)])
        if f == 4:
            pa = pb = None  # a reset
        ca, na = ref.denoise_temporal(m, prof, model, s, a, pa)
        cb, nb = orc.denoise_temporal(m, prof, model, s, a, pb)
        assert np.array_equal(ca, cb) and np.array_equal(na, nb), f
        pa, pb = na, nb
