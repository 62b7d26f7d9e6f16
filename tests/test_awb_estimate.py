"""The AWB estimator, the per-stream smoother and the locus conversions of
libcraw.so against the reference's own code (lib/awb.c, lib/awb_smoother.c,
lib/profile.c): bit for bit against the committed fixtures made from the
reference's build (tests/golden/make_golden.py), and against that build
directly where it is present. CPU only."""
import ctypes as C
import errno
from pathlib import Path

import numpy as np
import pytest

import libcraw_gb300 as L
import golden.awb_cases as AC
import golden.make_golden as MG
from oracle import REF_SO, reference_available

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_outputs.npz")
needs_ref = pytest.mark.skipif(not reference_available(), reason="reference build absent")
PROF = MG.golden_profile()


def ours():
    return AC.bind(L.lib())


def ref():
    return AC.bind(C.CDLL(str(REF_SO)))


def test_locus_golden():
    got = AC.run_locus(ours(), PROF)
    assert np.array_equal(got, GOLD["locus/rows"], equal_nan=True)
    # Inside the table the two conversions invert each other.
    ok = got[:, 0] == 0
    assert ok.sum() > 500


def test_locus_round_trip():
    lib = ours()
    for cct in (2500.0, 2900.0, 4000.0, 4711.0, 5500.0, 7499.0):
        for tint in (-0.05, 0.0, 0.03):
            rg, bg = AC.neutral(lib, PROF, cct, tint)
            il = L.Illuminant()
            assert lib.craw_profile_neutral_to_illuminant(C.byref(PROF), rg, bg, C.byref(il)) == 0
            assert abs(il.cct - cct) < 1e-2 * cct / 1000 + 0.05, (cct, il.cct)
            assert abs(il.tint - tint) < 1e-5


def test_locus_errors():
    lib = ours()
    il = L.Illuminant()
    assert lib.craw_profile_neutral_to_illuminant(C.byref(PROF), 0.0, 1.0, C.byref(il)) == -errno.EINVAL
    one = MG.golden_profile()
    one.nb_wb_knots = 1
    assert lib.craw_profile_neutral_to_illuminant(C.byref(one), 0.5, 0.5, C.byref(il)) == -errno.ENOTSUP
    none = MG.golden_profile()
    none.nb_wb_knots = 0
    r, b = C.c_float(), C.c_float()
    assert lib.craw_profile_illuminant_to_neutral(C.byref(none), C.byref(L.Illuminant(5000, 0)),
                                                  C.byref(r), C.byref(b)) == -errno.ENOTSUP
    assert lib.craw_profile_illuminant_to_neutral(C.byref(PROF), C.byref(L.Illuminant(float("nan"), 0)),
                                                  C.byref(r), C.byref(b)) == -errno.EINVAL


def golden_histograms():
    for name, _, _, _, kw in AC.histogram_cases(ref() if reference_available() else ours(), PROF):
        brt = GOLD[f"awb_est/{name}/weight_bright"] if f"awb_est/{name}/weight_bright" in GOLD.files else None
        yield name, GOLD[f"awb_est/{name}/count"], GOLD[f"awb_est/{name}/weight"], brt, kw


def test_estimate_golden():
    lib = ours()
    rows = []
    for name, cnt, wgt, brt, kw in golden_histograms():
        est = L.awb_estimate(PROF, cnt, wgt, brt, L.awb_params(**kw), library=lib)
        rows.append(AC.estimate_row(est))
    rows = np.array(rows)
    assert np.array_equal(rows, GOLD["awb_est/rows"], equal_nan=True), \
        np.argwhere(rows != GOLD["awb_est/rows"])[:5]
    # The readings cover every source and both outcomes.
    assert set(rows[:, 6]) == {0.0, 1.0, 2.0}
    assert set(rows[:, 0]) == {0.0, 1.0}


def test_estimate_of_a_developed_frame_golden():
    """The estimate from the histogram of a developed synthetic frame (its
    coloured rectangles put almost nothing inside the neutral band)."""
    lib, r = ours(), None
    est = L.awb_estimate(PROF, GOLD["awb/count"], GOLD["awb/weight"], GOLD["awb/weight_bright"],
                         library=lib)
    if reference_available():
        r = L.awb_estimate(PROF, GOLD["awb/count"], GOLD["awb/weight"], GOLD["awb/weight_bright"],
                           library=ref())
        assert np.array_equal(AC.estimate_row(est), AC.estimate_row(r), equal_nan=True)


def test_estimate_errors():
    lib = ours()
    z = np.zeros((L.AWB_BINS, L.AWB_BINS), np.uint32)
    one = MG.golden_profile()
    one.nb_wb_knots = 1
    with pytest.raises(L.CrawError) as e:
        L.awb_estimate(one, z, z, z, library=lib)
    assert e.value.errno == errno.ENOTSUP
    with pytest.raises(L.CrawError) as e:
        L.awb_estimate(PROF, z, z, z, L.awb_params(band=0.0), library=lib)
    assert e.value.errno == errno.EINVAL
    with pytest.raises(L.CrawError) as e:
        L.awb_estimate(PROF, z, z, z, log_min=1.0, log_max=1.0, library=lib)
    assert e.value.errno == errno.EINVAL
    est = L.awb_estimate(PROF, z, z, z, library=lib)
    assert not est.valid and est.source == 0


@pytest.mark.parametrize("case", AC.smoother_cases(), ids=[c[0] for c in AC.smoother_cases()])
def test_smoother_golden(case):
    name, params, seed_il, ev = case
    got = AC.run_smoother(ours(), params, seed_il, ev)
    assert np.array_equal(got, GOLD[f"awb_smooth/{name}"], equal_nan=True)
    assert got[0, 0] == -errno.EAGAIN or seed_il is not None


def test_smoother_params():
    lib = ours()
    for bad in ((0.0, 3.0, 30.0, 0.2), (1.0, -1.0, 30.0, 0.2), (1.0, 3.0, 0.0, 0.2),
                (float("inf"), 3.0, 30.0, 0.2), (1.0, 3.0, 30.0, float("nan"))):
        with pytest.raises(L.CrawError) as e:
            L.AwbSmoother(L.AwbSmootherParams(*bad), library=lib)
        assert e.value.errno == errno.EINVAL
    p = L.AwbSmootherParams()
    lib.craw_awb_smoother_params_init(C.byref(p))
    assert (p.time_constant, p.hysteresis_mired, p.max_slew_mired_per_s) == (1.0, 3.0, 30.0)


@needs_ref
def test_against_reference_build_more_cases():
    """More seeds than the fixtures hold, straight against the reference."""
    a, b = ours(), ref()
    for seed in range(5):
        for name, params, seed_il, ev in AC.smoother_cases(seed=900 + seed):
            assert np.array_equal(AC.run_smoother(a, params, seed_il, ev),
                                  AC.run_smoother(b, params, seed_il, ev), equal_nan=True), name
        pts = AC.locus_points(seed=950 + seed, n=300)
        for rg, bg in pts[:300]:
            ia, ib = L.Illuminant(), L.Illuminant()
            ra = a.craw_profile_neutral_to_illuminant(C.byref(PROF), float(rg), float(bg), C.byref(ia))
            rb = b.craw_profile_neutral_to_illuminant(C.byref(PROF), float(rg), float(bg), C.byref(ib))
            assert (ra, ia.cct, ia.tint) == (rb, ib.cct, ib.tint)
