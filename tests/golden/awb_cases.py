"""Seeded inputs of the AWB estimator, smoother and locus tests, shared by
the fixture generator (make_golden.py) and the tests. Every function takes
the C library that answers the locus questions (the reference's build or
this project's), so that histograms are placed from the same numbers."""
from __future__ import annotations

import ctypes as C

import numpy as np

import libcraw_gb300 as L

BINS = L.AWB_BINS
LMIN, LMAX = -2.5, 1.0


def bind(lib):
    """Gives `lib` (a CDLL of either build) the ctypes signatures of the
    locus, estimator and smoother functions; returns it."""
    for name, (res, args) in L.awb_signatures().items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def neutral(lib, prof, cct, tint=0.0):
    rg, bg = C.c_float(), C.c_float()
    assert lib.craw_profile_illuminant_to_neutral(C.byref(prof), C.byref(L.Illuminant(cct, tint)),
                                                  C.byref(rg), C.byref(bg)) == 0
    return rg.value, bg.value


def bin_of(rg, bg):
    ix = int(np.floor((np.log(rg) - LMIN) / (LMAX - LMIN) * BINS))
    iy = int(np.floor((np.log(bg) - LMIN) / (LMAX - LMIN) * BINS))
    return min(max(iy, 0), BINS - 1), min(max(ix, 0), BINS - 1)


def _empty():
    return [np.zeros((BINS, BINS), np.uint32) for _ in range(3)]


def _cluster(h, lib, prof, rng, cct, tint, n, spread, g_lo, g_hi, bright_boost=1.0):
    cnt, wgt, brt = h
    rg0, bg0 = neutral(lib, prof, cct, tint)
    for _ in range(n):
        rg = rg0 * np.exp(rng.normal(0.0, spread))
        bg = bg0 * np.exp(rng.normal(0.0, spread))
        iy, ix = bin_of(rg, bg)
        g = rng.uniform(g_lo, g_hi)
        cnt[iy, ix] += 1
        wgt[iy, ix] += int(round(min(g, 0.5) * 65536))
        brt[iy, ix] += int(round(g ** 4 * 65536 * bright_boost))


def _clutter(h, rng, n):
    cnt, wgt, brt = h
    for _ in range(n):
        iy, ix = rng.integers(0, BINS, 2)
        g = rng.uniform(0.01, 0.9)
        cnt[iy, ix] += 1
        wgt[iy, ix] += int(round(min(g, 0.5) * 65536))
        brt[iy, ix] += int(round(g ** 4 * 65536))


def histogram_cases(lib, prof):
    """(name, count, weight, weight_bright or None, params kwargs)."""
    out = []
    rng = np.random.default_rng(7001)
    for cct in (2700.0, 4300.0, 6500.0, 9000.0):
        h = _empty()
        _cluster(h, lib, prof, rng, cct, 0.0, 400, 0.03, 0.05, 0.6)
        _clutter(h, rng, 150)
        out.append((f"cluster_{int(cct)}", *h, {}))
    h = _empty()
    _cluster(h, lib, prof, rng, 6500.0, 0.04, 600, 0.04, 0.05, 0.4)
    _cluster(h, lib, prof, rng, 3000.0, -0.02, 60, 0.01, 0.7, 0.95, bright_boost=4.0)
    out.append(("bright_source", *h, {}))
    out.append(("bright_source_no_prefer", *h, {"prefer_bright": False}))
    out.append(("bright_source_no_bright_counter", h[0], h[1], None, {}))
    h = _empty()
    _cluster(h, lib, prof, rng, 2600.0, 0.0, 500, 0.02, 0.1, 0.5)
    out.append(("warm_ambience", *h, {"ambience": 0.6}))
    out.append(("warm_clamped", *h, {"cct_min": 3200.0, "cct_max": 6000.0}))
    out.append(("warm_inverted_clamps", *h, {"cct_min": 5000.0, "cct_max": 4000.0}))
    h = _empty()
    _clutter(h, rng, 40)
    out.append(("clutter_only", *h, {}))
    out.append(("clutter_narrow_band", *h, {"band": 0.01, "sigma": 0.2, "min_zone_fraction": 0.5}))
    h = _empty()
    out.append(("empty", *h, {}))
    return out


def smoother_cases(seed=7101):
    """(name, params or None, seed illuminant or None, events). An event is
    ("push", pts, valid, cct, tint, confidence, scene_cut) or ("reset",)."""
    rng = np.random.default_rng(seed)
    cases = []
    for name, params, seed_il in (
            ("default", None, None),
            ("fast", (0.5, 0.0, 100.0, 0.5), None),
            ("seeded", None, (5200.0, 0.01)),
            ("slow_hysteresis", (2.0, 10.0, 15.0, 0.1), (3000.0, 0.0))):
        ev = []
        pts = 0.0
        for i in range(60):
            r = rng.uniform()
            if r < 0.05:
                pts -= 0.1                   # a step backwards
            elif r < 0.1:
                pts += 3.0                   # a gap longer than the 1 s clamp
            else:
                pts += 1.0 / 24
            if i == 35:
                ev.append(("reset",))
            valid = bool(rng.uniform() < 0.8)
            cct = float(rng.uniform(2500.0, 8000.0)) if rng.uniform() < 0.3 else 5000.0 + float(rng.normal(0, 300))
            ev.append(("push", pts, valid, cct, float(rng.normal(0, 0.02)), float(rng.uniform()),
                       bool(rng.uniform() < 0.05)))
        # Before any track: an invalid estimate first.
        ev.insert(0, ("push", -0.5, False, 4000.0, 0.0, 0.9, False))
        cases.append((name, params, seed_il, ev))
    return cases


def run_smoother(lib, params, seed_il, events):
    """Drives one smoother through `events`; returns (ret, cct, tint) rows."""
    sp = None
    if params is not None:
        sp = L.AwbSmootherParams(*params)
    sm = L.AwbSmoother(sp, library=lib)
    if seed_il is not None:
        sm.set(0.0, L.Illuminant(*seed_il))
    rows = []
    for e in events:
        if e[0] == "reset":
            sm.reset()
            continue
        _, pts, valid, cct, tint, conf, cut = e
        est = L.AwbEstimate()
        est.valid = valid
        est.illuminant = L.Illuminant(cct, tint)
        est.confidence = conf
        ret, il = sm.push(pts, est, cut)
        rows.append((ret, il.cct, il.tint))
    sm.close()
    return np.array(rows, np.float64)


def locus_points(seed=7201, n=600):
    """(rg, bg) raw ratio pairs: along and across the locus, past both ends,
    and a few invalid ones."""
    rng = np.random.default_rng(seed)
    pts = np.exp(rng.uniform(-2.0, 0.6, size=(n, 2))).astype(np.float32)
    extra = np.array([[0.0, 0.5], [0.5, -1.0], [np.inf, 0.5], [np.nan, 0.4], [1e-30, 1e30],
                      [0.3, 0.3]], np.float32)
    return np.concatenate([pts, extra])


def estimate_row(e: L.AwbEstimate) -> np.ndarray:
    """Every field of an estimate as float64, for exact comparison."""
    f = [e.valid, e.illuminant.cct, e.illuminant.tint, e.confidence, e.in_zone_fraction,
         e.spread_mired, e.source]
    for c in (e.zone, e.bright):
        f += [c.valid, c.illuminant.cct, c.illuminant.tint, c.in_zone_fraction, c.spread_mired]
    return np.array(f, np.float64)


def run_estimates(lib, prof):
    rows = []
    for name, cnt, wgt, brt, kw in histogram_cases(lib, prof):
        params = L.AwbParams()
        lib.craw_awb_params_init(C.byref(params))
        for k, v in kw.items():
            setattr(params, k, v)
        est = L.awb_estimate(prof, cnt, wgt, brt, params, library=lib)
        rows.append(estimate_row(est))
    return np.array(rows)


def run_locus(lib, prof):
    rows = []
    for rg, bg in locus_points():
        il = L.Illuminant()
        ret = lib.craw_profile_neutral_to_illuminant(C.byref(prof), float(rg), float(bg), C.byref(il))
        r2, b2 = C.c_float(), C.c_float()
        ret2 = lib.craw_profile_illuminant_to_neutral(C.byref(prof), C.byref(il), C.byref(r2),
                                                      C.byref(b2)) if ret == 0 else ret
        rows.append((ret, il.cct if ret == 0 else 0.0, il.tint if ret == 0 else 0.0, ret2,
                     r2.value if ret == 0 else 0.0, b2.value if ret == 0 else 0.0))
    return np.array(rows, np.float64)
