"""Generates the golden fixtures in tests/golden/ from the reference's own
CPU implementation (lib/ref and its host code, compiled from the reference
tree by oracle/build_ref.sh into oracle/_ref/libcraw_ref.so).

Inputs are small seeded synthetic frames (libcraw_gb300.workloads); the
fixtures hold the inputs and the reference's outputs, so that the oracle
restatement can be pinned without the reference tree (e.g. on a machine
where it is not mounted).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import libcraw_gb300 as L  # noqa: E402
from libcraw_gb300 import build as B  # noqa: E402
from libcraw_gb300 import workloads as W  # noqa: E402
from oracle import GamutParams, Reference  # noqa: E402

#: Frame cases of craw_ref_process: (name, w, h, seed, debayer, space, flags, frame kwargs)
PROCESS_CASES = [
    ("bilinear_bt709", 64, 48, 101, L.DEBAYER_BILINEAR, L.CS_BT709, L.FLAG_AWB_HISTOGRAM, {}),
    ("mhc_xyz_exposure", 64, 48, 102, L.DEBAYER_MHC, L.CS_XYZ_D65, 0,
     {"exposure_stops": 0.75, "flags": L.FRAME_CLAMP_NEGATIVE}),
    ("rcd_nlm_ap1", 64, 48, 103, L.DEBAYER_RCD, L.CS_ACES_AP1, L.FLAG_DENOISE,
     {"denoise_strength": 1.0}),
    ("rcd_nlm2_ap0", 64, 48, 104, L.DEBAYER_RCD, L.CS_ACES_AP0, L.FLAG_DENOISE,
     {"denoise_strength": 2.0}),
    ("mhc_chroma_p3", 64, 48, 105, L.DEBAYER_MHC, L.CS_P3D65, L.FLAG_CHROMA_DENOISE,
     {"denoise_chroma_strength": 0.5}),
    ("bilinear_rebalance_bt2020", 64, 48, 106, L.DEBAYER_BILINEAR, L.CS_BT2020, 0,
     {"wb_mode": L.WB_REBALANCE, "illuminant": (3900.0, 0.03)}),
]

#: Highlight reconstruction cases: (name, w, h, seed, white balance).
HL_CASES = [("as_shot", 96, 64, 401, (2.0, 1.0, 1.5)), ("warm", 130, 78, 402, (1.7, 1.0, 2.2))]

#: A white balance / matrix table of this project's own, for the rebalance cases.
WB_KNOTS = [(2500.0, (1.05, 1.0, 3.10)), (4000.0, (1.55, 1.0, 2.05)), (5500.0, (2.00, 1.0, 1.50)),
            (7500.0, (2.40, 1.0, 1.25))]
M_KNOTS = [(3000.0, ((0.66, 0.19, 0.1005), (0.29, 0.71, 0.0), (0.01, -0.09, 1.169))),
           (6500.0, ((0.70, 0.145, 0.1055), (0.30, 0.78, -0.08), (0.005, 0.07, 1.014)))]
NOISE_KNOTS = [(100.0, 2.0e-5, 1.0e-7), (400.0, 8.5e-5, 6.0e-7), (1600.0, 3.3e-4, 5.5e-6),
               (6400.0, 1.4e-3, 0.0)]


def golden_profile() -> L.Profile:
    p = W.make_profile()
    for i, (cct, wb) in enumerate(WB_KNOTS):
        p.wb_knots[i].cct = cct
        for c in range(3):
            p.wb_knots[i].wb[c] = wb[c]
    p.nb_wb_knots = len(WB_KNOTS)
    for i, (cct, m) in enumerate(M_KNOTS):
        p.matrix_knots[i].cct = cct
        for r in range(3):
            for c in range(3):
                p.matrix_knots[i].m[r][c] = m[r][c]
    p.nb_matrix_knots = len(M_KNOTS)
    return p


def frame(w, h, seed, **kw):
    return W.synth_frame(w, h, seed, rects=8, zone_plates=1, noise_a_dn=4.0, noise_b_dn=40.0, **kw)


def main() -> None:
    B.build(with_reference=True)
    ref = Reference()
    prof = golden_profile()
    model = W.noise_model(4.0, 40.0)
    out: dict[str, np.ndarray] = {}

    for name, w, h, seed, deb, cs, flags, kw in PROCESS_CASES:
        m = frame(w, h, seed)
        pp = L.pipeline_params(w, h, debayer=deb, out_space=cs, flags=flags,
                               out_format=L.FORMAT_RGBA32F)
        fp = L.frame_params(prof, noise_override=model, **kw)
        out[f"process/{name}/in"] = m
        out[f"process/{name}/out"] = ref.process(m, pp, fp)

    # A temporal sequence: NLM 1.0 + temporal 0.8, three frames with movers.
    prev = None
    for f in range(3):
        m = frame(48, 40, 201, frame=f, movers=[(2.0, 0.5), (8.0, 2.0), (24.0, 10.0)])
        clean, nxt = ref.denoise_temporal(m, prof, model, 1.0, 0.8, prev)
        out[f"temporal/{f}/in"] = m
        out[f"temporal/{f}/clean"] = clean
        out[f"temporal/{f}/state"] = nxt
        prev = nxt
    # The temporal average alone.
    m = frame(48, 40, 202)
    clean, nxt = ref.denoise_temporal(m, prof, model, 0.0, 0.6, None)
    out["temporal_only/in"] = m
    out["temporal_only/clean"] = clean

    # AWB histogram of an intermediate (an RCD debayer of a frame).
    m = frame(64, 48, 301)
    rgb = ref.debayer_wb(m, prof, W.WB, L.DEBAYER_RCD)
    cnt, wgt, brt = ref.awb_histogram(rgb, W.WB)
    out["awb/rgb"] = rgb
    out["awb/count"], out["awb/weight"], out["awb/weight_bright"] = cnt, wgt, brt

    # Highlight reconstruction (lib/ref/ref_highlight.c): the rebuilt mosaic,
    # and a whole frame through it.
    for name, w, h, seed, wb in HL_CASES:
        m = W.highlight_frame(w, h, seed)
        out[f"highlights/{name}/in"] = m
        out[f"highlights/{name}/out"] = ref.highlights(m, prof, wb)
    m = W.highlight_frame(64, 48, 404)
    pp = L.pipeline_params(64, 48, debayer=L.DEBAYER_RCD, out_space=L.CS_ACES_AP1,
                           flags=L.FLAG_HIGHLIGHT_RECONSTRUCTION, out_format=L.FORMAT_RGBA32F)
    fp = L.frame_params(prof, flags=L.FRAME_HIGHLIGHT_RECONSTRUCTION)
    out["highlights/process/in"] = m
    out["highlights/process/out"] = ref.process(m, pp, fp)

    # Host constants.
    for cs in range(7):
        a, b = (C.c_float * 9)(), (C.c_float * 9)()
        assert ref.lib.craw_colorspace_from_xyz_d65(cs, C.byref(a)) == 0
        assert ref.lib.craw_colorspace_to_xyz_d65(cs, C.byref(b)) == 0
        out[f"cs/{cs}/from"] = np.array(a[:], np.float32).reshape(3, 3)
        out[f"cs/{cs}/to"] = np.array(b[:], np.float32).reshape(3, 3)
    g = GamutParams()
    ref.lib.craw_gamut_compress_params(C.byref(g))
    out["gamut"] = np.array(list(g.thr) + list(g.scl) + [g.pwr, g.inv_pwr], np.float32)
    knots = (L.NoiseKnot * 4)(*[L.NoiseKnot(*k) for k in NOISE_KNOTS])
    isos = np.array([0.0, 50.0, 100.0, 250.0, 400.0, 900.0, 3200.0, 6400.0, 12800.0], np.float32)
    nm = []
    for iso in isos:
        r = L.NoiseModel()
        assert ref.lib.craw_noise_model_eval(knots, 4, float(iso), C.byref(r)) == 0
        nm.append((r.a, r.b))
    out["noise/iso"] = isos
    out["noise/model"] = np.array(nm, np.float32)
    ills = np.array([(1800.0, 0.0), (2500.0, 0.0), (3300.0, -0.05), (5500.0, 0.0), (6100.0, 0.08),
                     (9000.0, 0.0)], np.float32)
    evals = []
    for cct, tint in ills:
        cp = L.ColorParams()
        assert ref.lib.craw_profile_eval(C.byref(prof), L.WB_REBALANCE,
                                         C.byref(L.Illuminant(float(cct), float(tint))), C.byref(cp)) == 0
        evals.append(list(cp.wb) + [x for row in cp.cam_to_xyz for x in row] + [cp.gain])
    out["profile/illuminants"] = ills
    out["profile/eval"] = np.array(evals, np.float32)
    ccts = np.array([1000.0, 2856.0, 4000.0, 6504.0, 10000.0, 15000.0], np.float32)
    xy = []
    for t in ccts:
        v = (C.c_float * 2)()
        assert ref.lib.craw_planckian_xy(float(t), C.byref(v)) == 0
        xy.append(v[:])
    out["planck/cct"] = ccts
    out["planck/xy"] = np.array(xy, np.float32)
    m9 = (C.c_float * 9)()
    assert ref.lib.craw_bradford_adaptation(C.byref((C.c_float * 2)(0.3457, 0.3585)),
                                            C.byref((C.c_float * 2)(0.3127, 0.3290)), C.byref(m9)) == 0
    out["bradford/d50_d65"] = np.array(m9[:], np.float32).reshape(3, 3)

    # AWB estimator, smoother and the locus conversions they stand on
    # (reference lib/awb.c, lib/awb_smoother.c, lib/profile.c).
    import awb_cases as AC
    AC.bind(ref.lib)
    for name, cnt, wgt, brt, _ in AC.histogram_cases(ref.lib, prof):
        out[f"awb_est/{name}/count"], out[f"awb_est/{name}/weight"] = cnt, wgt
        if brt is not None:
            out[f"awb_est/{name}/weight_bright"] = brt
    out["awb_est/rows"] = AC.run_estimates(ref.lib, prof)
    for name, params, seed_il, ev in AC.smoother_cases():
        out[f"awb_smooth/{name}"] = AC.run_smoother(ref.lib, params, seed_il, ev)
    out["locus/rows"] = AC.run_locus(ref.lib, prof)

    # Noise-model estimation (reference lib/noise.c:338-504).
    import noise_cases as NC
    for name, m, params in NC.cases():
        ret, est = ref.noise_estimate(m, prof, params)
        out[f"noise_est/{name}/in"] = m
        out[f"noise_est/{name}/out"] = NC.row(ret, est)

    np.savez_compressed(HERE / "reference_outputs.npz", **out)
    print(f"wrote {HERE / 'reference_outputs.npz'} ({len(out)} arrays)")


if __name__ == "__main__":
    main()
