"""Noise-model estimation, craw_noise_estimate() (reference lib/noise.c:
338-504): the oracle's restatement pinned to the reference's own build and
to the golden fixtures it made (CPU), then the GPU implementation against
the oracle (GPU).

The GPU's bins hold the same samples, counts and medians as the
reference's (order statistics and integer counts); a bin's level is the
exact sum of its float means rounded once, where the reference adds them
into a double one by one, so the bin levels may differ in their last
bits. The fitted floats are compared to 1e-6 relative (in practice they
are equal); counts of bins and inliers exactly."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

import libcraw_gb300 as L
from libcraw_gb300 import workloads as W
from oracle import Oracle, Reference, reference_available

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import noise_cases as NC  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_outputs.npz"
orc = Oracle()
PROF = W.make_profile()
ENODATA = -61


def test_struct_layout_and_defaults():
    assert C.sizeof(L.NoiseEstimateParams) == 64 and C.sizeof(L.NoiseEstimate) == 64
    p = L.noise_estimate_params()
    assert (p.nb_bins, p.min_bin_samples) == (128, 20000)
    assert abs(p.max_level - 0.98) < 1e-7


@pytest.mark.parametrize("name", [c[0] for c in NC.cases()])
def test_oracle_matches_golden(name):
    z = np.load(GOLDEN)
    params = dict((c[0], c[2]) for c in NC.cases())[name]
    ret, est = orc.noise_estimate(z[f"noise_est/{name}/in"], PROF, params)
    assert np.array_equal(NC.row(ret, est), z[f"noise_est/{name}/out"])


@pytest.mark.skipif(not reference_available(), reason="reference build absent")
@pytest.mark.parametrize("w,h,seed,kind,params", [
    (512, 384, 21, "scene", NC.params(64, 500)),
    (640, 480, 22, "ramp", NC.params(128, 300)),
    (96, 80, 23, "ramp", NC.params(8, 10, 0.5)),
    (34, 32, 24, "ramp", NC.params(8, 1)),
    (512, 256, 25, "highlights", NC.params(48, 100, 0.97)),
])
def test_oracle_matches_reference(w, h, seed, kind, params):
    m = {"scene": lambda: W.synth_frame(w, h, seed, noise_a_dn=4.0, noise_b_dn=40.0),
         "ramp": lambda: W.noise_ramp(w, h, seed),
         "highlights": lambda: W.highlight_frame(w, h, seed)}[kind]()
    ref = Reference()
    r1, e1 = orc.noise_estimate(m, PROF, params)
    r2, e2 = ref.noise_estimate(m, PROF, params)
    assert np.array_equal(NC.row(r1, e1), NC.row(r2, e2))


def bad_profile(**kw):
    p = W.make_profile()
    for k, v in kw.items():
        if k == "white0":
            p.white_level[0] = p.black_level[0]
        else:
            setattr(p, k, v)
    return p


ERROR_CASES = [
    ("odd", (33, 32), PROF, None, -22),
    ("small", (30, 32), PROF, None, -22),
    ("bins_low", (64, 64), PROF, NC.params(7), -22),
    ("bins_high", (64, 64), PROF, NC.params(513), -22),
    ("white_le_black", (64, 64), "white0", None, -22),
    ("cfa", (64, 64), "cfa", None, -95),
]


@pytest.mark.parametrize("name,wh,prof,params,code", ERROR_CASES)
def test_errors_before_any_device_work(name, wh, prof, params, code):
    """Argument errors come back before the GPU is touched, with the
    reference's codes; the oracle agrees."""
    w, h = wh
    if prof == "white0":
        prof = bad_profile(white0=True)
    elif prof == "cfa":
        prof = bad_profile(cfa=1)
    m = np.zeros((h, w), np.uint16)
    with pytest.raises(L.CrawError) as e:
        L.noise_estimate(m, prof, params)
    assert e.value.code == code
    assert orc.noise_estimate(m, prof, params)[0] == code


# ------------------------------------------------------------------ GPU

def close(got: L.NoiseEstimate, ref: L.NoiseEstimate):
    g, r = got.as_tuple(), ref.as_tuple()
    if (g[2], g[3]) != (r[2], r[3]):
        return False
    return all(abs(x - y) <= 1e-6 * max(abs(y), 1e-30) for x, y in zip(g[:2] + g[4:], r[:2] + r[4:]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", [c[0] for c in NC.cases()])
def test_gpu_matches_golden(name):
    z = np.load(GOLDEN)
    params = dict((c[0], c[2]) for c in NC.cases())[name]
    m = z[f"noise_est/{name}/in"]
    want = z[f"noise_est/{name}/out"]
    if want[0] < 0:
        with pytest.raises(L.CrawError) as e:
            L.noise_estimate(m, PROF, params)
        assert e.value.code == want[0]
        return
    got = L.noise_estimate(m, PROF, params)
    ref = L.NoiseEstimate()
    ref.model.a, ref.model.b, ref.nb_bins, ref.nb_inliers, ref.fit_rms, ref.read_noise_lsb = (
        want[1], want[2], int(want[3]), int(want[4]), want[5], want[6])
    assert close(got, ref), (got.as_tuple(), ref.as_tuple())


@pytest.mark.gpu
@pytest.mark.parametrize("w,h,seed,kind,params", [
    (2048, 1152, 31, "ramp", None),
    (1536, 1024, 32, "scene", NC.params(96, 5000)),
    (1000, 600, 33, "highlights", NC.params(40, 500, 0.95)),
    (520, 388, 34, "ramp", NC.params(512, 10)),
])
def test_gpu_matches_oracle(w, h, seed, kind, params):
    m = {"scene": lambda: W.synth_frame(w, h, seed, noise_a_dn=4.0, noise_b_dn=40.0),
         "ramp": lambda: W.noise_ramp(w, h, seed, lo=0.0),
         "highlights": lambda: W.highlight_frame(w, h, seed)}[kind]()
    r, want = orc.noise_estimate(m, PROF, params)
    assert r == 0
    got = L.noise_estimate(m, PROF, params)
    assert close(got, want), (got.as_tuple(), want.as_tuple())


@pytest.mark.gpu
def test_gpu_device_mosaic_and_stream():
    """craw_noise_estimate_cuda on a device image with padded rows, on a
    caller's stream, equals the host-pointer call."""
    import torch
    w, h = 1200, 800
    m = W.noise_ramp(w, h, 41, lo=0.0)
    t = torch.zeros((h, w + 40), dtype=torch.int16, device="cuda")
    t[:, :w] = torch.from_numpy(m.view(np.int16)).cuda()
    img = L.Image(t.data_ptr(), t.stride(0) * 2, L.FORMAT_R16_UNORM, w, h)
    s = torch.cuda.Stream()
    got = L.noise_estimate_cuda(img, PROF, NC.params(64, 1000), stream=s.cuda_stream)
    assert got.as_tuple() == L.noise_estimate(m, PROF, NC.params(64, 1000)).as_tuple()
    with pytest.raises(L.CrawError):
        L.noise_estimate_cuda(L.Image(t.data_ptr() + 2, t.stride(0) * 2, L.FORMAT_R16_UNORM, w, h), PROF)


@pytest.mark.gpu
def test_gpu_full_frame_recovers_the_model():
    """At 5760x3240 a noisy ramp gives back the model it was made with, and
    the GPU agrees with the oracle."""
    w, h = 5760, 3240
    m = W.noise_ramp(w, h, 51, lo=0.0)
    got = L.noise_estimate(m, PROF)
    a, b = W.noise_model(4.0, 40.0)
    assert abs(got.model.a / a - 1) < 0.02 and abs(got.model.b / b - 1) < 0.1, got.as_tuple()
    r, want = orc.noise_estimate(m, PROF, None)
    assert r == 0 and close(got, want), (got.as_tuple(), want.as_tuple())
