"""The synthetic frames and measures of the reference's behavioural checks
of the denoise (reference tests/test_pipeline.c:134-173, 543-575, 700-730
and 776-905), restated in numpy so that the GPU can be held to the same
known answers: a 256x160 still with flat patches and a 2x2 checkerboard,
and an eight-frame sequence whose noise is the model's own, with two bars
sliding across a flat background and two static checkerboards. The
scenes, levels, rectangles and thresholds are the reference's; the code is
this project's."""
from __future__ import annotations

import numpy as np

import libcraw_gb300 as L

W_, H_ = 256, 160
BLACK = np.float32(256.0 / 65535.0)
WHITE = np.float32(63743.0 / 65535.0)
WB = (2.02539, 1.0, 1.66797)
NOISE_A = 1.3e-5
_RANGE = float(WHITE) - float(BLACK)
NOISE_B = (17.0 * 17.0 - 1.0) / 12.0 / (65535.0 * _RANGE * 65535.0 * _RANGE)

# The still's rectangles (x0, y0, x1, y1), inclusive.
FLAT_NEUTRAL = (162, 26, 197, 53)
CHECKER = (212, 100, 243, 131)
# The sequence's.
TN_FRAMES, TN_ALPHA, TN_BG, TN_BAR, TN_STEP, TN_BAR_W = 8, 0.8, 0.10, 0.40, 12, 16
TN_STRONG = (88, 119)
TN_FAINT = (124, 151)
TN_FLAT = (162, 90, 221, 149)
TN_DETAIL = (164, 20, 219, 75)
TN_FAINT_CHECKER = (16, 16, 127, 79)


def profile() -> L.Profile:
    """Black 256, white 63743 at every site, the scene's as-shot gains and
    an identity camera matrix (the colour stage then hands back camera RGB
    as XYZ)."""
    p = L.profile_init()
    for s in range(4):
        p.black_level[s] = float(BLACK)
        p.white_level[s] = float(WHITE)
    for c in range(3):
        p.as_shot_wb[c] = WB[c]
        for j in range(3):
            p.as_shot_matrix[c][j] = 1.0 if c == j else 0.0
    p.as_shot_cct = 5500.0
    p.gain = 1.0
    p.name = b"behavioural checks"
    return p


def model() -> tuple[float, float]:
    return float(np.float32(NOISE_A)), float(np.float32(NOISE_B))


def _hash(x: np.ndarray) -> np.ndarray:
    """A 32-bit integer mixing hash (Wellons' lowbias32)."""
    x = x.astype(np.uint32)
    x ^= x >> np.uint32(16)
    x *= np.uint32(0x7FEB352D)
    x ^= x >> np.uint32(15)
    x *= np.uint32(0x846CA68B)
    x ^= x >> np.uint32(16)
    return x


def _in(x, y, r):
    return (x >= r[0]) & (x <= r[2]) & (y >= r[1]) & (y <= r[3])


def still() -> np.ndarray:
    """The still: affine colour ramps, three flat patches, a 2x2
    checkerboard, a clipped and a black rectangle, and a +-8 count hashed
    noise term, as raw R16 codes."""
    y, x = np.mgrid[0:H_, 0:W_]
    fx = (x / np.float32(W_ - 1)).astype(np.float32)
    fy = (y / np.float32(H_ - 1)).astype(np.float32)
    rgb = np.stack([np.float32(0.05) + np.float32(0.80) * fx, np.float32(0.08) + np.float32(0.75) * fy,
                    np.float32(0.10) + np.float32(0.40) * fx + np.float32(0.35) * fy], -1).astype(np.float32)
    for r, v in (((16, 16, 47, 47), (0.75, 0.30, 0.12)), ((64, 96, 103, 127), (0.12, 0.60, 0.80)),
                 ((160, 24, 199, 55), (0.45, 0.45, 0.45))):
        rgb[_in(x, y, r)] = np.array(v, np.float32)
    ck = _in(x, y, (208, 96, 247, 135))
    v = np.where((((x >> 1) + (y >> 1)) & 1) == 1, np.float32(0.82), np.float32(0.08)).astype(np.float32)
    rgb[ck] = v[ck][:, None]
    site = (y & 1) * 2 + (x & 1)
    chan = np.where(site == 0, 0, np.where(site == 3, 2, 1))
    c = np.take_along_axis(rgb, chan[..., None], -1)[..., 0]
    wb = np.array(WB, np.float32)[chan]
    raw = (BLACK + (c / wb).astype(np.float32) * (WHITE - BLACK)).astype(np.float32)
    iv = np.rint((raw * np.float32(65535.0)).astype(np.float32)).astype(np.int64)
    k = (y * W_ + x).astype(np.uint64) * np.uint64(2654435761)
    iv += (_hash(k & np.uint64(0xFFFFFFFF)) % np.uint32(17)).astype(np.int64) - 8
    iv = np.clip(iv, 0, 65535)
    iv[_in(x, y, (108, 4, 139, 35))] = 65535
    iv[_in(x, y, (44, 116, 75, 147))] = 256
    return iv.astype(np.uint16)


def plane_noise(m: np.ndarray, r) -> float:
    """Noise of a rectangle in counts: the median |3x3 per-plane high
    pass / 6| over it (positions two apart stay in one CFA plane), over
    0.6745."""
    x0, y0, x1, y1 = r
    m = m.astype(np.float64)
    ys, xs = slice(y0 + 2, y1 - 1), slice(x0 + 2, x1 - 1)
    def at(dy, dx):
        return m[y0 + 2 + dy:y1 - 1 + dy, x0 + 2 + dx:x1 - 1 + dx]
    hp = (at(-2, -2) + at(-2, 2) + at(2, -2) + at(2, 2) - 2.0 * (at(-2, 0) + at(2, 0) + at(0, -2) + at(0, 2))
          + 4.0 * at(0, 0))
    res = np.sort(np.abs(hp / 6.0).astype(np.float32).ravel())
    return float(res[res.size // 2]) / 0.6744897502


def _sigma(u):
    return np.sqrt(NOISE_A * u + NOISE_B)


def tn_bar_x(f: int) -> int:
    return 16 + TN_STEP * f


def tn_truth(f: int) -> np.ndarray:
    y, x = np.mgrid[0:H_, 0:W_]
    u = np.full((H_, W_), TN_BG)
    sq = (((x >> 2) + (y >> 2)) & 1) == 1
    faint = _in(x, y, (16, 16, 127, 79))
    u[faint] = (TN_BG + np.where(sq, 0.75, -0.75) * _sigma(TN_BG))[faint]
    bx = tn_bar_x(f)
    bar = (x >= bx) & (x < bx + TN_BAR_W)
    u[bar & (y >= TN_STRONG[0]) & (y <= TN_STRONG[1])] = TN_BAR
    u[bar & (y >= TN_FAINT[0]) & (y <= TN_FAINT[1])] = TN_BG + 2.0 * _sigma(TN_BG)
    strong = _in(x, y, (160, 16, 223, 79))
    u[strong] = np.where(sq, 0.25, 0.05)[strong]
    return u


def tn_frame(f: int, noisy: bool = True) -> np.ndarray:
    """Frame f of the sequence: the truth plus noise at the model's level,
    a normal deviate per sample and frame by Box-Muller on two hashed
    uniforms."""
    u = tn_truth(f)
    if noisy:
        y, x = np.mgrid[0:H_, 0:W_]
        k = ((f * H_ + y) * W_ + x).astype(np.uint64)
        u1 = (_hash((2 * k + 1) & 0xFFFFFFFF).astype(np.float64) + 0.5) / 4294967296.0
        u2 = (_hash(((2 * k + 2) & 0xFFFFFFFF) ^ 0x9E3779B9).astype(np.float64) + 0.5) / 4294967296.0
        u = u + _sigma(u) * np.sqrt(-2.0 * np.log(u1)) * np.cos(6.283185307179586 * u2)
    raw = float(BLACK) + u * (float(WHITE) - float(BLACK))
    return np.clip(np.rint(raw * 65535.0), 0, 65535).astype(np.uint16)


def tn_detail(m: np.ndarray, truth: np.ndarray, r) -> float:
    """How much of the truth's per-plane high pass over a rectangle
    survives in m: the regression coefficient of one on the other."""
    x0, y0, x1, y1 = r
    def hp(a):
        a = a.astype(np.float64)
        out = 0.0
        for ky in (-1, 0, 1):
            for kx in (-1, 0, 1):
                k = (1.0 if ky else -2.0) * (1.0 if kx else -2.0)
                out = out + k * a[y0 + 2 + 2 * ky:y1 - 1 + 2 * ky, x0 + 2 + 2 * kx:x1 - 1 + 2 * kx]
        return out
    hm, ht = hp(m), hp(truth)
    den = float((ht * ht).sum())
    return float((hm * ht).sum()) / den if den > 0 else 0.0


def tn_bias(m: np.ndarray, x0, y0, x1, y1, truth: float) -> float:
    """How far a rectangle's mean level sits from `truth`, in noise
    standard deviations of one frame."""
    u = (m[y0:y1 + 1, x0:x1 + 1].astype(np.float64) / 65535.0 - float(BLACK)) / (float(WHITE) - float(BLACK))
    return float((u.mean() - truth) / _sigma(truth))


def tn_bias_rgb(rgb: np.ndarray, x0, y0, x1, y1, truth: float) -> float:
    """The same over G of camera RGB (G carries the level itself)."""
    return float((rgb[y0:y1 + 1, x0:x1 + 1, 1].astype(np.float64).mean() - truth) / _sigma(truth))
