"""The restated scenes of the reference's behavioural denoise checks
(tests/kat_scenes.py), pinned on the CPU: the oracle's temporal average
over the eight-frame sequence gives the flat-patch noise the reference's
design notes publish for its own code (71.7, 60.0, 50.2, 43.2, 40.0, 36.3,
34.8, 31.9 counts), and its spatial filter passes the still's checks."""
import numpy as np

import kat_scenes as K
from oracle import Oracle


def test_sequence_reproduces_published_noise():
    orc = Oracle()
    prev, noise = None, []
    for f in range(K.TN_FRAMES):
        clean, prev = orc.denoise_temporal(K.tn_frame(f), K.profile(), K.model(), 0.0, K.TN_ALPHA, prev=prev)
        noise.append(K.plane_noise(clean, K.TN_FLAT))
    assert np.allclose(noise, [71.7, 60.0, 50.2, 43.2, 40.0, 36.3, 34.8, 31.9], atol=0.06), noise


def test_still_checks_on_the_oracle():
    orc = Oracle()
    m = K.still()
    clean, _ = orc.denoise_temporal(m, K.profile(), K.model(), 1.0, 0.0)
    assert K.plane_noise(clean, K.FLAT_NEUTRAL) <= 0.60 * K.plane_noise(m, K.FLAT_NEUTRAL)
    assert K.plane_noise(clean, K.CHECKER) >= 0.70 * K.plane_noise(m, K.CHECKER)
