"""The oracle's analyser factor (the reference GPU general kernel's top-hat /
Darwin acceptance, Beam.py:2350-2378) on known answers: one atom, pixels at
known angles from the analyser axis."""
import numpy as np

import oracle


def _one_atom(cx, cy, cz, analyser):
    wk = np.zeros((1, 11), np.float32)
    wk[0, 5] = 1.0                      # f0 = 1 everywhere
    z = np.zeros(1)
    return oracle.scatter_f64(np.zeros((1, 3)), wk, np.ones(1), z, z, np.ones(1), z, cx, cy, cz,
                              5e10, len(cx), 1, analyser=analyser)


def test_top_hat_and_darwin_known_answers():
    R = 0.5
    axis = np.array([np.cos(0.6), np.sin(0.6), 0.0])
    alpha = 2e-3
    th = np.array([0.0, 0.5 * alpha, 0.999 * alpha, 1.001 * alpha, 3 * alpha])
    ang = 0.6 + th                       # pixels in the x-y plane at these offsets
    cx, cy, cz = R * np.cos(ang), R * np.sin(ang), np.zeros_like(ang)
    plain = _one_atom(cx, cy, cz, None)
    top = _one_atom(cx, cy, cz, (1, axis, alpha, 0.0))
    assert np.allclose(top[:3], plain[:3], rtol=0, atol=0)
    assert np.all(top[3:] == 0)
    hw = 1e-3
    dar = _one_atom(cx, cy, cz, (2, axis, 0.0, hw))
    want = plain / (1.0 + (th / hw) ** 2)
    assert np.allclose(dar, want, rtol=1e-9, atol=0)
    # Darwin with a non-positive half-width is no analyser
    assert np.array_equal(_one_atom(cx, cy, cz, (2, axis, 0.0, 0.0)), plain)
