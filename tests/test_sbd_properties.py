"""Properties of the SBD distance the engine's bounds rest on, checked on the FP64
oracle's distances (CPU).

* Movement bound: for unit-normalised centroids c^ and c'^, every lag's NCC changes by
  at most |c'^ - c^| (Cauchy-Schwarz; circular shifts in compat and zero-filling
  shifts in canonical mode do not increase norms), and neither the max over lags nor
  the clamp at 2 widens that: |d(x, c') - d(x, c)| <= |c'^ - c^|.
* Scale invariance: d(x, a c) = d(x, c) for a > 0, so only the direction moves a
  distance.
"""
import numpy as np
import pytest


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("m", [64, 200, 333])
def test_distance_moves_at_most_the_centroid_direction(built, mode, m):
    T, O = built
    rng = np.random.default_rng(m + 7 * mode)
    X = O.znorm(rng.standard_normal((200, m)))
    F = T.fft_size(m, mode)
    clamp2 = mode == 0 and 2 * m - 1 < 512
    for step in (1e-3, 1e-2, 0.1, 1.0):
        c = rng.standard_normal(m)
        c2 = c + step * np.linalg.norm(c) * rng.standard_normal(m) / np.sqrt(m)
        _, d1, _, _ = O.assign(X, c[None, :], F, clamp2=clamp2)
        _, d2, _, _ = O.assign(X, c2[None, :], F, clamp2=clamp2)
        move = np.linalg.norm(c2 / np.linalg.norm(c2) - c / np.linalg.norm(c))
        assert np.max(np.abs(d2 - d1)) <= move * (1 + 1e-9) + 1e-12, (step, move)


def test_distance_is_scale_invariant(built):
    T, O = built
    rng = np.random.default_rng(3)
    X = O.znorm(rng.standard_normal((50, 128)))
    c = rng.standard_normal(128)
    F = T.fft_size(128, 0)
    _, d1, _, _ = O.assign(X, c[None, :], F, clamp2=True)
    _, d2, _, _ = O.assign(X, 3.5 * c[None, :], F, clamp2=True)
    np.testing.assert_allclose(d1, d2, rtol=0, atol=1e-12)
