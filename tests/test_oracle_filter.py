"""The oracle's pixel filter against an independent numpy restatement:
a separable (1 2 1)/4 x (1 2 1)/4 binomial over the region, edges clamped."""
import numpy as np

import oracle


def _numpy_filter(img, region):
    L, R, B, T = region
    sub = img[B:T + 1, L:R + 1].astype(np.float64)
    p = np.pad(sub, ((1, 1), (1, 1), (0, 0)), mode="edge")
    k = np.array([0.25, 0.5, 0.25])
    h = k[0] * p[:, :-2] + k[1] * p[:, 1:-1] + k[2] * p[:, 2:]
    v = k[0] * h[:-2] + k[1] * h[1:-1] + k[2] * h[2:]
    out = img.astype(np.float64).copy()
    out[B:T + 1, L:R + 1] = v
    return out


def test_filter_matches_numpy_restatement():
    rng = np.random.default_rng(0)
    img = rng.random((37, 53, 4)).astype(np.float32)
    for region in [(0, 52, 0, 36), (5, 20, 3, 30), (7, 7, 2, 9), (4, 30, 11, 11), (0, 0, 0, 0)]:
        got = oracle.filter_pixels(img, region)
        assert np.allclose(got, _numpy_filter(img, region), rtol=1e-6, atol=1e-7)


def test_filter_keeps_constants_and_leaves_outside_untouched():
    img = np.full((9, 11, 4), 0.37, np.float32)
    img[0, :] = 5.0
    got = oracle.filter_pixels(img, (2, 8, 3, 7))
    assert np.allclose(got[3:8, 2:9], 0.37, atol=1e-7)
    assert np.array_equal(got[0], img[0])


def test_row_below_is_clamped_to_the_top_of_the_region():
    # the reference clamps y+1 to region.bottom (utility.cu:241-243); with a
    # region starting at row 0 that pulls the top row's lower taps from row 0
    img = np.zeros((4, 3, 4), np.float32)
    img[3] = 1.0                                     # only the top row is lit
    got = oracle.filter_pixels(img, (0, 2, 0, 3))
    assert np.allclose(got[3, 1], 0.75)              # (1 + 2) / 4 of the vertical kernel sees row 3 twice
    assert np.allclose(got[2, 1], 0.25)
