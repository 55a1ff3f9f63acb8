"""Known answers for the oracle's texture fetch (the formula the CUDA
Programming Guide gives for linear filtering with wrap addressing)."""
import numpy as np

import oracle


def _tex(h, w, seed=0):
    return np.random.default_rng(seed).integers(0, 256, size=(h, w, 4), dtype=np.uint8)


def test_texel_centres_return_the_texel():
    t = _tex(5, 7)
    j, i = np.mgrid[0:5, 0:7]
    uv = np.stack([(i + 0.5) / 7, (j + 0.5) / 5], -1).reshape(-1, 2).astype(np.float32)
    rgb = oracle.texfetch(t, uv)
    assert np.array_equal(rgb, t[..., :3].reshape(-1, 3).astype(np.float32) / np.float32(255))


def test_wrap_is_periodic():
    t = _tex(9, 13, 1)
    # multiples of 2^-12, so that u + k is exact in float
    uv = (np.random.default_rng(2).integers(0, 4096, size=(4096, 2)) / 4096.0).astype(np.float32)
    base = oracle.texfetch(t, uv)
    for k in (1.0, 2.0, -1.0, -3.0):
        assert np.array_equal(oracle.texfetch(t, uv + np.float32(k)), base)


def test_weights_have_eight_fractional_bits():
    t = np.zeros((1, 2, 4), np.uint8)
    t[0, 1, :3] = 255                                  # black | white
    # x = u * 2 - 0.5: u = 0.25 + f / 2 gives frac(xB) = f between the two texels
    f = np.array([0.0, 0.3, 0.5, 0.25, 1.0 / 512, 3.0 / 1024, 0.999], np.float32)
    uv = np.stack([np.float32(0.25) + f / np.float32(2), np.full_like(f, 0.5)], -1)
    got = oracle.texfetch(t, uv)[:, 0]
    want = np.floor(f * 256 + 0.5) / 256               # rounded to nearest 1/256
    assert np.allclose(got, want, atol=1e-7), (got, want)


def test_edges_blend_with_the_opposite_side():
    t = np.zeros((1, 4, 4), np.uint8)
    t[0, 0, :3] = 200
    t[0, 3, :3] = 100
    got = oracle.texfetch(t, np.array([[0.0, 0.5], [1.0, 0.5]], np.float32))
    assert np.allclose(got[:, 0], (200 + 100) / 2 / 255, atol=1e-6)


def test_non_finite_coordinates_read_the_origin_cell():
    t = _tex(3, 3, 4)
    uv = np.array([[np.nan, 0.5], [np.inf, -np.inf], [0.0, 0.0]], np.float32)
    got = oracle.texfetch(t, uv)
    assert np.all(np.isfinite(got))
