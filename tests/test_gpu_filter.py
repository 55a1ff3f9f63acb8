"""aur_filter_pixels (cudaFilterPixels with the row-below clamp fixed) on
the GPU against the oracle, bit for bit."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("H,W,region", [(37, 53, None), (37, 53, (5, 20, 3, 30)), (1080, 1920, (100, 1800, 0, 1079)),
                                        (64, 64, (7, 7, 2, 9)), (5, 3, (0, 2, 4, 4))])
def test_filter_matches_oracle(ctx, H, W, region):
    import torch
    img = np.random.default_rng(H * W).random((H, W, 4)).astype(np.float32) * 3
    src = torch.from_numpy(img).cuda()
    out = torch.full_like(src, -1.0)
    api.filter_pixels(ctx, W, H, src, out, region)
    got = out.cpu().numpy()
    ref = oracle.filter_pixels(img, region)
    r = region or (0, W - 1, 0, H - 1)
    assert np.array_equal(got[r[2]:r[3] + 1, r[0]:r[1] + 1], ref[r[2]:r[3] + 1, r[0]:r[1] + 1])
    outside = np.ones((H, W), bool)
    outside[r[2]:r[3] + 1, r[0]:r[1] + 1] = False
    assert np.all(got[outside] == -1.0)


def test_filter_rejects_bad_arguments(ctx):
    import torch
    a = torch.zeros((8, 8, 4), device="cuda")
    b = torch.zeros_like(a)
    with pytest.raises(api.AuroraError):
        api.filter_pixels(ctx, 8, 8, a, a)                       # in place
    with pytest.raises(api.AuroraError):
        api.filter_pixels(ctx, 8, 8, a, b, (0, 8, 0, 7))         # right edge outside
    with pytest.raises(api.AuroraError):
        api.filter_pixels(ctx, 8, 8, a, b, (5, 4, 0, 7))         # empty
