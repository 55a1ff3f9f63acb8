"""Accumulation checkpoints: render part of the samples, save, load into a
fresh buffer, finish: bit-identical to the uninterrupted render."""
import numpy as np
import pytest

from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def test_resume_equals_uninterrupted(ctx, tmp_path):
    import torch
    sd = scenes.cornell_sphere(seed=4, slices=32, stacks=16)
    sc = api.Scene(ctx, sd)
    W, H, spp = 80, 60, 8
    full = sc.render(T.render_params(W, H, spp, 4, seed=9, mode=T.MODE_PATH)).cpu().numpy()
    part = sc.render(T.render_params(W, H, spp, 4, seed=9, mode=T.MODE_PATH, sample_end=3))
    path = str(tmp_path / "frame.ckpt")
    api.accum_save(ctx, path, part, 3, spp)
    resumed = torch.full((H, W, 4), -1.0, device="cuda")
    done, total = api.accum_load(ctx, path, resumed)
    assert (done, total) == (3, spp)
    sc.render(T.render_params(W, H, spp, 4, seed=9, mode=T.MODE_PATH, sample_begin=done), accum=resumed)
    assert np.array_equal(resumed.cpu().numpy(), full)


def test_bad_checkpoints_are_rejected(ctx, tmp_path):
    import torch
    buf = torch.zeros((10, 12, 4), device="cuda")
    path = str(tmp_path / "a.ckpt")
    api.accum_save(ctx, path, buf, 1, 4)
    with pytest.raises(api.AuroraError):
        api.accum_load(ctx, path, torch.zeros((10, 13, 4), device="cuda"))      # other size
    data = open(path, "rb").read()
    open(path, "wb").write(data[:-16])
    with pytest.raises(api.AuroraError):
        api.accum_load(ctx, path, buf)                                          # truncated
    open(path, "wb").write(b"XXXXXXXX" + data[8:])
    with pytest.raises(api.AuroraError):
        api.accum_load(ctx, path, buf)                                          # not a checkpoint
    with pytest.raises(api.AuroraError):
        api.accum_save(ctx, path, buf, 5, 4)                                    # more samples than spp
