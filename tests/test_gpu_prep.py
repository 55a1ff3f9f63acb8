"""Scene preparation entry points (cudaTransform, cudaGenerateTB) against the oracle."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes, types as T

pytestmark = pytest.mark.gpu


def _objects(count, rng):
    offs = np.sort(rng.choice(np.arange(1, count), size=5, replace=False))
    offs = np.concatenate([[3], offs, [offs[-1]]])           # a repeated offset: the later object wins
    xf = np.zeros(len(offs), T.object_transform_dtype)
    xf["offset"] = offs
    for i in range(len(offs)):
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] = rng.normal(size=(3, 3)).astype(np.float32)
        m[3, :3] = rng.normal(size=3).astype(np.float32)
        xf["world_matrix"][i] = m
        xf["normal_matrix"][i] = np.linalg.inv(m).T.astype(np.float32)
    return xf


def test_transform_matches_oracle(ctx):
    import torch
    rng = np.random.default_rng(4)
    sd = scenes.cornell_sphere(seed=1)
    xf = _objects(sd.count, rng)
    sv = torch.from_numpy(sd.vertices.reshape(-1)).cuda()
    sn = torch.from_numpy(sd.normals.reshape(-1)).cuda()
    dv = torch.full_like(sv, 7.0)
    dn = torch.full_like(sn, 7.0)
    api.transform(ctx, sv, sn, xf, dv, dn)
    ov, on = oracle.transform(sd.vertices, sd.normals, xf, np.full_like(sd.vertices, 7.0),
                              np.full_like(sd.normals, 7.0))
    assert np.array_equal(dv.cpu().numpy().reshape(-1, 9), ov)
    assert np.array_equal(dn.cpu().numpy().reshape(-1, 9), on)
    assert np.all(ov[:3] == 7.0)                               # before the first object: untouched


def test_transform_rejects_unsorted_offsets(ctx):
    import torch
    xf = np.zeros(2, T.object_transform_dtype)
    xf["offset"] = [5, 2]
    z = torch.zeros(9 * 8, device="cuda")
    with pytest.raises(api.AuroraError):
        api.transform(ctx, z, z, xf, z.clone(), z.clone())


def test_generate_tb_matches_oracle(ctx):
    import torch
    sd = scenes.cornell_sphere(seed=2)
    n = torch.from_numpy(sd.normals.reshape(-1)).cuda()
    t, b = torch.empty_like(n), torch.empty_like(n)
    api.generate_tb(ctx, n, t, b)
    ot, ob = oracle.generate_tb(sd.normals)
    assert np.array_equal(t.cpu().numpy().reshape(-1, 9), ot)
    assert np.array_equal(b.cpu().numpy().reshape(-1, 9), ob)
