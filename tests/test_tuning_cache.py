"""The autotuner's result cache: keys by GPU and batch shape, JSON round trip."""
from types import SimpleNamespace

import numpy as np

from aurora_gb300 import api, scenes, types as T


def _scene(n_tris, n_lights):
    return SimpleNamespace(data=SimpleNamespace(count=n_tris, lights=np.zeros(n_lights, T.light_dtype)))


def test_key_depends_on_gpu_and_shape():
    scs = [_scene(100, 1), _scene(2000, 2)]
    prm = [T.render_params(64, 64, 16, 4), T.render_params(32, 64, 16, 4)]
    k = api.tuning_key("GB300", 152, scs, prm)
    assert k == api.tuning_key("GB300", 152, scs, prm)
    assert k != api.tuning_key("B200", 148, scs, prm)
    assert k != api.tuning_key("GB300", 152, scs, [prm[0], T.render_params(32, 64, 16, 5)])
    assert k != api.tuning_key("GB300", 152, [scs[0], _scene(2001, 2)], prm)


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "tune.json")
    assert api.tuning_cache_get(path, "k") is None
    t = api.make_tuning(1 << 23, 0, 128, 8)
    api.tuning_cache_put(path, "k", t, 12.5)
    api.tuning_cache_put(path, "other", api.make_tuning(1 << 20, 1, 256, 4), 3.0)
    got, ms = api.tuning_cache_get(path, "k")
    assert ms == 12.5 and all(int(got[f]) == int(t[f]) for f in t.dtype.names)
