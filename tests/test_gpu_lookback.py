"""The NMH build's bounded device-side waits, made to run out on purpose.

The split and partition passes are single-pass scans: each tile waits for
its predecessor's prefix (decoupled look-back). A wait that never ends would
hang the GPU, so each gives up after a bounded number of spins; the build
must then return AUR_ERR_TIMEOUT, launch nothing that reads the half-written
lists, and leave the context usable. The test hook aur_debug_lookback_timeout
makes the next build's tiles wait on a prefix that nothing publishes; the
build after it must be bit-exact again. No GPU fault is involved: the wait
ends by its own limit."""
import numpy as np
import pytest

import oracle
from aurora_gb300 import api, scenes

pytestmark = pytest.mark.gpu
TIMEOUT = 4


@pytest.mark.parametrize("builds_before", [0, 1, 2, 3])
def test_lookback_wait_runs_out_and_the_next_build_is_exact(built, builds_before):
    """builds_before selects how the failing build runs: 0 launches directly,
    1 records the size's graph, 2 and 3 replay the recorded graph."""
    import torch
    V = scenes.random_soup(100_003, seed=21)
    ref_perm, _ = oracle.nmh_build(V)
    Vd = torch.from_numpy(V.reshape(-1)).cuda()
    ctx = api.Context(0)
    try:
        for _ in range(builds_before):
            api.Nmh(ctx, Vd, count=V.shape[0]).close()
        api.check(api.lib().aur_debug_lookback_timeout(ctx.handle, 64))
        with pytest.raises(api.AuroraError) as e:
            api.Nmh(ctx, Vd, count=V.shape[0])
        assert e.value.status == TIMEOUT, str(e.value)
        assert "gave up" in str(e.value)
        for _ in range(2):                         # the hook is spent; later builds are normal
            nmh = api.Nmh(ctx, Vd, count=V.shape[0])
            perm, _ = nmh.export(with_vertices=False)
            nmh.close()
            assert np.array_equal(perm, ref_perm)
        ctx.synchronize()
    finally:
        ctx.close()


def test_lookback_hook_leaves_small_soups_alone(ctx):
    """A soup of at most 4,096 triangles has a single scan tile per pass and
    no wait; the armed build succeeds, exact, and spends the hook."""
    import torch
    V = scenes.random_soup(3000, seed=22)
    ref_perm, _ = oracle.nmh_build(V)
    Vd = torch.from_numpy(V.reshape(-1)).cuda()
    api.check(api.lib().aur_debug_lookback_timeout(ctx.handle, 64))
    nmh = api.Nmh(ctx, Vd, count=V.shape[0])
    perm, _ = nmh.export(with_vertices=False)
    nmh.close()
    assert np.array_equal(perm, ref_perm)
