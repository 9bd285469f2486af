"""Pass sharding on the GPU, emulated with two contexts on one device: rank
0 renders passes 1, 3, 5, rank 1 passes 2, 4, 6 (pppm_render_skip over the
others), and the sum of their accumulators is the six-pass render up to the
order of float sums, for the canonical pass, the reference's compat pass
and the path tracer."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [P.MODE_CANONICAL, P.MODE_COMPAT, P.MODE_PATH_TRACING])
def test_shards_sum_to_the_full_render(mode):
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20000)
    kw = dict(mode=mode, photons=20000, num_streams=8)
    if mode == P.MODE_CANONICAL:
        kw.update(radius_scale=1 / 32, seed=9)
    par = P.Context.make_params(**kw)
    total = 6
    ctxs = [P.Context(0) for _ in range(3)]
    try:
        for c in ctxs:
            c.set_scene(sc)
        full = ctxs[0]
        full.render_begin(sc.camera, par)
        for t in range(1, total + 1):
            full.render_pass(t)
        ref = full.render_read()
        parts = [P.render_shard(ctxs[1 + r], sc.camera, par, total, r, 2) for r in range(2)]
    finally:
        for c in ctxs:
            c.close()
    merged = P.merge_shards(parts[0] + parts[1], 1)
    err = np.abs(merged - ref).max() / max(np.abs(ref).max(), 1e-12)
    assert err < 1e-4, err


def test_skip_refuses_dependent_passes():
    sc = S.small_test_scene(seed=3, subdiv=3, width=32, height=24, photons=5000)
    c = P.Context(0)
    try:
        c.set_scene(sc)
        c.render_begin(sc.camera, P.Context.make_params(mode=P.MODE_CLASSIC, photons=5000, num_streams=4))
        with pytest.raises(P.PppmError) as e:
            c.render_skip(1)
        assert e.value.code == P.E_STATE
    finally:
        c.close()
