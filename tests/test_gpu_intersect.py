"""Closest-hit parity: pppm_intersect vs QBVHAccel::intersect of the reference.

The fixtures hold the reference's own outputs (tests/golden/make_golden.py).
The GPU reproduces the reference arithmetic (float slab test with SSE
max/min semantics, double Moller-Trumbore, the same tree topology and child
order), so triangle ids and hit distances must be bit-identical, ties and
grazing rays included.
"""
import numpy as np
import pytest

from conftest import scene_from

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("suffix", ["", "2"])
def test_intersect_bit_exact(ctx, golden, suffix):
    g = golden("intersect")
    ctx.set_scene(scene_from(g["tris" + suffix]))
    tri, t, pos, nrm = ctx.intersect(np.ascontiguousarray(g["rays" + suffix]))
    ref_tri, ref_t = g["tri" + suffix], g["t" + suffix]
    bad = np.flatnonzero(tri != ref_tri)
    assert bad.size == 0, f"{bad.size} id mismatches, first {bad[:10]}: gpu {tri[bad[:10]]} ref {ref_tri[bad[:10]]}"
    assert np.array_equal(t.view(np.uint64), ref_t.view(np.uint64)), "hit distances differ in bits"
    hit = ref_tri >= 0
    assert hit.mean() > 0.3
    # positions/normals: the reference's doubles rounded to float
    np.testing.assert_array_equal(pos[hit], g["pos" + suffix][hit].astype(np.float32))
    np.testing.assert_array_equal(nrm[hit], g["nrm" + suffix][hit].astype(np.float32))


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
def test_intersect_tiny_scenes(ctx, golden, k):
    g = golden("intersect")
    ctx.set_scene(scene_from(g[f"tiny{k}_tris"]))
    tri, t, _, _ = ctx.intersect(np.ascontiguousarray(g[f"tiny{k}_rays"]), with_hit=False)
    assert np.array_equal(tri, g[f"tiny{k}_tri"])
    assert np.array_equal(t.view(np.uint64), g[f"tiny{k}_t"].view(np.uint64))


def test_intersect_device_arrays_and_empty(ctx, golden):
    import torch
    g = golden("intersect")
    ctx.set_scene(scene_from(g["tris"]))
    rays = torch.from_numpy(np.ascontiguousarray(g["rays"])).cuda()
    tri, t, pos, nrm = ctx.intersect(rays)
    ctx.sync()
    assert tri.is_cuda and np.array_equal(tri.cpu().numpy(), g["tri"])
    # empty scene: every ray misses with t = INFTY
    ctx.set_scene(scene_from(np.zeros((0, 9), np.float32)))
    tri, t, _, _ = ctx.intersect(np.ascontiguousarray(g["rays"][:100]), with_hit=False)
    assert (tri == -1).all() and (t == 1e20).all()


def test_hash_points_bit_exact(ctx, golden):
    g = golden("hash")
    for k in range(4):
        h = ctx.hash_points(np.ascontiguousarray(g[f"pts{k}"]), int(g[f"size{k}"]), float(g[f"scale{k}"]), g[f"bbmin{k}"])
        assert np.array_equal(h, g[f"hash{k}"]), k
