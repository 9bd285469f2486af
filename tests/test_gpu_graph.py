"""Canonical passes captured into one CUDA graph (pppm_render_graph and the
batch graph) give the render of pppm_render_pass: the same photons, paths
and radii, the image up to the order of float sums."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    return S.config2(width=192, height=108, freq=24)


def _params(**kw):
    base = dict(mode=P.MODE_CANONICAL, photons=200_000, max_bounce_photon=12, max_bounce_eye=12, radius_scale=1 / 64,
                seed=3)
    base.update(kw)
    return P.Context.make_params(**base)


def _close(img, ref):
    return np.abs(img - ref).max() / max(np.abs(ref).max(), 1e-12)


def test_graph_passes_match_eager_passes(scene):
    c = P.Context(0)
    try:
        c.set_scene(scene)
        c.render_begin(scene.camera, _params())
        eager = [c.render_pass(t) for t in range(1, 11)]
        ref = c.render_read()
        c.render_begin(scene.camera, _params())
        first = c.render_pass(1)
        graph = [first] + c.render_graph(9)
        img = c.render_read()
        assert _close(img, ref) < 1e-4
        for a, b in zip(eager, graph):
            assert a.photon_rays == b.photon_rays and a.eye_rays == b.eye_rays
            assert a.photons_stored == b.photons_stored and a.gather_queries == b.gather_queries
            assert a.radius == b.radius
        assert all(s.ms_photon > 0 and s.ms_gather > 0 for s in graph[1:])
        # the render goes on normally after a graph
        c.render_pass(11)
    finally:
        c.close()


def test_graph_from_the_first_pass(scene):
    c = P.Context(0)
    try:
        c.set_scene(scene)
        c.render_begin(scene.camera, _params(seed=4))
        st = c.render_graph(4)
        assert len(st) == 4 and all(s.photon_rays > 0 for s in st)
        img = c.render_read()
        c.render_begin(scene.camera, _params(seed=4))
        for t in range(1, 5):
            c.render_pass(t)
        assert _close(img, c.render_read()) < 1e-4
    finally:
        c.close()


def test_graph_refuses_other_renders(scene):
    c = P.Context(0)
    try:
        c.set_scene(scene)
        c.render_begin(scene.camera, _params(mode=P.MODE_COMPAT, num_streams=4, radius_scale=0.1))
        with pytest.raises(P.PppmError) as e:
            c.render_graph(2)
        assert e.value.code == P.E_STATE
    finally:
        c.close()


def test_batch_graph_matches_batch_without_graph():
    jobs = S.config4_jobs(seed=12, n=3, min_side=64, max_side=160, min_tris=2_000, max_tris=20_000,
                          min_photons=20_000, max_photons=80_000)
    imgs = {}
    for use_graph in (False, True):
        b = P.Batch(0)
        b.config(use_graph=use_graph)
        try:
            ids = []
            for k, (sc, alpha) in enumerate(jobs):
                par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=8,
                                            max_bounce_eye=8, alpha=alpha, radius_scale=1 / 32, seed=k + 1)
                ids.append(b.submit(sc, par, 10))
            b.run(autotune=True, max_concurrent=3)
            for i in ids:
                img, st = b.result(i)
                assert st["passes"] == 10 and st["rays"] > 0
                # every pass after the first, the 6 tuning passes (2 candidates) included
                assert st["graph_passes"] == (9 if use_graph else 0) and st["tune_passes"] == 6
                imgs.setdefault(i, []).append(img)
        finally:
            b.close()
    for i, (a, g) in imgs.items():
        assert _close(g, a) < 1e-4
