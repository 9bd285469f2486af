"""Batched uneven jobs: each job's image equals its stand-alone render, with
the autotuner's tuning passes (every pppm_tune knob, three interleaved
passes per candidate) captured in the first batch graph or run eagerly."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_single_renders(use_graph):
    passes = 14  # 4 candidates x 3 tuning passes after the first pass, then 1
    jobs = S.config4_jobs(seed=11, n=3, min_side=64, max_side=160, min_tris=2_000, max_tris=20_000,
                          min_photons=20_000, max_photons=80_000)
    b = P.Batch(0)
    b.config(use_graph=use_graph)
    ids = []
    pars = []
    for k, (sc, alpha) in enumerate(jobs):
        par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=8, max_bounce_eye=8,
                                    alpha=alpha, radius_scale=1 / 32, seed=k + 1)
        pars.append(par)
        ids.append(b.submit(sc, par, passes))
    b.run(autotune=True, max_concurrent=3)
    c = P.Context(0)
    try:
        for (sc, _), par, i in zip(jobs, pars, ids):
            img, st = b.result(i)
            assert st["passes"] == passes and st["rays"] > 0 and st["ms_pass_p99"] >= st["ms_pass_p50"] > 0
            assert st["tune_passes"] == 12 and 0 <= st["tune_candidate"] < 4, st
            assert st["graph_passes"] == (passes - 1 if use_graph else 0)
            assert st["gather_stage"] in (64, 128, 256) and 1 <= st["refill"] <= 32, st
            c.set_scene(sc)
            c.render_begin(sc.camera, par)
            for t in range(1, passes + 1):
                c.render_pass(t)
            ref = c.render_read()
            # same photons and paths; launch shapes only reorder float sums
            err = np.abs(img - ref).max() / max(np.abs(ref).max(), 1e-12)
            assert err < 1e-4, err
    finally:
        c.close()
        b.close()


def test_short_jobs_are_not_tuned():
    sc, alpha = S.config4_jobs(seed=12, n=1, min_side=64, max_side=64, min_tris=2_000, max_tris=2_000,
                               min_photons=10_000, max_photons=10_000)[0]
    b = P.Batch(0)
    try:
        par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=8,
                                    max_bounce_eye=8, alpha=alpha, radius_scale=1 / 32)
        i = b.submit(sc, par, 7)
        b.run(autotune=True, max_concurrent=1)
        _, st = b.result(i, image=False)
        assert st["tune_passes"] == 0 and st["tune_candidate"] == -1 and st["passes"] == 7
    finally:
        b.close()


def test_batch_tunes_compat_jobs_eagerly():
    """A compat job cannot be captured: it tunes through pppm_render_pass
    over the knobs its gather has (blocks, refill, exact batch) and keeps
    the reference's cell size; its image is the stand-alone render's."""
    sc, alpha = S.config4_jobs(seed=13, n=1, min_side=64, max_side=64, min_tris=3_000, max_tris=3_000,
                               min_photons=30_000, max_photons=30_000)[0]
    par = P.Context.make_params(mode=P.MODE_COMPAT, photons=sc.photons, num_streams=8, max_bounce_photon=8,
                                max_bounce_eye=8, alpha=alpha)
    b = P.Batch(0)
    c = P.Context(0)
    try:
        i = b.submit(sc, par, 10)
        b.run(autotune=True, max_concurrent=1)
        img, st = b.result(i)
        assert st["graph_passes"] == 0 and st["tune_passes"] == 6 and 0 <= st["tune_candidate"] < 2, st
        assert st["cell_factor"] == 1.0
        c.set_scene(sc)
        c.render_begin(sc.camera, par)
        for t in range(1, 11):
            c.render_pass(t)
        # compat renders repeat bit for bit, whatever the launch shapes
        np.testing.assert_array_equal(img, c.render_read())
    finally:
        c.close()
        b.close()
