"""Batched uneven jobs: each job's image equals its stand-alone render."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


def test_batch_matches_single_renders():
    jobs = S.config4_jobs(seed=11, n=3, min_side=64, max_side=160, min_tris=2_000, max_tris=20_000,
                          min_photons=20_000, max_photons=80_000)
    b = P.Batch(0)
    ids = []
    pars = []
    for k, (sc, alpha) in enumerate(jobs):
        par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=sc.photons, max_bounce_photon=8, max_bounce_eye=8,
                                    alpha=alpha, radius_scale=1 / 32, seed=k + 1)
        pars.append(par)
        ids.append(b.submit(sc, par, 8))
    b.run(autotune=True, max_concurrent=3)
    c = P.Context(0)
    try:
        for (sc, _), par, i in zip(jobs, pars, ids):
            img, st = b.result(i)
            assert st["passes"] == 8 and st["rays"] > 0 and st["ms_pass_p99"] >= st["ms_pass_p50"] > 0
            c.set_scene(sc)
            c.render_begin(sc.camera, par)
            for t in range(1, 9):
                c.render_pass(t)
            ref = c.render_read()
            # same photons and paths; launch shapes only reorder float sums
            err = np.abs(img - ref).max() / max(np.abs(ref).max(), 1e-12)
            assert err < 1e-4, err
    finally:
        c.close()
        b.close()
