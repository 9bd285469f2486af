"""The learned photon proposal inside a canonical render.

The proposal must not change the estimator's expectation. Without training
(PPPM_FLAG_LEARNED_FROZEN) the network is never used: the render is the
plain render, draw for draw. With training on, the network proposes the
environment direction of every photon (one-sample MIS with the reference's
own cell sampling at a floor of 0.3) and, optionally, the directions of
Lambertian bounces. The image must stay unbiased against a plain reference,
and the trained proposal must lower the error of the plain method at equal
passes: what the network gains over the method without it.
"""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu

LUM = np.array([0.2126, 0.7152, 0.0722])


@pytest.fixture(scope="module")
def setup():
    sc = S.config2(width=160, height=90, freq=32)
    c = P.Context(0)
    c.set_scene(sc)
    yield sc, c
    c.close()


@pytest.fixture(scope="module")
def reference(setup):
    sc, c = setup
    img, _ = _render(c, sc, 0, 1024, 99)
    return img


def _render(c, sc, flags, passes, seed, photons=300_000, guide_bounces=0):
    c.learned_config(retrain_every=2, steps=2, batch=65536, lr=4e-3, floor_bsdf=0.3, max_log_kappa=7.0,
                     guide_bounces=guide_bounces)
    par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=photons, max_bounce_photon=12, max_bounce_eye=12,
                                radius_scale=1 / 64, seed=seed, flags=flags)
    c.render_begin(sc.camera, par)
    stats = [c.render_pass(t) for t in range(1, passes + 1)]
    return c.render_read() / passes, stats


def _relmse(x, r):
    return float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2)))


def test_frozen_proposal_is_the_plain_render(setup):
    sc, c = setup
    plain, _ = _render(c, sc, 0, 12, 5)
    frozen, _ = _render(c, sc, P.FLAG_LEARNED | P.FLAG_LEARNED_FROZEN, 12, 5)
    # the same photons and paths; the order of the float sums in the gather
    # follows the atomics of the photon deposits, so the last bits may differ
    np.testing.assert_allclose(frozen, plain, rtol=1e-5, atol=1e-7)


def test_frozen_bounce_resolve_matches_plain(setup, reference):
    # every Lambertian bounce drawn by the MIS resolve kernel from the BSDF
    # lobe alone: other draws, the same expectation
    sc, c = setup
    r = (reference @ LUM).mean()
    frozen = np.mean([(_render(c, sc, P.FLAG_LEARNED | P.FLAG_LEARNED_FROZEN, 24, s, guide_bounces=1)[0]
                       @ LUM).mean() for s in (1, 2)])
    print(f"mean luminance: reference {r:.4f}, frozen bounce resolve {frozen:.4f}")
    assert abs(frozen / r - 1) < 0.06


def test_trained_proposal_gains_over_plain(setup, reference):
    sc, c = setup
    passes = 32
    plain = [_render(c, sc, 0, passes, s)[0] for s in (3, 4)]
    learned, stats = [], []
    for s in (3, 4):
        img, st = _render(c, sc, P.FLAG_LEARNED, passes, s)
        learned.append(img)
        stats += st
    assert all(np.isfinite(x).all() for x in learned)
    assert any(s.ms_train > 0 for s in stats), "the network was never trained"
    e_plain = np.mean([_relmse(x, reference) for x in plain])
    e_learned = np.mean([_relmse(x, reference) for x in learned])
    r = (reference @ LUM).mean()
    ratio = np.mean([(x @ LUM).mean() for x in learned]) / r
    print(f"relMSE at {passes} passes: plain {e_plain:.4f}, learned {e_learned:.4f} "
          f"({e_plain / e_learned:.1f}x lower); learned mean luminance / reference {ratio:.4f}")
    assert abs(ratio - 1) < 0.05
    assert e_learned < 0.5 * e_plain


def test_trained_bounce_guiding_stays_unbiased(setup, reference):
    sc, c = setup
    img, st = _render(c, sc, P.FLAG_LEARNED, 24, 6, guide_bounces=1)
    assert np.isfinite(img).all()
    assert any(s.ms_train > 0 for s in st)
    ratio = (img @ LUM).mean() / (reference @ LUM).mean()
    print(f"bounce guiding: mean luminance / reference {ratio:.4f}")
    assert abs(ratio - 1) < 0.06
