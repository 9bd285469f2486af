"""The learned photon proposal inside a canonical render.

The proposal must not change the estimator's expectation: with training
switched off (PPPM_FLAG_LEARNED_FROZEN) every direction still goes through
the MIS resolve kernel, drawn from the BSDF lobe alone, and the image must
agree with the plain render; with training on, the image stays unbiased and
the trained network sends more of the emitted photons into the part of the
scene the camera sees (what it is trained for).
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


def _render(c, sc, flags, passes, seed, photons=300_000):
    c.learned_config(retrain_every=4, steps=16, batch=65536, lr=1e-3, floor_bsdf=0.3, max_log_kappa=4.0,
                     guide_bounces=1)
    par = P.Context.make_params(mode=P.MODE_CANONICAL, photons=photons, max_bounce_photon=12, max_bounce_eye=12,
                                radius_scale=1 / 64, seed=seed, flags=flags)
    c.render_begin(sc.camera, par)
    stats = [c.render_pass(t) for t in range(1, passes + 1)]
    return c.render_read() / passes, stats


def _in_view(sc, pts):
    cam = sc.camera
    eye = np.array(cam.eye)
    f = np.array(cam.dir) / np.linalg.norm(cam.dir)
    u = np.cross(f, np.array(cam.up))
    u /= np.linalg.norm(u)
    v = np.cross(u, f)
    d = pts - eye
    z = d @ f
    h = np.tan(cam.fov * 0.5)
    x, y = (d @ u) / np.maximum(z, 1e-6), (d @ v) / np.maximum(z, 1e-6)
    return (z > 0) & (np.abs(x) < h * cam.width / cam.height) & (np.abs(y) < h)


def test_frozen_proposal_matches_plain(setup):
    sc, c = setup
    ref, _ = _render(c, sc, 0, 128, 99)
    plain = np.mean([(_render(c, sc, 0, 24, s)[0] @ LUM).mean() for s in (1, 2)])
    frozen = np.mean([(_render(c, sc, P.FLAG_LEARNED | P.FLAG_LEARNED_FROZEN, 24, s)[0] @ LUM).mean() for s in (1, 2)])
    r = (ref @ LUM).mean()
    print(f"mean luminance: reference {r:.4f}, plain {plain:.4f}, frozen proposal {frozen:.4f}")
    assert abs(plain / r - 1) < 0.06
    assert abs(frozen / r - 1) < 0.06


def test_trained_proposal_is_unbiased_and_sends_photons_into_view(setup):
    sc, c = setup
    ref, _ = _render(c, sc, 0, 128, 99)
    img, st = _render(c, sc, P.FLAG_LEARNED, 24, 3)
    assert np.isfinite(img).all()
    assert any(s.ms_train > 0 for s in st), "the network was never trained"
    ratio = (img @ LUM).mean() / (ref @ LUM).mean()
    view_learned = _in_view(sc, c.render_photons(4_000_000)[:, :3].astype(np.float64)).sum()
    _render(c, sc, P.FLAG_LEARNED | P.FLAG_LEARNED_FROZEN, 24, 3)
    view_frozen = _in_view(sc, c.render_photons(4_000_000)[:, :3].astype(np.float64)).sum()
    print(f"mean luminance ratio {ratio:.4f}; photons in view per pass: trained {view_learned}, without training "
          f"{view_frozen} ({view_learned / view_frozen:.2f}x)")
    assert abs(ratio - 1) < 0.08
    assert view_learned > 1.5 * view_frozen
