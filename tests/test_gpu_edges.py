"""Edge cases of the render API: the smallest image, zero bounces, a scene
every ray misses, and calls out of order (status codes, never aborts)."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    return S.small_test_scene(seed=3, subdiv=2, width=16, height=12, photons=5000)


@pytest.mark.parametrize("mode", [P.MODE_COMPAT, P.MODE_CANONICAL, P.MODE_CLASSIC, P.MODE_PATH_TRACING])
def test_one_pixel_one_photon(small, mode):
    cam = S.Camera(small.camera.eye, small.camera.dir, small.camera.up, small.camera.fov, 1, 1)
    c = P.Context(0)
    try:
        c.set_scene(small)
        c.render_begin(cam, P.Context.make_params(mode=mode, photons=1, num_streams=1))
        if mode == P.MODE_CLASSIC:
            # one render point: its box has no extent, so the reference's
            # initial radius is zero and its first update divides by it
            with pytest.raises(P.PppmError) as e:
                c.render_pass(1)
            assert e.value.code == P.E_UNDEFINED
            return
        for t in (1, 2):
            c.render_pass(t)
        img = c.render_read()
        assert img.shape == (1, 1, 3) and np.isfinite(img).all()
    finally:
        c.close()


@pytest.mark.parametrize("mode", [P.MODE_COMPAT, P.MODE_CANONICAL])
def test_zero_bounces_sees_the_environment(small, mode):
    # no eye bounce: every pixel returns the environment in its ray direction
    # and no photon is traced past emission
    c = P.Context(0)
    try:
        c.set_scene(small)
        c.render_begin(small.camera, P.Context.make_params(mode=mode, photons=5000, num_streams=4,
                                                           max_bounce_photon=0, max_bounce_eye=0))
        st = c.render_pass(1)
        assert st.photons_stored == 0 and st.photon_rays == 0 and st.gather_queries == 0
        img = c.render_read()
        assert np.isfinite(img).all() and (img > 0).any()
    finally:
        c.close()


def test_scene_that_every_ray_misses(small):
    # one tiny triangle far behind the camera: all light comes from the env map
    far = np.array([[[1e4, 1e4, 1e4], [1e4 + 1, 1e4, 1e4], [1e4, 1e4 + 1, 1e4]]], np.float32)
    sc = S.Scene("far", far.reshape(-1, 9), np.zeros(1, np.int32), small.mats[:1], small.env, small.camera,
                 photons=2000)
    c = P.Context(0)
    try:
        c.set_scene(sc)
        c.render_begin(sc.camera, P.Context.make_params(mode=P.MODE_CANONICAL, photons=2000, radius_scale=1 / 64))
        st = c.render_pass(1)
        assert st.photons_stored == 0 and st.gather_queries == 0
        assert np.isfinite(c.render_read()).all()
    finally:
        c.close()


def test_calls_out_of_order(small):
    c = P.Context(0)
    try:
        with pytest.raises(P.PppmError) as e:
            c.render_pass(1)
        assert e.value.code == P.E_STATE
        c.set_scene(small)
        c.render_begin(small.camera, P.Context.make_params(mode=P.MODE_CANONICAL, photons=1000, radius_scale=1 / 64))
        with pytest.raises(P.PppmError) as e:
            c.render_pass(2)  # passes run in order 1, 2, ...
        assert e.value.code == P.E_STATE
        with pytest.raises(P.PppmError) as e:
            c.render_begin(small.camera, P.Context.make_params(mode=P.MODE_CANONICAL, photons=0))
        assert e.value.code == P.E_ARG
        with pytest.raises(P.PppmError) as e:
            c.render_image()  # no pass rendered
        assert e.value.code == P.E_STATE
    finally:
        c.close()
