"""Parity of the path tracer (PPPM_MODE_PATH_TRACING) against the
reference's PathTracing::render.

The fixtures hold the reference's linear buffer after two samples per pixel
with eight XorShift streams (rows y to stream y % 8, a 200-number tape per
pixel), on the small mixed-material scene and, in a fresh process with
time(NULL) fixed, on the subsurface scene. The GPU draws the same tapes, so
paths follow the same random numbers and differ only where FP32 shading
moves a ray across a triangle edge: most pixels agree to 1e-3 and the image
to a small relMSE."""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


def _scene(g):
    mats = g["mats"].reshape(-1).view(S.MATERIAL_DTYPE)
    cam = S.Camera(tuple(g["eye"]), tuple(g["dir"]), tuple(g["up"]), float(g["fov"]), int(g["wh"][0]), int(g["wh"][1]))
    return S.Scene("pt", g["tris"], g["mat_id"], mats, g["env"], cam, photons=int(g["nphotons"]))


def _check(img, ref, tag):
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    close = np.all(rel < 1e-3, axis=2).mean()
    relmse = np.mean((img - ref) ** 2) / np.mean(ref ** 2)
    print(f"{tag}: pixels within 1e-3: {close:.4f}, relMSE {relmse:.3e}")
    assert close > 0.9
    assert relmse < 1e-3


@pytest.mark.parametrize("name", ["path_trace", "path_trace_sss"])
def test_path_trace_two_samples(golden, name):
    g = golden(name)
    sc = _scene(g)
    c = P.Context(0)
    try:
        c.set_scene(sc)
        par = P.Context.make_params(mode=P.MODE_PATH_TRACING, photons=sc.photons, num_streams=int(g["threads"]),
                                    max_bounce_eye=64, sss_time=int(g["sss_time"]) if "sss_time" in g.files else 0)
        c.render_begin(sc.camera, par)
        st = [c.render_pass(t) for t in (1, 2)]
        assert all(s.eye_rays > 0 for s in st)
        img = c.render_read()
    finally:
        c.close()
    _check(img, g["accum"].astype(np.float64), name)


def test_path_tracer_is_consistent():
    # more samples of the same estimator: 64-sample renders from different
    # streams agree with a 512-sample render in mean luminance (the
    # reference's PathTracing and its PPM differ by a constant factor in
    # brightness: the photon flux area / (pdf N) of Envmap::samplePhoton is
    # not the emission disc's, so PPM is not the comparison here)
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20000)
    c = P.Context(0)
    lum = np.array([0.2126, 0.7152, 0.0722])
    try:
        c.set_scene(sc)
        c.render_begin(sc.camera, P.Context.make_params(mode=P.MODE_PATH_TRACING, num_streams=16))
        n = 512
        for t in range(1, n + 1):
            c.render_pass(t)
        ref = (c.render_read() / n @ lum).mean()
        means = []
        for streams in (3, 5):
            c.render_begin(sc.camera, P.Context.make_params(mode=P.MODE_PATH_TRACING, num_streams=streams))
            for t in range(1, 65):
                c.render_pass(t)
            means.append((c.render_read() / 64 @ lum).mean())
    finally:
        c.close()
    print(f"mean luminance: 512 samples {ref:.4f}, 64 samples {means}")
    assert all(abs(m / ref - 1) < 0.03 for m in means)
