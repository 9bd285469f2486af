"""Classic PPM (ProgressivePhotonMapping) against the reference.

The fixture holds two passes of the reference's classic PPM with one OpenMP
thread (with more, its render-point updates run under a lock in an order
that changes between runs) and the first 64 requests of its permuted Halton
samplers seeded 0..7.
"""
import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

pytestmark = pytest.mark.gpu


def test_halton_matches_reference(ctx, golden):
    g = golden("classic")
    for s in range(8):
        assert np.array_equal(ctx.halton(s, 64, 200), g["halton"][s])


def test_classic_two_passes(golden):
    g = golden("classic")
    mats = g["mats"].reshape(-1).view(S.MATERIAL_DTYPE)
    cam = S.Camera(tuple(g["eye"]), tuple(g["dir"]), tuple(g["up"]), float(g["fov"]), int(g["wh"][0]), int(g["wh"][1]))
    sc = S.Scene("classic", g["tris"], g["mat_id"], mats, g["env"], cam, photons=int(g["nphotons"]))
    c = P.Context(0)
    try:
        c.set_scene(sc)
        par = P.Context.make_params(mode=P.MODE_CLASSIC, photons=sc.photons, num_streams=int(g["threads"]))
        c.render_begin(sc.camera, par)
        c.render_pass(1)
        c.render_pass(2)
        img = c.render_read()
    finally:
        c.close()
    ref = g["image"]
    rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    close = np.all(rel < 1e-3, axis=2).mean()
    relmse = np.mean((img - ref) ** 2) / np.mean(ref ** 2)
    print(f"pixels within 1e-3: {close:.4f}, relMSE {relmse:.3e}")
    assert close > 0.9
    assert relmse < 1e-3
