"""Pins the oracle port (oracle/pppm_port.cc) against the reference.

The fixtures hold the compiled reference's outputs (tests/golden/make_golden.py),
so these checks run on any machine. On x86-64, where the fixtures were made,
the port's double arithmetic must reproduce them bit for bit; elsewhere libm
may round transcendental functions differently in the last bit, so a 1e-9
relative tolerance applies to continuous values (indices stay exact).
"""
import platform

import numpy as np
import pytest

import port
import pppm_gb300 as P
import scenes as S
from conftest import scene_from

X86 = platform.machine() in ("x86_64", "AMD64")


def _close(a, b, rtol=1e-9):
    if X86:
        assert np.array_equal(np.asarray(a), np.asarray(b))
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=1e-300)


@pytest.mark.parametrize("suffix", ["", "2"])
def test_port_intersect_matches_reference(golden, suffix):
    g = golden("intersect")
    ps = port.PortScene(scene_from(g["tris" + suffix]))
    tri, t = ps.intersect(g["rays" + suffix])
    assert np.array_equal(tri, g["tri" + suffix])
    assert np.array_equal(t.view(np.uint64), g["t" + suffix].view(np.uint64))


def test_port_env_tables_match_reference(golden):
    g = golden("env")
    sc = scene_from(S.ground(-5.0, 20.0).reshape(-1, 9), env=g["decoded"].astype(np.float32))
    pdf, cdf = port.PortScene(sc).env_tables()
    _close(pdf, g["pdf"])
    _close(cdf, g["cdf"])


@pytest.mark.parametrize("case", [0, 1, 2, 3])
def test_port_knn_matches_reference(golden, case):
    g = golden("knn")
    idx, cnt = port.knn(g["pos"], g["queries"], int(g[f"ntp{case}"]), float(g[f"rad{case}"]))
    assert np.array_equal(cnt, g[f"cnt{case}"])
    assert np.array_equal(idx, g[f"idx{case}"])


def test_port_render_matches_reference(golden):
    g = golden("render_small")
    mats = g["mats"].reshape(-1).view(S.MATERIAL_DTYPE)
    cam = S.Camera(tuple(g["eye"]), tuple(g["dir"]), tuple(g["up"]), float(g["fov"]), int(g["wh"][0]), int(g["wh"][1]))
    sc = S.Scene("render_small", g["tris"], g["mat_id"], mats, g["env"], cam, photons=int(g["nphotons"]))
    ps = port.PortScene(sc)
    par = P.Context.make_params(mode=P.MODE_COMPAT, photons=sc.photons, num_streams=int(g["threads"]))
    out = ps.render(P.Context.make_camera(cam), par, 2, photon_cap=1 << 20)
    assert [s["radius"] for s in out["stats"]] == list(g["radii"])
    assert out["photon_count"] == int(g["photon_count"])
    a = out["photons"][:, :12]  # the port adds each record's path index
    b = g["photons"]
    ka = np.lexsort(a.T[::-1])
    kb = np.lexsort(b.T[::-1])
    _close(a[ka], b[kb])
    _close(out["accum"], g["accum"])
