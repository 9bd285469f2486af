"""The C++ host mirror (tatsy-pppm_gb300/host/pppm.hpp) and its appmain-shaped
driver: compile checks on the CPU, a render on the GPU that must equal the
same render through the Python binding (both call the same C ABI)."""
import math
import pathlib
import subprocess

import numpy as np
import pytest

import pppm_gb300 as P
import scenes as S

ROOT = pathlib.Path(__file__).resolve().parents[1]
HOST = ROOT / "tatsy-pppm_gb300" / "host"


def test_mirror_compiles_without_warnings():
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", str(HOST / "appmain_gpu.cc")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ply_round_trip_through_reference_layout(tmp_path):
    """PLY written by scenes.write_ply is read back by the mirror's loader
    rules; the reference loader reads the same file (checked in the oracle
    tests when the reference is built)."""
    tris = S.displace_sphere(S.geodesic_sphere(4), 3.0, 0.05, 1).reshape(-1, 9).astype(np.float32)
    path = tmp_path / "m.ply"
    S.write_ply(path, tris)
    data = path.read_bytes()
    head, body = data.split(b"end_header\n", 1)
    assert b"binary_little_endian" in head
    n = len(tris)
    verts = np.frombuffer(body[: n * 36], "<f4").reshape(-1, 9)
    assert np.array_equal(verts, tris)


@pytest.mark.gpu
def test_appmain_gpu_matches_python_api(tmp_path, golden):
    demo = ROOT / "tatsy-pppm_gb300" / "appmain_gpu"
    assert demo.exists(), "build() makes the demo binary"
    mesh = S.displace_sphere(S.geodesic_sphere(8), 6.0, 0.05, 2, center=(0.0, -4.0, 0.0)).reshape(-1, 9)
    S.write_ply(tmp_path / "mesh.ply", mesh)
    env = golden("env")["decoded"].astype(np.float32)
    S.write_hdr(tmp_path / "env.hdr", env)
    w, h, spp, photons = 96, 64, 2, 40000
    r = subprocess.run([str(demo), str(w), str(h), str(spp), str(tmp_path / "mesh.ply"), str(tmp_path / "env.hdr"),
                        str(tmp_path / "out.ppm"), str(photons), "compat"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    ppm = (tmp_path / "out.ppm").read_bytes()
    img = np.frombuffer(ppm.split(b"255\n", 1)[1], np.uint8).reshape(h, w, 3)
    # the same scene through the Python binding
    parts = [(mesh.reshape(-1, 3, 3).astype(np.float64), 0)]
    mats = [S.material(S.LAMBERTIAN, (0.75, 0.75, 0.75))]
    tiles, tile = 8, 8.0
    for i in range(tiles):
        for j in range(tiles):
            ii, jj = (i - tiles // 2) * tile, (j - tiles // 2) * tile
            p00, p01 = (ii, -10.0, jj), (ii + tile, -10.0, jj)
            p10, p11 = (ii, -10.0, jj + tile), (ii + tile, -10.0, jj + tile)
            even = (i + j) % 2 == 0
            mats.append(S.material(S.PHONG, (0.9, 0.9, 0.9), phong_n=128.0) if even else S.material(S.SPECULAR, (0.2, 0.2, 0.2)))
            parts.append((np.array([[p00, p11, p01]]), len(mats) - 1))
            mats.append(mats[-1])
            parts.append((np.array([[p00, p10, p11]]), len(mats) - 1))
    eye = np.array([-25.0, 5.0, -18.0])
    d = -eye / (np.linalg.norm(eye) + 1e-12)
    cam = S.Camera(tuple(map(float, eye)), tuple(float(np.float32(x)) for x in d), (0.0, 1.0, 0.0), float(np.float32(0.9)), w, h)
    sc = S._assemble("demo", parts, mats, env, cam, photons=photons)
    ctx = P.Context(0)
    ctx.set_scene(sc)
    ctx.render_begin(cam, P.Context.make_params(mode=P.MODE_COMPAT, photons=photons, num_streams=8))
    for t in range(1, spp + 1):
        ctx.render_pass(t)
    acc = ctx.render_read().astype(np.float64) / spp
    ctx.close()
    ref = np.clip(np.power(acc, 1 / 2.2), 0, 1)
    ref = (255.0 * ref).astype(np.uint8)[::-1]
    assert np.mean(np.abs(img.astype(int) - ref.astype(int)) <= 1) > 0.999


def _decode_png(data):
    import struct
    import zlib

    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    rows = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 3 * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 3)


@pytest.mark.gpu
def test_appmain_gpu_path_tracing_writes_pass_pngs(tmp_path, golden):
    """PathTracing through the mirror with a result directory: one PNG per
    sample (the reference's %03d.png), holding the same image as the demo's
    own output after the last sample."""
    demo = ROOT / "tatsy-pppm_gb300" / "appmain_gpu"
    assert demo.exists(), "build() makes the demo binary"
    mesh = S.displace_sphere(S.geodesic_sphere(8), 6.0, 0.05, 2, center=(0.0, -4.0, 0.0)).reshape(-1, 9)
    S.write_ply(tmp_path / "mesh.ply", mesh)
    S.write_hdr(tmp_path / "env.hdr", golden("env")["decoded"].astype(np.float32))
    out = tmp_path / "out"
    out.mkdir()
    w, h, spp = 80, 48, 3
    r = subprocess.run([str(demo), str(w), str(h), str(spp), str(tmp_path / "mesh.ply"), str(tmp_path / "env.hdr"),
                        str(tmp_path / "out.ppm"), "20000", "pt", str(out) + "/"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert sorted(p.name for p in out.iterdir()) == ["001.png", "002.png", "003.png"]
    png = _decode_png((out / "003.png").read_bytes())
    ppm = np.frombuffer((tmp_path / "out.ppm").read_bytes().split(b"255\n", 1)[1], np.uint8).reshape(h, w, 3)
    assert np.mean(np.abs(png.astype(int) - ppm.astype(int)) <= 1) > 0.999


def test_mirror_check_compiles_without_warnings():
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(HOST),
                        str(ROOT / "tests" / "mirror_check.cc")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _f(d, name, dtype):
    return np.fromfile(d / name, dtype)


@pytest.mark.gpu
def test_mirror_classes_match_c_abi(tmp_path, golden):
    """The mirror's Scene (one GPU context per scene: two scenes rendered in
    one program), the QMC sampler type, QBVHAccel, KdTree, HashGrid and
    SubsurfaceIntegrator, driven from C++ with the reference's signatures
    (tests/mirror_check.cc), give what the same calls give through the
    Python binding of the C ABI."""
    exe = tmp_path / "mirror_check"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(HOST), str(ROOT / "tests" / "mirror_check.cc"), "-o",
                        str(exe), f"-L{HOST.parent}", "-lpppm_gb300", f"-Wl,-rpath,{HOST.parent}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    sph = S.displace_sphere(S.geodesic_sphere(4), 4.0, 0.05, 3).reshape(-1, 9)
    a_tris = np.concatenate([sph, S.ground(-5.0, 15.0).reshape(-1, 9)]).astype(np.float32)
    b_tris = S.torus(6.0, 2.0, 40, 20, 0.05, 4, center=(0.0, 2.0, 3.0)).reshape(-1, 9).astype(np.float32)
    # the subsurface sphere in front of scene A's sphere, above its ground
    c_tris = S.displace_sphere(S.geodesic_sphere(5), 2.5, 0.05, 5, center=(0.0, -2.0, -9.0)).reshape(-1, 9)
    c_tris = c_tris.astype(np.float32)
    for name, t in (("a", a_tris), ("b", b_tris), ("c", c_tris)):
        S.write_ply(tmp_path / f"{name}.ply", t)
    envs = {}
    for name, seed in (("a", 1), ("b", 2), ("c", 3)):
        S.write_hdr(tmp_path / f"{name}.hdr", S.sky_env(128, 64, seed, sun_peak=300.0, sun_deg=5.0))
        envs[name] = P.hdr_decode((tmp_path / f"{name}.hdr").read_bytes())
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr + r.stdout

    lam = lambda refl: S.material(S.LAMBERTIAN, refl)  # noqa: E731
    d = np.array([0.0, -0.15, 1.0])
    # Vector3D::normalized multiplies by the reciprocal of (norm + 1e-12)
    inv = 1.0 / (math.sqrt(0.0 * 0.0 + (-0.15) * (-0.15) + 1.0 * 1.0) + 1e-12)
    cam = S.Camera((0.0, 4.0, -24.0), tuple(float(np.float32(x * inv)) for x in d),
                   (0.0, 1.0, 0.0), float(np.float32(0.8)), 48, 32)
    scene_a = S.Scene("a", a_tris, np.zeros(len(a_tris), np.int32), np.array([lam((0.7, 0.6, 0.5))], S.MATERIAL_DTYPE),
                      envs["a"], cam)
    scene_b = S.Scene("b", np.concatenate([b_tris, a_tris]),
                      np.r_[np.zeros(len(b_tris), np.int32), np.ones(len(a_tris), np.int32)],
                      np.array([S.material(S.SPECULAR, (0.9, 0.9, 0.9)), lam((0.3, 0.5, 0.7))], S.MATERIAL_DTYPE),
                      envs["b"], cam)
    ctx = P.Context(0)
    try:
        def py_render(sc, flags=0):
            ctx.set_scene(sc)
            ctx.render_begin(cam, P.Context.make_params(mode=P.MODE_COMPAT, photons=20000, num_streams=8,
                                                        flags=flags))
            for t in (1, 2):
                ctx.render_pass(t)
            return ctx.render_read().reshape(-1) / np.float32(2.0)

        a1, a2 = _f(tmp_path, "render_a1.f32", np.float32), _f(tmp_path, "render_a2.f32", np.float32)
        b = _f(tmp_path, "render_b.f32", np.float32)
        ref_a, ref_b = py_render(scene_a), py_render(scene_b)
        # each scene renders in its own context: A, B, A again in one program
        np.testing.assert_allclose(a1, ref_a, rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(a2, ref_a, rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(b, ref_b, rtol=1e-5, atol=1e-7)
        assert np.abs(a1 - b).mean() > 10 * np.abs(a1 - a2).mean() + 1e-6
        np.testing.assert_allclose(_f(tmp_path, "render_a_qmc.f32", np.float32), py_render(scene_a, P.FLAG_SAMPLER_QMC),
                                   rtol=1e-5, atol=1e-7)

        # QBVHAccel and Scene::intersect: the C ABI's closest hits
        rays = _f(tmp_path, "rays.f32", np.float32).reshape(-1, 6)
        ctx.set_scene(S.Scene("a", a_tris, np.zeros(len(a_tris), np.int32),
                              np.array([lam((0.5, 0.5, 0.5))], S.MATERIAL_DTYPE), None, cam))
        tri, t, _, _ = ctx.intersect(rays, with_hit=False)
        assert np.array_equal(_f(tmp_path, "qbvh_ids.i32", np.int32), tri)
        assert np.array_equal(_f(tmp_path, "scene_ids.i32", np.int32), tri)
        assert (tri >= 0).mean() > 0.2
        dist = _f(tmp_path, "qbvh_dist.f64", np.float64)
        assert np.array_equal(dist[tri >= 0], t[tri >= 0])

        # KdTree::knnSearch for each KnnQuery type
        pts = _f(tmp_path, "kd_points.f32", np.float32).reshape(-1, 3)
        qs = _f(tmp_path, "kd_queries.f32", np.float32).reshape(-1, 3)
        res = _f(tmp_path, "kd_results.i32", np.int32)
        types = [(P.KNN_K_NEAREST | P.KNN_EPSILON_BALL, 1.5, 10), (P.KNN_K_NEAREST, 0.0, 16),
                 (P.KNN_EPSILON_BALL, 0.9, 0)]
        got = [ctx.kdtree_knn(pts, qs, ty, eps, k) for ty, eps, k in types]
        pos = 0
        for i in range(len(qs)):
            for (idx, cnt) in got:
                n = res[pos]
                assert n == cnt[i] and np.array_equal(res[pos + 1:pos + 1 + n], idx[i, :n]), (i, pos)
                pos += 1 + n
        assert pos == len(res)

        # HashGrid::add / operator[]
        boxes = _f(tmp_path, "hash_boxes.f64", np.float64).reshape(-1, 6)
        hpts = _f(tmp_path, "hash_points.f64", np.float64).reshape(-1, 3)
        start, items = ctx.hashgrid_build(boxes[:, :3], boxes[:, 3:], 4093, 1.0 / 0.7, np.full(3, -12.0))
        bk = ctx.hash_points(hpts.astype(np.float32), 4093, 1.0 / 0.7, np.full(3, -12.0))
        got_b = _f(tmp_path, "hash_buckets.i32", np.int32)
        pos = 0
        for h in bk:
            n = got_b[pos]
            assert np.array_equal(got_b[pos + 1:pos + 1 + n], items[start[h]:start[h + 1]])
            pos += 1 + n
        assert pos == len(got_b)

        # SubsurfaceIntegrator::initialize + irradiance
        sss = S.material(S.LAMBERTIAN, (0.6, 0.55, 0.5), sigma_a=(0.01, 0.02, 0.03), sigmap_s=(1.0, 1.5, 2.0),
                         eta=1.3, scale=1.0, bssrdf=True)
        scene_c = S.Scene("c", np.concatenate([c_tris, a_tris]),
                          np.r_[np.zeros(len(c_tris), np.int32), np.ones(len(a_tris), np.int32)],
                          np.array([sss, lam((0.5, 0.5, 0.5))], S.MATERIAL_DTYPE), envs["c"], cam)
        pts_c, nrm_c, _ = ctx.poisson_disk(c_tris, 0.6)
        ctx.set_scene(scene_c)
        par = P.Context.make_params(mode=P.MODE_COMPAT, photons=20000, num_streams=8, sss_time=424242)
        ph = ctx.subsurface_photons(par)
        irad = ctx.subsurface_photon_irradiance(ph, np.concatenate([pts_c, nrm_c], 1), 20000, 16.0, 128)
        ipts = np.zeros((len(pts_c), 10), np.float32)
        ipts[:, :3], ipts[:, 3:6], ipts[:, 7:] = pts_c, nrm_c, irad
        ipts[:, 6] = np.float32((0.5 * 0.6) ** 2 * np.pi)
        at = _f(tmp_path, "sss_at.f64", np.float64).reshape(-1, 3)
        ref = ctx.dipole_irradiance(np.array([sss], S.MATERIAL_DTYPE)[0], ipts, 0.05, at.astype(np.float32))
        assert _f(tmp_path, "sss_points.i64", np.int64)[0] == len(pts_c) > 10
        got_i = _f(tmp_path, "sss_irradiance.f64", np.float64).reshape(-1, 3)
        assert np.abs(ref).max() > 0
        np.testing.assert_allclose(got_i, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
    finally:
        ctx.close()
