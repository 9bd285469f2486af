"""The C++ host mirror (tatsy-pppm_gb300/host/pppm.hpp) and its appmain-shaped
driver: compile checks on the CPU, a render on the GPU that must equal the
same render through the Python binding (both call the same C ABI)."""
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
