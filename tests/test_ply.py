"""PLY input and mesh placement (pppm_ply_decode, pppm_mesh_*) against the
reference's Trimesh::load, fitToBBox, scale, putOnPlane and translate
(trimesh.cc:139-320). Host code only: runs without a GPU.

The golden fixture holds synthetic PLY images with the reference's vertices
and faces after its placement (bit-exact), and digests of the reference's
own assets (bunny.ply, rt3.ply) placed as its demo driver places them; those
are checked where PPPM_REFERENCE_ASSETS names a directory holding the
assets.
"""
import hashlib
import os
import pathlib

import numpy as np
import pytest

import pppm_gb300 as P


def _place(m, fit, scale, plane, move):
    if fit is not None:
        m.fit_to_bbox(fit[0], fit[1])
    if scale != 1.0:
        m.scale(scale)
    if plane is not None:
        m.put_on_plane(plane[0], plane[1:])
    return m.translate(move)


def test_decode_and_placement_match_reference(golden):
    g = golden("ply")
    for i in range(int(g["cases"])):
        fit = None if np.isnan(g[f"fit_{i}"]).any() else g[f"fit_{i}"]
        plane = None if np.isnan(g[f"plane_{i}"]).any() else g[f"plane_{i}"]
        m = P.Trimesh.load(g[f"ply_{i}"].tobytes())
        _place(m, fit, float(g[f"scale_{i}"]), plane, g[f"move_{i}"])
        np.testing.assert_array_equal(m.faces, g[f"ref_faces_{i}"])
        # bit for bit, signed zeros included
        assert m.vertices.tobytes() == np.ascontiguousarray(g[f"ref_verts_{i}"]).tobytes(), i


def test_reference_assets(golden):
    d = os.environ.get("PPPM_REFERENCE_ASSETS")
    if not d:
        pytest.skip("PPPM_REFERENCE_ASSETS not set")
    g = golden("ply")
    demo = {"bunny.ply": (((-5, -5, -5), (5, 5, 5)), 0.8, (10.0, 0, 1, 0), (5, 0, -10)),
            "rt3.ply": (((-10, -10, -10), (10, 10, 10)), 1.5, (10.0, 0, 1, 0), (20, 0, -5))}
    for name, digest in zip(g["asset_names"], g["asset_digests"]):
        path = pathlib.Path(d) / str(name)
        if not path.exists():
            continue
        m = _place(P.Trimesh.load(path), *demo[str(name)])
        h = hashlib.sha256(m.vertices.astype("<f8").tobytes() + m.faces.astype("<i4").tobytes()).hexdigest()
        assert f"{m.num_verts()} {m.num_faces()} {h}" == str(digest)


def _ply(header_lines, body=b""):
    return ("\n".join(header_lines) + "\n").encode() + body


GOOD_HEAD = ["ply", "format binary_little_endian 1.0", "element vertex 3", "property float x", "property float y",
             "property float z", "element face 1", "property list uchar int vertex_indices", "end_header"]
GOOD_BODY = np.float32([0, 0, 0, 1, 0, 0, 0, 1, 0]).tobytes() + b"\x03" + np.int32([0, 1, 2]).tobytes()


def _status(data):
    lib = P.load()
    import ctypes
    buf = np.frombuffer(data, np.uint8)
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    v = np.zeros(64, np.float32)
    f = np.zeros(64, np.int32)
    r = lib.pppm_ply_decode(buf.ctypes.data, buf.size, v.ctypes.data, v.size, f.ctypes.data, f.size,
                            ctypes.byref(nv), ctypes.byref(nf))
    return r, nv.value, nf.value


def test_good_minimal_mesh():
    assert _status(_ply(GOOD_HEAD, GOOD_BODY)) == (P.OK, 3, 1)
    m = P.Trimesh.load(_ply(GOOD_HEAD, GOOD_BODY))
    np.testing.assert_array_equal(m.triangles(), np.float32([[0, 0, 0, 1, 0, 0, 0, 1, 0]]))


@pytest.mark.parametrize("what", ["crlf_id", "ascii", "big_endian", "other_element", "zero_faces", "quad",
                                  "truncated", "index_out_of_range", "negative_index"])
def test_inputs_the_reference_rejects(what):
    head, body = list(GOOD_HEAD), GOOD_BODY
    if what == "crlf_id":
        head[0] = "ply\r"
    elif what == "ascii":
        head[1] = "format ascii 1.0"
    elif what == "big_endian":
        head[1] = "format binary_big_endian 1.0"
    elif what == "other_element":
        head.insert(6, "element edge 1")
    elif what == "zero_faces":
        head[6] = "element face 0"
    elif what == "quad":
        body = body[:36] + b"\x04" + body[37:] + np.int32([2]).tobytes()
    elif what == "truncated":
        body = body[:-2]
    elif what == "index_out_of_range":
        body = body[:37] + np.int32([0, 1, 3]).tobytes()
    elif what == "negative_index":
        body = body[:37] + np.int32([0, -1, 2]).tobytes()
    assert _status(_ply(head, body))[0] == P.E_ARG


def test_header_without_end_is_an_empty_mesh():
    # the reference's reader leaves its mesh empty when end_header never comes
    assert _status(_ply(GOOD_HEAD[:-1]))[:3] == (P.OK, 0, 0)


def test_short_buffers_and_size_query():
    import ctypes
    lib = P.load()
    data = np.frombuffer(_ply(GOOD_HEAD, GOOD_BODY), np.uint8)
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    assert lib.pppm_ply_decode(data.ctypes.data, data.size, None, 0, None, 0, ctypes.byref(nv),
                               ctypes.byref(nf)) == P.OK
    assert (nv.value, nf.value) == (3, 1)
    v = np.zeros(8, np.float32)
    f = np.zeros(3, np.int32)
    assert lib.pppm_ply_decode(data.ctypes.data, data.size, v.ctypes.data, v.size, f.ctypes.data, f.size,
                               ctypes.byref(nv), ctypes.byref(nf)) == P.E_CAPACITY


MIRROR_DRIVER = r'''
#include <cstdio>
#include <cstdlib>
#include "pppm.hpp"
// argv: ply fit(0/1) minx miny minz maxx maxy maxz scale plane(0/1) d nx ny nz mx my mz
int main(int argc, char** argv) {
    if (argc != 18) return 2;
    double a[17];
    for (int i = 2; i < 18; i++) a[i - 1] = std::atof(argv[i]);
    Trimesh m(argv[1]);
    if (a[1] != 0.0) m.fitToBBox(BBox(a[2], a[3], a[4], a[5], a[6], a[7]));
    if (a[8] != 1.0) m.scale(a[8]);
    if (a[9] != 0.0) m.putOnPlane(Plane(a[10], Vector3D(a[11], a[12], a[13])));
    m.translate(Vector3D(a[14], a[15], a[16]));
    for (size_t i = 0; i < m.numVerts(); i++) {
        const Vector3D v = m.getVertex((int)i);
        std::printf("%a %a %a\n", v.x(), v.y(), v.z());
    }
    return 0;
}
'''


def test_host_mirror_trimesh_matches_reference(tmp_path, golden):
    """The C++ mirror's Trimesh (load, fitToBBox, scale, putOnPlane,
    translate) gives the reference's vertices bit for bit."""
    import subprocess
    root = pathlib.Path(__file__).resolve().parents[1]
    lib_dir = root / "tatsy-pppm_gb300"
    if not (lib_dir / "libpppm_gb300.so").exists():
        pytest.skip("library not built")
    src = tmp_path / "drv.cc"
    src.write_text(MIRROR_DRIVER)
    exe = tmp_path / "drv"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{lib_dir / 'host'}", str(src), "-o",
                        str(exe), f"-L{lib_dir}", "-lpppm_gb300", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = golden("ply")
    for i in range(int(g["cases"])):
        fit = g[f"fit_{i}"]
        plane = g[f"plane_{i}"]
        path = tmp_path / f"m{i}.ply"
        path.write_bytes(g[f"ply_{i}"].tobytes())
        args = [str(path), "0" if np.isnan(fit).any() else "1", *[repr(float(x)) for x in np.nan_to_num(fit).ravel()],
                repr(float(g[f"scale_{i}"])), "0" if np.isnan(plane).any() else "1",
                *[repr(float(x)) for x in np.nan_to_num(plane)], *[repr(float(x)) for x in g[f"move_{i}"]]]
        out = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=60)
        assert out.returncode == 0, out.stderr
        got = np.array([[float.fromhex(t) for t in line.split()] for line in out.stdout.splitlines()])
        ref = g[f"ref_verts_{i}"]
        assert got.shape == ref.shape
        assert np.array_equal(got, ref) and np.array_equal(np.signbit(got), np.signbit(ref)), i
