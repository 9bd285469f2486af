"""ctypes binding of the reference harness (oracle/_ref/libpppm_refharness.so).

Test infrastructure only: the library is the UNMODIFIED tatsy-pppm reference
compiled from its own sources by oracle/Makefile plus oracle/ref_harness.cc.
It exists only where the reference sources are present (this build
container); tests that need it skip elsewhere. Set OMP_NUM_THREADS before the
first call: the reference seeds one RNG stream per OpenMP thread
(ppm_probabilistic.cc:58-73), so the thread count is part of its input.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import tempfile

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libpppm_refharness.so"
REF_SOURCES = pathlib.Path("/root/reference/sources")

_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int32)
_U = ctypes.POINTER(ctypes.c_uint32)


def available() -> bool:
    return LIB_PATH.exists()


def build() -> bool:
    """Builds oracle/_ref from the reference sources when they are present."""
    if not REF_SOURCES.exists():
        return LIB_PATH.exists()
    import subprocess

    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"-j{os.cpu_count() or 4}"], check=True)
    return LIB_PATH.exists()


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError("reference harness not built (make -C oracle ref)")
        _lib = ctypes.CDLL(str(LIB_PATH))
        _lib.rh_scene_create.restype = ctypes.c_void_p
        for name in ("rh_scene_destroy", "rh_scene_finalize"):
            getattr(_lib, name).argtypes = [ctypes.c_void_p]
        _lib.rh_scene_add.argtypes = [ctypes.c_void_p, _F, ctypes.c_int, ctypes.c_void_p]
        _lib.rh_scene_add_ply.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        _lib.rh_mesh_place.argtypes = [ctypes.c_char_p, ctypes.c_int, _D, _D, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_double, _D, _D, _D, ctypes.c_int, _I, ctypes.c_int, _I]
        _lib.rh_mesh_place.restype = ctypes.c_int
        _lib.rh_scene_set_envmap.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        _lib.rh_write_hdr.argtypes = [ctypes.c_char_p, _F, ctypes.c_int, ctypes.c_int]
        _lib.rh_load_hdr.argtypes = [ctypes.c_char_p, _D, ctypes.c_int, _I, _I]
        _lib.rh_envmap_tables.argtypes = [ctypes.c_void_p, _D, _D]
        _lib.rh_envmap_lookup.argtypes = [ctypes.c_void_p, _D, ctypes.c_int, _D]
        _lib.rh_emit.argtypes = [ctypes.c_void_p, _D, ctypes.c_int, ctypes.c_int, _D, _D, _D]
        _lib.rh_intersect.argtypes = [ctypes.c_void_p, _F, ctypes.c_int, _I, _D, _D, _D]
        _lib.rh_xorshift.argtypes = [ctypes.c_uint32, ctypes.c_int, _U]
        _lib.rh_xorshift_reals.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_int, _D]
        _lib.rh_on_hemisphere.argtypes = [_D, _D, ctypes.c_int, _D]
        _lib.rh_bsdf_sample.argtypes = [ctypes.c_void_p, _D, _D, _D, ctypes.c_int, _D, _D]
        _lib.rh_camera_rays.argtypes = [_D, _D, _D, ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, _D, _D]
        _lib.rh_hash_points.argtypes = [ctypes.c_int, ctypes.c_double, _D, _D, _F, ctypes.c_int, _U]
        _lib.rh_hash_add_boxes.argtypes = [ctypes.c_int, ctypes.c_double, _D, _D, _D, _D, ctypes.c_int, _I, _I, ctypes.c_int]
        _lib.rh_hash_add_boxes.restype = ctypes.c_int
        _lib.rh_knn.argtypes = [_F, ctypes.c_int, _F, ctypes.c_int, ctypes.c_int, ctypes.c_double, _I, _I, ctypes.c_int]
        _lib.rh_knn.restype = ctypes.c_int
        _lib.rh_gather.argtypes = [ctypes.c_void_p, _F, ctypes.c_int, ctypes.c_double, ctypes.c_int, _F, ctypes.c_int, _D]
        _lib.rh_render_passes.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _D, _D, _D, ctypes.c_int, _I]
        _lib.rh_render_passes.restype = ctypes.c_int
        _lib.rh_dipole_rd.argtypes = [ctypes.c_void_p, _D, ctypes.c_int, _D]
        _lib.rh_dipole_fdr.argtypes = [ctypes.c_void_p]
        _lib.rh_dipole_fdr.restype = ctypes.c_double
        _lib.rh_dipole_irradiance.argtypes = [ctypes.c_void_p, _D, ctypes.c_int, ctypes.c_double, _D, ctypes.c_int, _D]
        _lib.rh_poisson_disk.argtypes = [_F, ctypes.c_int, ctypes.c_double, _D, _D, ctypes.c_int]
        _lib.rh_poisson_disk.restype = ctypes.c_int
        _lib.rh_classic_passes.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _D]
        _lib.rh_path_trace.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _D]
        _lib.rh_halton.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_int, _D]
        _lib.rh_sss_photons.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint, _D, ctypes.c_int, _I]
        _lib.rh_kdtree_knn.argtypes = [_F, ctypes.c_int, _F, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, _I, _I, ctypes.c_int]
        _lib.rh_kdtree_knn.restype = ctypes.c_int
        _lib.rh_image_bytes.argtypes = [_D, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, _D]
        _lib.rh_irradiance_pm.argtypes = [_D, ctypes.c_int, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, _D]
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def num_threads() -> int:
    return lib().rh_num_threads()


class RefScene:
    """A reference Scene built through Scene::add + setAccelerator."""

    def __init__(self, scene, env_path=None):
        L = lib()
        self.h = L.rh_scene_create()
        tris = np.ascontiguousarray(scene.tris, np.float32)
        mats = np.ascontiguousarray(scene.mats)
        # one Scene::add per material, triangles in scene order within it;
        # scene ids are kept by adding runs of equal material ids in order
        mid = scene.mat_id
        runs = np.flatnonzero(np.diff(mid)) + 1
        starts = np.concatenate([[0], runs])
        ends = np.concatenate([runs, [len(mid)]])
        for s, e in zip(starts, ends):
            m = np.ascontiguousarray(mats[mid[s]])
            L.rh_scene_add(self.h, _p(np.ascontiguousarray(tris[s:e]), _F), int(e - s), m.ctypes.data)
        L.rh_scene_finalize(self.h)
        self._tmp = None
        if scene.env is not None:
            if env_path is None:
                self._tmp = tempfile.TemporaryDirectory()
                env_path = os.path.join(self._tmp.name, "env.hdr")
            write_hdr(env_path, scene.env)
            L.rh_scene_set_envmap(self.h, env_path.encode())

    def close(self):
        if self.h:
            lib().rh_scene_destroy(self.h)
            self.h = None
        if self._tmp is not None:
            self._tmp.cleanup()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def intersect(self, rays):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = rays.shape[0]
        tri = np.zeros(n, np.int32)
        t = np.zeros(n)
        pos = np.zeros((n, 3))
        nrm = np.zeros((n, 3))
        lib().rh_intersect(self.h, _p(rays, _F), n, _p(tri, _I), _p(t, _D), _p(pos, _D), _p(nrm, _D))
        return tri, t, pos, nrm

    def env_tables(self):
        pdf = np.zeros(4096)
        cdf = np.zeros(4096)
        lib().rh_envmap_tables(self.h, _p(pdf, _D), _p(cdf, _D))
        return pdf, cdf

    def env_lookup(self, dirs):
        dirs = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
        out = np.zeros_like(dirs)
        lib().rh_envmap_lookup(self.h, _p(dirs, _D), dirs.shape[0], _p(out, _D))
        return out

    def emit(self, tapes, num_photons):
        tapes = np.ascontiguousarray(tapes, np.float64).reshape(-1, 5)
        n = tapes.shape[0]
        pos, d, flux = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        lib().rh_emit(self.h, _p(tapes, _D), n, int(num_photons), _p(pos, _D), _p(d, _D), _p(flux, _D))
        return pos, d, flux

    def gather(self, photons12, radius, gather_photons, rays):
        photons12 = np.ascontiguousarray(photons12, np.float32).reshape(-1, 12)
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.zeros((rays.shape[0], 3))
        lib().rh_gather(self.h, _p(photons12, _F), photons12.shape[0], float(radius), int(gather_photons), _p(rays, _F),
                        rays.shape[0], _p(out, _D))
        return out

    def classic_passes(self, camera, photons, npasses):
        """Passes of ProgressivePhotonMapping (classic PPM): the image
        (emission + flux / (pi r2)) * coeff per pixel, not divided by the
        pass count."""
        job = _PassJob()
        job.eye[:] = camera.eye
        job.dir[:] = camera.dir
        job.up[:] = camera.up
        job.fov = camera.fov
        job.w, job.h = camera.width, camera.height
        job.photons = photons
        job.npasses = npasses
        img = np.zeros((camera.height, camera.width, 3))
        lib().rh_classic_passes(self.h, ctypes.byref(job), _p(img, _D))
        return img

    def path_trace(self, camera, photons, npasses, sss_time=0):
        """npasses samples per pixel of PathTracing::render (pseudo-random
        sampler): the linear buffer, row y = camera row y, not divided by the
        sample count."""
        job = _PassJob()
        job.eye[:] = camera.eye
        job.dir[:] = camera.dir
        job.up[:] = camera.up
        job.fov = camera.fov
        job.w, job.h = camera.width, camera.height
        job.photons = photons
        job.gatherPhotons = 128
        job.gatherRadius = 16.0
        job.npasses = npasses
        job.sssTime = int(sss_time)
        accum = np.zeros((camera.height, camera.width, 3))
        lib().rh_path_trace(self.h, ctypes.byref(job), _p(accum, _D))
        return accum

    def sss_photons(self, photons, sss_time, cap=1 << 20):
        """SubsurfaceIntegrator::buildPhotonMap with time(NULL) = sss_time:
        its records, 12 doubles each (position, flux, direction, normal)."""
        out = np.zeros((cap, 12))
        cnt = np.zeros(1, np.int32)
        lib().rh_sss_photons(self.h, int(photons), int(sss_time), _p(out, _D), cap, _p(cnt, _I))
        return out[: min(int(cnt[0]), cap)]

    def render_passes(self, camera, photons, npasses, gather_photons=128, gather_radius=16.0, photon_cap=0,
                      sss_time=0, qmc=False):
        """Passes 1..npasses of ProgressivePhotonMappingProb::render. With a
        BSSRDF in the scene, pass t seeds its subsurface photon streams with
        time(NULL) = sss_time + t - 1 and the Poisson sampler continues the
        process-wide RNG (reproducible in a fresh process only). qmc: the
        RANDOM_SAMPLER_QUASI_MONTE_CARLO sampler type (Halton(200, true, i))."""
        job = _PassJob()
        job.eye[:] = camera.eye
        job.dir[:] = camera.dir
        job.up[:] = camera.up
        job.fov = camera.fov
        job.w, job.h = camera.width, camera.height
        job.photons = photons
        job.gatherPhotons = gather_photons
        job.gatherRadius = gather_radius
        job.npasses = npasses
        job.sssTime = int(sss_time)
        job.sampler = 1 if qmc else 0
        accum = np.zeros((camera.height, camera.width, 3))
        radii = np.zeros(npasses)
        cnt = np.zeros(1, np.int32)
        ph = np.zeros((max(photon_cap, 1), 12))
        lib().rh_render_passes(self.h, ctypes.byref(job), _p(accum, _D), _p(radii, _D), _p(ph, _D) if photon_cap else None,
                               photon_cap, _p(cnt, _I) if photon_cap else None)
        out = dict(accum=accum, radii=radii)
        if photon_cap:
            out["photons"] = ph[: min(cnt[0], photon_cap)]
            out["photon_count"] = int(cnt[0])
        return out


def image_bytes(buffer, t, tonemap=False):
    """The reference's pass output bytes (rh_image_bytes) of an H x W x 3
    accumulation buffer after t passes: H x W x 3 uint8, rows flipped, and
    the doubles Image::toByte received."""
    buf = np.ascontiguousarray(buffer, np.float64)
    h, w = buf.shape[:2]
    out = np.zeros((h, w, 3), np.uint8)
    vals = np.zeros((h, w, 3))
    lib().rh_image_bytes(_p(buf, _D), w, h, int(t), 1 if tonemap else 0, out.ctypes.data, _p(vals, _D))
    return out, vals


def halton(seed, count, n=200):
    out = np.zeros((count, n))
    lib().rh_halton(int(seed), int(count), int(n), _p(out, _D))
    return out


class _PassJob(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_double * 3), ("dir", ctypes.c_double * 3), ("up", ctypes.c_double * 3),
                ("fov", ctypes.c_double), ("w", ctypes.c_int), ("h", ctypes.c_int), ("photons", ctypes.c_int),
                ("gatherPhotons", ctypes.c_int), ("gatherRadius", ctypes.c_double), ("npasses", ctypes.c_int),
                ("sssTime", ctypes.c_uint), ("sampler", ctypes.c_int)]


def write_hdr(path, rgb):
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    lib().rh_write_hdr(str(path).encode(), _p(rgb, _F), w, h)


def load_hdr(path, cap_pixels=1 << 24):
    out = np.zeros(cap_pixels * 3)
    w = np.zeros(1, np.int32)
    h = np.zeros(1, np.int32)
    r = lib().rh_load_hdr(str(path).encode(), _p(out, _D), cap_pixels, _p(w, _I), _p(h, _I))
    if r != 0:
        raise RuntimeError("image larger than cap")
    return out[: w[0] * h[0] * 3].reshape(h[0], w[0], 3)


def xorshift(seed, n):
    out = np.zeros(n, np.uint32)
    lib().rh_xorshift(seed, n, _p(out, _U))
    return out


def xorshift_reals(seed, skip, n):
    out = np.zeros(n)
    lib().rh_xorshift_reals(seed, skip, n, _p(out, _D))
    return out


def on_hemisphere(normals, r):
    normals = np.ascontiguousarray(normals, np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(r, np.float64).reshape(-1, 2)
    out = np.zeros_like(normals)
    lib().rh_on_hemisphere(_p(normals, _D), _p(r, _D), normals.shape[0], _p(out, _D))
    return out


def bsdf_sample(mat, din, nrm, r):
    din = np.ascontiguousarray(din, np.float64).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(r, np.float64).reshape(-1, 2)
    out = np.zeros_like(din)
    pdf = np.zeros(din.shape[0])
    m = np.ascontiguousarray(mat)
    lib().rh_bsdf_sample(m.ctypes.data, _p(din, _D), _p(nrm, _D), _p(r, _D), din.shape[0], _p(out, _D), _p(pdf, _D))
    return out, pdf


def camera_rays(cam, pxy):
    pxy = np.ascontiguousarray(pxy, np.float64).reshape(-1, 2)
    e = np.array(cam.eye, np.float64)
    d = np.array(cam.dir, np.float64)
    u = np.array(cam.up, np.float64)
    org = np.zeros((pxy.shape[0], 3))
    dd = np.zeros((pxy.shape[0], 3))
    lib().rh_camera_rays(_p(e, _D), _p(d, _D), _p(u, _D), cam.fov, cam.width, cam.height, _p(pxy, _D), pxy.shape[0],
                         _p(org, _D), _p(dd, _D))
    return org, dd


def hash_points(hash_size, scale, bbmin, bbmax, pts):
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    bmn = np.ascontiguousarray(bbmin, np.float64)
    bmx = np.ascontiguousarray(bbmax, np.float64)
    out = np.zeros(pts.shape[0], np.uint32)
    lib().rh_hash_points(int(hash_size), float(scale), _p(bmn, _D), _p(bmx, _D), _p(pts, _F), pts.shape[0], _p(out, _U))
    return out


def hash_add_boxes(hash_size, scale, bbmin, bbmax, boxmin, boxmax, cap=1 << 22):
    bmn = np.ascontiguousarray(bbmin, np.float64)
    bmx = np.ascontiguousarray(bbmax, np.float64)
    lo = np.ascontiguousarray(boxmin, np.float64).reshape(-1, 3)
    hi = np.ascontiguousarray(boxmax, np.float64).reshape(-1, 3)
    start = np.zeros(hash_size + 1, np.int32)
    items = np.zeros(cap, np.int32)
    k = lib().rh_hash_add_boxes(int(hash_size), float(scale), _p(bmn, _D), _p(bmx, _D), _p(lo, _D), _p(hi, _D),
                                lo.shape[0], _p(start, _I), _p(items, _I), cap)
    if k < 0:
        raise RuntimeError("cap too small")
    return start, items[:k]


def knn(photon_pos, queries, num_target_photons, target_radius, cap=512):
    pp = np.ascontiguousarray(photon_pos, np.float32).reshape(-1, 3)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
    idx = np.full((q.shape[0], cap), -1, np.int32)
    cnt = np.zeros(q.shape[0], np.int32)
    r = lib().rh_knn(_p(pp, _F), pp.shape[0], _p(q, _F), q.shape[0], int(num_target_photons), float(target_radius),
                     _p(idx, _I), _p(cnt, _I), cap)
    if r != 0:
        raise RuntimeError("cap too small")
    return idx, cnt


def kdtree_knn(points, queries, type_, epsilon, k, cap=64):
    """KdTree<Photon>::knnSearch with KnnQuery(type, epsilon, k): ids farthest first."""
    p = np.ascontiguousarray(points, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    idx = np.full((len(q), cap), -1, np.int32)
    cnt = np.zeros(len(q), np.int32)
    r = lib().rh_kdtree_knn(_p(p, _F), len(p), _p(q, _F), len(q), int(type_), float(epsilon), int(k), _p(idx, _I),
                            _p(cnt, _I), cap)
    if r != 0:
        raise RuntimeError("cap too small")
    return idx, cnt


def dipole_rd(mat, d2):
    d2 = np.ascontiguousarray(d2, np.float64)
    out = np.zeros((d2.size, 3))
    m = np.ascontiguousarray(mat)
    lib().rh_dipole_rd(m.ctypes.data, _p(d2, _D), d2.size, _p(out, _D))
    return out


def dipole_fdr(mat):
    m = np.ascontiguousarray(mat)
    return lib().rh_dipole_fdr(m.ctypes.data)


def dipole_irradiance(mat, ipts10, max_error, queries):
    ipts = np.ascontiguousarray(ipts10, np.float64).reshape(-1, 10)
    q = np.ascontiguousarray(queries, np.float64).reshape(-1, 3)
    out = np.zeros_like(q)
    m = np.ascontiguousarray(mat)
    lib().rh_dipole_irradiance(m.ctypes.data, _p(ipts, _D), ipts.shape[0], float(max_error), _p(q, _D), q.shape[0],
                               _p(out, _D))
    return out


def irradiance_pm(photons8, points6, num_photons, gather_photons, gather_radius):
    ph = np.ascontiguousarray(photons8, np.float64).reshape(-1, 8)
    pt = np.ascontiguousarray(points6, np.float64).reshape(-1, 6)
    out = np.zeros((pt.shape[0], 3))
    lib().rh_irradiance_pm(_p(ph, _D), ph.shape[0], _p(pt, _D), pt.shape[0], int(num_photons), int(gather_photons),
                           float(gather_radius), _p(out, _D))
    return out


def poisson_disk(tris9, min_dist, cap=1 << 22):
    t = np.ascontiguousarray(tris9, np.float32).reshape(-1, 9)
    pts = np.zeros((cap, 3))
    nrm = np.zeros((cap, 3))
    n = lib().rh_poisson_disk(_p(t, _F), t.shape[0], float(min_dist), _p(pts, _D), _p(nrm, _D), cap)
    return pts[:n], nrm[:n]


def mesh_place(path, fit=None, scale_all=1.0, plane=None, move=(0.0, 0.0, 0.0), vcap=1 << 22, fcap=1 << 22):
    """Trimesh::load + fitToBBox / scale / putOnPlane / translate in the
    reference. fit: (bmin, bmax) or None; plane: (distance, normal) or None.
    Returns (double vertices [n, 3], int faces [m, 3])."""
    L = lib()
    bmin = np.ascontiguousarray(fit[0] if fit else (0, 0, 0), np.float64)
    bmax = np.ascontiguousarray(fit[1] if fit else (0, 0, 0), np.float64)
    pn = np.ascontiguousarray(plane[1] if plane else (0, 1, 0), np.float64)
    mv = np.ascontiguousarray(move, np.float64)
    verts = np.zeros((vcap, 3), np.float64)
    faces = np.zeros((fcap, 3), np.int32)
    nv = np.zeros(1, np.int32)
    nf = L.rh_mesh_place(str(path).encode(), 1 if fit else 0, _p(bmin, _D), _p(bmax, _D), float(scale_all),
                         1 if plane else 0, float(plane[0]) if plane else 0.0, _p(pn, _D), _p(mv, _D),
                         _p(verts, _D), vcap, _p(faces, _I), fcap, _p(nv, _I))
    if nf < 0:
        raise RuntimeError("mesh_place: buffers too small")
    return verts[: nv[0]].copy(), faces[:nf].copy()
