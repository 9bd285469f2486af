"""Python binding of the C ABI in include/pppm_c.h (libpppm_gb300.so).

Arrays may be numpy arrays (host memory) or CUDA torch tensors (device
memory); outputs are returned in the same kind of memory as the first
array argument. The library is required: nothing here falls back to a CPU
implementation, and `load()` raises when the shared object is missing.
"""
from __future__ import annotations

import ctypes
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libpppm_gb300.so"

OK = 0
E_ARG, E_CUDA, E_STATE, E_CAPACITY, E_UNDEFINED, E_TIMEOUT = -1, -2, -3, -4, -5, -6
MODE_COMPAT, MODE_CANONICAL, MODE_CLASSIC, MODE_PATH_TRACING = 0, 1, 2, 3
FLAG_COUNT_TRAVERSAL = 0x1
FLAG_LEARNED = 0x2
FLAG_LEARNED_FROZEN = 0x4
FLAG_SAMPLER_QMC = 0x8  # compat mode: the reference's QMC sampler type (permuted Halton)
KNN_EPSILON_BALL, KNN_K_NEAREST = 0x01, 0x02
NOALLOC_MAX_PHOTONS = 1 << 17  # PPPM_NOALLOC_MAX_PHOTONS
MLP_PARAMS = 16104  # PPPM_MLP_PARAMS

_lib = None


class PppmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pppm error {code}: {msg}")
        self.code = code


class Camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("dir", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov", ctypes.c_float), ("width", ctypes.c_int32), ("height", ctypes.c_int32)]


class Params(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("num_streams", ctypes.c_int32), ("photons", ctypes.c_int64),
                ("gather_photons", ctypes.c_int32), ("max_bounce_photon", ctypes.c_int32),
                ("max_bounce_eye", ctypes.c_int32), ("seed", ctypes.c_uint32), ("gather_radius", ctypes.c_double),
                ("alpha", ctypes.c_double), ("radius_scale", ctypes.c_double), ("cell_factor", ctypes.c_float),
                ("flags", ctypes.c_int32), ("sss_time", ctypes.c_uint32)]


class PassStats(ctypes.Structure):
    _fields_ = [("photons_traced", ctypes.c_int64), ("photons_stored", ctypes.c_int64),
                ("phantom_photons", ctypes.c_int64), ("photon_rays", ctypes.c_int64), ("eye_rays", ctypes.c_int64),
                ("gather_queries", ctypes.c_int64), ("radius", ctypes.c_double), ("ms_photon", ctypes.c_double),
                ("ms_grid", ctypes.c_double), ("ms_eye", ctypes.c_double), ("ms_gather", ctypes.c_double),
                ("ms_bounce", ctypes.c_double), ("kernel_launches", ctypes.c_int64), ("node_visits", ctypes.c_int64),
                ("tri_tests", ctypes.c_int64), ("photon_node_visits", ctypes.c_int64),
                ("photon_tri_tests", ctypes.c_int64), ("gather_pairs", ctypes.c_int64),
                ("gather_inside", ctypes.c_int64), ("sss_points", ctypes.c_int64), ("sss_photons", ctypes.c_int64),
                ("ms_subsurface", ctypes.c_double), ("ms_subsurface_host", ctypes.c_double),
                ("ms_train", ctypes.c_double), ("train_loss", ctypes.c_double), ("train_records", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_VP = ctypes.c_void_p


class Tune(ctypes.Structure):
    """pppm_tune: the launch-shape knobs of a render (none changes a result)."""
    _fields_ = [("cell_factor", ctypes.c_float), ("bounce_blocks_per_sm", ctypes.c_int32),
                ("eye_blocks_per_sm", ctypes.c_int32), ("refill", ctypes.c_int32), ("exact_batch", ctypes.c_int32),
                ("gather_stage", ctypes.c_int32), ("query_sub_bits", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Job(ctypes.Structure):
    _fields_ = [("tri_xyz", ctypes.c_void_p), ("ntri", ctypes.c_int64), ("mat_id", ctypes.c_void_p),
                ("mats", ctypes.c_void_p), ("nmat", ctypes.c_int32), ("env_rgb", ctypes.c_void_p),
                ("env_w", ctypes.c_int32), ("env_h", ctypes.c_int32), ("camera", Camera), ("params", Params),
                ("passes", ctypes.c_int32)]


class JobStats(ctypes.Structure):
    _fields_ = [("passes", ctypes.c_int32), ("bounce_blocks_per_sm", ctypes.c_int32),
                ("eye_blocks_per_sm", ctypes.c_int32), ("cell_factor", ctypes.c_float), ("rays", ctypes.c_int64),
                ("ms_total", ctypes.c_double), ("ms_pass_p50", ctypes.c_double), ("ms_pass_p99", ctypes.c_double),
                ("batch_wall_ms", ctypes.c_double), ("graph_passes", ctypes.c_int32),
                ("batch_graph_ms", ctypes.c_double), ("batch_graph_capture_ms", ctypes.c_double),
                ("batch_graph_instantiate_ms", ctypes.c_double), ("refill", ctypes.c_int32),
                ("exact_batch", ctypes.c_int32), ("gather_stage", ctypes.c_int32), ("query_sub_bits", ctypes.c_int32),
                ("tune_passes", ctypes.c_int32), ("tune_candidate", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

SIGNATURES = {
    "pppm_create": ([ctypes.c_int, ctypes.POINTER(_VP)], ctypes.c_int),
    "pppm_destroy": ([_VP], ctypes.c_int),
    "pppm_last_error": ([_VP], ctypes.c_char_p),
    "pppm_sync": ([_VP], ctypes.c_int),
    "pppm_stream": ([_VP], _VP),
    "pppm_scene_set": ([_VP, _VP, ctypes.c_int64, _VP, _VP, ctypes.c_int32], ctypes.c_int),
    "pppm_env_set": ([_VP, _VP, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "pppm_env_tables": ([_VP, _VP, _VP], ctypes.c_int),
    "pppm_env_importance": ([_VP, ctypes.c_double], ctypes.c_int),
    "pppm_material_emission": ([_VP, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_env_lookup": ([_VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_emit_photons": ([_VP, _VP, ctypes.c_int64, ctypes.c_int64, _VP, _VP, _VP, _VP], ctypes.c_int),
    "pppm_hdr_decode": ([_VP, ctypes.c_int64, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "pppm_ply_decode": ([_VP, ctypes.c_int64, _VP, ctypes.c_int64, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "pppm_mesh_translate": ([_VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_mesh_scale": ([_VP, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double], ctypes.c_int),
    "pppm_mesh_put_on_plane": ([_VP, ctypes.c_int64, ctypes.c_double, _VP], ctypes.c_int),
    "pppm_mesh_fit_bbox": ([_VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "pppm_intersect": ([_VP, _VP, ctypes.c_int64, _VP, _VP, _VP, _VP], ctypes.c_int),
    "pppm_hash_points": ([_VP, _VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _VP, _VP], ctypes.c_int),
    "pppm_knn": ([_VP, _VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _VP, _VP,
                  ctypes.c_int32], ctypes.c_int),
    "pppm_kdtree_knn": ([_VP, _VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                         ctypes.c_int32, _VP, _VP, ctypes.c_int32], ctypes.c_int),
    "pppm_hashgrid_build": ([_VP, _VP, _VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _VP, _VP, _VP,
                             ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_dipole_rd": ([_VP, _VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_render_graph": ([_VP, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_render_skip": ([_VP, ctypes.c_int32], ctypes.c_int),
    "pppm_render_image": ([_VP, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_image_bytes": ([_VP, _VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_png_encode": ([_VP, ctypes.c_int32, ctypes.c_int32, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_render_save": ([_VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_render_load": ([_VP, _VP, ctypes.c_int64], ctypes.c_int),
    "pppm_fast_exp_check": ([_VP, ctypes.c_uint64, ctypes.c_uint64, _VP, _VP], ctypes.c_int),
    "pppm_dipole_irradiance": ([_VP, _VP, _VP, ctypes.c_int64, ctypes.c_double, _VP, ctypes.c_int64, _VP],
                               ctypes.c_int),
    "pppm_poisson_disk": ([_VP, _VP, ctypes.c_int64, ctypes.c_double, _VP, _VP, _VP, ctypes.c_int64, _VP],
                          ctypes.c_int),
    "pppm_subsurface_photons": ([_VP, _VP, ctypes.c_int32, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_subsurface_photon_irradiance": ([_VP, _VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_double, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_halton": ([_VP, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_mlp_forward": ([_VP, _VP, _VP, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "pppm_learned_config": ([_VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, ctypes.c_int32], ctypes.c_int),
    "pppm_mlp_grad": ([_VP, _VP, _VP, ctypes.c_int64, _VP, _VP, _VP], ctypes.c_int),
    "pppm_knn_noalloc": ([_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _VP, _VP,
                          ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_gather": ([_VP, ctypes.c_int32, _VP, ctypes.c_int64, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_double,
                     ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_render_begin": ([_VP, _VP, _VP], ctypes.c_int),
    "pppm_render_pass": ([_VP, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_render_read": ([_VP, _VP], ctypes.c_int),
    "pppm_render": ([_VP, _VP, _VP, ctypes.c_int32, _VP], ctypes.c_int),
    "pppm_render_photons": ([_VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_render_queries": ([_VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "pppm_render_tune": ([_VP, ctypes.c_float, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "pppm_render_tune_ex": ([_VP, _VP], ctypes.c_int),
    "pppm_render_get_tune": ([_VP, _VP], ctypes.c_int),
    "pppm_batch_create": ([ctypes.c_int, ctypes.POINTER(_VP)], ctypes.c_int),
    "pppm_batch_destroy": ([_VP], ctypes.c_int),
    "pppm_batch_last_error": ([_VP], ctypes.c_char_p),
    "pppm_batch_submit": ([_VP, _VP, _VP], ctypes.c_int),
    "pppm_batch_run": ([_VP, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "pppm_batch_config": ([_VP, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "pppm_batch_result": ([_VP, ctypes.c_int32, _VP, _VP], ctypes.c_int),
}


def header_symbols():
    """Function names declared in include/pppm_c.h."""
    import re

    text = (HERE.parent / "include" / "pppm_c.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void\*|const char\*)\s+(pppm_\w+)\s*\(", text, re.M)))


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with tatsy-pppm_gb300/build.py")
        _lib = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(_lib, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = res
    return _lib


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _ptr(a):
    if a is None:
        return None
    if _is_torch(a):
        assert a.is_contiguous()
        return a.data_ptr()
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data


def _empty_like_kind(ref, shape, dtype):
    if _is_torch(ref):
        import torch

        tmap = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.uint32: torch.int32,
                np.int64: torch.int64}
        return torch.empty(shape, dtype=tmap[dtype], device=ref.device)
    return np.empty(shape, dtype)


class Context:
    """One pppm context (one CUDA stream, device memory owned by the context)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _VP()
        r = self.lib.pppm_create(device, ctypes.byref(h))
        if r != OK:
            raise PppmError(r, "pppm_create failed (no CUDA device?)")
        self.h = h
        self.scene = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.pppm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, r):
        if r != OK:
            raise PppmError(r, self.lib.pppm_last_error(self.h).decode())

    def sync(self):
        self._check(self.lib.pppm_sync(self.h))

    def stream_ptr(self):
        return self.lib.pppm_stream(self.h)

    # -------------------------------------------------------------- scene
    def set_scene(self, scene):
        tris = np.ascontiguousarray(scene.tris, np.float32)
        mid = np.ascontiguousarray(scene.mat_id, np.int32)
        mats = np.ascontiguousarray(scene.mats)
        self._check(self.lib.pppm_scene_set(self.h, tris.ctypes.data, tris.shape[0], mid.ctypes.data, mats.ctypes.data,
                                            mats.shape[0]))
        # a scene without a map replaces the previous scene's map by none
        self.set_env(scene.env)
        for mid, rgb in (getattr(scene, "emission", None) or {}).items():
            self.material_emission(mid, rgb)
        self.scene = scene

    def material_emission(self, mat_id, rgb):
        """pppm_material_emission: material mat_id emits rgb from its front side."""
        e = np.ascontiguousarray(rgb, np.float32).reshape(3)
        self._check(self.lib.pppm_material_emission(self.h, int(mat_id), e.ctypes.data))

    def set_env(self, rgb):
        """pppm_env_set: the equirect map (H x W x 3), or None for no map."""
        if rgb is None:
            self._check(self.lib.pppm_env_set(self.h, None, 0, 0))
            return
        rgb = np.ascontiguousarray(rgb, np.float32)
        self._check(self.lib.pppm_env_set(self.h, rgb.ctypes.data, rgb.shape[1], rgb.shape[0]))

    def env_tables(self):
        pdf = np.zeros(4096)
        cdf = np.zeros(4096)
        self._check(self.lib.pppm_env_tables(self.h, pdf.ctypes.data, cdf.ctypes.data))
        return pdf, cdf

    def env_importance(self, exponent=2.0):
        """pppm_env_importance: environment cell weight luminance^exponent (2: the reference)."""
        self._check(self.lib.pppm_env_importance(self.h, float(exponent)))

    def env_lookup(self, dirs):
        n = int(dirs.shape[0])
        out = _empty_like_kind(dirs, (n, 3), np.float32)
        self._check(self.lib.pppm_env_lookup(self.h, _ptr(dirs), n, _ptr(out)))
        return out

    def emit_photons(self, tapes, num_photons):
        n = int(tapes.shape[0])
        pos = _empty_like_kind(tapes, (n, 3), np.float32)
        d = _empty_like_kind(tapes, (n, 3), np.float32)
        flux = _empty_like_kind(tapes, (n, 3), np.float32)
        ok = _empty_like_kind(tapes, (n,), np.int32)
        self._check(self.lib.pppm_emit_photons(self.h, _ptr(tapes), n, int(num_photons), _ptr(pos), _ptr(d), _ptr(flux),
                                               _ptr(ok)))
        return pos, d, flux, ok

    # -------------------------------------------------------------- stages
    def intersect(self, rays, with_hit=True):
        n = int(rays.shape[0])
        tri = _empty_like_kind(rays, (n,), np.int32)
        t = _empty_like_kind(rays, (n,), np.float64)
        pos = _empty_like_kind(rays, (n, 3), np.float32) if with_hit else None
        nrm = _empty_like_kind(rays, (n, 3), np.float32) if with_hit else None
        self._check(self.lib.pppm_intersect(self.h, _ptr(rays), n, _ptr(tri), _ptr(t), _ptr(pos), _ptr(nrm)))
        return tri, t, pos, nrm

    def hash_points(self, pts, hash_size, scale, bbmin):
        n = int(pts.shape[0])
        out = _empty_like_kind(pts, (n,), np.uint32)
        bmin = np.ascontiguousarray(bbmin, np.float64)
        self._check(self.lib.pppm_hash_points(self.h, _ptr(pts), n, int(hash_size), float(scale), bmin.ctypes.data,
                                              _ptr(out)))
        return out

    def kdtree_knn(self, points, queries, type_, epsilon, k, cap=64):
        """pppm_kdtree_knn: KdTree::knnSearch with KnnQuery(type, epsilon, k)."""
        n, m = int(points.shape[0]), int(queries.shape[0])
        idx = _empty_like_kind(queries, (m, cap), np.int32)
        cnt = _empty_like_kind(queries, (m,), np.int32)
        self._check(self.lib.pppm_kdtree_knn(self.h, _ptr(points), n, _ptr(queries), m, int(type_), float(epsilon),
                                             int(k), _ptr(idx), _ptr(cnt), cap))
        return idx, cnt

    def hashgrid_build(self, boxmin, boxmax, hash_size, scale, bbmin):
        """pppm_hashgrid_build (HashGrid::init + add over boxes): (start, items)
        CSR bucket contents in the reference's insertion order."""
        lo = np.ascontiguousarray(boxmin, np.float64).reshape(-1, 3)
        hi = np.ascontiguousarray(boxmax, np.float64).reshape(-1, 3)
        bm = np.ascontiguousarray(bbmin, np.float64).reshape(3)
        n = ctypes.c_int64()
        self._check(self.lib.pppm_hashgrid_build(self.h, lo.ctypes.data, hi.ctypes.data, len(lo), int(hash_size),
                                                 float(scale), bm.ctypes.data, None, None, 0, ctypes.byref(n)))
        start = np.zeros(int(hash_size) + 1, np.uint32)
        items = np.zeros(max(n.value, 1), np.int32)
        self._check(self.lib.pppm_hashgrid_build(self.h, lo.ctypes.data, hi.ctypes.data, len(lo), int(hash_size),
                                                 float(scale), bm.ctypes.data, start.ctypes.data, items.ctypes.data,
                                                 n.value, ctypes.byref(n)))
        return start, items[: n.value]

    def knn(self, photon_pos, queries, num_target_photons, target_radius, cap=64):
        n, m = int(photon_pos.shape[0]), int(queries.shape[0])
        idx = _empty_like_kind(queries, (m, cap), np.int32)
        cnt = _empty_like_kind(queries, (m,), np.int32)
        self._check(self.lib.pppm_knn(self.h, _ptr(photon_pos), n, _ptr(queries), m, int(num_target_photons),
                                      float(target_radius), _ptr(idx), _ptr(cnt), cap))
        return idx, cnt

    def gather(self, mode, photons8, queries12, radius, gather_photons=128, phantoms=0):
        n, m = int(photons8.shape[0]), int(queries12.shape[0])
        out = _empty_like_kind(queries12, (m, 3), np.float32)
        self._check(self.lib.pppm_gather(self.h, int(mode), _ptr(photons8), n, int(phantoms), _ptr(queries12), m,
                                         float(radius), int(gather_photons), _ptr(out)))
        return out

    def poisson_disk(self, tri_xyz, min_dist, rng_state=None):
        """pppm_poisson_disk (sampler::poissonDisk) on a triangle soup. rng_state:
        4 uint32 XorShift words (default: XorShift(0), the reference's static
        sampler RNG at program start). Returns (points, normals, next state)."""
        tri = np.ascontiguousarray(tri_xyz, np.float32).reshape(-1, 9)
        st = np.ascontiguousarray(xorshift_state(0) if rng_state is None else rng_state, np.uint32).copy()
        # at most one point per candidate: ceil(4 A / d^2) per triangle (sampler.cc:44)
        t64 = tri.astype(np.float64).reshape(-1, 3, 3)
        area = 0.5 * np.linalg.norm(np.cross(t64[:, 1] - t64[:, 0], t64[:, 2] - t64[:, 1]), axis=1)
        cap = int(np.ceil(4.0 * area / (min_dist * min_dist)).sum()) + tri.shape[0] + 16
        pts = np.zeros((cap, 3), np.float32)
        nrm = np.zeros((cap, 3), np.float32)
        n = ctypes.c_int64()
        self._check(self.lib.pppm_poisson_disk(self.h, tri.ctypes.data, tri.shape[0], float(min_dist), st.ctypes.data,
                                               pts.ctypes.data, nrm.ctypes.data, cap, ctypes.byref(n)))
        assert n.value <= cap
        return pts[: n.value], nrm[: n.value], st

    def halton(self, seed, count, n=200):
        out = np.zeros((count, n))
        self._check(self.lib.pppm_halton(self.h, int(seed), int(count), int(n), out.ctypes.data))
        return out

    def mlp_forward(self, params, pos, nrm, bbox):
        """pppm_mlp_forward: the proposal network's 40 raw outputs per row."""
        prm = np.ascontiguousarray(params, np.float32).reshape(-1)
        assert prm.size == MLP_PARAMS
        p = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        n = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
        bb = np.ascontiguousarray(bbox, np.float64).reshape(6)
        out = np.zeros((p.shape[0], 40), np.float32)
        self._check(self.lib.pppm_mlp_forward(self.h, prm.ctypes.data, p.ctypes.data, n.ctypes.data, p.shape[0],
                                              bb.ctypes.data, out.ctypes.data))
        return out

    def learned_config(self, retrain_every=0, steps=0, batch=0, lr=0.0, floor_bsdf=0.0, max_log_kappa=0.0,
                       guide_bounces=-1):
        """pppm_learned_config: settings of the learned proposal (0 / -1 keep the default)."""
        self._check(self.lib.pppm_learned_config(self.h, int(retrain_every), int(steps), int(batch), float(lr),
                                                 float(floor_bsdf), float(max_log_kappa), int(guide_bounces)))

    def mlp_grad(self, params, records10, bbox):
        """pppm_mlp_grad: (loss, gradient) of the proposal's training loss."""
        prm = np.ascontiguousarray(params, np.float32).reshape(-1)
        assert prm.size == MLP_PARAMS
        rec = np.ascontiguousarray(records10, np.float32).reshape(-1, 10)
        bb = np.ascontiguousarray(bbox, np.float64).reshape(6)
        grad = np.zeros(MLP_PARAMS, np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.pppm_mlp_grad(self.h, prm.ctypes.data, rec.ctypes.data, rec.shape[0], bb.ctypes.data,
                                           grad.ctypes.data, ctypes.byref(loss)))
        return loss.value, grad

    def subsurface_photons(self, params, t=1):
        """pppm_subsurface_photons: the subsurface photon map (n x 8 floats)."""
        n = ctypes.c_int64()
        self._check(self.lib.pppm_subsurface_photons(self.h, ctypes.byref(params), int(t), None, 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), 8), np.float32)
        self._check(self.lib.pppm_subsurface_photons(self.h, ctypes.byref(params), int(t), out.ctypes.data, n.value,
                                                     ctypes.byref(n)))
        return out[: n.value]

    def subsurface_photon_irradiance(self, photons8, points6, num_photons, gather_radius, gather_photons):
        ph = np.ascontiguousarray(photons8, np.float32).reshape(-1, 8)
        pt = np.ascontiguousarray(points6, np.float32).reshape(-1, 6)
        out = np.zeros((pt.shape[0], 3), np.float32)
        self._check(self.lib.pppm_subsurface_photon_irradiance(self.h, ph.ctypes.data, ph.shape[0], pt.ctypes.data,
                                                               pt.shape[0], int(num_photons), float(gather_radius),
                                                               int(gather_photons), out.ctypes.data))
        return out

    def dipole_rd(self, mat, d2):
        d2 = np.ascontiguousarray(d2, np.float32)
        m = np.ascontiguousarray(mat)
        out = np.zeros((d2.size, 3), np.float32)
        self._check(self.lib.pppm_dipole_rd(self.h, m.ctypes.data, d2.ctypes.data, d2.size, out.ctypes.data))
        return out

    def fast_exp_check(self, begin=0, end=1 << 32):
        cov, dif = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self.lib.pppm_fast_exp_check(self.h, ctypes.c_uint64(begin), ctypes.c_uint64(end),
                                                 ctypes.byref(cov), ctypes.byref(dif)))
        return cov.value, dif.value

    def dipole_irradiance(self, mat, ipts10, max_error, queries):
        ip = np.ascontiguousarray(ipts10, np.float32).reshape(-1, 10)
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
        m = np.ascontiguousarray(mat)
        out = np.zeros((len(q), 3), np.float32)
        self._check(self.lib.pppm_dipole_irradiance(self.h, m.ctypes.data, ip.ctypes.data, len(ip), float(max_error),
                                                    q.ctypes.data, len(q), out.ctypes.data))
        return out

    # -------------------------------------------------------------- render
    @staticmethod
    def make_camera(cam):
        c = Camera()
        c.eye[:] = cam.eye
        c.dir[:] = cam.dir
        c.up[:] = cam.up
        c.fov = cam.fov
        c.width, c.height = cam.width, cam.height
        return c

    @staticmethod
    def make_params(mode=MODE_COMPAT, photons=200_000, num_streams=8, gather_photons=128, gather_radius=16.0,
                    alpha=0.7, radius_scale=0.1, max_bounce_photon=64, max_bounce_eye=64, seed=1, cell_factor=1.0,
                    flags=0, sss_time=0):
        p = Params()
        p.mode = mode
        p.num_streams = num_streams
        p.photons = photons
        p.gather_photons = gather_photons
        p.max_bounce_photon = max_bounce_photon
        p.max_bounce_eye = max_bounce_eye
        p.seed = seed
        p.gather_radius = gather_radius
        p.alpha = alpha
        p.radius_scale = radius_scale
        p.cell_factor = cell_factor
        p.flags = flags
        p.sss_time = sss_time
        return p

    def render_begin(self, cam, params):
        self._cam = self.make_camera(cam) if not isinstance(cam, Camera) else cam
        self._par = params
        self._check(self.lib.pppm_render_begin(self.h, ctypes.byref(self._cam), ctypes.byref(params)))

    def render_pass(self, t):
        st = PassStats()
        self._check(self.lib.pppm_render_pass(self.h, int(t), ctypes.byref(st)))
        return st

    def render_image(self, tonemap=False):
        """pppm_render_image: the reference's output bytes of the current pass (H x W x 3 uint8)."""
        out = np.zeros((self._cam.height, self._cam.width, 3), np.uint8)
        self._check(self.lib.pppm_render_image(self.h, 1 if tonemap else 0, out.ctypes.data))
        return out

    def image_bytes(self, accum, passes, tonemap=False):
        """pppm_image_bytes: the reference's output bytes of an explicit H x W x 3 accumulator."""
        acc = np.ascontiguousarray(accum, np.float32)
        h, w = acc.shape[:2]
        out = np.zeros((h, w, 3), np.uint8)
        self._check(self.lib.pppm_image_bytes(self.h, acc.ctypes.data, w, h, int(passes), 1 if tonemap else 0,
                                              out.ctypes.data))
        return out

    def render_save(self):
        """pppm_render_save: the checkpoint as bytes."""
        n = ctypes.c_int64()
        self._check(self.lib.pppm_render_save(self.h, None, 0, ctypes.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        self._check(self.lib.pppm_render_save(self.h, buf.ctypes.data, n.value, ctypes.byref(n)))
        return buf.tobytes()

    def render_load(self, blob):
        """pppm_render_load: resume a render from render_save's bytes."""
        b = np.frombuffer(blob, np.uint8)
        self._check(self.lib.pppm_render_load(self.h, b.ctypes.data, b.size))
        # the checkpoint header: magic (8 bytes), version, header size, camera
        self._cam = Camera.from_buffer_copy(bytes(blob[16:16 + ctypes.sizeof(Camera)]))

    def render_tune(self, **knobs):
        """pppm_render_tune_ex: set launch-shape knobs (Tune field names) from the next pass on."""
        t = Tune(0.0, -1, -1, -1, -1, -1, -1)
        for k, v in knobs.items():
            if k not in dict(Tune._fields_):
                raise TypeError(f"unknown knob {k}")
            setattr(t, k, v)
        self._check(self.lib.pppm_render_tune_ex(self.h, ctypes.byref(t)))

    def get_tune(self):
        """pppm_render_get_tune: the knobs of the next pass, as a dict."""
        t = Tune()
        self._check(self.lib.pppm_render_get_tune(self.h, ctypes.byref(t)))
        return t.as_dict()

    def render_skip(self, count):
        """pppm_render_skip: advance the render by `count` passes without rendering them."""
        self._check(self.lib.pppm_render_skip(self.h, int(count)))

    def render_graph(self, count):
        """pppm_render_graph: the next `count` canonical passes as one CUDA graph launch."""
        st = (PassStats * int(count))()
        self._check(self.lib.pppm_render_graph(self.h, int(count), st))
        return list(st)

    def render_read(self, out=None):
        if out is None:
            out = np.zeros((self._cam.height, self._cam.width, 3), np.float32)
        self._check(self.lib.pppm_render_read(self.h, _ptr(out)))
        return out

    def render_photons(self, cap):
        out = np.zeros((cap, 8), np.float32)
        n = ctypes.c_int64()
        self._check(self.lib.pppm_render_photons(self.h, out.ctypes.data, cap, ctypes.byref(n)))
        return out[: n.value]

    def render_queries(self):
        """pppm_render_queries: the last pass's gather queries, n x 12 floats
        (position, pixel bits, oriented normal, 0, weight, 0)."""
        n = ctypes.c_int64()
        self._check(self.lib.pppm_render_queries(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), 12), np.float32)
        self._check(self.lib.pppm_render_queries(self.h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out[: n.value]


class Batch:
    """pppm_batch: many uneven render jobs on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        r = self.lib.pppm_batch_create(device, ctypes.byref(h))
        if r != OK:
            raise PppmError(r, "batch_create failed")
        self.h = h
        self._keep = []
        self._cams = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.pppm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, r):
        if r != OK:
            raise PppmError(r, self.lib.pppm_batch_last_error(self.h).decode())

    def submit(self, scene, params, passes):
        """Adds one job (a scenes.Scene with its env map and camera)."""
        tris = np.ascontiguousarray(scene.tris, np.float32)
        mid = np.ascontiguousarray(scene.mat_id, np.int32)
        mats = np.ascontiguousarray(scene.mats)
        env = np.ascontiguousarray(scene.env, np.float32)
        j = Job()
        j.tri_xyz, j.ntri, j.mat_id = tris.ctypes.data, tris.shape[0], mid.ctypes.data
        j.mats, j.nmat = mats.ctypes.data, len(mats)
        j.env_rgb, j.env_w, j.env_h = env.ctypes.data, env.shape[1], env.shape[0]
        j.camera = Context.make_camera(scene.camera)
        j.params = params
        j.passes = passes
        jid = ctypes.c_int32()
        self._check(self.lib.pppm_batch_submit(self.h, ctypes.byref(j), ctypes.byref(jid)))
        self._cams.append(j.camera)
        return jid.value

    def config(self, use_graph=True, graph_lanes=0):
        """pppm_batch_config: capture the passes after each job's first into two CUDA graphs
        (the tuning passes, then the rest)."""
        self._check(self.lib.pppm_batch_config(self.h, 1 if use_graph else 0, int(graph_lanes)))

    def run(self, autotune=True, max_concurrent=8):
        self._check(self.lib.pppm_batch_run(self.h, 1 if autotune else 0, int(max_concurrent)))

    def result(self, job_id, image=True):
        cam = self._cams[job_id]
        out = np.zeros((cam.height, cam.width, 3), np.float32) if image else None
        st = JobStats()
        self._check(self.lib.pppm_batch_result(self.h, int(job_id), out.ctypes.data if image else None,
                                               ctypes.byref(st)))
        return out, st.as_dict()


def shard_passes(total, rank, world):
    """Passes 1..total of one image dealt round robin over `world` ranks:
    rank r renders r + 1, r + 1 + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    return list(range(rank + 1, total + 1, world))


def render_shard(ctx, camera, params, total, rank, world):
    """Renders this rank's passes of a `total`-pass image (pppm_render_skip
    over the others) and returns its accumulation buffer (not divided)."""
    ctx.render_begin(camera, params)
    done = 0
    for t in shard_passes(total, rank, world):
        if t - 1 > done:
            ctx.render_skip(t - 1 - done)
        ctx.render_pass(t)
        done = t
    return ctx.render_read()


def merge_shards(accum, total, group=None):
    """The image of all `total` passes from each rank's accumulation buffer:
    one sum over the ranks (torch.distributed, when initialised), divided by
    the pass count. accum: numpy array (host)."""
    import torch

    t = torch.from_numpy(np.ascontiguousarray(accum, np.float32))
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        nccl = torch.distributed.get_backend(group) == "nccl"
        x = t.cuda() if nccl else t
        torch.distributed.all_reduce(x, op=torch.distributed.ReduceOp.SUM, group=group)
        t = x.cpu() if nccl else x
    return t.numpy() / float(total)


def png_encode(rgb8):
    """pppm_png_encode: PNG file bytes of an H x W x 3 uint8 image (host only)."""
    lib = load()
    img = np.ascontiguousarray(rgb8, np.uint8)
    h, w = img.shape[:2]
    n = ctypes.c_int64()
    r = lib.pppm_png_encode(img.ctypes.data, w, h, None, 0, ctypes.byref(n))
    if r != OK:
        raise PppmError(r, "png_encode: bad arguments")
    out = np.zeros(n.value, np.uint8)
    r = lib.pppm_png_encode(img.ctypes.data, w, h, out.ctypes.data, n.value, ctypes.byref(n))
    if r != OK:
        raise PppmError(r, "png_encode failed")
    return out.tobytes()


def knn_noalloc(photon_pos, queries, num_target_photons, target_radius, idx, cnt, stream=None):
    """pppm_knn_noalloc on CUDA torch tensors (outputs passed in, nothing is
    allocated by the library). Returns the status code."""
    lib = load()
    return lib.pppm_knn_noalloc(_ptr(photon_pos), int(photon_pos.shape[0]), _ptr(queries), int(queries.shape[0]),
                                int(num_target_photons), float(target_radius), _ptr(idx), _ptr(cnt),
                                int(idx.shape[1]), stream)


def xorshift_state(seed):
    """The four state words of the reference's XorShift(seed) (random.h:23-31)."""
    s = int(seed) & 0xFFFFFFFF
    out = []
    for i in range(1, 5):
        s = (1812433253 * (s ^ (s >> 30)) + i) & 0xFFFFFFFF
        out.append(s)
    return np.array(out, np.uint32)


def hdr_decode(data: bytes):
    lib = load()
    buf = np.frombuffer(data, np.uint8)
    w = ctypes.c_int32()
    h = ctypes.c_int32()
    r = lib.pppm_hdr_decode(buf.ctypes.data, buf.size, None, 0, ctypes.byref(w), ctypes.byref(h))
    if r != OK:
        raise PppmError(r, "bad HDR header")
    out = np.zeros((h.value, w.value, 3), np.float32)
    r = lib.pppm_hdr_decode(buf.ctypes.data, buf.size, out.ctypes.data, out.size, ctypes.byref(w), ctypes.byref(h))
    if r != OK:
        raise PppmError(r, "bad HDR data")
    return out


def ply_decode(data: bytes):
    """pppm_ply_decode (Trimesh::loadPly, trimesh.cc:139-217) on a PLY file
    image: (vertices float32 [n, 3], faces int32 [m, 3])."""
    lib = load()
    buf = np.frombuffer(data, np.uint8)
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    r = lib.pppm_ply_decode(buf.ctypes.data, buf.size, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nf))
    if r != OK:
        raise PppmError(r, "bad PLY header")
    verts = np.zeros((nv.value, 3), np.float32)
    faces = np.zeros((nf.value, 3), np.int32)
    if nv.value:
        r = lib.pppm_ply_decode(buf.ctypes.data, buf.size, verts.ctypes.data, verts.size, faces.ctypes.data,
                                faces.size, ctypes.byref(nv), ctypes.byref(nf))
        if r != OK:
            raise PppmError(r, "bad PLY data")
    return verts, faces


class Trimesh:
    """The reference's Trimesh (trimesh.h:68-166) for scene setup: double
    vertices and int faces, loaded from a binary PLY and placed with the
    reference's own arithmetic (pppm_mesh_*). triangles() gives the FP32
    triangle soup that Context.set_scene / scenes.Scene take."""

    def __init__(self, vertices=None, faces=None):
        self.vertices = np.zeros((0, 3), np.float64) if vertices is None else np.array(vertices, np.float64)
        self.faces = np.zeros((0, 3), np.int32) if faces is None else np.array(faces, np.int32)

    @classmethod
    def load(cls, path_or_bytes):
        data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
        v, f = ply_decode(bytes(data))
        return cls(v.astype(np.float64), f)

    def _call(self, fn, *args):
        self.vertices = np.ascontiguousarray(self.vertices, np.float64)
        r = getattr(load(), fn)(self.vertices.ctypes.data, self.vertices.shape[0], *args)
        if r != OK:
            raise PppmError(r, fn)
        return self

    def translate(self, move):
        m = np.ascontiguousarray(move, np.float64)
        return self._call("pppm_mesh_translate", m.ctypes.data)

    def scale(self, sx, sy=None, sz=None):
        sy = sx if sy is None else sy
        sz = sx if sz is None else sz
        return self._call("pppm_mesh_scale", float(sx), float(sy), float(sz))

    def put_on_plane(self, distance, normal):
        n = np.ascontiguousarray(normal, np.float64)
        return self._call("pppm_mesh_put_on_plane", float(distance), n.ctypes.data)

    def fit_to_bbox(self, bmin, bmax):
        lo = np.ascontiguousarray(bmin, np.float64)
        hi = np.ascontiguousarray(bmax, np.float64)
        return self._call("pppm_mesh_fit_bbox", lo.ctypes.data, hi.ctypes.data)

    def num_verts(self):
        return self.vertices.shape[0]

    def num_faces(self):
        return self.faces.shape[0]

    def triangles(self):
        """Triangle soup, 9 floats per face (Trimesh::getTriangle rounded to FP32)."""
        return self.vertices[self.faces].reshape(-1, 9).astype(np.float32)
