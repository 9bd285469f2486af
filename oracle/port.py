"""ctypes binding of the oracle port (oracle/_build/libpppm_port.so).

Test infrastructure only (tests, smoke check, bench CPU baseline).
"""
from __future__ import annotations

import ctypes
import pathlib

import numpy as np

import build_port

_lib = None
_VP = ctypes.c_void_p


class PassStats(ctypes.Structure):
    _fields_ = [("radius", ctypes.c_double), ("stored", ctypes.c_int64), ("phantoms", ctypes.c_int64),
                ("ms_photon", ctypes.c_double), ("ms_eye", ctypes.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = build_port.build()
        _lib = ctypes.CDLL(str(path))
        _lib.port_scene_create.restype = _VP
        _lib.port_scene_create.argtypes = [_VP, ctypes.c_int64, _VP, _VP, ctypes.c_int32, _VP, ctypes.c_int32,
                                           ctypes.c_int32]
        _lib.port_scene_destroy.argtypes = [_VP]
        _lib.port_scene_emission.argtypes = [_VP, ctypes.c_int32, _VP]
        _lib.port_env_tables.argtypes = [_VP, _VP, _VP]
        _lib.port_intersect.argtypes = [_VP, _VP, ctypes.c_int64, _VP, _VP]
        _lib.port_render.argtypes = [_VP, _VP, _VP, ctypes.c_int32, _VP, _VP, _VP, ctypes.c_int64, _VP, _VP]
        _lib.port_render.restype = ctypes.c_int
        _lib.port_knn.argtypes = [_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, _VP, _VP,
                                  ctypes.c_int32]
        _lib.port_gather_canonical.argtypes = [_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_double, _VP]
        _lib.port_gather_bounds.argtypes = [_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, _VP, _VP, _VP, _VP, _VP]
    return _lib


class PortScene:
    def __init__(self, scene):
        L = lib()
        self._keep = [np.ascontiguousarray(scene.tris, np.float32), np.ascontiguousarray(scene.mat_id, np.int32),
                      np.ascontiguousarray(scene.mats)]
        env = np.ascontiguousarray(scene.env, np.float32) if scene.env is not None else None
        self._keep.append(env)
        self.h = L.port_scene_create(self._keep[0].ctypes.data, self._keep[0].shape[0], self._keep[1].ctypes.data,
                                     self._keep[2].ctypes.data, self._keep[2].shape[0],
                                     env.ctypes.data if env is not None else None,
                                     env.shape[1] if env is not None else 0, env.shape[0] if env is not None else 0)
        for mid, rgb in (getattr(scene, "emission", None) or {}).items():
            e = np.ascontiguousarray(rgb, np.float32).reshape(3)
            L.port_scene_emission(self.h, int(mid), e.ctypes.data)

    def __del__(self):
        try:
            lib().port_scene_destroy(self.h)
        except Exception:
            pass

    def env_tables(self):
        pdf, cdf = np.zeros(4096), np.zeros(4096)
        lib().port_env_tables(self.h, pdf.ctypes.data, cdf.ctypes.data)
        return pdf, cdf

    def intersect(self, rays):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        tri = np.zeros(n, np.int32)
        t = np.zeros(n)
        lib().port_intersect(self.h, rays.ctypes.data, n, tri.ctypes.data, t.ctypes.data)
        return tri, t

    def render(self, cam_struct, params, passes, photon_cap=0, queries=False):
        """cam_struct / params: pppm_gb300.Camera / Params (same C layout).
        queries=True adds each pixel's gather query of the last pass
        (H*W x 12 doubles: hit point, triangle id, oriented normal, specular
        bounces before the hit, weight, flag = 1 where the pixel gathered)."""
        w, h = cam_struct.width, cam_struct.height
        accum = np.zeros((h, w, 3))
        stats = (PassStats * max(passes, 1))()
        ph = np.zeros((max(photon_cap, 1), 13))
        qr = np.zeros((h * w, 12)) if queries else None
        n = ctypes.c_int64()
        r = lib().port_render(self.h, ctypes.byref(cam_struct), ctypes.byref(params), passes, accum.ctypes.data, stats,
                              ph.ctypes.data if photon_cap else None, photon_cap, ctypes.byref(n) if photon_cap else None,
                              qr.ctypes.data if queries else None)
        if r != 0:
            raise RuntimeError(f"port_render failed with status {r}")
        out = dict(accum=accum, stats=[{k: getattr(s, k) for k, _ in PassStats._fields_} for s in stats[:passes]])
        if photon_cap:
            out["photons"] = ph[: min(n.value, photon_cap)]
            out["photon_count"] = n.value
        if queries:
            out["queries"] = qr
        return out


def knn(pos, q, ntp, rad, cap=64):
    pos = np.ascontiguousarray(pos, np.float32)
    q = np.ascontiguousarray(q, np.float32)
    idx = np.zeros((len(q), cap), np.int32)
    cnt = np.zeros(len(q), np.int32)
    lib().port_knn(pos.ctypes.data, len(pos), q.ctypes.data, len(q), int(ntp), float(rad), idx.ctypes.data,
                   cnt.ctypes.data, cap)
    return idx, cnt


def gather_canonical(ph9, q12, radius):
    ph9 = np.ascontiguousarray(ph9, np.float64)
    q12 = np.ascontiguousarray(q12, np.float64)
    out = np.zeros((len(q12), 3))
    lib().port_gather_canonical(ph9.ctypes.data, len(ph9), q12.ctypes.data, len(q12), float(radius), out.ctypes.data)
    return out


def gather_bounds(ph9, q12, radius, d2band=1e-5, nband=1e-3):
    """Float64 canonical gather with the bounds of photons a float32 gather
    may decide either way (port_gather_bounds): (lo, hi, ref, ambiguous,
    inside), the last two photon counts per query."""
    ph9 = np.ascontiguousarray(ph9, np.float64)
    q12 = np.ascontiguousarray(q12, np.float64)
    m = len(q12)
    lo, hi, ref = np.zeros((m, 3)), np.zeros((m, 3)), np.zeros((m, 3))
    amb, inside = np.zeros(m, np.int64), np.zeros(m, np.int64)
    lib().port_gather_bounds(ph9.ctypes.data, len(ph9), q12.ctypes.data, m, float(radius), float(d2band), float(nband),
                             lo.ctypes.data, hi.ctypes.data, ref.ctypes.data, amb.ctypes.data, inside.ctypes.data)
    return lo, hi, ref, amb, inside
