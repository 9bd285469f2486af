"""Generates the golden fixtures in tests/golden/ from the UNMODIFIED reference.

Run in a container that has the reference sources (it builds oracle/_ref with
oracle/Makefile first):

    python tests/golden/make_golden.py [name ...]

Every fixture stores its exact float inputs next to the reference outputs, so
the tests never regenerate inputs (numpy's transcendental functions are not
bit-identical across machines). OMP_NUM_THREADS is pinned to 8 because the
reference seeds one XorShift stream per OpenMP thread.
"""
from __future__ import annotations

import os
import pathlib
import sys

os.environ.setdefault("OMP_NUM_THREADS", "8")

import numpy as np  # noqa: E402

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tatsy-pppm_gb300"))
import refharness as rh  # noqa: E402
import scenes as S  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent


def save(name, **arrays):
    np.savez_compressed(OUT / f"{name}.npz", **arrays)
    print(f"wrote {name}.npz", {k: v.shape for k, v in arrays.items()})


def scene_arrays(sc):
    return dict(tris=sc.tris, mat_id=sc.mat_id, mats=sc.mats.view(np.uint8).reshape(len(sc.mats), -1),
                env=sc.env if sc.env is not None else np.zeros((0, 0, 3), np.float32))


def special_rays(tris, rng, n):
    """Rays aimed at vertices, edge midpoints and grazing the triangle planes."""
    t = tris.reshape(-1, 3, 3).astype(np.float64)
    pick = rng.integers(0, t.shape[0], n)
    kind = rng.integers(0, 4, n)
    tgt = np.where(kind[:, None] == 0, t[pick, 0], np.where(kind[:, None] == 1, 0.5 * (t[pick, 0] + t[pick, 1]),
                                                            t[pick].mean(1)))
    org = tgt + rng.normal(size=(n, 3)) * 15.0
    # grazing: start in the triangle's plane
    e1 = t[pick, 1] - t[pick, 0]
    e2 = t[pick, 2] - t[pick, 0]
    graze = kind == 3
    org[graze] = tgt[graze] - 5.0 * (e1[graze] + 0.3 * e2[graze])
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([org, d], 1).astype(np.float32)


def random_rays(bbmin, bbmax, rng, n):
    c = 0.5 * (bbmin + bbmax)
    ext = (bbmax - bbmin)
    org = c + (rng.uniform(-1, 1, (n, 3)) * ext * 0.9)
    tgt = c + (rng.uniform(-0.5, 0.5, (n, 3)) * ext)
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([org, d], 1).astype(np.float32)
    # axis-aligned directions (zero components -> idir = 1e20)
    k = n // 10
    ax = rng.integers(0, 3, k)
    dd = np.zeros((k, 3), np.float32)
    dd[np.arange(k), ax] = rng.choice([-1.0, 1.0], k)
    rays[:k, 3:] = dd
    # renormalise in float so the reference's unit-direction assertion holds
    dn = rays[:, 3:].astype(np.float64)
    rays[:, 3:] = (dn / np.linalg.norm(dn, axis=1, keepdims=True)).astype(np.float32)
    return rays


def gen_intersect():
    sc = S.small_test_scene(seed=3, subdiv=3)
    rng = np.random.default_rng(11)
    bmn, bmx = sc.bbox()
    rays = np.concatenate([random_rays(bmn, bmx, rng, 16000), special_rays(sc.tris, rng, 8000)], 0)
    R = rh.RefScene(sc)
    tri, t, pos, nrm = R.intersect(rays)
    # a second, larger mesh (subdivision 5 sphere) for deeper trees
    sc2 = S.config1a(seed=1, width=16, height=16, subdiv=5)
    R2 = rh.RefScene(sc2)
    bmn2, bmx2 = sc2.bbox()
    rays2 = np.concatenate([random_rays(bmn2, bmx2, rng, 12000), special_rays(sc2.tris, rng, 6000)], 0)
    tri2, t2, pos2, nrm2 = R2.intersect(rays2)
    # degenerate scenes: empty, 1..3 triangles (root is a leaf), 4 (one inner node)
    small = {}
    for k in (1, 2, 3, 4, 5):
        tt = sc.tris[:k].copy()
        sk = S.Scene("tiny", tt, np.zeros(k, np.int32), sc.mats[:1], None, sc.camera)
        rk = rh.RefScene(sk)
        rr = special_rays(tt, rng, 400)
        a, b, _, _ = rk.intersect(rr)
        small[f"tiny{k}_tris"] = tt
        small[f"tiny{k}_rays"] = rr
        small[f"tiny{k}_tri"] = a
        small[f"tiny{k}_t"] = b
    save("intersect", tris=sc.tris, rays=rays, tri=tri, t=t, pos=pos, nrm=nrm, tris2=sc2.tris, rays2=rays2, tri2=tri2,
         t2=t2, pos2=pos2, nrm2=nrm2, **small)


def gen_hash():
    rng = np.random.default_rng(5)
    out = {}
    for k, (size, scale) in enumerate([(65536, 0.5), (1000003, 1.0 / 0.37), (12345, 3.0), (256 * 256, 1.0 / 1.6)]):
        bbmin = rng.uniform(-30, -10, 3)
        bbmax = rng.uniform(10, 30, 3)
        pts = rng.uniform(bbmin - 2.0, bbmax, (20000, 3)).astype(np.float32)  # some below bbmin: |(int)x| folding
        # points exactly on cell boundaries
        pts[:2000] = (bbmin + np.round(rng.uniform(0, 20, (2000, 3))) / scale).astype(np.float32)
        h = rh.hash_points(size, scale, bbmin, bbmax, pts)
        out[f"pts{k}"] = pts
        out[f"bbmin{k}"] = bbmin
        out[f"bbmax{k}"] = bbmax
        out[f"size{k}"] = np.array(size)
        out[f"scale{k}"] = np.array(scale)
        out[f"hash{k}"] = h
    save("hash", **out)


def gen_hash_boxes():
    """HashGrid<int>::add over boxes (hash_grid_detail.h:34-52): bucket
    contents in insertion order, from the reference. Boxes of render-point
    size, boxes reaching below bbmin (|(int)x| folding, empty axes), single
    cells and a table small enough that one item's cells share buckets."""
    rng = np.random.default_rng(9)
    out = {}
    for k, (size, scale, n, half) in enumerate([(4096, 0.5, 3000, 1.5), (65536, 1.0 / 0.37, 5000, 0.4),
                                                  (97, 2.0, 400, 1.2), (256 * 256, 1.0 / 1.6, 2000, 0.0)]):
        bbmin = rng.uniform(-30, -10, 3)
        bbmax = rng.uniform(10, 30, 3)
        c = rng.uniform(bbmin - 3.0, bbmax, (n, 3))
        h = rng.uniform(0, half, (n, 3)) if half > 0 else np.zeros((n, 3))
        lo, hi = c - h, c + h
        start, items = rh.hash_add_boxes(size, scale, bbmin, bbmax, lo, hi)
        out.update({f"bbmin{k}": bbmin, f"size{k}": np.array(size), f"scale{k}": np.array(scale), f"lo{k}": lo,
                    f"hi{k}": hi, f"start{k}": start, f"items{k}": items})
    save("hash_boxes", **out)


def gen_rng():
    out = {}
    for s in (0, 1, 7, 123456789):
        out[f"u32_{s}"] = rh.xorshift(s, 1000)
        out[f"real_{s}"] = rh.xorshift_reals(s, 0, 1000)
    save("xorshift", **out)


def gen_env():
    env = S.sky_env(256, 128, 9, sun_peak=500.0, sun_deg=4.0)
    path = OUT / "_tmp_env.hdr"
    rh.write_hdr(path, env)
    data = np.frombuffer(path.read_bytes(), np.uint8).copy()
    decoded = rh.load_hdr(path)
    gnd = S.ground(-5.0, 20.0)
    sc = S._assemble("env", [(gnd, 0)], [S.material(S.LAMBERTIAN, (0.5, 0.5, 0.5))], env, S.look_camera((0, 5, -30), (0, 0, 0), 0.8, 8, 8))
    R = rh.RefScene(sc, env_path=str(path))
    pdf, cdf = R.env_tables()
    rng = np.random.default_rng(3)
    d = rng.normal(size=(5000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    look = R.env_lookup(d)
    # emission on explicit tapes (Envmap::samplePhoton + onHemisphere)
    tapes = rng.uniform(0, 1, (5000, 5))
    tapes = (np.floor(tapes * 2.0**32) / 2.0**32)  # values a XorShift tape can hold
    epos, edir, eflux = R.emit(tapes, 100000)
    path.unlink()
    save("env", hdr_bytes=data, decoded=decoded, pdf=pdf, cdf=cdf, dirs=d, lookup=look, tapes=tapes, emit_pos=epos,
         emit_dir=edir, emit_flux=eflux)


GENERATORS = {"intersect": gen_intersect, "hash": gen_hash, "xorshift": gen_rng, "env": gen_env}


def surface_photons(rng, n):
    """Photons on a ground plane and on a sphere, like stored photon maps."""
    m = n // 2
    plane = np.stack([rng.uniform(-20, 20, m), np.full(m, -5.0), rng.uniform(-20, 20, m)], 1)
    d = rng.normal(size=(n - m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    sph = d * 4.0 + np.array([2.0, -1.0, 3.0])
    pos = np.concatenate([plane, sph], 0).astype(np.float32)
    flux = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32) * 1e-3
    nrm = np.concatenate([np.tile([0.0, 1.0, 0.0], (m, 1)), d], 0).astype(np.float32)
    return pos, flux, nrm


def gen_knn():
    rng = np.random.default_rng(21)
    pos, _, _ = surface_photons(rng, 40000)
    q = np.concatenate([pos[rng.integers(0, len(pos), 3000)] + rng.normal(size=(3000, 3)).astype(np.float32) * 0.3,
                        rng.uniform(-20, 20, (1000, 3))], 0).astype(np.float32)
    out = dict(pos=pos, queries=q)
    for k, (ntp, rad) in enumerate([(128, 8.7), (128, 1.0), (3, 16.9), (128, 40.2)]):
        idx, cnt = rh.knn(pos, q, ntp, rad, cap=64)
        out[f"ntp{k}"] = np.array(ntp)
        out[f"rad{k}"] = np.array(rad)
        out[f"idx{k}"] = idx
        out[f"cnt{k}"] = cnt
    save("knn", **out)


def gen_kdtree_knn():
    """KdTree::knnSearch (kdtree_detail.h:88-132) with each KnnQuery type:
    K_NEAREST | EPSILON_BALL, K_NEAREST alone (unbounded ball) and
    EPSILON_BALL alone (every point within epsilon), on surface photons."""
    rng = np.random.default_rng(12)
    pos = surface_photons(rng, 30000)[0]
    q = (pos[rng.integers(0, len(pos), 3000)] + rng.normal(size=(3000, 3)) * 0.3).astype(np.float32)
    out = {"pos": pos, "queries": q}
    for k, (t, eps, kk) in enumerate([(3, 2.5, 12), (2, 0.0, 20), (1, 0.35, 0), (3, 0.8, 64)]):
        idx, cnt = rh.kdtree_knn(pos, q, t, eps, kk, cap=64)
        out.update({f"type{k}": np.array(t), f"eps{k}": np.array(eps), f"k{k}": np.array(kk), f"idx{k}": idx,
                    f"cnt{k}": cnt})
    save("kdtree_knn", **out)


def gen_gather():
    """radiance() at bounce 0 on a Lambertian ground plane (y = -5): rays
    straight down from y = 10 hit at float-exact points (x, -5, z), so the
    query positions of the reference and of the GPU are identical."""
    rng = np.random.default_rng(31)
    gnd = S.ground(-5.0, 30.0)
    refl = (0.6, 0.5, 0.4)
    sc = S._assemble("gnd", [(gnd, 0)], [S.material(S.LAMBERTIAN, refl)], None,
                     S.look_camera((0, 5, -30), (0, 0, 0), 0.8, 8, 8))
    R = rh.RefScene(sc)
    pos, flux, nrm = surface_photons(rng, 30000)
    # lift a third of the plane photons off the plane: exercises the disc filter
    lift = rng.random(len(pos)) < 0.15
    pos[lift, 1] += rng.uniform(-1.5, 1.5, lift.sum()).astype(np.float32)
    ph12 = np.concatenate([pos, flux, np.zeros_like(pos), nrm], 1).astype(np.float32)
    m = 2000
    xz = np.round(rng.uniform(-18, 18, (m, 2)) * 64) / 64
    rays = np.stack([xz[:, 0], np.full(m, 10.0), xz[:, 1], np.zeros(m), np.full(m, -1.0), np.zeros(m)], 1).astype(np.float32)
    out = dict(photons=ph12, rays=rays, refl=np.array(refl, np.float32))
    for k, rad in enumerate([6.5, 9.3, 17.2, 3.2]):
        out[f"rad{k}"] = np.array(rad)
        out[f"L{k}"] = R.gather(ph12, rad, 128, rays)
    # phantom photons at the origin (zero flux): queries near the origin
    ph_ph = np.concatenate([ph12, np.zeros((500, 12), np.float32)], 0)
    xz2 = np.round(rng.uniform(-3, 3, (300, 2)) * 64) / 64
    rays2 = np.stack([xz2[:, 0], np.full(300, 10.0), xz2[:, 1], np.zeros(300), np.full(300, -1.0), np.zeros(300)], 1).astype(np.float32)
    out["photons_ph"] = ph_ph
    out["rays_ph"] = rays2
    out["L_ph"] = R.gather(ph_ph, 6.5, 128, rays2)
    save("gather", **out)


def quantize_env(env):
    """The env map as the reference sees it: through its own RGBE writer and
    loader (image.cc:436-482, 296-434). Idempotent, so the quantized map
    round-trips unchanged when the harness writes it again."""
    path = OUT / "_tmp_q.hdr"
    rh.write_hdr(path, env)
    q = rh.load_hdr(path).astype(np.float32)
    path.unlink()
    return q


def gen_render():
    """Whole passes of the reference render loop (compat semantics), N = 8."""
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20000)
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    res = R.render_passes(sc.camera, sc.photons, 2, photon_cap=200000)
    a = scene_arrays(sc)
    cam = sc.camera
    save("render_small", **a, accum=res["accum"], radii=res["radii"], photons=res["photons"],
         photon_count=np.array(res["photon_count"]), eye=np.array(cam.eye), dir=np.array(cam.dir), up=np.array(cam.up),
         fov=np.array(cam.fov), wh=np.array([cam.width, cam.height]), nphotons=np.array(sc.photons),
         threads=np.array(rh.num_threads()))


def gen_render_qmc():
    """The same two passes with the QMC sampler type (Halton(200, true, i)
    per thread, ppm_probabilistic.cc:58-73)."""
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20000)
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    res = R.render_passes(sc.camera, sc.photons, 2, photon_cap=200000, qmc=True)
    save("render_qmc", accum=res["accum"], radii=res["radii"], photons=res["photons"],
         photon_count=np.array(res["photon_count"]), threads=np.array(rh.num_threads()))


def gen_dipole():
    """DipoleBSSRDF::operator() tables and SubsurfaceIntegrator::irradiance
    over injected irradiance points (the reference's own photon pass for them
    is seeded with time(NULL), so points are injected, not traced)."""
    rng = np.random.default_rng(41)
    mats = [S.material(S.REFRACTION, (0.99, 0.99, 0.99), sigma_a=(0.0021, 0.0041, 0.0071), sigmap_s=(2.19, 2.62, 3.00),
                       eta=1.5, scale=1.0, bssrdf=True),
            S.material(S.LAMBERTIAN, (0.8, 0.8, 0.8), sigma_a=(0.013, 0.070, 0.145), sigmap_s=(1.09, 1.59, 1.79),
                       eta=1.3, scale=0.7, bssrdf=True),
            S.material(S.REFRACTION, (0.9, 0.9, 0.9), sigma_a=(0.02, 0.01, 0.04), sigmap_s=(0.6, 2.9, 1.4),
                       eta=0.8, scale=2.0, bssrdf=True)]
    d2 = np.concatenate([np.linspace(0, 4, 500), rng.uniform(0, 200, 1500) ** 2 / 100]).astype(np.float32)
    out = {"d2": d2}
    for k, m in enumerate(mats):
        out[f"mat{k}"] = np.ascontiguousarray(m).view(np.uint8).copy()
        out[f"rd{k}"] = rh.dipole_rd(m, d2.astype(np.float64))
        out[f"fdr{k}"] = np.array(rh.dipole_fdr(m))
    # irradiance points on a displaced sphere, spacing ~ Poisson disc radius
    sph = S.displace_sphere(S.geodesic_sphere(24), 5.0, 0.05, 3)
    pts = sph.mean(1)
    nrm = np.cross(sph[:, 1] - sph[:, 0], sph[:, 2] - sph[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    n = len(pts)
    area = np.full(n, np.pi * 0.25 ** 2)
    irad = rng.lognormal(0.0, 1.0, (n, 3)) * np.array([1.0, 0.8, 0.6])
    ip = np.concatenate([pts, nrm, area[:, None], irad], 1).astype(np.float32).astype(np.float64)
    q = (pts[rng.integers(0, n, 3000)] + rng.normal(size=(3000, 3)) * 0.05).astype(np.float32).astype(np.float64)
    out["ipts"] = ip
    out["queries"] = q
    for k, m in enumerate(mats):
        for e, me in enumerate((0.05, 0.5)):
            out[f"irr{k}_{e}"] = rh.dipole_irradiance(m, ip, me, q)
    save("dipole", **out)


def _sss_min_dist(sc):
    """areaRadius of render(): sqrt(sum of BSSRDF Triangle::area / all
    triangles) (ppm_probabilistic.cc:35-46)."""
    t = sc.tris.reshape(-1, 3, 3).astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 1]), axis=1)
    bss = sc.mats["has_bssrdf"][sc.mat_id] != 0
    return float(np.sqrt(area[bss].sum() / len(t))), bss


def gen_poisson():
    """sampler::poissonDisk twice in a fresh process: the candidate draws come
    from a process-wide XorShift seeded 0, so the second call continues the
    first one's stream."""
    sc = S.small_sss_scene()
    d, bss = _sss_min_dist(sc)
    tris = sc.tris[bss]
    tor = tris[sc.mat_id[bss] == 1]
    sph = tris[sc.mat_id[bss] == 2]
    p1, n1 = rh.poisson_disk(tor, d)
    p2, n2 = rh.poisson_disk(sph, 0.7 * d)
    save("poisson", tor=tor, sph=sph, min_dist=np.array([d, 0.7 * d]), pts1=p1, nrm1=n1, pts2=p2, nrm2=n2)


def gen_sss_irradiance():
    """SubsurfaceIntegrator::irradianceWithPM over injected photon maps for
    three parameter sets: the reference driver's (photons 2e6, gatherPhotons
    128, gatherRadius 16: normal filter always true) and two with an active
    normal filter and other k."""
    rng = np.random.default_rng(43)
    sph = S.displace_sphere(S.geodesic_sphere(16), 5.0, 0.05, 7)
    n = 40000
    pick = rng.integers(0, len(sph), n)
    u = rng.uniform(size=(n, 2))
    flip = u.sum(1) > 1
    u[flip] = 1 - u[flip]
    t = sph[pick]
    pos = t[:, 0] + u[:, :1] * (t[:, 1] - t[:, 0]) + u[:, 1:] * (t[:, 2] - t[:, 0])
    flux = rng.lognormal(0.0, 0.7, (n, 3)) * 1e-3
    photons = np.concatenate([pos, flux, np.zeros((n, 2))], 1).astype(np.float32).astype(np.float64)
    cent = sph.mean(1)
    nrm = np.cross(sph[:, 1] - sph[:, 0], sph[:, 2] - sph[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    q = rng.integers(0, len(sph), 4000)
    points = np.concatenate([cent[q], nrm[q]], 1).astype(np.float32).astype(np.float64)
    sets = [(2_000_000, 128, 16.0), (100_000, 8, 8.0), (50_000, 5, 23.5)]
    out = dict(photons=photons, points=points, sets=np.array(sets, np.float64))
    for i, (P, gp, gr) in enumerate(sets):
        out[f"irr{i}"] = rh.irradiance_pm(photons, points, P, gp, gr)
    save("sss_irradiance", **out)


def gen_sss_render():
    """Two whole passes with subsurface scattering (compat semantics, N = 8),
    in a fresh process (the Poisson sampler's RNG is process-wide) and with
    time(NULL) fixed at 1234567 + t - 1 for pass t's subsurface photons."""
    sc = S.small_sss_scene()
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    res = R.render_passes(sc.camera, sc.photons, 2, sss_time=1234567)
    a = scene_arrays(sc)
    cam = sc.camera
    save("render_sss", **a, accum=res["accum"], radii=res["radii"], eye=np.array(cam.eye), dir=np.array(cam.dir),
         up=np.array(cam.up), fov=np.array(cam.fov), wh=np.array([cam.width, cam.height]),
         nphotons=np.array(sc.photons), threads=np.array(rh.num_threads()), sss_time=np.array(1234567))


def gen_sss_photons():
    """SubsurfaceIntegrator::buildPhotonMap alone, with time(NULL) = 7654321
    (its photon streams are XorShift(time + i)), N = 8."""
    sc = S.small_sss_scene()
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    ph = R.sss_photons(sc.photons, 7654321)
    save("sss_photons", photons=ph, nphotons=np.array(sc.photons), sss_time=np.array(7654321),
         threads=np.array(rh.num_threads()))


def gen_classic():
    """Classic PPM (ProgressivePhotonMapping) with one OpenMP thread: with
    more threads its render-point updates run under a lock in an order that
    changes from run to run. Halton tables of the samplers seeded 0..7."""
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20000)
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    img = R.classic_passes(sc.camera, sc.photons, 2)
    a = scene_arrays(sc)
    cam = sc.camera
    hal = np.stack([rh.halton(s, 64, 200) for s in range(8)])
    save("classic", **a, image=img, eye=np.array(cam.eye), dir=np.array(cam.dir), up=np.array(cam.up),
         fov=np.array(cam.fov), wh=np.array([cam.width, cam.height]), nphotons=np.array(sc.photons),
         threads=np.array(rh.num_threads()), halton=hal)


def gen_path_trace():
    """Two samples per pixel of PathTracing::render (pseudo-random sampler,
    N = 8 streams) on the small mixed-material scene."""
    sc = S.small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20000)
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    acc = R.path_trace(sc.camera, sc.photons, 2)
    a = scene_arrays(sc)
    cam = sc.camera
    save("path_trace", **a, accum=acc, eye=np.array(cam.eye), dir=np.array(cam.dir), up=np.array(cam.up),
         fov=np.array(cam.fov), wh=np.array([cam.width, cam.height]), nphotons=np.array(sc.photons),
         threads=np.array(rh.num_threads()))


def gen_path_trace_sss():
    """Two samples per pixel of PathTracing::render with subsurface
    scattering, in a fresh process (process-wide Poisson RNG), time(NULL)
    fixed at 1234567 + t - 1 for sample t's subsurface photons."""
    sc = S.small_sss_scene()
    sc.env = quantize_env(sc.env)
    R = rh.RefScene(sc)
    acc = R.path_trace(sc.camera, sc.photons, 2, sss_time=1234567)
    a = scene_arrays(sc)
    cam = sc.camera
    save("path_trace_sss", **a, accum=acc, eye=np.array(cam.eye), dir=np.array(cam.dir), up=np.array(cam.up),
         fov=np.array(cam.fov), wh=np.array([cam.width, cam.height]), nphotons=np.array(sc.photons),
         threads=np.array(rh.num_threads()), sss_time=np.array(1234567))


def gen_image():
    """The reference's output bytes (Image::tonemap / gamma(2.2, true) /
    toByte through rh_image_bytes) of fixed FP32 accumulation buffers:
    rendered-like lognormal values, zeros, saturating values, values right at
    byte boundaries and, for the gamma-only path, negatives, NaN and inf."""
    rng = np.random.default_rng(21)
    h, w, t = 40, 56, 3
    acc = (rng.lognormal(-1.0, 1.2, (h, w, 3)) * t).astype(np.float32)
    acc[:4] = 0.0
    acc[4:6] = np.float32(t * 1.5)  # above 1 after division: saturates
    # exact byte boundaries k / 255 before gamma correction: (k/255)^2.2 * t
    k = rng.integers(1, 255, (2, w, 3))
    acc[6:8] = ((k / 255.0) ** 2.2 * t).astype(np.float32)
    tone = acc.copy()
    acc[8, :8, 0] = [-1.0, -0.0, np.nan, np.inf, -np.inf, 1e-30, 3e38, 1e-45]
    ref_gamma, val_gamma = rh.image_bytes(acc.astype(np.float64), t, tonemap=False)
    ref_tone, val_tone = rh.image_bytes(tone.astype(np.float64), t, tonemap=True)
    save("image", acc_gamma=acc, bytes_gamma=ref_gamma, vals_gamma=val_gamma, acc_tonemap=tone,
         bytes_tonemap=ref_tone, vals_tonemap=val_tone, passes=np.array(t))


def ply_bytes(verts, faces, counts=None, header_extra=(), vertex_props=("x", "y", "z"), trailer=b""):
    """Binary little-endian PLY image in the layout Trimesh::loadPly reads."""
    head = ["ply", "format binary_little_endian 1.0", *header_extra, f"element vertex {len(verts)}"]
    head += [f"property float {p}" for p in vertex_props]
    head += [f"element face {len(faces)}", "property list uchar int vertex_indices", "end_header"]
    rec = np.zeros(len(faces), np.dtype([("n", "u1"), ("i", "<i4", (3,))]))
    rec["n"] = 3 if counts is None else counts
    rec["i"] = faces
    return ("\n".join(head) + "\n").encode() + np.asarray(verts, "<f4").tobytes() + rec.tobytes() + trailer


def gen_ply():
    """Trimesh::loadPly and the placement helpers (fitToBBox, scale,
    putOnPlane, translate) of the reference on synthetic PLY images, and
    digests of the reference's own assets placed as its demo driver places
    them (main/appmain.cc:38-40, 69-80)."""
    import hashlib
    import tempfile

    rng = np.random.default_rng(21)
    v0 = rng.normal(size=(60, 3)) * [3.0, 1.0, 2.0] + [1.0, -2.0, 0.5]
    v3 = rng.normal(size=(40, 3)).astype(np.float32)
    v3[:4] = [[1e-30, -0.0, 3e38], [-1e-40, 7.0, -2.5], [0.0, 1e-38, 1.0], [-3e38, 2.0, 5e-45]]
    cases = [
        # comments and obj_info lines; the bunny's placement
        (ply_bytes(v0, rng.integers(0, 60, (100, 3)), header_extra=("comment made by a test", "obj_info x")),
         ((-5.0, -5.0, -5.0), (5.0, 5.0, 5.0)), 0.8, (10.0, (0.0, 1.0, 0.0)), (5.0, 0.0, -10.0)),
        # six vertex properties declared, three floats stored (the reader ignores declarations)
        (ply_bytes(rng.normal(size=(30, 3)), rng.integers(0, 30, (20, 3)),
                   vertex_props=("x", "y", "z", "nx", "ny", "nz")),
         ((-1.0, -2.0, -3.0), (4.0, 5.0, 6.0)), 1.0, (2.5, (0.0, 0.0, 1.0)), (0.1, 0.2, 0.3)),
        # faces with count 2 (three indices read anyway), non-unit plane normal, trailing bytes
        (ply_bytes(rng.uniform(-7, 9, (25, 3)), rng.integers(0, 25, (15, 3)), counts=rng.integers(2, 4, 15),
                   trailer=b"\x00garbage"),
         None, 1.5, (-3.0, (0.0, 2.0, 0.5)), (0.0, 0.0, 0.0)),
        # decode only, extreme and signed-zero coordinates
        (ply_bytes(v3, rng.integers(0, 40, (30, 3))), None, 1.0, None, (0.0, 0.0, 0.0)),
    ]
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for i, (data, fit, sc, plane, move) in enumerate(cases):
            path = pathlib.Path(d) / f"m{i}.ply"
            path.write_bytes(data)
            rv, rf = rh.mesh_place(path, fit=fit, scale_all=sc, plane=plane, move=move)
            out[f"ply_{i}"] = np.frombuffer(data, np.uint8)
            out[f"fit_{i}"] = np.array(fit if fit else [[np.nan] * 3, [np.nan] * 3], np.float64)
            out[f"scale_{i}"] = np.array(sc)
            out[f"plane_{i}"] = np.array([plane[0], *plane[1]] if plane else [np.nan] * 4, np.float64)
            out[f"move_{i}"] = np.array(move, np.float64)
            out[f"ref_verts_{i}"] = rv
            out[f"ref_faces_{i}"] = rf
    out["cases"] = np.array(len(cases))
    # the reference's assets with the demo driver's placement: digests only
    demo = {"bunny.ply": (((-5.0, -5.0, -5.0), (5.0, 5.0, 5.0)), 0.8, (10.0, (0.0, 1.0, 0.0)), (5.0, 0.0, -10.0)),
            "rt3.ply": (((-10.0, -10.0, -10.0), (10.0, 10.0, 10.0)), 1.5, (10.0, (0.0, 1.0, 0.0)), (20.0, 0.0, -5.0))}
    names, digests = [], []
    for name, (fit, sc, plane, move) in demo.items():
        path = pathlib.Path("/root/reference/assets") / name
        if not path.exists():
            continue
        rv, rf = rh.mesh_place(path, fit=fit, scale_all=sc, plane=plane, move=move)
        h = hashlib.sha256(rv.astype("<f8").tobytes() + rf.astype("<i4").tobytes()).hexdigest()
        names.append(name)
        digests.append(f"{len(rv)} {len(rf)} {h}")
    out["asset_names"] = np.array(names)
    out["asset_digests"] = np.array(digests)
    save("ply", **out)


GENERATORS.update({"knn": gen_knn, "gather": gen_gather, "render": gen_render, "dipole": gen_dipole,
                   "sss_irradiance": gen_sss_irradiance, "path_trace": gen_path_trace, "ply": gen_ply,
                   "image": gen_image, "render_qmc": gen_render_qmc, "hash_boxes": gen_hash_boxes,
                   "kdtree_knn": gen_kdtree_knn, "sss_photons": gen_sss_photons})
# generators that need a fresh process (process-wide reference RNG state)
FRESH = {"poisson": gen_poisson, "render_sss": gen_sss_render, "classic": gen_classic,
         "path_trace_sss": gen_path_trace_sss}
# fresh processes that must run with a given OpenMP thread count
FRESH_THREADS = {"classic": "1"}


if __name__ == "__main__":
    import subprocess

    if sys.argv[1:2] == ["--fresh"]:
        FRESH[sys.argv[2]]()
        sys.exit(0)
    rh.build()
    names = sys.argv[1:] or list(GENERATORS) + list(FRESH)
    for n in names:
        if n in FRESH:
            env = dict(os.environ)
            if n in FRESH_THREADS:
                env["OMP_NUM_THREADS"] = FRESH_THREADS[n]
            subprocess.run([sys.executable, __file__, "--fresh", n], check=True, env=env)
        else:
            GENERATORS[n]()
