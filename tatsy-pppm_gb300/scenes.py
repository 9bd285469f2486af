"""Seeded synthetic scenes for the PPM-APA pass.

The reference ships its contest assets only partly (dragon.ply, torus.ply and
sunrise.hdr are missing), so every workload here is generated from one seed:
noise-displaced geodesic spheres and tori, a ground quad, an open box, and an
equirect sky with a Gaussian sun lobe. Scenes are triangle soups (9 floats per
triangle) with one material id per triangle, which is exactly what
`pppm_scene_set` and the reference's `Scene::add` (scene.h:38-50) consume.

The reference emits env-map photons from a radius-50 sphere around the origin
(envmap.cc:63,85), so every scene is centred at the origin and fits inside it.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# pppm_material (include/pppm_c.h), 56 bytes.
MATERIAL_DTYPE = np.dtype(
    [
        ("type", "<i4"),
        ("has_bssrdf", "<i4"),
        ("refl", "<f4", (3,)),
        ("phong_n", "<f4"),
        ("sigma_a", "<f4", (3,)),
        ("sigmap_s", "<f4", (3,)),
        ("eta", "<f4"),
        ("scale", "<f4"),
    ]
)
assert MATERIAL_DTYPE.itemsize == 56

LAMBERTIAN, SPECULAR, PHONG, REFRACTION, BSSRDF = 0x01, 0x02, 0x04, 0x08, 0x10
MODE_COMPAT, MODE_CANONICAL = 0, 1


def material(kind, refl, phong_n=0.0, sigma_a=(0, 0, 0), sigmap_s=(0, 0, 0), eta=1.3, scale=1.0, bssrdf=False):
    m = np.zeros((), MATERIAL_DTYPE)
    m["type"] = kind
    m["has_bssrdf"] = 1 if bssrdf else 0
    m["refl"] = refl
    m["phong_n"] = phong_n
    m["sigma_a"] = sigma_a
    m["sigmap_s"] = sigmap_s
    m["eta"] = eta
    m["scale"] = scale
    return m


@dataclasses.dataclass
class Camera:
    eye: tuple
    dir: tuple
    up: tuple
    fov: float  # used as tan(fov * 0.5), like PerspectiveCamera (perspective_camera.cc:18)
    width: int
    height: int


@dataclasses.dataclass
class Scene:
    name: str
    tris: np.ndarray  # (T, 9) float32
    mat_id: np.ndarray  # (T,) int32
    mats: np.ndarray  # (M,) MATERIAL_DTYPE
    env: np.ndarray | None  # (H, W, 3) float32, row 0 = top
    camera: Camera
    photons: int = 200_000
    passes: int = 16
    max_depth: int = 64
    alpha: float = 0.7
    radius_scale: float = 0.1
    # material id -> emitted RGB radiance of its triangles' front side
    # (pppm_material_emission); the reference's scenes have none
    emission: dict | None = None

    @property
    def ntri(self):
        return int(self.tris.shape[0])

    def bbox(self):
        v = self.tris.reshape(-1, 3).astype(np.float64)
        return v.min(0), v.max(0)


# --------------------------------------------------------------------- noise
def _lattice(ix, iy, iz, seed):
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841))
    h ^= iz.astype(np.uint32) * np.uint32(0xCB1AB31F)
    h ^= np.uint32(seed * 0x9E3779B9 & 0xFFFFFFFF)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x2C1B3C6D)
    h ^= h >> np.uint32(12)
    h *= np.uint32(0x297A2D39)
    h ^= h >> np.uint32(15)
    return h.astype(np.float64) / 4294967295.0 * 2.0 - 1.0


def value_noise(p, seed, octaves=3, base_freq=2.0):
    """Seeded multi-octave value noise in [-1, 1] (trilinear, smoothstep)."""
    p = np.asarray(p, np.float64)
    total = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        q = p * freq + 17.0 * (o + 1)
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        s = f * f * (3.0 - 2.0 * f)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = (s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) * (s[:, 2] if dz else 1 - s[:, 2])
                    acc += w * _lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed + 101 * o)
        total += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


# --------------------------------------------------------------------- meshes
def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
         [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
         [8, 6, 7], [9, 8, 1]], np.int64)
    return v, f


def geodesic_sphere(freq):
    """Icosahedron with every face split into freq^2 triangles, projected to
    the unit sphere. 20*freq^2 triangles; freq = 2^k is subdivision level k.
    Returns (T, 3, 3) float64 corner positions (outward winding)."""
    v, f = _icosahedron()
    n = freq
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    mask = ii + jj <= n
    ii, jj = ii[mask], jj[mask]
    index = -np.ones((n + 1, n + 1), np.int64)
    index[ii, jj] = np.arange(ii.size)
    up, down = [], []
    for i in range(n):
        for j in range(n - i):
            up.append((index[i, j], index[i + 1, j], index[i, j + 1]))
            if j < n - i - 1:
                down.append((index[i + 1, j], index[i + 1, j + 1], index[i, j + 1]))
    local = np.array(up + down, np.int64)
    out = []
    for a, b, c in f:
        A, B, C = v[a], v[b], v[c]
        # points P = A + (B-A)*i/n + (C-A)*j/n, built symmetrically so that
        # shared edges produce identical coordinates on both faces
        wi = ii[:, None] / n
        wj = jj[:, None] / n
        P = A[None] * (1 - wi - wj) + B[None] * wi + C[None] * wj
        P /= np.linalg.norm(P, axis=1, keepdims=True)
        out.append(P[local])
    tris = np.concatenate(out, 0)
    return tris


def displace_sphere(tris, radius, amp, seed, center=(0, 0, 0)):
    """Scales unit-sphere triangles to `radius` and displaces every vertex
    along its direction by amp*radius*noise(p). Vertices shared between
    triangles get identical displacement (noise is a function of position)."""
    p = tris.reshape(-1, 3)
    # canonicalise shared vertices first so equal points stay bit-equal
    p = np.round(p, 12)
    n = value_noise(p * 1.0, seed)
    r = radius * (1.0 + amp * n)
    q = p * r[:, None] + np.asarray(center, np.float64)[None]
    return q.reshape(-1, 3, 3)


def torus(R, r, nu, nv, amp, seed, center=(0, 0, 0)):
    u = np.arange(nu) / nu * 2 * np.pi
    v = np.arange(nv) / nv * 2 * np.pi
    U, V = np.meshgrid(u, v, indexing="ij")

    def pt(U, V):
        x = (R + r * np.cos(V)) * np.cos(U)
        z = (R + r * np.cos(V)) * np.sin(U)
        y = r * np.sin(V)
        P = np.stack([x, y, z], -1)
        noise = value_noise(P.reshape(-1, 3) / r, seed).reshape(P.shape[:-1])
        nrm = np.stack([np.cos(V) * np.cos(U), np.sin(V), np.cos(V) * np.sin(U)], -1)
        return P + nrm * (amp * r * noise)[..., None]

    P = pt(U, V)
    i1 = (np.arange(nu) + 1) % nu
    j1 = (np.arange(nv) + 1) % nv
    a = P
    b = P[i1]
    c = P[:, j1]
    d = P[i1][:, j1]
    t1 = np.stack([a, c, b], -2).reshape(-1, 3, 3)
    t2 = np.stack([b, c, d], -2).reshape(-1, 3, 3)
    return np.concatenate([t1, t2], 0) + np.asarray(center, np.float64)[None, None]


def quad(c0, c1, c2, c3):
    """Two triangles (c0, c1, c2), (c0, c2, c3)."""
    c0, c1, c2, c3 = (np.asarray(c, np.float64) for c in (c0, c1, c2, c3))
    return np.stack([np.stack([c0, c1, c2]), np.stack([c0, c2, c3])])


def ground(y, half):
    return quad((-half, y, -half), (-half, y, half), (half, y, half), (half, y, -half))


def open_box(half):
    """Five walls (10 triangles) of a cube [-half, half]^3, open towards -z
    (the camera side), inward-facing winding."""
    h = half
    walls = [
        quad((-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h)),  # floor
        quad((-h, h, -h), (-h, h, h), (h, h, h), (h, h, -h)),  # ceiling
        quad((-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)),  # back
        quad((-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h)),  # left
        quad((h, -h, -h), (h, h, -h), (h, h, h), (h, -h, h)),  # right
    ]
    return np.concatenate(walls, 0)


# --------------------------------------------------------------------- env
def sky_env(w, h, seed, sun_dir=(0.4, 0.8, 0.45), sun_peak=5.0e4, sun_deg=0.5, sigma=0.3, sky=(0.6, 0.75, 1.0),
            horizon=(1.0, 0.95, 0.85), ground_rgb=(0.25, 0.22, 0.2)):
    """Equirect sky: vertical gradient + Gaussian sun lobe (peak `sun_peak`,
    `sun_deg` degrees wide) + lognormal per-texel noise of sigma `sigma`.
    Layout follows Envmap::sampleFromDir (envmap.cc:47-60): column = phi/2pi
    with phi = atan2(z, x), row = theta/pi with theta = acos(y)."""
    rng = np.random.default_rng(seed)
    ys = (np.arange(h) + 0.5) / h * np.pi
    xs = (np.arange(w) + 0.5) / w * 2 * np.pi
    th, ph = np.meshgrid(ys, xs, indexing="ij")
    d = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1)
    up = d[..., 1:2]
    t = np.clip(up, 0, 1)
    col = np.where(up > 0, np.asarray(horizon) * (1 - t) + np.asarray(sky) * t, np.asarray(ground_rgb))
    sd = np.asarray(sun_dir, np.float64)
    sd /= np.linalg.norm(sd)
    ang = np.degrees(np.arccos(np.clip((d * sd).sum(-1), -1, 1)))
    lobe = sun_peak * np.exp(-0.5 * (ang / (sun_deg * 0.5)) ** 2)
    col = col + lobe[..., None] * np.array([1.0, 0.95, 0.85])
    col = col * np.exp(sigma * rng.standard_normal((h, w, 1)))
    return col.astype(np.float32)


# --------------------------------------------------------------------- assembly
def _assemble(name, parts, mats, env, camera, **kw):
    tris = np.concatenate([p[0].reshape(-1, 9) for p in parts], 0).astype(np.float32)
    mat_id = np.concatenate([np.asarray(p[1], np.int32).reshape(-1) if np.ndim(p[1]) else np.full(p[0].shape[0], p[1], np.int32)
                             for p in parts]).astype(np.int32)
    return Scene(name, tris, mat_id, np.array(mats, MATERIAL_DTYPE), env, camera, **kw)


def look_camera(eye, target, fov, w, h):
    """Camera values are rounded to float32 so the C ABI (float fields) and
    the reference (doubles) see identical inputs."""
    eye = np.asarray(eye, np.float64)
    d = np.asarray(target, np.float64) - eye
    d /= np.linalg.norm(d)
    f32 = lambda v: tuple(float(np.float32(x)) for x in v)  # noqa: E731
    return Camera(f32(eye), f32(d), (0.0, 1.0, 0.0), float(np.float32(fov)), w, h)


def config1a(seed=1, width=256, height=256, photons=200_000, passes=16, subdiv=5, env_w=256, env_h=128):
    """Env-lit twin of the CPU-runnable configuration: open box of 10 wall
    triangles (side 40) around a noise-displaced icosphere (subdivision
    `subdiv`, 20*4^subdiv triangles, amplitude 5% of the radius), Lambertian
    albedos uniform in [0.2, 0.8]^3 per object."""
    rng = np.random.default_rng(seed)
    box = open_box(20.0)
    sph = displace_sphere(geodesic_sphere(2 ** subdiv), 8.0, 0.05, seed, center=(0, -12.0 + 8.0 * 1.0, 4.0))
    mats = [material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3)), material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3))]
    env = sky_env(env_w, env_h, seed, sun_peak=50.0, sun_deg=8.0)
    cam = look_camera((0.0, 2.0, -55.0), (0.0, 0.0, 0.0), 0.75, width, height)
    return _assemble("config1a", [(box, 0), (sph, 1)], mats, env, cam, photons=photons, passes=passes, max_depth=8)


def config1(seed=1, width=256, height=256, photons=200_000, passes=16, subdiv=5, emission=12.0):
    """The CPU-runnable configuration as written: the open box of 10 wall
    triangles (side 40) with a 2-triangle area light (10 x 10, just below
    the ceiling, facing down, emission `emission` RGB) around a
    noise-displaced icosphere (subdivision `subdiv`, 20*4^subdiv triangles,
    amplitude 5% of the radius); Lambertian albedos uniform in [0.2, 0.8]^3
    per object; no environment map (the light is the only source)."""
    rng = np.random.default_rng(seed)
    box = open_box(20.0)
    sph = displace_sphere(geodesic_sphere(2 ** subdiv), 8.0, 0.05, seed, center=(0, -12.0 + 8.0 * 1.0, 4.0))
    light = quad((-5.0, 19.5, -5.0), (5.0, 19.5, -5.0), (5.0, 19.5, 5.0), (-5.0, 19.5, 5.0))  # normal -y
    mats = [material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3)), material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3)),
            material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3))]
    cam = look_camera((0.0, 2.0, -55.0), (0.0, 0.0, 0.0), 0.75, width, height)
    sc = _assemble("config1", [(box, 0), (sph, 1), (light, 2)], mats, None, cam, photons=photons, passes=passes,
                   max_depth=8)
    sc.emission = {2: (emission, emission, emission)}
    return sc


def config2(seed=2, width=1920, height=1080, photons=4_000_000, passes=64, freq=209, env_w=2048, env_h=1024,
            clusters=64):
    """Plain PPM-APA at scale: a displaced geodesic sphere of 20*freq^2
    triangles (freq=209 -> 873,620) over a ground quad, lit by an equirect
    sky with a 0.5-degree sun lobe of peak 5e4 and lognormal texel noise
    sigma 0.3. Materials 60/20/20 Lambertian / mirror / dielectric (IOR 1.5),
    assigned per cluster of the sphere surface."""
    rng = np.random.default_rng(seed)
    sph = displace_sphere(geodesic_sphere(freq), 10.0, 0.05, seed, center=(0.0, 0.0, 0.0))
    cent = sph.mean(1)
    # clusters: k-means-free partition by longitude/latitude cells
    th = np.arccos(np.clip(cent[:, 1] / np.linalg.norm(cent, axis=1), -1, 1))
    ph = np.arctan2(cent[:, 2], cent[:, 0]) + np.pi
    nlat = int(round(math.sqrt(clusters / 2)))
    nlon = clusters // nlat
    cid = np.minimum((th / np.pi * nlat).astype(int), nlat - 1) * nlon + np.minimum((ph / (2 * np.pi) * nlon).astype(int), nlon - 1)
    kinds = rng.choice(3, size=clusters, p=[0.6, 0.2, 0.2])
    mats = [material(LAMBERTIAN, (0.7, 0.7, 0.7))]  # ground
    for k in range(clusters):
        if kinds[k] == 0:
            mats.append(material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3)))
        elif kinds[k] == 1:
            mats.append(material(SPECULAR, (0.95, 0.95, 0.95)))
        else:
            mats.append(material(REFRACTION, (0.99, 0.99, 0.99)))
    gnd = ground(-10.5, 30.0)
    env = sky_env(env_w, env_h, seed)
    cam = look_camera((-25.0, 8.0, -20.0), (0.0, -2.0, 0.0), 0.9, width, height)
    return _assemble("config2", [(gnd, 0), (sph, 1 + cid)], mats, env, cam, photons=photons, passes=passes,
                     max_depth=12)


def small_test_scene(seed=3, subdiv=3, width=64, height=48, photons=20_000):
    """Small mixed-material scene for parity tests (every BSDF kind)."""
    rng = np.random.default_rng(seed)
    gnd = ground(-6.0, 20.0)
    s1 = displace_sphere(geodesic_sphere(2 ** subdiv), 4.0, 0.05, seed, center=(-5.0, -2.0, 0.0))
    s2 = displace_sphere(geodesic_sphere(2 ** (subdiv - 1)), 3.0, 0.05, seed + 1, center=(5.0, -3.0, 2.0))
    s3 = displace_sphere(geodesic_sphere(2 ** (subdiv - 1)), 2.5, 0.05, seed + 2, center=(0.0, -3.5, -5.0))
    s4 = displace_sphere(geodesic_sphere(2 ** (subdiv - 1)), 2.0, 0.05, seed + 3, center=(1.0, 3.0, 4.0))
    mats = [material(LAMBERTIAN, (0.75, 0.7, 0.6)), material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3)),
            material(SPECULAR, (0.9, 0.9, 0.9)), material(REFRACTION, (0.99, 0.99, 0.99)),
            material(PHONG, (0.8, 0.8, 0.8), phong_n=64.0)]
    env = sky_env(128, 64, seed, sun_peak=200.0, sun_deg=6.0)
    cam = look_camera((0.0, 4.0, -30.0), (0.0, -1.0, 0.0), 0.8, width, height)
    return _assemble("small", [(gnd, 0), (s1, 1), (s2, 2), (s3, 3), (s4, 4)], mats, env, cam, photons=photons,
                     passes=4, max_depth=64)


def config3(seed=3, width=1280, height=720, photons=2_000_000, passes=32, nu=500, nv=200, env_w=1024, env_h=512):
    """Subsurface scattering: a noise-displaced torus of 2*nu*nv triangles
    (500 x 200 -> 200,000) with a refractive surface and a dipole BSSRDF
    (sigma_a ~ U[0.001, 0.05], sigma_s' ~ U[0.5, 3.0] per mm, eta 1.3; scene
    units are mm) on a Lambertian ground, sky-lit."""
    rng = np.random.default_rng(seed)
    tor = torus(10.0, 4.0, nu, nv, 0.05, seed, center=(0.0, 0.0, 0.0))
    gnd = ground(-4.5, 30.0)
    sa = rng.uniform(0.001, 0.05, 3)
    ss = rng.uniform(0.5, 3.0, 3)
    mats = [material(LAMBERTIAN, (0.7, 0.7, 0.7)),
            material(REFRACTION, (0.99, 0.99, 0.99), sigma_a=sa, sigmap_s=ss, eta=1.3, scale=1.0, bssrdf=True)]
    env = sky_env(env_w, env_h, seed, sun_peak=2.0e3, sun_deg=2.0)
    cam = look_camera((0.0, 14.0, -30.0), (0.0, -1.0, 0.0), 0.75, width, height)
    return _assemble("config3", [(gnd, 0), (tor, 1)], mats, env, cam, photons=photons, passes=passes, max_depth=12)


def small_sss_scene(seed=5, width=64, height=48, photons=20_000, nu=48, nv=24):
    """Small subsurface scene for parity tests: a refractive BSSRDF torus, a
    Lambertian BSSRDF sphere and a Lambertian ground."""
    rng = np.random.default_rng(seed)
    gnd = ground(-6.0, 20.0)
    tor = torus(6.0, 2.5, nu, nv, 0.05, seed, center=(-3.0, -3.0, 0.0))
    sph = displace_sphere(geodesic_sphere(6), 2.5, 0.05, seed + 1, center=(6.0, -3.5, -2.0))
    mats = [material(LAMBERTIAN, (0.75, 0.7, 0.6)),
            material(REFRACTION, (0.99, 0.99, 0.99), sigma_a=rng.uniform(0.001, 0.05, 3),
                     sigmap_s=rng.uniform(0.5, 3.0, 3), eta=1.3, scale=1.0, bssrdf=True),
            material(LAMBERTIAN, rng.uniform(0.3, 0.8, 3), sigma_a=rng.uniform(0.001, 0.05, 3),
                     sigmap_s=rng.uniform(0.5, 3.0, 3), eta=1.3, scale=1.0, bssrdf=True)]
    env = sky_env(128, 64, seed, sun_peak=200.0, sun_deg=6.0)
    cam = look_camera((0.0, 6.0, -28.0), (0.0, -2.0, 0.0), 0.8, width, height)
    return _assemble("small_sss", [(gnd, 0), (tor, 1), (sph, 2)], mats, env, cam, photons=photons, passes=4,
                     max_depth=64)


def config4_jobs(seed=4, n=64, min_side=128, max_side=1024, min_tris=5_000, max_tris=500_000,
                 min_photons=100_000, max_photons=2_000_000, passes=16):
    """Batched uneven jobs: n independent scenes (seeded displaced geodesic
    spheres or tori of log-uniform 5k-500k triangles over a ground quad, each
    under its own sky), image sides log-uniform in 128-1024 (16:9),
    photons log-uniform in 100k-2M, alpha in {0.6, 0.7, 0.8}, 16 passes.
    Returns [(scene, alpha)]."""
    rng = np.random.default_rng(seed)
    lu = lambda lo, hi: float(np.exp(rng.uniform(np.log(lo), np.log(hi))))  # noqa: E731
    jobs = []
    for k in range(n):
        tris = lu(min_tris, max_tris)
        if rng.uniform() < 0.5:
            freq = max(2, int(round(math.sqrt(tris / 20.0))))
            obj = displace_sphere(geodesic_sphere(freq), 8.0, 0.05, seed * 1000 + k, center=(0.0, 0.0, 0.0))
        else:
            nv = max(8, int(round(math.sqrt(tris / 2.0 / 2.5))))
            nu = max(8, int(round(tris / 2.0 / nv)))
            obj = torus(8.0, 3.0, nu, nv, 0.05, seed * 1000 + k)
        gnd = ground(-9.0, 25.0)
        mats = [material(LAMBERTIAN, (0.7, 0.7, 0.7)), material(LAMBERTIAN, rng.uniform(0.2, 0.8, 3))]
        side = lu(min_side, max_side)
        w = int(round(side)) // 16 * 16
        h = max(16, int(round(w * 9 / 16)))
        env = sky_env(256, 128, seed * 1000 + k, sun_peak=2.0e3, sun_deg=3.0)
        cam = look_camera((-22.0, 9.0, -18.0), (0.0, -1.0, 0.0), 0.9, max(w, 16), h)
        sc = _assemble(f"job{k}", [(gnd, 0), (obj, 1)], mats, env, cam,
                       photons=int(round(lu(min_photons, max_photons))), passes=passes, max_depth=8)
        jobs.append((sc, float(rng.choice([0.6, 0.7, 0.8]))))
    return jobs


# --------------------------------------------------------------------- files
def write_ply(path, tris):
    """Binary little-endian PLY in the layout Trimesh::loadPly reads
    (trimesh.cc:139-217): float x/y/z vertices, faces as uchar count + 3 int."""
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 3, 3)
    n = t.shape[0]
    verts = t.reshape(-1, 3)
    faces = np.zeros(n, np.dtype([("n", "u1"), ("i", "<i4", (3,))]))
    faces["n"] = 3
    faces["i"] = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    head = (f"ply\nformat binary_little_endian 1.0\nelement vertex {3 * n}\nproperty float x\nproperty float y\n"
            f"property float z\nelement face {n}\nproperty list uchar int vertex_indices\nend_header\n")
    with open(path, "wb") as f:
        f.write(head.encode())
        f.write(verts.astype("<f4").tobytes())
        f.write(faces.tobytes())


def write_hdr(path, rgb):
    """Radiance RGBE file with the layout of Image::saveHdr (image.cc:436-482):
    -Y H +X W, every scanline new-style RLE with literal runs of <= 127."""
    rgb = np.asarray(rgb, np.float64)
    h, w = rgb.shape[:2]
    m = rgb.max(2)
    e = np.zeros((h, w), np.int64)
    mant, ex = np.frexp(np.where(m > 1e-32, m, 1.0))
    e = np.where(m > 1e-32, ex, 0)
    scale = np.where(m > 1e-32, mant * 256.0 / np.where(m > 1e-32, m, 1.0), 0.0)
    px = np.zeros((h, w, 4), np.uint8)
    px[..., :3] = np.where(m[..., None] > 1e-32, np.floor(rgb * scale[..., None]), 0).astype(np.uint8)
    px[..., 3] = np.where(m > 1e-32, e + 128, 0).astype(np.uint8)
    out = bytearray(b"#?RADIANCE\n# synthetic\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0000000000000\n\n")
    out += f"-Y {h} +X {w}\n".encode()
    for y in range(h):
        out += bytes([2, 2, (w >> 8) & 0xFF, w & 0xFF])
        for c in range(4):
            row = px[y, :, c]
            for s in range(0, w, 127):
                chunk = row[s:s + 127]
                out.append(len(chunk))
                out += chunk.tobytes()
    with open(path, "wb") as f:
        f.write(bytes(out))
