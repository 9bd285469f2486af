// Classic progressive photon mapping: ProgressivePhotonMapping::render
// (progressive_photon_mapping.cc:31-345) on the GPU.
//
// Every pixel owns a render point (position, normal, path weight, radius^2,
// photon count, flux, accumulated emission). Per pass:
//   1. kClassicEye: each pixel's eye path (executePathTracing, :296-345)
//      re-places its render point at the first Lambertian hit;
//   2. the render-point hash grid (constructHashGrid, :121-155): bounding box
//      of all render points, initial radius from its mean extent, every point
//      registered in the buckets of the cells of its +-radius box, with the
//      reference's hash over numPixels buckets;
//   3. the photon pass (tracePhotons, :193-294) on the wavefront kernels: at
//      every Lambertian hit the bucket of the hit position is scanned and each
//      render point facing the same way within its radius gets an update
//      event (render point, photon order key, squared distance, flux);
//   4. kClassicUpdate applies each render point's events in the reference's
//      photon order in double: r2 *= g, n += 1, flux = (flux + w Phi/pi) g
//      with g = (n a + a) / (n a + 1), each test against the updated r2.
// Random numbers are the reference's permuted Halton sequences (halton.cc):
// sampler s (one per reference thread, seeded s) serves the pixels
// i = s, s + N, ... of a pass and then its ceil(P/N) photons; the radical
// inverse is evaluated in double with the reference's operation order. The
// reference applies the updates of N > 1 threads under a lock in a
// run-dependent order; N = 1 reproduces it, N > 1 uses photon index order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "grid.cuh"
#include "trace.h"

namespace pppm {

namespace {

constexpr double kPiD = 3.14159265358979323846;

struct RpView {
    double* pos;       // 3 per point
    float* nrm;        // 3 per point (the triangle normal, double-derived)
    double* flux;      // 3
    double* weight;    // 3
    double* emission;  // 3
    double* r2;
    int* n;
    float* coeff;
};

// Render point bucket view: the reference's HashGrid<RenderPoint*> over
// numPixels buckets.
struct RpGrid {
    const uint32_t* start;  // size + 1
    const int* entries;
    uint32_t size;
    double ox, oy, oz, scale;
};

__device__ __forceinline__ uint32_t rpBucket(const RpGrid& g, double x, double y, double z) {
    const int ix = abs(__double2int_rz(__dmul_rn(__dsub_rn(x, g.ox), g.scale)));
    const int iy = abs(__double2int_rz(__dmul_rn(__dsub_rn(y, g.oy), g.scale)));
    const int iz = abs(__double2int_rz(__dmul_rn(__dsub_rn(z, g.oz), g.scale)));
    return refHash(ix, iy, iz, g.size);
}

struct ClassicEvent {
    unsigned long long key;  // photon order, bounce, duplicate
    double d2;               // |rp - hit|^2
    float fx, fy, fz;
    int rp;
};

// ------------------------------------------------------------ eye pass
__global__ void __launch_bounds__(128, PPPM_TRACE_MINBLOCKS) kClassicEye(TraceParams tp, SceneView sc, EnvDev env,
                                                                         CameraDev cam, HaltonDev hd, RpView rp,
                                                                         int it, PassCounters* ctr) {
    __shared__ int order[128];
    __shared__ QNode sTop[kTopNodes];
    loadOrderTable(order);
    loadTopNodes(sTop, sc.nodes, sc.numNodes);
    const int64_t np = (int64_t)cam.w * cam.h;
    const int N = tp.numStreams;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < np; base += stride) {
        const int64_t pix = base + threadIdx.x;
        bool alive = pix < np;
        int traced = 0, visits = 0, tests = 0;
        HaltonTape tape{&hd, 0, 0, 0, false};
        f3 d = {0.f, 0.f, 1.f};
        double o[3] = {cam.ex, cam.ey, cam.ez};
        double wx = 1.0, wy = 1.0, wz = 1.0;
        if (alive) {
            const int s = (int)(pix % N);
            const int64_t pixOfStream = (np - s + N - 1) / N;
            tape.stream = s;
            tape.index = (unsigned long long)it * (unsigned long long)(pixOfStream + tp.taskPerThread) + pix / N;
            const int x = (int)(pix % cam.w), y = (int)(pix / cam.w);
            const double px = __dsub_rn(__dadd_rn((double)x, tape.popd()), 0.5);
            const double py = __dsub_rn(__dadd_rn((double)y, tape.popd()), 0.5);
            cameraRay(cam, (float)px, (float)py, &d);
        }
        for (int b = 0; __any_sync(0xffffffffu, alive); b++) {
            const bool doTrace = alive && b < tp.maxBounceEye;
            double best;
            const int slot = traverseExactWarp(sc.nodes, sc.tris, sc.rootCode, doTrace, o[0], o[1], o[2], d.x, d.y,
                                               d.z, order, sTop, &best, &visits, &tests);
            if (!alive) continue;
            if (doTrace) traced++;
            if (!doTrace || slot < 0) {
                // the path leaves: the render point keeps its place; weight,
                // coeff and the escaped radiance are recorded (:310-316)
                const f3 L = envLookup(env, d);
                rp.weight[3 * pix] = wx; rp.weight[3 * pix + 1] = wy; rp.weight[3 * pix + 2] = wz;
                rp.coeff[pix] = 1.0f;
                rp.emission[3 * pix] += wx * L.x;
                rp.emission[3 * pix + 1] += wy * L.y;
                rp.emission[3 * pix + 2] += wz * L.z;
                alive = false;
                continue;
            }
            const uint32_t r0 = tape.popu(), r1 = tape.popu();
            const float4 a = sc.tris[3 * slot], bb = sc.tris[3 * slot + 1], c = sc.tris[3 * slot + 2];
            const DevMaterial& m = sc.mats[sc.matId[__float_as_int(a.w)]];
            double hp[3];
            hitPosition(o[0], o[1], o[2], d.x, d.y, d.z, best, hp);
            const f3 nrm = triNormal(a, bb, c);
            const f3 on = dot(nrm, d) < 0.0f ? nrm : -nrm;
            if (m.type == PPPM_BSDF_LAMBERTIAN) {
                // the render point moves here (:325-332)
                wx *= m.refl[0]; wy *= m.refl[1]; wz *= m.refl[2];
                rp.pos[3 * pix] = hp[0]; rp.pos[3 * pix + 1] = hp[1]; rp.pos[3 * pix + 2] = hp[2];
                rp.nrm[3 * pix] = nrm.x; rp.nrm[3 * pix + 1] = nrm.y; rp.nrm[3 * pix + 2] = nrm.z;
                rp.weight[3 * pix] = wx; rp.weight[3 * pix + 1] = wy; rp.weight[3 * pix + 2] = wz;
                rp.coeff[pix] = 1.0f;
                alive = false;
                continue;
            }
            // every other BSDF (a BSSRDF never stands alone here) is sampled
            // around the oriented normal (:333-339)
            f3 nd;
            const float pdf = bsdfSample(m, d, on, r0, r1, &nd);
            wx = wx * m.refl[0] / pdf;
            wy = wy * m.refl[1] / pdf;
            wz = wz * m.refl[2] / pdf;
            o[0] = hp[0]; o[1] = hp[1]; o[2] = hp[2];
            d = nd;
        }
        if (tape.over) atomicAdd(&ctr->undefinedEye, 1ull);
        const unsigned nt = __reduce_add_sync(0xffffffffu, (unsigned)traced);
        if ((threadIdx.x & 31) == 0 && nt) atomicAdd(&ctr->eyeRays, (unsigned long long)nt);
    }
}

// ------------------------------------------------------------ grid
__global__ void kRpBbox(const double* __restrict__ pos, int64_t n, double* __restrict__ part) {
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < 3; d++) {
            const double v = pos[3 * i + d];
            mn[d] = fmin(mn[d], v);
            mx[d] = fmax(mx[d], v);
        }
    __shared__ double s[6][256];
    for (int d = 0; d < 3; d++) { s[d][threadIdx.x] = mn[d]; s[3 + d][threadIdx.x] = mx[d]; }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < 3; d++) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + w]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 6; d++) part[6 * blockIdx.x + d] = s[d][0];
}

__global__ void kRpBboxFinal(const double* __restrict__ part, int nb, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double r[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
    for (int b = 0; b < nb; b++)
        for (int d = 0; d < 3; d++) {
            r[d] = fmin(r[d], part[6 * b + d]);
            r[3 + d] = fmax(r[3 + d], part[6 * b + 3 + d]);
        }
    for (int d = 0; d < 6; d++) out[d] = r[d];
}

// Cells of a render point's +-irad box (hash_grid_detail.h:34-52).
__device__ __forceinline__ void rpBox(const RpGrid& g, const double* p, double irad, int* lo, int* hi) {
    const double o[3] = {g.ox, g.oy, g.oz};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        lo[d] = abs(__double2int_rz(__dmul_rn(__dsub_rn(__dsub_rn(p[d], irad), o[d]), g.scale)));
        hi[d] = abs(__double2int_rz(__dmul_rn(__dsub_rn(__dadd_rn(p[d], irad), o[d]), g.scale)));
    }
}

// kFill = false: n == 0 points take the initial radius (:132-137) and the
// bucket histogram is counted; kFill = true: entries are scattered.
template <bool kFill>
__global__ void kRpCells(RpView rp, int64_t n, RpGrid g, double irad, uint32_t* __restrict__ hist,
                         uint32_t* __restrict__ cursor, int* __restrict__ entries) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!kFill && rp.n[i] == 0) {
            rp.r2[i] = __dmul_rn(irad, irad);
            rp.flux[3 * i] = rp.flux[3 * i + 1] = rp.flux[3 * i + 2] = 0.0;
        }
        const double p[3] = {rp.pos[3 * i], rp.pos[3 * i + 1], rp.pos[3 * i + 2]};
        int lo[3], hi[3];
        rpBox(g, p, irad, lo, hi);
        for (int iz = lo[2]; iz <= hi[2]; iz++)
            for (int iy = lo[1]; iy <= hi[1]; iy++)
                for (int ix = lo[0]; ix <= hi[0]; ix++) {
                    const uint32_t h = refHash(ix, iy, iz, g.size);
                    if (kFill) entries[atomicAdd(&cursor[h], 1u)] = (int)i;
                    else atomicAdd(&hist[h], 1u);
                }
    }
}

// ------------------------------------------------------------ photon pass
__device__ inline bool classicEmit(const EnvDev& e, HaltonTape& tp, f3* emitDir, f3* dir, f3* flux) {
    // Envmap::samplePhoton (envmap.cc:62-86): lower_bound over the double CDF
    const double r = tp.popd();
    int lo = 0, hi = 4096;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&e.cdf[mid]) < r) lo = mid + 1; else hi = mid;
    }
    const int index = lo;
    const int ix = index % 64, iy = index / 64;
    const float u = ((float)ix + (float)tp.popd()) * (1.0f / 64.0f);
    const float v = ((float)iy + (float)tp.popd()) * (1.0f / 64.0f);
    const float phi = u * kPiF * 2.0f;
    const float y = (1.0f - v) * 2.0f - 1.0f;
    const float sxz = sqrtf(fmaxf(0.0f, 1.0f - y * y));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const f3 d = {sxz * cp, y, sxz * sp};
    *flux = envLookup(e, d) * __ldg(&e.fluxScale[min(index, 4095)]);
    *emitDir = d;
    // onHemisphere(normalLight, &nextDir, rseq.pop(), rseq.pop()) (:210): the
    // arguments are evaluated right to left, as in ppm_probabilistic.cc
    const float a0 = (float)tp.popd();
    const float a1 = (float)tp.popd();
    *dir = onHemisphere(-d, a1, a0);
    return index < 4096;
}

// Path tape state in PathState.rng: [0,1] sample index, [2] dim, [3] stream.
__device__ __forceinline__ HaltonTape tapeOf(const HaltonDev* hd, const PathState& p) {
    return HaltonTape{hd, (int)p.rng[3], (unsigned long long)p.rng[0] | ((unsigned long long)p.rng[1] << 32),
                      (int)p.rng[2], false};
}

__global__ void kClassicEmit(TraceParams tp, EnvDev env, HaltonDev hd, int64_t np, int it, PathState* __restrict__ q,
                             PassCounters* ctr) {
    const int N = tp.numStreams;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < tp.numPaths;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g / tp.taskPerThread);
        const int64_t i = g % tp.taskPerThread;
        const int64_t pixOfStream = (np - s + N - 1) / N;
        HaltonTape tape{&hd, s, (unsigned long long)it * (unsigned long long)(pixOfStream + tp.taskPerThread) +
                                    (unsigned long long)(pixOfStream + i),
                        0, false};
        f3 d, dir, flux;
        const bool ok = classicEmit(env, tape, &d, &dir, &flux);
        if (!ok || tape.over) atomicAdd(&ctr->undefinedEmit, 1ull);
        PathState p;
        p.ox = 50.0 * (double)d.x;
        p.oy = 50.0 * (double)d.y;
        p.oz = 50.0 * (double)d.z;
        p.dx = dir.x; p.dy = dir.y; p.dz = dir.z;
        p.fx = ok ? flux.x : 0.f; p.fy = ok ? flux.y : 0.f; p.fz = ok ? flux.z : 0.f;
        p.rng[0] = (uint32_t)tape.index;
        p.rng[1] = (uint32_t)(tape.index >> 32);
        p.rng[2] = (uint32_t)tape.dim;
        p.rng[3] = (uint32_t)s;
        p.id = (int)(i * N + s);  // the reference's photon order: round i, thread s
        p.bounce = 0;
        p.pad[0] = p.pad[1] = 0;
        q[g] = p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctr->queue[0] = (unsigned long long)tp.numPaths;
        ctr->queue[1] = 0;
        ctr->queue[2] = 0;
    }
}

__global__ void __launch_bounds__(128, PPPM_TRACE_MINBLOCKS) kClassicBounce(TraceParams tp, SceneView sc, HaltonDev hd,
                                                                            RpView rp, RpGrid rg, int bounce,
                                                                            const PathState* __restrict__ in,
                                                                            PathState* __restrict__ out,
                                                                            int64_t maxPaths, ClassicEvent* ev,
                                                                            int64_t evCap, PassCounters* ctr) {
    __shared__ int order[128];
    __shared__ QNode sTop[kTopNodes];
    const int qi = bounce % 3, qo = (bounce + 1) % 3, qz = (bounce + 2) % 3;
    const int64_t n = min((int64_t)ctr->queue[qi], maxPaths);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr->queue[qz] = 0;
    if ((int64_t)blockIdx.x * blockDim.x >= n) return;  // past the live paths
    loadOrderTable(order);
    loadTopNodes(sTop, sc.nodes, sc.numNodes);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool alive = false;
        PathState p;
        p.ox = p.oy = p.oz = 0.0;
        p.dx = p.dy = 0.f;
        p.dz = 1.f;
        if (i < n) {
            p = in[i];
            alive = p.bounce < tp.maxBouncePhoton && fmaxf(p.fx, fmaxf(p.fy, p.fz)) > 0.0f;
        }
        int traced = 0, visits = 0, tests = 0;
        double best;
        const int slot = traverseExactWarp(sc.nodes, sc.tris, sc.rootCode, alive, p.ox, p.oy, p.oz, p.dx, p.dy, p.dz,
                                           order, sTop, &best, &visits, &tests);
        if (alive) {
            traced = 1;
            if (slot < 0) {
                alive = false;
            } else {
                HaltonTape tape = tapeOf(&hd, p);
                const double rd0 = tape.popd();
                const uint32_t r0 = (uint32_t)fmin(rd0 * 4294967296.0, 4294967295.0);
                const uint32_t r1 = tape.popu(), r2 = tape.popu();
                if (tape.over) atomicAdd(&ctr->undefinedEye, 1ull);
                const float4 a = sc.tris[3 * slot], b = sc.tris[3 * slot + 1], c = sc.tris[3 * slot + 2];
                const DevMaterial& m = sc.mats[sc.matId[__float_as_int(a.w)]];
                double hp[3];
                hitPosition(p.ox, p.oy, p.oz, p.dx, p.dy, p.dz, best, hp);
                const f3 nrm = triNormal(a, b, c);
                const f3 din = {p.dx, p.dy, p.dz};
                const f3 on = dot(nrm, din) < 0.0f ? nrm : -nrm;
                f3 flux = {p.fx, p.fy, p.fz};
                const f3 refl = {m.refl[0], m.refl[1], m.refl[2]};
                f3 nd;
                if (m.type == PPPM_BSDF_LAMBERTIAN) {
                    // the render points of the hit's bucket (:241-260)
                    const uint32_t h = rpBucket(rg, hp[0], hp[1], hp[2]);
                    int dup = 0, last = -1;
                    for (uint32_t e = rg.start[h]; e < rg.start[h + 1]; e++) {
                        const int k = rg.entries[e];
                        dup = k == last ? dup + 1 : 0;
                        last = k;
                        const float dn = rp.nrm[3 * k] * nrm.x + rp.nrm[3 * k + 1] * nrm.y + rp.nrm[3 * k + 2] * nrm.z;
                        if (!(dn > 1e-12f)) continue;
                        const double vx = __dsub_rn(rp.pos[3 * k], hp[0]), vy = __dsub_rn(rp.pos[3 * k + 1], hp[1]),
                                     vz = __dsub_rn(rp.pos[3 * k + 2], hp[2]);
                        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
                        if (!(d2 <= rp.r2[k])) continue;  // r2 only shrinks during the pass
                        const unsigned long long ei = atomicAdd(&ctr->deposits, 1ull);
                        if ((int64_t)ei < evCap) {
                            ClassicEvent E;
                            E.key = ((unsigned long long)(unsigned)p.id << 16) | ((unsigned long long)p.bounce << 8) |
                                    (unsigned long long)min(dup, 255);
                            E.d2 = d2;
                            E.fx = flux.x; E.fy = flux.y; E.fz = flux.z;
                            E.rp = k;
                            ev[ei] = E;
                        }
                    }
                    // Russian roulette on the mean albedo (:262-271), in double
                    if (rd0 < m.rr_photon) {
                        bsdfSample(m, din, on, r1, r2, &nd);
                        flux = flux * refl * m.invRr;
                    } else {
                        alive = false;
                    }
                } else {
                    // other BSDFs: the flux keeps no 1/pdf here (:273-278)
                    bsdfSample(m, din, on, r0, r1, &nd);
                    flux = flux * refl;
                }
                p.ox = hp[0]; p.oy = hp[1]; p.oz = hp[2];
                p.dx = nd.x; p.dy = nd.y; p.dz = nd.z;
                p.fx = flux.x; p.fy = flux.y; p.fz = flux.z;
                p.rng[0] = (uint32_t)tape.index;
                p.rng[1] = (uint32_t)(tape.index >> 32);
                p.rng[2] = (uint32_t)tape.dim;
                p.bounce += 1;
            }
        }
        const unsigned long long oi = warpAppend(alive, &ctr->queue[qo]);
        if (alive) out[oi] = p;
        const unsigned nt = __reduce_add_sync(0xffffffffu, (unsigned)traced);
        if ((threadIdx.x & 31) == 0 && nt) atomicAdd(&ctr->photonRays, (unsigned long long)nt);
    }
}

// ------------------------------------------------------------ updates
__global__ void kEvHist(const ClassicEvent* __restrict__ ev, const unsigned long long* count, int64_t cap,
                        uint32_t* __restrict__ hist) {
    const int64_t n = min((int64_t)*count, cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&hist[ev[i].rp], 1u);
}

__global__ void kEvScatter(const ClassicEvent* __restrict__ ev, const unsigned long long* count, int64_t cap,
                           uint32_t* __restrict__ cursor, ClassicEvent* __restrict__ sorted) {
    const int64_t n = min((int64_t)*count, cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const ClassicEvent e = ev[i];
        sorted[atomicAdd(&cursor[e.rp], 1u)] = e;
    }
}

// Each render point applies its events in photon order (:248-256).
__global__ void kClassicUpdate(RpView rp, int64_t np, const uint32_t* __restrict__ start,
                               ClassicEvent* __restrict__ ev, double alpha) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = start[k], e = start[k + 1];
        if (s == e) continue;
        // insertion sort by key (a render point sees few photons per pass)
        for (uint32_t i = s + 1; i < e; i++) {
            const ClassicEvent x = ev[i];
            uint32_t j = i;
            while (j > s && ev[j - 1].key > x.key) {
                ev[j] = ev[j - 1];
                j--;
            }
            ev[j] = x;
        }
        double r2 = rp.r2[k];
        int n = rp.n[k];
        double fx = rp.flux[3 * k], fy = rp.flux[3 * k + 1], fz = rp.flux[3 * k + 2];
        const double wx = rp.weight[3 * k], wy = rp.weight[3 * k + 1], wz = rp.weight[3 * k + 2];
        const double invPi = 1.0 / kPiD;
        for (uint32_t i = s; i < e; i++) {
            const ClassicEvent& x = ev[i];
            if (!(x.d2 <= r2)) continue;
            const double na = __dmul_rn((double)n, alpha);
            const double g = __ddiv_rn(__dadd_rn(na, alpha), __dadd_rn(na, 1.0));
            r2 = __dmul_rn(r2, g);
            n += 1;
            fx = __dmul_rn(__dadd_rn(fx, __dmul_rn(__dmul_rn(wx, (double)x.fx), invPi)), g);
            fy = __dmul_rn(__dadd_rn(fy, __dmul_rn(__dmul_rn(wy, (double)x.fy), invPi)), g);
            fz = __dmul_rn(__dadd_rn(fz, __dmul_rn(__dmul_rn(wz, (double)x.fz), invPi)), g);
        }
        rp.r2[k] = r2;
        rp.n[k] = n;
        rp.flux[3 * k] = fx;
        rp.flux[3 * k + 1] = fy;
        rp.flux[3 * k + 2] = fz;
    }
}

// The pass image, not divided by the pass count: (emission + flux / (pi r2)) * coeff.
__global__ void kClassicImage(RpView rp, int64_t np, float* __restrict__ out) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
        const double inv = 1.0 / (kPiD * rp.r2[k]);
        const double c = rp.coeff[k];
        for (int d = 0; d < 3; d++) out[3 * k + d] = (float)((rp.emission[3 * k + d] + rp.flux[3 * k + d] * inv) * c);
    }
}

unsigned blocksOf(int64_t n, int bs, int cap = 152 * 16) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + bs - 1) / bs, cap));
}

RpView rpView(ClassicState& s) {
    return RpView{s.pos.as<double>(), s.nrm.as<float>(), s.flux.as<double>(), s.weight.as<double>(),
                  s.emission.as<double>(), s.r2.as<double>(), s.n.as<int>(), s.coeff.as<float>()};
}

HaltonDev haltonView(ClassicState& s) {
    return HaltonDev{s.haltonPerm.as<uint16_t>(), s.haltonPrime.as<int>(), s.haltonOffset.as<int>(), s.haltonSum};
}

}  // namespace

// Halton(200, true, seed) permutation tables (halton.cc:88-112): bases are
// the first 200 primes; with permutation, each base's digits are shuffled by
// XorShift(seed): for i < d, swap p[i] with p[i + nextInt(d - i)].
static bool haltonTables(int streams, std::vector<uint16_t>* perm, std::vector<int>* primes, std::vector<int>* offs,
                         int* sum) {
    primes->clear();
    for (int v = 2; (int)primes->size() < kHaltonDims; v++) {
        bool pr = true;
        for (int q : *primes) {
            if (q * q > v) break;
            if (v % q == 0) { pr = false; break; }
        }
        if (pr) primes->push_back(v);
    }
    offs->assign(kHaltonDims, 0);
    int s = 0;
    for (int i = 0; i < kHaltonDims; i++) {
        (*offs)[i] = s;
        s += (*primes)[i];
    }
    *sum = s;
    perm->assign((size_t)streams * s, 0);
    for (int st = 0; st < streams; st++) {
        XorShift x;
        x.seed((uint32_t)st);
        uint16_t* p = perm->data() + (size_t)st * s;
        for (int i = 0; i < kHaltonDims; i++) {
            const int d = (*primes)[i];
            for (int k = 0; k < d; k++) p[k] = (uint16_t)k;
            for (int k = 0; k < d; k++) {
                const uint32_t v = x.next();
                if (v == 0x80000000u) return false;  // abs(INT_MIN): undefined in nextInt
                const int r = std::abs((int)v) % (d - k);
                std::swap(p[k], p[k + r]);
            }
            p += d;
        }
    }
    return true;
}

int haltonBegin(pppm_ctx* c, int streams) {
    ClassicState& s = c->rs.classic;
    std::vector<uint16_t> perm;
    std::vector<int> primes, offs;
    if (!haltonTables(streams, &perm, &primes, &offs, &s.haltonSum))
        return fail(c, PPPM_E_UNDEFINED, "render_begin: a Halton permutation draws abs(INT_MIN) (undefined)");
    PPPM_CUDA(c, s.haltonPerm.ensure(perm.size() * 2));
    PPPM_CUDA(c, s.haltonPrime.ensure(primes.size() * 4));
    PPPM_CUDA(c, s.haltonOffset.ensure(offs.size() * 4));
    PPPM_CUDA(c, cudaMemcpy(s.haltonPerm.p, perm.data(), perm.size() * 2, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(s.haltonPrime.p, primes.data(), primes.size() * 4, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(s.haltonOffset.p, offs.data(), offs.size() * 4, cudaMemcpyHostToDevice));
    return PPPM_OK;
}

HaltonDev haltonDev(pppm_ctx* c) { return haltonView(c->rs.classic); }

int classicBegin(pppm_ctx* c, int64_t pixels) {
    ClassicState& s = c->rs.classic;
    {
        const int e = haltonBegin(c, c->rs.par.num_streams);
        if (e) return e;
    }
    const size_t P = (size_t)pixels;
    PPPM_CUDA(c, s.pos.ensure(P * 24));
    PPPM_CUDA(c, s.nrm.ensure(P * 12));
    PPPM_CUDA(c, s.flux.ensure(P * 24));
    PPPM_CUDA(c, s.weight.ensure(P * 24));
    PPPM_CUDA(c, s.emission.ensure(P * 24));
    PPPM_CUDA(c, s.r2.ensure(P * 8));
    PPPM_CUDA(c, s.n.ensure(P * 4));
    PPPM_CUDA(c, s.coeff.ensure(P * 4));
    // RenderPoint(): position, normal, flux, weight, emission 0; n = 0 (:60-75)
    for (DBuf* b : {&s.pos, &s.nrm, &s.flux, &s.weight, &s.emission, &s.r2, &s.n, &s.coeff})
        PPPM_CUDA(c, cudaMemsetAsync(b->p, 0, b->cap, c->stream));
    PPPM_CUDA(c, s.gridCount.ensure((P + 1) * 4));
    PPPM_CUDA(c, s.gridCursor.ensure((P + 1) * 4));
    PPPM_CUDA(c, s.gridTmp.ensure((size_t)scanTmpWords((int64_t)P + 1) * 4));
    PPPM_CUDA(c, s.evCount.ensure((P + 1) * 4));
    PPPM_CUDA(c, s.evCursor.ensure((P + 1) * 4));
    PPPM_CUDA(c, s.evTmp.ensure((size_t)scanTmpWords((int64_t)P + 1) * 4));
    PPPM_CUDA(c, s.bbox.ensure((6 + 6 * 152 * 4) * 8));
    PPPM_CUDA(c, s.misc.ensure(64));
    if (s.evCap == 0) s.evCap = std::max<int64_t>(4 * c->rs.par.photons, 1 << 20);
    PPPM_CUDA(c, s.ev.ensure((size_t)s.evCap * sizeof(ClassicEvent)));
    PPPM_CUDA(c, s.evSorted.ensure((size_t)s.evCap * sizeof(ClassicEvent)));
    return PPPM_OK;
}

int classicPass(pppm_ctx* c, int t, const TraceParams& tp0, const SceneView& sv, const EnvDev& ev, const CameraDev& cd,
                pppm_pass_stats* stats) {
    RenderState& rs = c->rs;
    ClassicState& s = rs.classic;
    const int W = rs.cam.width, H = rs.cam.height;
    const int64_t np = (int64_t)W * H;
    const int it = t - 1;
    TraceParams tp = tp0;
    HaltonDev hd = haltonView(s);
    RpView rp = rpView(s);
    PassCounters* ctr = rs.photonCount.as<PassCounters>();
    int64_t launches = 0;
    PPPM_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(PassCounters), c->stream));
    // 1st pass: rays from the camera
    kClassicEye<<<blocksOf(np, 128, 152 * rs.eyePerSm), 128, 0, c->stream>>>(tp, sv, ev, cd, hd, rp, it, ctr);
    PPPM_CUDA(c, cudaGetLastError());
    PPPM_CUDA(c, cudaEventRecord(c->ev[3], c->stream));
    // render-point hash grid
    const int nb = 152 * 4;
    kRpBbox<<<nb, 256, 0, c->stream>>>(s.pos.as<double>(), np, s.bbox.as<double>() + 6);
    kRpBboxFinal<<<1, 32, 0, c->stream>>>(s.bbox.as<double>() + 6, nb, s.bbox.as<double>());
    double hb[6];
    PPPM_CUDA(c, cudaMemcpyAsync(hb, s.bbox.p, 48, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    const double irad = ((hb[3] - hb[0] + (hb[4] - hb[1]) + (hb[5] - hb[2])) / 3.0) / ((W + H) / 2.0) * 8.0;
    if (!(irad > 0.0) || !std::isfinite(irad))
        return fail(c, PPPM_E_UNDEFINED,
                    "render_pass: all render points coincide (zero initial radius: the reference divides by zero)");
    RpGrid rg;
    rg.ox = hb[0] - irad;
    rg.oy = hb[1] - irad;
    rg.oz = hb[2] - irad;
    rg.scale = 1.0 / (irad * 2.0);
    rg.size = (uint32_t)np;
    s.irad = irad;
    uint32_t* hist = s.gridCount.as<uint32_t>();
    PPPM_CUDA(c, cudaMemsetAsync(hist, 0, (size_t)(np + 1) * 4, c->stream));
    kRpCells<false><<<blocksOf(np, 256), 256, 0, c->stream>>>(rp, np, rg, irad, hist, nullptr, nullptr);
    PPPM_CUDA(c, exclusiveScan(hist, np, s.gridCursor.as<uint32_t>(), s.gridTmp.as<uint32_t>(), c->stream));
    uint32_t entries = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&entries, hist + np, 4, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    PPPM_CUDA(c, s.gridEntries.ensure((size_t)std::max<uint32_t>(entries, 1) * 4));
    kRpCells<true><<<blocksOf(np, 256), 256, 0, c->stream>>>(rp, np, rg, irad, nullptr, s.gridCursor.as<uint32_t>(),
                                                            s.gridEntries.as<int>());
    rg.start = hist;
    rg.entries = s.gridEntries.as<int>();
    launches += 8;
    PPPM_CUDA(c, cudaEventRecord(c->ev[2], c->stream));
    // 2nd pass: photons
    const int64_t paths = tp.numPaths;
    PassCounters hc;
    for (int attempt = 0;; attempt++) {
        PPPM_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(PassCounters), c->stream));
        kClassicEmit<<<blocksOf(paths, 256), 256, 0, c->stream>>>(tp, ev, hd, np, it, rs.pathA.as<PathState>(), ctr);
        PPPM_CUDA(c, cudaGetLastError());
        for (int b = 0; b < tp.maxBouncePhoton; b++) {
            PathState* in = (b & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
            PathState* out = (b & 1) ? rs.pathA.as<PathState>() : rs.pathB.as<PathState>();
            kClassicBounce<<<blocksOf(paths, 128, 152 * rs.bouncePerSm), 128, 0, c->stream>>>(
                tp, sv, hd, rp, rg, b, in, out, paths, s.ev.as<ClassicEvent>(), s.evCap, ctr);
        }
        PPPM_CUDA(c, cudaGetLastError());
        launches += 1 + tp.maxBouncePhoton;
        PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
        if ((int64_t)hc.deposits <= s.evCap) break;
        if (attempt > 0) return fail(c, PPPM_E_CAPACITY, "render_pass: photon update events overflow");
        s.evCap = (int64_t)(hc.deposits * 1.25) + 1024;
        PPPM_CUDA(c, s.ev.ensure((size_t)s.evCap * sizeof(ClassicEvent)));
        PPPM_CUDA(c, s.evSorted.ensure((size_t)s.evCap * sizeof(ClassicEvent)));
    }
    PPPM_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
    if (hc.undefinedEmit)
        return fail(c, PPPM_E_UNDEFINED, "render_pass: a photon draw fell past the env CDF (reference reads _pdf out of bounds)");
    if (hc.undefinedEye)
        return fail(c, PPPM_E_UNDEFINED, "render_pass: a path drew more than the 200 Halton dimensions (the reference aborts)");
    // render-point updates in photon order
    uint32_t* eh = s.evCount.as<uint32_t>();
    PPPM_CUDA(c, cudaMemsetAsync(eh, 0, (size_t)(np + 1) * 4, c->stream));
    const unsigned long long* evn = &ctr->deposits;
    kEvHist<<<blocksOf((int64_t)hc.deposits, 256), 256, 0, c->stream>>>(s.ev.as<ClassicEvent>(), evn, s.evCap, eh);
    PPPM_CUDA(c, exclusiveScan(eh, np, s.evCursor.as<uint32_t>(), s.evTmp.as<uint32_t>(), c->stream));
    kEvScatter<<<blocksOf((int64_t)hc.deposits, 256), 256, 0, c->stream>>>(s.ev.as<ClassicEvent>(), evn, s.evCap,
                                                                           s.evCursor.as<uint32_t>(),
                                                                           s.evSorted.as<ClassicEvent>());
    kClassicUpdate<<<blocksOf(np, 128), 128, 0, c->stream>>>(rp, np, eh, s.evSorted.as<ClassicEvent>(), rs.par.alpha);
    PPPM_CUDA(c, cudaGetLastError());
    launches += 6;
    PPPM_CUDA(c, cudaEventRecord(c->ev[4], c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->photons_traced = paths;
        stats->photons_stored = (int64_t)hc.deposits;  // render-point update events
        stats->photon_rays = (int64_t)hc.photonRays;
        stats->radius = irad;
        float ms;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[3]);
        stats->ms_eye = ms;
        cudaEventElapsedTime(&ms, c->ev[3], c->ev[2]);
        stats->ms_grid = ms;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[1]);
        stats->ms_photon = ms;
        stats->ms_bounce = ms;
        cudaEventElapsedTime(&ms, c->ev[1], c->ev[4]);
        stats->ms_gather = ms;
        stats->kernel_launches = launches;
        PassCounters he;
        PPPM_CUDA(c, cudaMemcpy(&he, ctr, sizeof(he), cudaMemcpyDeviceToHost));
        stats->eye_rays = (int64_t)he.eyeRays;
    }
    return PPPM_OK;
}

namespace {
__global__ void kHalton(HaltonDev hd, int stream, int count, int n, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count * n) return;
    out[i] = haltonValue(hd, stream, (unsigned long long)(i / n), i % n);
}
}  // namespace

int classicRead(pppm_ctx* c, float* out) {
    RenderState& rs = c->rs;
    const int64_t np = (int64_t)rs.cam.width * rs.cam.height;
    kClassicImage<<<blocksOf(np, 256), 256, 0, c->stream>>>(rpView(rs.classic), np, rs.accum.as<float>());
    PPPM_CUDA(c, cudaGetLastError());
    return PPPM_OK;
}

}  // namespace pppm

using namespace pppm;

// Halton(200, true, seed)::request values for requests 0 .. count-1, n
// numbers each, on the GPU (the sampler of classic PPM). No counterpart as
// a function in the reference; it checks the device radical inverse.
extern "C" int pppm_halton(pppm_ctx* c, uint32_t seed, int32_t count, int32_t n, double* out) {
    if (!c || count < 0 || n < 0 || n > 200 || (count * n > 0 && !out)) return fail(c, PPPM_E_ARG, "halton: bad arguments");
    if (count * n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    std::vector<uint16_t> perm;
    std::vector<int> primes, offs;
    int sum = 0;
    if (!haltonTables((int)seed + 1, &perm, &primes, &offs, &sum))
        return fail(c, PPPM_E_UNDEFINED, "halton: a permutation draws abs(INT_MIN)");
    PPPM_CUDA(c, c->stage[3].ensure(perm.size() * 2));
    PPPM_CUDA(c, c->stage[4].ensure(primes.size() * 4));
    PPPM_CUDA(c, c->stage[5].ensure(offs.size() * 4));
    PPPM_CUDA(c, cudaMemcpy(c->stage[3].p, perm.data(), perm.size() * 2, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(c->stage[4].p, primes.data(), primes.size() * 4, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(c->stage[5].p, offs.data(), offs.size() * 4, cudaMemcpyHostToDevice));
    void* dout;
    int r;
    if ((r = stageOut(c, out, (size_t)count * n * 8, 6, &dout))) return r;
    HaltonDev hd{c->stage[3].as<uint16_t>(), c->stage[4].as<int>(), c->stage[5].as<int>(), sum};
    kHalton<<<(count * n + 255) / 256, 256, 0, c->stream>>>(hd, (int)seed, count, n, (double*)dout);
    PPPM_CUDA(c, cudaGetLastError());
    if ((r = finishOut(c, out, dout, (size_t)count * n * 8))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}
