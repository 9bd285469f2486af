// Photon emission and bounce wavefront, eye paths, and the RNG tapes that
// reproduce the reference's per-thread XorShift streams.
#include <cstring>

#include "trace.h"

// Minimum resident blocks per SM for the traversal kernels (register cap
// 65536 / (128 * n)); overridable at build time.

namespace pppm {

// ------------------------------------------------------------------ jump-ahead (host)
namespace {

struct Gf2Mat {
    uint32_t col[128][4];
};

void gf2Apply(const Gf2Mat& m, const uint32_t in[4], uint32_t out[4]) {
    uint32_t r[4] = {0, 0, 0, 0};
    for (int j = 0; j < 128; j++)
        if ((in[j >> 5] >> (j & 31)) & 1u)
            for (int w = 0; w < 4; w++) r[w] ^= m.col[j][w];
    std::memcpy(out, r, sizeof(r));
}

void gf2Mul(const Gf2Mat& a, const Gf2Mat& b, Gf2Mat* c) {  // c = a * b (apply b first)
    Gf2Mat t;
    for (int j = 0; j < 128; j++) gf2Apply(a, b.col[j], t.col[j]);
    *c = t;
}

}  // namespace

void xorshiftJumpTables(std::vector<uint32_t>* tables, uint32_t stride) {
    // one XorShift step as a 128x128 GF(2) matrix
    Gf2Mat m;
    for (int j = 0; j < 128; j++) {
        XorShift x;
        for (int w = 0; w < 4; w++) x.s[w] = 0;
        x.s[j >> 5] = 1u << (j & 31);
        x.next();
        std::memcpy(m.col[j], x.s, 16);
    }
    // T = M^stride by square and multiply
    Gf2Mat t, p = m;
    bool first = true;
    for (uint32_t e = stride; e > 0; e >>= 1) {
        if (e & 1) {
            if (first) { t = p; first = false; } else gf2Mul(p, t, &t);
        }
        if (e > 1) gf2Mul(p, p, &p);
    }
    tables->assign((size_t)kJumpLevels * 128 * 4, 0u);
    Gf2Mat cur = t;
    for (int k = 0; k < kJumpLevels; k++) {
        std::memcpy(tables->data() + (size_t)k * 512, cur.col, sizeof(cur.col));
        gf2Mul(cur, cur, &cur);
    }
}

void xorshiftJumpHost(const std::vector<uint32_t>& tables, uint64_t tapes, XorShift* st) {
    for (int k = 0; k < kJumpLevels && tapes; k++, tapes >>= 1) {
        if (!(tapes & 1)) continue;
        Gf2Mat const* m = reinterpret_cast<const Gf2Mat*>(tables.data() + (size_t)k * 512);
        gf2Apply(*m, st->s, st->s);
    }
}

namespace {

unsigned blocksFor(int64_t n, int bs, int cap = 152 * 16) {
    const int64_t want = (n + bs - 1) / bs;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, cap));
}


// Canonical mode: an independent XorShift state per (seed, pass, path).
__device__ __forceinline__ void seedCanonical(uint32_t seed, int pass, uint64_t id, XorShift& x) {
    const uint32_t a = mix32(seed ^ 0x9e3779b9u * (uint32_t)(pass + 1));
    const uint32_t b = mix32((uint32_t)id ^ mix32((uint32_t)(id >> 32) + a));
    x.s[0] = mix32(a ^ b) | 1u;
    x.s[1] = mix32(b + 0x632be59bu);
    x.s[2] = mix32(a + 0x85157af5u + b);
    x.s[3] = mix32(b ^ 0xa54ff53au);
}

constexpr int kRun = 32;  // tapes generated sequentially per thread
// 1: the trace kernels stage the top BVH levels (85 nodes, 10.9 KB) in
// shared memory per block. 0: they read them through L1 like the rest of
// the tree; the shared memory this frees is L1 cache for the BVH (measured
// faster, 0 is the default).
#ifndef PPPM_TOP_SMEM
#define PPPM_TOP_SMEM 0
#endif
constexpr int kMaxEyeSegments = 4096;  // eye path segments before a path is cut (subsurface scenes)

// Start state of every photon tape and pixel tape of this pass. Stream s
// (one per reference OpenMP thread) draws, in order, ceil(P/N) photon tapes
// (ppm_probabilistic.cc:131-135) and then one tape per pixel of the rows
// y = s, s + N, ... (ppm_probabilistic.cc:213-228).
__global__ void kTapeStates(TraceParams tp, const uint32_t* __restrict__ streamStates, const uint32_t* __restrict__ jump,
                            int W, int H, uint32_t* __restrict__ photonStates, uint32_t* __restrict__ pixelStates) {
    const int N = tp.numStreams;
    const int64_t T = tp.taskPerThread;
    const int64_t maxRows = (H + N - 1) / N;
    const int64_t maxItems = T + maxRows * W;
    const int64_t runsPer = (maxItems + kRun - 1) / kRun;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < runsPer * N;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g / runsPer);
        const int64_t run = g % runsPer;
        const int64_t rows = s < H ? (H - 1 - s) / N + 1 : 0;
        const int64_t items = T + rows * W;
        const int64_t o = run * kRun;
        if (o >= items) continue;
        uint32_t st[4] = {streamStates[4 * s], streamStates[4 * s + 1], streamStates[4 * s + 2], streamStates[4 * s + 3]};
        uint64_t k = (uint64_t)o;
        for (int lvl = 0; k; lvl++, k >>= 1)
            if (k & 1) jumpApply(jump + (size_t)lvl * 512, st);
        XorShift x;
        x.s[0] = st[0]; x.s[1] = st[1]; x.s[2] = st[2]; x.s[3] = st[3];
        const int64_t end = min(o + kRun, items);
        for (int64_t j = o; j < end; j++) {
            uint32_t* dst;
            if (j < T) {
                dst = photonStates + 4 * ((int64_t)s * T + j);
            } else {
                const int64_t pj = j - T;
                const int64_t y = s + (int64_t)N * (pj / W), xx = pj % W;
                dst = pixelStates + 4 * (y * W + xx);
            }
            *reinterpret_cast<uint4*>(dst) = make_uint4(x.s[0], x.s[1], x.s[2], x.s[3]);
            for (int t = 0; t < 200; t++) x.next();
        }
    }
}

// Learned emission (canonical mode): one-sample MIS of the environment
// direction between the reference's cell draw (probability c) and the
// network's vMF mixture m. The density of the mixture in cell units is
//     p = c pdf[cell(d)] + (1 - c) q_m(d) 4 pi / 4096
// (cells are equal in solid angle and uniform inside), and the flux
// L(d) emitK / p is the reference's L(d) area / (pdf numPhotons) with p in
// place of pdf, so the photon set keeps the plain estimator's expectation.
// The cosine draw of the first direction is the reference's.
template <class TapeT>
__device__ bool emitPhotonMis(const EnvDev& e, TapeT& tp, const VmfMix& m, float c, float emitK, f3* emitDir, f3* dir,
                              f3* flux) {
    const float us = tp.popf();
    f3 d;
    int index;
    if (us < c) {
        d = envCellDraw(e, tp, &index);
        if (index >= 4096) return false;
    } else {
        const float u0 = tp.popf(), u1 = tp.popf(), u2 = tp.popf();
        d = vmfMixSample(m, u0, u1, u2);
        index = envCellOf(d);
    }
    const float pMix = c * (float)__ldg(&e.pdf[index]) + (1.0f - c) * vmfMixPdf(m, d) * (4.0f * kPiF / 4096.0f);
    const float s = (pMix > 0.0f && isfinite(pMix)) ? emitK / pMix : 0.0f;
    *flux = envLookup(e, d) * s;
    *emitDir = d;
    const float a0 = tp.popf();
    const float a1 = tp.popf();
    *dir = onHemisphere(-d, a1, a0);
    return true;
}

__device__ inline bool vmfMixFinite(const VmfMix& m) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kMlpLobes; k++) s += m.w[k] + m.mu[k][0] + m.mu[k][1] + m.mu[k][2] + m.kappa[k] + m.norm[k];
    return isfinite(s);
}

// Octahedral cell (2^bits per side, Morton order) of a direction.
__device__ __forceinline__ uint32_t octCell(const f3& v, int bits) {
    const float s = 1.0f / (fabsf(v.x) + fabsf(v.y) + fabsf(v.z));
    float u = v.x * s, w = v.y * s;
    if (v.z < 0.0f) {
        const float uu = (1.0f - fabsf(w)) * (u >= 0.0f ? 1.0f : -1.0f);
        w = (1.0f - fabsf(u)) * (w >= 0.0f ? 1.0f : -1.0f);
        u = uu;
    }
    const int m = (1 << bits) - 1;
    const uint32_t qu = (uint32_t)min(max(__float2int_rd((u + 1.0f) * 0.5f * (float)(m + 1)), 0), m);
    const uint32_t qw = (uint32_t)min(max(__float2int_rd((w + 1.0f) * 0.5f * (float)(m + 1)), 0), m);
    uint32_t r = 0;
    for (int b = 0; b < bits; b++) r |= (((qu >> b) & 1u) << (2 * b)) | (((qw >> b) & 1u) << (2 * b + 1));
    return r;
}

// Emission kinds, one kernel each so that the common one carries no other
// kind's registers: the environment with XorShift tapes, the same with the
// learned mixture (one-sample MIS), emissive triangles, permuted Halton.
enum EmitKind { kEmitEnv = 0, kEmitMis = 1, kEmitLights = 2, kEmitQmc = 3 };

template <int kKind>
__global__ void kPhotonEmit(TraceParams tp, EnvDev env, const uint32_t* __restrict__ photonStates,
                            PathState* __restrict__ queue, PassCounters* ctr, uint32_t* __restrict__ sortKeys,
                            uint32_t* __restrict__ sortHist) {
    const GuideView& gv = tp.guide;
    VmfMix mix;
    bool learned = false;
    if constexpr (kKind == kEmitMis) {
        vmfMixFromRaw(gv.emitRaw, &mix, gv.maxLogKappa);
        learned = vmfMixFinite(mix);  // a non-finite network output: the reference's sampling alone
    }
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < tp.numPaths;
         g += (int64_t)gridDim.x * blockDim.x) {
        f3 d, dir, flux;
        bool ok;
        PathState p;
        double org[3];
        const bool fromLight = kKind == kEmitLights;
        if constexpr (kKind == kEmitLights) {
            // emissive triangles: the scene's light instead of the environment
            Tape tape;
            tape.pos = 0;
            tape.scramble = tp.mode == PPPM_MODE_CANONICAL;
            if (tp.mode == PPPM_MODE_COMPAT) {
                const uint4 s = *reinterpret_cast<const uint4*>(photonStates + 4 * g);
                tape.x.s[0] = s.x; tape.x.s[1] = s.y; tape.x.s[2] = s.z; tape.x.s[3] = s.w;
            } else {
                seedCanonical(tp.seed, tp.pass, (uint64_t)g, tape.x);
            }
            ok = emitFromLights(env, tape, org, &dir, &flux, &d);
            storeTape(tape, p);
        } else if constexpr (kKind == kEmitQmc) {
            // photon round i of thread s draws sample i of the pass from
            // sampler s (tracePhotons, ppm_probabilistic.cc:131-135)
            const int s = (int)(g / tp.taskPerThread);
            HaltonTape tape{&tp.halton, s, qmcIndex(tp, s, g % tp.taskPerThread), 0, false};
            ok = emitPhoton(env, tape, tp.numPhotons, &d, &dir, &flux, false);
            if (tape.over) ok = false;
            storeTape(tape, p);
        } else {
            Tape tape;
            tape.pos = 0;
            tape.scramble = tp.mode == PPPM_MODE_CANONICAL;
            if (tp.mode == PPPM_MODE_COMPAT) {
                const uint4 s = *reinterpret_cast<const uint4*>(photonStates + 4 * g);
                tape.x.s[0] = s.x; tape.x.s[1] = s.y; tape.x.s[2] = s.z; tape.x.s[3] = s.w;
            } else {
                seedCanonical(tp.seed, tp.pass, (uint64_t)g, tape.x);
            }
            if constexpr (kKind == kEmitMis)
                ok = learned ? emitPhotonMis(env, tape, mix, gv.emitFloor, gv.emitK, &d, &dir, &flux)
                             : emitPhoton(env, tape, tp.numPhotons, &d, &dir, &flux, tp.sssPass != 0);
            else
                ok = emitPhoton(env, tape, tp.numPhotons, &d, &dir, &flux, tp.sssPass != 0);
            storeTape(tape, p);
        }
        if (!ok) atomicAdd(&ctr->undefinedEmit, 1ull);
        if (fromLight) {
            p.ox = org[0]; p.oy = org[1]; p.oz = org[2];
        } else {
            p.ox = 50.0 * (double)d.x;  // R * dir with R = 50 (envmap.cc:63,85)
            p.oy = 50.0 * (double)d.y;
            p.oz = 50.0 * (double)d.z;
        }
        p.dx = dir.x; p.dy = dir.y; p.dz = dir.z;
        p.fx = ok ? flux.x : 0.f; p.fy = ok ? flux.y : 0.f; p.fz = ok ? flux.z : 0.f;
        p.id = (int)g;
        p.bounce = 0;
        p.pad[0] = -1;  // no pending bounce record
        p.pad[1] = 0;
        if (tp.guided && gv.rec && ok &&
            mix32((uint32_t)g * 0x85EBCA77u + (uint32_t)tp.pass * 0xC2B2AE3Du + 0x27D4EB2Fu) % gv.recEvery == 0) {
            // emission record: the network's emission input and the direction;
            // its weight collects the importance of the path's deposits
            const unsigned long long r = atomicAdd(gv.recCount, 1ull);
            if ((int64_t)r < gv.recCap) {
                MlpRecord rec;
                rec.px = gv.epx; rec.py = gv.epy; rec.pz = gv.epz;
                rec.w = 0.0f;
                rec.nx = rec.ny = rec.nz = 0.0f;
                rec.pad0 = 0.0f;
                rec.dx = d.x; rec.dy = d.y; rec.dz = d.z;
                rec.pad1 = 0.0f;
                gv.rec[r] = rec;
                p.pad[1] = (int)((r + 1) << kPathEmitRecShift);
            }
        }
        queue[g] = p;
        if (sortKeys) {
            const uint32_t kd = octCell(dir, kSortDirBits), ke = octCell(d, kSortEnvBits);
            const uint32_t key = PPPM_SORT_ENV_HIGH ? (ke << (2 * kSortDirBits)) | kd : (kd << (2 * kSortEnvBits)) | ke;
            sortKeys[g] = key;
            atomicAdd(&sortHist[key], 1u);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctr->queue[0] = (unsigned long long)tp.numPaths;
        ctr->queue[1] = 0;
        ctr->queue[2] = 0;
    }
}


// The hit of a photon path at triangle slot `slot`, distance `best`
// (ppm_probabilistic.cc:150-193; subsurface pass: subsurface_integrator.cc:
// 262-320): three draws from the path's tape, the deposit (store, da, db) on
// Lambertian (subsurface pass: BSSRDF) surfaces, Russian roulette, and the
// next ray in p. alive turns false when the path ends here.
// The ray is given as (ox, oy, oz, din); the next ray leaves through hp and
// nd. p supplies and receives everything else of the path (flux, tape,
// bounce, records): callers that keep the ray in their traversal state do
// not hold a second copy of it in p.
template <bool kSss, class TapeT = Tape>
__device__ __forceinline__ void photonHitRay(const TraceParams& tp, const SceneView& sc, PathState& p, int slot,
                                             double best, double ox, double oy, double oz, const f3 din, bool& alive,
                                             bool& store, float4& da, float4& db, double* hp, f3& nd) {
    TapeT tape;
    loadTape(tp, p, tape);
    const auto r0 = tape.draw(), r1 = tape.draw(), r2 = tape.draw();
    const float4 a = sc.tris[3 * slot], b = sc.tris[3 * slot + 1], c = sc.tris[3 * slot + 2];
    const int tid = __float_as_int(a.w);
    const DevMaterial& m = sc.mats[sc.matId[tid]];
    hitPosition(ox, oy, oz, din.x, din.y, din.z, best, hp);
    const f3 nrm = triNormalF(a, b, c);
    const f3 on = dot(nrm, din) < 0.0f ? nrm : -nrm;
    f3 flux = {p.fx, p.fy, p.fz};
    const f3 refl = {m.refl[0], m.refl[1], m.refl[2]};
    if (kSss) {
        if (kSss && (m.type & PPPM_BSDF_BSSRDF)) {
            store = true;
            da = make_float4(__double2float_rn(hp[0]), __double2float_rn(hp[1]), __double2float_rn(hp[2]),
                             __uint_as_float(packNormal(on)));
            db = make_float4(flux.x, flux.y, flux.z, __int_as_float(p.id));
            const float prob = (flux.x + flux.y + flux.z) / 3.0f;
            if (!(r0.f() < prob)) alive = false;  // rands[0] >= probability: break
        }
        if (alive) {
            const float pdf = bsdfSample(m, din, nrm, r1.u, r2.u, &nd);
            flux = flux * refl * (1.0f / pdf);
        }
    } else if (m.type & PPPM_BSDF_LAMBERTIAN) {
        store = true;
        da = make_float4(__double2float_rn(hp[0]), __double2float_rn(hp[1]), __double2float_rn(hp[2]),
                         __uint_as_float(packNormal(on)));
        db = make_float4(flux.x, flux.y, flux.z, __int_as_float(p.id));
        const int er = p.pad[1] >> kPathEmitRecShift;
        if (tp.guided && er > 0 && tp.guide.imp) {
            // emission record: importance-weighted flux of this deposit
            const int v = impVoxel(tp.guide, da.x, da.y, da.z);
            if (v >= 0)
                tp.guide.rec[er - 1].w +=
                    (0.2126f * flux.x + 0.7152f * flux.y + 0.0722f * flux.z) * __ldg(&tp.guide.imp[v]);
        }
        if (r0.lt(m.rrCeil, m.rr_photon)) {  // rands[0] < probability
            if (tp.guided && tp.guide.guideBounces) {
                nd = on;  // kGuideResolve draws the direction around the normal
                p.pad[1] |= kPathNeedsDir;
            } else {
                bsdfSample(m, din, on, r1.u, r2.u, &nd);
            }
            flux = flux * refl * m.invRr;
        } else {
            alive = false;
        }
    } else {
        const float pdf = bsdfSample(m, din, on, r0.u, r1.u, &nd);
        flux = flux * refl * (1.0f / pdf);
    }
    p.fx = flux.x; p.fy = flux.y; p.fz = flux.z;
    storeTape(tape, p);
    p.bounce += 1;
}

// photonHitRay for a path that carries its ray in p.
template <bool kSss, class TapeT = Tape>
__device__ __forceinline__ void photonHit(const TraceParams& tp, const SceneView& sc, PathState& p, int slot, double best,
                                          bool& alive, bool& store, float4& da, float4& db) {
    double hp[3];
    f3 nd;
    photonHitRay<kSss, TapeT>(tp, sc, p, slot, best, p.ox, p.oy, p.oz, mk(p.dx, p.dy, p.dz), alive, store, da, db, hp,
                              nd);
    p.ox = hp[0]; p.oy = hp[1]; p.oz = hp[2];
    p.dx = nd.x; p.dy = nd.y; p.dz = nd.z;
}

// Every bounce of every emitted photon path in one launch. Warps stay
// resident and keep their lanes busy: the warp advances its lanes'
// traversals together until at least tp.refill of them have found their hit
// (or all have), shades those (photonHit: deposit, roulette, next ray), and
// lanes whose path ended take the next path of the emitted queue (one
// atomic per warp). A path's own random numbers and traversal are those of
// the per-bounce kernels; only the order in which paths are processed and
// deposits appended changes. kFixed: the default refill and exact-test
// thresholds as constants (the tuned values are read from tp otherwise).
template <bool kSss, bool kFixed>
__global__ void __launch_bounds__(128, PPPM_TRACE_MINBLOCKS) kPhotonPersistent(TraceParams tp, SceneView sc,
                                                                               const PathState* __restrict__ in,
                                                                               int64_t maxPaths, float4* __restrict__ dep,
                                                                               int64_t depCap, PassCounters* ctr,
                                                                               const uint32_t* __restrict__ perm) {
    __shared__ int order[128];
#if PPPM_TOP_SMEM
    __shared__ QNode sTopBuf[kTopNodes];
    QNode* sTop = sTopBuf;
#else
    QNode* sTop = nullptr;  // top levels through L1 like the rest of the tree
#endif
    const int64_t n = min((int64_t)ctr->queue[0], maxPaths);
    loadOrderTable(order);
#if PPPM_TOP_SMEM
    loadTopNodes(sTop, sc.nodes, sc.numNodes);
#endif
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    PathState p;
    WarpTrav s;
    s.sp = 0;
    s.ncand = 0;
    bool has = false;
    int traced = 0, visits = 0, tests = 0;
    for (;;) {
        // lanes without a path take the next ones of the queue
        const unsigned empty = __ballot_sync(0xffffffffu, !has);
        if (empty) {
            const int leader = __ffs(empty) - 1;
            unsigned long long b = 0;
            if (lane == leader) b = atomicAdd(&ctr->fetched, (unsigned long long)__popc(empty));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (!has) {
                const int64_t i = (int64_t)(b + __popc(empty & lt));
                if (i < n) {
                    p = in[perm ? (int64_t)perm[i] : i];
                    has = p.bounce < tp.maxBouncePhoton && fmaxf(p.fx, fmaxf(p.fy, p.fz)) > 0.0f;
                    if (has) s.begin(sc.rootCode, p.ox, p.oy, p.oz, p.dx, p.dy, p.dz);
                }
            }
            // a path that was dead on arrival leaves its lane empty: refill
            // again while the queue lasts
            if (__any_sync(0xffffffffu, !has) && b + __popc(empty) < (unsigned long long)n) continue;
        }
        if (!__any_sync(0xffffffffu, has)) break;
        warpTravRun(s, has, kFixed ? kRefill : tp.refill, sc.nodes, sc.tris, order, sTop, &visits, &tests, sc.triE,
                    kFixed ? kExactBatch : tp.exactBatch);
        const bool fin = has && s.done();
        bool store = false;
        float4 da, db;
        if (fin) {
            traced++;
            bool alive = true;
            if (s.hit < 0) {
                alive = false;
            } else {
                // the ray lives in the traversal state only
                double hp[3];
                f3 nd;
                photonHitRay<kSss>(tp, sc, p, s.hit, s.best, s.odx, s.ody, s.odz, mk(s.dx, s.dy, s.dz), alive, store,
                                   da, db, hp, nd);
                if (alive) alive = p.bounce < tp.maxBouncePhoton && fmaxf(p.fx, fmaxf(p.fy, p.fz)) > 0.0f;
                if (alive) s.begin(sc.rootCode, hp[0], hp[1], hp[2], nd.x, nd.y, nd.z);
            }
            if (!alive) has = false;
        }
        const unsigned long long di = warpAppend(store, &ctr->deposits);
        if (store && (int64_t)di < depCap) {
            dep[2 * di] = da;
            dep[2 * di + 1] = db;
        }
    }
    const unsigned nt = __reduce_add_sync(0xffffffffu, (unsigned)traced);
    if (lane == 0 && nt) atomicAdd(&ctr->photonRays, (unsigned long long)nt);
    if (tp.countTraversal) {
        const unsigned nv = __reduce_add_sync(0xffffffffu, (unsigned)visits);
        const unsigned nx = __reduce_add_sync(0xffffffffu, (unsigned)tests);
        if (lane == 0) {
            atomicAdd(&ctr->nodeVisits[0], (unsigned long long)nv);
            atomicAdd(&ctr->triTests[0], (unsigned long long)nx);
        }
    }
}

// One bounce of every live photon path (ppm_probabilistic.cc:150-193):
// closest hit, three draws, deposit + Russian roulette on Lambertian
// surfaces, BSDF sampling elsewhere. Survivors are compacted into `out`
// with one atomic per warp; queue lengths rotate through ctr->queue[b % 3].
// kSss: the photon pass of SubsurfaceIntegrator::buildPhotonMap
// (subsurface_integrator.cc:240-327) instead: records only on BSSRDF
// surfaces, Russian roulette there on the mean flux, and every BSDF sampled
// with the geometric normal and draws 1, 2.
// kTail: the remaining bounces of the queue in one launch. The few paths
// left after the first bounces are long chains (inside refractive and
// mirrored geometry) that leave most of a per-bounce launch idle; here each
// warp carries its paths to the end (no queue output, `out` unused).
template <bool kSss, bool kTail, class TapeT = Tape>
__global__ void __launch_bounds__(128, PPPM_TRACE_MINBLOCKS) kPhotonBounce(TraceParams tp, SceneView sc, int bounce, const PathState* __restrict__ in,
                                                     PathState* __restrict__ out, int64_t maxPaths,
                                                     float4* __restrict__ dep, int64_t depCap, PassCounters* ctr) {
    __shared__ int order[128];
#if PPPM_TOP_SMEM
    __shared__ QNode sTopBuf[kTopNodes];
    QNode* sTop = sTopBuf;
#else
    QNode* sTop = nullptr;  // top levels through L1 like the rest of the tree
#endif
    const int qi = bounce % 3, qo = (bounce + 1) % 3, qz = (bounce + 2) % 3;
    const int64_t n = min((int64_t)ctr->queue[qi], maxPaths);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr->queue[qz] = 0;
    // the grid is sized for the first bounce; blocks past the live paths of
    // later bounces leave before staging anything (uniform per block)
    if ((int64_t)blockIdx.x * blockDim.x >= n) return;
    loadOrderTable(order);
#if PPPM_TOP_SMEM
    loadTopNodes(sTop, sc.nodes, sc.numNodes);
#endif
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool alive = false, store = false;
        PathState p;
        p.ox = p.oy = p.oz = 0.0;
        p.dx = p.dy = 0.f;
        p.dz = 1.f;
        float4 da, db;
        if (i < n) {
            p = in[i];
            alive = p.bounce < tp.maxBouncePhoton && fmaxf(p.fx, fmaxf(p.fy, p.fz)) > 0.0f;
        }
        int traced = 0, visits = 0, tests = 0;
        do {
        double best;
        const int slot = traverseExactWarp(sc.nodes, sc.tris, sc.rootCode, alive, p.ox, p.oy, p.oz, p.dx, p.dy, p.dz,
                                           order, sTop, &best, &visits, &tests, sc.triE, tp.exactBatch);
        if (alive) {
            traced++;
            if (tp.guided && p.pad[0] >= 0) {
                // training record of the draw that led here: weight cos I(y) / p
                float V = 0.0f;
                if (slot >= 0 && tp.guide.imp) {
                    double y[3];
                    hitPosition(p.ox, p.oy, p.oz, p.dx, p.dy, p.dz, best, y);
                    const int v = impVoxel(tp.guide, (float)y[0], (float)y[1], (float)y[2]);
                    if (v >= 0) V = __ldg(&tp.guide.imp[v]);
                }
                MlpRecord& r = tp.guide.rec[p.pad[0]];
                r.w = r.pad0 * V;
                p.pad[0] = -1;
            }
            if (slot < 0) {
                alive = false;
            } else {
                photonHit<kSss, TapeT>(tp, sc, p, slot, best, alive, store, da, db);
                if (kTail && alive)
                    alive = p.bounce < tp.maxBouncePhoton && fmaxf(p.fx, fmaxf(p.fy, p.fz)) > 0.0f;
            }
        }
        const unsigned long long di = warpAppend(store, &ctr->deposits);
        if (store && (int64_t)di < depCap) {
            dep[2 * di] = da;
            dep[2 * di + 1] = db;
        }
        store = false;
        } while (kTail && __any_sync(0xffffffffu, alive));
        if (!kTail) {
            const unsigned long long oi = warpAppend(alive, &ctr->queue[qo]);
            if (alive) out[oi] = p;
        }
        const unsigned nt = __reduce_add_sync(0xffffffffu, (unsigned)traced);
        if ((threadIdx.x & 31) == 0 && nt) atomicAdd(&ctr->photonRays, (unsigned long long)nt);
        if (tp.countTraversal) {
            const unsigned nv = __reduce_add_sync(0xffffffffu, (unsigned)visits);
            const unsigned nx = __reduce_add_sync(0xffffffffu, (unsigned)tests);
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&ctr->nodeVisits[0], (unsigned long long)nv);
                atomicAdd(&ctr->triTests[0], (unsigned long long)nx);
            }
        }
    }
}


// Eye paths of ProgressivePhotonMappingProb::radiance (ppm_probabilistic.cc:
// 236-344) without BSSRDF: tail recursion through specular and refractive
// surfaces, Russian roulette after 3 bounces, a gather query at the first
// Lambertian hit, the env map on a miss. Environment terms go straight into
// the accumulation buffer; queries are compacted with one atomic per warp.
// kSss: the scene has BSSRDF materials (the subsurface branches of radiance
// are compiled in only then).
// kPT: PathTracing::radiance (path_tracing.cc:137-198) instead: a Lambertian
// hit continues with the BSDF sample (pdf 1) like every other surface; the
// rest of the recursion is the same.
#ifndef PPPM_EYE_TILES
#define PPPM_EYE_TILES 1
#endif
constexpr bool kEyeTiles = PPPM_EYE_TILES != 0;

template <bool kSss, bool kPT, class TapeT = Tape>
__global__ void __launch_bounds__(128, PPPM_EYE_MINBLOCKS) kEyeTrace(TraceParams tp, SceneView sc, EnvDev env, CameraDev cam,
                                                 OctView oct, const uint32_t* __restrict__ pixelStates,
                                                 float* __restrict__ accum, float4* __restrict__ queries,
                                                 float4* __restrict__ sssQ, int64_t sssCap, PassCounters* ctr) {
    __shared__ int order[128];
#if PPPM_TOP_SMEM
    __shared__ QNode sTopBuf[kTopNodes];
    QNode* sTop = sTopBuf;
#else
    QNode* sTop = nullptr;  // top levels through L1 like the rest of the tree
#endif
    loadOrderTable(order);
#if PPPM_TOP_SMEM
    loadTopNodes(sTop, sc.nodes, sc.numNodes);
#endif
    const int64_t np = (int64_t)cam.w * cam.h;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // a block takes a 16x8 pixel tile, each warp an 8x4 quarter of it, so
    // the lanes' secondary rays leave nearby points of nearby pixels
    const int tilesX = (cam.w + 15) >> 4;
    const int64_t nt = (int64_t)tilesX * ((cam.h + 7) >> 3) * 128;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < (kEyeTiles ? nt : np); base += stride) {
        int64_t pix = base + threadIdx.x;
        if (kEyeTiles) {
            const int64_t tile = base >> 7;
            const int wv = threadIdx.x >> 5, ln = threadIdx.x & 31;
            const int x = (int)(tile % tilesX) * 16 + (wv & 1) * 8 + (ln & 7);
            const int y = (int)(tile / tilesX) * 8 + (wv >> 1) * 4 + (ln >> 3);
            pix = (x < cam.w && y < cam.h) ? (int64_t)y * cam.w + x : np;
        }
        bool query = false;
        float4 q0, q1, q2;
        int traced = 0, visits = 0, tests = 0;
        // every lane of the warp stays in the bounce loop until all paths end
        // (the traversal is warp-cooperative)
        bool alive = pix < np;
        TapeT tape;
        if constexpr (TapeT::kExact32) {
            tape.pos = 0;
            tape.scramble = tp.mode == PPPM_MODE_CANONICAL;
            tape.x.s[0] = tape.x.s[1] = tape.x.s[2] = tape.x.s[3] = 1u;
        } else {
            tape = HaltonTape{&tp.halton, 0, 0, 0, false};
        }
        f3 d = {0.f, 0.f, 1.f};
        double o[3] = {cam.ex, cam.ey, cam.ez};
        f3 w = {1.f, 1.f, 1.f}, L = {0.f, 0.f, 0.f};
        if (alive) {
            const int x = (int)(pix % cam.w), y = (int)(pix / cam.w);
            if constexpr (!TapeT::kExact32) {
                // pixel x of the stream's k-th row: sample taskPerThread + k w + x
                // of sampler y % N (traceRays, ppm_probabilistic.cc:214-229)
                const int s = y % tp.numStreams;
                tape.stream = s;
                tape.index = qmcIndex(tp, s, tp.taskPerThread + (int64_t)(y / tp.numStreams) * cam.w + x);
            } else if (tp.mode == PPPM_MODE_COMPAT || tp.mode == PPPM_MODE_PATH_TRACING) {
                const uint4 s = *reinterpret_cast<const uint4*>(pixelStates + 4 * pix);
                tape.x.s[0] = s.x; tape.x.s[1] = s.y; tape.x.s[2] = s.z; tape.x.s[3] = s.w;
            } else {
                seedCanonical(tp.seed, tp.pass, (uint64_t)tp.numPaths + (uint64_t)pix, tape.x);
            }
            const float px = (float)x + tape.popf() - 0.5f;
            const float py = (float)y + tape.popf() - 0.5f;
            cameraRay(cam, px, py, &d);
        }
        const bool onImage = alive;
        // bnc: the reference's `bounces` argument, which the Fresnel
        // reflection of a refractive BSSRDF surface passes on unchanged
        int bnc = 0;
        int iter = 0;
        while (__any_sync(0xffffffffu, alive)) {
            // Fresnel reflections that keep `bnc` draw 3 numbers each, so a
            // compat tape ends them after 66; the cap bounds canonical paths
            if (kSss && alive && ++iter > kMaxEyeSegments) {
                atomicAdd(&ctr->undefinedEye, 1ull);
                alive = false;
            }
            const bool doTrace = alive && bnc < tp.maxBounceEye;
            if (alive && !doTrace) {
                L = L + w * envLookup(env, d);
                alive = false;
            }
            double best;
            const int slot = traverseExactWarp(sc.nodes, sc.tris, sc.rootCode, doTrace, o[0], o[1], o[2], d.x, d.y,
                                               d.z, order, sTop, &best, &visits, &tests, sc.triE, tp.exactBatch);
            if (!doTrace) continue;
            traced++;
            if (slot < 0) {
                L = L + w * envLookup(env, d);
                alive = false;
                continue;
            }
            const auto r0 = tape.draw(), r1 = tape.draw(), r2 = tape.draw();
            const float4 a = sc.tris[3 * slot], bb = sc.tris[3 * slot + 1], c = sc.tris[3 * slot + 2];
            const DevMaterial& m = sc.mats[sc.matId[__float_as_int(a.w)]];
            double hp[3];
            hitPosition(o[0], o[1], o[2], d.x, d.y, d.z, best, hp);
            const f3 nrm = triNormalF(a, bb, c);
            // an emissive surface seen from its front side (no counterpart in
            // the reference, which has no emitters)
            if (m.emissive && dot(nrm, d) < 0.0f) L = L + w * mk(m.emit[0], m.emit[1], m.emit[2]);
            float roul = m.roulette;
            if (bnc >= 3) {
                // rands[0] > roulette: the path ends and contributes nothing more
                if (r0.gt(m.roulFloor, (double)m.roulette)) {
                    alive = false;
                    continue;
                }
            } else {
                roul = 1.0f;
            }
            const f3 refl = {m.refl[0], m.refl[1], m.refl[2]};
            if (kSss && (m.type & PPPM_BSDF_BSSRDF)) {
                // ppm_probabilistic.cc:273-298; reflect probability 0.25 + 0.5 * 0.5
                const float hx = __double2float_rn(hp[0]), hy = __double2float_rn(hp[1]), hz = __double2float_rn(hp[2]);
                bool sss = false;
                f3 sssAdd;
                if (m.type & PPPM_BSDF_REFRACTION) {
                    const FresnelSplit s = fresnelSplit(d, nrm, dot(nrm, d) < 0.0f);
                    o[0] = hp[0]; o[1] = hp[1]; o[2] = hp[2];
                    if (s.total) {
                        d = s.rdir;
                        bnc++;
                    } else if (r1.lt(0x80000000ull, 0.5)) {  // rands[1] < 0.5: reflect, same bounce count
                        w = w * refl * (s.Re / 0.5f);
                        d = s.rdir;
                    } else {  // transmit: diffuse subsurface radiance
                        sssAdd = w * (s.Tr / 0.5f);
                        sss = true;
                        alive = false;
                    }
                } else {
                    sssAdd = w * 0.5f;
                    sss = true;
                }
                if (sss) {
                    // deferred to kSubsurfaceGather (one coherent pass over the
                    // octree); evaluated here only when the queue is full
                    const unsigned long long si = atomicAdd(&ctr->sssQueries, 1ull);
                    if ((int64_t)si < sssCap) {
                        sssQ[2 * si] = make_float4(hx, hy, hz, __int_as_float((int)pix));
                        sssQ[2 * si + 1] = make_float4(sssAdd.x, sssAdd.y, sssAdd.z,
                                                       __int_as_float(sc.matId[__float_as_int(a.w)]));
                    } else {
                        L = L + sssAdd * subsurfaceIrradiance(oct, m.dip, hx, hy, hz, nullptr);
                    }
                    sss = false;
                }
                if (m.type & PPPM_BSDF_REFRACTION) continue;
            }
            if (!kPT && (m.type & PPPM_BSDF_LAMBERTIAN)) {
                const f3 on = dot(nrm, d) < 0.0f ? nrm : -nrm;
                const f3 wq = w * refl * (1.0f / roul);
                q0 = make_float4(__double2float_rn(hp[0]), __double2float_rn(hp[1]), __double2float_rn(hp[2]),
                                 __int_as_float((int)pix));
                // .w: the specular/refractive bounces before this hit and the
                // hit triangle's id (int bits), for parity checks of single
                // hit points; the gathers read neither
                q1 = make_float4(on.x, on.y, on.z, __int_as_float(bnc));
                q2 = make_float4(wq.x, wq.y, wq.z, a.w);
                query = true;
                alive = false;
                continue;
            }
            f3 nd;
            const float pdf = bsdfSample(m, d, nrm, r1.u, r2.u, &nd);
            w = w * refl * (1.0f / (pdf * roul));
            o[0] = hp[0]; o[1] = hp[1]; o[2] = hp[2];
            d = nd;
            bnc++;
        }
        // a compat tape holds 200 numbers (ppm_probabilistic.cc:222); the
        // reference aborts when a path pops more
        if ((tp.mode == PPPM_MODE_COMPAT || tp.mode == PPPM_MODE_PATH_TRACING) && tape.exhausted())
            atomicAdd(&ctr->undefinedEye, 1ull);
        if (onImage) {
            accum[3 * pix] += L.x;
            accum[3 * pix + 1] += L.y;
            accum[3 * pix + 2] += L.z;
        }
        const unsigned long long qi = warpAppend(query, &ctr->queries);
        if (query) {
            queries[3 * qi] = q0;
            queries[3 * qi + 1] = q1;
            queries[3 * qi + 2] = q2;
        }
        const unsigned nt = __reduce_add_sync(0xffffffffu, (unsigned)traced);
        if ((threadIdx.x & 31) == 0 && nt) atomicAdd(&ctr->eyeRays, (unsigned long long)nt);
        if (tp.countTraversal) {
            const unsigned nv = __reduce_add_sync(0xffffffffu, (unsigned)visits);
            const unsigned nx = __reduce_add_sync(0xffffffffu, (unsigned)tests);
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&ctr->nodeVisits[1], (unsigned long long)nv);
                atomicAdd(&ctr->triTests[1], (unsigned long long)nx);
            }
        }
    }
}

// The subsurface radiance queued by the eye pass: SubsurfaceIntegrator::
// irradiance at each query times its path weight, added to the pixel.
__global__ void __launch_bounds__(128) kSubsurfaceGather(OctView oct, const DevMaterial* __restrict__ mats,
                                                         const float4* __restrict__ q, const unsigned long long* count,
                                                         int64_t cap, float* __restrict__ accum,
                                                         unsigned long long* visits) {
    const int64_t n = min((int64_t)*count, cap);
    int v = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = q[2 * i], b = q[2 * i + 1];
        const DipoleDev& dip = mats[__float_as_int(b.w)].dip;
        const f3 irr = subsurfaceIrradiance(oct, dip, a.x, a.y, a.z, visits ? &v : nullptr);
        const int64_t px = __float_as_int(a.w);
        atomicAdd(&accum[3 * px], b.x * irr.x);
        atomicAdd(&accum[3 * px + 1], b.y * irr.y);
        atomicAdd(&accum[3 * px + 2], b.z * irr.z);
    }
    if (visits) {
        const unsigned t = __reduce_add_sync(0xffffffffu, (unsigned)v);
        if ((threadIdx.x & 31) == 0 && t) atomicAdd(visits, (unsigned long long)t);
    }
}

__global__ void kStreamCounts(const float4* __restrict__ dep, const unsigned long long* count, int64_t cap, int64_t tpt,
                              int N, unsigned long long* perStream) {
    extern __shared__ unsigned long long hist[];
    for (int s = threadIdx.x; s < N; s += blockDim.x) hist[s] = 0;
    __syncthreads();
    const int64_t n = min((int64_t)*count, cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int id = __float_as_int(dep[2 * i + 1].w);
        atomicAdd(&hist[min((int64_t)id / tpt, (int64_t)N - 1)], 1ull);
    }
    __syncthreads();
    for (int s = threadIdx.x; s < N; s += blockDim.x)
        if (hist[s]) atomicAdd(&perStream[s], hist[s]);
}

}  // namespace

cudaError_t launchTapeStates(const TraceParams& tp, const uint32_t* streamStates, const uint32_t* jump, int width,
                             int height, uint32_t* photonStates, uint32_t* pixelStates, cudaStream_t st) {
    const int64_t maxRows = (height + tp.numStreams - 1) / tp.numStreams;
    const int64_t runs = ((tp.taskPerThread + maxRows * width + kRun - 1) / kRun) * tp.numStreams;
    kTapeStates<<<blocksFor(runs, 128, 152 * 64), 128, 0, st>>>(tp, streamStates, jump, width, height, photonStates,
                                                                pixelStates);
    return cudaGetLastError();
}

cudaError_t launchPhotonEmit(const TraceParams& tp, const EnvDev& env, const uint32_t* photonStates, PathState* queue,
                             PassCounters* ctr, cudaStream_t st, const PhotonSort* sort) {
    // the kernel's own order of precedence: lights, Halton, then XorShift
    // tapes with the learned mixture when the network has an output
    const unsigned blocks = blocksFor(tp.numPaths, 256);
    uint32_t* keys = sort ? sort->keys : nullptr;
    uint32_t* hist = sort ? sort->hist : nullptr;
    if (env.numLights > 0)
        kPhotonEmit<kEmitLights><<<blocks, 256, 0, st>>>(tp, env, photonStates, queue, ctr, keys, hist);
    else if (tp.qmc)
        kPhotonEmit<kEmitQmc><<<blocks, 256, 0, st>>>(tp, env, photonStates, queue, ctr, keys, hist);
    else if (tp.guided && tp.guide.emitRaw != nullptr)
        kPhotonEmit<kEmitMis><<<blocks, 256, 0, st>>>(tp, env, photonStates, queue, ctr, keys, hist);
    else
        kPhotonEmit<kEmitEnv><<<blocks, 256, 0, st>>>(tp, env, photonStates, queue, ctr, keys, hist);
    return cudaGetLastError();
}

namespace {
__global__ void kPathOrder(const uint32_t* __restrict__ keys, uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm,
                           int64_t n) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
        perm[atomicAdd(&cursor[keys[g]], 1u)] = (uint32_t)g;
}

__global__ void kPathMove(const uint32_t* __restrict__ keys, uint32_t* __restrict__ cursor,
                          const PathState* __restrict__ from, PathState* __restrict__ to, int64_t n) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
        to[atomicAdd(&cursor[keys[g]], 1u)] = from[g];
}
}  // namespace

cudaError_t photonSortPaths(const PhotonSort& sort, int64_t paths, cudaStream_t st, const PathState* from,
                            PathState* moveTo) {
    cudaError_t e = exclusiveScan(sort.hist, kPhotonSortBins, sort.cursor, sort.tmp, st);
    if (e != cudaSuccess) return e;
    if (moveTo)
        kPathMove<<<blocksFor(paths, 256), 256, 0, st>>>(sort.keys, sort.cursor, from, moveTo, paths);
    else
        kPathOrder<<<blocksFor(paths, 256), 256, 0, st>>>(sort.keys, sort.cursor, sort.perm, paths);
    return cudaGetLastError();
}

cudaError_t launchPhotonBounce(const TraceParams& tp, const SceneView& sc, int bounce, const PathState* in,
                               PathState* out, int64_t maxPaths, float4* deposits, int64_t depositCap,
                               PassCounters* ctr, cudaStream_t st) {
    const unsigned blocks = blocksFor(maxPaths, 128, 152 * tp.bouncePerSm);
    if (tp.sssPass)
        kPhotonBounce<true, false><<<blocks, 128, 0, st>>>(tp, sc, bounce, in, out, maxPaths, deposits, depositCap, ctr);
    else if (tp.qmc)
        kPhotonBounce<false, false, HaltonTape><<<blocks, 128, 0, st>>>(tp, sc, bounce, in, out, maxPaths, deposits,
                                                                         depositCap, ctr);
    else
        kPhotonBounce<false, false><<<blocks, 128, 0, st>>>(tp, sc, bounce, in, out, maxPaths, deposits, depositCap, ctr);
    return cudaGetLastError();
}

cudaError_t launchPhotonPersistent(const TraceParams& tp, const SceneView& sc, const PathState* in, int64_t maxPaths,
                                   float4* deposits, int64_t depositCap, PassCounters* ctr, cudaStream_t st,
                                   const uint32_t* perm) {
    // resident warps only: every block stays until the queue is drained
    const unsigned blocks = 152 * std::max(1, std::min(tp.bouncePerSm, PPPM_TRACE_MINBLOCKS));
    const bool fixed = tp.refill == kRefill && tp.exactBatch == kExactBatch;
    if (tp.sssPass)
        kPhotonPersistent<true, false><<<blocks, 128, 0, st>>>(tp, sc, in, maxPaths, deposits, depositCap, ctr, perm);
    else if (fixed)
        kPhotonPersistent<false, true><<<blocks, 128, 0, st>>>(tp, sc, in, maxPaths, deposits, depositCap, ctr, perm);
    else
        kPhotonPersistent<false, false><<<blocks, 128, 0, st>>>(tp, sc, in, maxPaths, deposits, depositCap, ctr, perm);
    return cudaGetLastError();
}

cudaError_t launchPhotonTail(const TraceParams& tp, const SceneView& sc, int bounce, const PathState* in,
                             int64_t maxPaths, float4* deposits, int64_t depositCap, PassCounters* ctr,
                             cudaStream_t st) {
    const unsigned blocks = blocksFor(maxPaths, 128, 152 * tp.bouncePerSm);
    if (tp.sssPass)
        kPhotonBounce<true, true><<<blocks, 128, 0, st>>>(tp, sc, bounce, in, nullptr, maxPaths, deposits, depositCap,
                                                           ctr);
    else if (tp.qmc)
        kPhotonBounce<false, true, HaltonTape><<<blocks, 128, 0, st>>>(tp, sc, bounce, in, nullptr, maxPaths, deposits,
                                                                        depositCap, ctr);
    else
        kPhotonBounce<false, true><<<blocks, 128, 0, st>>>(tp, sc, bounce, in, nullptr, maxPaths, deposits, depositCap,
                                                            ctr);
    return cudaGetLastError();
}

cudaError_t launchEyeTrace(const TraceParams& tp, const SceneView& sc, const EnvDev& env, const CameraDev& cam,
                           const OctView& oct, const uint32_t* pixelStates, float* accum, float4* queries,
                           float4* sssQ, int64_t sssCap, PassCounters* ctr, cudaStream_t st, bool pathTrace) {
    const unsigned blocks = blocksFor((int64_t)cam.w * cam.h, 128, 152 * tp.eyePerSm);
    const bool sss = oct.numNodes > 0 || tp.hasSss;
    if (tp.qmc && !pathTrace && sss)
        kEyeTrace<true, false, HaltonTape><<<blocks, 128, 0, st>>>(tp, sc, env, cam, oct, pixelStates, accum, queries,
                                                                    sssQ, sssCap, ctr);
    else if (tp.qmc && !pathTrace)
        kEyeTrace<false, false, HaltonTape><<<blocks, 128, 0, st>>>(tp, sc, env, cam, oct, pixelStates, accum, queries,
                                                                     sssQ, sssCap, ctr);
    else if (pathTrace && sss)
        kEyeTrace<true, true><<<blocks, 128, 0, st>>>(tp, sc, env, cam, oct, pixelStates, accum, queries, sssQ, sssCap, ctr);
    else if (pathTrace)
        kEyeTrace<false, true><<<blocks, 128, 0, st>>>(tp, sc, env, cam, oct, pixelStates, accum, queries, sssQ, sssCap,
                                                       ctr);
    else if (sss)
        kEyeTrace<true, false><<<blocks, 128, 0, st>>>(tp, sc, env, cam, oct, pixelStates, accum, queries, sssQ, sssCap,
                                                       ctr);
    else
        kEyeTrace<false, false><<<blocks, 128, 0, st>>>(tp, sc, env, cam, oct, pixelStates, accum, queries, sssQ, sssCap,
                                                        ctr);
    return cudaGetLastError();
}

cudaError_t launchSubsurfaceGather(const OctView& oct, const DevMaterial* mats, const float4* q,
                                   const unsigned long long* count, int64_t cap, float* accum,
                                   unsigned long long* visits, cudaStream_t st) {
    kSubsurfaceGather<<<blocksFor(cap, 128, 152 * 16), 128, 0, st>>>(oct, mats, q, count, cap, accum, visits);
    return cudaGetLastError();
}

cudaError_t launchStreamCounts(const float4* deposits, const unsigned long long* count, int64_t cap, int64_t tpt,
                               int numStreams, unsigned long long* perStream, cudaStream_t st) {
    kStreamCounts<<<152 * 4, 256, numStreams * sizeof(unsigned long long), st>>>(deposits, count, cap, tpt, numStreams,
                                                                                perStream);
    return cudaGetLastError();
}

}  // namespace pppm
