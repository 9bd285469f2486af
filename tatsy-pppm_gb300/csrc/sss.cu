// Subsurface stage of the render: SubsurfaceIntegrator::initialize
// (subsurface_integrator.cc:180-210), run before every pass's photon pass
// (ppm_probabilistic.cc:83-85), and its stage entry points.
//
//   1. subsurface photon map: the photon pass of buildPhotonMap
//      (subsurface_integrator.cc:240-327) on the wavefront kernels, with the
//      reference's per-pass streams XorShift(time + i);
//   2. Poisson-disc points on the BSSRDF triangles (k_poisson.cu: the
//      reference's sequential dart throwing, reproduced exactly in parallel);
//   3. irradiance at the points: irradianceWithPM (subsurface_integrator.cc:
//      329-365), the compat kNN gather with k = (int)gatherRadius,
//      epsilon = #photons and the normal filter gatherPhotons^2 * 0.01;
//   4. octree over the points (k_octree.cu, constructRec's tree) on the aux
//      stream while the pass's main photons are traced.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "context.h"
#include "trace.h"

namespace pppm {

namespace {

constexpr double kPiD = 3.14159265358979323846;  // 4 atan(1) (common.h:14)
constexpr int kSssBounceLimit = 64;             // buildPhotonMap(scene, photons, 64)

double msSince(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Poisson points -> gather queries (pos | index, normal, unit weight).
void packPointQueries(const std::vector<float>& p, const std::vector<float>& n, std::vector<float4>* q) {
    const size_t m = p.size() / 3;
    q->resize(3 * m);
    for (size_t i = 0; i < m; i++) {
        const int id = (int)i;
        float idBits;
        std::memcpy(&idBits, &id, 4);
        (*q)[3 * i] = make_float4(p[3 * i], p[3 * i + 1], p[3 * i + 2], idBits);
        (*q)[3 * i + 1] = make_float4(n[3 * i], n[3 * i + 1], n[3 * i + 2], 0.0f);
        (*q)[3 * i + 2] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    }
}

// The subsurface photon bounces: a few wavefront launches, then the tail.
int tracePhotonsTo(pppm_ctx* c, const TraceParams& tp, const SceneView& sv, int64_t paths, float4* dep, int64_t cap,
                   PassCounters* ctr, int64_t* launches, const PathState* traced, const uint32_t* perm) {
    RenderState& rs = c->rs;
    if (kPersistentPhotons) {
        PPPM_CUDA(c, launchPhotonPersistent(tp, sv, traced, paths, dep, cap, ctr, c->stream, perm));
        *launches += 1;
        return PPPM_OK;
    }
    const int waves = std::min(kSssBounceLimit, kWaveBounces);
    for (int b = 0; b < waves; b++) {
        PathState* in = (b & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
        PathState* out = (b & 1) ? rs.pathA.as<PathState>() : rs.pathB.as<PathState>();
        PPPM_CUDA(c, launchPhotonBounce(tp, sv, b, in, out, paths, dep, cap, ctr, c->stream));
    }
    PathState* in = (waves & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
    PPPM_CUDA(c, launchPhotonTail(tp, sv, waves, in, paths, dep, cap, ctr, c->stream));
    *launches += 2 + waves;
    return PPPM_OK;
}

double sssCell(const pppm_ctx* c, int k, int64_t stored) {
    const double area = c->bssrdfArea > 0.0 ? c->bssrdfArea : 1.0;
    const double f = c->rs.par.cell_factor >= 1.0f ? c->rs.par.cell_factor : 1.0;
    return f * std::sqrt(area * (double)std::max(k, 1) / (double)std::max<int64_t>(stored, 1));
}

}  // namespace

int sssBegin(pppm_ctx* c) {
    SssState& s = c->rs.sss;
    s.enabled = c->anyBssrdf && !c->bssrdfTris.empty();
    s.octNodes = 0;
    s.numPoints = 0;
    if (!s.enabled) return PPPM_OK;
    // ppm_probabilistic.cc:35-46: the BSSRDF area is averaged over ALL triangles
    const double avgArea = c->bssrdfArea / (double)c->ntri;
    s.areaRadius = std::sqrt(avgArea) * 1.0;
    s.dA = (0.5 * s.areaRadius) * (0.5 * s.areaRadius) * kPiD;
    s.k = (int)c->rs.par.gather_radius;
    if (s.k < 1)
        return fail(c, PPPM_E_UNDEFINED,
                    "render_begin: subsurface kNN count (int)gather_radius < 1 pops an empty queue in the reference");
    if (s.k > kMaxKnn) return fail(c, PPPM_E_CAPACITY, "render_begin: subsurface kNN count (int)gather_radius above 64");
    if (!(s.areaRadius > 0.0)) return fail(c, PPPM_E_UNDEFINED, "render_begin: BSSRDF triangles have zero area");
    // the BSSRDF triangles in scene order (ppm_probabilistic.cc via
    // SubsurfaceIntegrator::initialize, subsurface_integrator.cc:189-195)
    std::vector<float> tri(c->bssrdfTris.size() * 9);
    for (size_t i = 0; i < c->bssrdfTris.size(); i++)
        std::memcpy(&tri[9 * i], &c->hostTri[9 * (size_t)c->bssrdfTris[i]], 36);
    {
        const int e = poissonBegin(c, s.poisson, tri.data(), (int64_t)c->bssrdfTris.size(), s.areaRadius);
        if (e) return e;
    }
    const size_t cand = (size_t)std::max<int64_t>(s.poisson.n, 1);
    PPPM_CUDA(c, s.points.ensure(cand * 48));
    PPPM_CUDA(c, s.ptsD.ensure(cand * 12));
    PPPM_CUDA(c, s.nrmD.ensure(cand * 12));
    PPPM_CUDA(c, s.irad.ensure(cand * 12));
    // eye-pass subsurface queries: two per pixel before the inline fallback
    s.queueCap = 2 * (int64_t)c->rs.cam.width * c->rs.cam.height;
    PPPM_CUDA(c, s.queue.ensure((size_t)s.queueCap * 32));
    return PPPM_OK;
}

// Kernel parameters and photon tape states of pass t's subsurface photon set
// (SubsurfaceIntegrator::buildPhotonMap, subsurface_integrator.cc:240-327).
static int sssPhotonSetup(pppm_ctx* c, int t, const TraceParams& base, TraceParams* tpOut, uint32_t** statesOut,
                          int64_t* launches) {
    RenderState& rs = c->rs;
    const pppm_params& par = rs.par;
    // the path tracer's subsurface stage is the reference's, as in compat mode
    const bool compat = par.mode == PPPM_MODE_COMPAT || par.mode == PPPM_MODE_PATH_TRACING;
    const int N = par.num_streams;
    TraceParams tp = base;
    if (compat) tp.mode = PPPM_MODE_COMPAT;
    tp.sssPass = 1;
    tp.qmc = 0;  // its streams are XorShift(time + i) whatever sampler the eye paths use
    tp.maxBouncePhoton = kSssBounceLimit;
    // the subsurface photon set keeps the reference's own sampling
    tp.guided = 0;
    // canonical mode: an independent counter-based key for this photon set
    tp.seed = base.seed ^ 0x5bd1e995u;
    uint32_t* photonStates = compat ? rs.tapeStates.as<uint32_t>() : nullptr;
    if (compat) {
        // Random::generateSampler((unsigned long)time(NULL) + i) per thread
        // (subsurface_integrator.cc:246-249); time is par.sss_time + t - 1
        std::vector<uint32_t> ss((size_t)N * 4);
        for (int i = 0; i < N; i++) {
            XorShift x;
            x.seed((uint32_t)((unsigned long)(par.sss_time + (uint32_t)(t - 1)) + (unsigned long)i));
            std::memcpy(&ss[4 * (size_t)i], x.s, 16);
        }
        PPPM_CUDA(c, cudaMemcpyAsync(rs.streamStatesD.p, ss.data(), ss.size() * 4, cudaMemcpyHostToDevice, c->stream));
        PPPM_CUDA(c, launchTapeStates(tp, rs.streamStatesD.as<uint32_t>(), rs.jumpMats.as<uint32_t>(), 0, 0,
                                      photonStates, nullptr, c->stream));
        *launches += 1;
    }
    *tpOut = tp;
    *statesOut = photonStates;
    return PPPM_OK;
}

// Emission and every bounce of the subsurface photons into s.photons.
static int sssPhotonLaunch(pppm_ctx* c, const TraceParams& tp, const SceneView& sv, const EnvDev& ev,
                           const uint32_t* photonStates, PassCounters* ctr, int64_t* launches) {
    SssState& s = c->rs.sss;
    PPPM_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(PassCounters), c->stream));
    const uint32_t* perm = nullptr;
    const PathState* traced = nullptr;
    int e = emitPhotonPaths(c, tp, ev, photonStates, ctr, kPersistentPhotons, &traced, &perm, launches);
    if (!e) e = tracePhotonsTo(c, tp, sv, tp.numPaths, s.photons.as<float4>(), s.cap, ctr, launches, traced, perm);
    return e;
}

int sssPrepare(pppm_ctx* c, int t, const TraceParams& base, const SceneView& sv, const EnvDev& ev, int64_t* launches) {
    SssState& s = c->rs.sss;
    RenderState& rs = c->rs;
    const pppm_params& par = rs.par;
    const int64_t paths = base.numPaths;
    TraceParams tp;
    uint32_t* photonStates = nullptr;
    {
        const int e = sssPhotonSetup(c, t, base, &tp, &photonStates, launches);
        if (e) return e;
    }
    PassCounters* ctr = rs.photonCount.as<PassCounters>();
    if (s.cap == 0) s.cap = std::max<int64_t>(paths, 1 << 16);
    PPPM_CUDA(c, s.photons.ensure((size_t)s.cap * 32));

    // the subsurface photon pass
    {
        const int e = sssPhotonLaunch(c, tp, sv, ev, photonStates, ctr, launches);
        if (e) return e;
    }

    // points on the GPU after the photon pass
    int64_t m = 0;
    {
        const int e = poissonRun(c, s.poisson, c->poissonRng, s.points.as<float4>(), s.ptsD.as<float>(),
                                 s.nrmD.as<float>(), std::max<int64_t>(s.poisson.n, 1), &m);
        if (e) return e;
    }
    s.numPoints = m;
    s.msHost = 0.0;

    // (a pageable readback blocks until the stream drains: issued after the sampling)
    PassCounters hc;
    PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (hc.undefinedEmit)
        return fail(c, PPPM_E_UNDEFINED,
                    "render_pass: a subsurface photon draw fell past the env CDF (reference reads _pdf out of bounds)");
    if ((int64_t)hc.deposits > s.cap) {
        // grow and trace the same photons again (tapes and keys are unchanged)
        s.cap = (int64_t)(hc.deposits * 1.25) + 1024;
        PPPM_CUDA(c, s.photons.ensure((size_t)s.cap * 32));
        {
            const int e = sssPhotonLaunch(c, tp, sv, ev, photonStates, ctr, launches);
            if (e) return e;
        }
        PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
        if ((int64_t)hc.deposits > s.cap) return fail(c, PPPM_E_CAPACITY, "render_pass: subsurface photon overflow");
    }
    s.stored = (int64_t)hc.deposits;

    // irradiance at the points
    if (m > 0) {
        if (s.stored == 0) {
            // empty photon map: findKNN returns nothing, maxdist stays 0
            PPPM_CUDA(c, cudaMemsetAsync(s.irad.p, 0, (size_t)m * 12, c->stream));
        } else {
            PPPM_CUDA(c, gridLayout(s.grid, c->bbmin, c->bbmax, sssCell(c, s.k, s.stored), s.stored));
            GridDev gv = gridView(s.grid, c->bbmin, c->bbmax);
            PPPM_CUDA(c, gridBuild(s.grid, gv, s.photons.as<float4>(), reinterpret_cast<const uint64_t*>(&ctr->deposits),
                                   s.cap, c->stream));
            gv = gridView(s.grid, c->bbmin, c->bbmax);
            QueryView qv{s.points.as<float4>(), nullptr, m};
            const int gp = par.gather_photons;
            const float rlim = (float)((double)gp * (double)gp * 0.01);  // subsurface_integrator.cc:343
            PPPM_CUDA(c, launchGatherCompat(gv, qv, s.k, (float)par.photons, rlim, 0, s.irad.as<float>(), false,
                                            c->stream));
            *launches += 6;
        }
    }
    PPPM_CUDA(c, cudaEventRecord(s.done, c->stream));
    return PPPM_OK;
}

int sssFinish(pppm_ctx* c, int64_t* launches) {
    SssState& s = c->rs.sss;
    const auto t0 = std::chrono::steady_clock::now();
    // on the aux stream, beside the photon pass; the main stream waits for it
    PPPM_CUDA(c, cudaStreamWaitEvent(c->aux, s.done, 0));
    const OctreePoints op{s.ptsD.as<float>(), 3, s.irad.as<float>(), 3, nullptr, 0, s.dA};
    int nodes = 0;
    const int e = octreeBuild(c, s.oct, op, s.numPoints, c->aux, &nodes, launches);
    if (e) return e;
    s.octNodes = nodes;
    PPPM_CUDA(c, cudaEventRecord(s.octDone, c->aux));
    PPPM_CUDA(c, cudaStreamWaitEvent(c->stream, s.octDone, 0));
    s.msHost += msSince(t0);
    return PPPM_OK;
}

OctView sssView(const pppm_ctx* c) {
    const SssState& s = c->rs.sss;
    return {s.octNodes > 0 ? s.oct.out.as<OctNodeDev>() : nullptr, s.octNodes, 0.05f};
}

}  // namespace pppm

using namespace pppm;

extern "C" {

int pppm_subsurface_photons(pppm_ctx* c, const pppm_params* par, int32_t t, float* out, int64_t cap, int64_t* n) {
    if (!c || !par || !n || t < 1 || cap < 0 || (cap > 0 && !out))
        return fail(c, PPPM_E_ARG, "subsurface_photons: bad arguments");
    if (par->mode != PPPM_MODE_COMPAT && par->mode != PPPM_MODE_CANONICAL)
        return fail(c, PPPM_E_ARG, "subsurface_photons: compat or canonical mode");
    pppm_params p = *par;
    p.flags &= ~(PPPM_FLAG_LEARNED | PPPM_FLAG_LEARNED_FROZEN | PPPM_FLAG_SAMPLER_QMC);
    const pppm_camera cam{{0.f, 0.f, 0.f}, {0.f, 0.f, 1.f}, {0.f, 1.f, 0.f}, 1.0f, 1, 1};
    int r = pppm_render_begin(c, &cam, &p);
    if (r) return r;
    RenderState& rs = c->rs;
    rs.active = false;  // a set-up for this stage only: no render pass follows
    SssState& s = rs.sss;
    if (!s.enabled) return fail(c, PPPM_E_STATE, "subsurface_photons: the scene has no BSSRDF material");
    TraceParams base, tp;
    CameraDev cd;
    const int64_t paths = p.mode == PPPM_MODE_COMPAT ? rs.taskPerThread * p.num_streams : p.photons;
    passSetup(c, t, paths, &base, &cd);
    int64_t launches = 0;
    uint32_t* photonStates = nullptr;
    if ((r = sssPhotonSetup(c, t, base, &tp, &photonStates, &launches))) return r;
    PassCounters* ctr = rs.photonCount.as<PassCounters>();
    if (s.cap == 0) s.cap = std::max<int64_t>(paths, 1 << 16);
    const SceneView sv = sceneView(c);
    const EnvDev ev = envView(c);
    for (int attempt = 0;; attempt++) {
        PPPM_CUDA(c, s.photons.ensure((size_t)s.cap * 32));
        if ((r = sssPhotonLaunch(c, tp, sv, ev, photonStates, ctr, &launches))) return r;
        PassCounters hc;
        PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
        if (hc.undefinedEmit)
            return fail(c, PPPM_E_UNDEFINED, "subsurface_photons: a photon draw fell past the env CDF");
        if ((int64_t)hc.deposits <= s.cap) {
            s.stored = (int64_t)hc.deposits;
            break;
        }
        if (attempt > 0) return fail(c, PPPM_E_CAPACITY, "subsurface_photons: photon overflow");
        s.cap = (int64_t)(hc.deposits * 1.25) + 1024;
    }
    *n = s.stored;
    const int64_t m = std::min(s.stored, cap);
    if (m > 0) {
        void* dout;
        if ((r = stageOut(c, out, (size_t)m * 32, 0, &dout))) return r;
        PPPM_CUDA(c, launchUnpackRecords(s.photons.as<float4>(), m, (float*)dout, c->stream));
        if ((r = finishOut(c, out, dout, (size_t)m * 32))) return r;
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PPPM_OK;
}

int pppm_poisson_disk(pppm_ctx* c, const float* tri_xyz, int64_t ntri, double min_dist, uint32_t* rng_state,
                      float* pts, float* nrm, int64_t cap, int64_t* count) {
    if (!c || ntri < 0 || (ntri > 0 && !tri_xyz) || !rng_state || !count || cap < 0 || (cap > 0 && (!pts || !nrm)) ||
        !(min_dist > 0.0))
        return fail(c, PPPM_E_ARG, "poisson_disk: bad arguments");
    if (isDevicePtr(tri_xyz) || isDevicePtr(pts) || isDevicePtr(nrm))
        return fail(c, PPPM_E_ARG, "poisson_disk: arrays must be host memory");
    cudaSetDevice(c->device);
    PoissonGpu& g = c->stagePoisson;
    int r;
    if ((r = poissonBegin(c, g, tri_xyz, ntri, min_dist))) return r;
    const size_t cand = (size_t)std::max<int64_t>(g.n, 1);
    PPPM_CUDA(c, c->stageQ.ensure(cand * 48));
    PPPM_CUDA(c, c->stage[0].ensure(cand * 12));
    PPPM_CUDA(c, c->stage[1].ensure(cand * 12));
    int64_t m = 0;
    if ((r = poissonRun(c, g, rng_state, c->stageQ.as<float4>(), c->stage[0].as<float>(), c->stage[1].as<float>(),
                        (int64_t)cand, &m)))
        return r;
    *count = m;
    const int64_t w = std::min(m, cap);
    if (w > 0) {
        PPPM_CUDA(c, cudaMemcpyAsync(pts, c->stage[0].p, (size_t)w * 12, cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaMemcpyAsync(nrm, c->stage[1].p, (size_t)w * 12, cudaMemcpyDeviceToHost, c->stream));
    }
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

}  // extern "C"

extern "C" int pppm_subsurface_photon_irradiance(pppm_ctx* c, const float* photons, int64_t n, const float* points,
                                                 int64_t m, int64_t num_photons, double gather_radius,
                                                 int32_t gather_photons, float* out) {
    if (!c || n < 0 || m < 0 || (n > 0 && !photons) || (m > 0 && (!points || !out)))
        return fail(c, PPPM_E_ARG, "subsurface_photon_irradiance: bad arguments");
    // findKNN(query, &photons, params.photons(), params.gatherRadius()):
    // epsilon = #photons, k = (int)gatherRadius (kdtree.h:17, photon_map.cc:25)
    const int k = (int)gather_radius;
    if (k < 1) return fail(c, PPPM_E_UNDEFINED, "subsurface_photon_irradiance: k = (int)gather_radius < 1");
    if (k > kMaxKnn) return fail(c, PPPM_E_CAPACITY, "subsurface_photon_irradiance: k above 64");
    if (m == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    std::vector<float> ph((size_t)n * 8), pq((size_t)m * 6);
    if (n > 0) {
        if (isDevicePtr(photons)) PPPM_CUDA(c, cudaMemcpy(ph.data(), photons, ph.size() * 4, cudaMemcpyDeviceToHost));
        else std::memcpy(ph.data(), photons, ph.size() * 4);
    }
    if (isDevicePtr(points)) PPPM_CUDA(c, cudaMemcpy(pq.data(), points, pq.size() * 4, cudaMemcpyDeviceToHost));
    else std::memcpy(pq.data(), points, pq.size() * 4);
    double mn[3] = {1e30, 1e30, 1e30}, mx[3] = {-1e30, -1e30, -1e30};
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            mn[d] = std::min(mn[d], (double)ph[8 * i + d]);
            mx[d] = std::max(mx[d], (double)ph[8 * i + d]);
        }
    if (n == 0)
        for (int d = 0; d < 3; d++) { mn[d] = 0.0; mx[d] = 1.0; }
    std::vector<float4> rec((size_t)std::max<int64_t>(n, 1) * 2);
    for (int64_t i = 0; i < n; i++) {
        const float* p = &ph[8 * i];
        const int id = (int)i;
        float idBits;
        std::memcpy(&idBits, &id, 4);
        rec[2 * i] = make_float4(p[0], p[1], p[2], 0.0f);
        rec[2 * i + 1] = make_float4(p[3], p[4], p[5], idBits);
    }
    std::vector<float> pts((size_t)m * 3), nrm((size_t)m * 3);
    for (int64_t i = 0; i < m; i++)
        for (int d = 0; d < 3; d++) {
            pts[3 * i + d] = pq[6 * i + d];
            nrm[3 * i + d] = pq[6 * i + 3 + d];
        }
    std::vector<float4> q;
    packPointQueries(pts, nrm, &q);
    PPPM_CUDA(c, c->stageRec.ensure(rec.size() * 16));
    PPPM_CUDA(c, c->stageQ.ensure(q.size() * 16));
    PPPM_CUDA(c, c->stageCount.ensure(64));
    PPPM_CUDA(c, cudaMemcpyAsync(c->stageRec.p, rec.data(), rec.size() * 16, cudaMemcpyHostToDevice, c->stream));
    PPPM_CUDA(c, cudaMemcpyAsync(c->stageQ.p, q.data(), q.size() * 16, cudaMemcpyHostToDevice, c->stream));
    const uint64_t cnt = (uint64_t)n;
    PPPM_CUDA(c, cudaMemcpyAsync(c->stageCount.p, &cnt, 8, cudaMemcpyHostToDevice, c->stream));
    void* dout;
    int r;
    if ((r = stageOut(c, out, (size_t)m * 12, 2, &dout))) return r;
    if (n == 0) {
        PPPM_CUDA(c, cudaMemsetAsync(dout, 0, (size_t)m * 12, c->stream));
    } else {
        const double ex = std::max({mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2], 1e-6});
        const double cell = ex * std::cbrt(std::min(1.0, (double)k / (double)n));
        PPPM_CUDA(c, gridLayout(c->stageGrid, mn, mx, cell, n));
        GridDev gv = gridView(c->stageGrid, mn, mx);
        PPPM_CUDA(c, gridBuild(c->stageGrid, gv, c->stageRec.as<float4>(), c->stageCount.as<uint64_t>(), n, c->stream));
        gv = gridView(c->stageGrid, mn, mx);
        QueryView qv{c->stageQ.as<float4>(), nullptr, m};
        const float rlim = (float)((double)gather_photons * (double)gather_photons * 0.01);
        PPPM_CUDA(c, launchGatherCompat(gv, qv, k, (float)num_photons, rlim, 0, (float*)dout, false, c->stream));
    }
    if ((r = finishOut(c, out, dout, (size_t)m * 12))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}
