// Render loop (ProgressivePhotonMappingProb::render, ppm_probabilistic.cc:
// 24-121) and the stage entry points for kNN and gather.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "trace.h"

namespace pppm {

namespace {

void hostBbox(const float* p, int64_t n, double* mn, double* mx) {
    for (int d = 0; d < 3; d++) { mn[d] = 1e30; mx[d] = -1e30; }
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            mn[d] = std::min(mn[d], (double)p[3 * i + d]);
            mx[d] = std::max(mx[d], (double)p[3 * i + d]);
        }
    if (n == 0)
        for (int d = 0; d < 3; d++) { mn[d] = 0; mx[d] = 1; }
}

// Positions (stride floats apart) to host, for the grid extent.
int fetchPositions(pppm_ctx* c, const float* src, int64_t n, int stride, std::vector<float>* out) {
    out->resize((size_t)n * 3);
    if (n == 0) return PPPM_OK;
    std::vector<float> all((size_t)n * stride);
    if (isDevicePtr(src)) {
        PPPM_CUDA(c, cudaMemcpyAsync(all.data(), src, all.size() * 4, cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    } else {
        std::memcpy(all.data(), src, all.size() * 4);
    }
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) (*out)[3 * i + d] = all[(size_t)i * stride + d];
    return PPPM_OK;
}

// disc filter threshold _radius * _radius * 0.01 (ppm_probabilistic.cc:314)
float compatDiscLimit(double radius) { return (float)(radius * radius * 0.01); }

double knnCell(const double* mn, const double* mx, int64_t n, int k) {
    const double ex = std::max({mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2], 1e-6});
    const double frac = std::min(1.0, (double)std::max(k, 1) / (double)std::max<int64_t>(n, 1));
    return ex * std::cbrt(frac);
}

}  // namespace

}  // namespace pppm

using namespace pppm;

namespace pppm {

int emitPhotonPaths(pppm_ctx* c, const TraceParams& tp, const EnvDev& ev, const uint32_t* photonStates,
                    PassCounters* ctr, bool sorted, const PathState** paths, const uint32_t** perm,
                    int64_t* launches) {
    RenderState& rs = c->rs;
    sorted = sorted && kPhotonSort && rs.sortPerm.p != nullptr;
    const PhotonSort sort{rs.sortKeys.as<uint32_t>(), rs.sortHist.as<uint32_t>(), rs.sortCursor.as<uint32_t>(),
                          rs.sortTmp.as<uint32_t>(), rs.sortPerm.as<uint32_t>()};
    if (sorted) PPPM_CUDA(c, cudaMemsetAsync(sort.hist, 0, ((size_t)kPhotonSortBins + 1) * 4, c->stream));
    PPPM_CUDA(c, launchPhotonEmit(tp, ev, photonStates, rs.pathA.as<PathState>(), ctr, c->stream,
                                  sorted ? &sort : nullptr));
    *launches += 1;
    const bool move = sorted && kSortMove;
    if (sorted) {
        PPPM_CUDA(c, photonSortPaths(sort, tp.numPaths, c->stream, rs.pathA.as<PathState>(),
                                     move ? rs.pathB.as<PathState>() : nullptr));
        *launches += 4;
    }
    *paths = move ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
    *perm = sorted && !move ? sort.perm : nullptr;
    return PPPM_OK;
}

// Kernel parameters and camera of pass t (everything a pass needs from the
// host besides its buffers).
void passSetup(pppm_ctx* c, int t, int64_t paths, TraceParams* tp, CameraDev* cd) {
    RenderState& rs = c->rs;
    const pppm_params& par = rs.par;
    const int N = par.num_streams;
    const int W = rs.cam.width, H = rs.cam.height;
    const int64_t T = rs.taskPerThread;
    tp->mode = par.mode;
    tp->numStreams = N;
    tp->taskPerThread = T;
    tp->numPaths = paths;
    tp->numPhotons = (double)par.photons;
    tp->maxBouncePhoton = par.max_bounce_photon;
    tp->maxBounceEye = par.max_bounce_eye;
    tp->seed = par.seed;
    tp->pass = t;
    tp->countTraversal = (par.flags & PPPM_FLAG_COUNT_TRAVERSAL) ? 1 : 0;
    tp->sssPass = 0;
    tp->hasSss = rs.sss.enabled ? 1 : 0;
    tp->bouncePerSm = rs.bouncePerSm;
    tp->eyePerSm = rs.eyePerSm;
    tp->refill = rs.refill;
    tp->exactBatch = rs.exactBatch;
    tp->guided = rs.guide.enabled ? 1 : 0;
    tp->guide = guideView(c, 3 * paths);
    tp->qmc = (par.mode == PPPM_MODE_COMPAT && (par.flags & PPPM_FLAG_SAMPLER_QMC)) ? 1 : 0;
    if (tp->qmc) tp->halton = haltonDev(c);
    tp->width = W;
    tp->height = H;
    {
        const double ex = rs.cam.eye[0], ey = rs.cam.eye[1], ez = rs.cam.eye[2];
        const double dx = rs.cam.dir[0], dy = rs.cam.dir[1], dz = rs.cam.dir[2];
        const double ux = rs.cam.up[0], uy = rs.cam.up[1], uz = rs.cam.up[2];
        // ICamera: unitU = cross(direction, up), unitV = cross(unitU, direction) (camera_interface.h:40-41)
        const double Ux = dy * uz - dz * uy, Uy = dz * ux - dx * uz, Uz = dx * uy - dy * ux;
        const double Vx = Uy * dz - Uz * dy, Vy = Uz * dx - Ux * dz, Vz = Ux * dy - Uy * dx;
        cd->ex = ex; cd->ey = ey; cd->ez = ez;
        cd->dx = (float)dx; cd->dy = (float)dy; cd->dz = (float)dz;
        cd->ux = (float)Ux; cd->uy = (float)Uy; cd->uz = (float)Uz;
        cd->vx = (float)Vx; cd->vy = (float)Vy; cd->vz = (float)Vz;
        cd->halfTan = (float)std::tan((double)rs.cam.fov * 0.5);
        cd->aspect = (float)((double)W / (double)H);
        cd->w = W;
        cd->h = H;
    }
}

// Sample t of PathTracing::render (path_tracing.cc:74-97): the subsurface
// stage as in PPM (path_tracing.cc:30-46, 75-77), then one path per pixel.
// Rows go to stream y % N and every pixel of a row draws a 200-number tape
// from its stream (path_tracing.cc:82-90), so the tapes of sample t start
// where sample t - 1's ended. The accumulation keeps row y = camera row y
// (the reference stores pixel (x, y) at buffer(x, H - 1 - y)).
int ptPass(pppm_ctx* c, int t, const TraceParams& tp, const SceneView& sv, const EnvDev& ev, const CameraDev& cd,
           pppm_pass_stats* stats) {
    RenderState& rs = c->rs;
    const pppm_params& par = rs.par;
    const int N = par.num_streams;
    const int W = rs.cam.width, H = rs.cam.height;
    PassCounters* ctr = rs.photonCount.as<PassCounters>();
    int64_t launches = 0;
    PPPM_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    if (rs.sss.enabled) {
        int e = sssPrepare(c, t, tp, sv, ev, &launches);
        if (!e) e = sssFinish(c, &launches);
        if (e) return e;
    }
    PPPM_CUDA(c, cudaEventRecord(c->ev[7], c->stream));
    // pixel tapes only (no photon tapes in this integrator)
    std::vector<uint32_t> ss((size_t)N * 4);
    for (int s = 0; s < N; s++) std::memcpy(&ss[4 * s], rs.streams[s].s, 16);
    PPPM_CUDA(c, cudaMemcpyAsync(rs.streamStatesD.p, ss.data(), ss.size() * 4, cudaMemcpyHostToDevice, c->stream));
    TraceParams tt = tp;
    tt.taskPerThread = 0;
    uint32_t* pixelStates = rs.tapeStates.as<uint32_t>() + 4 * tp.numPaths;
    PPPM_CUDA(c, launchTapeStates(tt, rs.streamStatesD.as<uint32_t>(), rs.jumpMats.as<uint32_t>(), W, H,
                                  rs.tapeStates.as<uint32_t>(), pixelStates, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(PassCounters), c->stream));
    PPPM_CUDA(c, cudaEventRecord(c->ev[2], c->stream));
    PPPM_CUDA(c, launchEyeTrace(tp, sv, ev, cd, sssView(c), pixelStates, rs.accum.as<float>(), rs.queries.as<float4>(),
                                rs.sss.queue.as<float4>(), rs.sss.queueCap, ctr, c->stream, true));
    launches += 2;
    if (rs.sss.enabled) {
        PPPM_CUDA(c, launchSubsurfaceGather(sssView(c), sv.mats, rs.sss.queue.as<float4>(), &ctr->sssQueries,
                                            rs.sss.queueCap, rs.accum.as<float>(),
                                            tp.countTraversal ? &ctr->sssVisits : nullptr, c->stream));
        launches += 1;
    }
    PPPM_CUDA(c, cudaEventRecord(c->ev[3], c->stream));
    PassCounters hc;
    PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->eye_rays = (int64_t)hc.eyeRays;
        float ms;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[7]);
        stats->ms_subsurface = rs.sss.enabled ? ms : 0.0;
        stats->ms_subsurface_host = rs.sss.enabled ? rs.sss.msHost : 0.0;
        stats->sss_points = rs.sss.enabled ? rs.sss.numPoints : 0;
        stats->sss_photons = rs.sss.enabled ? rs.sss.stored : 0;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        stats->ms_eye = ms;
        stats->kernel_launches = launches;
        stats->node_visits = (int64_t)hc.nodeVisits[1];
        stats->tri_tests = (int64_t)hc.triTests[1];
    }
    if (hc.undefinedEye)
        return fail(c, PPPM_E_UNDEFINED, "render_pass: a path drew more than its 200 random numbers (the reference aborts)");
    for (int s = 0; s < N; s++) {
        const int64_t rows = s < H ? (H - 1 - s) / N + 1 : 0;
        xorshiftJumpHost(c->jumpTables, (uint64_t)(rows * W), &rs.streams[s]);
    }
    return PPPM_OK;
}

}  // namespace pppm

extern "C" {

// The k nearest of n points within distance eps of each query (k <= 64),
// farthest first: KdTree::knnSearch (kdtree_detail.h:88-132) on the hash grid.
static int knnRun(pppm_ctx* c, const float* photonPos, int64_t n, const float* queries, int64_t m, int k, float eps,
                  int32_t* idx, int32_t* cnt, int32_t cap) {
    if (m == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    std::vector<float> hp;
    int r;
    if ((r = fetchPositions(c, photonPos, n, 3, &hp))) return r;
    double mn[3], mx[3];
    hostBbox(hp.data(), n, mn, mx);
    const void *dp, *dq;
    void *didx, *dcnt;
    if ((r = stageIn(c, photonPos, (size_t)n * 12, 0, &dp))) return r;
    if ((r = stageIn(c, queries, (size_t)m * 12, 1, &dq))) return r;
    if ((r = stageOut(c, idx, (size_t)m * cap * 4, 2, &didx))) return r;
    if ((r = stageOut(c, cnt, (size_t)m * 4, 3, &dcnt))) return r;
    PPPM_CUDA(c, c->stageRec.ensure((size_t)std::max<int64_t>(n, 1) * 32));
    PPPM_CUDA(c, c->stageCount.ensure(64));
    PPPM_CUDA(c, launchPackPositions((const float*)dp, n, c->stageRec.as<float4>(), c->stageCount.as<uint64_t>(), c->stream));
    PPPM_CUDA(c, gridLayout(c->stageGrid, mn, mx, knnCell(mn, mx, n, k), n));
    GridDev gv = gridView(c->stageGrid, mn, mx);
    PPPM_CUDA(c, gridBuild(c->stageGrid, gv, c->stageRec.as<float4>(), c->stageCount.as<uint64_t>(), n, c->stream,
                           true));
    gv = gridView(c->stageGrid, mn, mx);
    PPPM_CUDA(c, launchKnn(gv, (const float*)dq, m, k, eps, (int32_t*)didx, (int32_t*)dcnt, cap, c->stream));
    if ((r = finishOut(c, idx, didx, (size_t)m * cap * 4))) return r;
    if ((r = finishOut(c, cnt, dcnt, (size_t)m * 4))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_knn(pppm_ctx* c, const float* photonPos, int64_t n, const float* queries, int64_t m, int32_t numTarget,
             double targetRadius, int32_t* idx, int32_t* cnt, int32_t cap) {
    if (!c || n < 0 || m < 0 || cap < 0 || (n > 0 && !photonPos) || (m > 0 && (!queries || !cnt || (cap > 0 && !idx))))
        return fail(c, PPPM_E_ARG, "knn: bad arguments");
    // KnnQuery(type, epsilon, k) receives (numTargetPhotons, targetRadius):
    // k = (int)targetRadius, epsilon = numTargetPhotons (photon_map.cc:25, kdtree.h:17)
    const int k = (int)targetRadius;
    const float eps = (float)numTarget;
    if (k < 1) return fail(c, PPPM_E_UNDEFINED, "knn: k = (int)radius < 1 pops an empty queue in the reference");
    if (k > kMaxKnn) return fail(c, PPPM_E_CAPACITY, "knn: k above 64");
    return knnRun(c, photonPos, n, queries, m, k, eps, idx, cnt, cap);
}

int pppm_kdtree_knn(pppm_ctx* c, const float* points, int64_t n, const float* queries, int64_t m, int32_t type,
                    double epsilon, int32_t k, int32_t* idx, int32_t* cnt, int32_t cap) {
    if (!c || n < 0 || m < 0 || cap < 0 || (n > 0 && !points) || (m > 0 && (!queries || !cnt || (cap > 0 && !idx))) ||
        (type & ~(PPPM_KNN_EPSILON_BALL | PPPM_KNN_K_NEAREST)) != 0 || !(epsilon >= 0.0))
        return fail(c, PPPM_E_ARG, "kdtree_knn: bad arguments");
    // without EPSILON_BALL the ball is unbounded (knnSearch sets INFTY)
    const float eps = (type & PPPM_KNN_EPSILON_BALL) ? (float)std::min(epsilon, 1e30) : 1e30f;
    if (type & PPPM_KNN_K_NEAREST) {
        // k = 0 pops the queue's only element at once, then reads the top of
        // an empty queue (kdtree_detail.h:110-113)
        if (k < 1) return fail(c, PPPM_E_UNDEFINED, "kdtree_knn: k < 1 reads an empty queue in the reference");
        if (k > kMaxKnn || k > cap) return fail(c, PPPM_E_CAPACITY, "kdtree_knn: k above 64 or above cap");
        return knnRun(c, points, n, queries, m, k, eps, idx, cnt, cap);
    }
    // EPSILON_BALL alone: every point within epsilon. Searched as the cap
    // nearest (cap <= 64); a query that fills cap may have more: refused.
    const int kk = std::min<int32_t>(cap, kMaxKnn);
    if (kk < 1) return fail(c, PPPM_E_CAPACITY, "kdtree_knn: cap < 1");
    const int r = knnRun(c, points, n, queries, m, kk, eps, idx, cnt, cap);
    if (r) return r;
    if (m > 0) {
        std::vector<int32_t> hc((size_t)m);
        if (isDevicePtr(cnt)) PPPM_CUDA(c, cudaMemcpy(hc.data(), cnt, (size_t)m * 4, cudaMemcpyDeviceToHost));
        else std::memcpy(hc.data(), cnt, (size_t)m * 4);
        for (int32_t v : hc)
            if (v >= kk) return fail(c, PPPM_E_CAPACITY, "kdtree_knn: more than min(cap, 64) points within epsilon");
    }
    return PPPM_OK;
}

int pppm_gather(pppm_ctx* c, int32_t mode, const float* photons, int64_t n, int64_t phantoms, const float* queries,
                int64_t m, double radius, int32_t gatherPhotons, float* out) {
    if (!c || n < 0 || m < 0 || phantoms < 0 || (n > 0 && !photons) || (m > 0 && (!queries || !out)) ||
        (mode != PPPM_MODE_COMPAT && mode != PPPM_MODE_CANONICAL) || !(radius > 0.0))
        return fail(c, PPPM_E_ARG, "gather: bad arguments");
    const int k = (int)radius;
    if (mode == PPPM_MODE_COMPAT) {
        if (k < 1) return fail(c, PPPM_E_UNDEFINED, "gather: k = (int)radius < 1 pops an empty queue in the reference");
        if (k > kMaxKnn) return fail(c, PPPM_E_CAPACITY, "gather: k above 64");
    }
    if (m == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    std::vector<float> hp;
    int r;
    if ((r = fetchPositions(c, photons, n, 8, &hp))) return r;
    double mn[3], mx[3];
    hostBbox(hp.data(), n, mn, mx);
    const void *dp, *dq;
    void* dout;
    if ((r = stageIn(c, photons, (size_t)n * 32, 0, &dp))) return r;
    if ((r = stageIn(c, queries, (size_t)m * 48, 1, &dq))) return r;
    if ((r = stageOut(c, out, (size_t)m * 12, 2, &dout))) return r;
    PPPM_CUDA(c, c->stageRec.ensure((size_t)std::max<int64_t>(n, 1) * 32));
    PPPM_CUDA(c, c->stageQ.ensure((size_t)m * 48));
    PPPM_CUDA(c, c->stageCount.ensure(64));
    PPPM_CUDA(c, launchPackPhotons((const float*)dp, n, c->stageRec.as<float4>(), c->stageCount.as<uint64_t>(), c->stream));
    PPPM_CUDA(c, launchPackQueries((const float*)dq, m, c->stageQ.as<float4>(), c->stream));
    const double cell = mode == PPPM_MODE_CANONICAL ? radius : knnCell(mn, mx, n, k);
    PPPM_CUDA(c, gridLayout(c->stageGrid, mn, mx, cell, n));
    GridDev gv = gridView(c->stageGrid, mn, mx);
    PPPM_CUDA(c, gridBuild(c->stageGrid, gv, c->stageRec.as<float4>(), c->stageCount.as<uint64_t>(), n, c->stream,
                           mode != PPPM_MODE_CANONICAL));
    gv = gridView(c->stageGrid, mn, mx);
    QueryView qv{c->stageQ.as<float4>(), nullptr, m};
    if (mode == PPPM_MODE_CANONICAL) {
        PPPM_CUDA(c, querySortLayout(c->stageQsort, m));
        PPPM_CUDA(c, launchGatherTiled(gv, qv, c->stageQsort, (float)radius, (float*)dout, false, nullptr, c->stream));
    }
    else
        PPPM_CUDA(c, launchGatherCompat(gv, qv, k, (float)gatherPhotons, compatDiscLimit(radius), phantoms,
                                        (float*)dout, false, c->stream));
    if ((r = finishOut(c, out, dout, (size_t)m * 12))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

// default grid cap of the eye kernel, blocks of 128 per SM: 128 gives each
// block one 16x8 pixel tile at 1080p, so that eye blocks leave the SMs
// sooner to the photon kernel beside them (64: 0.9 % slower, 16: 4 %)
#ifndef PPPM_EYE_PER_SM
#define PPPM_EYE_PER_SM 128
#endif
constexpr int kEyePerSmMax = 128;

int pppm_render_begin(pppm_ctx* c, const pppm_camera* cam, const pppm_params* par) {
    if (!c || !cam || !par) return fail(c, PPPM_E_ARG, "render_begin: null argument");
    if (!c->hasScene) return fail(c, PPPM_E_STATE, "render_begin: no scene");
    // The default Scene env map has no importance tables (scene.cc:11-12):
    // photon emission would read an empty CDF. Emissive triangles light a
    // scene without one.
    if (!c->hasEnv && c->numLights == 0)
        return fail(c, PPPM_E_STATE, "render_begin: no env map (the only light of the reference) and no emitter");
    if (c->numLights > 0 && par->mode != PPPM_MODE_CANONICAL && par->mode != PPPM_MODE_PATH_TRACING)
        return fail(c, PPPM_E_ARG, "render_begin: emissive materials have no reference semantics; canonical mode and "
                                   "the path tracer render them");
    if (c->numLights > 0 && (par->flags & PPPM_FLAG_LEARNED))
        return fail(c, PPPM_E_ARG, "render_begin: the learned proposal proposes environment directions");
    if (par->mode != PPPM_MODE_COMPAT && par->mode != PPPM_MODE_CANONICAL && par->mode != PPPM_MODE_CLASSIC &&
        par->mode != PPPM_MODE_PATH_TRACING)
        return fail(c, PPPM_E_ARG, "render_begin: unknown mode");
    if ((par->mode == PPPM_MODE_CLASSIC || par->mode == PPPM_MODE_PATH_TRACING) && (par->flags & PPPM_FLAG_LEARNED))
        return fail(c, PPPM_E_ARG, "render_begin: the learned proposal needs canonical mode");
    if ((par->flags & PPPM_FLAG_SAMPLER_QMC) && par->mode != PPPM_MODE_COMPAT)
        return fail(c, PPPM_E_ARG, "render_begin: the Halton sampler belongs to compat mode (the reference's sampler "
                                   "types); classic PPM always uses it");
    if (par->num_streams < 1 || par->num_streams > 4096 || par->photons < 1 || cam->width < 1 || cam->height < 1 ||
        par->max_bounce_photon < 0 || par->max_bounce_eye < 0 || !(par->alpha > 0.0) || !(par->radius_scale > 0.0))
        return fail(c, PPPM_E_ARG, "render_begin: bad parameters");
    cudaSetDevice(c->device);
    RenderState& rs = c->rs;
    rs.active = false;
    rs.cam = *cam;
    rs.par = *par;
    if (!(rs.par.cell_factor >= 1.0f)) rs.par.cell_factor = 1.0f;
    // grid caps of the trace kernels (blocks of 128 per SM): more blocks
    // than can be resident balance the long paths better
    rs.bouncePerSm = 64;
    rs.eyePerSm = PPPM_EYE_PER_SM;
    rs.refill = kRefill;
    rs.exactBatch = kExactBatch;
    rs.qsort.stage = PPPM_GATHER_WSTAGE;  // (querySortLayout below sets the sub-cell bits)
    const double dx = c->bbmax[0] - c->bbmin[0], dy = c->bbmax[1] - c->bbmin[1], dz = c->bbmax[2] - c->bbmin[2];
    rs.bboxDiag = std::sqrt(dx * dx + dy * dy + dz * dz);
    rs.radius = rs.bboxDiag * par->radius_scale;  // ppm_probabilistic.cc:51-55
    const int N = par->num_streams;
    const bool perStream = par->mode != PPPM_MODE_CANONICAL;  // compat and classic: N streams of ceil(P/N)
    rs.taskPerThread = perStream ? (par->photons + N - 1) / N : par->photons;
    const int64_t paths = perStream ? rs.taskPerThread * N : par->photons;
    const int64_t pixels = (int64_t)cam->width * cam->height;
    rs.streams.assign(N, XorShift());
    for (int i = 0; i < N; i++) rs.streams[i].seed((uint32_t)i);  // Random::generateSampler(i)
    if (par->mode == PPPM_MODE_COMPAT || par->mode == PPPM_MODE_PATH_TRACING) {
        if (c->jumpTables.empty()) xorshiftJumpTables(&c->jumpTables);
        PPPM_CUDA(c, rs.jumpMats.ensure(c->jumpTables.size() * 4));
        PPPM_CUDA(c, cudaMemcpy(rs.jumpMats.p, c->jumpTables.data(), c->jumpTables.size() * 4, cudaMemcpyHostToDevice));
        PPPM_CUDA(c, rs.tapeStates.ensure((size_t)(paths + pixels) * 16));
    }
    PPPM_CUDA(c, rs.accum.ensure((size_t)pixels * 12));
    PPPM_CUDA(c, cudaMemsetAsync(rs.accum.p, 0, (size_t)pixels * 12, c->stream));
    PPPM_CUDA(c, rs.pathA.ensure((size_t)paths * sizeof(PathState)));
    PPPM_CUDA(c, rs.pathB.ensure((size_t)paths * sizeof(PathState)));
    if (kPhotonSort) {
        PPPM_CUDA(c, rs.sortKeys.ensure((size_t)paths * 4));
        PPPM_CUDA(c, rs.sortPerm.ensure((size_t)paths * 4));
        PPPM_CUDA(c, rs.sortHist.ensure(((size_t)kPhotonSortBins + 1) * 4));
        PPPM_CUDA(c, rs.sortCursor.ensure(((size_t)kPhotonSortBins + 1) * 4));
        PPPM_CUDA(c, rs.sortTmp.ensure((size_t)scanTmpWords(kPhotonSortBins) * 4));
    }
    if (rs.depositCap == 0) rs.depositCap = std::max<int64_t>(2 * paths, 1 << 16);
    PPPM_CUDA(c, rs.photons.ensure((size_t)rs.depositCap * 32));
    PPPM_CUDA(c, rs.queries.ensure((size_t)pixels * 48));
    PPPM_CUDA(c, rs.photonCount.ensure(sizeof(PassCounters) + 8 * (size_t)N));
    PPPM_CUDA(c, rs.streamStatesD.ensure((size_t)N * 16));
    PPPM_CUDA(c, querySortLayout(rs.qsort, pixels));
    PPPM_CUDA(c, rs.gatherWork.ensure(16));
    if (c->hasEnv) {
        const int e = envFluxScale(c, (double)par->photons);
        if (e) return e;
    }
    // emitter photons: Le * pi * area / P (area pdf 1/A, cosine pdf cos/pi)
    c->lightFluxScale = (float)(3.14159265358979323846 * c->lightArea / (double)par->photons);
    if (par->flags & PPPM_FLAG_SAMPLER_QMC) {
        const int e = haltonBegin(c, N);
        if (e) return e;
    }
    if (par->mode == PPPM_MODE_CLASSIC) {
        // classic PPM has no subsurface stage for these materials (its test is
        // type == BSSRDF, progressive_photon_mapping.cc:42) and no proposal
        rs.sss.enabled = false;
        rs.guide.enabled = false;
        const int e = classicBegin(c, pixels);
        if (e) return e;
    } else {
        const int e = sssBegin(c);
        if (e) return e;
    }
    if (par->mode != PPPM_MODE_CLASSIC) {
        const int e = guideBegin(c, paths);
        if (e) return e;
    }
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    rs.passesDone = 0;
    rs.storedLast = 0;
    rs.queriesLast = 0;
    rs.storedMax = 0;
    rs.phantomsLast = 0;
    rs.active = true;
    return PPPM_OK;
}

int pppm_render_pass(pppm_ctx* c, int32_t t, pppm_pass_stats* stats) {
    if (!c) return PPPM_E_ARG;
    RenderState& rs = c->rs;
    if (!rs.active) return fail(c, PPPM_E_STATE, "render_pass: call render_begin first");
    if (t != rs.passesDone + 1) return fail(c, PPPM_E_STATE, "render_pass: passes must run in order 1, 2, ...");
    cudaSetDevice(c->device);
    const pppm_params& par = rs.par;
    const bool compat = par.mode == PPPM_MODE_COMPAT;
    const int N = par.num_streams;
    const int W = rs.cam.width, H = rs.cam.height;
    const int64_t pixels = (int64_t)W * H;
    const int64_t T = rs.taskPerThread;
    const int64_t paths = par.mode != PPPM_MODE_CANONICAL ? T * N : par.photons;
    const int k = (int)rs.radius;
    if (compat && k < 1) return fail(c, PPPM_E_UNDEFINED, "render_pass: k = (int)radius < 1 pops an empty queue in the reference");
    if (compat && k > kMaxKnn) return fail(c, PPPM_E_CAPACITY, "render_pass: k = (int)radius above 64");

    TraceParams tp;
    CameraDev cd;
    passSetup(c, t, paths, &tp, &cd);
    int64_t launches = 0;
    const SceneView sv = sceneView(c);
    const EnvDev ev = envView(c);
    if (par.mode == PPPM_MODE_CLASSIC) {
        const int e = classicPass(c, t, tp, sv, ev, cd, stats);
        if (e) return e;
        rs.passesDone = t;
        return PPPM_OK;
    }
    if (par.mode == PPPM_MODE_PATH_TRACING) {
        const int e = ptPass(c, t, tp, sv, ev, cd, stats);
        if (e) return e;
        rs.passesDone = t;
        return PPPM_OK;
    }
    PassCounters* ctr = rs.photonCount.as<PassCounters>();
    unsigned long long* perStream = reinterpret_cast<unsigned long long*>(ctr + 1);
    uint32_t* photonStates = compat ? rs.tapeStates.as<uint32_t>() : nullptr;
    uint32_t* pixelStates = compat ? photonStates + 4 * paths : nullptr;

    PPPM_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    if (rs.sss.enabled) {
        // SubsurfaceIntegrator::initialize before tracePhotons (ppm_probabilistic.cc:83-88)
        const int e = sssPrepare(c, t, tp, sv, ev, &launches);
        if (e) return e;
    }
    PPPM_CUDA(c, cudaEventRecord(c->ev[7], c->stream));
    if (compat && !tp.qmc) {
        std::vector<uint32_t> ss((size_t)N * 4);
        for (int s = 0; s < N; s++) std::memcpy(&ss[4 * s], rs.streams[s].s, 16);
        PPPM_CUDA(c, cudaMemcpyAsync(rs.streamStatesD.p, ss.data(), ss.size() * 4, cudaMemcpyHostToDevice, c->stream));
        PPPM_CUDA(c, launchTapeStates(tp, rs.streamStatesD.as<uint32_t>(), rs.jumpMats.as<uint32_t>(), W, H, photonStates,
                                      pixelStates, c->stream));
        launches += 1;
    }
    PassCounters hc;
    PPPM_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(PassCounters) + 8 * (size_t)N, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(rs.gatherWork.p, 0, 16, c->stream));
    // Eye paths do not depend on the photons: without subsurface scattering
    // (whose eye pass reads this pass's octree) they are traced on the side
    // stream while the photon pass runs, filling the SMs its long late
    // chains leave idle.
    const bool sideEye = !rs.sss.enabled;
    // every exit of this function leaves the main stream behind the side
    // stream's work, so later syncs, reallocations and passes wait for it
    struct SideJoin {
        pppm_ctx* c;
        bool on = false;
        ~SideJoin() {
            if (on) cudaStreamWaitEvent(c->stream, c->ev[11], 0);
        }
    } sideJoin{c};
    // canonical: the queries are sorted on the side stream right after the
    // eye paths (the sort needs only the grid's geometry), beside the photons
    const bool sideSort = sideEye && !compat;
    if (sideEye) {
        PPPM_CUDA(c, cudaEventRecord(c->ev[8], c->stream));
        PPPM_CUDA(c, cudaStreamWaitEvent(c->side, c->ev[8], 0));
        PPPM_CUDA(c, cudaEventRecord(c->ev[9], c->side));
        PPPM_CUDA(c, launchEyeTrace(tp, sv, ev, cd, sssView(c), pixelStates, rs.accum.as<float>(),
                                    rs.queries.as<float4>(), rs.sss.queue.as<float4>(), rs.sss.queueCap, ctr, c->side));
        PPPM_CUDA(c, cudaEventRecord(c->ev[10], c->side));
        if (sideSort) {
            const GridDev geom = gridGeometry(c->bbmin, c->bbmax, par.cell_factor * rs.radius);
            const QueryView qs{rs.queries.as<float4>(), reinterpret_cast<const uint32_t*>(&ctr->queries), pixels};
            PPPM_CUDA(c, querySort(geom, qs, rs.qsort, c->side));
        }
        PPPM_CUDA(c, cudaEventRecord(c->ev[11], c->side));
        sideJoin.on = true;
    }
    for (int attempt = 0;; attempt++) {
        if (attempt > 0) {
            // the photon half of the counters (the eye half may be in flight)
            PPPM_CUDA(c, cudaMemsetAsync(ctr->queue, 0, sizeof(ctr->queue) + sizeof(ctr->deposits), c->stream));
            PPPM_CUDA(c, cudaMemsetAsync(&ctr->photonRays, 0, 8, c->stream));
            PPPM_CUDA(c, cudaMemsetAsync(&ctr->undefinedEmit, 0, 8, c->stream));
            PPPM_CUDA(c, cudaMemsetAsync(&ctr->nodeVisits[0], 0, 8, c->stream));
            PPPM_CUDA(c, cudaMemsetAsync(&ctr->triTests[0], 0, 8, c->stream));
            PPPM_CUDA(c, cudaMemsetAsync(&ctr->fetched, 0, 8, c->stream));
            PPPM_CUDA(c, cudaMemsetAsync(perStream, 0, 8 * (size_t)N, c->stream));
        }
        if (tp.guided && rs.guide.trained) {
            // the network's emission mixture for this pass
            const int e = guideEmission(c);
            if (e) return e;
            launches += 2;
        }
        // per-bounce launches while the queue is wide, then one tail launch
        // (guided bounces need every bounce as a queue step)
        const bool guideBounces = tp.guided && rs.guide.guideBounces;
        // the Halton photons run on the per-bounce kernels
        const bool persistent = kPersistentPhotons && !guideBounces && !tp.qmc;
        const uint32_t* perm = nullptr;
        const PathState* traced = nullptr;
        {
            int64_t emitLaunches = 0;
            const int e = emitPhotonPaths(c, tp, ev, photonStates, ctr, persistent, &traced, &perm, &emitLaunches);
            if (e) return e;
            launches += emitLaunches - 1;  // the emission launch is counted below
        }
        PPPM_CUDA(c, cudaEventRecord(c->ev[5], c->stream));
        const int waves = persistent ? 0
                          : guideBounces ? par.max_bounce_photon : std::min(par.max_bounce_photon, kWaveBounces);
        launches += 1 + waves + (waves < par.max_bounce_photon ? 1 : 0);
        if (persistent && par.max_bounce_photon > 0)
            PPPM_CUDA(c, launchPhotonPersistent(tp, sv, traced, paths, rs.photons.as<float4>(), rs.depositCap, ctr,
                                                c->stream, perm));
        for (int b = 0; b < waves; b++) {
            PathState* in = (b & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
            PathState* out = (b & 1) ? rs.pathA.as<PathState>() : rs.pathB.as<PathState>();
            PPPM_CUDA(c, launchPhotonBounce(tp, sv, b, in, out, paths, rs.photons.as<float4>(), rs.depositCap, ctr,
                                            c->stream));
            if (guideBounces && b + 1 < par.max_bounce_photon) {
                const int e = guideStep(c, tp, out, &ctr->queue[(b + 1) % 3], paths, b + 1);
                if (e) return e;
                launches += rs.guide.trained ? 3 : 1;
            }
        }
        if (!persistent && waves < par.max_bounce_photon) {
            PathState* in = (waves & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
            PPPM_CUDA(c, launchPhotonTail(tp, sv, waves, in, paths, rs.photons.as<float4>(), rs.depositCap, ctr,
                                          c->stream));
        }
        PPPM_CUDA(c, cudaEventRecord(c->ev[6], c->stream));
        if (attempt == 0 && rs.sss.enabled) {
            // octree build beside this pass's photons
            const int e = sssFinish(c, &launches);
            if (e) return e;
        }
        PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
        if ((int64_t)hc.deposits <= rs.depositCap) break;
        if (attempt > 0) return fail(c, PPPM_E_CAPACITY, "render_pass: photon buffer overflow");
        // grow and trace the same photons again (the tapes are unchanged)
        rs.depositCap = (int64_t)(hc.deposits * 1.25) + 1024;
        PPPM_CUDA(c, rs.photons.ensure((size_t)rs.depositCap * 32));
    }
    const int64_t stored = (int64_t)hc.deposits;
    int64_t phantoms = 0;
    if (compat) {
        // ppm_probabilistic.cc:202-207: thread i's photons are copied to slot
        // i * ceil(P/N); unused slots keep default Photon() records.
        PPPM_CUDA(c, launchStreamCounts(rs.photons.as<float4>(), &ctr->deposits, rs.depositCap, T, N, perStream,
                                        c->stream));
        launches += 1;
        std::vector<unsigned long long> ps(N);
        PPPM_CUDA(c, cudaMemcpyAsync(ps.data(), perStream, 8 * (size_t)N, cudaMemcpyDeviceToHost, c->stream));
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int s = 0; s < N; s++) {
            if ((int64_t)ps[s] > T)
                return fail(c, PPPM_E_UNDEFINED,
                            "render_pass: a thread stored more photons than its ceil(P/N) slots; the reference then "
                            "overwrites other threads' photons or writes past the photon array");
            phantoms += T - (int64_t)ps[s];
        }
    }
    PPPM_CUDA(c, cudaEventRecord(c->ev[1], c->stream));

    // photon map
    double cell;
    if (compat) {
        const double area = c->lambertArea > 0.0 ? c->lambertArea : 1.0;
        cell = par.cell_factor * std::sqrt(area * (double)std::max(k, 1) / (double)std::max<int64_t>(stored, 1));
    } else {
        cell = par.cell_factor * rs.radius;
    }
    PPPM_CUDA(c, gridLayout(rs.grid, c->bbmin, c->bbmax, cell, stored));
    GridDev gv = gridView(rs.grid, c->bbmin, c->bbmax);
    // the k-nearest search (compat) skips buckets of other cells and the
    // per-photon cell test in buckets of one cell
    PPPM_CUDA(c, gridBuild(rs.grid, gv, rs.photons.as<float4>(), reinterpret_cast<const uint64_t*>(&ctr->deposits),
                           rs.depositCap, c->stream, compat));
    gv = gridView(rs.grid, c->bbmin, c->bbmax);
    launches += 5;
    PPPM_CUDA(c, cudaEventRecord(c->ev[2], c->stream));

    // eye paths and gather
    if (sideEye)
        PPPM_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev[11], 0));
    else
        PPPM_CUDA(c, launchEyeTrace(tp, sv, ev, cd, sssView(c), pixelStates, rs.accum.as<float>(),
                                    rs.queries.as<float4>(), rs.sss.queue.as<float4>(), rs.sss.queueCap, ctr, c->stream));
    if (rs.sss.enabled) {
        PPPM_CUDA(c, launchSubsurfaceGather(sssView(c), sv.mats, rs.sss.queue.as<float4>(), &ctr->sssQueries,
                                            rs.sss.queueCap, rs.accum.as<float>(),
                                            tp.countTraversal ? &ctr->sssVisits : nullptr, c->stream));
        launches += 1;
    }
    if (tp.guided) {
        const int e = guideImportance(c, rs.queries.as<float4>(), &ctr->queries, pixels, t);
        if (e) return e;
        launches += 1;
    }
    PPPM_CUDA(c, cudaEventRecord(c->ev[3], c->stream));
    QueryView qv{rs.queries.as<float4>(), reinterpret_cast<const uint32_t*>(&ctr->queries), pixels};
    if (compat)
        PPPM_CUDA(c, launchGatherCompat(gv, qv, k, (float)par.gather_photons, compatDiscLimit(rs.radius), phantoms,
                                        rs.accum.as<float>(), true, c->stream));
    else if (sideSort)
        PPPM_CUDA(c, launchGatherSorted(gv, qv, rs.qsort, (float)rs.radius, rs.accum.as<float>(), true,
                                        tp.countTraversal ? rs.gatherWork.as<unsigned long long>() : nullptr,
                                        c->stream));
    else
        PPPM_CUDA(c, launchGatherTiled(gv, qv, rs.qsort, (float)rs.radius, rs.accum.as<float>(), true,
                                       tp.countTraversal ? rs.gatherWork.as<unsigned long long>() : nullptr,
                                       c->stream));
    launches += compat ? 2 : 8;
    PPPM_CUDA(c, cudaEventRecord(c->ev[4], c->stream));
    PPPM_CUDA(c, cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));

    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->photons_traced = paths;
        stats->photons_stored = stored;
        stats->phantom_photons = phantoms;
        stats->photon_rays = (int64_t)hc.photonRays;
        stats->eye_rays = (int64_t)hc.eyeRays;
        stats->gather_queries = (int64_t)hc.queries;
        stats->radius = rs.radius;
        float ms;
        cudaEventElapsedTime(&ms, c->ev[7], c->ev[1]);
        stats->ms_photon = ms;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[7]);
        stats->ms_subsurface = rs.sss.enabled ? ms : 0.0;
        stats->ms_subsurface_host = rs.sss.enabled ? rs.sss.msHost : 0.0;
        stats->sss_points = rs.sss.enabled ? rs.sss.numPoints : 0;
        stats->sss_photons = rs.sss.enabled ? rs.sss.stored : 0;
        cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]);
        stats->ms_grid = ms;
        // with the side stream: the eye trace itself (it overlaps ms_photon)
        cudaEventElapsedTime(&ms, sideEye ? c->ev[9] : c->ev[2], sideEye ? c->ev[10] : c->ev[3]);
        stats->ms_eye = ms;
        cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]);
        stats->ms_gather = ms;
        cudaEventElapsedTime(&ms, c->ev[5], c->ev[6]);
        stats->ms_bounce = ms;
        stats->kernel_launches = launches;
        stats->node_visits = (int64_t)(hc.nodeVisits[0] + hc.nodeVisits[1]);
        stats->tri_tests = (int64_t)(hc.triTests[0] + hc.triTests[1]);
        stats->photon_node_visits = (int64_t)hc.nodeVisits[0];
        stats->photon_tri_tests = (int64_t)hc.triTests[0];
        unsigned long long gw[2] = {0, 0};
        if (tp.countTraversal) PPPM_CUDA(c, cudaMemcpy(gw, rs.gatherWork.p, 16, cudaMemcpyDeviceToHost));
        stats->gather_pairs = (int64_t)gw[0];
        stats->gather_inside = (int64_t)gw[1];
    }
    if (hc.undefinedEmit)
        return fail(c, PPPM_E_UNDEFINED, "render_pass: a photon draw fell past the env CDF (reference reads _pdf out of bounds)");
    if (hc.undefinedEye)
        return fail(c, compat ? PPPM_E_UNDEFINED : PPPM_E_CAPACITY,
                    compat ? "render_pass: an eye path drew more than its 200 random numbers (the reference aborts)"
                           : "render_pass: an eye path exceeded 4096 segments");

    // radius update (ppm_probabilistic.cc:94 in compat; Knaus-Zwicker
    // r^2_{t+1} = r^2_t (t + alpha) / (t + 1) in canonical mode)
    if (compat) rs.radius = (t + 1.0) / (t + par.alpha) * rs.radius;
    else rs.radius = rs.radius * std::sqrt((t + par.alpha) / (t + 1.0));
    if (compat) {
        // each stream drew ceil(P/N) photon tapes and one tape per pixel of its rows
        for (int s = 0; s < N; s++) {
            const int64_t rows = s < H ? (H - 1 - s) / N + 1 : 0;
            xorshiftJumpHost(c->jumpTables, (uint64_t)(T + rows * W), &rs.streams[s]);
        }
    }
    rs.storedLast = stored;
    rs.queriesLast = (int64_t)hc.queries;
    rs.storedMax = std::max(rs.storedMax, stored);
    rs.phantomsLast = phantoms;
    rs.passesDone = t;
    if (rs.guide.enabled) {
        const int e = guideEndPass(c, t);
        if (e) return e;
        if (stats) {
            stats->ms_train = rs.guide.msTrain;
            stats->train_loss = rs.guide.lastLoss;
            stats->train_records = rs.guide.lastRecords;
        }
    }
    return PPPM_OK;
}

int pppm_render_skip(pppm_ctx* c, int32_t count) {
    if (!c || count < 0) return fail(c, PPPM_E_ARG, "render_skip: bad arguments");
    RenderState& rs = c->rs;
    if (!rs.active) return fail(c, PPPM_E_STATE, "render_skip: call render_begin first");
    const pppm_params& par = rs.par;
    if ((par.mode != PPPM_MODE_CANONICAL && par.mode != PPPM_MODE_COMPAT && par.mode != PPPM_MODE_PATH_TRACING) ||
        rs.sss.enabled || rs.guide.enabled)
        return fail(c, PPPM_E_STATE,
                    "render_skip: passes depend on earlier ones here (classic PPM, subsurface stage, learned proposal)");
    const int N = par.num_streams;
    const int W = rs.cam.width, H = rs.cam.height;
    const int64_t T = par.mode == PPPM_MODE_PATH_TRACING ? 0 : rs.taskPerThread;
    for (int i = 0; i < count; i++) {
        const int t = rs.passesDone + 1;
        // what pass t would leave behind: its radius update and, with the
        // reference's streams, the tapes it would have drawn
        if (par.mode == PPPM_MODE_COMPAT) rs.radius = (t + 1.0) / (t + par.alpha) * rs.radius;
        else if (par.mode == PPPM_MODE_CANONICAL) rs.radius = rs.radius * std::sqrt((t + par.alpha) / (t + 1.0));
        if (par.mode != PPPM_MODE_CANONICAL)
            for (int s = 0; s < N; s++) {
                const int64_t rows = s < H ? (H - 1 - s) / N + 1 : 0;
                xorshiftJumpHost(c->jumpTables, (uint64_t)(T + rows * W), &rs.streams[s]);
            }
        rs.passesDone = t;
    }
    return PPPM_OK;
}

int pppm_render_tune(pppm_ctx* c, float cell_factor, int32_t bounce_blocks_per_sm, int32_t eye_blocks_per_sm) {
    if (!c) return PPPM_E_ARG;
    if (!c->rs.active) return fail(c, PPPM_E_STATE, "render_tune: no render");
    if (cell_factor > 0.0f) {
        if (cell_factor < 1.0f) return fail(c, PPPM_E_ARG, "render_tune: cell_factor must be >= 1");
        c->rs.par.cell_factor = cell_factor;
    }
    if (bounce_blocks_per_sm > 0) c->rs.bouncePerSm = std::min(bounce_blocks_per_sm, 64);
    if (eye_blocks_per_sm > 0) c->rs.eyePerSm = std::min(eye_blocks_per_sm, kEyePerSmMax);
    return PPPM_OK;
}

int pppm_render_tune_ex(pppm_ctx* c, const pppm_tune* t) {
    if (!c || !t) return fail(c, PPPM_E_ARG, "render_tune_ex: null argument");
    if (!c->rs.active) return fail(c, PPPM_E_STATE, "render_tune_ex: no render");
    auto in = [](int32_t v, int lo, int hi) { return v < 0 || (v >= lo && v <= hi); };
    if ((t->cell_factor > 0.0f && !(t->cell_factor >= 1.0f)) || !in(t->bounce_blocks_per_sm, 1, 64) ||
        !in(t->eye_blocks_per_sm, 1, kEyePerSmMax) || !in(t->refill, 1, 32) || !in(t->exact_batch, 1, 32) ||
        !in(t->gather_stage, 32, kGatherStageMax) || (t->gather_stage > 0 && t->gather_stage % 32 != 0) ||
        !in(t->query_sub_bits, 0, 3))
        return fail(c, PPPM_E_ARG, "render_tune_ex: a knob out of range");
    RenderState& rs = c->rs;
    if (t->cell_factor > 0.0f) rs.par.cell_factor = t->cell_factor;
    if (t->bounce_blocks_per_sm > 0) rs.bouncePerSm = t->bounce_blocks_per_sm;
    if (t->eye_blocks_per_sm > 0) rs.eyePerSm = t->eye_blocks_per_sm;
    if (t->refill > 0) rs.refill = t->refill;
    if (t->exact_batch > 0) rs.exactBatch = t->exact_batch;
    if (t->gather_stage > 0) rs.qsort.stage = t->gather_stage;
    if (t->query_sub_bits >= 0) rs.qsort.subBits = t->query_sub_bits;
    return PPPM_OK;
}

int pppm_render_get_tune(pppm_ctx* c, pppm_tune* out) {
    if (!c || !out) return fail(c, PPPM_E_ARG, "render_get_tune: null argument");
    if (!c->rs.active) return fail(c, PPPM_E_STATE, "render_get_tune: no render");
    const RenderState& rs = c->rs;
    out->cell_factor = rs.par.cell_factor;
    out->bounce_blocks_per_sm = rs.bouncePerSm;
    out->eye_blocks_per_sm = rs.eyePerSm;
    out->refill = rs.refill;
    out->exact_batch = rs.exactBatch;
    out->gather_stage = rs.qsort.stage;
    out->query_sub_bits = rs.qsort.subBits;
    return PPPM_OK;
}

int pppm_render_read(pppm_ctx* c, float* accum) {
    if (!c || !accum) return fail(c, PPPM_E_ARG, "render_read: bad arguments");
    if (!c->rs.active) return fail(c, PPPM_E_STATE, "render_read: no render");
    if (c->rs.par.mode == PPPM_MODE_CLASSIC) {
        const int e = classicRead(c, nullptr);
        if (e) return e;
    }
    const size_t bytes = (size_t)c->rs.cam.width * c->rs.cam.height * 12;
    PPPM_CUDA(c, cudaMemcpyAsync(accum, c->rs.accum.p, bytes, isDevicePtr(accum) ? cudaMemcpyDeviceToDevice
                                                                                  : cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_render(pppm_ctx* c, const pppm_camera* cam, const pppm_params* par, int32_t passes, float* accum) {
    if (passes < 0) return fail(c, PPPM_E_ARG, "render: negative pass count");
    int r = pppm_render_begin(c, cam, par);
    if (r) return r;
    for (int t = 1; t <= passes; t++)
        if ((r = pppm_render_pass(c, t, nullptr))) return r;
    return accum ? pppm_render_read(c, accum) : PPPM_OK;
}

int pppm_render_photons(pppm_ctx* c, float* out, int64_t cap, int64_t* n) {
    if (!c || !n || cap < 0 || (cap > 0 && !out)) return fail(c, PPPM_E_ARG, "render_photons: bad arguments");
    if (!c->rs.active) return fail(c, PPPM_E_STATE, "render_photons: no render");
    const int64_t cnt = std::min<int64_t>(c->rs.storedLast, c->rs.depositCap);
    *n = cnt;
    const int64_t m = std::min(cnt, cap);
    if (m > 0) {
        void* dout;
        int r;
        if ((r = stageOut(c, out, (size_t)m * 32, 0, &dout))) return r;
        PPPM_CUDA(c, launchUnpackRecords(c->rs.photons.as<float4>(), m, (float*)dout, c->stream));
        if ((r = finishOut(c, out, dout, (size_t)m * 32))) return r;
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PPPM_OK;
}

int pppm_render_queries(pppm_ctx* c, float* out, int64_t cap, int64_t* n) {
    if (!c || !n || cap < 0 || (cap > 0 && !out)) return fail(c, PPPM_E_ARG, "render_queries: bad arguments");
    if (!c->rs.active) return fail(c, PPPM_E_STATE, "render_queries: no render");
    const int64_t cnt = std::min<int64_t>(c->rs.queriesLast, (int64_t)c->rs.cam.width * c->rs.cam.height);
    *n = cnt;
    const int64_t m = std::min(cnt, cap);
    if (m > 0) {
        // 3 float4 per query as the eye kernel wrote them: (position, pixel
        // as int bits), (oriented normal, 0), (path weight * refl / roulette, 0)
        void* dout;
        int r;
        if ((r = stageOut(c, out, (size_t)m * 48, 0, &dout))) return r;
        PPPM_CUDA(c, cudaMemcpyAsync(dout, c->rs.queries.p, (size_t)m * 48, cudaMemcpyDeviceToDevice, c->stream));
        if ((r = finishOut(c, out, dout, (size_t)m * 48))) return r;
        PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PPPM_OK;
}

}  // extern "C"
