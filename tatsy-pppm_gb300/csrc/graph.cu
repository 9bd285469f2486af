// Canonical render passes as one CUDA graph.
//
// A canonical pass without the subsurface stage, the learned proposal or
// traversal counting needs the host only to size its buffers and to read its
// counters. With the capacities fixed in advance (the photon buffer at 1.5x
// the most photons one pass stored so far, the grid table and sort buffers
// for that capacity, the queries for one per pixel), the whole pass is a
// fixed sequence of memsets, kernels, events and one counter copy into
// pinned host memory, and consecutive passes differ only in their kernel
// parameters (pass index and radius, which follow a schedule the host
// knows). graphEnqueuePass records one pass into a stream under capture:
// photons on the context stream, eye paths on the side stream (joined before
// the gather). graphFinishPass reads the pass's counters after the graph
// ran. pppm_render_graph captures the next passes of one render; the batch
// captures the remaining passes of all its eligible jobs into one graph.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "trace.h"

namespace pppm {

namespace {

// stage timing per captured pass (event record nodes cost a few
// microseconds each): start, eye paths done (or photons emitted, with the
// side stream), photon bounces done, gather done
constexpr int kPassEvents = 4;

}  // namespace

bool graphEligible(const pppm_ctx* c) {
    const RenderState& rs = c->rs;
    return rs.active && rs.par.mode == PPPM_MODE_CANONICAL && !rs.sss.enabled && !rs.guide.enabled &&
           !(rs.par.flags & PPPM_FLAG_COUNT_TRAVERSAL);
}

int graphPrepare(pppm_ctx* c, int count) {
    RenderState& rs = c->rs;
    const int64_t want = std::max<int64_t>(rs.depositCap, rs.storedMax + rs.storedMax / 2 + 1024);
    if (want > rs.depositCap) {
        rs.depositCap = want;
        PPPM_CUDA(c, rs.photons.ensure((size_t)want * 32));
    }
    PPPM_CUDA(c, gridLayout(rs.grid, c->bbmin, c->bbmax, std::max(rs.radius * rs.par.cell_factor, 1e-30),
                            rs.depositCap));
    PPPM_CUDA(c, rs.grid.keys.ensure((size_t)rs.depositCap * 4));
    PPPM_CUDA(c, rs.grid.sorted.ensure((size_t)rs.depositCap * 32));
    PPPM_CUDA(c, rs.graphSlots.ensure((size_t)count * sizeof(PassCounters)));
    const size_t nev = (size_t)count * kPassEvents;
    while (c->graphEvents.size() < nev) {
        cudaEvent_t e;
        PPPM_CUDA(c, cudaEventCreate(&e));
        c->graphEvents.push_back(e);
    }
    return PPPM_OK;
}

PassCounters* graphSlot(pppm_ctx* c, int i) { return c->rs.graphSlots.as<PassCounters>() + i; }

int graphEnqueuePass(pppm_ctx* c, int t, int slot, bool sideEye) {
    RenderState& rs = c->rs;
    const pppm_params& par = rs.par;
    const int64_t paths = par.photons;
    const int64_t pixels = (int64_t)rs.cam.width * rs.cam.height;
    TraceParams tp;
    CameraDev cd;
    passSetup(c, t, paths, &tp, &cd);
    const SceneView sv = sceneView(c);
    const EnvDev ev = envView(c);
    // stage timing: event record nodes of the graph (external records); the
    // fork and join of the side stream are capture dependencies only
    cudaEvent_t* e = c->graphEvents.data() + (size_t)slot * kPassEvents;
    PassCounters* ctr = rs.photonCount.as<PassCounters>();
    PPPM_CUDA(c, cudaEventRecordWithFlags(e[0], c->stream, cudaEventRecordExternal));
    PPPM_CUDA(c, cudaMemsetAsync(ctr, 0, sizeof(PassCounters), c->stream));
    // eye paths: beside the photon pass on the side stream, or first on the
    // context stream (in the batch graph the other jobs fill the GPU, and a
    // fork per pass costs more than it overlaps)
    cudaStream_t eyeSt = c->stream;
    if (sideEye) {
        PPPM_CUDA(c, cudaEventRecord(c->ev[8], c->stream));
        PPPM_CUDA(c, cudaStreamWaitEvent(c->side, c->ev[8], 0));
        eyeSt = c->side;
    }
    PPPM_CUDA(c, launchEyeTrace(tp, sv, ev, cd, sssView(c), nullptr, rs.accum.as<float>(), rs.queries.as<float4>(),
                                rs.sss.queue.as<float4>(), rs.sss.queueCap, ctr, eyeSt));
    if (sideEye) PPPM_CUDA(c, cudaEventRecord(c->ev[10], c->side));
    else PPPM_CUDA(c, cudaEventRecordWithFlags(e[1], c->stream, cudaEventRecordExternal));
    // photons: two wavefront bounces, then the tail
    const uint32_t* perm = nullptr;
    const PathState* traced = nullptr;
    {
        int64_t emitLaunches = 0;
        const int r = emitPhotonPaths(c, tp, ev, nullptr, ctr, kPersistentPhotons, &traced, &perm, &emitLaunches);
        if (r) return r;
    }
    if (sideEye) PPPM_CUDA(c, cudaEventRecordWithFlags(e[1], c->stream, cudaEventRecordExternal));
    const int waves = kPersistentPhotons ? 0 : std::min(par.max_bounce_photon, kWaveBounces);
    if (kPersistentPhotons && par.max_bounce_photon > 0)
        PPPM_CUDA(c, launchPhotonPersistent(tp, sv, traced, paths, rs.photons.as<float4>(), rs.depositCap, ctr,
                                            c->stream, perm));
    for (int b = 0; b < waves; b++) {
        PathState* in = (b & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
        PathState* out = (b & 1) ? rs.pathA.as<PathState>() : rs.pathB.as<PathState>();
        PPPM_CUDA(c, launchPhotonBounce(tp, sv, b, in, out, paths, rs.photons.as<float4>(), rs.depositCap, ctr,
                                        c->stream));
    }
    if (!kPersistentPhotons && waves < par.max_bounce_photon) {
        PathState* in = (waves & 1) ? rs.pathB.as<PathState>() : rs.pathA.as<PathState>();
        PPPM_CUDA(c, launchPhotonTail(tp, sv, waves, in, paths, rs.photons.as<float4>(), rs.depositCap, ctr, c->stream));
    }
    PPPM_CUDA(c, cudaEventRecordWithFlags(e[2], c->stream, cudaEventRecordExternal));
    // photon map: the table sized for the capacity, the cells for this pass's radius
    PPPM_CUDA(c, gridLayout(rs.grid, c->bbmin, c->bbmax, par.cell_factor * rs.radius, rs.depositCap));
    GridDev gv = gridView(rs.grid, c->bbmin, c->bbmax);
    PPPM_CUDA(c, gridBuild(rs.grid, gv, rs.photons.as<float4>(), reinterpret_cast<const uint64_t*>(&ctr->deposits),
                           rs.depositCap, c->stream));
    gv = gridView(rs.grid, c->bbmin, c->bbmax);
    if (sideEye) PPPM_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev[10], 0));
    QueryView qv{rs.queries.as<float4>(), reinterpret_cast<const uint32_t*>(&ctr->queries), pixels};
    PPPM_CUDA(c, launchGatherTiled(gv, qv, rs.qsort, (float)rs.radius, rs.accum.as<float>(), true, nullptr, c->stream));
    PPPM_CUDA(c, cudaEventRecordWithFlags(e[3], c->stream, cudaEventRecordExternal));
    PPPM_CUDA(c, cudaMemcpyAsync(graphSlot(c, slot), ctr, sizeof(PassCounters), cudaMemcpyDeviceToHost, c->stream));
    // Knaus-Zwicker radius schedule, as pppm_render_pass
    rs.graphRadius.resize(std::max<size_t>(rs.graphRadius.size(), (size_t)slot + 1));
    rs.graphRadius[slot] = rs.radius;
    rs.graphSideEye = sideEye;
    rs.radius = rs.radius * std::sqrt((t + par.alpha) / (t + 1.0));
    rs.passesDone = t;
    return PPPM_OK;
}

int graphFinishPass(pppm_ctx* c, int slot, pppm_pass_stats* st, double* msPass) {
    RenderState& rs = c->rs;
    const PassCounters& hc = *graphSlot(c, slot);
    const cudaEvent_t* e = c->graphEvents.data() + (size_t)slot * kPassEvents;
    if ((int64_t)hc.deposits > rs.depositCap)
        return fail(c, PPPM_E_CAPACITY, "render_graph: a captured pass stored more photons than its fixed capacity");
    if (hc.undefinedEmit)
        return fail(c, PPPM_E_UNDEFINED, "render_graph: a photon draw fell past the env CDF");
    if (hc.undefinedEye) return fail(c, PPPM_E_CAPACITY, "render_graph: an eye path exceeded 4096 segments");
    rs.storedLast = (int64_t)hc.deposits;
    rs.queriesLast = (int64_t)hc.queries;
    rs.storedMax = std::max(rs.storedMax, rs.storedLast);
    float ms = 0.0f;
    if (msPass) *msPass = cudaEventElapsedTime(&ms, e[0], e[3]) == cudaSuccess ? ms : 0.0;
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->photons_traced = rs.par.photons;
        st->photons_stored = (int64_t)hc.deposits;
        st->photon_rays = (int64_t)hc.photonRays;
        st->eye_rays = (int64_t)hc.eyeRays;
        st->gather_queries = (int64_t)hc.queries;
        st->radius = rs.graphRadius[slot];
        // side stream: e0..e1 emission, e1..e2 bounces (eye paths alongside);
        // else e0..e1 eye paths, e1..e2 photon pass. e2..e3: grid + gather.
        if (rs.graphSideEye) {
            if (cudaEventElapsedTime(&ms, e[0], e[2]) == cudaSuccess) st->ms_photon = ms;
            if (cudaEventElapsedTime(&ms, e[1], e[2]) == cudaSuccess) st->ms_bounce = ms;
        } else {
            if (cudaEventElapsedTime(&ms, e[0], e[1]) == cudaSuccess) st->ms_eye = ms;
            if (cudaEventElapsedTime(&ms, e[1], e[2]) == cudaSuccess) st->ms_photon = ms;
        }
        if (cudaEventElapsedTime(&ms, e[2], e[3]) == cudaSuccess) st->ms_gather = ms;
        // emit, bounces, eye, grid (keys, scan 3, scatter), gather (keys, scan 3, scatter, gather)
        st->kernel_launches = 2 + std::min(rs.par.max_bounce_photon, kWaveBounces) +
                              (kWaveBounces < rs.par.max_bounce_photon ? 1 : 0) + 5 + 6;
    }
    cudaGetLastError();
    return PPPM_OK;
}

// A capture on `st` that failed after it began: end it and drop the graph.
void graphAbort(cudaStream_t st) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
}

int graphRun(pppm_ctx* c, cudaGraph_t g, cudaStream_t st, double* instantiateMs) {
    cudaGraphExec_t exec = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    if (instantiateMs)
        *instantiateMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(c, PPPM_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    e = cudaGraphLaunch(exec, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) return fail(c, PPPM_E_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    return PPPM_OK;
}

}  // namespace pppm

using namespace pppm;

extern "C" int pppm_render_graph(pppm_ctx* c, int32_t count, pppm_pass_stats* stats) {
    if (!c || count < 1) return fail(c, PPPM_E_ARG, "render_graph: bad arguments");
    RenderState& rs = c->rs;
    if (!rs.active) return fail(c, PPPM_E_STATE, "render_graph: call render_begin first");
    if (!graphEligible(c))
        return fail(c, PPPM_E_STATE,
                    "render_graph: canonical renders without subsurface scattering, learned proposal or traversal "
                    "counting only");
    cudaSetDevice(c->device);
    int done = 0;
    if (rs.passesDone == 0) {
        // the first pass sizes the photon buffer
        const int r = pppm_render_pass(c, 1, stats ? &stats[0] : nullptr);
        if (r) return r;
        done = 1;
    }
    const int n = count - done;
    if (n == 0) return PPPM_OK;
    int r = graphPrepare(c, n);
    if (r) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    const double radius0 = rs.radius;
    const int passes0 = rs.passesDone;
    PPPM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < n; i++) {
        r = graphEnqueuePass(c, passes0 + 1 + i, i, true);
        if (r) {
            graphAbort(c->stream);
            rs.radius = radius0;
            rs.passesDone = passes0;
            return r;
        }
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (ce != cudaSuccess || !g) {
        rs.radius = radius0;
        rs.passesDone = passes0;
        cudaGetLastError();
        return fail(c, PPPM_E_CUDA, std::string("render_graph: capture: ") + cudaGetErrorString(ce));
    }
    if ((r = graphRun(c, g, c->stream))) return r;
    for (int i = 0; i < n; i++)
        if ((r = graphFinishPass(c, i, stats ? &stats[done + i] : nullptr, nullptr))) return r;
    return PPPM_OK;
}
