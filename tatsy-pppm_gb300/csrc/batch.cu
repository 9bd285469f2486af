// Batched uneven render jobs: each job owns a context (scene, BVH, env map,
// render state, stream); worker threads drive up to max_concurrent jobs at a
// time, so their kernels overlap on the GPU, longest jobs first.
//
// Autotuning: a job's passes after the first try the launch shapes of a
// candidate table (every pppm_tune knob: hash cell factor, photon and eye
// blocks per SM, refill threshold, exact-test batch, gather tile, query
// sort sub-cells; no knob changes a result), each candidate for kRounds
// passes in interleaved rounds (forward, backward, forward, so that the
// shrinking radius favours no candidate), and the rest of the job runs the
// candidate with the lowest median device time per pass. The tuning passes
// are real passes of the render.
//
// Jobs that can be captured (canonical, no subsurface stage, no learned
// proposal) run everything after their first pass in two CUDA graphs, one
// branch per job: the first holds the tuning passes of all jobs (each
// captured with its candidate's knobs, timed by the graph's event nodes),
// the second the remaining passes with each job's choice. Other jobs tune
// eagerly. Per-pass latencies are recorded per job. No counterpart in the
// reference (its render() handles one scene at a time).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "context.h"

using namespace pppm;

struct pppm_batch {
    int device = 0;
    struct Job {
        pppm_ctx* ctx = nullptr;
        pppm_camera cam{};
        pppm_params par{};
        int passes = 0;
        double work = 0.0;  // photons x passes + pixels x passes: scheduling order
        std::vector<double> passMs;
        int64_t rays = 0;
        float cell = 1.0f;
        int bounceBlocks = 16, eyeBlocks = 16;
        pppm_tune base{};         // knobs the render began with
        pppm_tune tune{};         // knobs after the tuning
        std::vector<int> plan;    // candidate of each tuning pass
        int chosen = -1;          // candidate kept (-1: no tuning)
        bool graph = false;       // passes after the first go into the batch graphs
        int graphPasses = 0;      // of which plan.size() in the tuning graph
        int status = PPPM_OK;
        std::string err;
    };
    std::vector<Job> jobs;
    double wallMs = 0.0;
    double graphMs = 0.0;  // capture, instantiation and run of the graph
    double graphCaptureMs = 0.0, graphInstantiateMs = 0.0;
    bool useGraph = true;
    int graphLanes = 0;  // jobs at once inside the graph (0: 2 x max_concurrent)
    std::string err;
};

namespace {

int jobFail(pppm_batch::Job& j, int code) {
    j.status = code;
    j.err = pppm_last_error(j.ctx);
    return code;
}

// Candidate launch shapes: the defaults first, then variants along every
// knob (cell factor, bounce and eye blocks per SM, refill, exact batch,
// gather tile, query sub-cell bits). A job with P passes tries the first
// min(6, (P - 2) / kRounds) of them.
// query_sub_bits -1: the render's own choice (set by the image size)
const pppm_tune kCandidates[] = {
    {1.0f, 64, 128, 24, 12, 128, -1}, {1.25f, 64, 64, 24, 12, 256, 2}, {1.0f, 32, 32, 16, 8, 128, 3},
    {1.0f, 64, 128, 32, 16, 64, 1},   {1.5f, 64, 128, 24, 12, 256, 2}, {1.0f, 5, 32, 24, 12, 128, -1},
};
constexpr int kNumCandidates = (int)(sizeof(kCandidates) / sizeof(kCandidates[0]));
constexpr int kRounds = 3;  // timed passes per candidate

// The knobs of candidate k for a render of this mode (base: the knobs the
// render began with): compat renders keep their cell size (it follows k)
// and use the kNN gather (no tiles).
pppm_tune candidate(int k, bool canonical, const pppm_tune& base) {
    pppm_tune t = kCandidates[k];
    if (t.query_sub_bits < 0) t.query_sub_bits = base.query_sub_bits;
    if (!canonical) {
        t.cell_factor = 0.0f;
        t.gather_stage = -1;
        t.query_sub_bits = -1;
    }
    return t;
}

// Tuning passes of a job with `passes` passes: candidates in rounds of
// alternating order, kRounds passes each; none when the job is too short.
std::vector<int> tuningPlan(int passes, bool autotune) {
    std::vector<int> plan;
    const int k = autotune ? std::min(kNumCandidates, std::max(0, (passes - 2) / kRounds)) : 0;
    if (k < 2) return plan;
    for (int r = 0; r < kRounds; r++)
        for (int i = 0; i < k; i++) plan.push_back((r & 1) ? k - 1 - i : i);
    return plan;
}

// The candidate with the lowest median device time over its tuning passes
// (ms[i]: device time of tuning pass i).
int bestCandidate(const std::vector<int>& plan, const std::vector<double>& ms) {
    int best = 0;
    double bestMs = 1e300;
    for (int k = 0; k < kNumCandidates; k++) {
        std::vector<double> v;
        for (size_t i = 0; i < plan.size() && i < ms.size(); i++)
            if (plan[i] == k) v.push_back(ms[i]);
        if (v.empty()) continue;
        std::sort(v.begin(), v.end());
        const double m = v[v.size() / 2];
        if (m < bestMs) {
            bestMs = m;
            best = k;
        }
    }
    return best;
}

void recordShape(pppm_batch::Job& j) {
    pppm_render_get_tune(j.ctx, &j.tune);
    j.cell = j.tune.cell_factor;
    j.bounceBlocks = j.tune.bounce_blocks_per_sm;
    j.eyeBlocks = j.tune.eye_blocks_per_sm;
}

int runJob(pppm_batch::Job& j, bool autotune, bool useGraph) {
    pppm_ctx* c = j.ctx;
    int r = pppm_render_begin(c, &j.cam, &j.par);
    if (r) return jobFail(j, r);
    pppm_render_get_tune(c, &j.base);
    const bool canonical = j.par.mode == PPPM_MODE_CANONICAL;
    j.plan = tuningPlan(j.passes, autotune);
    j.chosen = -1;
    // pass 1 pays the allocations (default shape); with the graphs, every
    // later pass (tuning included) is captured
    j.graph = useGraph && graphEligible(c) && j.passes > 1;
    const int eager = j.graph ? 1 : j.passes;
    j.graphPasses = j.passes - eager;
    const int nPlan = (int)j.plan.size();
    std::vector<double> dev;
    for (int t = 1; t <= eager; t++) {
        const int i = t - 2;  // tuning pass index
        if (i >= 0 && i < nPlan) {
            const pppm_tune s = candidate(j.plan[i], canonical, j.base);
            pppm_render_tune_ex(c, &s);
        } else if (nPlan > 0 && i == nPlan) {
            j.chosen = bestCandidate(j.plan, dev);
            const pppm_tune s = candidate(j.chosen, canonical, j.base);
            pppm_render_tune_ex(c, &s);
        }
        pppm_pass_stats st;
        const auto t0 = std::chrono::steady_clock::now();
        r = pppm_render_pass(c, t, &st);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (r) return jobFail(j, r);
        j.passMs.push_back(ms);
        j.rays += st.photon_rays + st.eye_rays;
        // device time of the stages the knobs affect
        if (i >= 0 && i < nPlan) dev.push_back(st.ms_photon + st.ms_grid + st.ms_eye + st.ms_gather);
    }
    recordShape(j);
    return PPPM_OK;
}

// Passes of the graph jobs: one capture on `origin`, one launch. tuning:
// each job's tuning passes, each captured with its candidate's knobs; else
// the passes after them. Each job is a branch (its context stream); the
// branches form `lanes` chains. Jobs go, longest first, to the chain with
// the least work so far (the work of a job: its passes in this graph times
// the median of its passes so far), so at most `lanes` jobs run at once and
// the chains end close together.
int passesIn(const pppm_batch::Job& j, bool tuning) {
    return tuning ? (int)j.plan.size() : j.graphPasses - (int)j.plan.size();
}

int runGraph(pppm_batch* b, std::vector<pppm_batch::Job*>& gj, int lanes, bool tuning) {
    cudaSetDevice(b->device);
    for (auto* j : gj) {
        const int r = graphPrepare(j->ctx, passesIn(*j, tuning));
        if (r) return jobFail(*j, r);
        if (cudaStreamSynchronize(j->ctx->stream) != cudaSuccess) return jobFail(*j, PPPM_E_CUDA);
    }
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join(gj.size(), nullptr);
    auto cleanup = [&]() {
        for (auto e : join)
            if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (origin) cudaStreamDestroy(origin);
    };
    auto failAll = [&](const std::string& msg) {
        for (auto* j : gj) {
            j->status = PPPM_E_CUDA;
            j->err = msg;
        }
        cleanup();
        return PPPM_E_CUDA;
    };
    if (cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess)
        return failAll("batch graph: cannot create its stream");
    for (auto& e : join)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return failAll("batch graph: cannot create its events");
    const auto t0 = std::chrono::steady_clock::now();
    if (cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess ||
        cudaEventRecord(fork, origin) != cudaSuccess)
        return failAll("batch graph: cannot begin the capture");
    lanes = std::max(1, std::min<int>(lanes, (int)gj.size()));
    std::vector<double> est(gj.size());
    for (size_t k = 0; k < gj.size(); k++) {
        std::vector<double> s(gj[k]->passMs.begin() + std::min<size_t>(1, gj[k]->passMs.size()), gj[k]->passMs.end());
        std::sort(s.begin(), s.end());
        est[k] = (s.empty() ? 1.0 : s[s.size() / 2]) * passesIn(*gj[k], tuning);
    }
    std::vector<size_t> order(gj.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = k;
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return est[x] > est[y]; });
    std::vector<double> laneWork(lanes, 0.0);
    std::vector<int> laneLast(lanes, -1);  // last job of each chain
    for (size_t k : order) {
        const int l = (int)(std::min_element(laneWork.begin(), laneWork.end()) - laneWork.begin());
        pppm_ctx* c = gj[k]->ctx;
        // after the fork, or after the previous job of its chain
        cudaStreamWaitEvent(c->stream, laneLast[l] >= 0 ? join[laneLast[l]] : fork, 0);
        laneWork[l] += est[k];
        laneLast[l] = (int)k;
        const int first = c->rs.passesDone + 1;
        const bool canonical = gj[k]->par.mode == PPPM_MODE_CANONICAL;
        for (int i = 0; i < passesIn(*gj[k], tuning); i++) {
            if (tuning) {
                const pppm_tune s = candidate(gj[k]->plan[i], canonical, gj[k]->base);
                pppm_render_tune_ex(c, &s);
            }
            const int r = graphEnqueuePass(c, first + i, i, false);
            if (r) {
                graphAbort(origin);
                return failAll(std::string("batch graph: ") + pppm_last_error(c));
            }
        }
        cudaEventRecord(join[k], c->stream);
    }
    for (int l = 0; l < lanes; l++)
        if (laneLast[l] >= 0) cudaStreamWaitEvent(origin, join[laneLast[l]], 0);
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(origin, &g) != cudaSuccess || !g) {
        cudaGetLastError();
        return failAll("batch graph: the capture failed");
    }
    b->graphCaptureMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    double instMs = 0.0;
    const int r = graphRun(gj[0]->ctx, g, origin, &instMs);
    b->graphInstantiateMs += instMs;
    b->graphMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (r) return failAll(std::string("batch graph: ") + pppm_last_error(gj[0]->ctx));
    for (auto* j : gj) {
        std::vector<double> dev;
        for (int i = 0; i < passesIn(*j, tuning); i++) {
            pppm_pass_stats st;
            double ms = 0.0;
            const int e = graphFinishPass(j->ctx, i, &st, &ms);
            if (e) {
                jobFail(*j, e);
                break;
            }
            j->passMs.push_back(ms);
            dev.push_back(ms);
            j->rays += st.photon_rays + st.eye_rays;
        }
        if (tuning && j->status == PPPM_OK) {
            // the remaining passes run the fastest candidate
            j->chosen = bestCandidate(j->plan, dev);
            const pppm_tune s = candidate(j->chosen, j->par.mode == PPPM_MODE_CANONICAL, j->base);
            pppm_render_tune_ex(j->ctx, &s);
            recordShape(*j);
        }
    }
    cleanup();
    return PPPM_OK;
}

}  // namespace

extern "C" {

int pppm_batch_create(int device, pppm_batch** out) {
    if (!out) return PPPM_E_ARG;
    *out = new (std::nothrow) pppm_batch();
    if (!*out) return PPPM_E_CAPACITY;
    (*out)->device = device;
    return PPPM_OK;
}

int pppm_batch_destroy(pppm_batch* b) {
    if (!b) return PPPM_E_ARG;
    for (auto& j : b->jobs)
        if (j.ctx) pppm_destroy(j.ctx);
    delete b;
    return PPPM_OK;
}

const char* pppm_batch_last_error(const pppm_batch* b) { return b ? b->err.c_str() : "null batch"; }

int pppm_batch_config(pppm_batch* b, int32_t use_graph, int32_t graph_lanes) {
    if (!b || graph_lanes < 0) return PPPM_E_ARG;
    b->useGraph = use_graph != 0;
    b->graphLanes = graph_lanes;
    return PPPM_OK;
}

int pppm_batch_submit(pppm_batch* b, const pppm_job* job, int32_t* job_id) {
    if (!b || !job || job->passes < 1) return PPPM_E_ARG;
    pppm_batch::Job j;
    int r = pppm_create(b->device, &j.ctx);
    if (r) {
        b->err = "batch_submit: cannot create a context";
        return r;
    }
    if ((r = pppm_scene_set(j.ctx, job->tri_xyz, job->ntri, job->mat_id, job->mats, job->nmat)) ||
        (r = pppm_env_set(j.ctx, job->env_rgb, job->env_w, job->env_h))) {
        b->err = std::string("batch_submit: ") + pppm_last_error(j.ctx);
        pppm_destroy(j.ctx);
        return r;
    }
    j.cam = job->camera;
    j.par = job->params;
    j.passes = job->passes;
    j.work = (double)job->passes * ((double)job->params.photons + (double)job->camera.width * job->camera.height);
    if (job_id) *job_id = (int32_t)b->jobs.size();
    b->jobs.push_back(std::move(j));
    return PPPM_OK;
}

int pppm_batch_run(pppm_batch* b, int32_t autotune, int32_t max_concurrent) {
    if (!b || max_concurrent < 1) return PPPM_E_ARG;
    std::vector<int> order(b->jobs.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return b->jobs[x].work > b->jobs[y].work; });
    std::atomic<size_t> next(0);
    const auto t0 = std::chrono::steady_clock::now();
    auto worker = [&]() {
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= order.size()) return;
            pppm_batch::Job& j = b->jobs[order[k]];
            j.passMs.clear();
            j.rays = 0;
            j.status = runJob(j, autotune != 0, b->useGraph);
        }
    };
    const int nw = std::min<int>(max_concurrent, (int)order.size());
    std::vector<std::thread> pool;
    for (int w = 0; w < nw; w++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    b->graphMs = b->graphCaptureMs = b->graphInstantiateMs = 0.0;
    // inside the graphs no host thread bounds the jobs in flight: twice as
    // many as the eager phase measured best on the batched workload
    const int lanes = b->graphLanes > 0 ? b->graphLanes : 2 * max_concurrent;
    for (const bool tuning : {true, false}) {
        std::vector<pppm_batch::Job*> gj;
        for (auto& j : b->jobs)
            if (j.status == PPPM_OK && j.graph && passesIn(j, tuning) > 0) gj.push_back(&j);
        if (!gj.empty()) runGraph(b, gj, lanes, tuning);
    }
    b->wallMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (auto& j : b->jobs)
        if (j.status) {
            b->err = "batch_run: " + j.err;
            return j.status;
        }
    return PPPM_OK;
}

int pppm_batch_result(pppm_batch* b, int32_t id, float* accum, pppm_job_stats* stats) {
    if (!b || id < 0 || id >= (int32_t)b->jobs.size()) return PPPM_E_ARG;
    pppm_batch::Job& j = b->jobs[id];
    if (accum) {
        const int r = pppm_render_read(j.ctx, accum);
        if (r) return r;
    }
    if (stats) {
        std::vector<double> s = j.passMs;
        std::sort(s.begin(), s.end());
        auto q = [&](double f) { return s.empty() ? 0.0 : s[std::min(s.size() - 1, (size_t)(f * (s.size() - 1) + 0.5))]; };
        stats->passes = (int32_t)j.passMs.size();
        stats->rays = j.rays;
        stats->ms_total = 0.0;
        for (double v : j.passMs) stats->ms_total += v;
        stats->ms_pass_p50 = q(0.5);
        stats->ms_pass_p99 = q(0.99);
        stats->cell_factor = j.cell;
        stats->bounce_blocks_per_sm = j.bounceBlocks;
        stats->eye_blocks_per_sm = j.eyeBlocks;
        stats->batch_wall_ms = b->wallMs;
        stats->graph_passes = j.graph ? j.graphPasses : 0;
        stats->batch_graph_ms = b->graphMs;
        stats->batch_graph_capture_ms = b->graphCaptureMs;
        stats->batch_graph_instantiate_ms = b->graphInstantiateMs;
        stats->refill = j.tune.refill;
        stats->exact_batch = j.tune.exact_batch;
        stats->gather_stage = j.tune.gather_stage;
        stats->query_sub_bits = j.tune.query_sub_bits;
        stats->tune_passes = (int32_t)j.plan.size();
        stats->tune_candidate = j.chosen;
    }
    return PPPM_OK;
}

}  // extern "C"
