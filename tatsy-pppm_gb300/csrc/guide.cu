// Host side of the learned photon proposal in a canonical render: state set
// up at render_begin, the emission mixture of each pass, the per-bounce
// network step, the importance grid after the eye pass, and the retraining
// schedule (every 2 passes: 2 Adam steps of 65,536 records at lr 4e-3).
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>

#include "context.h"
#include "trace.h"

namespace pppm {

int guideBegin(pppm_ctx* c, int64_t maxPaths) {
    GuideState& g = c->rs.guide;
    const pppm_params& par = c->rs.par;
    g.enabled = par.mode == PPPM_MODE_CANONICAL && (par.flags & PPPM_FLAG_LEARNED);
    g.trained = false;
    g.adamStep = 0;
    g.impValid = false;
    g.cur = 0;
    g.msTrain = 0.0;
    g.lastLoss = 0.0f;
    g.lastRecords = 0;
    if (!g.enabled) return PPPM_OK;
    // He initialisation, seeded by the render seed
    std::vector<float> p(kMlpParams, 0.0f);
    std::mt19937_64 rng(0x5eed0000ull + par.seed);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    for (int l = 0; l < kMlpLayers; l++) {
        const float s = std::sqrt(2.0f / (float)mlpK(l));
        for (int i = 0; i < mlpNReal(l) * mlpK(l); i++) p[mlpWOffset(l) + i] = nd(rng) * s;
    }
    PPPM_CUDA(c, g.params.ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, g.adamM.ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, g.adamV.ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, g.grad.ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, g.blob.ensure((size_t)kMlpBlobBytes));
    PPPM_CUDA(c, g.misc.ensure(64));
    PPPM_CUDA(c, g.counters.ensure(64));
    PPPM_CUDA(c, cudaMemcpyAsync(g.params.p, p.data(), p.size() * 4, cudaMemcpyHostToDevice, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(g.adamM.p, 0, (size_t)kMlpParams * 4, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(g.adamV.p, 0, (size_t)kMlpParams * 4, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(g.blob.p, 0, (size_t)kMlpBlobBytes, c->stream));
    PPPM_CUDA(c, launchMlpPack(g.params.as<float>(), g.blob.as<uint8_t>(), c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(g.counters.p, 0, 64, c->stream));
    PPPM_CUDA(c, g.raw.ensure((size_t)maxPaths * kMlpOut * 4));
    PPPM_CUDA(c, g.inPos.ensure((size_t)maxPaths * 12));
    PPPM_CUDA(c, g.inNrm.ensure((size_t)maxPaths * 12));
    g.recCap = std::max<int64_t>(g.batch * 8, 1 << 20);
    PPPM_CUDA(c, g.rec.ensure((size_t)g.recCap * sizeof(MlpRecord)));
    // importance grid: cubic voxels over the scene box
    const double ext = std::max({c->bbmax[0] - c->bbmin[0], c->bbmax[1] - c->bbmin[1], c->bbmax[2] - c->bbmin[2],
                                 1e-6});
    const double vox = ext * 1.001 / g.G;
    g.gox = (float)(c->bbmin[0] - 0.0005 * ext);
    g.goy = (float)(c->bbmin[1] - 0.0005 * ext);
    g.goz = (float)(c->bbmin[2] - 0.0005 * ext);
    g.ginv = (float)(1.0 / vox);
    for (int k = 0; k < 2; k++) {
        PPPM_CUDA(c, g.imp[k].ensure((size_t)g.G * g.G * g.G * 4));
        PPPM_CUDA(c, cudaMemsetAsync(g.imp[k].p, 0, (size_t)g.G * g.G * g.G * 4, c->stream));
    }
    // network input box: the scene and the emission sphere of radius 50
    for (int d = 0; d < 3; d++) {
        g.box[d] = std::min(c->bbmin[d], -50.0);
        g.box[3 + d] = std::max(c->bbmax[d], 50.0);
    }
    // the emission distribution's input: the box centre with a zero normal
    // (surface rows carry unit normals)
    const float ein[6] = {(float)(0.5 * (g.box[0] + g.box[3])), (float)(0.5 * (g.box[1] + g.box[4])),
                          (float)(0.5 * (g.box[2] + g.box[5])), 0.0f, 0.0f, 0.0f};
    PPPM_CUDA(c, g.emitIn.ensure(sizeof(ein)));
    PPPM_CUDA(c, g.emitRaw.ensure((size_t)kMlpOut * 4));
    PPPM_CUDA(c, cudaMemcpy(g.emitIn.p, ein, sizeof(ein), cudaMemcpyHostToDevice));
    return PPPM_OK;
}

GuideView guideView(pppm_ctx* c, int64_t decisionsPerPass) {
    GuideState& g = c->rs.guide;
    GuideView v;
    std::memset(&v, 0, sizeof(v));
    if (!g.enabled) return v;
    v.rec = g.rec.as<MlpRecord>();
    v.recCount = g.counters.as<unsigned long long>();
    v.recCap = g.recCap;
    // about two batches of records per pass
    const int64_t want = 2 * g.batch;
    v.recEvery = (uint32_t)std::max<int64_t>(1, decisionsPerPass / want);
    v.imp = g.impValid ? g.imp[g.cur].as<float>() : nullptr;
    v.G = g.G;
    v.ox = g.gox;
    v.oy = g.goy;
    v.oz = g.goz;
    v.inv = g.ginv;
    v.maxLogKappa = g.maxLogKappa;
    v.guideBounces = g.guideBounces;
    v.emitRaw = g.trained ? g.emitRaw.as<float>() : nullptr;
    v.emitFloor = g.floorBsdf;
    // Envmap::samplePhoton's flux factor area / (pdf numPhotons) without the pdf
    const double area = ((double)((unsigned)c->envW * (unsigned)c->envH)) / (4.0 * 3.14159265358979323846 * 64 * 64);
    v.emitK = (float)(area / (double)c->rs.par.photons);
    v.epx = (float)(0.5 * (g.box[0] + g.box[3]));
    v.epy = (float)(0.5 * (g.box[1] + g.box[4]));
    v.epz = (float)(0.5 * (g.box[2] + g.box[5]));
    return v;
}

// The network's environment-direction mixture for this pass: one row, the
// emission input.
int guideEmission(pppm_ctx* c) {
    GuideState& g = c->rs.guide;
    const float* in = g.emitIn.as<float>();
    PPPM_CUDA(c, launchMlpForward(mlpInputs(g.box, in, in + 3), g.blob.as<uint8_t>(), 1, g.emitRaw.as<float>(),
                                  reinterpret_cast<int*>(g.misc.as<float>() + 1), c->stream));
    return PPPM_OK;
}

// Directions of the pending paths of queue q (count on the device).
int guideStep(pppm_ctx* c, const TraceParams& tp, PathState* q, const unsigned long long* count, int64_t cap,
              int bounce) {
    GuideState& g = c->rs.guide;
    const float* raw = nullptr;
    if (g.trained) {
        PPPM_CUDA(c, launchGuidePack(q, count, cap, g.inPos.as<float>(), g.inNrm.as<float>(), c->stream));
        const MlpInputs in = mlpInputs(g.box, g.inPos.as<float>(), g.inNrm.as<float>());
        PPPM_CUDA(c, launchMlpForward(in, g.blob.as<uint8_t>(), cap, g.raw.as<float>(),
                                      reinterpret_cast<int*>(g.misc.as<float>() + 1), c->stream, count));
        raw = g.raw.as<float>();
    }
    PPPM_CUDA(c, launchGuideResolve(tp, q, count, cap, raw, g.floorBsdf, bounce, c->stream));
    return PPPM_OK;
}

// Importance of this pass's gather queries into the other grid.
int guideImportance(pppm_ctx* c, const float4* queries, const unsigned long long* count, int64_t cap, int t) {
    GuideState& g = c->rs.guide;
    const int next = g.cur ^ 1;
    PPPM_CUDA(c, cudaMemsetAsync(g.imp[next].p, 0, (size_t)g.G * g.G * g.G * 4, c->stream));
    GuideView v = guideView(c, 1);
    // pixel estimate: the accumulator holds passes 1..t-1 and this pass's
    // paths that ended in the environment
    PPPM_CUDA(c, launchImportanceSplat(v, queries, count, cap, c->rs.accum.as<float>(), 1.0f / (float)t, g.floorLum,
                                       g.imp[next].as<float>(), c->stream));
    return PPPM_OK;
}

// End of pass t: swap the importance grids; every retrainEvery passes run
// the Adam steps on the records gathered since the last training.
int guideEndPass(pppm_ctx* c, int t) {
    GuideState& g = c->rs.guide;
    g.cur ^= 1;
    g.impValid = true;
    g.msTrain = 0.0;
    if (t % g.retrainEvery != 0 || (c->rs.par.flags & PPPM_FLAG_LEARNED_FROZEN)) return PPPM_OK;
    unsigned long long cnt = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&cnt, g.counters.p, 8, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    const int64_t n = std::min<int64_t>((int64_t)cnt, g.recCap);
    g.lastRecords = n;
    if (n < g.batch) return PPPM_OK;
    const auto t0 = std::chrono::steady_clock::now();
    float* misc = g.misc.as<float>();
    PPPM_CUDA(c, cudaMemsetAsync(misc, 0, 8, c->stream));
    const MlpInputs box = mlpInputs(g.box, nullptr, nullptr);
    const int64_t windows = std::max<int64_t>(1, n / g.batch);
    for (int s = 0; s < g.stepsPerTrain; s++) {
        const MlpRecord* r = g.rec.as<MlpRecord>() + (s % windows) * g.batch;
        PPPM_CUDA(c, cudaMemsetAsync(g.grad.p, 0, (size_t)kMlpParams * 4, c->stream));
        if (s == g.stepsPerTrain - 1) PPPM_CUDA(c, cudaMemsetAsync(misc, 0, 4, c->stream));
        PPPM_CUDA(c, launchRecordInvSum(r, g.batch, misc + 2, c->stream));
        PPPM_CUDA(c, launchMlpTrain(r, g.batch, misc + 2, box, g.blob.as<uint8_t>(), g.grad.as<float>(), misc,
                                    reinterpret_cast<int*>(misc + 1), c->stream, g.maxLogKappa));
        g.adamStep++;
        PPPM_CUDA(c, launchMlpAdam(g.params.as<float>(), g.grad.as<float>(), g.adamM.as<float>(), g.adamV.as<float>(),
                                   g.adamStep, g.lr, c->stream));
        PPPM_CUDA(c, launchMlpPack(g.params.as<float>(), g.blob.as<uint8_t>(), c->stream));
    }
    float hm[2];
    PPPM_CUDA(c, cudaMemcpyAsync(hm, misc, 8, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(g.counters.p, 0, 8, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    int e;
    std::memcpy(&e, &hm[1], 4);
    if (e) return fail(c, PPPM_E_CUDA, "learned proposal: a tensor-core wait timed out");
    g.lastLoss = hm[0];
    g.trained = true;
    g.msTrain = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return PPPM_OK;
}

}  // namespace pppm

using namespace pppm;

extern "C" int pppm_learned_config(pppm_ctx* c, int32_t retrainEvery, int32_t steps, int64_t batch, float lr,
                                   float floorBsdf, float maxLogKappa, int32_t guideBounces) {
    if (!c) return PPPM_E_ARG;
    GuideState& g = c->rs.guide;
    if (floorBsdf > 1.0f || (batch > 0 && batch % 128 != 0))
        return fail(c, PPPM_E_ARG, "learned_config: floor_bsdf must be <= 1 and batch a multiple of 128");
    if (retrainEvery > 0) g.retrainEvery = retrainEvery;
    if (steps > 0) g.stepsPerTrain = steps;
    if (batch > 0) g.batch = batch;
    if (lr > 0.0f) g.lr = lr;
    if (floorBsdf > 0.0f) g.floorBsdf = floorBsdf;
    if (maxLogKappa > 0.0f) g.maxLogKappa = maxLogKappa;
    if (guideBounces >= 0) g.guideBounces = guideBounces ? 1 : 0;
    return PPPM_OK;
}
