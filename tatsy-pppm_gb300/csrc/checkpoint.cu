// Checkpoint and resume of a render (no counterpart in the reference: its
// render() keeps the accumulation buffer in memory and writes one image per
// pass). The checkpoint holds everything a later pass reads: the camera and
// parameters, the pass count and radius, the tuned launch shapes, the
// accumulation buffer, the per-stream XorShift states (compat and classic),
// the Poisson sampler's XorShift state (subsurface stage), the per-pixel
// render points of classic PPM, and the learned proposal's network, Adam
// moments, importance grids and pending training records. Loading it into a
// context holding the same scene and environment map continues the render
// as if it had not stopped.
#include <cstring>
#include <vector>

#include "context.h"
#include "trace.h"

namespace pppm {

namespace {

constexpr char kMagic[8] = {'P', 'P', 'P', 'M', 'C', 'K', 'P', '1'};

struct CkHeader {
    char magic[8];
    uint32_t version;
    uint32_t headerBytes;
    pppm_camera cam;
    pppm_params par;
    int32_t passesDone;
    int32_t bouncePerSm, eyePerSm;
    float cellFactor;
    double radius;
    int64_t storedLast, storedMax, depositCap;
    // scene identity: a checkpoint loads only into a context with this scene
    int64_t ntri;
    double bbmin[3], bbmax[3];
    int32_t envW, envH;
    uint32_t poissonRng[4];
    int32_t numStreams;
    int32_t classic;      // classic PPM arrays follow
    int32_t learned;      // learned-proposal state follows
    int32_t learnedTrained, learnedCur, learnedImpValid, learnedAdamStep;
    int64_t learnedRecords;
    double classicBbmin[3], classicScale, classicIrad;
};

// Sections in order: accumulation (W*H*3 floats); stream states (N x 16 B);
// classic arrays (pos, nrm, flux, weight, emission, r2, n, coeff); learned
// (params, adam m, adam v, importance grids 0 and 1, records).
struct Writer {
    uint8_t* out;
    int64_t cap;
    int64_t pos = 0;
    bool ok = true;
    cudaError_t err = cudaSuccess;
    void host(const void* p, size_t n) {
        if (out && pos + (int64_t)n <= cap) std::memcpy(out + pos, p, n);
        else if (out) ok = false;
        pos += (int64_t)n;
    }
    void device(const void* p, size_t n) {
        if (out && pos + (int64_t)n <= cap) {
            if (n) {
                const cudaError_t e = cudaMemcpy(out + pos, p, n, cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) err = e;
            }
        } else if (out) {
            ok = false;
        }
        pos += (int64_t)n;
    }
};

struct Reader {
    const uint8_t* in;
    int64_t size;
    int64_t pos = 0;
    bool ok = true;
    cudaError_t err = cudaSuccess;
    const uint8_t* take(size_t n) {
        if (pos + (int64_t)n > size) {
            ok = false;
            return nullptr;
        }
        const uint8_t* p = in + pos;
        pos += (int64_t)n;
        return p;
    }
    void device(void* dst, size_t n) {
        const uint8_t* p = take(n);
        if (p && n) {
            const cudaError_t e = cudaMemcpy(dst, p, n, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) err = e;
        }
    }
};

}  // namespace

}  // namespace pppm

using namespace pppm;

extern "C" {

int pppm_render_save(pppm_ctx* c, uint8_t* out, int64_t cap, int64_t* size) {
    if (!c || !size || (out && cap < 0)) return fail(c, PPPM_E_ARG, "render_save: bad arguments");
    RenderState& rs = c->rs;
    if (!rs.active) return fail(c, PPPM_E_STATE, "render_save: no render");
    cudaSetDevice(c->device);
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    const int64_t pixels = (int64_t)rs.cam.width * rs.cam.height;
    const bool classic = rs.par.mode == PPPM_MODE_CLASSIC;
    const GuideState& g = rs.guide;
    unsigned long long recs = 0;
    if (g.enabled) PPPM_CUDA(c, cudaMemcpy(&recs, g.counters.p, 8, cudaMemcpyDeviceToHost));
    const int64_t nrec = g.enabled ? std::min<int64_t>((int64_t)recs, g.recCap) : 0;
    CkHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = 1;
    h.headerBytes = sizeof(CkHeader);
    h.cam = rs.cam;
    h.par = rs.par;
    h.passesDone = rs.passesDone;
    h.bouncePerSm = rs.bouncePerSm;
    h.eyePerSm = rs.eyePerSm;
    h.cellFactor = rs.par.cell_factor;
    h.radius = rs.radius;
    h.storedLast = rs.storedLast;
    h.storedMax = rs.storedMax;
    h.depositCap = rs.depositCap;
    h.ntri = c->ntri;
    for (int d = 0; d < 3; d++) {
        h.bbmin[d] = c->bbmin[d];
        h.bbmax[d] = c->bbmax[d];
    }
    h.envW = c->hasEnv ? c->envW : 0;  // 0 x 0: no environment map
    h.envH = c->hasEnv ? c->envH : 0;
    std::memcpy(h.poissonRng, c->poissonRng, 16);
    h.numStreams = (int32_t)rs.streams.size();
    h.classic = classic ? 1 : 0;
    h.learned = g.enabled ? 1 : 0;
    h.learnedTrained = g.trained ? 1 : 0;
    h.learnedCur = g.cur;
    h.learnedImpValid = g.impValid ? 1 : 0;
    h.learnedAdamStep = g.adamStep;
    h.learnedRecords = nrec;
    if (classic) {
        const ClassicState& s = rs.classic;
        for (int d = 0; d < 3; d++) h.classicBbmin[d] = s.bbmin[d];
        h.classicScale = s.scale;
        h.classicIrad = s.irad;
    }
    Writer w{out, cap};
    w.host(&h, sizeof(h));
    w.device(rs.accum.p, (size_t)pixels * 12);
    for (const XorShift& x : rs.streams) w.host(x.s, 16);
    if (classic) {
        const ClassicState& s = rs.classic;
        w.device(s.pos.p, (size_t)pixels * 24);
        w.device(s.nrm.p, (size_t)pixels * 12);
        w.device(s.flux.p, (size_t)pixels * 24);
        w.device(s.weight.p, (size_t)pixels * 24);
        w.device(s.emission.p, (size_t)pixels * 24);
        w.device(s.r2.p, (size_t)pixels * 8);
        w.device(s.n.p, (size_t)pixels * 4);
        w.device(s.coeff.p, (size_t)pixels * 4);
    }
    if (g.enabled) {
        const size_t grid = (size_t)g.G * g.G * g.G * 4;
        w.device(g.params.p, (size_t)kMlpParams * 4);
        w.device(g.adamM.p, (size_t)kMlpParams * 4);
        w.device(g.adamV.p, (size_t)kMlpParams * 4);
        w.device(g.imp[0].p, grid);
        w.device(g.imp[1].p, grid);
        w.device(g.rec.p, (size_t)nrec * sizeof(MlpRecord));
    }
    *size = w.pos;
    if (w.err != cudaSuccess) return fail(c, PPPM_E_CUDA, std::string("render_save: ") + cudaGetErrorString(w.err));
    if (out && !w.ok) return fail(c, PPPM_E_CAPACITY, "render_save: the buffer is smaller than the checkpoint");
    return PPPM_OK;
}

int pppm_render_load(pppm_ctx* c, const uint8_t* in, int64_t size) {
    if (!c || !in || size < (int64_t)sizeof(CkHeader)) return fail(c, PPPM_E_ARG, "render_load: bad arguments");
    CkHeader h;
    std::memcpy(&h, in, sizeof(h));
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != 1 || h.headerBytes != sizeof(CkHeader))
        return fail(c, PPPM_E_ARG, "render_load: not a checkpoint of this library version");
    bool same = c->hasScene && h.ntri == c->ntri && h.envW == (c->hasEnv ? c->envW : 0) &&
                h.envH == (c->hasEnv ? c->envH : 0);
    for (int d = 0; d < 3 && same; d++) same = h.bbmin[d] == c->bbmin[d] && h.bbmax[d] == c->bbmax[d];
    if (!same) return fail(c, PPPM_E_STATE, "render_load: the context holds another scene or environment map");
    int r = pppm_render_begin(c, &h.cam, &h.par);
    if (r) return r;
    RenderState& rs = c->rs;
    const int64_t pixels = (int64_t)rs.cam.width * rs.cam.height;
    if ((int32_t)rs.streams.size() != h.numStreams || (h.classic != 0) != (rs.par.mode == PPPM_MODE_CLASSIC) ||
        (h.learned != 0) != rs.guide.enabled)
        return fail(c, PPPM_E_ARG, "render_load: inconsistent checkpoint");
    cudaSetDevice(c->device);
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    Reader rd{in, size};
    rd.take(sizeof(CkHeader));
    rd.device(rs.accum.p, (size_t)pixels * 12);
    for (XorShift& x : rs.streams) {
        const uint8_t* p = rd.take(16);
        if (p) std::memcpy(x.s, p, 16);
    }
    if (h.classic) {
        ClassicState& s = rs.classic;
        rd.device(s.pos.p, (size_t)pixels * 24);
        rd.device(s.nrm.p, (size_t)pixels * 12);
        rd.device(s.flux.p, (size_t)pixels * 24);
        rd.device(s.weight.p, (size_t)pixels * 24);
        rd.device(s.emission.p, (size_t)pixels * 24);
        rd.device(s.r2.p, (size_t)pixels * 8);
        rd.device(s.n.p, (size_t)pixels * 4);
        rd.device(s.coeff.p, (size_t)pixels * 4);
        for (int d = 0; d < 3; d++) s.bbmin[d] = h.classicBbmin[d];
        s.scale = h.classicScale;
        s.irad = h.classicIrad;
    }
    if (h.learned) {
        GuideState& g = rs.guide;
        const size_t grid = (size_t)g.G * g.G * g.G * 4;
        if (h.learnedRecords > g.recCap) return fail(c, PPPM_E_ARG, "render_load: inconsistent checkpoint");
        rd.device(g.params.p, (size_t)kMlpParams * 4);
        rd.device(g.adamM.p, (size_t)kMlpParams * 4);
        rd.device(g.adamV.p, (size_t)kMlpParams * 4);
        rd.device(g.imp[0].p, grid);
        rd.device(g.imp[1].p, grid);
        rd.device(g.rec.p, (size_t)h.learnedRecords * sizeof(MlpRecord));
        const unsigned long long n = (unsigned long long)h.learnedRecords;
        PPPM_CUDA(c, cudaMemcpy(g.counters.p, &n, 8, cudaMemcpyHostToDevice));
        PPPM_CUDA(c, launchMlpPack(g.params.as<float>(), g.blob.as<uint8_t>(), c->stream));
        g.trained = h.learnedTrained != 0;
        g.cur = h.learnedCur;
        g.impValid = h.learnedImpValid != 0;
        g.adamStep = h.learnedAdamStep;
    }
    if (!rd.ok || rd.pos != size) {
        rs.active = false;
        return fail(c, PPPM_E_ARG, "render_load: truncated or oversized checkpoint");
    }
    if (rd.err != cudaSuccess) {
        rs.active = false;
        return fail(c, PPPM_E_CUDA, std::string("render_load: ") + cudaGetErrorString(rd.err));
    }
    rs.passesDone = h.passesDone;
    rs.radius = h.radius;
    rs.storedLast = h.storedLast;
    rs.storedMax = h.storedMax;
    if (h.depositCap > rs.depositCap) {
        rs.depositCap = h.depositCap;
        PPPM_CUDA(c, rs.photons.ensure((size_t)rs.depositCap * 32));
    }
    rs.bouncePerSm = h.bouncePerSm;
    rs.eyePerSm = h.eyePerSm;
    rs.par.cell_factor = h.cellFactor;
    std::memcpy(c->poissonRng, h.poissonRng, 16);
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

}  // extern "C"
