// Wavefront photon tracing, eye paths and RNG tapes.
#pragma once

#include "dipole.cuh"
#include "kernels.h"
#include "mlp_dev.cuh"

// blocks per SM promised to ptxas for the traversal kernels
#ifndef PPPM_TRACE_MINBLOCKS
#define PPPM_TRACE_MINBLOCKS 7
#endif
// blocks per SM the eye kernel's registers are sized for (it runs beside
// the photon kernel in short blocks of one pixel tile)
#ifndef PPPM_EYE_MINBLOCKS
#define PPPM_EYE_MINBLOCKS PPPM_TRACE_MINBLOCKS
#endif

namespace pppm {

// One photon path in the wavefront queue (80 bytes).
struct __align__(16) PathState {
    double ox, oy, oz;  // origin in double, as the reference keeps hit points
    float dx, dy, dz;   // unit direction
    float fx, fy, fz;   // flux
    uint32_t rng[4];    // XorShift state positioned at the next draw
    int id;             // path id (stream = id / taskPerThread in compat mode)
    int bounce;
    int pad[2];
};
static_assert(sizeof(PathState) == 80, "PathState layout");

// Device counters of one pass.
struct PassCounters {
    unsigned long long queue[3];      // rotating queue lengths (see launchPhotonBounce)
    unsigned long long deposits;      // photon records written (may exceed capacity)
    unsigned long long queries;       // gather queries written
    unsigned long long photonRays;    // photon traversals
    unsigned long long eyeRays;       // eye traversals
    unsigned long long undefinedEmit; // CDF inversion past the last entry (reference reads out of bounds)
    unsigned long long nodeVisits[2]; // [photon, eye] BVH nodes visited (counting flag)
    unsigned long long triTests[2];   // [photon, eye] triangles tested (counting flag)
    unsigned long long undefinedEye;  // eye paths past their 200-number tape (compat) or the segment cap
    unsigned long long sssQueries;    // subsurface radiance queries queued by the eye pass
    unsigned long long sssVisits;     // octree nodes visited by them (counting flag)
    unsigned long long fetched;       // paths taken from the emitted queue by the persistent photon kernel
};

struct CameraDev {
    double ex, ey, ez;
    float dx, dy, dz;
    float ux, uy, uz;
    float vx, vy, vz;
    float halfTan, aspect;
    int w, h;
};

// Learned proposal inside the photon pass (canonical mode): training
// records and the importance grid that weights them.
struct GuideView {
    MlpRecord* rec;                // record pool
    unsigned long long* recCount;  // records written (may exceed recCap)
    int64_t recCap;
    uint32_t recEvery;             // one record per recEvery guided decisions
    const float* imp;              // importance grid (G^3, previous pass) or nullptr
    int G;
    float ox, oy, oz, inv;         // grid origin and 1 / voxel edge
    float maxLogKappa;             // clamp of the lobes' log concentration
    int guideBounces;              // 1: Lambertian bounces are guided too
    // emission: the network's direction mixture at one fixed input (emission
    // position epx..epz, zero normal) proposes the environment direction
    const float* emitRaw;          // its 40 outputs, or nullptr before the first training
    float emitFloor;               // MIS probability of the reference's environment sampling
    float emitK;                   // area / numPhotons of Envmap::samplePhoton (flux = L emitK / p_cell)
    float epx, epy, epz;
};

__device__ __forceinline__ int impVoxel(const GuideView& g, float x, float y, float z) {
    const int ix = (int)floorf((x - g.ox) * g.inv), iy = (int)floorf((y - g.oy) * g.inv),
              iz = (int)floorf((z - g.oz) * g.inv);
    if (ix < 0 || iy < 0 || iz < 0 || ix >= g.G || iy >= g.G || iz >= g.G) return -1;
    return (iz * g.G + iy) * g.G + ix;
}

constexpr int kPathNeedsDir = 1;  // PathState.pad[1]: direction still to be drawn (normal in d)
// PathState.pad[1] >> kPathEmitRecShift: 1 + index of the path's emission
// record (0: none); its weight collects the path's importance-weighted deposits
constexpr int kPathEmitRecShift = 8;

// Compaction: each taking lane gets a slot; one atomic per warp.
__device__ __forceinline__ unsigned long long warpAppend(bool take, unsigned long long* counter) {
    const unsigned mask = __ballot_sync(0xffffffffu, take);
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (mask) {
        const int leader = __ffs(mask) - 1;
        if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return base + (unsigned long long)__popc(mask & ((1u << lane) - 1u));
}

struct TraceParams {
    int mode;
    int numStreams;
    int64_t taskPerThread;  // ceil(P / N)
    int64_t numPaths;       // N * taskPerThread (compat) or P (canonical)
    double numPhotons;      // flux divisor (RenderParameters::photons)
    int maxBouncePhoton;
    int maxBounceEye;
    uint32_t seed;
    int pass;
    int countTraversal;
    int sssPass;  // 1: the subsurface photon pass (buildPhotonMap semantics)
    int hasSss;   // 1: the scene has BSSRDF materials
    int bouncePerSm = 16;  // photon bounce kernel: blocks per SM (tunable)
    int eyePerSm = 16;     // eye kernel: blocks per SM (tunable)
    int refill = kRefill;  // persistent photon kernel: lanes done before a warp shades (tunable)
    int exactBatch = kExactBatch;  // lanes waiting before a warp runs the double tests (tunable)
    int guided;   // 1: learned proposal (emission direction; Lambertian bounces through kGuideResolve)
    GuideView guide;
    // compat mode with the reference's RANDOM_SAMPLER_QUASI_MONTE_CARLO
    // sampler: each stream s is Halton(200, true, s); per pass it serves its
    // taskPerThread photons, then the pixels of its rows y = s, s + N, ...
    int qmc = 0;
    HaltonDev halton = {};
    int width = 0, height = 0;  // image size (sample indices of the QMC streams)
};

// Halton sample index of pass tp.pass for stream s: the samples of earlier
// passes (taskPerThread photons + the pixels of the stream's rows each),
// then `offset` (photon round i, or taskPerThread + row k * width + x).
__host__ __device__ inline unsigned long long qmcIndex(const TraceParams& tp, int s, int64_t offset) {
    const int64_t rows = s < tp.height ? (tp.height - 1 - s) / tp.numStreams + 1 : 0;
    return (unsigned long long)(tp.pass - 1) * (unsigned long long)(tp.taskPerThread + rows * tp.width) +
           (unsigned long long)offset;
}

// The tape of a photon path between bounces, held in PathState.rng:
// XorShift, the four state words; Halton, the sample index (two words), the
// next dimension and the stream.
__device__ __forceinline__ void loadTape(const TraceParams& tp, const PathState& p, Tape& t) {
    t.pos = 0;
    t.scramble = tp.mode == PPPM_MODE_CANONICAL;
    t.x.s[0] = p.rng[0]; t.x.s[1] = p.rng[1]; t.x.s[2] = p.rng[2]; t.x.s[3] = p.rng[3];
}
__device__ __forceinline__ void loadTape(const TraceParams& tp, const PathState& p, HaltonTape& t) {
    t.h = &tp.halton;
    t.stream = (int)p.rng[3];
    t.index = (unsigned long long)p.rng[0] | ((unsigned long long)p.rng[1] << 32);
    t.dim = (int)p.rng[2];
    t.over = false;
}
__device__ __forceinline__ void storeTape(const Tape& t, PathState& p) {
    p.rng[0] = t.x.s[0]; p.rng[1] = t.x.s[1]; p.rng[2] = t.x.s[2]; p.rng[3] = t.x.s[3];
}
__device__ __forceinline__ void storeTape(const HaltonTape& t, PathState& p) {
    p.rng[0] = (uint32_t)t.index;
    p.rng[1] = (uint32_t)(t.index >> 32);
    p.rng[2] = (uint32_t)t.dim;
    p.rng[3] = (uint32_t)t.stream;
}

// PerspectiveCamera::getRay (perspective_camera.cc:42-46) in FP32.
__device__ __forceinline__ void cameraRay(const CameraDev& c, float px, float py, f3* d) {
    const float a = c.halfTan * c.aspect * (2.0f * px / (float)c.w - 1.0f);
    const float b = c.halfTan * (2.0f * py / (float)c.h - 1.0f);
    const f3 dir = {c.dx + a * c.ux + b * c.vx, c.dy + a * c.uy + b * c.vy, c.dz + a * c.uz + b * c.vz};
    *d = normalized(dir);
}

// Jump-ahead matrices: J[k] advances a XorShift state by stride * 2^k draws
// (stride 200: one tape per photon or pixel). Column j of a matrix is the
// image of state bit j; 128 columns of 4 words each.
constexpr int kJumpLevels = 40;
void xorshiftJumpTables(std::vector<uint32_t>* tables, uint32_t stride = 200);
void xorshiftJumpHost(const std::vector<uint32_t>& tables, uint64_t tapes, XorShift* st);

cudaError_t launchTapeStates(const TraceParams& tp, const uint32_t* streamStates, const uint32_t* jump, int width,
                             int height, uint32_t* photonStates, uint32_t* pixelStates, cudaStream_t st);
// Coherent trace order of the emitted photon paths: a 16-bit key per path
// (the octahedral cell of its first direction, 2^kSortDirBits per side in
// Morton order, then the 2^kSortEnvBits-per-side cell of its emission
// direction) counted while emitting, then a counting sort of the path
// indices. Neighbouring lanes of the persistent
// kernel then start from nearby origins in nearby directions. The order in
// which paths are traced changes no path.
#ifndef PPPM_PHOTON_SORT
#define PPPM_PHOTON_SORT 1
#endif
#ifndef PPPM_SORT_DIR_BITS
#define PPPM_SORT_DIR_BITS 7
#endif
#ifndef PPPM_SORT_ENV_BITS
#define PPPM_SORT_ENV_BITS 1
#endif
#ifndef PPPM_SORT_ENV_HIGH
#define PPPM_SORT_ENV_HIGH 0
#endif
constexpr bool kPhotonSort = PPPM_PHOTON_SORT != 0;
constexpr int kSortDirBits = PPPM_SORT_DIR_BITS;  // per octahedral axis
constexpr int kSortEnvBits = PPPM_SORT_ENV_BITS;
constexpr int kPhotonSortBins = 1 << (2 * (kSortDirBits + kSortEnvBits));
struct PhotonSort {
    uint32_t* keys;    // one per path
    uint32_t* hist;    // kPhotonSortBins + 1 counts, zero before emission
    uint32_t* cursor;  // kPhotonSortBins + 1
    uint32_t* tmp;     // scanTmpWords(kPhotonSortBins)
    uint32_t* perm;    // one per path: trace position -> path index
};
cudaError_t launchPhotonEmit(const TraceParams& tp, const EnvDev& env, const uint32_t* photonStates, PathState* queue,
                             PassCounters* ctr, cudaStream_t st, const PhotonSort* sort = nullptr);
// Scan of the key counts and the scatter of path indices into sort.perm,
// or (moveTo != nullptr) of the path records themselves into moveTo.
cudaError_t photonSortPaths(const PhotonSort& sort, int64_t paths, cudaStream_t st, const PathState* from = nullptr,
                            PathState* moveTo = nullptr);
#ifndef PPPM_SORT_MOVE
#define PPPM_SORT_MOVE 0
#endif
constexpr bool kSortMove = PPPM_SORT_MOVE != 0;
cudaError_t launchPhotonBounce(const TraceParams& tp, const SceneView& sc, int bounce, const PathState* in,
                               PathState* out, int64_t maxPaths, float4* deposits, int64_t depositCap,
                               PassCounters* ctr, cudaStream_t st);
// Every bounce of the emitted queue (ctr->queue[0] paths in `in`) in one
// persistent launch with dynamic ray fetching (kPhotonPersistent).
// perm (optional): the order in which the paths of `in` are taken.
cudaError_t launchPhotonPersistent(const TraceParams& tp, const SceneView& sc, const PathState* in, int64_t maxPaths,
                                   float4* deposits, int64_t depositCap, PassCounters* ctr, cudaStream_t st,
                                   const uint32_t* perm = nullptr);
// The bounces from `bounce` on of the queue left after the wavefront
// launches, in one launch (kPhotonBounce<.., true>).
cudaError_t launchPhotonTail(const TraceParams& tp, const SceneView& sc, int bounce, const PathState* in,
                             int64_t maxPaths, float4* deposits, int64_t depositCap, PassCounters* ctr,
                             cudaStream_t st);
// Photon passes without guided bounces run in the persistent kernel (1) or
// as wavefront launches plus the tail kernel (0).
#ifndef PPPM_PERSISTENT
#define PPPM_PERSISTENT 1
#endif
constexpr bool kPersistentPhotons = PPPM_PERSISTENT != 0;
// Bounces traced as one launch each before the tail kernel takes the rest.
#ifndef PPPM_WAVE_BOUNCES
#define PPPM_WAVE_BOUNCES 2
#endif
constexpr int kWaveBounces = PPPM_WAVE_BOUNCES;

cudaError_t launchEyeTrace(const TraceParams& tp, const SceneView& sc, const EnvDev& env, const CameraDev& cam,
                           const OctView& oct, const uint32_t* pixelStates, float* accum, float4* queries,
                           float4* sssQ, int64_t sssCap, PassCounters* ctr, cudaStream_t st,
                           bool pathTrace = false);
cudaError_t launchSubsurfaceGather(const OctView& oct, const DevMaterial* mats, const float4* q,
                                   const unsigned long long* count, int64_t cap, float* accum,
                                   unsigned long long* visits, cudaStream_t st);
// GPU Poisson-disc sampling (k_poisson.cu). popOrder: RandomQueue(-1) pop
// positions of n pushes (false where the reference's nextInt is undefined).
bool popOrder(int64_t n, std::vector<int>* rank);
int poissonBegin(pppm_ctx* c, PoissonGpu& g, const float* tri9, int64_t ntri, double minDist);
int poissonRun(pppm_ctx* c, PoissonGpu& g, uint32_t rng[4], float4* queries, float* pts, float* nrm, int64_t cap,
               int64_t* count);

// Subsurface stage of a render (sss.cu): per-render setup, the per-pass
// photon map + points + irradiance (enqueued), and the octree build.
int sssBegin(pppm_ctx* c);
int sssPrepare(pppm_ctx* c, int t, const TraceParams& base, const SceneView& sv, const EnvDev& ev, int64_t* launches);
int sssFinish(pppm_ctx* c, int64_t* launches);
OctView sssView(const pppm_ctx* c);

// Learned proposal (k_guide.cu): MLP inputs of the queue's pending paths,
// direction draw from the BSDF / vMF mixture, importance grid, record sums.
cudaError_t launchGuidePack(const PathState* q, const unsigned long long* count, int64_t cap, float* pos, float* nrm,
                            cudaStream_t st);
cudaError_t launchGuideResolve(const TraceParams& tp, PathState* q, const unsigned long long* count, int64_t cap,
                               const float* raw, float floorBsdf, int bounce, cudaStream_t st);
cudaError_t launchImportanceSplat(const GuideView& g, const float4* queries, const unsigned long long* count,
                                  int64_t cap, const float* accum, float invPasses, float floorLum, float* grid,
                                  cudaStream_t st);
cudaError_t launchRecordInvSum(const MlpRecord* rec, int64_t n, float* sum, cudaStream_t st);

// Learned proposal in a canonical render (guide.cu).
// Kernel parameters and camera of pass t of the current render (render.cu).
void passSetup(pppm_ctx* c, int t, int64_t paths, TraceParams* tp, CameraDev* cd);
// Emission of the pass's photon paths into rs.pathA; with `sorted`, also the
// coherent trace order (memset, emission with keys, scan, scatter): either
// the records moved in that order into rs.pathB (*paths points there) or a
// permutation in *perm. Otherwise *paths = rs.pathA and *perm = nullptr.
// Adds its launches.
int emitPhotonPaths(pppm_ctx* c, const TraceParams& tp, const EnvDev& ev, const uint32_t* photonStates,
                    PassCounters* ctr, bool sorted, const PathState** paths, const uint32_t** perm,
                    int64_t* launches);

int guideBegin(pppm_ctx* c, int64_t maxPaths);
GuideView guideView(pppm_ctx* c, int64_t decisionsPerPass);
int guideStep(pppm_ctx* c, const TraceParams& tp, PathState* q, const unsigned long long* count, int64_t cap,
              int bounce);
int guideImportance(pppm_ctx* c, const float4* queries, const unsigned long long* count, int64_t cap, int t);
int guideEmission(pppm_ctx* c);
int guideEndPass(pppm_ctx* c, int t);

// Classic PPM (k_classic.cu).
int classicBegin(pppm_ctx* c, int64_t pixels);
// Halton(200, true, s) tables of samplers s < streams (permutations, primes,
// offsets) on the device, and their view (k_classic.cu).
int haltonBegin(pppm_ctx* c, int streams);
HaltonDev haltonDev(pppm_ctx* c);
int classicPass(pppm_ctx* c, int t, const TraceParams& tp, const SceneView& sv, const EnvDev& ev, const CameraDev& cd,
                pppm_pass_stats* stats);
int classicRead(pppm_ctx* c, float* out);

cudaError_t launchStreamCounts(const float4* deposits, const unsigned long long* count, int64_t cap, int64_t tpt,
                               int numStreams, unsigned long long* perStream, cudaStream_t st);

}  // namespace pppm
