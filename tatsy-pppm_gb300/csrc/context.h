// The C-ABI context: device memory owned per context, staging of host
// arguments, and the render state carried between passes.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pppm_c.h"
#include "pppm_device.cuh"

namespace pppm {

// Growable device allocation owned by the context.
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    ~DBuf() { release(); }
};

struct GridBufs {
    DBuf counts;   // uint32 per bucket (+1), becomes start offsets
    DBuf cursor;   // uint32 per bucket
    DBuf sorted;   // float4 x 2 per photon, bucket order
    DBuf keys;     // uint32 bucket per photon
    DBuf scanTmp;  // scan partials
    DBuf owner;    // uint64 per bucket: the cell of its photons (GridDev::owner)
    bool hasOwner = false;  // the last build recorded owner
    uint32_t size = 0;   // buckets (power of two)
    float cell = 0.0f;   // cell edge
    float invCell = 0.0f;
    float origin[3] = {0, 0, 0};
    int64_t count = 0;   // photons in the grid
};

// Counting sort of gather queries by grid cell (tiled gather).
// Canonical gather shape (tunable per render; neither changes a result):
// photons per warp tile (a multiple of 32, 32..256) and sub-cells per axis
// of the query sort key (2^bits, bits 0..3). querySortLayout sets the bits
// to the most, up to PPPM_GATHER_SUBBITS, that leave the sort at least 4096
// cell buckets (3 at 1080p; 1 for images of up to ~64k pixels).
#ifndef PPPM_GATHER_WSTAGE
#define PPPM_GATHER_WSTAGE 128
#endif
#ifndef PPPM_GATHER_SUBBITS
#define PPPM_GATHER_SUBBITS 3
#endif
constexpr int kGatherStageMax = 256;

struct QuerySortBufs {
    DBuf hist, cursor, tmp, keys, sorted;
    uint32_t size = 0;
    int stage = PPPM_GATHER_WSTAGE;
    int subBits = PPPM_GATHER_SUBBITS;
};

// Pinned host buffer (grown on demand).
struct HostPinned {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    ~HostPinned() {
        if (p) cudaFreeHost(p);
    }
};

// GPU Poisson-disc sampler of the BSSRDF triangles (k_poisson.cu): per-render
// triangle tables and the candidate pop order, per-pass candidate buffers.
struct PoissonGpu {
    bool ready = false;
    int64_t ntri = 0;
    int64_t n = 0;       // candidates per pass
    int64_t rounds = 0;  // decision rounds of the last run
    double minDist = 0.0;
    std::vector<uint32_t> jumpHost;  // XorShift jump matrices for 2^k draws
    DBuf jump, tri, offs, triNrm, scanCursor, scanTmp, rank, pos, rec, triOf, own, box, state, conf, list, byPop,
        flag, cursor, tmp, bbox, misc;
    GridBufs grid;
};

// Subsurface stage of a render (SubsurfaceIntegrator, rebuilt every pass).
// Scratch and output of the GPU octree build (k_octree.cu).
struct OctreeBufs {
    DBuf idx, active, big, chunks, chunkCnt, box, nodes, acc, ctr;
    DBuf out;  // OctNodeDev per node, preorder
    HostPinned hostCtr;
    int64_t nodeCap = 0;
};

// Irradiance points of an octree build (device): position and irradiance
// (3 floats each, `stride` floats apart) and area (per point or constant).
struct OctreePoints {
    const float* pos;
    int posStride;
    const float* irad;
    int iradStride;
    const float* area;  // null: areaConst for every point
    int areaStride;
    double areaConst;
};

struct SssState {
    bool enabled = false;
    double areaRadius = 0.0;  // sqrt(BSSRDF area / all triangles) (ppm_probabilistic.cc:35-46)
    double dA = 0.0;          // irradiance point area (subsurface_integrator.cc:202)
    int k = 0;                // (int)gatherRadius: kNN count of irradianceWithPM
    DBuf photons;             // 2 x float4 per stored subsurface photon
    int64_t cap = 0;
    GridBufs grid;
    PoissonGpu poisson;
    DBuf points;              // 3 x float4 per irradiance point (gather query layout)
    DBuf ptsD, nrmD;          // float3 per point
    DBuf irad;                // float3 per point
    OctreeBufs oct;           // octree of the points (GPU build)
    int octNodes = 0;
    DBuf queue;               // eye-pass subsurface queries: 2 float4 each
    int64_t queueCap = 0;
    int64_t numPoints = 0;
    int64_t stored = 0;
    double msHost = 0.0;      // host time of the octree build loop
    cudaEvent_t done = nullptr;     // irradiance of the points computed
    cudaEvent_t octDone = nullptr;  // octree written
};

// Learned photon proposal of a canonical render (PPPM_FLAG_LEARNED).
struct GuideState {
    bool enabled = false;
    bool trained = false;
    int retrainEvery = 2;       // passes between trainings
    int stepsPerTrain = 2;      // Adam steps per training
    int64_t batch = 65536;      // records per step
    float lr = 4e-3f;
    float floorBsdf = 0.3f;     // one-sample MIS: probability of the reference's sampling
    float maxLogKappa = 7.0f;   // clamp of the lobes' log concentration
    int guideBounces = 0;       // guide Lambertian bounces too (1) or the emission direction only (0)
    float floorLum = 0.01f;     // luminance floor of the relative-error importance
    int adamStep = 0;
    DBuf params, adamM, adamV, grad, blob, misc;  // misc: loss, error flag, 1 / sum w
    DBuf raw;                   // network outputs per queue slot (40 floats)
    DBuf inPos, inNrm;          // network inputs per queue slot
    DBuf emitIn, emitRaw;       // the emission input row (position, zero normal) and its 40 outputs
    DBuf rec;                   // training records
    int64_t recCap = 0;
    DBuf counters;              // record count
    DBuf imp[2];                // importance grids (this pass, previous pass)
    int cur = 0;
    bool impValid = false;
    int G = 64;
    float gox = 0, goy = 0, goz = 0, ginv = 1;
    double box[6] = {0, 0, 0, 1, 1, 1};  // network input box
    double msTrain = 0.0;
    float lastLoss = 0.0f;
    int64_t lastRecords = 0;
};

// Classic PPM (ProgressivePhotonMapping): render points, Halton tables,
// render-point hash grid and photon-update events.
// Scratch of pppm_hashgrid_build (k_hashgrid.cu).
struct HashGridBufs {
    DBuf offs, offsCursor, offsTmp;  // per item: first insertion index (scanned cell counts)
    DBuf hist, cursor, tmp;          // per bucket: start offsets
    DBuf order, flag;                // entries' insertion indices by bucket; oversize flag
};

struct ClassicState {
    DBuf pos, nrm, flux, weight, emission, r2, n, coeff;  // per render point (pixel), SoA, double where the reference is
    DBuf haltonPerm, haltonPrime, haltonOffset;          // permutation tables per stream, first 200 primes
    int haltonSum = 0;                                   // sum of the first 200 primes
    DBuf gridCount, gridCursor, gridTmp, gridEntries;     // bucket -> render points
    int64_t gridEntriesCap = 0;
    DBuf ev, evCount, evSorted, evCursor, evTmp, evRp;   // photon-update events
    int64_t evCap = 0;
    DBuf bbox, misc;
    double bbmin[3] = {0, 0, 0}, scale = 1.0, irad = 0.0;
};

struct RenderState {
    bool active = false;
    pppm_camera cam{};
    pppm_params par{};
    double radius = 0.0;
    double bboxDiag = 0.0;
    int64_t taskPerThread = 0;  // ceil(P / N)
    int passesDone = 0;
    // per-stream XorShift state at the start of the next pass (compat)
    std::vector<XorShift> streams;
    DBuf accum;       // float3 per pixel (W*H*3 floats)
    DBuf photons;     // 2 x float4 per stored photon (pos|normal, flux|stream)
    DBuf photonCount; // counters (see render.cu)
    DBuf pathA, pathB;  // wavefront path state
    DBuf sortKeys, sortHist, sortCursor, sortTmp, sortPerm;  // trace order of the emitted photon paths
    DBuf queries;     // gather queries
    DBuf tapeStates;  // uint4 start state per photon / pixel (compat)
    DBuf jumpMats;    // jump-ahead matrices
    DBuf streamStatesD;  // N x uint4 per-stream state at the start of the pass
    GridBufs grid;
    QuerySortBufs qsort;
    DBuf gatherWork;  // 2 counters: photon pairs tested, pairs within the radius
    int64_t depositCap = 0;
    int64_t storedLast = 0;
    int64_t queriesLast = 0;  // gather queries written by the last pass
    int64_t storedMax = 0;     // most photons stored by one pass of this render
    HostPinned graphSlots;      // counters of captured passes (graph.cu)
    std::vector<double> graphRadius;  // radius of each captured pass
    bool graphSideEye = false;        // the captured passes traced eye paths on the side stream
    int64_t phantomsLast = 0;
    SssState sss;
    GuideState guide;
    ClassicState classic;
    // launch shapes the autotuner may change between passes (with
    // qsort.stage and qsort.subBits)
    int bouncePerSm = 16;
    int eyePerSm = 16;
    int refill = kRefill;
    int exactBatch = kExactBatch;
};

}  // namespace pppm

struct pppm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // scene
    bool hasScene = false;
    int64_t ntri = 0;
    int rootCode = 0;
    int bvhDepth = 0;
    int numNodes = 0;
    double bbmin[3] = {0, 0, 0}, bbmax[3] = {0, 0, 0};
    std::vector<pppm_material> mats;
    bool anyBssrdf = false;
    pppm::DBuf nodes, tris, matId, devMats, triE;
    double lambertArea = 0.0;  // summed area of Lambertian triangles
    std::vector<float> hostTri;        // triangle soup (9 floats each), for the Poisson sampler
    std::vector<int32_t> hostMatId;    // material of each triangle
    // emissive materials (pppm_material_emission) and their triangles
    std::vector<float> matEmit;        // 3 per material
    pppm::DBuf lightTri, lightCdf, lightUcdf, lightLe;
    int numLights = 0;
    double lightArea = 0.0;            // summed area of the emitters
    float lightFluxScale = 0.0f;       // pi * lightArea / photons of the active render
    std::vector<int64_t> bssrdfTris;   // triangles with a BSSRDF, in scene order
    double bssrdfArea = 0.0;           // their summed Triangle::area, in scene order
    // sampler.cc's static Random (seeded 0) of the Poisson-disc sampler; it
    // lives as long as the process there and as long as the context here
    uint32_t poissonRng[4] = {0, 0, 0, 0};
    cudaStream_t aux = nullptr;        // readbacks that overlap the main stream
    cudaStream_t side = nullptr;       // eye paths traced beside the photon pass
    // env
    bool hasEnv = false;
    int envW = 0, envH = 0;
    std::vector<double> envPdf, envCdf;
    pppm::DBuf envRgb, envPdfD, envCdfD, envUcdfD, envScaleD;
    double envScaleFor = -1.0;  // numPhotons the flux-scale table was built for
    double envExponent = 2.0;   // cell weight = luminance^envExponent (2: the reference)
    // staging for host arguments
    pppm::DBuf stage[8];
    std::vector<void*> pinned;
    pppm::RenderState rs;
    pppm::HashGridBufs hashGrid;  // pppm_hashgrid_build
    std::vector<uint32_t> jumpTables;  // XorShift jump-ahead matrices (host copy)
    // scratch of the kNN / gather stage entry points
    pppm::DBuf stageRec, stageQ, stageCount;
    pppm::GridBufs stageGrid;
    pppm::QuerySortBufs stageQsort;
    pppm::PoissonGpu stagePoisson;
    pppm::OctreeBufs stageOct;
    // stage timing: 0-7 main stream; 8 fork of the side stream, 9-10 its
    // eye trace
    cudaEvent_t ev[12] = {};
    std::vector<cudaEvent_t> graphEvents;  // stage timing of captured passes
};

namespace pppm {

inline int fail(pppm_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

// Octree of n irradiance points on stream st (k_octree.cu): the tree of the
// reference's Octree::construct in preorder, in b.out; *numNodes its size.
// Synchronises st a few times (level counts).
int octreeBuild(pppm_ctx* c, OctreeBufs& b, const OctreePoints& pts, int64_t n, cudaStream_t st, int* numNodes,
                int64_t* launches);

// Captured canonical passes (graph.cu). graphEligible: canonical, no
// subsurface stage, no learned proposal, no traversal counting.
// graphPrepare fixes the capacities of `count` passes; graphEnqueuePass
// records pass t (counter slot `slot`) into the context stream under capture
// (sideEye: eye paths on the side stream beside the photon pass); graphFinishPass reads a slot after the graph ran (msPass: the
// pass's device time); graphAbort ends a failed capture; graphRun
// instantiates, launches and waits.
bool graphEligible(const pppm_ctx* c);
int graphPrepare(pppm_ctx* c, int count);
int graphEnqueuePass(pppm_ctx* c, int t, int slot, bool sideEye);
int graphFinishPass(pppm_ctx* c, int slot, pppm_pass_stats* st, double* msPass);
void graphAbort(cudaStream_t st);
int graphRun(pppm_ctx* c, cudaGraph_t g, cudaStream_t st, double* instantiateMs = nullptr);

inline int cudaFail(pppm_ctx* c, cudaError_t e, const char* where) {
    return fail(c, PPPM_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define PPPM_CUDA(ctx, call)                                   \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return ::pppm::cudaFail((ctx), e_, #call); \
    } while (0)

bool isDevicePtr(const void* p);

// Dipole constants of a material (capi.cu).
DipoleDev dipoleFrom(const pppm_material& mat);

// Returns a device pointer holding `bytes` of `src`: src itself when it is
// device memory, else a staging copy (slot chooses the staging buffer).
int stageIn(pppm_ctx* c, const void* src, size_t bytes, int slot, const void** out);
// Returns where a kernel should write `bytes` destined for `dst`.
int stageOut(pppm_ctx* c, void* dst, size_t bytes, int slot, void** out);
// Copies staged output back to a host `dst` (no-op for device dst).
int finishOut(pppm_ctx* c, void* dst, const void* staged, size_t bytes);

// Uploads the scene device view used by kernels.
struct SceneView {
    const QNode* nodes;
    const float4* tris;
    const int* matId;
    const DevMaterial* mats;
    int rootCode;
    int numNodes;
    const double* triE;  // per slot: double p0, e1 = b - a, e2 = c - a (10 doubles), or nullptr
};
inline SceneView sceneView(const pppm_ctx* c) {
    return {c->nodes.as<QNode>(), c->tris.as<float4>(), c->matId.as<int>(), c->devMats.as<DevMaterial>(), c->rootCode,
            c->numNodes, kTriEdges ? c->triE.as<double>() : nullptr};
}
inline EnvDev envView(const pppm_ctx* c) {
    EnvDev e;
    e.rgb = c->envRgb.as<float>();
    e.cdf = c->envCdfD.as<double>();
    e.pdf = c->envPdfD.as<double>();
    e.ucdf = c->envUcdfD.as<unsigned long long>();
    e.fluxScale = c->envScaleD.as<float>();
    e.w = c->hasEnv ? c->envW : 0;
    e.h = c->hasEnv ? c->envH : 0;
    e.lightTri = c->lightTri.as<float4>();
    e.lightCdf = c->lightCdf.as<double>();
    e.lightUcdf = c->lightUcdf.as<unsigned long long>();
    e.lightLe = c->lightLe.as<float>();
    e.numLights = c->numLights;
    e.lightFluxScale = c->lightFluxScale;
    return e;
}
// Fills the per-CDF-cell photon flux scale for numPhotons.
int envFluxScale(pppm_ctx* c, double numPhotons);

// Kernel launchers (defined in the .cu files).
cudaError_t launchIntersect(const SceneView& s, const float* rays, int64_t n, int32_t* tri, double* t, float* pos,
                            float* nrm, cudaStream_t st, bool prefilter);
cudaError_t launchEnvLookup(const EnvDev& env, const float* dirs, int64_t n, float* out, cudaStream_t st);
cudaError_t launchEmit(const EnvDev& env, const double* tapes, int64_t n, double numPhotons, float* pos, float* dir,
                       float* flux, int* ok, cudaStream_t st);
cudaError_t launchHashPoints(const float* pts, int64_t n, uint32_t size, double scale, const double* bbmin, uint32_t* out,
                             cudaStream_t st);

}  // namespace pppm
