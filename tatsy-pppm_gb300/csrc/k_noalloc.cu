// pppm_knn_noalloc: the k-nearest photon query (PhotonMap::findKNN
// semantics, as pppm_knn) without any memory allocation, for callers that
// own every byte of device memory themselves and cannot let a library call
// cudaMalloc: a host application that runs this code as a plugin under a
// fixed GPU memory budget, a frame loop that must not stall on cudaMalloc's
// device-wide synchronisation, or a program that must not create the
// context pppm_create allocates. The caller passes device (or managed)
// arrays and a stream; the grid scratch lives in one file-scope device array
// of fixed size that every GPU loading the library holds until exit.
#include <mutex>

#include "kernels.h"
#include "noalloc_check.h"

namespace pppm {

namespace {

constexpr int64_t kNaMaxPhotons = PPPM_NOALLOC_MAX_PHOTONS;
constexpr uint32_t kNaTable = 1u << 18;  // buckets: power of two >= 2 * max photons
constexpr size_t kNaChunkWords = kNaTable / 2048 + 2;

// Scratch layout (bytes, each region 256-byte aligned).
struct NaLayout {
    static constexpr size_t params = 0;                                   // NaParams
    static constexpr size_t sorted = 256;                                 // 2 float4 per photon
    static constexpr size_t keys = sorted + 32 * (size_t)kNaMaxPhotons;   // uint32 per photon
    static constexpr size_t hist = keys + 4 * (size_t)kNaMaxPhotons;      // table + 1 counts -> offsets
    static constexpr size_t cursor = hist + 4 * ((size_t)kNaTable + 64);  // table + 1
    static constexpr size_t tmp = cursor + 4 * ((size_t)kNaTable + 64);   // scan chunk sums
    static constexpr size_t total = tmp + 4 * ((kNaChunkWords + 63) / 64 * 64);
};

static __device__ __align__(256) unsigned char gScratch[NaLayout::total];

struct NaParams {
    int bbmin[3];  // order-preserving integer images of the bounding box
    int bbmax[3];
    GridDev grid;
};
static_assert(sizeof(NaParams) <= NaLayout::sorted, "the parameters must fit their scratch region");

// float <-> int mapping that preserves order, for atomicMin/atomicMax
__device__ __forceinline__ int orderedInt(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float orderedFloat(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void kNaInit(NaParams* p) {
    for (int d = 0; d < 3; d++) {
        p->bbmin[d] = orderedInt(3.0e38f);
        p->bbmax[d] = orderedInt(-3.0e38f);
    }
}

__global__ void kNaBbox(const float* __restrict__ pos, int64_t n, NaParams* p) {
    float mn[3] = {3.0e38f, 3.0e38f, 3.0e38f}, mx[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < 3; d++) {
            mn[d] = fminf(mn[d], pos[3 * i + d]);
            mx[d] = fmaxf(mx[d], pos[3 * i + d]);
        }
    for (int d = 0; d < 3; d++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&p->bbmin[d], orderedInt(mn[d]));
            atomicMax(&p->bbmax[d], orderedInt(mx[d]));
        }
    }
}

// The grid layout of pppm_knn (render.cu knnCell + k_grid.cu gridLayout),
// computed on the device from the reduced bounding box.
__global__ void kNaParams(NaParams* p, int64_t n, int k, float4* sorted, uint32_t* hist) {
    double mn[3], mx[3];
    for (int d = 0; d < 3; d++) {
        mn[d] = orderedFloat(p->bbmin[d]);
        mx[d] = orderedFloat(p->bbmax[d]);
    }
    if (n == 0)
        for (int d = 0; d < 3; d++) { mn[d] = 0.0; mx[d] = 1.0; }
    double ex = 1e-6;
    for (int d = 0; d < 3; d++) ex = fmax(ex, mx[d] - mn[d]);
    const double frac = fmin(1.0, (double)(k > 1 ? k : 1) / (double)(n > 1 ? n : 1));
    double cell = ex * cbrt(frac);
    double ext = 0.0;
    for (int d = 0; d < 3; d++) ext = fmax(ext, mx[d] - mn[d]);
    if (cell < ext / (double)(1 << 20)) cell = ext / (double)(1 << 20);
    if (!(cell > 0.0)) cell = 1.0;
    uint32_t size = 1u << 12;
    while ((int64_t)size < 2 * n && size < kNaTable) size <<= 1;
    GridDev& g = p->grid;
    g.rec = sorted;
    g.start = hist;
    g.mask = size - 1;
    g.cell = (float)cell;
    g.invCell = (float)(1.0 / cell);
    g.ox = (float)(mn[0] - 1e-3 * cell);
    g.oy = (float)(mn[1] - 1e-3 * cell);
    g.oz = (float)(mn[2] - 1e-3 * cell);
    g.nx = max(1, (int)ceil((mx[0] - g.ox) * g.invCell) + 1);
    g.ny = max(1, (int)ceil((mx[1] - g.oy) * g.invCell) + 1);
    g.nz = max(1, (int)ceil((mx[2] - g.oz) * g.invCell) + 1);
    g.owner = nullptr;  // no bucket owners recorded: the search tests every photon's cell
}

__global__ void kNaKeys(const float* __restrict__ pos, int64_t n, const NaParams* p, uint32_t* __restrict__ keys,
                        uint32_t* __restrict__ hist) {
    const GridDev g = p->grid;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = bucketOf(cellCoord(pos[3 * i], g.ox, g.invCell, g.nx),
                                    cellCoord(pos[3 * i + 1], g.oy, g.invCell, g.ny),
                                    cellCoord(pos[3 * i + 2], g.oz, g.invCell, g.nz), g.mask);
        keys[i] = k;
        atomicAdd(&hist[k], 1u);
    }
}

__global__ void kNaScatter(const float* __restrict__ pos, int64_t n, const uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ cursor, float4* __restrict__ sorted) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t dst = atomicAdd(&cursor[keys[i]], 1u);
        sorted[2 * (int64_t)dst] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.0f);
        sorted[2 * (int64_t)dst + 1] = make_float4(0.f, 0.f, 0.f, __int_as_float((int)i));
    }
}

unsigned naBlocks(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 152 * 8 ? 152 * 8 : b));
}

// Device address of gScratch per device ordinal, looked up once per device
// with that device current. Host code may not use &gScratch as a device
// address: on the host it names a host-side shadow of the symbol. The
// address belongs to the device's primary context as it was at the first
// call; a cudaDeviceReset while the library is loaded discards that context
// and the cached address with it, so resetting a device that has used this
// entry point is not supported.
std::mutex gScratchMutex;
void* gScratchAddr[256] = {nullptr};

static_assert(kNaUnregistered == (int)cudaMemoryTypeUnregistered && kNaHost == (int)cudaMemoryTypeHost &&
                  kNaDevice == (int)cudaMemoryTypeDevice && kNaManaged == (int)cudaMemoryTypeManaged,
              "NaMemoryType mirrors cudaMemoryType");

// naPointerUsable on the pointer's attributes (noalloc_check.h).
bool usableOn(const void* ptr, int device) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return naPointerUsable((int)a.type, a.device, device);
}

// Clears the pending CUDA error so that it does not surface in the
// caller's next unrelated cudaGetLastError, and reports the failure.
int cudaFailure() {
    cudaGetLastError();
    return PPPM_E_CUDA;
}

int scratchFor(int device, unsigned char** out) {
    if (device < 0 || device >= 256) return PPPM_E_ARG;
    std::lock_guard<std::mutex> lock(gScratchMutex);
    if (gScratchAddr[device] == nullptr) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, gScratch) != cudaSuccess || ptr == nullptr) return cudaFailure();
        gScratchAddr[device] = ptr;
    }
    *out = static_cast<unsigned char*>(gScratchAddr[device]);
    return PPPM_OK;
}

}  // namespace

}  // namespace pppm

using namespace pppm;

extern "C" int pppm_knn_noalloc(const float* photon_pos, int64_t n, const float* queries, int64_t m,
                                int32_t num_target_photons, double target_radius, int32_t* idx, int32_t* cnt,
                                int32_t cap, void* stream) {
    if (n < 0 || m < 0 || cap < 0 || (n > 0 && !photon_pos) || (m > 0 && (!queries || !cnt || (cap > 0 && !idx))))
        return PPPM_E_ARG;
    if (n > kNaMaxPhotons) return PPPM_E_CAPACITY;
    const int k = (int)target_radius;  // the reference's swapped KnnQuery arguments (photon_map.cc:25)
    if (k < 1) return PPPM_E_UNDEFINED;
    if (k > kMaxKnn) return PPPM_E_CAPACITY;
    if (m == 0) return PPPM_OK;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return cudaFailure();
    // nothing is staged: every array must already be memory the current
    // device reads directly (its own device memory, or managed memory)
    if ((n > 0 && !usableOn(photon_pos, device)) || !usableOn(queries, device) || !usableOn(cnt, device) ||
        (cap > 0 && !usableOn(idx, device)))
        return PPPM_E_ARG;
    unsigned char* s = nullptr;
    const int r = scratchFor(device, &s);
    if (r) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NaParams* p = reinterpret_cast<NaParams*>(s + NaLayout::params);
    float4* sorted = reinterpret_cast<float4*>(s + NaLayout::sorted);
    uint32_t* keys = reinterpret_cast<uint32_t*>(s + NaLayout::keys);
    uint32_t* hist = reinterpret_cast<uint32_t*>(s + NaLayout::hist);
    uint32_t* cursor = reinterpret_cast<uint32_t*>(s + NaLayout::cursor);
    uint32_t* tmp = reinterpret_cast<uint32_t*>(s + NaLayout::tmp);
    // the previous call's contents stay in the array: clear what starts at zero
    if (cudaMemsetAsync(hist, 0, 4 * ((size_t)kNaTable + 1), st) != cudaSuccess) return cudaFailure();
    kNaInit<<<1, 1, 0, st>>>(p);
    kNaBbox<<<naBlocks(n), 256, 0, st>>>(photon_pos, n, p);
    kNaParams<<<1, 1, 0, st>>>(p, n, k, sorted, hist);
    kNaKeys<<<naBlocks(n), 256, 0, st>>>(photon_pos, n, p, keys, hist);
    // the bucket table size depends only on n (as in pppm_knn)
    uint32_t size = 1u << 12;
    while ((int64_t)size < 2 * n && size < kNaTable) size <<= 1;
    if (exclusiveScan(hist, size, cursor, tmp, st) != cudaSuccess) return cudaFailure();
    kNaScatter<<<naBlocks(n), 256, 0, st>>>(photon_pos, n, keys, cursor, sorted);
    // the query kernel takes the grid description by value: read it back
    // into host stack memory (this waits for the stream)
    NaParams hp;
    if (cudaMemcpyAsync(&hp, p, sizeof(hp), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return cudaFailure();
    if (launchKnn(hp.grid, queries, m, k, (float)num_target_photons, idx, cnt, cap, st) != cudaSuccess)
        return cudaFailure();
    if (cudaStreamSynchronize(st) != cudaSuccess) return cudaFailure();
    return PPPM_OK;
}
