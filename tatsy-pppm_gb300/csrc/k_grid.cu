// Hash-grid build: per-photon bucket keys with a bucket histogram, an
// exclusive prefix sum over the histogram, and a scatter into bucket order.
#include "context.h"
#include "grid.cuh"
#include "kernels.h"

namespace pppm {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanThreads * kScanItems;  // 2048 counts per block

// kOwner: also records each bucket's cell (first photon's cell by
// compare-and-swap; a photon of another cell marks the bucket mixed)
template <bool kOwner>
__global__ void kKeys(const float4* __restrict__ rec, const uint64_t* __restrict__ count, int64_t capacity, GridDev g,
                      uint32_t* __restrict__ keys, uint32_t* __restrict__ hist, unsigned long long* __restrict__ owner) {
    const int64_t n = min((int64_t)*count, capacity);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = rec[2 * i];
        const int cx = cellCoord(a.x, g.ox, g.invCell, g.nx);
        const int cy = cellCoord(a.y, g.oy, g.invCell, g.ny);
        const int cz = cellCoord(a.z, g.oz, g.invCell, g.nz);
        const uint32_t k = bucketOf(cx, cy, cz, g.mask);
        keys[i] = k;
        atomicAdd(&hist[k], 1u);
        if (kOwner) {
            const unsigned long long code = cellCode(cx, cy, cz);
            const unsigned long long old = atomicCAS(&owner[k], kBucketEmpty, code);
            if (old != kBucketEmpty && old != code && old != kBucketMixed) atomicExch(&owner[k], kBucketMixed);
        }
    }
}

__device__ __forceinline__ uint32_t warpInclusive(uint32_t v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of kScanItems values per thread; returns the
// block total.
__device__ __forceinline__ uint32_t blockExclusive(uint32_t (&v)[kScanItems], uint32_t* warpSums) {
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const uint32_t x = v[k];
        v[k] = run;
        run += x;
    }
    const uint32_t inc = warpInclusive(run);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < (kScanThreads / 32) ? warpSums[lane] : 0u;
        s = warpInclusive(s);
        if (lane < (kScanThreads / 32)) warpSums[lane] = s;
    }
    __syncthreads();
    const uint32_t warpBase = warp > 0 ? warpSums[warp - 1] : 0u;
    const uint32_t base = warpBase + inc - run;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) v[k] += base;
    const uint32_t total = warpSums[kScanThreads / 32 - 1];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(kScanThreads) kScanChunks(const uint32_t* in, uint32_t* out,
                                                            uint32_t* __restrict__ chunkSums, int64_t n) {
    __shared__ uint32_t warpSums[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) v[k] = (base + k < n) ? in[base + k] : 0u;
    const uint32_t total = blockExclusive(v, warpSums);
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) out[base + k] = v[k];
    if (threadIdx.x == 0) chunkSums[blockIdx.x] = total;
}

// Exclusive scan of the chunk sums by one block (nChunks <= kScanChunk * 32).
__global__ void __launch_bounds__(kScanThreads) kScanSums(uint32_t* __restrict__ sums, int64_t nChunks,
                                                          uint32_t* __restrict__ grandTotal) {
    __shared__ uint32_t warpSums[kScanThreads / 32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t off = 0; off < nChunks; off += kScanChunk) {
        const int64_t base = off + threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; k++) v[k] = (base + k < nChunks) ? sums[base + k] : 0u;
        const uint32_t c = carry;
        const uint32_t total = blockExclusive(v, warpSums);
#pragma unroll
        for (int k = 0; k < kScanItems; k++)
            if (base + k < nChunks) sums[base + k] = v[k] + c;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grandTotal = carry;
}

__global__ void kAddChunkBase(uint32_t* __restrict__ out, const uint32_t* __restrict__ chunkBase, int64_t n,
                              uint32_t* __restrict__ cursor) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t v = out[i] + chunkBase[i / kScanChunk];
        out[i] = v;
        cursor[i] = v;
    }
}

__global__ void kScatter(const float4* __restrict__ rec, const uint64_t* __restrict__ count, int64_t capacity,
                         const uint32_t* __restrict__ keys, uint32_t* __restrict__ cursor, float4* __restrict__ sorted) {
    const int64_t n = min((int64_t)*count, capacity);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t dst = atomicAdd(&cursor[keys[i]], 1u);
        const float4 a = rec[2 * i], b = rec[2 * i + 1];
        sorted[2 * (int64_t)dst] = a;
        sorted[2 * (int64_t)dst + 1] = b;
    }
}

unsigned gridFor(int64_t n, int bs) {
    const int64_t want = (n + bs - 1) / bs;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, 152 * 16));
}

}  // namespace

// In-place exclusive prefix sum of data[0..n); data[n] receives the total and
// cursor[0..n) a copy of the offsets. tmp holds ceil(n / 2048) + 1 words.
cudaError_t exclusiveScan(uint32_t* data, int64_t n, uint32_t* cursor, uint32_t* tmp, cudaStream_t st) {
    const int64_t chunks = (n + kScanChunk - 1) / kScanChunk;
    kScanChunks<<<(unsigned)chunks, kScanThreads, 0, st>>>(data, data, tmp, n);
    kScanSums<<<1, kScanThreads, 0, st>>>(tmp, chunks, data + n);
    kAddChunkBase<<<gridFor(n, 256), 256, 0, st>>>(data, tmp, n, cursor);
    return cudaGetLastError();
}

int64_t scanTmpWords(int64_t n) { return (n + kScanChunk - 1) / kScanChunk + 1; }

namespace {
// cell edge, its inverse and the origin of the grid over the box; the cell
// count per axis stays below 2^20
void gridGeom(const double* bbmin, const double* bbmax, double cell, float* cellF, float* inv, float* origin) {
    double ext = 0.0;
    for (int d = 0; d < 3; d++) ext = std::max(ext, bbmax[d] - bbmin[d]);
    if (cell < ext / (double)(1 << 20)) cell = ext / (double)(1 << 20);
    if (!(cell > 0.0)) cell = 1.0;
    *cellF = (float)cell;
    *inv = (float)(1.0 / cell);
    for (int d = 0; d < 3; d++) origin[d] = (float)(bbmin[d] - 1e-3 * cell);
}

int cellsAlong(double hi, float origin, float inv) { return std::max(1, (int)std::ceil((hi - origin) * inv) + 1); }
}  // namespace

GridDev gridGeometry(const double* bbmin, const double* bbmax, double cell) {
    GridDev d{};
    float origin[3];
    gridGeom(bbmin, bbmax, cell, &d.cell, &d.invCell, origin);
    d.ox = origin[0];
    d.oy = origin[1];
    d.oz = origin[2];
    d.nx = cellsAlong(bbmax[0], origin[0], d.invCell);
    d.ny = cellsAlong(bbmax[1], origin[1], d.invCell);
    d.nz = cellsAlong(bbmax[2], origin[2], d.invCell);
    return d;
}

cudaError_t gridLayout(GridBufs& g, const double* bbmin, const double* bbmax, double cell, int64_t nPhotons) {
    // bucket table: next power of two >= 2 * photons, within [2^12, 2^26]
    uint32_t size = 1u << 12;
    while ((int64_t)size < 2 * nPhotons && size < (1u << 26)) size <<= 1;
    g.size = size;
    gridGeom(bbmin, bbmax, cell, &g.cell, &g.invCell, g.origin);
    cudaError_t e;
    if ((e = g.counts.ensure(((size_t)size + 1) * 4)) != cudaSuccess) return e;
    if ((e = g.cursor.ensure(((size_t)size + 1) * 4)) != cudaSuccess) return e;
    const int64_t chunks = ((int64_t)size + kScanChunk - 1) / kScanChunk;
    if ((e = g.scanTmp.ensure((size_t)(chunks + 1) * 4)) != cudaSuccess) return e;
    return cudaSuccess;
}

GridDev gridView(const GridBufs& g, const double* bbmin, const double* bbmax) {
    GridDev d;
    d.rec = g.sorted.as<float4>();
    d.start = g.counts.as<uint32_t>();
    d.mask = g.size - 1;
    d.ox = g.origin[0];
    d.oy = g.origin[1];
    d.oz = g.origin[2];
    d.cell = g.cell;
    d.invCell = g.invCell;
    d.nx = cellsAlong(bbmax[0], g.origin[0], g.invCell);
    d.ny = cellsAlong(bbmax[1], g.origin[1], g.invCell);
    d.nz = cellsAlong(bbmax[2], g.origin[2], g.invCell);
    d.owner = g.hasOwner ? g.owner.as<unsigned long long>() : nullptr;
    return d;
}

cudaError_t gridBuild(GridBufs& g, const GridDev& view, const float4* rec, const uint64_t* dCount, int64_t capacity,
                      cudaStream_t st, bool withOwner) {
    cudaError_t e;
    if ((e = g.keys.ensure((size_t)std::max<int64_t>(capacity, 1) * 4)) != cudaSuccess) return e;
    if ((e = g.sorted.ensure((size_t)std::max<int64_t>(capacity, 1) * 32)) != cudaSuccess) return e;
    uint32_t* hist = g.counts.as<uint32_t>();
    if ((e = cudaMemsetAsync(hist, 0, ((size_t)g.size + 1) * 4, st)) != cudaSuccess) return e;
    GridDev v = view;
    const int bs = 256;
    g.hasOwner = withOwner;
    if (withOwner) {
        if ((e = g.owner.ensure((size_t)g.size * 8)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(g.owner.p, 0xFF, (size_t)g.size * 8, st)) != cudaSuccess) return e;
        kKeys<true><<<gridFor(capacity, bs), bs, 0, st>>>(rec, dCount, capacity, v, g.keys.as<uint32_t>(), hist,
                                                          g.owner.as<unsigned long long>());
    } else {
        kKeys<false><<<gridFor(capacity, bs), bs, 0, st>>>(rec, dCount, capacity, v, g.keys.as<uint32_t>(), hist,
                                                           nullptr);
    }
    cudaError_t se = exclusiveScan(hist, (int64_t)g.size, g.cursor.as<uint32_t>(), g.scanTmp.as<uint32_t>(), st);
    if (se != cudaSuccess) return se;
    kScatter<<<gridFor(capacity, bs), bs, 0, st>>>(rec, dCount, capacity, g.keys.as<uint32_t>(), g.cursor.as<uint32_t>(),
                                                   g.sorted.as<float4>());
    return cudaGetLastError();
}

}  // namespace pppm
