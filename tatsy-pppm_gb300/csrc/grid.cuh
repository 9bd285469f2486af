// Photon hash grid shared by the build and gather kernels.
//
// Cells are cubes of edge `cell` anchored at `origin`; a cell (cx, cy, cz)
// maps to bucket refHash(cx, cy, cz) & mask, the reference's HashGrid hash
// (hash_grid_detail.h:60-63) over a power-of-two table. Photons are counting-
// sorted by bucket, so a bucket is a contiguous range [start[b], start[b+1]).
// Different cells may share a bucket; gathers either dedupe buckets or keep
// only photons whose own cell is the scanned cell.
#pragma once

#include "pppm_device.cuh"

namespace pppm {

struct GridDev {
    const float4* rec;       // 2 float4 per photon: (pos, packed normal), (flux, stream)
    const uint32_t* start;   // size + 1 offsets
    uint32_t mask;
    float ox, oy, oz;        // origin
    float invCell, cell;
    int nx, ny, nz;          // cells per axis
    // per bucket the one cell its photons lie in (cellCode), kBucketMixed
    // when photons of several cells share it, kBucketEmpty when it has none;
    // nullptr when the build did not record it
    const unsigned long long* owner = nullptr;
};

constexpr unsigned long long kBucketEmpty = ~0ull;
constexpr unsigned long long kBucketMixed = ~0ull - 1;

// cell coordinates (each below 2^20) packed into one 64-bit code
__host__ __device__ __forceinline__ unsigned long long cellCode(int cx, int cy, int cz) {
    return (unsigned long long)cx | ((unsigned long long)cy << 21) | ((unsigned long long)cz << 42);
}

__device__ __forceinline__ uint32_t bucketOf(int cx, int cy, int cz, uint32_t mask) {
    const uint32_t h = ((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u) ^ ((uint32_t)cz * 83492791u);
    return h & mask;
}

__device__ __forceinline__ int cellCoord(float p, float o, float inv, int n) {
    const int c = __float2int_rd((p - o) * inv);
    return min(max(c, 0), n - 1);
}

}  // namespace pppm
