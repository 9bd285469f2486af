// Canonical gather with shared-memory staging of grid cells.
//
// Queries are counting-sorted by the cell they fall in, then each block
// takes 128 consecutive sorted queries. For every distinct cell among them
// the block stages the photons of the cell's 3x3x3 neighbourhood (cell edge
// >= radius, so the neighbourhood covers every photon within the radius of
// any query in the cell) into shared memory in rounds of kStage photons, and
// each query of that cell tests every staged photon. The photons of a
// neighbourhood are read from L2/HBM once per block instead of once per
// query; hundreds of eye hit points typically share a cell.
#include "kernels.h"

namespace pppm {

namespace {

constexpr int kTileQ = 128;  // threads per block
#ifndef PPPM_GATHER_QPT
#define PPPM_GATHER_QPT 2
#endif
constexpr int kQ = PPPM_GATHER_QPT;  // queries per thread
constexpr int kStage = 1024;

unsigned blocksFor(int64_t n, int bs, int cap = 152 * 32) {
    const int64_t want = (n + bs - 1) / bs;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, cap));
}

__device__ __forceinline__ int64_t queryCount(const QueryView& qv) {
    return qv.count ? min((int64_t)*qv.count, qv.n) : qv.n;
}

__global__ void kQueryKeys(QueryView qv, GridDev g, uint32_t qmask, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ hist) {
    const int64_t n = queryCount(qv);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 q0 = qv.q[3 * i];
        const uint32_t k = bucketOf(cellCoord(q0.x, g.ox, g.invCell, g.nx), cellCoord(q0.y, g.oy, g.invCell, g.ny),
                                    cellCoord(q0.z, g.oz, g.invCell, g.nz), qmask);
        keys[i] = k;
        atomicAdd(&hist[k], 1u);
    }
}

__global__ void kQueryScatter(QueryView qv, const uint32_t* __restrict__ keys, uint32_t* __restrict__ cursor,
                              float4* __restrict__ sorted) {
    const int64_t n = queryCount(qv);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t dst = atomicAdd(&cursor[keys[i]], 1u);
        sorted[3 * (int64_t)dst] = qv.q[3 * i];
        sorted[3 * (int64_t)dst + 1] = qv.q[3 * i + 1];
        sorted[3 * (int64_t)dst + 2] = qv.q[3 * i + 2];
    }
}

// Each thread owns kQ consecutive sorted queries (usually of the same cell),
// so every staged photon is read from shared memory once for kQ tests.
template <bool kAccum, bool kCount>
__global__ void __launch_bounds__(kTileQ) kGatherTiled(GridDev g, const float4* __restrict__ sq,
                                                       const uint32_t* __restrict__ qcount, int64_t qcap, float r,
                                                       float* __restrict__ out, unsigned long long* __restrict__ work) {
    __shared__ float4 sA[kStage];  // pos.xyz, normal.x
    __shared__ float4 sB[kStage];  // flux.xyz, normal.y
    __shared__ float sC[kStage];   // normal.z
    __shared__ uint32_t sKey[27];
    __shared__ uint32_t sBeg[27];
    __shared__ uint32_t sOff[28];
    __shared__ int sNk, sLeader, sCx, sCy, sCz;

    const int64_t n = qcount ? min((int64_t)*qcount, qcap) : qcap;
    const int64_t base = (int64_t)blockIdx.x * (kTileQ * kQ);
    if (base >= n) return;  // uniform for the whole block
    float4 q0[kQ], q1[kQ], q2[kQ];
    int cx[kQ], cy[kQ], cz[kQ];
    bool valid[kQ], pending[kQ];
    float sx[kQ], sy[kQ], sz[kQ];
#pragma unroll
    for (int j = 0; j < kQ; j++) {
        const int64_t i = base + (int64_t)kQ * threadIdx.x + j;
        valid[j] = i < n;
        q0[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        q1[j] = q0[j];
        q2[j] = q0[j];
        cx[j] = cy[j] = cz[j] = -1;
        if (valid[j]) {
            q0[j] = sq[3 * i];
            q1[j] = sq[3 * i + 1];
            q2[j] = sq[3 * i + 2];
            cx[j] = cellCoord(q0[j].x, g.ox, g.invCell, g.nx);
            cy[j] = cellCoord(q0[j].y, g.oy, g.invCell, g.ny);
            cz[j] = cellCoord(q0[j].z, g.oz, g.invCell, g.nz);
        }
        pending[j] = valid[j];
        sx[j] = sy[j] = sz[j] = 0.f;
    }
    const float r2 = r * r;
    unsigned long long pairs = 0, inside = 0;
    for (;;) {
        if (threadIdx.x == 0) sLeader = kTileQ * kQ;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kQ; j++)
            if (pending[j]) atomicMin(&sLeader, kQ * (int)threadIdx.x + j);
        __syncthreads();
        const int leader = sLeader;
        if (leader == kTileQ * kQ) break;
        if ((int)threadIdx.x == leader / kQ) {
            const int j = leader % kQ;
            sCx = cx[j];
            sCy = cy[j];
            sCz = cz[j];
        }
        __syncthreads();
        bool active[kQ];
        bool any = false;
#pragma unroll
        for (int j = 0; j < kQ; j++) {
            active[j] = pending[j] && cx[j] == sCx && cy[j] == sCy && cz[j] == sCz;
            any |= active[j];
        }
        if (threadIdx.x == 0) {
            // the 3x3x3 neighbourhood of the leader's cell, buckets deduplicated
            int nk = 0;
            uint32_t off = 0;
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int x = sCx + dx, y = sCy + dy, z = sCz + dz;
                        if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) continue;
                        const uint32_t k = bucketOf(x, y, z, g.mask);
                        bool dup = false;
                        for (int t = 0; t < nk; t++) dup |= sKey[t] == k;
                        if (dup) continue;
                        const uint32_t b0 = g.start[k], b1 = g.start[k + 1];
                        if (b1 == b0) continue;
                        sKey[nk] = k;
                        sBeg[nk] = b0;
                        sOff[nk] = off;
                        off += b1 - b0;
                        nk++;
                    }
            sOff[nk] = off;
            sNk = nk;
        }
        __syncthreads();
        const int nk = sNk;
        const uint32_t total = sOff[nk];
        for (uint32_t cb = 0; cb < total; cb += kStage) {
            const uint32_t cnt = min((uint32_t)kStage, total - cb);
            for (uint32_t t = threadIdx.x; t < cnt; t += kTileQ) {
                const uint32_t v = cb + t;
                int b = 0;
                while (b + 1 < nk && sOff[b + 1] <= v) b++;
                const int64_t jj = (int64_t)sBeg[b] + (v - sOff[b]);
                const float4 a = __ldg(&g.rec[2 * jj]);
                const float4 f = __ldg(&g.rec[2 * jj + 1]);
                const f3 nn = unpackNormal(__float_as_uint(a.w));
                sA[t] = make_float4(a.x, a.y, a.z, nn.x);
                sB[t] = make_float4(f.x, f.y, f.z, nn.y);
                sC[t] = nn.z;
            }
            __syncthreads();
            if (any) {
                if (kCount) {
#pragma unroll
                    for (int j = 0; j < kQ; j++) pairs += active[j] ? cnt : 0;
                }
#pragma unroll 2
                for (uint32_t t = 0; t < cnt; t++) {
                    const float4 a = sA[t];
                    bool in[kQ];
                    bool anyIn = false;
#pragma unroll
                    for (int j = 0; j < kQ; j++) {
                        const float dx = a.x - q0[j].x, dy = a.y - q0[j].y, dz = a.z - q0[j].z;
                        in[j] = active[j] && dx * dx + dy * dy + dz * dz < r2;
                        anyIn |= in[j];
                    }
                    if (anyIn) {
                        const float4 b = sB[t];
                        const float c = sC[t];
#pragma unroll
                        for (int j = 0; j < kQ; j++) {
                            if (!in[j]) continue;
                            if (kCount) inside++;
                            if (a.w * q1[j].x + b.w * q1[j].y + c * q1[j].z > 0.0f) {
                                sx[j] += b.x;
                                sy[j] += b.y;
                                sz[j] += b.z;
                            }
                        }
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int j = 0; j < kQ; j++)
            if (active[j]) pending[j] = false;
    }
    const float norm = 1.0f / (kPiF * kPiF * r2);
#pragma unroll
    for (int j = 0; j < kQ; j++) {
        if (!valid[j]) continue;
        const float lx = q2[j].x * sx[j] * norm, ly = q2[j].y * sy[j] * norm, lz = q2[j].z * sz[j] * norm;
        const int64_t px = __float_as_int(q0[j].w);
        if (kAccum) {
            out[3 * px] += lx;
            out[3 * px + 1] += ly;
            out[3 * px + 2] += lz;
        } else {
            out[3 * px] = lx;
            out[3 * px + 1] = ly;
            out[3 * px + 2] = lz;
        }
    }
    if (kCount) {
        const unsigned long long wp = __reduce_add_sync(0xffffffffu, (unsigned)pairs);
        const unsigned long long wi = __reduce_add_sync(0xffffffffu, (unsigned)inside);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&work[0], wp);
            atomicAdd(&work[1], wi);
        }
    }
}

}  // namespace

cudaError_t querySortLayout(QuerySortBufs& qs, int64_t maxQueries) {
    uint32_t size = 1u << 10;
    while ((int64_t)size < 2 * maxQueries && size < (1u << 26)) size <<= 1;
    qs.size = size;
    cudaError_t e;
    if ((e = qs.hist.ensure(((size_t)size + 1) * 4)) != cudaSuccess) return e;
    if ((e = qs.cursor.ensure(((size_t)size + 1) * 4)) != cudaSuccess) return e;
    if ((e = qs.tmp.ensure((size_t)scanTmpWords(size) * 4)) != cudaSuccess) return e;
    if ((e = qs.keys.ensure((size_t)std::max<int64_t>(maxQueries, 1) * 4)) != cudaSuccess) return e;
    return qs.sorted.ensure((size_t)std::max<int64_t>(maxQueries, 1) * 48);
}

cudaError_t launchGatherTiled(const GridDev& g, QueryView qv, QuerySortBufs& qs, float radius, float* out,
                              bool accumulate, unsigned long long* work, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(qs.hist.p, 0, ((size_t)qs.size + 1) * 4, st)) != cudaSuccess) return e;
    kQueryKeys<<<blocksFor(qv.n, 256), 256, 0, st>>>(qv, g, qs.size - 1, qs.keys.as<uint32_t>(), qs.hist.as<uint32_t>());
    if ((e = exclusiveScan(qs.hist.as<uint32_t>(), qs.size, qs.cursor.as<uint32_t>(), qs.tmp.as<uint32_t>(), st)) !=
        cudaSuccess)
        return e;
    kQueryScatter<<<blocksFor(qv.n, 256), 256, 0, st>>>(qv, qs.keys.as<uint32_t>(), qs.cursor.as<uint32_t>(),
                                                        qs.sorted.as<float4>());
    // the sorted count equals the query count; the tiled kernel reads it
    // from the end of the scanned histogram
    const uint32_t* total = qs.hist.as<uint32_t>() + qs.size;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, (qv.n + kTileQ * kQ - 1) / (kTileQ * kQ));
    const float4* sq = qs.sorted.as<float4>();
    if (accumulate && work) kGatherTiled<true, true><<<blocks, kTileQ, 0, st>>>(g, sq, total, qv.n, radius, out, work);
    else if (accumulate) kGatherTiled<true, false><<<blocks, kTileQ, 0, st>>>(g, sq, total, qv.n, radius, out, work);
    else if (work) kGatherTiled<false, true><<<blocks, kTileQ, 0, st>>>(g, sq, total, qv.n, radius, out, work);
    else kGatherTiled<false, false><<<blocks, kTileQ, 0, st>>>(g, sq, total, qv.n, radius, out, work);
    return cudaGetLastError();
}

}  // namespace pppm
