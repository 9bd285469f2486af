// Canonical gather with shared-memory staging of grid cells.
//
// Queries are counting-sorted by the cell they fall in, then each warp
// takes 64 consecutive sorted queries. For every distinct cell among them
// the warp stages the photons of the cell's 3x3x3 neighbourhood (cell edge
// >= radius, so the neighbourhood covers every photon within the radius of
// any query in the cell) into its shared-memory tile in rounds of `stage`
// photons, and each query of that cell tests every staged photon. The
// photons of a neighbourhood are read from L2/HBM once per warp instead of
// once per query; hundreds of eye hit points typically share a cell.
#include <type_traits>

#include "kernels.h"

namespace pppm {

namespace {

constexpr int kTileQ = 128;  // threads per block
#ifndef PPPM_GATHER_QPT
#define PPPM_GATHER_QPT 2
#endif
constexpr int kQ = PPPM_GATHER_QPT;  // queries per thread
constexpr int kWarps = kTileQ / 32;
#ifndef PPPM_GATHER_MINBLOCKS
#define PPPM_GATHER_MINBLOCKS 7
#endif
// photons per iteration of the tile loop
#ifndef PPPM_GATHER_UNROLL
#define PPPM_GATHER_UNROLL 4
#endif
constexpr int kUnroll = PPPM_GATHER_UNROLL;

// distance tests in coordinates relative to the centre of the warp's cell:
// the tile holds p - c and |p - c|^2, so that a test is three FMAs and a
// compare, |p'|^2 - 2 p'.q' < r^2 - |q'|^2 (1: default; 0: the difference
// vector's squared length, seven instructions). With |p'|, |q'| a few radii
// at most, the rounding of d^2 - r^2 stays below 2e-6 r^2 for cells up to
// 2r (4e-6 r^2 at 4r), inside the 1e-5 r^2 band in which the float64
// restatement treats a photon as on the sphere. The centre depends only on
// the query's own cell, so a query's sum does not depend on which queries
// share its warp.
#ifndef PPPM_GATHER_LOCAL
#define PPPM_GATHER_LOCAL 1
#endif
constexpr bool kLocal = PPPM_GATHER_LOCAL != 0;
// the third tile array: normal.z (float), or normal.yz (float2) in local form
using TileC = std::conditional_t<kLocal, float2, float>;

// dynamic shared memory of a gather block with tiles of `stage` photons
size_t gatherSmem(int stage) { return (size_t)kWarps * stage * (2 * sizeof(float4) + sizeof(TileC)); }

unsigned blocksFor(int64_t n, int bs, int cap = 152 * 32) {
    const int64_t want = (n + bs - 1) / bs;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, cap));
}

__device__ __forceinline__ int64_t queryCount(const QueryView& qv) {
    return qv.count ? min((int64_t)*qv.count, qv.n) : qv.n;
}

// Sort key of a query: its cell's bucket, then the Morton index of its
// sub-cell (2^subBits per axis), so that the 64 queries of a warp lie close
// together and the photons it stages can be culled against their bounding
// box.
__device__ __forceinline__ uint32_t spread3(uint32_t v, int subBits) {
    uint32_t r = 0;
    for (int b = 0; b < subBits; b++) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}

__global__ void kQueryKeys(QueryView qv, GridDev g, uint32_t qmask, int subBits, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ hist) {
    const int64_t n = queryCount(qv);
    const int kSub = 1 << subBits;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 q0 = qv.q[3 * i];
        const float fx = (q0.x - g.ox) * g.invCell, fy = (q0.y - g.oy) * g.invCell, fz = (q0.z - g.oz) * g.invCell;
        const int cx = cellCoord(q0.x, g.ox, g.invCell, g.nx), cy = cellCoord(q0.y, g.oy, g.invCell, g.ny),
                  cz = cellCoord(q0.z, g.oz, g.invCell, g.nz);
        const uint32_t sx = (uint32_t)min(max(__float2int_rd((fx - (float)cx) * kSub), 0), kSub - 1);
        const uint32_t sy = (uint32_t)min(max(__float2int_rd((fy - (float)cy) * kSub), 0), kSub - 1);
        const uint32_t sz = (uint32_t)min(max(__float2int_rd((fz - (float)cz) * kSub), 0), kSub - 1);
        const uint32_t k = (bucketOf(cx, cy, cz, qmask >> (3 * subBits)) << (3 * subBits)) | spread3(sx, subBits) |
                           (spread3(sy, subBits) << 1) | (spread3(sz, subBits) << 2);
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

// Each warp owns 32 * kQ consecutive sorted queries (kQ per lane, usually of
// one cell) and stages the photons of its cell's 3x3x3 neighbourhood in its
// own shared-memory tile of `stage` photons (dynamic shared memory,
// gatherSmem(stage) bytes per block), synchronising with __syncwarp only:
// warps whose queries lie in different cells work on their neighbourhoods
// side by side instead of waiting for one another at block barriers. Every
// staged photon is read from shared memory once for kQ tests per lane. The
// tile size changes only how often a warp flushes its tile, not which
// photons a query sums or in which order.
// kStage > 0: tiles of kStage photons in static shared memory (the default
// shape); 0: tiles of `stageRt` photons in dynamic shared memory.
template <bool kAccum, bool kCount, int kStage>
__global__ void __launch_bounds__(kTileQ, PPPM_GATHER_MINBLOCKS) kGatherTiled(GridDev g, const float4* __restrict__ sq,
                                                       const uint32_t* __restrict__ qcount, int64_t qcap, float r,
                                                       int stageRt, float* __restrict__ out,
                                                       unsigned long long* __restrict__ work) {
    // per warp: pos.xyz|normal.x, flux.xyz|normal.y, normal.z of `stage`
    // photons; local form: (p - c).xyz|(|p - c|^2), flux.xyz|normal.x, normal.yz
    const int stage = kStage > 0 ? kStage : stageRt;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t n = qcount ? min((int64_t)*qcount, qcap) : qcap;
    const int64_t base = ((int64_t)blockIdx.x * kWarps + warp) * (32 * kQ);
    if (base >= n) return;  // uniform for the warp; the kernel has no block barrier
    float4* wA;
    float4* wB;
    TileC* wC;
    if constexpr (kStage > 0) {
        __shared__ float4 sA[kWarps][kStage > 0 ? kStage : 1];
        __shared__ float4 sB[kWarps][kStage > 0 ? kStage : 1];
        __shared__ TileC sC[kWarps][kStage > 0 ? kStage : 1];
        wA = sA[warp];
        wB = sB[warp];
        wC = sC[warp];
    } else {
        extern __shared__ float4 tileDynamic[];
        wA = tileDynamic + (size_t)warp * stage;
        wB = tileDynamic + (size_t)(kWarps + warp) * stage;
        wC = reinterpret_cast<TileC*>(tileDynamic + (size_t)2 * kWarps * stage) + (size_t)warp * stage;
    }
    // position and normal of each query stay in registers; its weight and
    // pixel are read again for the final write
    float3 q0[kQ], q1[kQ];
    int cx[kQ], cy[kQ], cz[kQ];
    bool valid[kQ], pending[kQ];
    float sx[kQ], sy[kQ], sz[kQ];
#pragma unroll
    for (int j = 0; j < kQ; j++) {
        const int64_t i = base + (int64_t)kQ * lane + j;
        valid[j] = i < n;
        q0[j] = make_float3(0.f, 0.f, 0.f);
        q1[j] = q0[j];
        cx[j] = cy[j] = cz[j] = -1;
        if (valid[j]) {
            const float4 a = sq[3 * i], b = sq[3 * i + 1];
            q0[j] = make_float3(a.x, a.y, a.z);
            q1[j] = make_float3(b.x, b.y, b.z);
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
        // the leader: the first pending query of the warp
        bool pend = false;
        int fx = 0, fy = 0, fz = 0;
#pragma unroll
        for (int j = kQ - 1; j >= 0; j--)
            if (pending[j]) {
                pend = true;
                fx = cx[j];
                fy = cy[j];
                fz = cz[j];
            }
        const unsigned pm = __ballot_sync(0xffffffffu, pend);
        if (pm == 0) break;
        const int leader = __ffs(pm) - 1;
        const int lx = __shfl_sync(0xffffffffu, fx, leader);
        const int ly = __shfl_sync(0xffffffffu, fy, leader);
        const int lz = __shfl_sync(0xffffffffu, fz, leader);
        bool active[kQ];
        bool any = false;
#pragma unroll
        for (int j = 0; j < kQ; j++) {
            active[j] = pending[j] && cx[j] == lx && cy[j] == ly && cz[j] == lz;
            any |= active[j];
        }
        // lane i < 27 holds neighbour cell (i % 3 - 1, i / 3 % 3 - 1, i / 9 - 1)
        // of the leader's cell; a bucket reached from two cells (hash
        // collision) is kept at its first lane only
        uint32_t key = 0xffffffffu, b0 = 0, nc = 0;
        if (lane < 27) {
            const int x = lx + lane % 3 - 1, y = ly + (lane / 3) % 3 - 1, z = lz + lane / 9 - 1;
            if (x >= 0 && y >= 0 && z >= 0 && x < g.nx && y < g.ny && z < g.nz) key = bucketOf(x, y, z, g.mask);
        }
        const unsigned same = __match_any_sync(0xffffffffu, key);
        if (key != 0xffffffffu && (same & ((1u << lane) - 1u)) == 0) {
            b0 = g.start[key];
            nc = g.start[key + 1] - b0;
        }
        // the active queries' positions; the local form reads them again from
        // the sorted queries, so that none stays live across the tests (kept
        // in registers, they spilled)
        float3 qp[kQ];
#pragma unroll
        for (int j = 0; j < kQ; j++) {
            if constexpr (kLocal) {
                qp[j] = make_float3(0.f, 0.f, 0.f);
                if (active[j]) {
                    const float4 a = sq[3 * (base + (int64_t)kQ * lane + j)];
                    qp[j] = make_float3(a.x, a.y, a.z);
                }
            } else {
                qp[j] = q0[j];
            }
        }
        // bounding box of the warp's active queries; a photon farther than r
        // from the box is farther than r from each of them (kept with a
        // margin over the rounding of the distance tests)
        const float inf = __int_as_float(0x7f800000);
        float blx = inf, bly = inf, blz = inf, bhx = -inf, bhy = -inf, bhz = -inf;
#pragma unroll
        for (int j = 0; j < kQ; j++)
            if (active[j]) {
                blx = fminf(blx, qp[j].x);
                bly = fminf(bly, qp[j].y);
                blz = fminf(blz, qp[j].z);
                bhx = fmaxf(bhx, qp[j].x);
                bhy = fmaxf(bhy, qp[j].y);
                bhz = fmaxf(bhz, qp[j].z);
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            blx = fminf(blx, __shfl_xor_sync(0xffffffffu, blx, o));
            bly = fminf(bly, __shfl_xor_sync(0xffffffffu, bly, o));
            blz = fminf(blz, __shfl_xor_sync(0xffffffffu, blz, o));
            bhx = fmaxf(bhx, __shfl_xor_sync(0xffffffffu, bhx, o));
            bhy = fmaxf(bhy, __shfl_xor_sync(0xffffffffu, bhy, o));
            bhz = fmaxf(bhz, __shfl_xor_sync(0xffffffffu, bhz, o));
        }
        const float rc2 = r2 * 1.0001f;
        // local form: the leader's cell centre, each active query's -2 q' and
        // its threshold r^2 - |q'|^2 (-inf for the others: no photon passes)
        const float ccx = g.ox + ((float)lx + 0.5f) * g.cell, ccy = g.oy + ((float)ly + 0.5f) * g.cell,
                    ccz = g.oz + ((float)lz + 0.5f) * g.cell;
        float mx[kQ], my[kQ], mz[kQ], thr[kQ];
        if constexpr (kLocal) {
#pragma unroll
            for (int j = 0; j < kQ; j++) {
                const float x = qp[j].x - ccx, y = qp[j].y - ccy, z = qp[j].z - ccz;
                mx[j] = -2.0f * x;
                my[j] = -2.0f * y;
                mz[j] = -2.0f * z;
                thr[j] = active[j] ? r2 - (x * x + y * y + z * z) : -inf;
            }
        }
        // tests every query of the leader's cell against the tile's photons
        auto testTile = [&](uint32_t fill) {
            __syncwarp();
            if (any) {
                if (kCount) {
#pragma unroll
                    for (int j = 0; j < kQ; j++) pairs += active[j] ? fill : 0;
                }
#pragma unroll kUnroll
                for (uint32_t t = 0; t < fill; t++) {
                    if constexpr (kLocal) {
                        const float4 a = wA[t];
                        bool in[kQ];
                        bool anyIn = false;
#pragma unroll
                        for (int j = 0; j < kQ; j++) {
                            in[j] = fmaf(mz[j], a.z, fmaf(my[j], a.y, fmaf(mx[j], a.x, a.w))) < thr[j];
                            anyIn |= in[j];
                        }
                        if (anyIn) {
                            const float4 b = wB[t];
                            const float2 c = *reinterpret_cast<const float2*>(&wC[t]);
#pragma unroll
                            for (int j = 0; j < kQ; j++) {
                                if (!in[j]) continue;
                                if (kCount) inside++;
                                if (b.w * q1[j].x + c.x * q1[j].y + c.y * q1[j].z > 0.0f) {
                                    sx[j] += b.x;
                                    sy[j] += b.y;
                                    sz[j] += b.z;
                                }
                            }
                        }
                        continue;
                    }
                    const float4 a = wA[t];
                    bool in[kQ];
                    bool anyIn = false;
#pragma unroll
                    for (int j = 0; j < kQ; j++) {
                        const float dx = a.x - q0[j].x, dy = a.y - q0[j].y, dz = a.z - q0[j].z;
                        in[j] = active[j] && dx * dx + dy * dy + dz * dz < r2;
                        anyIn |= in[j];
                    }
                    if (anyIn) {
                        const float4 b = wB[t];
                        const float c = *reinterpret_cast<const float*>(&wC[t]);
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
            __syncwarp();
        };
        // the neighbourhood's photons in bucket order, 32 at a time; those
        // within reach are packed into the tile in the same order
        const unsigned lt = (1u << lane) - 1u;
        unsigned segs = __ballot_sync(0xffffffffu, nc > 0);
        uint32_t fill = 0;
        while (segs) {
            const int sgi = __ffs(segs) - 1;
            segs &= segs - 1;
            const uint32_t sb = __shfl_sync(0xffffffffu, b0, sgi), sn = __shfl_sync(0xffffffffu, nc, sgi);
            for (uint32_t i = 0; i < sn; i += 32) {
                if (fill > (uint32_t)stage - 32) {
                    testTile(fill);
                    fill = 0;
                }
                const uint32_t t = i + lane;
                bool keep = false;
                float4 a;
                if (t < sn) {
                    a = __ldg(&g.rec[2 * ((int64_t)sb + t)]);
                    const float ex = fmaxf(fmaxf(blx - a.x, a.x - bhx), 0.0f);
                    const float ey = fmaxf(fmaxf(bly - a.y, a.y - bhy), 0.0f);
                    const float ez = fmaxf(fmaxf(blz - a.z, a.z - bhz), 0.0f);
                    keep = ex * ex + ey * ey + ez * ez < rc2;
                }
                const unsigned km = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const float4 f = __ldg(&g.rec[2 * ((int64_t)sb + t) + 1]);
                    const f3 nn = unpackNormal(__float_as_uint(a.w));
                    const uint32_t k = fill + __popc(km & lt);
                    if constexpr (kLocal) {
                        const float x = a.x - ccx, y = a.y - ccy, z = a.z - ccz;
                        wA[k] = make_float4(x, y, z, x * x + y * y + z * z);
                        wB[k] = make_float4(f.x, f.y, f.z, nn.x);
                        *reinterpret_cast<float2*>(&wC[k]) = make_float2(nn.y, nn.z);
                    } else {
                        wA[k] = make_float4(a.x, a.y, a.z, nn.x);
                        wB[k] = make_float4(f.x, f.y, f.z, nn.y);
                        *reinterpret_cast<float*>(&wC[k]) = nn.z;
                    }
                }
                fill += __popc(km);
            }
        }
        if (fill) testTile(fill);
#pragma unroll
        for (int j = 0; j < kQ; j++)
            if (active[j]) pending[j] = false;
    }
    const float norm = 1.0f / (kPiF * kPiF * r2);
#pragma unroll
    for (int j = 0; j < kQ; j++) {
        if (!valid[j]) continue;
        const int64_t i = base + (int64_t)kQ * lane + j;
        const float4 w = sq[3 * i + 2];
        const float lx = w.x * sx[j] * norm, ly = w.y * sy[j] * norm, lz = w.z * sz[j] * norm;
        const int64_t px = __float_as_int(sq[3 * i].w);
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
        if (lane == 0) {
            atomicAdd(&work[0], wp);
            atomicAdd(&work[1], wi);
        }
    }
}

}  // namespace

namespace {

// Tiles of kStage photons in static shared memory (64, 128, 256), or of
// `stage` photons in dynamic shared memory (kStage 0). Static tiles let the
// compiler address them as shared memory directly: the same kernel with its
// tiles behind a generic pointer ran 4 % slower.
template <int kStage>
cudaError_t gatherLaunch(const GridDev& g, const float4* sq, const uint32_t* total, int64_t n, float radius, int stage,
                         float* out, bool accumulate, unsigned long long* work, unsigned blocks, cudaStream_t st) {
    const size_t smem = kStage > 0 ? 0 : gatherSmem(stage);
    if (accumulate && work)
        kGatherTiled<true, true, kStage><<<blocks, kTileQ, smem, st>>>(g, sq, total, n, radius, stage, out, work);
    else if (accumulate)
        kGatherTiled<true, false, kStage><<<blocks, kTileQ, smem, st>>>(g, sq, total, n, radius, stage, out, work);
    else if (work)
        kGatherTiled<false, true, kStage><<<blocks, kTileQ, smem, st>>>(g, sq, total, n, radius, stage, out, work);
    else
        kGatherTiled<false, false, kStage><<<blocks, kTileQ, smem, st>>>(g, sq, total, n, radius, stage, out, work);
    return cudaGetLastError();
}

}  // namespace

cudaError_t querySortLayout(QuerySortBufs& qs, int64_t maxQueries) {
    uint32_t size = 1u << 10;
    while ((int64_t)size < 2 * maxQueries && size < (1u << 26)) size <<= 1;
    qs.size = size;
    // sub-cell bits: the most (up to the default) that keep 4096 cell
    // buckets; at least 1
    int bits = 1;
    while (bits < PPPM_GATHER_SUBBITS && (size >> (3 * (bits + 1))) >= 4096u) bits++;
    qs.subBits = bits;
    cudaError_t e;
    if ((e = qs.hist.ensure(((size_t)size + 1) * 4)) != cudaSuccess) return e;
    if ((e = qs.cursor.ensure(((size_t)size + 1) * 4)) != cudaSuccess) return e;
    if ((e = qs.tmp.ensure((size_t)scanTmpWords(size) * 4)) != cudaSuccess) return e;
    if ((e = qs.keys.ensure((size_t)std::max<int64_t>(maxQueries, 1) * 4)) != cudaSuccess) return e;
    return qs.sorted.ensure((size_t)std::max<int64_t>(maxQueries, 1) * 48);
}

cudaError_t querySort(const GridDev& g, QueryView qv, QuerySortBufs& qs, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(qs.hist.p, 0, ((size_t)qs.size + 1) * 4, st)) != cudaSuccess) return e;
    kQueryKeys<<<blocksFor(qv.n, 256), 256, 0, st>>>(qv, g, qs.size - 1, qs.subBits, qs.keys.as<uint32_t>(),
                                                     qs.hist.as<uint32_t>());
    if ((e = exclusiveScan(qs.hist.as<uint32_t>(), qs.size, qs.cursor.as<uint32_t>(), qs.tmp.as<uint32_t>(), st)) !=
        cudaSuccess)
        return e;
    kQueryScatter<<<blocksFor(qv.n, 256), 256, 0, st>>>(qv, qs.keys.as<uint32_t>(), qs.cursor.as<uint32_t>(),
                                                        qs.sorted.as<float4>());
    return cudaGetLastError();
}

cudaError_t launchGatherTiled(const GridDev& g, QueryView qv, QuerySortBufs& qs, float radius, float* out,
                              bool accumulate, unsigned long long* work, cudaStream_t st) {
    const cudaError_t e = querySort(g, qv, qs, st);
    if (e != cudaSuccess) return e;
    return launchGatherSorted(g, qv, qs, radius, out, accumulate, work, st);
}

cudaError_t launchGatherSorted(const GridDev& g, QueryView qv, QuerySortBufs& qs, float radius, float* out,
                               bool accumulate, unsigned long long* work, cudaStream_t st) {
    // the sorted count equals the query count; the tiled kernel reads it
    // from the end of the scanned histogram
    const uint32_t* total = qs.hist.as<uint32_t>() + qs.size;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, (qv.n + kTileQ * kQ - 1) / (kTileQ * kQ));
    const float4* sq = qs.sorted.as<float4>();
    switch (qs.stage) {
        case 64: return gatherLaunch<64>(g, sq, total, qv.n, radius, 64, out, accumulate, work, blocks, st);
        case 128: return gatherLaunch<128>(g, sq, total, qv.n, radius, 128, out, accumulate, work, blocks, st);
        case 256: return gatherLaunch<256>(g, sq, total, qv.n, radius, 256, out, accumulate, work, blocks, st);
        default: return gatherLaunch<0>(g, sq, total, qv.n, radius, qs.stage, out, accumulate, work, blocks, st);
    }
}

}  // namespace pppm
