// The compat radiance gather over the photon hash grid (the canonical
// gather is k_gather_tiled.cu).
//
// Compat: the reference's k-nearest search (k = (int)radius, epsilon =
// gatherPhotons, kdtree_detail.h:90-132), its disc filter and its cone filter
// with the flux/distance index mismatch (ppm_probabilistic.cc:300-335).
#include "kernels.h"

namespace pppm {

namespace {

unsigned blocksFor(int64_t n, int bs) {
    const int64_t want = (n + bs - 1) / bs;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, 152 * 32));
}

__device__ __forceinline__ int64_t queryCount(const QueryView& qv) {
    return qv.count ? min((int64_t)*qv.count, qv.n) : qv.n;
}

// Strict order of kNN candidates: squared distance, then (for the rare
// exact FP32 ties) the photon's path id, position, flux and normal bits, so
// that the selected set and its order do not depend on the order in which
// deposits reached the photon map (atomic appends). Ties are not only
// equidistant photons: a path whose next ray starts at its hit point (the
// reference offsets nothing) can hit the same surface again at t ~ 1e-10
// and deposit twice at the same position with another flux. id < 0: a
// phantom record at the origin (all alike), after real photons at the same
// distance.
__device__ __forceinline__ bool knnBefore(float da, int ia, float db, int ib, const float4* __restrict__ rec) {
    if (da != db) return da < db;
    if (ia == ib || (ia < 0 && ib < 0)) return false;
    if (ia < 0 || ib < 0) return ib < 0;
    const uint32_t pa = __float_as_uint(__ldg(&rec[2 * (int64_t)ia + 1]).w);
    const uint32_t pb = __float_as_uint(__ldg(&rec[2 * (int64_t)ib + 1]).w);
    if (pa != pb) return pa < pb;
    const float4 a = __ldg(&rec[2 * (int64_t)ia]), b = __ldg(&rec[2 * (int64_t)ib]);
    const float4 fa = __ldg(&rec[2 * (int64_t)ia + 1]), fb = __ldg(&rec[2 * (int64_t)ib + 1]);
    const uint32_t ka[7] = {__float_as_uint(a.x), __float_as_uint(a.y), __float_as_uint(a.z), __float_as_uint(fa.x),
                            __float_as_uint(fa.y), __float_as_uint(fa.z), __float_as_uint(a.w)};
    const uint32_t kb[7] = {__float_as_uint(b.x), __float_as_uint(b.y), __float_as_uint(b.z), __float_as_uint(fb.x),
                            __float_as_uint(fb.y), __float_as_uint(fb.z), __float_as_uint(b.w)};
    for (int i = 0; i < 7; i++)
        if (ka[i] != kb[i]) return ka[i] < kb[i];
    return false;  // identical records: either order gives the same list
}

// Sorted (ascending, knnBefore) candidate list of the k nearest photons.
struct KnnList {
    float d2[kMaxKnn];
    int idx[kMaxKnn];
    int cnt;
    float kd = 3.4e38f;  // d2[k - 1] once the list is full: most candidates stop at this register
    __device__ __forceinline__ bool insert(float d, int id, int k, const float4* __restrict__ rec) {
        if (d > kd) return false;  // farther than the k-th: cannot enter
        int pos;
        if (cnt < k) {
            pos = cnt++;
        } else if (knnBefore(d, id, d2[k - 1], idx[k - 1], rec)) {
            pos = k - 1;
        } else {
            return false;
        }
        while (pos > 0 && knnBefore(d, id, d2[pos - 1], idx[pos - 1], rec)) {
            d2[pos] = d2[pos - 1];
            idx[pos] = idx[pos - 1];
            pos--;
        }
        d2[pos] = d;
        idx[pos] = id;
        if (cnt == k) kd = d2[k - 1];
        return true;
    }
};

// k nearest photons with distance < eps (the reference's K_NEAREST |
// EPSILON_BALL query), expanding shells of cells around the query cell.
// Each photon is accepted only while its own cell is being scanned, so a
// bucket shared by several cells never yields duplicates. After shell s the
// search stops once the k-th distance is within `cov`, the distance from the
// query to the nearest cell not yet scanned.
__device__ __forceinline__ void knnVisit(const GridDev& g, int cx, int cy, int cz, float qx, float qy, float qz,
                                         float eps2, int k, KnnList& L) {
    const uint32_t key = bucketOf(cx, cy, cz, g.mask);
    // a bucket whose photons all lie in one cell: this cell's (no per-photon
    // test) or another's (nothing to visit)
    bool pure = false;
    if (g.owner) {
        const unsigned long long own = __ldg(&g.owner[key]);
        if (own != kBucketMixed) {
            if (own != cellCode(cx, cy, cz)) return;
            pure = true;
        }
    }
    const uint32_t b0 = __ldg(&g.start[key]), b1 = __ldg(&g.start[key + 1]);
    for (uint32_t j = b0; j < b1; j++) {
        const float4 a = __ldg(&g.rec[2 * (int64_t)j]);
        if (!pure && (cellCoord(a.x, g.ox, g.invCell, g.nx) != cx || cellCoord(a.y, g.oy, g.invCell, g.ny) != cy ||
                      cellCoord(a.z, g.oz, g.invCell, g.nz) != cz))
            continue;
        const float dx = qx - a.x, dy = qy - a.y, dz = qz - a.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < eps2) L.insert(d2, (int)j, k, g.rec);
    }
}

__device__ __forceinline__ float sideGap(float q, float o, float cell, int c0, int s, int n, bool* any) {
    float cov = 3.0e38f;
    if (c0 - s > 0) { cov = fminf(cov, q - (o + (float)(c0 - s) * cell)); *any = true; }
    if (c0 + s < n - 1) { cov = fminf(cov, (o + (float)(c0 + s + 1) * cell) - q); *any = true; }
    return cov;
}

__device__ void knnSearch(const GridDev& g, float qx, float qy, float qz, int k, float eps, int64_t phantoms,
                          KnnList& L) {
    L.cnt = 0;
    L.kd = 3.4e38f;
    const float eps2 = eps * eps;
    const int c0x = cellCoord(qx, g.ox, g.invCell, g.nx);
    const int c0y = cellCoord(qy, g.oy, g.invCell, g.ny);
    const int c0z = cellCoord(qz, g.oz, g.invCell, g.nz);
    // margin for cell boundaries rounded differently from floor((p-o)/cell)
    const float margin = 1e-4f * g.cell + 1e-6f * (fabsf(qx) + fabsf(qy) + fabsf(qz) + fabsf(g.ox) + fabsf(g.oy) + fabsf(g.oz));
    for (int s = 0;; s++) {
        const int lz = max(c0z - s, 0), hz = min(c0z + s, g.nz - 1);
        const int ly = max(c0y - s, 0), hy = min(c0y + s, g.ny - 1);
        const int lx = max(c0x - s, 0), hx = min(c0x + s, g.nx - 1);
        for (int cz = lz; cz <= hz; cz++) {
            const bool zEdge = cz == c0z - s || cz == c0z + s;
            for (int cy = ly; cy <= hy; cy++) {
                const bool yEdge = cy == c0y - s || cy == c0y + s;
                if (zEdge || yEdge) {
                    for (int cx = lx; cx <= hx; cx++) knnVisit(g, cx, cy, cz, qx, qy, qz, eps2, k, L);
                } else {
                    if (c0x - s >= 0) knnVisit(g, c0x - s, cy, cz, qx, qy, qz, eps2, k, L);
                    if (s > 0 && c0x + s < g.nx) knnVisit(g, c0x + s, cy, cz, qx, qy, qz, eps2, k, L);
                }
            }
        }
        bool any = false;
        float cov = sideGap(qx, g.ox, g.cell, c0x, s, g.nx, &any);
        cov = fminf(cov, sideGap(qy, g.oy, g.cell, c0y, s, g.ny, &any));
        cov = fminf(cov, sideGap(qz, g.oz, g.cell, c0z, s, g.nz, &any));
        if (!any) break;  // every cell of the grid has been scanned
        cov -= margin;
        if (cov >= eps) break;
        if (cov > 0.0f && L.cnt == k && L.d2[k - 1] <= cov * cov) break;
    }
    if (phantoms > 0) {
        // default Photon() records at the origin (ppm_probabilistic.cc:202-207)
        const float d2 = qx * qx + qy * qy + qz * qz;
        if (d2 < eps2) {
            const int64_t np = phantoms < k ? phantoms : k;
            for (int64_t t = 0; t < np; t++)
                if (!L.insert(d2, -1, k, g.rec)) break;
        }
    }
}

__global__ void __launch_bounds__(128) kKnn(GridDev g, const float* __restrict__ q, int64_t m, int k, float eps,
                                            int32_t* __restrict__ idxOut, int32_t* __restrict__ cntOut, int cap) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        KnnList L;
        knnSearch(g, q[3 * i], q[3 * i + 1], q[3 * i + 2], k, eps, 0, L);
        cntOut[i] = L.cnt;
        for (int t = 0; t < L.cnt && t < cap; t++) {
            const int j = L.idx[L.cnt - 1 - t];  // farthest first
            idxOut[i * cap + t] = __float_as_int(__ldg(&g.rec[2 * (int64_t)j + 1]).w);
        }
        for (int t = L.cnt; t < cap; t++) idxOut[i * cap + t] = -1;
    }
}

template <bool kAccum>
__global__ void __launch_bounds__(128) kGatherCompat(GridDev g, QueryView qv, int k, float eps, float rlim,
                                                     int64_t phantoms, float* __restrict__ out) {
    const int64_t n = queryCount(qv);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 q0 = qv.q[3 * i], q1 = qv.q[3 * i + 1], q2 = qv.q[3 * i + 2];
        KnnList L;
        knnSearch(g, q0.x, q0.y, q0.z, k, eps, phantoms, L);
        // results in the reference's order: farthest first
        const int m = L.cnt;
        float vd[kMaxKnn];
        int nv = 0;
        float maxd = 0.0f;
        for (int t = 0; t < m; t++) {
            const int j = L.idx[m - 1 - t];
            float px = 0.f, py = 0.f, pz = 0.f;
            if (j >= 0) {
                const float4 a = __ldg(&g.rec[2 * (int64_t)j]);
                px = a.x; py = a.y; pz = a.z;
            }
            const float dx = q0.x - px, dy = q0.y - py, dz = q0.z - pz;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            const float c = fabsf((q1.x * dx + q1.y * dy + q1.z * dz) / dist);
            if (c < rlim) {  // false for dist == 0 (NaN), as in the reference
                vd[nv++] = dist;
                maxd = fmaxf(maxd, dist);
            }
        }
        // cone filter: the j-th valid distance weights the flux of the j-th
        // photon of the unfiltered list (photons[i] at :327)
        float tx = 0.f, ty = 0.f, tz = 0.f;
        for (int t = 0; t < nv; t++) {
            const float w = 1.0f - vd[t] / (1.1f * maxd);
            const int j = L.idx[m - 1 - t];
            if (j >= 0) {
                const float4 b = __ldg(&g.rec[2 * (int64_t)j + 1]);
                tx += w * b.x;
                ty += w * b.y;
                tz += w * b.z;
            }
        }
        float lx = 0.f, ly = 0.f, lz = 0.f;
        if (maxd > 1e-12f) {
            const float s = (1.0f / kPiF) / (1.0f - 2.0f / (3.0f * 1.1f)) / (kPiF * maxd * maxd);
            lx = q2.x * tx * s;
            ly = q2.y * ty * s;
            lz = q2.z * tz * s;
        }
        if (kAccum) {
            const int64_t px = __float_as_int(q0.w);
            out[3 * px] += lx;
            out[3 * px + 1] += ly;
            out[3 * px + 2] += lz;
        } else {
            out[3 * i] = lx;
            out[3 * i + 1] = ly;
            out[3 * i + 2] = lz;
        }
    }
}

__global__ void kPackPhotons(const float* __restrict__ in, int64_t n, float4* __restrict__ rec) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* p = in + 8 * i;
        rec[2 * i] = make_float4(p[0], p[1], p[2], p[6]);
        rec[2 * i + 1] = make_float4(p[3], p[4], p[5], __int_as_float((int)i));
    }
}

__global__ void kPackPositions(const float* __restrict__ in, int64_t n, float4* __restrict__ rec) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        rec[2 * i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.0f);
        rec[2 * i + 1] = make_float4(0.f, 0.f, 0.f, __int_as_float((int)i));
    }
}

__global__ void kPackQueries(const float* __restrict__ in, int64_t m, float4* __restrict__ q) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const float* p = in + 12 * i;
        q[3 * i] = make_float4(p[0], p[1], p[2], __int_as_float((int)i));
        q[3 * i + 1] = make_float4(p[3], p[4], p[5], 0.0f);
        q[3 * i + 2] = make_float4(p[6] * p[9], p[7] * p[10], p[8] * p[11], 0.0f);
    }
}

__global__ void kSetCount(uint64_t* c, int64_t n) { *c = (uint64_t)n; }

}  // namespace

cudaError_t launchGatherCompat(const GridDev& g, QueryView q, int k, float eps, float rlim, int64_t phantoms,
                               float* out, bool accumulate, cudaStream_t st) {
    const int bs = 128;
    if (accumulate) kGatherCompat<true><<<blocksFor(q.n, bs), bs, 0, st>>>(g, q, k, eps, rlim, phantoms, out);
    else kGatherCompat<false><<<blocksFor(q.n, bs), bs, 0, st>>>(g, q, k, eps, rlim, phantoms, out);
    return cudaGetLastError();
}

cudaError_t launchKnn(const GridDev& g, const float* queries, int64_t m, int k, float eps, int32_t* idx, int32_t* cnt,
                      int cap, cudaStream_t st) {
    const int bs = 128;
    kKnn<<<blocksFor(m, bs), bs, 0, st>>>(g, queries, m, k, eps, idx, cnt, cap);
    return cudaGetLastError();
}

cudaError_t launchPackPhotons(const float* in8, int64_t n, float4* rec, uint64_t* count, cudaStream_t st) {
    kPackPhotons<<<blocksFor(n, 256), 256, 0, st>>>(in8, n, rec);
    kSetCount<<<1, 1, 0, st>>>(count, n);
    return cudaGetLastError();
}

cudaError_t launchPackPositions(const float* pos3, int64_t n, float4* rec, uint64_t* count, cudaStream_t st) {
    kPackPositions<<<blocksFor(n, 256), 256, 0, st>>>(pos3, n, rec);
    kSetCount<<<1, 1, 0, st>>>(count, n);
    return cudaGetLastError();
}

cudaError_t launchPackQueries(const float* in12, int64_t m, float4* q, cudaStream_t st) {
    kPackQueries<<<blocksFor(m, 256), 256, 0, st>>>(in12, m, q);
    return cudaGetLastError();
}

}  // namespace pppm

namespace pppm {

namespace {
// Photon records (pos|normal, flux|id) -> 8 floats (pos, flux, normal, id),
// the layout of pppm_gather's photon input.
__global__ void kUnpackRecords(const float4* __restrict__ rec, int64_t n, float* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = rec[2 * i], b = rec[2 * i + 1];
        float* o = out + 8 * i;
        o[0] = a.x; o[1] = a.y; o[2] = a.z;
        o[3] = b.x; o[4] = b.y; o[5] = b.z;
        o[6] = a.w; o[7] = b.w;
    }
}
}  // namespace

cudaError_t launchUnpackRecords(const float4* rec, int64_t n, float* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    kUnpackRecords<<<blocksFor(n, 256), 256, 0, st>>>(rec, n, out);
    return cudaGetLastError();
}

}  // namespace pppm
