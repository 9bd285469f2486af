// Poisson-disc sampling of the BSSRDF surfaces on the GPU with exactly the
// result of the reference's sequential dart throwing (sampler::poissonDisk,
// sampler.cc:36-101).
//
// The reference draws ceil(4A/d^2) candidates per triangle from one XorShift
// stream, pops them from a RandomQueue (a Fisher-Yates order that depends
// only on the candidate count, random_queue.h:66-73) and accepts a candidate
// when no earlier accepted point registered in the candidate's hash bucket
// lies within d (registration covers the buckets of the cells of a +-2d box,
// with the |(int)x| cell folding of hash_grid_detail.h:34-52). The accepted
// set is the greedy maximal independent set, in pop order, of the directed
// conflict relation
//     p -> c  iff  p pops before c, c's bucket is among p's registered
//                  buckets and |p - c|^2 <= d^2,
// so the GPU builds that relation once per pass (CSR) and decides candidates
// in rounds: c is rejected as soon as an earlier conflicting candidate is
// accepted and accepted once all of them are rejected. Every round decides at
// least the earliest undecided candidate, and the fixed point is the
// sequential result. All double arithmetic uses explicitly rounded
// intrinsics so no contraction changes a bit of the reference's values.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "context.h"
#include "grid.cuh"
#include "kernels.h"
#include "trace.h"

namespace pppm {

namespace {

constexpr int kCandRun = 32;  // candidates generated sequentially per thread

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

unsigned gridFor(int64_t n, int bs, int cap = 152 * 32) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + bs - 1) / bs, cap));
}

// Per BSSRDF triangle: candidate count ceil(4 A / d^2) with Triangle::area
// (0.5 |(p1 - p0) x (p2 - p1)|, triangle.cc:80-84) and the unit normal
// (p1 - p0) x (p2 - p0) / (|.| + EPS) (triangle.cc:45-47, vector3d.cc:63-65).
__global__ void kTriPrep(const float* __restrict__ tri, int64_t ntri, double dd, uint32_t* __restrict__ nSample,
                         float* __restrict__ nrm) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ntri; i += (int64_t)gridDim.x * blockDim.x) {
        const float* p = tri + 9 * i;
        const double p0x = p[0], p0y = p[1], p0z = p[2], p1x = p[3], p1y = p[4], p1z = p[5];
        const double p2x = p[6], p2y = p[7], p2z = p[8];
        {
            const double ax = dsub(p1x, p0x), ay = dsub(p1y, p0y), az = dsub(p1z, p0z);
            const double bx = dsub(p2x, p1x), by = dsub(p2y, p1y), bz = dsub(p2z, p1z);
            const double cx = dsub(dmul(ay, bz), dmul(az, by));
            const double cy = dsub(dmul(az, bx), dmul(ax, bz));
            const double cz = dsub(dmul(ax, by), dmul(ay, bx));
            const double A = dmul(0.5, __dsqrt_rn(dadd(dadd(dmul(cx, cx), dmul(cy, cy)), dmul(cz, cz))));
            nSample[i] = (uint32_t)ceil(__ddiv_rn(dmul(4.0, A), dd));
        }
        {
            const double ax = dsub(p1x, p0x), ay = dsub(p1y, p0y), az = dsub(p1z, p0z);
            const double bx = dsub(p2x, p0x), by = dsub(p2y, p0y), bz = dsub(p2z, p0z);
            const double cx = dsub(dmul(ay, bz), dmul(az, by));
            const double cy = dsub(dmul(az, bx), dmul(ax, bz));
            const double cz = dsub(dmul(ax, by), dmul(ay, bx));
            const double len = __dsqrt_rn(dadd(dadd(dmul(cx, cx), dmul(cy, cy)), dmul(cz, cz)));
            const double inv = __drcp_rn(dadd(len, 1e-12));
            nrm[3 * i] = (float)dmul(cx, inv);
            nrm[3 * i + 1] = (float)dmul(cy, inv);
            nrm[3 * i + 2] = (float)dmul(cz, inv);
        }
    }
}

// Candidates j = offs[t] .. offs[t+1]-1 of triangle t use draws 2j, 2j+1 of
// the sampler stream: u, v; reflected when u + v >= 1; p0 + u e1 + v e2.
__global__ void kCandidates(const float* __restrict__ tri, const uint32_t* __restrict__ offs, int64_t ntri, int64_t n,
                            const uint32_t* __restrict__ jump, uint4 s0, double* __restrict__ pos,
                            float4* __restrict__ rec, int* __restrict__ triOf) {
    const int64_t runs = (n + kCandRun - 1) / kCandRun;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < runs; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t first = r * kCandRun;
        uint32_t st[4] = {s0.x, s0.y, s0.z, s0.w};
        uint64_t k = 2ull * (uint64_t)first;
        for (int lvl = 0; k; lvl++, k >>= 1)
            if (k & 1) jumpApply(jump + (size_t)lvl * 512, st);
        XorShift x;
        x.s[0] = st[0]; x.s[1] = st[1]; x.s[2] = st[2]; x.s[3] = st[3];
        // triangle of the first candidate: last t with offs[t] <= first
        int64_t lo = 0, hi = ntri;
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if ((int64_t)offs[mid] <= first) lo = mid; else hi = mid;
        }
        int64_t t = lo;
        const int64_t end = min(first + kCandRun, n);
        for (int64_t j = first; j < end; j++) {
            while ((int64_t)offs[t + 1] <= j) t++;
            double u = u32ToReal(x.next());
            double v = u32ToReal(x.next());
            if (dadd(u, v) >= 1.0) {
                u = dsub(1.0, u);
                v = dsub(1.0, v);
            }
            const float* p = tri + 9 * t;
            const double p0[3] = {p[0], p[1], p[2]}, p1[3] = {p[3], p[4], p[5]}, p2[3] = {p[6], p[7], p[8]};
            double q[3];
#pragma unroll
            for (int d = 0; d < 3; d++) q[d] = dadd(dadd(p0[d], dmul(u, dsub(p1[d], p0[d]))), dmul(v, dsub(p2[d], p0[d])));
            pos[3 * j] = q[0];
            pos[3 * j + 1] = q[1];
            pos[3 * j + 2] = q[2];
            rec[2 * j] = make_float4((float)q[0], (float)q[1], (float)q[2], 0.0f);
            rec[2 * j + 1] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float((int)j));
            triOf[j] = (int)t;
        }
    }
}

__global__ void kBboxPartial(const double* __restrict__ pos, int64_t n, double* __restrict__ part) {
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < 3; d++) {
            const double v = pos[3 * i + d];
            mn[d] = fmin(mn[d], v);
            mx[d] = fmax(mx[d], v);
        }
    __shared__ double s[6][256];
    for (int d = 0; d < 3; d++) { s[d][threadIdx.x] = mn[d]; s[3 + d][threadIdx.x] = mx[d]; }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < 3; d++) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + w]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 6; d++) part[6 * blockIdx.x + d] = s[d][0];
}

// one block of 256 threads over the partial boxes
__global__ void kBboxFinal(const double* __restrict__ part, int nb, double* __restrict__ out) {
    double r[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int d = 0; d < 3; d++) {
            r[d] = fmin(r[d], part[6 * b + d]);
            r[3 + d] = fmax(r[3 + d], part[6 * b + 3 + d]);
        }
    for (int o = 16; o > 0; o >>= 1)
        for (int d = 0; d < 3; d++) {
            r[d] = fmin(r[d], __shfl_xor_sync(0xffffffffu, r[d], o));
            r[3 + d] = fmax(r[3 + d], __shfl_xor_sync(0xffffffffu, r[3 + d], o));
        }
    __shared__ double s[8][6];
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 6; d++) s[threadIdx.x >> 5][d] = r[d];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        double v = s[0][d];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = d < 3 ? fmin(v, s[w][d]) : fmax(v, s[w][d]);
        out[d] = v;
    }
}

// HashGrid<int> on the candidates (hash_grid_detail.h): the bucket a
// candidate reads (operator[]) and the cell ranges it registers into when
// accepted (add with a +-2d box), both with |(int)x| per axis.
__global__ void kCellInfo(const double* __restrict__ pos, int64_t n, const double* __restrict__ bbox, double scale,
                          double margin, uint32_t hsize, uint32_t* __restrict__ own, int* __restrict__ box) {
    const double bx = bbox[0], by = bbox[1], bz = bbox[2];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        const double o[3] = {bx, by, bz};
        int c[3], lo[3], hi[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            c[d] = abs(__double2int_rz(dmul(dsub(v[d], o[d]), scale)));
            lo[d] = abs(__double2int_rz(dmul(dsub(dsub(v[d], margin), o[d]), scale)));
            hi[d] = abs(__double2int_rz(dmul(dsub(dadd(v[d], margin), o[d]), scale)));
        }
        own[i] = refHash(c[0], c[1], c[2], hsize);
        int* b = box + 6 * i;
        b[0] = lo[0]; b[1] = hi[0]; b[2] = lo[1]; b[3] = hi[1]; b[4] = lo[2]; b[5] = hi[2];
    }
}

__device__ __forceinline__ bool registersInto(const int* __restrict__ b, uint32_t h, uint32_t hsize) {
    for (int iz = b[4]; iz <= b[5]; iz++)
        for (int iy = b[2]; iy <= b[3]; iy++)
            for (int ix = b[0]; ix <= b[1]; ix++)
                if (refHash(ix, iy, iz, hsize) == h) return true;
    return false;
}

// Earlier candidates that block candidate c. kMode 0 counts them into
// cnt[c]; 1 writes them at cnt[c] (exclusive offsets); 2 (one pass) writes
// the first kConflictSlots of them at list[c * kConflictSlots], their count
// into cnt[c] and the largest count into *maxCount.
constexpr int kConflictSlots = 16;

template <int kMode>
__global__ void kConflicts(GridDev g, const double* __restrict__ pos, const uint32_t* __restrict__ own,
                           const int* __restrict__ box, const int* __restrict__ rank, int64_t n, uint32_t hsize,
                           double dd, float reach, uint32_t* __restrict__ cnt, int* __restrict__ list,
                           unsigned* __restrict__ maxCount) {
    constexpr bool kFill = kMode == 1;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const double cx = pos[3 * c], cy = pos[3 * c + 1], cz = pos[3 * c + 2];
        const float fx = (float)cx, fy = (float)cy, fz = (float)cz;
        const int rc = rank[c];
        const uint32_t hc = own[c];
        const int gx = cellCoord(fx, g.ox, g.invCell, g.nx), gy = cellCoord(fy, g.oy, g.invCell, g.ny),
                  gz = cellCoord(fz, g.oz, g.invCell, g.nz);
        uint32_t k = 0;
        const uint32_t base = kFill ? cnt[c] : (kMode == 2 ? (uint32_t)c * kConflictSlots : 0u);
        for (int dz = -1; dz <= 1; dz++) {
            const int zz = gz + dz;
            if (zz < 0 || zz >= g.nz) continue;
            for (int dy = -1; dy <= 1; dy++) {
                const int yy = gy + dy;
                if (yy < 0 || yy >= g.ny) continue;
                for (int dx = -1; dx <= 1; dx++) {
                    const int xx = gx + dx;
                    if (xx < 0 || xx >= g.nx) continue;
                    const uint32_t bkt = bucketOf(xx, yy, zz, g.mask);
                    const uint32_t s = g.start[bkt], e = g.start[bkt + 1];
                    for (uint32_t j = s; j < e; j++) {
                        const float4 a = g.rec[2 * (size_t)j];
                        // photons of other cells hashed to this bucket: keep only this cell's
                        if (cellCoord(a.x, g.ox, g.invCell, g.nx) != xx || cellCoord(a.y, g.oy, g.invCell, g.ny) != yy ||
                            cellCoord(a.z, g.oz, g.invCell, g.nz) != zz)
                            continue;
                        const float ex = a.x - fx, ey = a.y - fy, ez = a.z - fz;
                        if (ex * ex + ey * ey + ez * ez > reach * reach) continue;
                        const int p = __float_as_int(g.rec[2 * (size_t)j + 1].w);
                        if (p == (int)c || rank[p] > rc) continue;
                        // (candPoints[k] - v).squaredNorm() <= minDist * minDist (sampler.cc:81)
                        const double qx = dsub(pos[3 * (size_t)p], cx), qy = dsub(pos[3 * (size_t)p + 1], cy),
                                     qz = dsub(pos[3 * (size_t)p + 2], cz);
                        const double q2 = dadd(dadd(dmul(qx, qx), dmul(qy, qy)), dmul(qz, qz));
                        if (!(q2 <= dd)) continue;
                        if (!registersInto(box + 6 * (size_t)p, hc, hsize)) continue;
                        if (kFill || (kMode == 2 && k < kConflictSlots)) list[base + k] = p;
                        k++;
                    }
                }
            }
        }
        if (!kFill) cnt[c] = k;
        if (kMode == 2 && k > kConflictSlots) atomicMax(maxCount, k);
    }
}

// One round: state 0 undecided, 1 accepted, 2 rejected. kSlots: the lists
// of kConflicts<2> (conf = counts), else CSR (conf = offsets).
template <bool kSlots>
__global__ void kDecide(const uint32_t* __restrict__ conf, const int* __restrict__ list, int64_t n,
                        uint8_t* __restrict__ state, unsigned long long* __restrict__ undecided) {
    unsigned left = 0;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        if (state[c] != 0) continue;
        bool open = false, blocked = false;
        const uint32_t j0 = kSlots ? (uint32_t)c * kConflictSlots : conf[c];
        const uint32_t j1 = kSlots ? j0 + conf[c] : conf[c + 1];
        for (uint32_t j = j0; j < j1; j++) {
            const uint8_t s = ((volatile uint8_t*)state)[list[j]];
            if (s == 1) { blocked = true; break; }
            if (s == 0) open = true;
        }
        if (blocked) state[c] = 2;
        else if (!open) state[c] = 1;
        else left++;
    }
    left = __reduce_add_sync(0xffffffffu, left);
    if ((threadIdx.x & 31) == 0 && left) atomicAdd(undecided, (unsigned long long)left);
}

// flag[k] = 1 when the k-th popped candidate was accepted.
__global__ void kPopFlags(const uint8_t* __restrict__ state, const int* __restrict__ rank, int64_t n,
                          int* __restrict__ byPop, uint32_t* __restrict__ flag) {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int r = rank[c];
        byPop[r] = (int)c;
        flag[r] = state[c] == 1 ? 1u : 0u;
    }
}

// Accepted points in the reference's output order (acceptance = pop order):
// gather queries (pos | index, normal, unit weight) plus float copies.
__global__ void kEmitPoints(const int* __restrict__ byPop, const uint32_t* __restrict__ outIdx, int64_t n,
                            const double* __restrict__ pos, const int* __restrict__ triOf,
                            const float* __restrict__ triNrm, float4* __restrict__ q, float* __restrict__ pts,
                            float* __restrict__ nrm) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        if (outIdx[k + 1] == outIdx[k]) continue;
        const int64_t o = outIdx[k];
        const int c = byPop[k];
        const int t = triOf[c];
        const float px = (float)pos[3 * (size_t)c], py = (float)pos[3 * (size_t)c + 1], pz = (float)pos[3 * (size_t)c + 2];
        const float nx = triNrm[3 * t], ny = triNrm[3 * t + 1], nz = triNrm[3 * t + 2];
        q[3 * o] = make_float4(px, py, pz, __int_as_float((int)o));
        q[3 * o + 1] = make_float4(nx, ny, nz, 0.0f);
        q[3 * o + 2] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        pts[3 * o] = px; pts[3 * o + 1] = py; pts[3 * o + 2] = pz;
        nrm[3 * o] = nx; nrm[3 * o + 1] = ny; nrm[3 * o + 2] = nz;
    }
}

__global__ void kSetU64(uint64_t* p, uint64_t v) { *p = v; }

}  // namespace

// RandomQueue<int> seeded -1 (random_queue.h:20-28,66-73) over n pushes
// 0..n-1: rank[id] = the position at which id is popped.
bool popOrder(int64_t n, std::vector<int>* rank) {
    XorShift q;
    q.seed((uint32_t)-1);
    std::vector<int> que((size_t)n);
    for (int64_t i = 0; i < n; i++) que[i] = (int)i;
    rank->assign((size_t)n, 0);
    int64_t pos = n;
    for (int64_t k = 0; k < n; k++) {
        const uint32_t x = q.next();
        // XorShift::nextInt: abs((int)x) % n; abs(INT_MIN) is undefined and
        // the reference then indexes before its queue
        if (x == 0x80000000u) return false;
        const int r = std::abs((int)x) % (int)pos;
        pos--;
        std::swap(que[r], que[pos]);
        (*rank)[que[pos]] = (int)k;
    }
    return true;
}

int poissonBegin(pppm_ctx* c, PoissonGpu& g, const float* tri9, int64_t ntri, double minDist) {
    g.ready = false;
    g.ntri = ntri;
    g.minDist = minDist;
    g.n = 0;
    if (ntri == 0) {
        g.ready = true;
        return PPPM_OK;
    }
    if (g.jumpHost.empty()) xorshiftJumpTables(&g.jumpHost, 1);
    PPPM_CUDA(c, g.jump.ensure(g.jumpHost.size() * 4));
    PPPM_CUDA(c, cudaMemcpyAsync(g.jump.p, g.jumpHost.data(), g.jumpHost.size() * 4, cudaMemcpyHostToDevice, c->stream));
    PPPM_CUDA(c, g.tri.ensure((size_t)ntri * 36));
    PPPM_CUDA(c, cudaMemcpyAsync(g.tri.p, tri9, (size_t)ntri * 36, cudaMemcpyHostToDevice, c->stream));
    PPPM_CUDA(c, g.offs.ensure((size_t)(ntri + 1) * 4));
    PPPM_CUDA(c, g.triNrm.ensure((size_t)ntri * 12));
    PPPM_CUDA(c, g.scanCursor.ensure((size_t)(ntri + 1) * 4));
    PPPM_CUDA(c, g.scanTmp.ensure((size_t)scanTmpWords(ntri + 1) * 4));
    kTriPrep<<<gridFor(ntri, 256), 256, 0, c->stream>>>(g.tri.as<float>(), ntri, minDist * minDist,
                                                          g.offs.as<uint32_t>(), g.triNrm.as<float>());
    PPPM_CUDA(c, cudaGetLastError());
    PPPM_CUDA(c, exclusiveScan(g.offs.as<uint32_t>(), ntri, g.scanCursor.as<uint32_t>(), g.scanTmp.as<uint32_t>(),
                               c->stream));
    uint32_t total = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&total, g.offs.as<uint32_t>() + ntri, 4, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    g.n = (int64_t)total;
    const int64_t n = g.n;
    // the pop order depends on the candidate count only: once per render
    std::vector<int> rank;
    if (!popOrder(n, &rank))
        return fail(c, PPPM_E_UNDEFINED, "poisson: the candidate queue draws abs(INT_MIN) (undefined in the reference)");
    const size_t m = (size_t)std::max<int64_t>(n, 1);
    PPPM_CUDA(c, g.rank.ensure(m * 4));
    if (n) PPPM_CUDA(c, cudaMemcpy(g.rank.p, rank.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, g.pos.ensure(m * 24));
    PPPM_CUDA(c, g.rec.ensure(m * 32));
    PPPM_CUDA(c, g.triOf.ensure(m * 4));
    PPPM_CUDA(c, g.own.ensure(m * 4));
    PPPM_CUDA(c, g.box.ensure(m * 24));
    PPPM_CUDA(c, g.state.ensure(m));
    PPPM_CUDA(c, g.conf.ensure((m + 1) * 4));
    PPPM_CUDA(c, g.byPop.ensure(m * 4));
    PPPM_CUDA(c, g.flag.ensure((m + 1) * 4));
    PPPM_CUDA(c, g.cursor.ensure((m + 1) * 4));
    PPPM_CUDA(c, g.tmp.ensure((size_t)scanTmpWords((int64_t)m + 1) * 4));
    PPPM_CUDA(c, g.bbox.ensure(6 * 8 + 152 * 4 * 6 * 8));
    PPPM_CUDA(c, g.misc.ensure(64));
    g.ready = true;
    return PPPM_OK;
}

int poissonRun(pppm_ctx* c, PoissonGpu& g, uint32_t rng[4], float4* queries, float* pts, float* nrm, int64_t cap,
               int64_t* count) {
    *count = 0;
    const int64_t n = g.n;
    if (n == 0) return PPPM_OK;
    cudaStream_t st = c->stream;
    const uint4 s0 = make_uint4(rng[0], rng[1], rng[2], rng[3]);
    const int64_t runs = (n + kCandRun - 1) / kCandRun;
    kCandidates<<<gridFor(runs, 128), 128, 0, st>>>(g.tri.as<float>(), g.offs.as<uint32_t>(), g.ntri, n,
                                                     g.jump.as<uint32_t>(), s0, g.pos.as<double>(), g.rec.as<float4>(),
                                                     g.triOf.as<int>());
    // the stream moves on by 2 draws per candidate
    {
        XorShift x;
        std::memcpy(x.s, rng, 16);
        xorshiftJumpHost(g.jumpHost, 2ull * (uint64_t)n, &x);
        std::memcpy(rng, x.s, 16);
    }
    const int nb = 152 * 4;
    double* bbox = g.bbox.as<double>();
    kBboxPartial<<<nb, 256, 0, st>>>(g.pos.as<double>(), n, bbox + 6);
    kBboxFinal<<<1, 256, 0, st>>>(bbox + 6, nb, bbox);
    double hb[6];
    PPPM_CUDA(c, cudaMemcpyAsync(hb, bbox, 48, cudaMemcpyDeviceToHost, st));
    PPPM_CUDA(c, cudaStreamSynchronize(st));
    const double d = g.minDist;
    // HashGrid::init(numPoints, 1 / (2 d), bbox) (sampler.cc:60-66)
    const double scale = 1.0 / (2.0 * d);
    kCellInfo<<<gridFor(n, 256), 256, 0, st>>>(g.pos.as<double>(), n, bbox, scale, 2.0 * d, (uint32_t)n,
                                               g.own.as<uint32_t>(), g.box.as<int>());
    // candidate grid for the neighbour search (float positions, reach d plus a
    // margin far above their rounding)
    const double mn[3] = {hb[0], hb[1], hb[2]}, mx[3] = {hb[3], hb[4], hb[5]};
    const double ext = std::max({mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2], 1e-30});
    const float reach = (float)(d + 1e-5 * ext + 1e-30);
    uint64_t* cntD = reinterpret_cast<uint64_t*>(g.misc.p);
    kSetU64<<<1, 1, 0, st>>>(cntD, (uint64_t)n);
    PPPM_CUDA(c, gridLayout(g.grid, mn, mx, (double)reach * 1.001, n));
    GridDev gv = gridView(g.grid, mn, mx);
    PPPM_CUDA(c, gridBuild(g.grid, gv, g.rec.as<float4>(), cntD, n, st));
    gv = gridView(g.grid, mn, mx);
    uint32_t* conf = g.conf.as<uint32_t>();
    // one pass into fixed slots; a candidate with more conflicts than slots
    // sends the whole set through the counted CSR form (its counts are in conf)
    PPPM_CUDA(c, g.list.ensure((size_t)std::max<int64_t>(n, 1) * kConflictSlots * 4));
    unsigned* maxCount = reinterpret_cast<unsigned*>(g.misc.as<char>() + 16);
    PPPM_CUDA(c, cudaMemsetAsync(maxCount, 0, 4, st));
    kConflicts<2><<<gridFor(n, 128), 128, 0, st>>>(gv, g.pos.as<double>(), g.own.as<uint32_t>(), g.box.as<int>(),
                                                   g.rank.as<int>(), n, (uint32_t)n, d * d, reach, conf,
                                                   g.list.as<int>(), maxCount);
    unsigned over = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&over, maxCount, 4, cudaMemcpyDeviceToHost, st));
    PPPM_CUDA(c, cudaStreamSynchronize(st));
    const bool slots = over == 0;
    if (!slots) {
        PPPM_CUDA(c, exclusiveScan(conf, n, g.cursor.as<uint32_t>(), g.tmp.as<uint32_t>(), st));
        uint32_t links = 0;
        PPPM_CUDA(c, cudaMemcpyAsync(&links, conf + n, 4, cudaMemcpyDeviceToHost, st));
        PPPM_CUDA(c, cudaStreamSynchronize(st));
        PPPM_CUDA(c, g.list.ensure((size_t)std::max<uint32_t>(links, 1) * 4));
        kConflicts<1><<<gridFor(n, 128), 128, 0, st>>>(gv, g.pos.as<double>(), g.own.as<uint32_t>(), g.box.as<int>(),
                                                       g.rank.as<int>(), n, (uint32_t)n, d * d, reach, conf,
                                                       g.list.as<int>(), nullptr);
    }
    PPPM_CUDA(c, cudaMemsetAsync(g.state.p, 0, (size_t)n, st));
    unsigned long long* und = reinterpret_cast<unsigned long long*>(g.misc.as<char>() + 8);
    // each round decides at least the earliest undecided candidate; rounds
    // go in groups of kRoundsPerSync between reads of the undecided count
    // (rounds after the last decision change nothing)
    constexpr int kRoundsPerSync = 4;
    int64_t rounds = 0;
    for (;;) {
        if (rounds > n + 1) return fail(c, PPPM_E_CUDA, "poisson: decision rounds did not converge");
        for (int r = 0; r < kRoundsPerSync; r++) {
            if (r == kRoundsPerSync - 1) PPPM_CUDA(c, cudaMemsetAsync(und, 0, 8, st));
            if (slots)
                kDecide<true><<<gridFor(n, 256), 256, 0, st>>>(conf, g.list.as<int>(), n, g.state.as<uint8_t>(), und);
            else
                kDecide<false><<<gridFor(n, 256), 256, 0, st>>>(conf, g.list.as<int>(), n, g.state.as<uint8_t>(), und);
        }
        rounds += kRoundsPerSync;
        unsigned long long left = 0;
        PPPM_CUDA(c, cudaMemcpyAsync(&left, und, 8, cudaMemcpyDeviceToHost, st));
        PPPM_CUDA(c, cudaStreamSynchronize(st));
        if (left == 0) break;
    }
    g.rounds = rounds;
    uint32_t* flag = g.flag.as<uint32_t>();
    kPopFlags<<<gridFor(n, 256), 256, 0, st>>>(g.state.as<uint8_t>(), g.rank.as<int>(), n, g.byPop.as<int>(), flag);
    PPPM_CUDA(c, exclusiveScan(flag, n, g.cursor.as<uint32_t>(), g.tmp.as<uint32_t>(), st));
    uint32_t m = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&m, flag + n, 4, cudaMemcpyDeviceToHost, st));
    PPPM_CUDA(c, cudaStreamSynchronize(st));
    *count = m;
    if ((int64_t)m > cap) return PPPM_OK;  // caller grows and asks again
    kEmitPoints<<<gridFor(n, 256), 256, 0, st>>>(g.byPop.as<int>(), flag, n, g.pos.as<double>(), g.triOf.as<int>(),
                                                 g.triNrm.as<float>(), queries, pts, nrm);
    PPPM_CUDA(c, cudaGetLastError());
    return PPPM_OK;
}

}  // namespace pppm
