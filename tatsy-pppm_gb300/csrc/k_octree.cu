// Octree of the subsurface irradiance points on the GPU: the tree of
// SubsurfaceIntegrator::Octree::constructRec (subsurface_integrator.cc:
// 83-145), node for node, with the aggregates formed by the same double
// operations in the same order, written in preorder with skip links for the
// stackless walk of octreeSum.
//
// The build is level-synchronous. Level l holds the nodes of depth l with at
// least two points; a node of up to kWarpMax points is split by one warp,
// a larger one by blocks over chunks of kChunk points (box and octant counts
// per chunk, a scan over the node's chunks, a stable scatter per chunk):
//   1. the node's box: min / max over its points (the reference's tight
//      child box, BBox::merge over the child's points);
//   2. the split point mid = (min + max) * 0.5 and each point's octant
//      (x < mid.x ? 0 : 4) + (y < mid.y ? 0 : 2) + (z < mid.z ? 0 : 1);
//   3. a stable 8-way partition of the node's range of the permutation
//      (ballot ranks; the reference pushes points into its child vectors in
//      order, which keeps their relative order);
//   4. one child node per non-empty octant; children with one point are
//      leaves (their point is read back from the permutation when the
//      aggregates are formed), the others join the next level's lists.
// A node's points stay a contiguous range of the permutation, which the
// levels pass between two buffers. Aggregation runs bottom-up one level at a
// time (children before parents), subtree sizes with it; the preorder index
// of every node follows top-down (parent + 1 + sizes of the earlier
// siblings), and one kernel writes the nodes at their preorder slots.
#include <algorithm>
#include <cstring>

#include "context.h"
#include "dipole.cuh"

namespace pppm {

namespace {

constexpr int kSplitBlocks = 152 * 4;
constexpr int kWarpMax = 256;  // larger nodes take the chunked path
constexpr int kChunk = 1024;   // points per chunk
constexpr int kLevelsPerSync = 4;
// Distinct float coordinates separate within ~300 halvings of the box; the
// cap only stops a build that could not end.
constexpr int kMaxOctLevels = 1024;

struct OctBNode {
    int lo, hi;    // range of the permutation
    int pt;        // leaf: point index, or -3: the point at `lo` of the
                   // permutation of depth `depth`; -1 internal; -2 repeated points
    int depth;
    int child[8];  // octant order, -1 empty
    double bmin[3], bmax[3];
    int firstChunk, numChunks;  // chunked nodes: their entries of the level's chunk list
};

struct OctBAcc {
    double pos[3], irad[3], area;
    int size;  // nodes in the subtree
    int pre;   // preorder index
};

struct OctBCtr {
    unsigned nodeCount;
    unsigned active[3];  // rotating lengths of the warp-split lists
    unsigned big[3];     // rotating lengths of the chunked-node lists
    unsigned chunks[3];  // rotating lengths of the chunk lists
    unsigned overflow;
    unsigned degenerate;
};

struct OctBView {
    const float* pos;
    int posStride;
    const float* irad;
    int iradStride;
    const float* area;  // per point, or null: areaConst
    int areaStride;
    double areaConst;
    int n;
    int cap;
    int* idx;       // 2 x n: permutation buffers
    int* active;    // 3 x n: warp-split lists
    int* big;       // 3 x listCap: chunked-node lists
    int2* chunks;   // 3 x listCap: (node, chunk index in the node)
    int listCap;
    unsigned long long* box;  // 6 per node: ordered bits of a chunked node's box (min xyz, max xyz)
    int* chunkCnt;            // 8 per chunk of the level: octant counts, then scatter bases
    OctBNode* nodes;
    OctBAcc* acc;
    OctBCtr* ctr;
};

__device__ __forceinline__ void pointPos(const OctBView& v, int i, double p[3]) {
    const float* q = v.pos + (size_t)i * v.posStride;
    p[0] = (double)q[0];
    p[1] = (double)q[1];
    p[2] = (double)q[2];
}

__device__ __forceinline__ int octant(const double p[3], const double mid[3]) {
    return (p[0] < mid[0] ? 0 : 4) + (p[1] < mid[1] ? 0 : 2) + (p[2] < mid[2] ? 0 : 1);
}

// doubles as unsigned keys with the same order (atomic min / max)
__device__ __forceinline__ unsigned long long orderedBits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double fromOrdered(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// A new node of depth d with range [lo, lo + cnt): a leaf, a warp-split
// node or a chunked node (lists of depth d, slot d % 3).
__device__ int newNode(const OctBView& v, int d, int lo, int cnt) {
    const int id = (int)atomicAdd(&v.ctr->nodeCount, 1u);
    if (id >= v.cap) {
        atomicExch(&v.ctr->overflow, 1u);
        return -1;
    }
    OctBNode& ch = v.nodes[id];
    ch.lo = lo;
    ch.hi = lo + cnt;
    ch.pt = cnt == 1 ? -3 : -1;
    ch.depth = d;
    for (int c = 0; c < 8; c++) ch.child[c] = -1;
    ch.firstChunk = 0;
    ch.numChunks = 0;
    const int q = d % 3;
    if (cnt >= 2 && cnt <= kWarpMax) {
        const unsigned s = atomicAdd(&v.ctr->active[q], 1u);
        v.active[(size_t)q * v.n + s] = id;
    } else if (cnt > kWarpMax) {
        const int nc = (cnt + kChunk - 1) / kChunk;
        const unsigned s = atomicAdd(&v.ctr->big[q], 1u);
        const unsigned f = atomicAdd(&v.ctr->chunks[q], (unsigned)nc);
        if ((int)s >= v.listCap || (int)(f + nc) > v.listCap) {
            atomicExch(&v.ctr->overflow, 1u);
            return id;
        }
        v.big[(size_t)q * v.listCap + s] = id;
        for (int j = 0; j < nc; j++) v.chunks[(size_t)q * v.listCap + f + j] = make_int2(id, j);
        ch.firstChunk = (int)f;
        ch.numChunks = nc;
        unsigned long long* bx = v.box + (size_t)id * 6;
        for (int e = 0; e < 3; e++) {
            bx[e] = ~0ull;
            bx[3 + e] = 0ull;
        }
    }
    return id;
}

__device__ __forceinline__ void chunkMid(const OctBView& v, int node, double mid[3]) {
    const unsigned long long* bx = v.box + (size_t)node * 6;
    for (int e = 0; e < 3; e++) mid[e] = __dmul_rn(__dadd_rn(fromOrdered(bx[e]), fromOrdered(bx[3 + e])), 0.5);
}

__global__ void kOctInit(OctBView v) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < v.n; k += gridDim.x * blockDim.x) v.idx[k] = k;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int q = 0; q < 3; q++) v.ctr->active[q] = v.ctr->big[q] = v.ctr->chunks[q] = 0;
        v.ctr->nodeCount = 0;
        v.ctr->overflow = 0;
        v.ctr->degenerate = 0;
        newNode(v, 0, 0, v.n);
    }
}

// Chunked path, step 1: the node's box (ordered-bit atomics per block).
__global__ void __launch_bounds__(256) kChunkBox(OctBView v, int level) {
    const int q = level % 3;
    const unsigned nc = v.ctr->chunks[q];
    const int* in = v.idx + (size_t)(level & 1) * v.n;
    __shared__ unsigned long long sBox[6];
    for (unsigned e = blockIdx.x; e < nc; e += gridDim.x) {
        const int2 ch = v.chunks[(size_t)q * v.listCap + e];
        const OctBNode& nd = v.nodes[ch.x];
        const int lo = nd.lo + ch.y * kChunk, hi = min(nd.hi, lo + kChunk);
        if (threadIdx.x < 6) sBox[threadIdx.x] = threadIdx.x < 3 ? ~0ull : 0ull;
        __syncthreads();
        unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
        for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
            double p[3];
            pointPos(v, in[k], p);
            for (int d = 0; d < 3; d++) {
                const unsigned long long b = orderedBits(p[d]);
                mn[d] = min(mn[d], b);
                mx[d] = max(mx[d], b);
            }
        }
        for (int o = 16; o > 0; o >>= 1)
            for (int d = 0; d < 3; d++) {
                mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
                mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
            }
        if ((threadIdx.x & 31) == 0)
            for (int d = 0; d < 3; d++) {
                atomicMin(&sBox[d], mn[d]);
                atomicMax(&sBox[3 + d], mx[d]);
            }
        __syncthreads();
        if (threadIdx.x < 3) atomicMin(&v.box[(size_t)ch.x * 6 + threadIdx.x], sBox[threadIdx.x]);
        else if (threadIdx.x < 6) atomicMax(&v.box[(size_t)ch.x * 6 + threadIdx.x], sBox[threadIdx.x]);
        __syncthreads();
    }
}

// Chunked path, step 2: octant counts per chunk.
__global__ void __launch_bounds__(256) kChunkCount(OctBView v, int level) {
    const int q = level % 3;
    const unsigned nc = v.ctr->chunks[q];
    const int* in = v.idx + (size_t)(level & 1) * v.n;
    __shared__ int sCnt[8];
    for (unsigned e = blockIdx.x; e < nc; e += gridDim.x) {
        const int2 ch = v.chunks[(size_t)q * v.listCap + e];
        const OctBNode& nd = v.nodes[ch.x];
        const int lo = nd.lo + ch.y * kChunk, hi = min(nd.hi, lo + kChunk);
        double mid[3];
        chunkMid(v, ch.x, mid);
        if (threadIdx.x < 8) sCnt[threadIdx.x] = 0;
        __syncthreads();
        for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
            double p[3];
            pointPos(v, in[k], p);
            atomicAdd(&sCnt[octant(p, mid)], 1);
        }
        __syncthreads();
        if (threadIdx.x < 8) v.chunkCnt[(size_t)e * 8 + threadIdx.x] = sCnt[threadIdx.x];
        __syncthreads();
    }
}

// Chunked path, step 3: one warp per node: the node's box, the scan of its
// chunks' counts into scatter bases, and its children.
__global__ void kChunkScan(OctBView v, int level) {
    const int q = level % 3;
    const unsigned nb = v.ctr->big[q];
    const int lane = threadIdx.x & 31;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned a = warp; a < nb; a += nwarps) {
        const int id = v.big[(size_t)q * v.listCap + a];
        OctBNode& nd = v.nodes[id];
        const unsigned long long* bx = v.box + (size_t)id * 6;
        if (lane < 3) {
            nd.bmin[lane] = fromOrdered(bx[lane]);
            nd.bmax[lane] = fromOrdered(bx[3 + lane]);
        }
        if (bx[0] == bx[3] && bx[1] == bx[4] && bx[2] == bx[5]) {
            // repeated points: the reference's recursion does not end
            if (lane == 0) {
                nd.pt = -2;
                atomicExch(&v.ctr->degenerate, 1u);
            }
            continue;
        }
        // lane c < 8: running count of octant c over the chunks in order
        int run = 0;
        for (int j = 0; j < nd.numChunks; j++) {
            int* cc = v.chunkCnt + (size_t)(nd.firstChunk + j) * 8;
            if (lane < 8) {
                const int t = cc[lane];
                cc[lane] = run;  // base within the octant; the octant's start is added below
                run += t;
            }
        }
        int incl = lane < 8 ? run : 0;
        for (int off = 1; off < 8; off <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
        }
        const int start = nd.lo + incl - run;
        for (int j = 0; j < nd.numChunks; j++)
            if (lane < 8) v.chunkCnt[(size_t)(nd.firstChunk + j) * 8 + lane] += start;
        int child = -1;
        if (lane < 8 && run > 0) child = newNode(v, level + 1, start, run);
        if (lane < 8) nd.child[lane] = child;
    }
}

// Chunked path, step 4: stable scatter of each chunk (rounds of 256 points
// in order; ballot ranks within warps, warp offsets through shared memory).
__global__ void __launch_bounds__(256) kChunkScatter(OctBView v, int level) {
    const int q = level % 3;
    const unsigned nc = v.ctr->chunks[q];
    const int* in = v.idx + (size_t)(level & 1) * v.n;
    int* out = v.idx + (size_t)((level + 1) & 1) * v.n;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned ltMask = (1u << lane) - 1u;
    __shared__ int sWarp[8][8];  // [warp][octant] counts of a round
    __shared__ int sOff[8][8];   // [warp][octant] destinations of a round
    __shared__ int sRun[8];
    for (unsigned e = blockIdx.x; e < nc; e += gridDim.x) {
        const int2 ch = v.chunks[(size_t)q * v.listCap + e];
        const OctBNode& nd = v.nodes[ch.x];
        const int lo = nd.lo + ch.y * kChunk, hi = min(nd.hi, lo + kChunk);
        double mid[3];
        chunkMid(v, ch.x, mid);
        if (threadIdx.x < 8) sRun[threadIdx.x] = v.chunkCnt[(size_t)e * 8 + threadIdx.x];
        for (int base = lo; base < hi; base += blockDim.x) {
            const int k = base + threadIdx.x;
            int o = 8, src = 0;
            if (k < hi) {
                src = in[k];
                double p[3];
                pointPos(v, src, p);
                o = octant(p, mid);
            }
            int rank = 0;
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const unsigned m = __ballot_sync(0xffffffffu, o == c);
                if (o == c) rank = __popc(m & ltMask);
                if (lane == c) sWarp[w][c] = __popc(m);
            }
            __syncthreads();
            if (threadIdx.x < 64) {
                const int c = threadIdx.x & 7, ww = threadIdx.x >> 3;
                int off = sRun[c];
                for (int x = 0; x < ww; x++) off += sWarp[x][c];
                sOff[ww][c] = off;
            }
            __syncthreads();
            if (k < hi) out[sOff[w][o] + rank] = src;
            if (threadIdx.x < 8) {
                int t = 0;
                for (int x = 0; x < 8; x++) t += sWarp[x][threadIdx.x];
                sRun[threadIdx.x] += t;
            }
            __syncthreads();
        }
    }
}

// One level of warp-split nodes (at most kWarpMax points each). The last
// kernel of a level: it also empties the lists of depth level + 2.
__global__ void __launch_bounds__(256) kOctSplit(OctBView v, int level) {
    const int qi = level % 3, qz = (level + 2) % 3;
    const unsigned na = v.ctr->active[qi];
    if (blockIdx.x == 0 && threadIdx.x == 0) v.ctr->active[qz] = v.ctr->big[qz] = v.ctr->chunks[qz] = 0;
    const int lane = threadIdx.x & 31;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const int* in = v.idx + (size_t)(level & 1) * v.n;
    int* out = v.idx + (size_t)((level + 1) & 1) * v.n;
    const unsigned ltMask = (1u << lane) - 1u;
    for (unsigned a = warp; a < na; a += nwarps) {
        const int id = v.active[(size_t)qi * v.n + a];
        OctBNode& nd = v.nodes[id];
        const int lo = nd.lo, hi = nd.hi;
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
        for (int k = lo + lane; k < hi; k += 32) {
            double p[3];
            pointPos(v, in[k], p);
            for (int d = 0; d < 3; d++) {
                mn[d] = p[d] < mn[d] ? p[d] : mn[d];
                mx[d] = p[d] > mx[d] ? p[d] : mx[d];
            }
        }
        for (int o = 16; o > 0; o >>= 1)
            for (int d = 0; d < 3; d++) {
                const double a0 = __shfl_xor_sync(0xffffffffu, mn[d], o);
                const double a1 = __shfl_xor_sync(0xffffffffu, mx[d], o);
                mn[d] = a0 < mn[d] ? a0 : mn[d];
                mx[d] = a1 > mx[d] ? a1 : mx[d];
            }
        if (lane == 0)
            for (int d = 0; d < 3; d++) {
                nd.bmin[d] = mn[d];
                nd.bmax[d] = mx[d];
            }
        if (mn[0] == mx[0] && mn[1] == mx[1] && mn[2] == mx[2]) {
            if (lane == 0) {
                nd.pt = -2;
                atomicExch(&v.ctr->degenerate, 1u);
            }
            continue;
        }
        double mid[3];
        for (int d = 0; d < 3; d++) mid[d] = __dmul_rn(__dadd_rn(mn[d], mx[d]), 0.5);
        // lane c < 8 counts octant c
        int cnt = 0;
        for (int base = lo; base < hi; base += 32) {
            const int k = base + lane;
            int o = 8;
            if (k < hi) {
                double p[3];
                pointPos(v, in[k], p);
                o = octant(p, mid);
            }
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const unsigned m = __ballot_sync(0xffffffffu, o == c);
                if (lane == c) cnt += __popc(m);
            }
        }
        int incl = cnt;
        for (int off = 1; off < 8; off <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
        }
        const int start = lo + incl - cnt;
        int run = start;
        for (int base = lo; base < hi; base += 32) {
            const int k = base + lane;
            int o = 8, src = 0, dst = 0;
            if (k < hi) {
                src = in[k];
                double p[3];
                pointPos(v, src, p);
                o = octant(p, mid);
            }
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const unsigned m = __ballot_sync(0xffffffffu, o == c);
                const int rc = __shfl_sync(0xffffffffu, run, c);
                if (o == c) dst = rc + __popc(m & ltMask);
                if (lane == c) run += __popc(m);
            }
            if (k < hi) out[dst] = src;
        }
        int child = -1;
        if (lane < 8 && cnt > 0) child = newNode(v, level + 1, start, cnt);
        if (lane < 8) nd.child[lane] = child;
    }
}

// Aggregates of the nodes of depth d (children done): constructRec's
// accumulation (subsurface_integrator.cc:123-144) with the luminance weight
// 0.2126 r + 0.7152 g + 0.0722 b.
__global__ void kOctAggregate(OctBView v, int d) {
    const int nn = min((int)v.ctr->nodeCount, v.cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        OctBNode& nd = v.nodes[i];
        if (nd.depth != d) continue;
        OctBAcc a;
        for (int k = 0; k < 3; k++) a.pos[k] = a.irad[k] = 0.0;
        a.area = 0.0;
        a.size = 1;
        a.pre = 0;
        if (nd.pt == -3) nd.pt = v.idx[(size_t)(nd.depth & 1) * v.n + nd.lo];
        if (nd.pt >= 0) {
            double p[3];
            pointPos(v, nd.pt, p);
            const float* ir = v.irad + (size_t)nd.pt * v.iradStride;
            for (int k = 0; k < 3; k++) {
                a.pos[k] = p[k];
                a.irad[k] = (double)ir[k];
                nd.bmin[k] = nd.bmax[k] = p[k];
            }
            a.area = v.area ? (double)v.area[(size_t)nd.pt * v.areaStride] : v.areaConst;
        } else if (nd.pt == -1) {
            double weight = 0.0;
            int count = 0;
            for (int c = 0; c < 8; c++) {
                const int ch = nd.child[c];
                if (ch < 0) continue;
                const OctBAcc& k = v.acc[ch];
                const double w = __dadd_rn(__dadd_rn(__dmul_rn(k.irad[0], 0.2126), __dmul_rn(k.irad[1], 0.7152)),
                                           __dmul_rn(k.irad[2], 0.0722));
                for (int e = 0; e < 3; e++) {
                    a.pos[e] = __dadd_rn(a.pos[e], __dmul_rn(k.pos[e], w));
                    a.irad[e] = __dadd_rn(a.irad[e], k.irad[e]);
                }
                a.area = __dadd_rn(a.area, k.area);
                weight = __dadd_rn(weight, w);
                count += 1;
                a.size += k.size;
            }
            // Vector3D's division by a scalar multiplies by its reciprocal
            if (weight > 0.0) {
                const double inv = __ddiv_rn(1.0, weight);
                for (int e = 0; e < 3; e++) a.pos[e] = __dmul_rn(a.pos[e], inv);
            }
            if (count != 0) {
                const double inv = __ddiv_rn(1.0, (double)count);
                for (int e = 0; e < 3; e++) a.irad[e] = __dmul_rn(a.irad[e], inv);
            }
        }
        v.acc[i] = a;
    }
}

// Preorder indices of the children of the internal nodes of depth d.
__global__ void kOctPreorder(OctBView v, int d) {
    const int nn = min((int)v.ctr->nodeCount, v.cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const OctBNode& nd = v.nodes[i];
        if (nd.depth != d) continue;
        if (d == 0) v.acc[i].pre = 0;
        if (nd.pt != -1) continue;
        int r = v.acc[i].pre + 1;
        for (int c = 0; c < 8; c++) {
            const int ch = nd.child[c];
            if (ch < 0) continue;
            v.acc[ch].pre = r;
            r += v.acc[ch].size;
        }
    }
}

__global__ void kOctEmit(OctBView v, OctNodeDev* __restrict__ out) {
    const int nn = min((int)v.ctr->nodeCount, v.cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const OctBNode& nd = v.nodes[i];
        const OctBAcc& a = v.acc[i];
        OctNodeDev o;
        o.posArea = make_float4(__double2float_rn(a.pos[0]), __double2float_rn(a.pos[1]), __double2float_rn(a.pos[2]),
                                __double2float_rn(a.area));
        o.iradSkip = make_float4(__double2float_rn(a.irad[0]), __double2float_rn(a.irad[1]),
                                 __double2float_rn(a.irad[2]), __int_as_float(a.pre + a.size));
        o.bminLeaf = make_float4(__double2float_rn(nd.bmin[0]), __double2float_rn(nd.bmin[1]),
                                 __double2float_rn(nd.bmin[2]), __int_as_float(nd.pt != -1 ? 1 : 0));
        o.bmax = make_float4(__double2float_rn(nd.bmax[0]), __double2float_rn(nd.bmax[1]), __double2float_rn(nd.bmax[2]),
                             0.0f);
        out[a.pre] = o;
    }
}

unsigned nodeBlocks(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

}  // namespace

int octreeBuild(pppm_ctx* c, OctreeBufs& b, const OctreePoints& pts, int64_t n, cudaStream_t st, int* numNodes,
                int64_t* launches) {
    *numNodes = 0;
    if (n <= 0) return PPPM_OK;
    if (n > (1 << 28)) return fail(c, PPPM_E_CAPACITY, "octree: too many irradiance points");
    PPPM_CUDA(c, b.hostCtr.ensure(sizeof(OctBCtr)));
    int64_t cap = std::max<int64_t>(b.nodeCap, 2 * n + 1024);
    for (int attempt = 0;; attempt++) {
        const int listCap = (int)(n / 128 + 64);
        PPPM_CUDA(c, b.idx.ensure((size_t)n * 2 * 4));
        PPPM_CUDA(c, b.active.ensure((size_t)n * 3 * 4));
        PPPM_CUDA(c, b.big.ensure((size_t)listCap * 3 * 4));
        PPPM_CUDA(c, b.chunks.ensure((size_t)listCap * 3 * 8));
        PPPM_CUDA(c, b.chunkCnt.ensure((size_t)listCap * 8 * 4));
        PPPM_CUDA(c, b.box.ensure((size_t)cap * 6 * 8));
        PPPM_CUDA(c, b.nodes.ensure((size_t)cap * sizeof(OctBNode)));
        PPPM_CUDA(c, b.acc.ensure((size_t)cap * sizeof(OctBAcc)));
        PPPM_CUDA(c, b.ctr.ensure(sizeof(OctBCtr)));
        OctBView v;
        v.pos = pts.pos;
        v.posStride = pts.posStride;
        v.irad = pts.irad;
        v.iradStride = pts.iradStride;
        v.area = pts.area;
        v.areaStride = pts.areaStride;
        v.areaConst = pts.areaConst;
        v.n = (int)n;
        v.cap = (int)cap;
        v.idx = b.idx.as<int>();
        v.active = b.active.as<int>();
        v.big = b.big.as<int>();
        v.chunks = b.chunks.as<int2>();
        v.listCap = listCap;
        v.box = b.box.as<unsigned long long>();
        v.chunkCnt = b.chunkCnt.as<int>();
        v.nodes = b.nodes.as<OctBNode>();
        v.acc = b.acc.as<OctBAcc>();
        v.ctr = b.ctr.as<OctBCtr>();
        OctBCtr* hc = b.hostCtr.as<OctBCtr>();
        kOctInit<<<nodeBlocks(n), 256, 0, st>>>(v);
        PPPM_CUDA(c, cudaGetLastError());
        *launches += 1;
        int levels = 0;
        // Chunked nodes exist only near the top (a child has fewer points
        // than its parent): the chunk kernels run while the last counts read
        // back show chunked nodes at the next level.
        bool chunked = n > kWarpMax;
        for (;;) {
            for (int j = 0; j < kLevelsPerSync; j++) {
                if (chunked) {
                    kChunkBox<<<kSplitBlocks, 256, 0, st>>>(v, levels + j);
                    kChunkCount<<<kSplitBlocks, 256, 0, st>>>(v, levels + j);
                    kChunkScan<<<16, 256, 0, st>>>(v, levels + j);
                    kChunkScatter<<<kSplitBlocks, 256, 0, st>>>(v, levels + j);
                    *launches += 4;
                }
                kOctSplit<<<kSplitBlocks, 256, 0, st>>>(v, levels + j);
                *launches += 1;
            }
            PPPM_CUDA(c, cudaGetLastError());
            levels += kLevelsPerSync;
            PPPM_CUDA(c, cudaMemcpyAsync(hc, v.ctr, sizeof(OctBCtr), cudaMemcpyDeviceToHost, st));
            PPPM_CUDA(c, cudaStreamSynchronize(st));
            const int q = levels % 3;
            if (hc->overflow || hc->degenerate || (hc->active[q] == 0 && hc->big[q] == 0)) break;
            chunked = hc->big[q] > 0;
            if (levels >= kMaxOctLevels) return fail(c, PPPM_E_UNDEFINED, "octree: no end of the subdivision");
        }
        if (hc->degenerate)
            return fail(c, PPPM_E_UNDEFINED,
                        "octree: repeated irradiance points (the reference recursion does not terminate)");
        if (hc->overflow) {
            if (attempt > 2) return fail(c, PPPM_E_CAPACITY, "octree: node capacity");
            cap = (int64_t)hc->nodeCount * 2 + 1024;
            continue;
        }
        b.nodeCap = cap;
        // nodes have depth `levels` at most
        const unsigned nb = nodeBlocks(hc->nodeCount);
        for (int d = levels; d >= 0; d--) kOctAggregate<<<nb, 256, 0, st>>>(v, d);
        for (int d = 0; d <= levels; d++) kOctPreorder<<<nb, 256, 0, st>>>(v, d);
        PPPM_CUDA(c, b.out.ensure((size_t)hc->nodeCount * sizeof(OctNodeDev)));
        kOctEmit<<<nb, 256, 0, st>>>(v, b.out.as<OctNodeDev>());
        PPPM_CUDA(c, cudaGetLastError());
        *launches += 2 * (levels + 1) + 1;
        *numNodes = (int)hc->nodeCount;
        return PPPM_OK;
    }
}

}  // namespace pppm
