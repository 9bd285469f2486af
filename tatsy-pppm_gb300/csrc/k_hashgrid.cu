// HashGrid<T>::init / add / operator[] (hash_grid_detail.h:26-72) on the
// GPU: every item is inserted into the buckets of all cells its box covers,
// and each bucket lists its items in the reference's insertion order (items
// in add order; an item whose cells share a bucket appears once per cell, in
// the z-y-x loop order of add).
//
// Build: per item the number of covered cells, a scan of those counts (the
// global insertion index of every (item, cell) entry), a bucket histogram
// and its scan, an atomic scatter of the entries' insertion indices, then a
// sort of each bucket's short list by insertion index.
#include "kernels.h"

namespace pppm {

namespace {

struct HgGrid {
    double ox, oy, oz;  // bbox.posMin()
    double scale;
    uint32_t size;
};

// |(int)((v - posMin) * scale)| per axis (hash_grid_detail.h:35-45, 66-69):
// Vector3D subtraction then scaling, each rounded in double; (int) truncates.
__device__ __forceinline__ int hgCoord(double v, double o, double scale) {
    return abs(__double2int_rz(__dmul_rn(__dsub_rn(v, o), scale)));
}

__device__ __forceinline__ void hgRange(const HgGrid& g, const double* lo, const double* hi, int* mn, int* mx) {
    mn[0] = hgCoord(lo[0], g.ox, g.scale); mx[0] = hgCoord(hi[0], g.ox, g.scale);
    mn[1] = hgCoord(lo[1], g.oy, g.scale); mx[1] = hgCoord(hi[1], g.oy, g.scale);
    mn[2] = hgCoord(lo[2], g.oz, g.scale); mx[2] = hgCoord(hi[2], g.oz, g.scale);
}

// cells per item (an axis whose minimum folds above its maximum covers none)
__global__ void kHgCount(const double* __restrict__ bmin, const double* __restrict__ bmax, int64_t n, HgGrid g,
                         uint32_t* __restrict__ cnt, unsigned long long* __restrict__ over) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int mn[3], mx[3];
        hgRange(g, bmin + 3 * i, bmax + 3 * i, mn, mx);
        unsigned long long c = 1;
        for (int d = 0; d < 3; d++) c *= mx[d] >= mn[d] ? (unsigned long long)(mx[d] - mn[d] + 1) : 0ull;
        if (c > 0xFFFFFFull) {  // more than 2^24 cells for one box: refuse instead of looping for minutes
            atomicAdd(over, 1ull);
            c = 0;
        }
        cnt[i] = (uint32_t)c;
    }
}

// kScatter = false: bucket histogram; true: insertion index of every entry
// scattered into its bucket's range
template <bool kScatter>
__global__ void kHgCells(const double* __restrict__ bmin, const double* __restrict__ bmax, int64_t n, HgGrid g,
                         const uint32_t* __restrict__ offs, uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor,
                         uint32_t* __restrict__ order) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int mn[3], mx[3];
        hgRange(g, bmin + 3 * i, bmax + 3 * i, mn, mx);
        if (offs[i + 1] == offs[i]) continue;
        uint32_t e = offs[i];
        for (int iz = mn[2]; iz <= mx[2]; iz++)
            for (int iy = mn[1]; iy <= mx[1]; iy++)
                for (int ix = mn[0]; ix <= mx[0]; ix++, e++) {
                    const uint32_t h = refHash(ix, iy, iz, g.size);
                    if (kScatter) order[atomicAdd(&cursor[h], 1u)] = e;
                    else atomicAdd(&hist[h], 1u);
                }
    }
}

// Each bucket's insertion indices in ascending order, then the item of each
// (the last item whose first index is <= the entry's, by binary search).
__global__ void kHgSortBuckets(const uint32_t* __restrict__ start, uint32_t size, uint32_t* __restrict__ order,
                               const uint32_t* __restrict__ offs, int64_t n, int32_t* __restrict__ items) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < size; b += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = start[b], e = start[b + 1];
        for (uint32_t k = s + 1; k < e; k++) {  // insertion sort: buckets hold few entries
            const uint32_t v = order[k];
            uint32_t j = k;
            while (j > s && order[j - 1] > v) {
                order[j] = order[j - 1];
                j--;
            }
            order[j] = v;
        }
        for (uint32_t k = s; k < e; k++) {
            const uint32_t v = order[k];
            int64_t lo = 0, hi = n - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi + 1) >> 1;
                if (offs[mid] <= v) lo = mid; else hi = mid - 1;
            }
            items[k] = (int32_t)lo;
        }
    }
}

unsigned hgBlocks(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace

}  // namespace pppm

using namespace pppm;

extern "C" int pppm_hashgrid_build(pppm_ctx* c, const double* boxmin, const double* boxmax, int64_t n,
                                   int32_t hash_size, double scale, const double* bbmin, uint32_t* start,
                                   int32_t* items, int64_t cap, int64_t* count) {
    if (!c || n < 0 || hash_size <= 0 || !bbmin || !count || (n > 0 && (!boxmin || !boxmax)) || cap < 0 ||
        (cap > 0 && !items) || n >= (int64_t)1 << 31)
        return fail(c, PPPM_E_ARG, "hashgrid_build: bad arguments");
    cudaSetDevice(c->device);
    HashGridBufs& hb = c->hashGrid;
    const HgGrid g{bbmin[0], bbmin[1], bbmin[2], scale, (uint32_t)hash_size};
    const void *dlo = nullptr, *dhi = nullptr;
    int r;
    if (n > 0) {
        if ((r = stageIn(c, boxmin, (size_t)n * 24, 0, &dlo))) return r;
        if ((r = stageIn(c, boxmax, (size_t)n * 24, 1, &dhi))) return r;
    }
    const double* lo = static_cast<const double*>(dlo);
    const double* hi = static_cast<const double*>(dhi);
    PPPM_CUDA(c, hb.offs.ensure(((size_t)n + 1) * 4));
    PPPM_CUDA(c, hb.offsCursor.ensure(((size_t)n + 1) * 4));
    PPPM_CUDA(c, hb.offsTmp.ensure((size_t)scanTmpWords(n + 1) * 4));
    PPPM_CUDA(c, hb.hist.ensure(((size_t)hash_size + 1) * 4));
    PPPM_CUDA(c, hb.cursor.ensure(((size_t)hash_size + 1) * 4));
    PPPM_CUDA(c, hb.tmp.ensure((size_t)scanTmpWords((int64_t)hash_size + 1) * 4));
    PPPM_CUDA(c, hb.flag.ensure(8));
    uint32_t* offs = hb.offs.as<uint32_t>();
    uint32_t* hist = hb.hist.as<uint32_t>();
    unsigned long long* over = hb.flag.as<unsigned long long>();
    PPPM_CUDA(c, cudaMemsetAsync(offs, 0, ((size_t)n + 1) * 4, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(hist, 0, ((size_t)hash_size + 1) * 4, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(over, 0, 8, c->stream));
    if (n > 0) kHgCount<<<hgBlocks(n), 256, 0, c->stream>>>(lo, hi, n, g, offs, over);
    PPPM_CUDA(c, cudaGetLastError());
    if (n > 0) PPPM_CUDA(c, exclusiveScan(offs, n, hb.offsCursor.as<uint32_t>(), hb.offsTmp.as<uint32_t>(), c->stream));
    uint32_t total = 0;
    unsigned long long overH = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&total, offs + n, 4, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaMemcpyAsync(&overH, over, 8, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (overH) return fail(c, PPPM_E_CAPACITY, "hashgrid_build: a box covers more than 2^24 cells");
    *count = total;
    if (!start && !items) return PPPM_OK;
    if (!start) return fail(c, PPPM_E_ARG, "hashgrid_build: start is required with items");
    if (items && (int64_t)total > cap) return fail(c, PPPM_E_CAPACITY, "hashgrid_build: items holds fewer entries");
    PPPM_CUDA(c, hb.order.ensure((size_t)std::max<uint32_t>(total, 1) * 4));
    if (n > 0)
        kHgCells<false><<<hgBlocks(n), 256, 0, c->stream>>>(lo, hi, n, g, offs, hist, nullptr, nullptr);
    PPPM_CUDA(c, cudaGetLastError());
    PPPM_CUDA(c, exclusiveScan(hist, hash_size, hb.cursor.as<uint32_t>(), hb.tmp.as<uint32_t>(), c->stream));
    void *dstart, *ditems = nullptr;
    if ((r = stageOut(c, start, ((size_t)hash_size + 1) * 4, 2, &dstart))) return r;
    if (items && total > 0) {
        if ((r = stageOut(c, items, (size_t)total * 4, 3, &ditems))) return r;
        if (n > 0)
            kHgCells<true><<<hgBlocks(n), 256, 0, c->stream>>>(lo, hi, n, g, offs, nullptr, hb.cursor.as<uint32_t>(),
                                                               hb.order.as<uint32_t>());
        kHgSortBuckets<<<hgBlocks(hash_size), 256, 0, c->stream>>>(hist, (uint32_t)hash_size, hb.order.as<uint32_t>(),
                                                                   offs, n, static_cast<int32_t*>(ditems));
        PPPM_CUDA(c, cudaGetLastError());
    }
    PPPM_CUDA(c, cudaMemcpyAsync(dstart, hist, ((size_t)hash_size + 1) * 4, cudaMemcpyDeviceToDevice, c->stream));
    if ((r = finishOut(c, start, dstart, ((size_t)hash_size + 1) * 4))) return r;
    if (ditems && (r = finishOut(c, items, ditems, (size_t)total * 4))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}
