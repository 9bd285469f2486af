// Stage entry points of the dipole BSSRDF: Rd tables and the hierarchical
// irradiance over injected irradiance points (octree built by k_octree.cu).
#include <cmath>
#include <cstring>

#include "context.h"
#include "dipole.cuh"

namespace pppm {

namespace {

__global__ void kDipoleRd(DipoleDev m, const float* __restrict__ d2, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 r = dipoleRd(m, d2[i]);
    out[3 * i] = r.x;
    out[3 * i + 1] = r.y;
    out[3 * i + 2] = r.z;
}

__global__ void kDipoleIrradiance(OctView o, DipoleDev m, const float* __restrict__ q, int64_t nq,
                                  float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const f3 s = subsurfaceIrradiance(o, m, q[3 * i], q[3 * i + 1], q[3 * i + 2], nullptr);
    out[3 * i] = s.x;
    out[3 * i + 1] = s.y;
    out[3 * i + 2] = s.z;
}

// Both forms of fast_exp over the float bit patterns [begin, end): count
// of arguments the integer form covers and of covered arguments whose
// results differ in any bit.
__global__ void kFastExpCheck(uint64_t begin, uint64_t end, unsigned long long* counts) {
    unsigned long long covered = 0, differ = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = begin + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < end; b += stride) {
        const float y = __uint_as_float((uint32_t)b);
        float v;
        if (!fastExpRefInt(y, &v)) continue;
        covered++;
        if (__float_as_uint(v) != __float_as_uint(fastExpRefD(y))) differ++;
    }
    for (int o = 16; o > 0; o >>= 1) {
        covered += __shfl_xor_sync(0xffffffffu, covered, o);
        differ += __shfl_xor_sync(0xffffffffu, differ, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&counts[0], covered);
        atomicAdd(&counts[1], differ);
    }
}

}  // namespace

}  // namespace pppm

using namespace pppm;

extern "C" {

int pppm_dipole_rd(pppm_ctx* c, const pppm_material* mat, const float* d2, int64_t n, float* rgb) {
    if (!c || !mat || n < 0 || (n > 0 && (!d2 || !rgb))) return fail(c, PPPM_E_ARG, "dipole_rd: bad arguments");
    if (n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    const void* dd;
    void* dout;
    int r;
    if ((r = stageIn(c, d2, (size_t)n * 4, 0, &dd))) return r;
    if ((r = stageOut(c, rgb, (size_t)n * 12, 1, &dout))) return r;
    kDipoleRd<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(dipoleFrom(*mat), (const float*)dd, n, (float*)dout);
    PPPM_CUDA(c, cudaGetLastError());
    if ((r = finishOut(c, rgb, dout, (size_t)n * 12))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_dipole_irradiance(pppm_ctx* c, const pppm_material* mat, const float* ipts, int64_t n, double maxError,
                           const float* queries, int64_t m, float* rgb) {
    if (!c || !mat || n < 0 || m < 0 || (n > 0 && !ipts) || (m > 0 && (!queries || !rgb)))
        return fail(c, PPPM_E_ARG, "dipole_irradiance: bad arguments");
    if (m == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    const void* dp = nullptr;
    int r;
    if (n > 0 && (r = stageIn(c, ipts, (size_t)n * 40, 2, &dp))) return r;
    const float* P = static_cast<const float*>(dp);
    // IrradiancePoint rows: pos xyz, normal xyz, area, irradiance rgb
    const OctreePoints op{P, 10, P ? P + 7 : nullptr, 10, P ? P + 6 : nullptr, 10, 0.0};
    int numNodes = 0;
    int64_t launches = 0;
    if ((r = octreeBuild(c, c->stageOct, op, n, c->stream, &numNodes, &launches))) return r;
    const void* dq;
    void* dout;
    if ((r = stageIn(c, queries, (size_t)m * 12, 0, &dq))) return r;
    if ((r = stageOut(c, rgb, (size_t)m * 12, 1, &dout))) return r;
    const OctView ov{numNodes > 0 ? c->stageOct.out.as<OctNodeDev>() : nullptr, numNodes, (float)maxError};
    kDipoleIrradiance<<<(unsigned)((m + 127) / 128), 128, 0, c->stream>>>(ov, dipoleFrom(*mat), (const float*)dq, m,
                                                                          (float*)dout);
    PPPM_CUDA(c, cudaGetLastError());
    if ((r = finishOut(c, rgb, dout, (size_t)m * 12))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_fast_exp_check(pppm_ctx* c, uint64_t begin, uint64_t end, uint64_t* covered, uint64_t* differ) {
    if (!c || !covered || !differ || begin > end || end > (1ull << 32))
        return fail(c, PPPM_E_ARG, "fast_exp_check: bad arguments");
    cudaSetDevice(c->device);
    PPPM_CUDA(c, c->stageCount.ensure(16));
    unsigned long long* d = c->stageCount.as<unsigned long long>();
    PPPM_CUDA(c, cudaMemsetAsync(d, 0, 16, c->stream));
    if (end > begin) kFastExpCheck<<<152 * 8, 256, 0, c->stream>>>(begin, end, d);
    PPPM_CUDA(c, cudaGetLastError());
    unsigned long long h[2];
    PPPM_CUDA(c, cudaMemcpyAsync(h, d, 16, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    *covered = h[0];
    *differ = h[1];
    return PPPM_OK;
}

}  // extern "C"
