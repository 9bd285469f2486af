// Fused forward pass of the proposal network on the 5th-generation tensor
// cores: one CTA of 128 threads holds the FP16 weights of all four layers in
// shared memory (canonical no-swizzle K-major layout), computes the input
// encoding of 128 rows, and runs the four GEMMs as tcgen05.mma (M=128,
// N=64/48, K=16 steps) with the FP32 accumulator in TMEM. After each layer
// the four warps read their 32 rows back with tcgen05.ld, add the bias,
// apply ReLU, and write the FP16 activations as the next A operand. The
// last layer's outputs go through the (then free) A buffer so that the
// tile's 20 KB of results leave in coalesced 16-byte stores, and each
// thread loads its row of the next tile before the current tile's GEMMs so
// that the input latency overlaps them. Every mbarrier wait is bounded; on a
// timeout the CTA records an error, waits for its MMAs to drain and frees
// its TMEM.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "mlp.cuh"
#include "mlp_dev.cuh"
#include "umma.cuh"

namespace pppm {

namespace {

constexpr int kSmemW = kMlpTilesBytes;        // 32768
constexpr int kSmemBias = 1024;               // 240 floats, padded
constexpr int kSmemA = kMlpRows * kMlpIn * 2;  // 20480
constexpr int kSmemTotal = kSmemW + kSmemBias + kSmemA + 64 + 1024;  // + barrier/slot + alignment slack

__global__ void __launch_bounds__(128) kMlpForward(MlpInputs in, const uint8_t* __restrict__ blob, int64_t cap,
                                                   const unsigned long long* count, float* __restrict__ out,
                                                   int* __restrict__ err, bool vecOut) {
    const int64_t n = count ? min((int64_t)*count, cap) : cap;
    extern __shared__ uint8_t smemRaw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~(uintptr_t)1023);
    uint8_t* sW = smem;
    float* sBias = reinterpret_cast<float*>(smem + kSmemW);
    uint8_t* sA = smem + kSmemW + kSmemBias;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sA + kSmemA);
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;

    for (int i = tid; i < (kSmemW + kMlpBiasFloats * 4) / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(smem)[i] = __ldg(reinterpret_cast<const uint4*>(blob) + i);
    const uint32_t mb = smemAddr(mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                     "r"(64));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asyncProxyFence();
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    const uint32_t tmem = *tmemSlot;
    const uint32_t aBase = smemAddr(sA), wBase = smemAddr(sW);
    uint32_t phase = 0;
    bool ok = true;

    float cur[6];
    {
        const int64_t row0 = (int64_t)blockIdx.x * kMlpRows + tid;
        mlpLoadRow(in, row0 < n ? row0 : -1, cur);
    }
    for (int64_t tile = blockIdx.x; ok && tile * kMlpRows < n; tile += gridDim.x) {
        const int64_t row = tile * kMlpRows + tid;
        {
            float f[kMlpIn];
            mlpFeaturesOf(in, cur, row < n, f);
#pragma unroll
            for (int c = 0; c < kMlpIn / 8; c++) storeChunk(sA, mlpCanon(tid, 8 * c, kMlpIn), f + 8 * c);
        }
        // the next tile's row, in flight during this tile's GEMMs
        float nxt[6];
        {
            const int64_t nrow = (tile + gridDim.x) * kMlpRows + tid;
            mlpLoadRow(in, nrow < n ? nrow : -1, nxt);
        }
        asyncProxyFence();
        tcFenceBefore();
        __syncthreads();
#pragma unroll
        for (int l = 0; l < kMlpLayers; l++) {
            const int K = mlpK(l), N = mlpN(l);
            if (tid == 0) {
                tcFenceAfter();
                const uint32_t idesc = umIdesc(kMlpRows, N);
                const uint32_t sbo = (uint32_t)(K / 8) * 128u;
#pragma unroll
                for (int kk = 0; kk < K / 16; kk++) {
                    const uint64_t a = umDesc(aBase + kk * 256, 128, sbo);
                    const uint64_t b = umDesc(wBase + mlpTileOffset(l) + kk * 256, 128, sbo);
                    umma(tmem, a, b, idesc, kk > 0 ? 1u : 0u);
                }
                umCommit(mb);
            }
            const bool got = mbarWait(mb, phase);
            phase ^= 1u;
            ok = !__syncthreads_or(!got);
            if (!ok) break;
            tcFenceAfter();
            float v[kMlpHidden];
            const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
            for (int c = 0; c < N / 16; c++) tmemLd16(lane + c * 16, v + 16 * c);
            tmemWaitLd();
            const float* bias = sBias + l * kMlpHidden;
            if (l < kMlpLayers - 1) {
#pragma unroll
                for (int j = 0; j < kMlpHidden; j++) v[j] = fmaxf(v[j] + bias[j], 0.0f);
#pragma unroll
                for (int c = 0; c < kMlpHidden / 8; c++) storeChunk(sA, mlpCanon(tid, 8 * c, kMlpHidden), v + 8 * c);
                asyncProxyFence();
                tcFenceBefore();
                __syncthreads();
            } else {
                // the tile's outputs, row-major in the A buffer (its MMAs are done)
                float4* sOut = reinterpret_cast<float4*>(sA);
#pragma unroll
                for (int c = 0; c < kMlpOut / 4; c++)
                    sOut[tid * (kMlpOut / 4) + c] = make_float4(v[4 * c] + bias[4 * c], v[4 * c + 1] + bias[4 * c + 1],
                                                                v[4 * c + 2] + bias[4 * c + 2], v[4 * c + 3] + bias[4 * c + 3]);
                __syncthreads();
                const int rows = (int)min((int64_t)kMlpRows, n - tile * kMlpRows);
                if (vecOut) {
                    float4* o = reinterpret_cast<float4*>(out + tile * kMlpRows * kMlpOut);
                    for (int i = tid; i < rows * (kMlpOut / 4); i += blockDim.x) o[i] = sOut[i];
                } else {
                    float* o = out + tile * kMlpRows * kMlpOut;
                    const float* so = reinterpret_cast<const float*>(sOut);
                    for (int i = tid; i < rows * kMlpOut; i += blockDim.x) o[i] = so[i];
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 6; i++) cur[i] = nxt[i];
        tcFenceBefore();
        __syncthreads();
    }
    if (!ok && tid == 0) {
        atomicExch(err, 1);
        // the last commit may still be outstanding: wait (bounded) before freeing TMEM
        mbarWait(mb, phase);
    }
    tcFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcFenceAfter();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(64));
    }
}

}  // namespace

cudaError_t launchMlpForward(const MlpInputs& in, const uint8_t* blob, int64_t n, float* out, int* err,
                             cudaStream_t st, const unsigned long long* count) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(kMlpForward, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTotal);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + kMlpRows - 1) / kMlpRows;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, 152 * 4);  // 4 CTAs per SM fit the shared memory
    const bool vecOut = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    kMlpForward<<<grid, 128, kSmemTotal, st>>>(in, blob, n, count, out, err, vecOut);
    return cudaGetLastError();
}

}  // namespace pppm

using namespace pppm;

extern "C" int pppm_mlp_forward(pppm_ctx* c, const float* params, const float* pos, const float* nrm, int64_t n,
                                const double* bbox, float* out) {
    if (!c || !params || !bbox || n < 0 || (n > 0 && (!pos || !nrm || !out)))
        return fail(c, PPPM_E_ARG, "mlp_forward: bad arguments");
    if (n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    PPPM_CUDA(c, c->stage[3].ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, cudaMemcpyAsync(c->stage[3].p, params, (size_t)kMlpParams * 4,
                                 isDevicePtr(params) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
    PPPM_CUDA(c, c->stageRec.ensure((size_t)kMlpBlobBytes));
    PPPM_CUDA(c, launchMlpPack(c->stage[3].as<float>(), c->stageRec.as<uint8_t>(), c->stream));
    const void *dp, *dn;
    void* dout;
    int r;
    if ((r = stageIn(c, pos, (size_t)n * 12, 0, &dp))) return r;
    if ((r = stageIn(c, nrm, (size_t)n * 12, 1, &dn))) return r;
    if ((r = stageOut(c, out, (size_t)n * kMlpOut * 4, 2, &dout))) return r;
    PPPM_CUDA(c, c->stageCount.ensure(64));
    PPPM_CUDA(c, cudaMemsetAsync(c->stageCount.p, 0, 4, c->stream));
    MlpInputs in = mlpInputs(bbox, (const float*)dp, (const float*)dn);
    PPPM_CUDA(c, launchMlpForward(in, c->stageRec.as<uint8_t>(), n, (float*)dout, c->stageCount.as<int>(), c->stream));
    if ((r = finishOut(c, out, dout, (size_t)n * kMlpOut * 4))) return r;
    int err = 0;
    PPPM_CUDA(c, cudaMemcpyAsync(&err, c->stageCount.p, 4, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    if (err) return fail(c, PPPM_E_CUDA, "mlp_forward: a tensor-core wait timed out");
    return PPPM_OK;
}
