// Training of the proposal network on the tensor cores.
//
// kMlpTrain: one persistent CTA per SM (128 threads, 176 KB shared memory,
// all 512 TMEM columns). Per 128-record tile it recomputes the forward pass
// (keeping ReLU masks in registers and the FP16 activations of every layer
// in shared memory, transposed), evaluates the gradient of the weighted
// negative log-likelihood of the record directions under the vMF mixture,
// and back-propagates with tcgen05.mma:
//   dA_{l-1} = dZ_l W_l          (M = 128 records, N = fan-in, K = fan-out)
//   dW_l    += dZ_l^T A_{l-1}    (M = fan-out padded to 128, N = fan-in,
//                                 K = 128 records; accumulated in TMEM over
//                                 the CTA's tiles, added to the global
//                                 gradient once at the end)
// kMlpPack turns the FP32 parameters into the FP16 blob (forward tiles,
// biases, transposed tiles); kMlpAdam applies Adam to the FP32 master copy.
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

constexpr int kOffW = 0;
constexpr int kOffB = kMlpTilesBytes;                    // 32768
constexpr int kOffWT = kOffB + kMlpBiasBytes;            // 33792
constexpr int kOffA = kOffWT + kMlpTTilesBytes;          // 56320
constexpr int kOffAct = kOffA + kMlpRows * kMlpIn * 2;   // 76800
constexpr int kActBytes0 = kMlpIn * kMlpRows * 2;        // a0^T: 20480
constexpr int kActBytes = kMlpHidden * kMlpRows * 2;     // a1..a3^T: 16384 each
constexpr int kOffDz = kOffAct + kActBytes0 + 3 * kActBytes;  // 146432
constexpr int kOffBg = kOffDz + 128 * kMlpRows * 2;           // 179200
constexpr int kOffMisc = kOffBg + 1024;                       // 180224
constexpr int kTrainSmem = kOffMisc + 64 + 1024;              // + alignment slack
// TMEM columns
constexpr int kColWork = 0;
__host__ __device__ constexpr int dwCol(int l) { return l == 0 ? 64 : l == 1 ? 144 : l == 2 ? 208 : 272; }

__device__ __forceinline__ int actOffset(int l) { return l == 0 ? 0 : kActBytes0 + (l - 1) * kActBytes; }

__device__ __forceinline__ void storeHalf(uint8_t* base, int off, float v) {
    *reinterpret_cast<__half*>(base + off) = __float2half_rn(v);
}

// d(-s log q)/d(raw outputs) for one record; returns -s log q.
__device__ float vmfLossGrad(const float* raw, float dx, float dy, float dz, float s, float* g, float maxLk) {
    float logt[kMlpLobes], lw[kMlpLobes], dlog_dlk[kMlpLobes], kap[kMlpLobes], inl[kMlpLobes], cosv[kMlpLobes];
    float mu[kMlpLobes][3], mlen[kMlpLobes];
    float lmax = -1e30f;
    for (int k = 0; k < kMlpLobes; k++) lmax = fmaxf(lmax, raw[5 * k]);
    float se = 0.0f;
    for (int k = 0; k < kMlpLobes; k++) se += __expf(raw[5 * k] - lmax);
    const float lse = lmax + __logf(se);
    for (int k = 0; k < kMlpLobes; k++) {
        lw[k] = raw[5 * k] - lse;
        const float mx = raw[5 * k + 1], my = raw[5 * k + 2], mz = raw[5 * k + 3];
        const float len = sqrtf(mx * mx + my * my + mz * mz);
        mlen[k] = fmaxf(len, 1e-12f);
        mu[k][0] = mx / mlen[k];
        mu[k][1] = my / mlen[k];
        mu[k][2] = mz / mlen[k];
        const float lkr = raw[5 * k + 4];
        inl[k] = (lkr >= -4.0f && lkr <= maxLk) ? 1.0f : 0.0f;
        const float lk = fminf(fmaxf(lkr, -4.0f), maxLk);
        const float kk = __expf(lk);
        kap[k] = kk;
        cosv[k] = mu[k][0] * dx + mu[k][1] * dy + mu[k][2] * dz;
        const float om = -expm1f(-2.0f * kk);  // 1 - e^{-2 kappa}
        // log vMF = log kappa - log(2 pi) - log(1 - e^{-2 kappa}) + kappa (mu.d - 1)
        const float logf_k = lk - 1.8378770664093453f - __logf(om) + kk * (cosv[k] - 1.0f);
        logt[k] = lw[k] + logf_k;
        dlog_dlk[k] = 1.0f - 2.0f * kk * (1.0f - om) / om + kk * (cosv[k] - 1.0f);
    }
    float tmax = -1e30f;
    for (int k = 0; k < kMlpLobes; k++) tmax = fmaxf(tmax, logt[k]);
    float ts = 0.0f;
    for (int k = 0; k < kMlpLobes; k++) ts += __expf(logt[k] - tmax);
    const float logq = tmax + __logf(ts);
    for (int k = 0; k < kMlpLobes; k++) {
        const float r = __expf(logt[k] - logq);
        const float pi = __expf(lw[k]);
        g[5 * k] = s * (pi - r);
        const float c = -s * r * kap[k] / mlen[k];
        g[5 * k + 1] = c * (dx - cosv[k] * mu[k][0]);
        g[5 * k + 2] = c * (dy - cosv[k] * mu[k][1]);
        g[5 * k + 3] = c * (dz - cosv[k] * mu[k][2]);
        g[5 * k + 4] = -s * r * dlog_dlk[k] * inl[k];
    }
    return -s * logq;
}

// Column sums of a warp's 64 x 32 values (t[j] of lane i: column j, record
// i): five halving steps with shuffles; afterwards lane i holds in t[0] and
// t[1] the sums of columns c and c + 1, c = 32 b4 + 16 b3 + 8 b2 + 4 b1 + 2 b0
// for the bits b4..b0 of i. t[2..63] are left undefined.
__device__ __forceinline__ void warpColumnSums(float* t) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int half = 32, off = 16; half >= 2; half >>= 1, off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int j = 0; j < half; j++) {
            const float send = upper ? t[j] : t[j + half];
            const float keep = upper ? t[j + half] : t[j];
            t[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
}

__global__ void __launch_bounds__(128, 1) kMlpTrain(const MlpRecord* __restrict__ rec, int64_t n, const float* invSumW,
                                                    MlpInputs box, const uint8_t* __restrict__ blob,
                                                    float* __restrict__ grad, float* __restrict__ loss,
                                                    int* __restrict__ err, float maxLk) {
    extern __shared__ uint8_t smemRaw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem + kOffA;
    uint8_t* sAct = smem + kOffAct;
    uint8_t* sDz = smem + kOffDz;
    const float* sBias = reinterpret_cast<const float*>(smem + kOffB);
    float* sBg = reinterpret_cast<float*>(smem + kOffBg);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kOffMisc);
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;

    for (int i = tid; i < kOffA / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(smem)[i] = __ldg(reinterpret_cast<const uint4*>(blob) + i);
    for (int i = tid; i < kMlpBiasFloats; i += blockDim.x) sBg[i] = 0.0f;
    const uint32_t mb = smemAddr(mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asyncProxyFence();
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    const uint32_t tmem = *tmemSlot;
    const uint32_t base = smemAddr(smem);
    const uint32_t aA = base + kOffA, aAct = base + kOffAct, aDz = base + kOffDz, aW = base + kOffW,
                   aWT = base + kOffWT;
    // the backward pass runs on weights normalised to mean 1 (s = w n / sum w)
    // so FP16 gradients stay far from underflow; 1/n rescales the results
    const float s0 = *invSumW * (float)n, outScale = 1.0f / (float)n;
    uint32_t phase = 0;
    bool ok = true, first = true;
    float lossSum = 0.0f;

    auto waitMma = [&]() -> bool {
        const bool got = mbarWait(mb, phase);
        phase ^= 1u;
        const bool all = !__syncthreads_or(!got);
        tcFenceAfter();
        return all;
    };
    auto syncForMma = [&]() {
        asyncProxyFence();
        tcFenceBefore();
        __syncthreads();
    };

    for (int64_t tile = blockIdx.x; ok && tile * kMlpRows < n; tile += gridDim.x) {
        const int64_t row = tile * kMlpRows + tid;
        float dx = 0.f, dy = 0.f, dz = 1.f, w = 0.f;
        {
            float f[kMlpIn];
            if (row < n) {
                const MlpRecord r = rec[row];
                mlpEncode((r.px - box.ox) * box.sx, (r.py - box.oy) * box.sy, (r.pz - box.oz) * box.sz, r.nx, r.ny,
                          r.nz, f);
                dx = r.dx; dy = r.dy; dz = r.dz; w = r.w;
            } else {
#pragma unroll
                for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
            }
#pragma unroll
            for (int c = 0; c < kMlpIn / 8; c++) storeChunk(sA, mlpCanon(tid, 8 * c, kMlpIn), f + 8 * c);
#pragma unroll
            for (int k = 0; k < kMlpIn; k++) storeHalf(sAct, actOffset(0) + mlpCanon(k, tid, kMlpRows), f[k]);
        }
        syncForMma();
        uint64_t mask[3] = {0, 0, 0};
        float v[kMlpHidden];
        // ---------------- forward
#pragma unroll
        for (int l = 0; l < kMlpLayers; l++) {
            const int K = mlpK(l), N = mlpN(l);
            if (tid == 0) {
                tcFenceAfter();
                const uint32_t sbo = (uint32_t)(K / 8) * 128u;
#pragma unroll
                for (int kk = 0; kk < K / 16; kk++)
                    umma(tmem + kColWork, umDesc(aA + kk * 256, 128, sbo),
                         umDesc(aW + mlpTileOffset(l) + kk * 256, 128, sbo), umIdesc(kMlpRows, N), kk > 0);
                umCommit(mb);
            }
            if (!(ok = waitMma())) break;
            const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
            for (int c = 0; c < N / 16; c++) tmemLd16(lane + kColWork + c * 16, v + 16 * c);
            tmemWaitLd();
            const float* bias = sBias + l * kMlpHidden;
            if (l < kMlpLayers - 1) {
                uint64_t m = 0;
#pragma unroll
                for (int j = 0; j < kMlpHidden; j++) {
                    const float z = v[j] + bias[j];
                    if (z > 0.0f) m |= 1ull << j;
                    v[j] = fmaxf(z, 0.0f);
                }
                mask[l] = m;
#pragma unroll
                for (int c = 0; c < kMlpHidden / 8; c++) storeChunk(sA, mlpCanon(tid, 8 * c, kMlpHidden), v + 8 * c);
#pragma unroll
                for (int k = 0; k < kMlpHidden; k++)
                    storeHalf(sAct, actOffset(l + 1) + mlpCanon(k, tid, kMlpRows), v[k]);
                syncForMma();
            } else {
#pragma unroll
                for (int j = 0; j < kMlpOut; j++) v[j] += bias[j];
            }
        }
        if (!ok) break;
        // ---------------- loss gradient w.r.t. the raw outputs
        float g[kMlpHidden];  // dZ of the current layer (48 output columns, then 64 hidden)
#pragma unroll
        for (int j = kMlpOut; j < kMlpHidden; j++) g[j] = 0.0f;
        if (row < n && w > 0.0f) {
            // weights clipped at 256x the batch mean keep FP16 gradients finite
            lossSum += vmfLossGrad(v, dx, dy, dz, fminf(w * s0, 256.0f), g, maxLk);
        } else {
#pragma unroll
            for (int j = 0; j < kMlpOut; j++) g[j] = 0.0f;
        }
        // ---------------- backward: layers 4, 3, 2, 1
#pragma unroll
        for (int l = kMlpLayers - 1; l >= 0; l--) {
            const int Kout = l == kMlpLayers - 1 ? kMlpOutPad : kMlpHidden;  // dZ columns
            const int nOut = mlpNReal(l);
            // dZ_l: transposed for dW, row-major (K = fan-out) for dA
#pragma unroll
            for (int o = 0; o < Kout; o++) storeHalf(sDz, mlpCanon(o, tid, kMlpRows), g[o]);
            if (l > 0) {
#pragma unroll
                for (int c = 0; c < Kout / 8; c++) storeChunk(sA, mlpCanon(tid, 8 * c, Kout), g + 8 * c);
            }
            // bias gradient: the column sums of dZ over the warp's 32 records by
            // recursive halving (each step a lane keeps half of its columns and
            // adds its partner's copy of them), then one shared atomic per lane
            // and column pair instead of one per record and column
            warpColumnSums(g);
            {
                const int lane = tid & 31;
                const int col = ((lane >> 4) & 1) * 32 + ((lane >> 3) & 1) * 16 + ((lane >> 2) & 1) * 8 +
                                ((lane >> 1) & 1) * 4 + (lane & 1) * 2;
                const int bOff = l * kMlpHidden;
                if (col < nOut && g[0] != 0.0f) atomicAdd(&sBg[bOff + col], g[0]);
                if (col + 1 < nOut && g[1] != 0.0f) atomicAdd(&sBg[bOff + col + 1], g[1]);
            }
            syncForMma();
            if (tid == 0) {
                tcFenceAfter();
                // dW_l += dZ^T A_{l-1}^T: M = 128 (fan-out padded), N = fan-in, K = 128 records
                const int Nin = mlpK(l);
#pragma unroll
                for (int kk = 0; kk < kMlpRows / 16; kk++)
                    umma(tmem + dwCol(l), umDesc(aDz + kk * 256, 128, 2048),
                         umDesc(aAct + actOffset(l) + kk * 256, 128, 2048), umIdesc(128, Nin),
                         (!first || kk > 0) ? 1u : 0u);
                if (l > 0) {
                    // dA_{l-1} = dZ W_l: M = 128 records, N = fan-in (64), K = fan-out
                    const uint32_t sbo = (uint32_t)(Kout / 8) * 128u;
#pragma unroll
                    for (int kk = 0; kk < Kout / 16; kk++)
                        umma(tmem + kColWork, umDesc(aA + kk * 256, 128, sbo),
                             umDesc(aWT + mlpTTileOffset(l) + kk * 256, 128, sbo), umIdesc(kMlpRows, kMlpHidden),
                             kk > 0);
                }
                umCommit(mb);
            }
            if (!(ok = waitMma())) break;
            if (l > 0) {
                const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
                for (int c = 0; c < kMlpHidden / 16; c++) tmemLd16(lane + kColWork + c * 16, v + 16 * c);
                tmemWaitLd();
                const uint64_t m = mask[l - 1];
#pragma unroll
                for (int j = 0; j < kMlpHidden; j++) g[j] = ((m >> j) & 1ull) ? v[j] : 0.0f;
                tcFenceBefore();
            }
        }
        first = false;
        tcFenceBefore();
        __syncthreads();
    }
    // loss
    {
        float t = lossSum;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((tid & 31) == 0 && t != 0.0f) atomicAdd(loss, t * outScale);
    }
    if (!ok) {
        if (tid == 0) {
            atomicExch(err, 1);
            mbarWait(mb, phase);  // let the outstanding MMAs drain before freeing TMEM
        }
    } else if (!first) {
        // weight gradients: lane t of dW_l holds row (fan-out index) t
        tcFenceAfter();
        const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int l = 0; l < kMlpLayers; l++) {
            const int Nin = mlpK(l), nOut = mlpNReal(l);
            float* gw = grad + mlpWOffset(l);
#pragma unroll
            for (int c = 0; c < Nin / 16; c++) {
                float t16[16];
                tmemLd16(lane + dwCol(l) + c * 16, t16);
                tmemWaitLd();
                if (tid < nOut)
#pragma unroll
                    for (int i = 0; i < 16; i++) atomicAdd(&gw[tid * Nin + c * 16 + i], t16[i] * outScale);
            }
        }
    }
    __syncthreads();
    if (ok && !first)
        for (int i = tid; i < kMlpBiasFloats; i += blockDim.x) {
            const int l = i / kMlpHidden, o = i % kMlpHidden;
            if (o < mlpNReal(l) && sBg[i] != 0.0f) atomicAdd(&grad[mlpBOffset(l) + o], sBg[i] * outScale);
        }
    tcFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcFenceAfter();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

// FP32 parameters -> FP16 blob (forward tiles, biases, transposed tiles).
__global__ void kMlpPack(const float* __restrict__ p, uint8_t* __restrict__ blob) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // forward tiles: element (n, k) of layer l
    int e = i;
    for (int l = 0; l < kMlpLayers; l++) {
        const int K = mlpK(l), N = mlpN(l);
        if (e < N * K) {
            const int nn = e / K, k = e % K;
            const float v = nn < mlpNReal(l) ? p[mlpWOffset(l) + nn * K + k] : 0.0f;
            storeHalf(blob, mlpTileOffset(l) + mlpCanon(nn, k, K), v);
            return;
        }
        e -= N * K;
    }
    if (e < kMlpBiasFloats) {
        const int l = e / kMlpHidden, o = e % kMlpHidden;
        reinterpret_cast<float*>(blob + kMlpTilesBytes)[e] = o < mlpNReal(l) ? p[mlpBOffset(l) + o] : 0.0f;
        return;
    }
    e -= kMlpBiasFloats;
    // transposed tiles of layers 1..3: element (in i, out o)
    for (int l = 1; l < kMlpLayers; l++) {
        const int Kout = mlpTKOut(l), Nin = kMlpHidden;
        if (e < Nin * Kout) {
            const int i2 = e / Kout, o = e % Kout;
            const float v = o < mlpNReal(l) ? p[mlpWOffset(l) + o * Nin + i2] : 0.0f;
            storeHalf(blob, kMlpTilesBytes + kMlpBiasBytes + mlpTTileOffset(l) + mlpCanon(i2, o, Kout), v);
            return;
        }
        e -= Nin * Kout;
    }
}

constexpr int kPackElems = 64 * 80 + 64 * 64 * 2 + 48 * 64 + kMlpBiasFloats + 64 * 64 * 2 + 64 * 48;

__global__ void kMlpAdam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                         float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = isfinite(g[i]) ? g[i] : 0.0f;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

}  // namespace

cudaError_t launchMlpPack(const float* params, uint8_t* blob, cudaStream_t st) {
    kMlpPack<<<(kPackElems + 255) / 256, 256, 0, st>>>(params, blob);
    return cudaGetLastError();
}

cudaError_t launchMlpTrain(const MlpRecord* rec, int64_t n, const float* invSumW, const MlpInputs& box,
                           const uint8_t* blob, float* grad, float* loss, int* err, cudaStream_t st,
                           float maxLogKappa) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(kMlpTrain, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + kMlpRows - 1) / kMlpRows;
    kMlpTrain<<<(unsigned)std::min<int64_t>(tiles, 152), 128, kTrainSmem, st>>>(rec, n, invSumW, box, blob, grad, loss,
                                                                               err, maxLogKappa);
    return cudaGetLastError();
}

cudaError_t launchMlpAdam(float* params, const float* grad, float* m, float* v, int step, float lr,
                          cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, step)));
    kMlpAdam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(params, grad, m, v, kMlpParams, lr, b1, b2, 1e-8f, c1, c2);
    return cudaGetLastError();
}

}  // namespace pppm

using namespace pppm;

extern "C" int pppm_mlp_grad(pppm_ctx* c, const float* params, const float* records, int64_t n, const double* bbox,
                             float* grad, float* loss) {
    if (!c || !params || !bbox || !grad || !loss || n < 0 || (n > 0 && !records))
        return fail(c, PPPM_E_ARG, "mlp_grad: bad arguments");
    cudaSetDevice(c->device);
    std::vector<float> hr((size_t)n * 10);
    if (n > 0) {
        if (isDevicePtr(records)) PPPM_CUDA(c, cudaMemcpy(hr.data(), records, hr.size() * 4, cudaMemcpyDeviceToHost));
        else std::memcpy(hr.data(), records, hr.size() * 4);
    }
    std::vector<MlpRecord> rv((size_t)n);
    double sw = 0.0;
    for (int64_t i = 0; i < n; i++) {
        const float* s = &hr[10 * i];
        rv[i] = MlpRecord{s[0], s[1], s[2], s[9], s[3], s[4], s[5], 0.f, s[6], s[7], s[8], 0.f};
        sw += s[9];
    }
    const float inv = sw > 0.0 ? (float)(1.0 / sw) : 0.0f;
    // scratch: params, blob, records, grad, loss/err/invSumW
    PPPM_CUDA(c, c->stage[3].ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, c->stage[4].ensure((size_t)kMlpBlobBytes));
    PPPM_CUDA(c, c->stage[5].ensure((size_t)std::max<int64_t>(n, 1) * sizeof(MlpRecord)));
    PPPM_CUDA(c, c->stage[6].ensure((size_t)kMlpParams * 4));
    PPPM_CUDA(c, c->stage[7].ensure(64));
    PPPM_CUDA(c, cudaMemcpyAsync(c->stage[3].p, params, (size_t)kMlpParams * 4,
                                 isDevicePtr(params) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(c->stage[4].p, 0, (size_t)kMlpBlobBytes, c->stream));
    PPPM_CUDA(c, launchMlpPack(c->stage[3].as<float>(), c->stage[4].as<uint8_t>(), c->stream));
    if (n > 0)
        PPPM_CUDA(c, cudaMemcpyAsync(c->stage[5].p, rv.data(), (size_t)n * sizeof(MlpRecord), cudaMemcpyHostToDevice,
                                     c->stream));
    PPPM_CUDA(c, cudaMemsetAsync(c->stage[6].p, 0, (size_t)kMlpParams * 4, c->stream));
    float* misc = c->stage[7].as<float>();  // [0] loss, [1] err, [2] 1/sum w
    PPPM_CUDA(c, cudaMemsetAsync(misc, 0, 8, c->stream));
    PPPM_CUDA(c, cudaMemcpyAsync(misc + 2, &inv, 4, cudaMemcpyHostToDevice, c->stream));
    const MlpInputs box = mlpInputs(bbox, nullptr, nullptr);
    PPPM_CUDA(c, launchMlpTrain(c->stage[5].as<MlpRecord>(), n, misc + 2, box, c->stage[4].as<uint8_t>(),
                                c->stage[6].as<float>(), misc, reinterpret_cast<int*>(misc + 1), c->stream));
    float hm[2] = {0.f, 0.f};
    PPPM_CUDA(c, cudaMemcpyAsync(hm, misc, 8, cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaMemcpyAsync(grad, c->stage[6].p, (size_t)kMlpParams * 4,
                                 isDevicePtr(grad) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    int e;
    std::memcpy(&e, &hm[1], 4);
    if (e) return fail(c, PPPM_E_CUDA, "mlp_grad: a tensor-core wait timed out");
    *loss = hm[0];
    return PPPM_OK;
}
