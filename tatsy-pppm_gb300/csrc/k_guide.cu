// Learned photon proposal in the wavefront photon pass (canonical mode).
//
// Emission and every Lambertian bounce that survives Russian roulette leave
// the path with its direction pending (the oriented normal kept in the
// direction field). Between bounce kernels the proposal network evaluates
// all pending paths of the queue (kGuidePack + the tcgen05 MLP), and
// kGuideResolve draws the direction by one-sample MIS from the mixture
//     p(w) = c p_bsdf(w) + (1 - c) q_vMF(w | x, n),   c = floor (0.3)
// of the cosine BSDF lobe (the reference's own sampling) and the network's
// von Mises-Fisher mixture, multiplying the flux by p_bsdf(w) / p(w), so the
// photon distribution keeps the plain estimator's expectation. A sampled
// subset of the draws become training records (x, n, w); the bounce kernel
// that finds the next hit y fills in the record weight
// Phi cos(w) I(y) / p(w): Phi the photon's flux luminance at the draw, I the
// eye-query importance of y's voxel from the previous pass
// (kImportanceSplat).
#include "context.h"
#include "trace.h"

namespace pppm {

namespace {

unsigned blocksOf(int64_t n, int bs, int cap = 152 * 16) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + bs - 1) / bs, cap));
}


__global__ void kGuidePack(const PathState* __restrict__ q, const unsigned long long* count, int64_t cap,
                           float* __restrict__ pos, float* __restrict__ nrm) {
    const int64_t n = min((int64_t)*count, cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const PathState& p = q[i];
        pos[3 * i] = (float)p.ox;
        pos[3 * i + 1] = (float)p.oy;
        pos[3 * i + 2] = (float)p.oz;
        nrm[3 * i] = p.dx;
        nrm[3 * i + 1] = p.dy;
        nrm[3 * i + 2] = p.dz;
    }
}

__global__ void kGuideResolve(TraceParams tp, PathState* __restrict__ q, const unsigned long long* count, int64_t cap,
                              const float* __restrict__ raw, float floorBsdf, int bounce) {
    const int64_t n = min((int64_t)*count, cap);
    const GuideView& g = tp.guide;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        PathState p = q[i];
        if (!(p.pad[1] & kPathNeedsDir)) continue;
        XorShift x;
        x.s[0] = p.rng[0]; x.s[1] = p.rng[1]; x.s[2] = p.rng[2]; x.s[3] = p.rng[3];
        const f3 nn = {p.dx, p.dy, p.dz};
        // canonical-mode draws: scrambled xorshift outputs (see Tape)
        const float us = u32ToFloat(mix32(x.next()));
        const float u1 = u32ToFloat(mix32(x.next()));
        const float u2 = u32ToFloat(mix32(x.next()));
        f3 d;
        float pdfCos, pdfMix;
        if (raw) {
            VmfMix m;
            vmfMixFromRaw(raw + (size_t)i * kMlpOut, &m, g.maxLogKappa);
            if (us < floorBsdf) {
                d = onHemisphere(nn, u1, u2);
            } else {
                const float u0 = (us - floorBsdf) / (1.0f - floorBsdf);
                d = vmfMixSample(m, u0, u1, u2);
            }
            const float c = dot(nn, d);
            pdfCos = fmaxf(c, 0.0f) * (1.0f / kPiF);
            pdfMix = floorBsdf * pdfCos + (1.0f - floorBsdf) * vmfMixPdf(m, d);
            if (!isfinite(pdfMix) || !isfinite(d.x + d.y + d.z)) {
                // a non-finite network output: the BSDF lobe alone for this draw
                d = onHemisphere(nn, u1, u2);
                pdfCos = fmaxf(dot(nn, d), 0.0f) * (1.0f / kPiF);
                pdfMix = pdfCos;
            }
        } else {
            d = onHemisphere(nn, u1, u2);
            pdfCos = fmaxf(dot(nn, d), 0.0f) * (1.0f / kPiF);
            pdfMix = pdfCos;
        }
        // directions the BSDF lobe cannot produce carry no flux
        const float wgt = (pdfCos > 0.0f && pdfMix > 0.0f) ? pdfCos / pdfMix : 0.0f;
        // photon flux at the decision: records of bright photons (the rare
        // high-flux ones that dominate the estimator's variance) weigh more
        const float lumFlux = 0.2126f * p.fx + 0.7152f * p.fy + 0.0722f * p.fz;
        p.fx *= wgt;
        p.fy *= wgt;
        p.fz *= wgt;
        p.dx = d.x;
        p.dy = d.y;
        p.dz = d.z;
        p.pad[1] &= ~kPathNeedsDir;
        p.pad[0] = -1;
        if (g.rec && wgt > 0.0f && mix32((uint32_t)p.id * 0x9E3779B1u + (uint32_t)bounce + tp.pass * 0x85EBCA77u) %
                                           g.recEvery == 0) {
            const unsigned long long r = atomicAdd(g.recCount, 1ull);
            if ((int64_t)r < g.recCap) {
                MlpRecord rec;
                rec.px = (float)p.ox; rec.py = (float)p.oy; rec.pz = (float)p.oz;
                rec.w = 0.0f;  // cos I(y) / p, filled in when the next hit y is known
                rec.nx = nn.x; rec.ny = nn.y; rec.nz = nn.z;
                rec.pad0 = lumFlux * fmaxf(dot(nn, d), 0.0f) / pdfMix;
                rec.dx = d.x; rec.dy = d.y; rec.dz = d.z;
                rec.pad1 = 0.0f;
                g.rec[r] = rec;
                p.pad[0] = (int)r;
            }
        }
        p.rng[0] = x.s[0]; p.rng[1] = x.s[1]; p.rng[2] = x.s[2]; p.rng[3] = x.s[3];
        q[i] = p;
    }
}

// Importance of a voxel for the relative error of the image: summed over the
// gather queries inside it, the luminance of the eye-path weight divided by
// the pixel's current estimate (accumulated radiance / passes, plus a floor),
// so dim pixels ask for as many photons per unit of their radiance as bright
// ones.
__global__ void kImportanceSplat(GuideView g, const float4* __restrict__ qs, const unsigned long long* count,
                                 int64_t cap, const float* __restrict__ accum, float invPasses, float floorLum,
                                 float* __restrict__ grid) {
    const int64_t n = min((int64_t)*count, cap);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = qs[3 * i], w = qs[3 * i + 2];
        const int v = impVoxel(g, a.x, a.y, a.z);
        if (v < 0) continue;
        const int64_t px = __float_as_int(a.w);
        const float L = (0.2126f * accum[3 * px] + 0.7152f * accum[3 * px + 1] + 0.0722f * accum[3 * px + 2]) *
                        invPasses;
        atomicAdd(&grid[v], (0.2126f * w.x + 0.7152f * w.y + 0.0722f * w.z) / (L + floorLum));
    }
}

__global__ void kRecordSum(const MlpRecord* __restrict__ rec, int64_t n, float* sum) {
    float s = 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += rec[i].w;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.0f) atomicAdd(sum, s);
}

__global__ void kInvert(float* v) {
    const float s = *v;
    *v = s > 0.0f ? 1.0f / s : 0.0f;
}

}  // namespace

cudaError_t launchGuidePack(const PathState* q, const unsigned long long* count, int64_t cap, float* pos, float* nrm,
                            cudaStream_t st) {
    kGuidePack<<<blocksOf(cap, 256), 256, 0, st>>>(q, count, cap, pos, nrm);
    return cudaGetLastError();
}

cudaError_t launchGuideResolve(const TraceParams& tp, PathState* q, const unsigned long long* count, int64_t cap,
                               const float* raw, float floorBsdf, int bounce, cudaStream_t st) {
    kGuideResolve<<<blocksOf(cap, 128), 128, 0, st>>>(tp, q, count, cap, raw, floorBsdf, bounce);
    return cudaGetLastError();
}

cudaError_t launchImportanceSplat(const GuideView& g, const float4* queries, const unsigned long long* count,
                                  int64_t cap, const float* accum, float invPasses, float floorLum, float* grid,
                                  cudaStream_t st) {
    kImportanceSplat<<<blocksOf(cap, 256), 256, 0, st>>>(g, queries, count, cap, accum, invPasses, floorLum, grid);
    return cudaGetLastError();
}

// 1 / sum of the record weights of rec[0, n) into *sum (device)
cudaError_t launchRecordInvSum(const MlpRecord* rec, int64_t n, float* sum, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(sum, 0, 4, st);
    if (e != cudaSuccess) return e;
    kRecordSum<<<blocksOf(n, 256, 152 * 4), 256, 0, st>>>(rec, n, sum);
    kInvert<<<1, 1, 0, st>>>(sum);
    return cudaGetLastError();
}

}  // namespace pppm
