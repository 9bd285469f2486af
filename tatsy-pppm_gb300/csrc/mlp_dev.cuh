// Device side of the proposal network: input encoding and the von
// Mises-Fisher mixture it outputs (pdf and sampling).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "mlp.cuh"
#include "pppm_device.cuh"

namespace pppm {

// Rows of the network input: positions and normals (3 floats each) and the
// scene box that normalises positions to [0, 1]^3.
struct MlpInputs {
    float ox, oy, oz;  // box minimum
    float sx, sy, sz;  // 1 / box extent per axis
    const float* pos;
    const float* nrm;
};

inline MlpInputs mlpInputs(const double* bbox, const float* pos, const float* nrm) {
    MlpInputs in;
    in.ox = (float)bbox[0];
    in.oy = (float)bbox[1];
    in.oz = (float)bbox[2];
    in.sx = (float)(1.0 / std::max(bbox[3] - bbox[0], 1e-12));
    in.sy = (float)(1.0 / std::max(bbox[4] - bbox[1], 1e-12));
    in.sz = (float)(1.0 / std::max(bbox[5] - bbox[2], 1e-12));
    in.pos = pos;
    in.nrm = nrm;
    return in;
}

// features[a*24 + 2k] = sin(2^k pi x_a), [a*24 + 2k + 1] = cos(2^k pi x_a),
// x_a the normalised coordinate; [72..74] = normal; [75..79] = 0.
// Every fourth frequency is evaluated directly (sincospif of 2^k x_a, an
// exact argument); the three above it by the double-angle identities
// sin 2t = 2 sin t cos t, cos 2t = (cos t - sin t)(cos t + sin t), each of
// which at most doubles the absolute error: under 1e-6 after three steps,
// far below the FP16 rounding (2^-11) the features then go through.
__device__ __forceinline__ void mlpEncode(float x, float y, float z, float nx, float ny, float nz, float* f) {
    const float c[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
#pragma unroll
        for (int k0 = 0; k0 < kMlpFreqs; k0 += 4) {
            float sn, cs;
            sincospif(c[a] * (float)(1 << k0), &sn, &cs);
#pragma unroll
            for (int k = k0; k < k0 + 4 && k < kMlpFreqs; k++) {
                f[a * 24 + 2 * k] = sn;
                f[a * 24 + 2 * k + 1] = cs;
                const float s2 = 2.0f * sn * cs;
                cs = (cs - sn) * (cs + sn);
                sn = s2;
            }
        }
    }
    f[72] = nx;
    f[73] = ny;
    f[74] = nz;
#pragma unroll
    for (int i = 75; i < kMlpIn; i++) f[i] = 0.0f;
}

// The 6 input floats of a row (position, normal), or zeros for row < 0.
__device__ __forceinline__ void mlpLoadRow(const MlpInputs& in, int64_t row, float* r) {
    if (row < 0) {
#pragma unroll
        for (int i = 0; i < 6; i++) r[i] = 0.0f;
        return;
    }
    const float* p = in.pos + 3 * row;
    const float* n = in.nrm + 3 * row;
    r[0] = __ldg(p);
    r[1] = __ldg(p + 1);
    r[2] = __ldg(p + 2);
    r[3] = __ldg(n);
    r[4] = __ldg(n + 1);
    r[5] = __ldg(n + 2);
}

// Features of a row loaded by mlpLoadRow (valid = false: all zero).
__device__ __forceinline__ void mlpFeaturesOf(const MlpInputs& in, const float* r, bool valid, float* f) {
    if (!valid) {
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
        return;
    }
    mlpEncode((r[0] - in.ox) * in.sx, (r[1] - in.oy) * in.sy, (r[2] - in.oz) * in.sz, r[3], r[4], r[5], f);
}

__device__ __forceinline__ void mlpFeatures(const MlpInputs& in, int64_t row, float* f) {
    if (row < 0) {
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) f[i] = 0.0f;
        return;
    }
    const float* p = in.pos + 3 * row;
    const float* n = in.nrm + 3 * row;
    mlpEncode((p[0] - in.ox) * in.sx, (p[1] - in.oy) * in.sy, (p[2] - in.oz) * in.sz, n[0], n[1], n[2], f);
}

// ---------------------------------------------------------------- vMF mixture
// The network's 40 outputs as a mixture of 8 von Mises-Fisher lobes:
// weights = softmax(logits), means = normalised 3-vectors, kappa =
// exp(clamp(log kappa, -4, 7)).
struct VmfMix {
    float w[kMlpLobes];
    float mu[kMlpLobes][3];
    float kappa[kMlpLobes];
    float norm[kMlpLobes];  // kappa / (2 pi (1 - e^{-2 kappa}))
};

__device__ inline void vmfMixFromRaw(const float* raw, VmfMix* m, float maxLogKappa = 7.0f) {
    float lmax = -1e30f;
#pragma unroll
    for (int k = 0; k < kMlpLobes; k++) lmax = fmaxf(lmax, raw[5 * k]);
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kMlpLobes; k++) {
        m->w[k] = __expf(raw[5 * k] - lmax);
        s += m->w[k];
    }
    const float inv = 1.0f / s;
#pragma unroll
    for (int k = 0; k < kMlpLobes; k++) {
        m->w[k] *= inv;
        const float x = raw[5 * k + 1], y = raw[5 * k + 2], z = raw[5 * k + 3];
        const float l = fmaxf(sqrtf(x * x + y * y + z * z), 1e-12f);
        m->mu[k][0] = x / l;
        m->mu[k][1] = y / l;
        m->mu[k][2] = z / l;
        const float kk = __expf(fminf(fmaxf(raw[5 * k + 4], -4.0f), maxLogKappa));
        m->kappa[k] = kk;
        m->norm[k] = kk / (6.283185307179586f * -expm1f(-2.0f * kk));
    }
}

__device__ inline float vmfMixPdf(const VmfMix& m, f3 d) {
    float p = 0.0f;
#pragma unroll
    for (int k = 0; k < kMlpLobes; k++) {
        const float c = m.mu[k][0] * d.x + m.mu[k][1] * d.y + m.mu[k][2] * d.z;
        p += m.w[k] * m.norm[k] * __expf(m.kappa[k] * (c - 1.0f));
    }
    return p;
}

// Lobe by u0, then the vMF sample of the lobe (cosine to the mean from
// 1 + log(u1 + (1 - u1) e^{-2 kappa}) / kappa, azimuth 2 pi u2).
__device__ inline f3 vmfMixSample(const VmfMix& m, float u0, float u1, float u2) {
    int k = 0;
    float acc = m.w[0];
    while (k < kMlpLobes - 1 && u0 >= acc) acc += m.w[++k];
    const float kk = m.kappa[k];
    const float e = __expf(-2.0f * kk);
    const float cw = fminf(fmaxf(1.0f + __logf(u1 + (1.0f - u1) * e) / kk, -1.0f), 1.0f);
    const float sw = sqrtf(fmaxf(0.0f, 1.0f - cw * cw));
    float sp, cp;
    sincospif(2.0f * u2, &sp, &cp);
    const f3 w = {m.mu[k][0], m.mu[k][1], m.mu[k][2]};
    f3 u = fabsf(w.x) > 0.1f ? cross(mk(0.f, 1.f, 0.f), w) : cross(mk(1.f, 0.f, 0.f), w);
    u = normalized(u);
    const f3 v = cross(w, u);
    return normalized(u * (sw * cp) + v * (sw * sp) + w * cw);
}

cudaError_t launchMlpPack(const float* params, uint8_t* blob, cudaStream_t st);
// n: rows (or capacity when count != nullptr: rows = min(*count, n))
cudaError_t launchMlpForward(const MlpInputs& in, const uint8_t* blob, int64_t n, float* out, int* err,
                             cudaStream_t st, const unsigned long long* count = nullptr);
cudaError_t launchMlpTrain(const MlpRecord* rec, int64_t n, const float* invSumW, const MlpInputs& box,
                           const uint8_t* blob, float* grad, float* loss, int* err, cudaStream_t st,
                           float maxLogKappa = 7.0f);
cudaError_t launchMlpAdam(float* params, const float* grad, float* m, float* v, int step, float lr, cudaStream_t st);

}  // namespace pppm
