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
__device__ __forceinline__ void mlpEncode(float x, float y, float z, float nx, float ny, float nz, float* f) {
    const float c[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float s = c[a];
#pragma unroll
        for (int k = 0; k < kMlpFreqs; k++) {
            float sn, cs;
            sincospif(s, &sn, &cs);
            f[a * 24 + 2 * k] = sn;
            f[a * 24 + 2 * k + 1] = cs;
            s *= 2.0f;
        }
    }
    f[72] = nx;
    f[73] = ny;
    f[74] = nz;
#pragma unroll
    for (int i = 75; i < kMlpIn; i++) f[i] = 0.0f;
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

cudaError_t launchMlpPack(const float* params, uint8_t* blob, cudaStream_t st);
cudaError_t launchMlpForward(const MlpInputs& in, const uint8_t* blob, int64_t n, float* out, int* err,
                             cudaStream_t st);
cudaError_t launchMlpTrain(const MlpRecord* rec, int64_t n, const float* invSumW, const MlpInputs& box,
                           const uint8_t* blob, float* grad, float* loss, int* err, cudaStream_t st);
cudaError_t launchMlpAdam(float* params, const float* grad, float* m, float* v, int step, float lr, cudaStream_t st);

}  // namespace pppm
