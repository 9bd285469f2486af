// The learned photon proposal's network: 80 inputs (12-frequency encoding of
// the position in the scene box + the normal), three hidden layers of 64
// (ReLU), 40 outputs = 8 von Mises-Fisher lobes x (weight logit, mean xyz,
// log kappa). FP16 weights and activations, FP32 accumulation on the
// tcgen05 tensor cores (accumulators in TMEM).
#pragma once

#include <cstdint>

namespace pppm {

constexpr int kMlpIn = 80;       // 72 encoding + 3 normal + 5 zero
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 40;      // 8 lobes x 5
constexpr int kMlpOutPad = 48;   // N of the last MMA (multiple of 16)
constexpr int kMlpLobes = 8;
constexpr int kMlpFreqs = 12;
constexpr int kMlpLayers = 4;
constexpr int kMlpRows = 128;    // rows per tile (M of every MMA)

// fan-in / fan-out per layer
__host__ __device__ constexpr int mlpK(int l) { return l == 0 ? kMlpIn : kMlpHidden; }
__host__ __device__ constexpr int mlpN(int l) { return l == 3 ? kMlpOutPad : kMlpHidden; }
__host__ __device__ constexpr int mlpNReal(int l) { return l == 3 ? kMlpOut : kMlpHidden; }

// Parameter count of the flat FP32 layout W1 b1 W2 b2 W3 b3 W4 b4, each W
// row-major [out][in].
constexpr int kMlpParams = 64 * 80 + 64 + 64 * 64 + 64 + 64 * 64 + 64 + 40 * 64 + 40;
static_assert(kMlpParams == 16104, "parameter count of the C ABI");

// Byte offsets of the packed FP16 B tiles (canonical K-major layout, N x K
// per layer) and FP32 biases in the device weight blob.
__host__ __device__ constexpr int mlpTileBytes(int l) { return mlpN(l) * mlpK(l) * 2; }
__host__ __device__ constexpr int mlpTileOffset(int l) {
    return l == 0 ? 0 : mlpTileOffset(l - 1) + mlpTileBytes(l - 1);
}
constexpr int kMlpTilesBytes = mlpTileOffset(4);  // 10240 + 8192 + 8192 + 6144
constexpr int kMlpBiasFloats = 64 + 64 + 64 + kMlpOutPad;
constexpr int kMlpBiasBytes = 1024;  // biases, padded
// Transposed tiles for the backward pass: W_l^T as [in = N][out = K] for
// layers 2..4 (K = 64, 64, 48).
__host__ __device__ constexpr int mlpTKOut(int l) { return l == 3 ? kMlpOutPad : kMlpHidden; }
__host__ __device__ constexpr int mlpTTileOffset(int l) { return (l - 1) * kMlpHidden * kMlpHidden * 2; }
constexpr int kMlpTTilesBytes = 2 * 8192 + 6144;
// blob: [forward tiles][biases][transposed tiles]
constexpr int kMlpBlobBytes = kMlpTilesBytes + kMlpBiasBytes + kMlpTTilesBytes;

// Offsets of W_l and b_l in the flat parameter vector.
__host__ __device__ constexpr int mlpWOffset(int l) {
    return l == 0 ? 0 : mlpWOffset(l - 1) + mlpNReal(l - 1) * mlpK(l - 1) + mlpNReal(l - 1);
}
__host__ __device__ constexpr int mlpBOffset(int l) { return mlpWOffset(l) + mlpNReal(l) * mlpK(l); }
static_assert(mlpBOffset(3) + kMlpOut == kMlpParams, "parameter layout");

// One training record: position, normal, direction, weight.
struct MlpRecord {
    float px, py, pz, w;
    float nx, ny, nz, pad0;
    float dx, dy, dz, pad1;
};

// Offset of element (row r, column k) of a [rows x K] FP16 operand in the
// no-swizzle K-major canonical layout: 8x8 core matrices of 128 contiguous
// bytes, K-adjacent cores 128 B apart (LBO), 8-row groups K/8*128 B apart
// (SBO).
__host__ __device__ inline int mlpCanon(int r, int k, int K) {
    return (r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

}  // namespace pppm
