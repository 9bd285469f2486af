// Device-side data layouts and inner routines shared by the kernels.
//
// Exactness policy: every step whose result decides something discrete
// (which triangle is hit, which bucket a point falls in, Russian roulette,
// CDF inversion) repeats the reference's own arithmetic with explicitly
// rounded IEEE operations (no FMA contraction), in float where the
// reference uses float and in double where it uses double. Continuous
// shading (directions, fluxes, radiance) runs in FP32.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pppm {

constexpr double kEps = 1.0e-12;    // EPS (common.h:13)
constexpr double kInfty = 1.0e20;   // INFTY (common.h:12)
constexpr float kPiF = 3.14159265358979323846f;
constexpr double kPi = 3.14159265358979323846;
#ifndef PPPM_STACK_SIZE
#define PPPM_STACK_SIZE 64
#endif
constexpr int kStackSize = PPPM_STACK_SIZE;  // traversal stack; the builder caps depth at 20
constexpr int kMaxBvhDepth = 20;

// ------------------------------------------------------------------ layouts
// One 4-wide BVH node, 128 bytes (one L2 line). Boxes are the reference's
// float child boxes (qbvh_accel.cc:178-191) in [x/y/z][child] order.
// child[i] >= 0: inner node index; < 0: leaf code ~(first_slot << 2 | count).
struct __align__(16) QNode {
    float4 bmin[3];  // bmin[d] = (child0..3) min along axis d
    float4 bmax[3];
    int4 child;
    int4 meta;  // x: sepAxes packed (sep0 | sep1 << 2 | sep2 << 4), y,z,w unused
};
static_assert(sizeof(QNode) == 128, "QNode must be one 128-byte line");

// Leaf triangles are 3 float4 (p0,p1,p2); p0.w holds the original id bits.
__host__ __device__ inline int leafCode(int slot, int count) { return ~((slot << 2) | count); }

// Dipole BSSRDF constants (DipoleBSSRDF ctor, bssrdf.cc:48-63), derived on
// the host in double and rounded once.
struct DipoleDev {
    float sigma_tr[3], alphap[3], zpos[3], zneg[3];
    float scale;
    float coeff;  // (1/pi) * (1 - Fdr) (subsurface_integrator.cc:236-237)
};

struct DevMaterial {
    int type;        // BsdfType bitmask including the BSSRDF bit
    float refl[3];
    float phong_n;
    float roulette;  // max(refl) (ppm_probabilistic.cc:261)
    double rr_photon;  // (r+g+b)/3.0 in double (ppm_probabilistic.cc:177)
    // The reference compares draws x * 2^-32 (x a 32-bit integer) with these
    // doubles; the same decisions as integer compares:
    //   x * 2^-32 <  rr_photon  <=>  x <  rrCeil   = ceil(rr_photon * 2^32)
    //   x * 2^-32 >  roulette   <=>  x >  roulFloor = floor(roulette * 2^32)
    unsigned long long rrCeil;
    unsigned long long roulFloor;
    float invRr;     // 1 / rr_photon for the flux update
    float pad0;
    DipoleDev dip;   // valid when type has the BSSRDF bit
    float emit[3];   // emitted radiance of the front side (pppm_material_emission); 0 for the reference's materials
    int emissive;    // emit != 0
};

struct EnvDev {
    const float* rgb;    // w*h*3
    const double* cdf;   // 4096
    const double* pdf;   // 4096
    // lower_bound(cdf, x * 2^-32) as an integer search: the first i with
    // x <= ucdf[i] = floor(cdf[i] * 2^32)
    const unsigned long long* ucdf;
    // per CDF cell: (float)(area / (pdf * numPhotons)) (envmap.cc:80-83),
    // filled per render because numPhotons is a render parameter
    const float* fluxScale;
    int w, h;         // 0 x 0: no environment map (eye rays that miss see black)
    // emissive triangles (no counterpart in the reference, whose only light
    // is the environment): per emitter 3 float4 (p0, p1 - p0, p2 - p0; w of
    // the first: emitter material), the area CDF in double and as the
    // integer comparison values floor(cdf * 2^32), and the flux scale
    // pi * total area / photons. numLights > 0: every photon leaves an emitter.
    const float4* lightTri;
    const double* lightCdf;
    const unsigned long long* lightUcdf;
    const float* lightLe;   // 3 per emitter
    int numLights;
    float lightFluxScale;
};

// ------------------------------------------------------------------ RNG
// XorShift128 of the reference (random.h:16-62).
struct XorShift {
    uint32_t s[4];
    __host__ __device__ inline void seed(uint32_t init) {
        uint32_t v = init;
        for (int i = 1; i <= 4; i++) { v = 1812433253u * (v ^ (v >> 30)) + (uint32_t)i; s[i - 1] = v; }
    }
    __host__ __device__ inline uint32_t next() {
        const uint32_t t = s[0] ^ (s[0] << 11);
        s[0] = s[1]; s[1] = s[2]; s[2] = s[3];
        s[3] = (s[3] ^ (s[3] >> 19)) ^ (t ^ (t >> 8));
        return s[3];
    }
};

// s <- J s for one 128x128 GF(2) jump matrix J (128 columns of 4 words).
__device__ __forceinline__ void jumpApply(const uint32_t* __restrict__ J, uint32_t s[4]) {
    uint32_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    const uint4* cols = reinterpret_cast<const uint4*>(J);
#pragma unroll 1
    for (int w = 0; w < 4; w++) {
        const uint32_t word = s[w];
#pragma unroll 8
        for (int b = 0; b < 32; b++) {
            const uint32_t m = 0u - ((word >> b) & 1u);
            const uint4 c = __ldg(&cols[w * 32 + b]);
            r0 ^= c.x & m;
            r1 ^= c.y & m;
            r2 ^= c.z & m;
            r3 ^= c.w & m;
        }
    }
    s[0] = r0; s[1] = r1; s[2] = r2; s[3] = r3;
}

// nextReal() = next() * (float)(1/UINT_MAX) = next() * 2^-32 exactly (random.h:45-47)
__host__ __device__ inline double u32ToReal(uint32_t x) { return (double)x * 2.3283064365386963e-10; }

// nextReal() rounded to float without FP64: (float)(x * 2^-32) equals
// rn(x) * 2^-32 because scaling by a power of two commutes with rounding.
__device__ __forceinline__ float u32ToFloat(uint32_t x) { return __uint2float_rn(x) * 2.3283064365386963e-10f; }

// A 200-number tape consumed in order (RandomSequence, random_sequence.h).
// Murmur3's 32-bit finaliser: a nonlinear bijection of 32-bit words.
__host__ __device__ inline uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// scramble = 1 (canonical mode) passes every output through mix32.
// xorshift128 is linear: output k+4 is a fixed XOR combination of outputs k
// and k+3, so draws taken four apart on one path are tied together (the
// azimuth of a photon's first direction is a function of its env-CDF draw
// and polar draw, which folds all photons of one small bright env cell onto
// one curve of directions). Compat mode keeps the raw outputs, as the
// reference does.
//
// A draw of a tape, with the comparisons the shading code makes against
// double thresholds. A XorShift draw x stands for x * 2^-32 exactly, so the
// comparisons run on integers: x * 2^-32 < p <=> x < ceil(p * 2^32) and
// x * 2^-32 > p <=> x > floor(p * 2^32) (the thresholds are precomputed).
struct Draw32 {
    uint32_t u;
    __device__ inline bool lt(unsigned long long ceilThr, double) const { return u < ceilThr; }
    __device__ inline bool gt(unsigned long long floorThr, double) const { return u > floorThr; }
    __device__ inline float f() const { return u32ToFloat(u); }
};
// A draw of an arbitrary double in [0, 1) (the permuted Halton sampler):
// compared in double; u = floor(d * 2^32) feeds the float conversions.
struct DrawD {
    uint32_t u;
    double d;
    __device__ inline bool lt(unsigned long long, double thr) const { return d < thr; }
    __device__ inline bool gt(unsigned long long, double thr) const { return d > thr; }
    __device__ inline float f() const { return (float)d; }
};

struct Tape {
    static constexpr bool kExact32 = true;  // every draw is x * 2^-32
    XorShift x;
    int pos;
    uint32_t scramble = 0;
    __device__ inline uint32_t next() {
        const uint32_t v = x.next();
        return scramble ? mix32(v) : v;
    }
    __device__ inline double popd() { pos++; return u32ToReal(next()); }
    __device__ inline float popf() { pos++; return u32ToFloat(next()); }
    __device__ inline uint32_t popu() { pos++; return next(); }
    __device__ inline Draw32 draw() { return Draw32{popu()}; }
    __device__ inline bool exhausted() const { return pos > 200; }
};

// A tape given explicitly (stage tests feed the reference's own numbers).
struct ArrayTape {
    static constexpr bool kExact32 = true;
    const double* v;
    int pos;
    __device__ inline double popd() { return v[pos++]; }
    __device__ inline float popf() { return (float)popd(); }
    // tape values are x * 2^-32 with x < 2^32, so this is exact
    __device__ inline uint32_t popu() { return (uint32_t)(v[pos++] * 4294967296.0); }
    __device__ inline Draw32 draw() { return Draw32{popu()}; }
};

// ------------------------------------------------------------------ Halton
// Halton(200, true, seed) (halton.cc:88-152), the reference's
// RANDOM_SAMPLER_QUASI_MONTE_CARLO sampler: dimension j of sample n is the
// radical inverse of n in the j-th prime base with that base's digits
// permuted per sampler. Tables: permutations [stream][sum of bases], the
// first 200 primes and each base's offset in a stream's table.
constexpr int kHaltonDims = 200;

struct HaltonDev {
    const uint16_t* perm;
    const int* prime;
    const int* offset;
    int sum;
};

// Halton::radicalInverse (halton.cc:142-152) with its permutation, in
// double with the reference's operation order.
__device__ inline double haltonValue(const HaltonDev& h, int stream, unsigned long long n, int dim) {
    const int base = h.prime[dim];
    const uint16_t* p = h.perm + (size_t)stream * h.sum + h.offset[dim];
    const double invBase = __drcp_rn((double)base);
    double val = 0.0, invBi = invBase;
    while (n > 0xFFFFFFFFull) {  // 64-bit digits only while the index needs them
        const unsigned long long q = n / (unsigned)base;
        const int d = p[n - q * base];
        val = __dadd_rn(val, __dmul_rn((double)d, invBi));
        invBi = __dmul_rn(invBi, invBase);
        n = q;
    }
    for (uint32_t m = (uint32_t)n; m > 0;) {
        const uint32_t q = m / (uint32_t)base;
        const int d = p[m - q * (uint32_t)base];
        val = __dadd_rn(val, __dmul_rn((double)d, invBi));
        invBi = __dmul_rn(invBi, invBase);
        m = q;
    }
    return val;
}

// One RandomSequence of 200 numbers: sample `index` of sampler `stream`.
struct HaltonTape {
    static constexpr bool kExact32 = false;
    const HaltonDev* h;
    int stream;
    unsigned long long index;
    int dim;
    bool over;
    __device__ inline double popd() {
        if (dim >= kHaltonDims) {
            over = true;  // RandomSequence::pop asserts (random_sequence.h:50-53)
            return 0.0;
        }
        return haltonValue(*h, stream, index, dim++);
    }
    __device__ inline float popf() { return (float)popd(); }
    // a draw in [0, 1) as the 32-bit integer floor(r * 2^32): comparisons
    // against 0.5 and float conversions keep their meaning
    __device__ inline uint32_t popu() { return (uint32_t)fmin(popd() * 4294967296.0, 4294967295.0); }
    __device__ inline DrawD draw() {
        const double d = popd();
        return DrawD{(uint32_t)fmin(d * 4294967296.0, 4294967295.0), d};
    }
    __device__ inline bool exhausted() const { return over || dim > kHaltonDims; }
};

// ------------------------------------------------------------------ vectors
struct f3 { float x, y, z; };
__device__ inline f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ inline f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ inline f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ inline f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline f3 cross(f3 u, f3 v) { return {u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x}; }
// Vector3D::normalized divides by (norm + EPS) (vector3d.cc:63-65)
__device__ inline f3 normalized(f3 v) { return v * (1.0f / (sqrtf(dot(v, v)) + 1e-12f)); }
__device__ inline f3 reflect(f3 v, f3 n) { return v - n * (2.0f * dot(n, v)); }
__device__ inline float maxc(f3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }

// ------------------------------------------------------------------ exact geometry
// Moller-Trumbore in double with the reference's operation order
// (triangle.cc:53-78); every product and sum is an explicitly rounded IEEE
// double op so the result is bit-identical to the reference.
// The test after the edges: p0 = (double)a, e1 = b - a, e2 = c - a.
__device__ __forceinline__ bool triHitExactEdges(double ox, double oy, double oz, double dx, double dy, double dz,
                                                 double p0x, double p0y, double p0z, double e1x, double e1y,
                                                 double e1z, double e2x, double e2y, double e2z, double* tOut) {
    // pVec = cross(d, e2)
    const double px = __dsub_rn(__dmul_rn(dy, e2z), __dmul_rn(dz, e2y));
    const double py = __dsub_rn(__dmul_rn(dz, e2x), __dmul_rn(dx, e2z));
    const double pz = __dsub_rn(__dmul_rn(dx, e2y), __dmul_rn(dy, e2x));
    const double det = __dadd_rn(__dadd_rn(__dmul_rn(e1x, px), __dmul_rn(e1y, py)), __dmul_rn(e1z, pz));
    if (det > -kEps && det < kEps) return false;
    const double invdet = __drcp_rn(det);  // == 1.0 / det, correctly rounded
    const double tx = __dsub_rn(ox, p0x), ty = __dsub_rn(oy, p0y), tz = __dsub_rn(oz, p0z);
    const double u = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(tx, px), __dmul_rn(ty, py)), __dmul_rn(tz, pz)), invdet);
    if (u < 0.0 || u > 1.0) return false;
    // qVec = cross(tVec, e1)
    const double qx = __dsub_rn(__dmul_rn(ty, e1z), __dmul_rn(tz, e1y));
    const double qy = __dsub_rn(__dmul_rn(tz, e1x), __dmul_rn(tx, e1z));
    const double qz = __dsub_rn(__dmul_rn(tx, e1y), __dmul_rn(ty, e1x));
    const double v = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, qx), __dmul_rn(dy, qy)), __dmul_rn(dz, qz)), invdet);
    if (v < 0.0 || __dadd_rn(u, v) > 1.0) return false;
    const double t = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(e2x, qx), __dmul_rn(e2y, qy)), __dmul_rn(e2z, qz)), invdet);
    if (t > kEps) { *tOut = t; return true; }
    return false;
}

__device__ __forceinline__ bool triHitExact(double ox, double oy, double oz, double dx, double dy, double dz,
                                            const float4& a, const float4& b, const float4& c, double* tOut) {
    const double p0x = a.x, p0y = a.y, p0z = a.z;
    const double e1x = __dsub_rn((double)b.x, p0x), e1y = __dsub_rn((double)b.y, p0y), e1z = __dsub_rn((double)b.z, p0z);
    const double e2x = __dsub_rn((double)c.x, p0x), e2y = __dsub_rn((double)c.y, p0y), e2z = __dsub_rn((double)c.z, p0z);
    return triHitExactEdges(ox, oy, oz, dx, dy, dz, p0x, p0y, p0z, e1x, e1y, e1z, e2x, e2y, e2z, tOut);
}

#ifndef PPPM_TRI_EDGES
#define PPPM_TRI_EDGES 1
#endif
constexpr bool kTriEdges = PPPM_TRI_EDGES != 0;

// The same test from the slot's double vertex and edges, computed on the
// host with the same operations (10 doubles per slot: p0, e1, e2, pad), so
// that the test converts nothing and subtracts no vertices.
__device__ __forceinline__ bool triHitExactPre(double ox, double oy, double oz, double dx, double dy, double dz,
                                               const double* __restrict__ triE, int slot, double* tOut) {
    const double2* q = reinterpret_cast<const double2*>(triE + 10 * (int64_t)slot);
    const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3), e = __ldg(q + 4);
    return triHitExactEdges(ox, oy, oz, dx, dy, dz, a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y, e.x, tOut);
}

// Conservative FP32 pre-test for triHitExact. Returns false only when the
// exact double test is certain to reject the triangle or to produce a
// distance that cannot beat `best` (the caller's current closest hit);
// returns true when the exact test must decide. Rounding-error bounds follow
// the standard a-priori bound |fl(x) - x| <= gamma_k * S where S is the same
// expression evaluated on absolute values (Higham, Accuracy and Stability of
// Numerical Algorithms, ch. 3); gamma is inflated well above the tight
// value so the double reference's own rounding (2^-53) is covered too.
__device__ __forceinline__ bool triMayHit(float ox, float oy, float oz, float dx, float dy, float dz,
                                          const float4& a, const float4& b, const float4& c, float best) {
    const float kG = 3.0e-6f;  // ~ 48 * 2^-24
    const float e1x = b.x - a.x, e1y = b.y - a.y, e1z = b.z - a.z;
    const float e2x = c.x - a.x, e2y = c.y - a.y, e2z = c.z - a.z;
    const float ae1x = fabsf(e1x), ae1y = fabsf(e1y), ae1z = fabsf(e1z);
    const float ae2x = fabsf(e2x), ae2y = fabsf(e2y), ae2z = fabsf(e2z);
    const float adx = fabsf(dx), ady = fabsf(dy), adz = fabsf(dz);
    const float px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
    const float apx = ady * ae2z + adz * ae2y, apy = adz * ae2x + adx * ae2z, apz = adx * ae2y + ady * ae2x;
    const float det = e1x * px + e1y * py + e1z * pz;
    const float sdet = ae1x * apx + ae1y * apy + ae1z * apz;
    const float edet = kG * sdet + 2e-12f;
    if (fabsf(det) <= edet) return true;  // sign or EPS test undecided
    const float tx = ox - a.x, ty = oy - a.y, tz = oz - a.z;
    const float atx = fabsf(tx), aty = fabsf(ty), atz = fabsf(tz);
    const float nu = tx * px + ty * py + tz * pz;
    const float enu = kG * (atx * apx + aty * apy + atz * apz);
    const float qx = ty * e1z - tz * e1y, qy = tz * e1x - tx * e1z, qz = tx * e1y - ty * e1x;
    const float aqx = aty * ae1z + atz * ae1y, aqy = atz * ae1x + atx * ae1z, aqz = atx * ae1y + aty * ae1x;
    const float nv = dx * qx + dy * qy + dz * qz;
    const float env_ = kG * (adx * aqx + ady * aqy + adz * aqz);
    const float nt = e2x * qx + e2y * qy + e2z * qz;
    const float ent = kG * (ae2x * aqx + ae2y * aqy + ae2z * aqz);
    // Work with det > 0 by flipping the numerators' signs.
    const float s = det > 0.0f ? 1.0f : -1.0f;
    const float D = det * s, U = nu * s, V = nv * s, T = nt * s;
    // u < 0, v < 0, u > 1, u + v > 1, t <= 0 certain -> reject
    if (U < -enu) return false;
    if (V < -env_) return false;
    if (U - D > enu + edet) return false;
    if (U + V - D > enu + env_ + edet + kG * (fabsf(U) + fabsf(V) + D)) return false;
    if (T < -ent) return false;
    // t certainly not below best: cannot become the closest hit
    const float lo = (T - ent) / (D + edet);
    if (lo > best * (1.0f + 1e-5f)) return false;
    return true;
}

// orderTable of qbvh_accel.cc:21-39: for each (hitMask, sepMask) the child
// visiting order as nibbles, 0x4 terminating. Indexed [hitMask * 8 + sepMask].
static __device__ __constant__ int kOrderTableDev[128] = {
    0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44444,
    0x44440, 0x44440, 0x44440, 0x44440, 0x44440, 0x44440, 0x44440, 0x44440,
    0x44441, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441,
    0x44401, 0x44401, 0x44410, 0x44410, 0x44401, 0x44401, 0x44410, 0x44410,
    0x44442, 0x44442, 0x44442, 0x44442, 0x44442, 0x44442, 0x44442, 0x44442,
    0x44402, 0x44402, 0x44402, 0x44402, 0x44420, 0x44420, 0x44420, 0x44420,
    0x44412, 0x44412, 0x44412, 0x44412, 0x44421, 0x44421, 0x44421, 0x44421,
    0x44012, 0x44012, 0x44102, 0x44102, 0x44201, 0x44201, 0x44210, 0x44210,
    0x44443, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443,
    0x44403, 0x44403, 0x44403, 0x44403, 0x44430, 0x44430, 0x44430, 0x44430,
    0x44413, 0x44413, 0x44413, 0x44413, 0x44431, 0x44431, 0x44431, 0x44431,
    0x44013, 0x44013, 0x44103, 0x44103, 0x44301, 0x44301, 0x44310, 0x44310,
    0x44423, 0x44432, 0x44423, 0x44432, 0x44423, 0x44432, 0x44423, 0x44432,
    0x44023, 0x44032, 0x44023, 0x44032, 0x44230, 0x44320, 0x44230, 0x44320,
    0x44123, 0x44132, 0x44123, 0x44132, 0x44231, 0x44321, 0x44231, 0x44321,
    0x40123, 0x40132, 0x41023, 0x41032, 0x42301, 0x43201, 0x42310, 0x43210,
};

__device__ __forceinline__ void loadOrderTable(int* s) {
    for (int i = threadIdx.x; i < 128; i += blockDim.x) s[i] = kOrderTableDev[i];
    __syncthreads();
}


// Closest hit over the QBVH, reproducing QBVHAccel::intersect
// (qbvh_accel.cc:205-285): float slab test with SSE max/min semantics,
// orderTable child order, LIFO stack, leaf triangles in stored order with a
// strict `<` update. orderTab points at a shared-memory copy of the table.
// Returns the triangle slot or -1 and the hit distance in *bestOut.
constexpr int kTopNodes = 85;  // BFS levels 0-3 of the QBVH (1 + 4 + 16 + 64), staged in shared memory

// Cooperative copy of the top BVH levels into shared memory; nodes are in
// BFS order so the first kTopNodes are levels 0-3.
__device__ __forceinline__ void loadTopNodes(QNode* sTop, const QNode* __restrict__ nodes, int numNodes) {
    const int n = min(numNodes, kTopNodes) * (int)(sizeof(QNode) / sizeof(float4));
    const float4* src = reinterpret_cast<const float4*>(nodes);
    float4* dst = reinterpret_cast<float4*>(sTop);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = __ldg(&src[i]);
    __syncthreads();
}

template <bool kPrefilter>
__device__ __forceinline__ int traverseExact(const QNode* __restrict__ nodes, const float4* __restrict__ tris, int rootCode,
                                             double odx, double ody, double odz, float dx, float dy, float dz,
                                             const int* orderTab, double* bestOut, int* nodeVisits, int* triTests,
                                             const QNode* sTop = nullptr) {
    // the slab test runs on the float-rounded origin (qbvh_accel.cc:211-213),
    // the triangle test on the double origin
    const float ox = __double2float_rn(odx), oy = __double2float_rn(ody), oz = __double2float_rn(odz);
    const double ddx = dx, ddy = dy, ddz = dz;
    // idir = dir == 0 ? 1e20f : (float)(1.0 / dir)  (qbvh_accel.cc:219-221);
    // rounding 1/d to double then to float equals a correctly rounded float
    // reciprocal (double rounding is innocuous for p' >= 2p + 2).
    const float idx = dx == 0.0f ? 1.0e20f : __frcp_rn(dx);
    const float idy = dy == 0.0f ? 1.0e20f : __frcp_rn(dy);
    const float idz = dz == 0.0f ? 1.0e20f : __frcp_rn(dz);
    const int sx = idx > 0.0f ? 0 : 1, sy = idy > 0.0f ? 0 : 1, sz = idz > 0.0f ? 0 : 1;
    const int sgnBits = sx | (sy << 1) | (sz << 2);

    int stack[kStackSize];
    int sp = 0;
    stack[sp++] = rootCode;
    double best = kInfty;
    float bestf = 1.0e20f;  // (float)best, refreshed whenever best changes
    int hit = -1;
    int visits = 0, tests = 0;
    while (sp > 0) {
        const int code = stack[--sp];
        if (code < 0) {
            const int lc = ~code;
            const int first = lc >> 2, cnt = lc & 3;
            for (int i = 0; i < cnt; i++) {
                const float4 a = tris[3 * (first + i)], b = tris[3 * (first + i) + 1], c = tris[3 * (first + i) + 2];
                tests++;
                if (kPrefilter && !triMayHit(ox, oy, oz, dx, dy, dz, a, b, c, bestf)) continue;
                double t;
                if (triHitExact(odx, ody, odz, ddx, ddy, ddz, a, b, c, &t) && best > t) {
                    best = t;
                    bestf = __double2float_rn(t);
                    hit = first + i;
                }
            }
            continue;
        }
        visits++;
        // levels 0-3 come from shared memory, deeper nodes from L2/HBM
        const QNode* nd = (sTop != nullptr && code < kTopNodes) ? sTop + code : nodes + code;
        const float hd = bestf;
        float tmin[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float tmax[4] = {hd, hd, hd, hd};
        const float o3[3] = {ox, oy, oz};
        const float i3[3] = {idx, idy, idz};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float4 lo = nd->bmin[d];
            const float4 hi = nd->bmax[d];
            const bool neg = (sgnBits >> d) & 1;
            const float4 nearB = neg ? hi : lo;
            const float4 farB = neg ? lo : hi;
            const float nb[4] = {nearB.x, nearB.y, nearB.z, nearB.w};
            const float fb[4] = {farB.x, farB.y, farB.z, farB.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float t0 = __fmul_rn(__fsub_rn(nb[k], o3[d]), i3[d]);
                const float t1 = __fmul_rn(__fsub_rn(fb[k], o3[d]), i3[d]);
                tmin[k] = tmin[k] > t0 ? tmin[k] : t0;  // _mm_max_ps(tMin, t0)
                tmax[k] = tmax[k] < t1 ? tmax[k] : t1;  // _mm_min_ps(tMax, t1)
            }
        }
        int hitMask = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) hitMask |= (tmax[k] >= tmin[k]) ? (1 << k) : 0;
        if (hitMask != 0) {
            const int4 ch = nd->child;
            const int meta = nd->meta.x;
            const int a0 = meta & 3, a1 = (meta >> 2) & 3, a2 = (meta >> 4) & 3;
            const int sepMask = (((sgnBits >> a0) & 1) << 2) | (((sgnBits >> a1) & 1) << 1) | ((sgnBits >> a2) & 1);
            int ord = orderTab[hitMask * 8 + sepMask];
            const int c4[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                if (ord & 0x04) break;
                stack[sp++] = c4[ord & 0x03];
                ord >>= 4;
            }
        }
    }
    *bestOut = best;
    if (nodeVisits) *nodeVisits += visits;
    if (triTests) *triTests += tests;
    return hit;
}

// Warp-cooperative form of traverseExact with the same results. The double
// triangle test costs a warp ~50 FP64 instructions at 1/64 of the FP32 rate
// whenever any lane needs it, and lanes reach their leaves at different
// iterations. Here a lane whose FP32 pre-test passes records the leaf's
// candidate triangles (in leaf order) and pauses; the warp runs the double
// tests for all paused lanes together once kBatch lanes wait or no lane can
// advance. A paused lane does nothing else until its tests are done, so each
// lane performs the reference's operations in the reference's order: the
// same box tests against the same (float)best, the same strict updates.
// All 32 lanes of the warp must call it (inactive lanes pass active=false).
#ifndef PPPM_EXACT_BATCH
#define PPPM_EXACT_BATCH 12
#endif
constexpr int kExactBatch = PPPM_EXACT_BATCH;  // default; a render may tune it (1..32)
// persistent photon kernel: lanes of a warp that must have their closest
// hit before the warp shades them and refills (default; tunable, 1..32)
#ifndef PPPM_REFILL
#define PPPM_REFILL 24
#endif
constexpr int kRefill = PPPM_REFILL;

__device__ __forceinline__ int traverseExactWarp(const QNode* __restrict__ nodes, const float4* __restrict__ tris,
                                                 int rootCode, bool active, double odx, double ody, double odz,
                                                 float dx, float dy, float dz, const int* orderTab,
                                                 const QNode* sTop, double* bestOut, int* nodeVisits,
                                                 int* triTests, const double* __restrict__ triE = nullptr,
                                                 int exactBatch = kExactBatch) {
    const float ox = __double2float_rn(odx), oy = __double2float_rn(ody), oz = __double2float_rn(odz);
    const float idx = dx == 0.0f ? 1.0e20f : __frcp_rn(dx);
    const float idy = dy == 0.0f ? 1.0e20f : __frcp_rn(dy);
    const float idz = dz == 0.0f ? 1.0e20f : __frcp_rn(dz);
    const int sx = idx > 0.0f ? 0 : 1, sy = idy > 0.0f ? 0 : 1, sz = idz > 0.0f ? 0 : 1;
    const int sgnBits = sx | (sy << 1) | (sz << 2);
    int stack[kStackSize];
    int sp = 0;
    if (active) stack[sp++] = rootCode;
    double best = kInfty;
    float bestf = 1.0e20f;
    int hit = -1;
    int visits = 0, tests = 0;
    int cand0 = -1, cand1 = -1, cand2 = -1, ncand = 0;  // pending exact tests, leaf order
    for (;;) {
        const bool canRun = sp > 0 && ncand == 0;
        const unsigned runMask = __ballot_sync(0xffffffffu, canRun);
        const unsigned pendMask = __ballot_sync(0xffffffffu, ncand > 0);
        if ((runMask | pendMask) == 0) break;
        if (pendMask != 0 && (__popc(pendMask) >= exactBatch || runMask == 0)) {
            if (ncand > 0) {
                const double ddx = dx, ddy = dy, ddz = dz;
                for (int c = 0; c < ncand; c++) {
                    const int slot = c == 0 ? cand0 : (c == 1 ? cand1 : cand2);
                    double t;
                    bool h;
                    if (triE) {
                        h = triHitExactPre(odx, ody, odz, ddx, ddy, ddz, triE, slot, &t);
                    } else {
                        const float4 a = tris[3 * slot], b = tris[3 * slot + 1], cc = tris[3 * slot + 2];
                        h = triHitExact(odx, ody, odz, ddx, ddy, ddz, a, b, cc, &t);
                    }
                    if (h && best > t) {
                        best = t;
                        bestf = __double2float_rn(t);
                        hit = slot;
                    }
                }
                ncand = 0;
            }
            continue;
        }
        if (!canRun) continue;
        const int code = stack[--sp];
        if (code < 0) {
            const int lc = ~code;
            const int first = lc >> 2, cnt = lc & 3;
            for (int i = 0; i < cnt; i++) {
                const int slot = first + i;
                const float4 a = tris[3 * slot], b = tris[3 * slot + 1], c = tris[3 * slot + 2];
                tests++;
                if (!triMayHit(ox, oy, oz, dx, dy, dz, a, b, c, bestf)) continue;
                if (ncand == 0) cand0 = slot; else if (ncand == 1) cand1 = slot; else cand2 = slot;
                ncand++;
            }
            continue;
        }
        visits++;
        const QNode* nd = (sTop != nullptr && code < kTopNodes) ? sTop + code : nodes + code;
        const float hd = bestf;
        float tmin[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float tmax[4] = {hd, hd, hd, hd};
        const float o3[3] = {ox, oy, oz};
        const float i3[3] = {idx, idy, idz};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float4 lo = nd->bmin[d];
            const float4 hi = nd->bmax[d];
            const bool neg = (sgnBits >> d) & 1;
            const float4 nearB = neg ? hi : lo;
            const float4 farB = neg ? lo : hi;
            const float nb[4] = {nearB.x, nearB.y, nearB.z, nearB.w};
            const float fb[4] = {farB.x, farB.y, farB.z, farB.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float t0 = __fmul_rn(__fsub_rn(nb[k], o3[d]), i3[d]);
                const float t1 = __fmul_rn(__fsub_rn(fb[k], o3[d]), i3[d]);
                tmin[k] = tmin[k] > t0 ? tmin[k] : t0;
                tmax[k] = tmax[k] < t1 ? tmax[k] : t1;
            }
        }
        int hitMask = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) hitMask |= (tmax[k] >= tmin[k]) ? (1 << k) : 0;
        if (hitMask != 0) {
            const int4 ch = nd->child;
            const int meta = nd->meta.x;
            const int a0 = meta & 3, a1 = (meta >> 2) & 3, a2 = (meta >> 4) & 3;
            const int sepMask = (((sgnBits >> a0) & 1) << 2) | (((sgnBits >> a1) & 1) << 1) | ((sgnBits >> a2) & 1);
            int ord = orderTab[hitMask * 8 + sepMask];
            const int c4[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                if (ord & 0x04) break;
                stack[sp++] = c4[ord & 0x03];
                ord >>= 4;
            }
        }
    }
    *bestOut = best;
    if (nodeVisits) *nodeVisits += visits;
    if (triTests) *triTests += tests;
    return hit;
}

// Resumable form of traverseExactWarp for persistent kernels: one lane's
// traversal state, advanced by the whole warp (warpTravRun) until enough
// lanes have finished that the kernel can give them new rays. Each lane
// still performs the reference's operations in the reference's order (the
// same box tests against the same (float)best, the same strict updates), so
// the hits equal traverseExact's.
struct WarpTrav {
    int stack[kStackSize];
    int sp;
    double best;
    float bestf;
    int hit;
    int cand0, cand1, cand2, ncand;
    double odx, ody, odz;
    float dx, dy, dz;
    float ox, oy, oz, idx, idy, idz;
    int sgnBits;

    __device__ __forceinline__ void begin(int rootCode, double x, double y, double z, float ux, float uy, float uz) {
        odx = x; ody = y; odz = z;
        dx = ux; dy = uy; dz = uz;
        ox = __double2float_rn(x); oy = __double2float_rn(y); oz = __double2float_rn(z);
        idx = ux == 0.0f ? 1.0e20f : __frcp_rn(ux);
        idy = uy == 0.0f ? 1.0e20f : __frcp_rn(uy);
        idz = uz == 0.0f ? 1.0e20f : __frcp_rn(uz);
        const int sx = idx > 0.0f ? 0 : 1, sy = idy > 0.0f ? 0 : 1, sz = idz > 0.0f ? 0 : 1;
        sgnBits = sx | (sy << 1) | (sz << 2);
        sp = 0;
        stack[sp++] = rootCode;
        best = kInfty;
        bestf = 1.0e20f;
        hit = -1;
        ncand = 0;
    }
    __device__ __forceinline__ bool done() const { return sp == 0 && ncand == 0; }
};

// Advances the traversals of the lanes in `live` until every one of them is
// done or at least minDone of them are (lanes outside `live` only take part
// in the warp votes). All 32 lanes call it.
__device__ __forceinline__ void warpTravRun(WarpTrav& s, bool live, int minDone, const QNode* __restrict__ nodes,
                                            const float4* __restrict__ tris, const int* orderTab, const QNode* sTop,
                                            int* nodeVisits, int* triTests, const double* __restrict__ triE = nullptr,
                                            int exactBatch = kExactBatch) {
    for (;;) {
        const bool canRun = live && s.sp > 0 && s.ncand == 0;
        const unsigned runMask = __ballot_sync(0xffffffffu, canRun);
        const unsigned pendMask = __ballot_sync(0xffffffffu, live && s.ncand > 0);
        if ((runMask | pendMask) == 0) break;
        if (__popc(__ballot_sync(0xffffffffu, live && s.done())) >= minDone) break;
        if (pendMask != 0 && (__popc(pendMask) >= exactBatch || runMask == 0)) {
            if (live && s.ncand > 0) {
                const double ddx = s.dx, ddy = s.dy, ddz = s.dz;
                for (int c = 0; c < s.ncand; c++) {
                    const int slot = c == 0 ? s.cand0 : (c == 1 ? s.cand1 : s.cand2);
                    double t;
                    bool h;
                    if (triE) {
                        h = triHitExactPre(s.odx, s.ody, s.odz, ddx, ddy, ddz, triE, slot, &t);
                    } else {
                        const float4 a = tris[3 * slot], b = tris[3 * slot + 1], cc = tris[3 * slot + 2];
                        h = triHitExact(s.odx, s.ody, s.odz, ddx, ddy, ddz, a, b, cc, &t);
                    }
                    if (h && s.best > t) {
                        s.best = t;
                        s.bestf = __double2float_rn(t);
                        s.hit = slot;
                    }
                }
                s.ncand = 0;
            }
            continue;
        }
        if (!canRun) continue;
        const int code = s.stack[--s.sp];
        if (code < 0) {
            const int lc = ~code;
            const int first = lc >> 2, cnt = lc & 3;
            for (int i = 0; i < cnt; i++) {
                const int slot = first + i;
                const float4 a = tris[3 * slot], b = tris[3 * slot + 1], c = tris[3 * slot + 2];
                (*triTests)++;
                if (!triMayHit(s.ox, s.oy, s.oz, s.dx, s.dy, s.dz, a, b, c, s.bestf)) continue;
                if (s.ncand == 0) s.cand0 = slot; else if (s.ncand == 1) s.cand1 = slot; else s.cand2 = slot;
                s.ncand++;
            }
            continue;
        }
        (*nodeVisits)++;
        const QNode* nd = (sTop != nullptr && code < kTopNodes) ? sTop + code : nodes + code;
        const float hd = s.bestf;
        float tmin[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float tmax[4] = {hd, hd, hd, hd};
        const float o3[3] = {s.ox, s.oy, s.oz};
        const float i3[3] = {s.idx, s.idy, s.idz};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float4 lo = nd->bmin[d];
            const float4 hi = nd->bmax[d];
            const bool neg = (s.sgnBits >> d) & 1;
            const float4 nearB = neg ? hi : lo;
            const float4 farB = neg ? lo : hi;
            const float nb[4] = {nearB.x, nearB.y, nearB.z, nearB.w};
            const float fb[4] = {farB.x, farB.y, farB.z, farB.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float t0 = __fmul_rn(__fsub_rn(nb[k], o3[d]), i3[d]);
                const float t1 = __fmul_rn(__fsub_rn(fb[k], o3[d]), i3[d]);
                tmin[k] = tmin[k] > t0 ? tmin[k] : t0;
                tmax[k] = tmax[k] < t1 ? tmax[k] : t1;
            }
        }
        int hitMask = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) hitMask |= (tmax[k] >= tmin[k]) ? (1 << k) : 0;
        if (hitMask != 0) {
            const int4 ch = nd->child;
            const int meta = nd->meta.x;
            const int a0 = meta & 3, a1 = (meta >> 2) & 3, a2 = (meta >> 4) & 3;
            const int sepMask = (((s.sgnBits >> a0) & 1) << 2) | (((s.sgnBits >> a1) & 1) << 1) | ((s.sgnBits >> a2) & 1);
            int ord = orderTab[hitMask * 8 + sepMask];
            const int c4[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                if (ord & 0x04) break;
                s.stack[s.sp++] = c4[ord & 0x03];
                ord >>= 4;
            }
        }
    }
}

// Hit record of the exact path: position o + t*d and the triangle's
// normal cross(p1-p0, p2-p0).normalized() computed in double like
// Triangle::normal (triangle.cc:45-47), rounded to float.
__device__ inline void hitPosition(double ox, double oy, double oz, float dx, float dy, float dz, double t, double* p) {
    p[0] = __dadd_rn(ox, __dmul_rn((double)dx, t));
    p[1] = __dadd_rn(oy, __dmul_rn((double)dy, t));
    p[2] = __dadd_rn(oz, __dmul_rn((double)dz, t));
}

__device__ inline f3 triNormal(const float4& a, const float4& b, const float4& c) {
    const double e1x = (double)b.x - a.x, e1y = (double)b.y - a.y, e1z = (double)b.z - a.z;
    const double e2x = (double)c.x - a.x, e2y = (double)c.y - a.y, e2z = (double)c.z - a.z;
    const double cx = __dsub_rn(__dmul_rn(e1y, e2z), __dmul_rn(e1z, e2y));
    const double cy = __dsub_rn(__dmul_rn(e1z, e2x), __dmul_rn(e1x, e2z));
    const double cz = __dsub_rn(__dmul_rn(e1x, e2y), __dmul_rn(e1y, e2x));
    const double nn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)), __dmul_rn(cz, cz)));
    const double inv = __drcp_rn(__dadd_rn(nn, kEps));
    return {__double2float_rn(__dmul_rn(cx, inv)), __double2float_rn(__dmul_rn(cy, inv)), __double2float_rn(__dmul_rn(cz, inv))};
}

// The same normal in FP32 for the shading kernels (direction sampling and
// orientation only; pppm_intersect reports the double-derived normal).
__device__ inline f3 triNormalF(const float4& a, const float4& b, const float4& c) {
    const f3 e1 = {b.x - a.x, b.y - a.y, b.z - a.z}, e2 = {c.x - a.x, c.y - a.y, c.z - a.z};
    return normalized(cross(e1, e2));
}

__device__ inline void hitRecord(double ox, double oy, double oz, float dx, float dy, float dz, double t, const float4& a,
                                 const float4& b, const float4& c, f3* pos, f3* nrm) {
    double p[3];
    hitPosition(ox, oy, oz, dx, dy, dz, t, p);
    pos->x = __double2float_rn(p[0]);
    pos->y = __double2float_rn(p[1]);
    pos->z = __double2float_rn(p[2]);
    *nrm = triNormal(a, b, c);
}

// ------------------------------------------------------------------ hashing
// HashGrid::hash (hash_grid_detail.h:60-63): 32-bit wrapping products,
// XOR, unsigned modulo.
__host__ __device__ inline uint32_t refHash(int ix, int iy, int iz, uint32_t size) {
    const uint32_t h = ((uint32_t)ix * 73856093u) ^ ((uint32_t)iy * 19349663u) ^ ((uint32_t)iz * 83492791u);
    return h % size;
}

// Octahedral normal packing (2 x 16-bit) for photon records.
__device__ inline uint32_t packNormal(f3 n) {
    const float l1 = fabsf(n.x) + fabsf(n.y) + fabsf(n.z) + 1e-20f;
    float u = n.x / l1, v = n.y / l1;
    if (n.z < 0.0f) {
        const float pu = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        const float pv = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = pu; v = pv;
    }
    const uint32_t qu = (uint32_t)__float2int_rn((fminf(fmaxf(u, -1.0f), 1.0f) * 0.5f + 0.5f) * 65535.0f);
    const uint32_t qv = (uint32_t)__float2int_rn((fminf(fmaxf(v, -1.0f), 1.0f) * 0.5f + 0.5f) * 65535.0f);
    return qu | (qv << 16);
}
__device__ inline f3 unpackNormal(uint32_t p) {
    const float u = (float)(p & 0xffffu) / 65535.0f * 2.0f - 1.0f;
    const float v = (float)(p >> 16) / 65535.0f * 2.0f - 1.0f;
    f3 n = {u, v, 1.0f - fabsf(u) - fabsf(v)};
    if (n.z < 0.0f) {
        const float ox = n.x;
        n.x = (1.0f - fabsf(n.y)) * (ox >= 0.0f ? 1.0f : -1.0f);
        n.y = (1.0f - fabsf(ox)) * (n.y >= 0.0f ? 1.0f : -1.0f);
    }
    return normalized(n);
}

// ------------------------------------------------------------------ sampling
// sampler::onHemisphere (sampler.cc:17-32)
__device__ inline f3 onHemisphere(f3 w, float r1, float r2) {
    f3 u = fabsf(w.x) > 1e-12f ? cross(mk(0.f, 1.f, 0.f), w) : cross(mk(1.f, 0.f, 0.f), w);
    u = normalized(u);
    const f3 v = cross(w, u);
    float st, ct;
    sincosf(2.0f * kPiF * r1, &st, &ct);
    const float z2s = sqrtf(r2);
    return normalized(u * (ct * z2s) + v * (st * z2s) + w * sqrtf(1.0f - r2));
}

// checkTotalReflection (reflectance.h:7-34) with the fixed IOR 1.5
// (common.h:16); the caller decides `into` as its reference code does.
struct FresnelSplit {
    f3 rdir, tdir;
    float Re, Tr;
    bool total;
};
__device__ inline FresnelSplit fresnelSplit(f3 in, f3 normal, bool into) {
    FresnelSplit s;
    const f3 on = into ? normal : -normal;
    s.rdir = reflect(in, normal);
    const float nnt = into ? (1.0f / 1.5f) : 1.5f;
    const float ddn = dot(in, on);
    const float cos2t = 1.0f - nnt * nnt * (1.0f - ddn * ddn);
    s.total = cos2t < 0.0f;
    if (s.total) {
        s.tdir = {0.f, 0.f, 0.f};
        s.Re = 1.0f;
        s.Tr = 0.0f;
        return s;
    }
    s.tdir = normalized(in * nnt - normal * (into ? 1.0f : -1.0f) * (ddn * nnt + sqrtf(cos2t)));
    const float R0 = 0.04f;  // ((1.5-1)/(1.5+1))^2
    const float c = 1.0f - (into ? -ddn : dot(s.tdir, -on));
    s.Re = R0 + (1.0f - R0) * (c * c * c * c * c);
    s.Tr = 1.0f - s.Re;
    return s;
}

// BSDF::sample dispatch (brdf.cc:23-142, reflectance.h:7-34). `normal` is
// whatever the calling reference code passes (oriented in tracePhotons,
// geometric in radiance). u1, u2 are the two draws as 32-bit integers
// (rand = u * 2^-32). Returns the pdf written by the reference (1.0 where it
// leaves the caller's initial value).
__device__ inline float bsdfSample(const DevMaterial& m, f3 in, f3 normal, uint32_t u1, uint32_t u2, f3* out) {
    const int t = m.type & 0x0f;
    const float r1 = u32ToFloat(u1), r2 = u32ToFloat(u2);
    if (t == 0x01) {  // Lambertian
        const f3 on = dot(in, normal) < 0.0f ? normal : -normal;
        *out = onHemisphere(on, r1, r2);
        return 1.0f;
    }
    if (t == 0x02) {  // specular
        const f3 on = dot(in, normal) < 0.0f ? normal : -normal;
        *out = reflect(in, on);
        return 1.0f;
    }
    if (t == 0x04) {  // Phong lobe
        const f3 on = dot(in, normal) < 0.0f ? normal : -normal;
        const f3 w = reflect(in, on);
        f3 u = fabsf(w.x) > 1e-12f ? cross(mk(0.f, 1.f, 0.f), w) : cross(mk(1.f, 0.f, 0.f), w);
        u = normalized(u);
        const f3 v = cross(w, u);
        const float theta = acosf(powf(r1, 1.0f / (m.phong_n + 1.0f)));
        const float phi = 2.0f * kPiF * r2;
        float sth, cth, sph, cph;
        sincosf(theta, &sth, &cth);
        sincosf(phi, &sph, &cph);
        *out = u * (sth * cph) + w * cth + v * (sth * sph);
        return 1.0f;
    }
    // refraction (brdf.cc:110-142): reflect with probability 0.25 + 0.5 *
    // REFLECT_PROBABILITY = 0.5, pdf p / Re or (1 - p) / Tr
    const FresnelSplit s = fresnelSplit(in, normal, !(dot(in, normal) >= 0.0f));
    if (s.total) { *out = s.rdir; return 1.0f; }
    const float p = 0.5f;
    if (u1 < 0x80000000u) { *out = s.rdir; return p / s.Re; }  // rand1 < 0.5, decided on the integer draw
    *out = s.tdir;
    return (1.0f - p) / s.Tr;
}

// Envmap::sampleFromDir (envmap.cc:11-17,47-60), nearest texel.
__device__ inline f3 envLookup(const EnvDev& e, f3 d) {
    if (e.w == 0) return {0.f, 0.f, 0.f};  // no environment map
    const float theta = acosf(fminf(fmaxf(d.y, -1.0f), 1.0f));
    float phi = atan2f(d.z, d.x);
    if (phi < 0.0f) phi += 2.0f * kPiF;
    int ix = (int)(phi / (2.0f * kPiF) * (float)e.w);
    int iy = (int)(theta / kPiF * (float)e.h);
    ix = min(max(ix, 0), e.w - 1);
    iy = min(max(iy, 0), e.h - 1);
    const float* p = e.rgb + 3 * ((size_t)iy * e.w + ix);
    return {p[0], p[1], p[2]};
}

// The cell draw of Envmap::samplePhoton (envmap.cc:62-79): the first cell
// whose CDF reaches the draw, then a uniform point of the cell in (u, v),
// i.e. uniform in solid angle (y is linear in v). *index = 4096 past the CDF.
template <class TapeT>
__device__ inline f3 envCellDraw(const EnvDev& e, TapeT& tp, int* index) {
    int lo = 0, hi = 4096;  // first index with cdf[i] >= r
    if constexpr (TapeT::kExact32) {
        const unsigned long long r = tp.popu();  // r * 2^-32 exactly: compare on integers
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(&e.ucdf[mid]) < r) lo = mid + 1; else hi = mid;
        }
    } else {
        const double r = tp.popd();
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(&e.cdf[mid]) < r) lo = mid + 1; else hi = mid;
        }
    }
    *index = lo;
    const int ix = lo % 64, iy = lo / 64;
    const float u = ((float)ix + tp.popf()) * (1.0f / 64.0f);
    const float v = ((float)iy + tp.popf()) * (1.0f / 64.0f);
    const float phi = u * kPiF * 2.0f;
    const float y = (1.0f - v) * 2.0f - 1.0f;
    const float sxz = sqrtf(fmaxf(0.0f, 1.0f - y * y));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return {sxz * cp, y, sxz * sp};
}

// The importance cell of a direction (the inverse of envCellDraw's map).
__device__ inline int envCellOf(f3 d) {
    float phi = atan2f(d.z, d.x);
    if (phi < 0.0f) phi += 2.0f * kPiF;
    const int ix = min(max((int)(phi * (64.0f / (2.0f * kPiF))), 0), 63);
    const int iy = min(max((int)((1.0f - d.y) * 0.5f * 64.0f), 0), 63);
    return iy * 64 + ix;
}

// A photon from the emissive triangles (no counterpart in the reference):
// the emitter by area (first CDF entry >= the draw), a uniform point of it
// (u = sqrt(r1): barycentrics (1 - u, u (1 - r2), u r2)), a cosine direction
// about its geometric normal (e1 x e2, the emitting side), and the flux
// Le * pi * total area / photons (area pdf 1 / A, direction pdf cos / pi).
// o: the point in double. Returns false past the last CDF entry.
template <class TapeT>
__device__ inline bool emitFromLights(const EnvDev& e, TapeT& tp, double* o, f3* dir, f3* flux, f3* normal) {
    int lo = 0, hi = e.numLights;
    if constexpr (TapeT::kExact32) {
        const unsigned long long r = tp.popu();
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(&e.lightUcdf[mid]) < r) lo = mid + 1; else hi = mid;
        }
    } else {
        const double r = tp.popd();
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(&e.lightCdf[mid]) < r) lo = mid + 1; else hi = mid;
        }
    }
    const bool ok = lo < e.numLights;
    const int k = min(lo, e.numLights - 1);
    const float r1 = tp.popf(), r2 = tp.popf();
    const float su = sqrtf(r1);
    const double b1 = (double)(su * (1.0f - r2)), b2 = (double)(su * r2);
    const float4 p0 = e.lightTri[3 * k], e1 = e.lightTri[3 * k + 1], e2 = e.lightTri[3 * k + 2];
    o[0] = (double)p0.x + b1 * (double)e1.x + b2 * (double)e2.x;
    o[1] = (double)p0.y + b1 * (double)e1.y + b2 * (double)e2.y;
    o[2] = (double)p0.z + b1 * (double)e1.z + b2 * (double)e2.z;
    const f3 n = normalized(cross(mk(e1.x, e1.y, e1.z), mk(e2.x, e2.y, e2.z)));
    const float a0 = tp.popf(), a1 = tp.popf();
    *dir = onHemisphere(n, a0, a1);
    *normal = n;
    const float* le = e.lightLe + 3 * k;
    *flux = mk(le[0], le[1], le[2]) * e.lightFluxScale;
    return ok;
}

// Envmap::samplePhoton (envmap.cc:62-86) followed by the cosine hemisphere
// draw of tracePhotons (ppm_probabilistic.cc:137-144). The CDF inversion is
// std::lower_bound over the double CDF, done in double. Returns false when
// the draw lies past the last CDF entry, where the reference indexes _pdf
// out of bounds. emitDir: the sampled env direction (photon origin is
// 50 * emitDir); dir: the first ray direction.
template <class TapeT>
__device__ inline bool emitPhoton(const EnvDev& e, TapeT& tp, double numPhotons, f3* emitDir, f3* dir, f3* flux,
                                  bool inOrder = false) {
    int index;
    const f3 d = envCellDraw(e, tp, &index);
    *flux = envLookup(e, d) * __ldg(&e.fluxScale[min(index, 4095)]);
    *emitDir = d;
    // onHemisphere(normalLight, &nextDir, rseq.pop(), rseq.pop()) in
    // tracePhotons: the reference build evaluates these arguments right to
    // left, so the first number drawn becomes r2 and the second r1. The
    // subsurface photon pass draws r1 then r2 in separate statements.
    const float a0 = tp.popf();
    const float a1 = tp.popf();
    *dir = inOrder ? onHemisphere(-d, a0, a1) : onHemisphere(-d, a1, a0);
    (void)numPhotons;
    return index < 4096;
}

}  // namespace pppm
