// Dipole BSSRDF (Jensen et al.) and the hierarchical irradiance sum of the
// reference's SubsurfaceIntegrator, shared by the stage kernels and the eye
// pass.
//
// Rd(d^2) follows DipoleBSSRDF::operator() (bssrdf.cc:92-104) in FP32 except
// for the reference's fast_exp (vector3d.cc:11-16), whose result depends on
// the truncation (int)(1512775 * y + 1072632447): that integer is formed
// with one double FMA (the product is exact in double, so one rounding of
// the sum equals the reference's), which keeps the approximation's
// staircase identical. The octree (built on the host with the reference's
// splits, host_build.cc) is stored in preorder with skip links, so each
// query walks it without a stack in the reference's recursion order.
#pragma once

#include "pppm_device.cuh"

namespace pppm {

struct OctNodeDev {
    float4 posArea;  // pos, area
    float4 iradSkip; // irad, skip index (int bits)
    float4 bminLeaf; // bbox min, leaf flag (int bits)
    float4 bmax;     // bbox max
};

// Octree of one pass's irradiance points.
struct OctView {
    const OctNodeDev* nodes;
    int numNodes;
    float maxError;  // 0.05 in the render (ppm_probabilistic.cc:84)
};

// fast_exp(y) of the reference for a float argument, formed in double:
// (float) of the double whose high word is (int)(1512775 y + 1072632447).
__device__ __forceinline__ float fastExpRefD(float y) {
    const int hi = __double2int_rz(__fma_rn(1512775.0, (double)y, 1072632447.0));
    return (float)__hiloint2double(hi, 0);
}

// The same function in 64-bit integer arithmetic, for |y| <= 700 (every
// argument of the dipole: y = -sigma_tr d <= 0); other arguments return
// false. With y = M 2^-k (M the 24-bit significand), S = 1512775 y +
// 1072632447 is n + f exactly; its double rounding moves it up to n + 1
// only when the distance to n + 1 is at most half a unit in the last place
// of S, 2^(L - 53) with L = floor(log2 n), ties going to n + 1 (its
// significand is even). The double (hi, 0) is then narrowed to float by
// hand: its 20 significand bits fit, exponents below the float range give
// denormals rounded to nearest even.
__host__ __device__ inline bool fastExpRefInt(float y, float* out) {
    uint32_t b;
#ifdef __CUDA_ARCH__
    b = __float_as_uint(y);
#else
    __builtin_memcpy(&b, &y, 4);
#endif
    const uint32_t ex = (b >> 23) & 0xffu, man = b & 0x7fffffu;
    const bool neg = (b >> 31) != 0;
    // |y| <= 700: exponent field at most 136 (700 < 2^10)
    if (ex > 136 || (ex == 136 && man > 0x2f0000u)) return false;  // 0x2f0000: 700 = 1.3671875 * 2^9
    constexpr int64_t kC = 1072632447;
    int64_t hi;
    if (ex == 0 && man == 0) {
        hi = kC;
    } else {
        const uint64_t M = ex ? (uint64_t)(man | 0x800000u) : (uint64_t)man;
        const int k = ex ? 150 - (int)ex : 149;  // y = M 2^-k, k >= 14
        const uint64_t P = 1512775ull * M;        // < 2^45
        const uint64_t q = k >= 64 ? 0 : P >> k;
        const uint64_t r = k >= 64 ? P : P & ((1ull << k) - 1);
        if (r == 0) {
            hi = neg ? kC - (int64_t)q : kC + (int64_t)q;
        } else {
            // S in (n, n + 1): n = C + q (y > 0) or C - q - 1 (y < 0), n >= 2^23
            const int64_t n = neg ? kC - (int64_t)q - 1 : kC + (int64_t)q;
#ifdef __CUDA_ARCH__
            const int L = 63 - __clzll(n);
#else
            const int L = 63 - __builtin_clzll((unsigned long long)n);
#endif
            const int t = k + L - 53;
            bool up;
            if (t < 0) {
                up = false;  // the distance to n + 1 is at least 2^-k > 2^t
            } else if (neg) {
                // distance r 2^-k <= 2^(t - k)
                up = t >= 45 || r <= (1ull << t);
            } else {
                // distance (2^k - r) 2^-k; k >= 64 leaves it above 2^(k-1) > 2^t
                up = k < 64 && ((1ull << k) - r) <= (1ull << t);
            }
            hi = n + (up ? 1 : 0);
        }
    }
    // hi in (0, 2^31): a positive finite double with exponent field Ed
    const uint32_t h = (uint32_t)hi;
    const int Ed = (int)(h >> 20);
    const uint32_t m20 = h & 0xfffffu;
    const int Ef = Ed - 896;  // float exponent field (1023 - 127)
    uint32_t fb;
    if (Ef >= 255) {
        fb = 0x7f800000u;  // above the float range: +inf
    } else if (Ef >= 1) {
        fb = ((uint32_t)Ef << 23) | (m20 << 3);
    } else {
        // denormal: (2^20 + m20) 2^(Ed - 894) units of 2^-149
        const uint64_t v = (1ull << 20) | m20;
        const int sh = 894 - Ed;
        if (sh <= 0) {
            fb = (uint32_t)(v << -sh);
        } else if (sh > 22) {
            fb = 0;  // below half the smallest denormal (v < 2^21)
        } else {
            uint64_t mq = v >> sh;
            const uint64_t rem = v & ((1ull << sh) - 1), half = 1ull << (sh - 1);
            if (rem > half || (rem == half && (mq & 1))) mq++;
            fb = (uint32_t)mq;
        }
    }
#ifdef __CUDA_ARCH__
    *out = __uint_as_float(fb);
#else
    __builtin_memcpy(out, &fb, 4);
#endif
    return true;
}

__device__ __forceinline__ float fastExpRef(float y) {
    float v;
    return fastExpRefInt(y, &v) ? v : fastExpRefD(y);
}

__device__ __forceinline__ f3 dipoleRd(const DipoleDev& m, float d2) {
    const float d2s = d2 / m.scale;
    float out[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float dpos = sqrtf(d2s + m.zpos[c] * m.zpos[c]);
        const float dneg = sqrtf(d2s + m.zneg[c] * m.zneg[c]);
        const float dpos3 = dpos * dpos * dpos, dneg3 = dneg * dneg * dneg;
        const float posTerm = m.zpos[c] * (dpos * m.sigma_tr[c] + 1.0f) * fastExpRef(-m.sigma_tr[c] * dpos);
        const float negTerm = m.zneg[c] * (dneg * m.sigma_tr[c] + 1.0f) * fastExpRef(-m.sigma_tr[c] * dneg);
        const float r = (m.alphap[c] * (posTerm * dneg3 - negTerm * dpos3)) /
                        ((4.0f * kPiF) * m.sigma_tr[c] * dpos3 * dneg3);
        // Vector3D::clamp(ret / scale^2, 0, INFTY) = max(0, min(v, 1e20)) with
        // std::min/std::max argument order: NaN -> 0, +inf -> 1e20
        float v = r / (m.scale * m.scale);
        v = (1.0e20f < v) ? 1.0e20f : v;
        out[c] = (0.0f < v) ? v : 0.0f;
    }
    return {out[0], out[1], out[2]};
}

// Octree::iradSubsurfaceRec (subsurface_integrator.cc:151-167) for one query:
// a node is taken whole when it is a leaf or when area / d^2 < maxError and
// the query lies outside its box; otherwise its children are visited.
__device__ __forceinline__ f3 octreeSum(const OctView& o, const DipoleDev& m, float px, float py, float pz,
                                        int* visited) {
    f3 sum = {0.f, 0.f, 0.f};
    int i = 0;
    int v = 0;
    while (i < o.numNodes) {
        v++;
        const float4 pa = __ldg(&o.nodes[i].posArea);
        const float4 bl = __ldg(&o.nodes[i].bminLeaf);
        const float dx = pa.x - px, dy = pa.y - py, dz = pa.z - pz;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float dw = pa.w / d2;
        bool take = __float_as_int(bl.w) != 0;
        if (!take && dw < o.maxError) {
            const float4 bx = __ldg(&o.nodes[i].bmax);
            const bool inside = bl.x <= px && px <= bx.x && bl.y <= py && py <= bx.y && bl.z <= pz && pz <= bx.z;
            take = !inside;
        }
        const float4 is = __ldg(&o.nodes[i].iradSkip);
        if (take) {
            const f3 rd = dipoleRd(m, d2);
            sum.x += rd.x * is.x * pa.w;
            sum.y += rd.y * is.y * pa.w;
            sum.z += rd.z * is.z * pa.w;
            i = max(__float_as_int(is.w), i + 1);  // skip > i for a well-formed tree
        } else {
            i = i + 1;  // first child in preorder
        }
    }
    if (visited) *visited += v;
    return sum;
}

// SubsurfaceIntegrator::irradiance (subsurface_integrator.cc:234-238).
__device__ __forceinline__ f3 subsurfaceIrradiance(const OctView& o, const DipoleDev& m, float px, float py, float pz,
                                                   int* visited) {
    const f3 s = octreeSum(o, m, px, py, pz, visited);
    return {m.coeff * s.x, m.coeff * s.y, m.coeff * s.z};
}

}  // namespace pppm
