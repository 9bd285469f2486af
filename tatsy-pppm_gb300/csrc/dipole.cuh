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

// fast_exp(y) of the reference for a float argument.
__device__ __forceinline__ float fastExpRef(float y) {
    const int hi = __double2int_rz(__fma_rn(1512775.0, (double)y, 1072632447.0));
    return (float)__hiloint2double(hi, 0);
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
