// Dipole BSSRDF (Jensen et al.) and the hierarchical irradiance sum of the
// reference's SubsurfaceIntegrator.
//
// Rd(d^2) follows DipoleBSSRDF::operator() (bssrdf.cc:92-104) in FP32 except
// for the reference's fast_exp (vector3d.cc:11-16), whose result depends on
// the truncation (int)(1512775 * y + 1072632447): that integer is formed
// with one double FMA (the product is exact in double, so one rounding of
// the sum equals the reference's), which keeps the approximation's
// staircase identical. The octree (built on the host with the reference's
// splits, host_build.cc) is stored in preorder with skip links, so each
// query walks it without a stack in the reference's recursion order.
#include <cmath>
#include <cstring>

#include "context.h"
#include "host_build.h"

namespace pppm {

struct OctNodeDev {
    float4 posArea;  // pos, area
    float4 iradSkip; // irad, skip index (int bits)
    float4 bminLeaf; // bbox min, leaf flag (int bits)
    float4 bmax;     // bbox max
};
static_assert(sizeof(OctNodeDev) == sizeof(HostOctNode), "octree node layout");

struct DipoleDev {
    float sigma_tr[3], alphap[3], zpos[3], zneg[3];
    float scale;
    float coeff;  // (1/pi) * (1 - Fdr) (subsurface_integrator.cc:236-237)
};

namespace {

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

__global__ void kDipoleRd(DipoleDev m, const float* __restrict__ d2, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 r = dipoleRd(m, d2[i]);
    out[3 * i] = r.x;
    out[3 * i + 1] = r.y;
    out[3 * i + 2] = r.z;
}

// Octree::iradSubsurfaceRec (subsurface_integrator.cc:151-167) for one query:
// a node is taken whole when it is a leaf or when area / d^2 < maxError and
// the query lies outside its box; otherwise its children are visited.
__device__ __forceinline__ f3 octreeSum(const OctNodeDev* __restrict__ nodes, int numNodes, const DipoleDev& m,
                                        float maxError, float px, float py, float pz, int* visited) {
    f3 sum = {0.f, 0.f, 0.f};
    int i = 0;
    int v = 0;
    while (i < numNodes) {
        v++;
        const float4 pa = __ldg(&nodes[i].posArea);
        const float4 bl = __ldg(&nodes[i].bminLeaf);
        const float dx = pa.x - px, dy = pa.y - py, dz = pa.z - pz;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float dw = pa.w / d2;
        bool take = __float_as_int(bl.w) != 0;
        if (!take && dw < maxError) {
            const float4 bx = __ldg(&nodes[i].bmax);
            const bool inside = bl.x <= px && px <= bx.x && bl.y <= py && py <= bx.y && bl.z <= pz && pz <= bx.z;
            take = !inside;
        }
        const float4 is = __ldg(&nodes[i].iradSkip);
        if (take) {
            const f3 rd = dipoleRd(m, d2);
            sum.x += rd.x * is.x * pa.w;
            sum.y += rd.y * is.y * pa.w;
            sum.z += rd.z * is.z * pa.w;
            i = __float_as_int(is.w);
        } else {
            i = i + 1;  // first child in preorder
        }
    }
    if (visited) *visited += v;
    return sum;
}

__global__ void kDipoleIrradiance(const OctNodeDev* __restrict__ nodes, int numNodes, DipoleDev m, float maxError,
                                  const float* __restrict__ q, int64_t nq, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const f3 s = octreeSum(nodes, numNodes, m, maxError, q[3 * i], q[3 * i + 1], q[3 * i + 2], nullptr);
    out[3 * i] = m.coeff * s.x;
    out[3 * i + 1] = m.coeff * s.y;
    out[3 * i + 2] = m.coeff * s.z;
}

DipoleDev dipoleFrom(const pppm_material& mat) {
    DipoleDev d;
    const double eta = mat.eta, eta2 = eta * eta, eta3 = eta2 * eta;
    // BSSRDFBase::Fdr (bssrdf.cc:33-42)
    const double fdr = eta >= 1.0 ? (-1.439 + 0.7099 * eta + 0.6681 * eta2 + 0.0636 * eta3) / eta2
                                  : (-0.4399 * eta3 + 0.7099 * eta2 - 0.3319 * eta + 0.0636) / eta3;
    const double A = (1.0 + fdr) / (1.0 - fdr);
    for (int k = 0; k < 3; k++) {
        const double sa = mat.sigma_a[k], ss = mat.sigmap_s[k], st = sa + ss;
        d.sigma_tr[k] = (float)std::sqrt(3.0 * sa * st);
        d.alphap[k] = (float)(ss / st);
        const double zp = 1.0 / st;
        d.zpos[k] = (float)zp;
        d.zneg[k] = (float)(zp * (1.0 + (4.0 / 3.0) * A));
    }
    d.scale = mat.scale;
    d.coeff = (float)((1.0 / 3.14159265358979323846) * (1.0 - fdr));
    return d;
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
    // irradiance points to host doubles for the octree build
    std::vector<float> hp((size_t)n * 10);
    if (n > 0) {
        if (isDevicePtr(ipts)) {
            PPPM_CUDA(c, cudaMemcpy(hp.data(), ipts, hp.size() * 4, cudaMemcpyDeviceToHost));
        } else {
            std::memcpy(hp.data(), ipts, hp.size() * 4);
        }
    }
    std::vector<double> pd(hp.begin(), hp.end());
    std::vector<HostOctNode> nodes;
    std::string err;
    if (n > 0 && !buildOctree(pd.data(), n, &nodes, &err)) return fail(c, PPPM_E_UNDEFINED, "dipole_irradiance: " + err);
    PPPM_CUDA(c, c->stageRec.ensure(std::max<size_t>(nodes.size(), 1) * sizeof(OctNodeDev)));
    if (!nodes.empty())
        PPPM_CUDA(c, cudaMemcpy(c->stageRec.p, nodes.data(), nodes.size() * sizeof(OctNodeDev), cudaMemcpyHostToDevice));
    const void* dq;
    void* dout;
    int r;
    if ((r = stageIn(c, queries, (size_t)m * 12, 0, &dq))) return r;
    if ((r = stageOut(c, rgb, (size_t)m * 12, 1, &dout))) return r;
    kDipoleIrradiance<<<(unsigned)((m + 127) / 128), 128, 0, c->stream>>>(
        c->stageRec.as<OctNodeDev>(), (int)nodes.size(), dipoleFrom(*mat), (float)maxError, (const float*)dq, m,
        (float*)dout);
    PPPM_CUDA(c, cudaGetLastError());
    if ((r = finishOut(c, rgb, dout, (size_t)m * 12))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

}  // extern "C"
