// Stage entry points of the dipole BSSRDF: Rd tables and the hierarchical
// irradiance over injected irradiance points (octree built on the host).
#include <cmath>
#include <cstring>

#include "context.h"
#include "dipole.cuh"
#include "host_build.h"

namespace pppm {

static_assert(sizeof(OctNodeDev) == sizeof(HostOctNode), "octree node layout");

namespace {

__global__ void kDipoleRd(DipoleDev m, const float* __restrict__ d2, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 r = dipoleRd(m, d2[i]);
    out[3 * i] = r.x;
    out[3 * i + 1] = r.y;
    out[3 * i + 2] = r.z;
}

__global__ void kDipoleIrradiance(OctView o, DipoleDev m, const float* __restrict__ q, int64_t nq,
                                  float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const f3 s = subsurfaceIrradiance(o, m, q[3 * i], q[3 * i + 1], q[3 * i + 2], nullptr);
    out[3 * i] = s.x;
    out[3 * i + 1] = s.y;
    out[3 * i + 2] = s.z;
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
    const OctView ov{c->stageRec.as<OctNodeDev>(), (int)nodes.size(), (float)maxError};
    kDipoleIrradiance<<<(unsigned)((m + 127) / 128), 128, 0, c->stream>>>(ov, dipoleFrom(*mat), (const float*)dq, m,
                                                                          (float*)dout);
    PPPM_CUDA(c, cudaGetLastError());
    if ((r = finishOut(c, rgb, dout, (size_t)m * 12))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

}  // extern "C"
