// Closest-hit queries and reference-hash bucket selection.
#include "context.h"

namespace pppm {

template <bool kPrefilter>
__global__ void __launch_bounds__(128) kIntersect(SceneView sc, const float* __restrict__ rays, int64_t n,
                                                   int32_t* __restrict__ triOut, double* __restrict__ tOut,
                                                   float* __restrict__ posOut, float* __restrict__ nrmOut) {
    __shared__ int order[128];
    __shared__ QNode sTop[kTopNodes];
    loadOrderTable(order);
    loadTopNodes(sTop, sc.nodes, sc.numNodes);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;  // all lanes traverse together (warp-cooperative)
    const float* r = rays + 6 * (valid ? i : 0);
    const double ox = r[0], oy = r[1], oz = r[2];
    const float dx = r[3], dy = r[4], dz = r[5];
    double best;
    int slot;
    if (kPrefilter) {
        slot = traverseExactWarp(sc.nodes, sc.tris, sc.rootCode, valid, ox, oy, oz, dx, dy, dz, order, sTop, &best,
                                 nullptr, nullptr, sc.triE);
    } else {
        if (!valid) return;
        slot = traverseExact<false>(sc.nodes, sc.tris, sc.rootCode, ox, oy, oz, dx, dy, dz, order, &best, nullptr,
                                    nullptr, sTop);
    }
    if (!valid) return;
    int id = -1;
    if (slot >= 0) {
        const float4 a = sc.tris[3 * slot], b = sc.tris[3 * slot + 1], c = sc.tris[3 * slot + 2];
        id = __float_as_int(a.w);
        if (posOut || nrmOut) {
            f3 p, nn;
            hitRecord(ox, oy, oz, dx, dy, dz, best, a, b, c, &p, &nn);
            if (posOut) { posOut[3 * i] = p.x; posOut[3 * i + 1] = p.y; posOut[3 * i + 2] = p.z; }
            if (nrmOut) { nrmOut[3 * i] = nn.x; nrmOut[3 * i + 1] = nn.y; nrmOut[3 * i + 2] = nn.z; }
        }
    } else {
        if (posOut) { posOut[3 * i] = 0.f; posOut[3 * i + 1] = 0.f; posOut[3 * i + 2] = 0.f; }
        if (nrmOut) { nrmOut[3 * i] = 0.f; nrmOut[3 * i + 1] = 0.f; nrmOut[3 * i + 2] = 0.f; }
    }
    triOut[i] = id;
    tOut[i] = best;
}

cudaError_t launchIntersect(const SceneView& s, const float* rays, int64_t n, int32_t* tri, double* t, float* pos,
                            float* nrm, cudaStream_t st, bool prefilter) {
    if (n <= 0) return cudaSuccess;
    const int bs = 128;
    const int64_t grid = (n + bs - 1) / bs;
    if (prefilter) kIntersect<true><<<(unsigned)grid, bs, 0, st>>>(s, rays, n, tri, t, pos, nrm);
    else kIntersect<false><<<(unsigned)grid, bs, 0, st>>>(s, rays, n, tri, t, pos, nrm);
    return cudaGetLastError();
}

// HashGrid::operator[] (hash_grid_detail.h:66-72): cell = |(int)((p - bbmin)
// * scale)| per axis in double, then the reference hash.
__global__ void kHashPoints(const float* __restrict__ pts, int64_t n, uint32_t size, double scale, double mx, double my,
                            double mz, uint32_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double bx = __dmul_rn(__dsub_rn((double)pts[3 * i], mx), scale);
    const double by = __dmul_rn(__dsub_rn((double)pts[3 * i + 1], my), scale);
    const double bz = __dmul_rn(__dsub_rn((double)pts[3 * i + 2], mz), scale);
    const int ix = abs(__double2int_rz(bx)), iy = abs(__double2int_rz(by)), iz = abs(__double2int_rz(bz));
    out[i] = refHash(ix, iy, iz, size);
}

cudaError_t launchHashPoints(const float* pts, int64_t n, uint32_t size, double scale, const double* bbmin, uint32_t* out,
                             cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int bs = 256;
    kHashPoints<<<(unsigned)((n + bs - 1) / bs), bs, 0, st>>>(pts, n, size, scale, bbmin[0], bbmin[1], bbmin[2], out);
    return cudaGetLastError();
}

}  // namespace pppm

namespace pppm {

__global__ void kEnvLookup(EnvDev env, const float* __restrict__ dirs, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 c = envLookup(env, mk(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
    out[3 * i] = c.x;
    out[3 * i + 1] = c.y;
    out[3 * i + 2] = c.z;
}

__global__ void kEmit(EnvDev env, const double* __restrict__ tapes, int64_t n, double numPhotons, float* __restrict__ pos,
                      float* __restrict__ dir, float* __restrict__ flux, int* __restrict__ ok) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ArrayTape t{tapes + 5 * i, 0};
    f3 e, d, f;
    ok[i] = emitPhoton(env, t, numPhotons, &e, &d, &f) ? 1 : 0;
    pos[3 * i] = 50.0f * e.x;
    pos[3 * i + 1] = 50.0f * e.y;
    pos[3 * i + 2] = 50.0f * e.z;
    dir[3 * i] = d.x;
    dir[3 * i + 1] = d.y;
    dir[3 * i + 2] = d.z;
    flux[3 * i] = f.x;
    flux[3 * i + 1] = f.y;
    flux[3 * i + 2] = f.z;
}

cudaError_t launchEnvLookup(const EnvDev& env, const float* dirs, int64_t n, float* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    kEnvLookup<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(env, dirs, n, out);
    return cudaGetLastError();
}

cudaError_t launchEmit(const EnvDev& env, const double* tapes, int64_t n, double numPhotons, float* pos, float* dir,
                       float* flux, int* ok, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    kEmit<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(env, tapes, n, numPhotons, pos, dir, flux, ok);
    return cudaGetLastError();
}

}  // namespace pppm
