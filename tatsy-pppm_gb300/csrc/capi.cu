// C-ABI entry points: lifetime, staging, scene, env map and stage queries.
#include <cmath>
#include <cstring>
#include <memory>
#include <new>

#include "context.h"
#include "host_build.h"

namespace pppm {

bool isDevicePtr(const void* p) {
    if (p == nullptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int stageIn(pppm_ctx* c, const void* src, size_t bytes, int slot, const void** out) {
    if (bytes == 0 || isDevicePtr(src)) {
        *out = src;
        return PPPM_OK;
    }
    PPPM_CUDA(c, c->stage[slot].ensure(bytes));
    PPPM_CUDA(c, cudaMemcpyAsync(c->stage[slot].p, src, bytes, cudaMemcpyHostToDevice, c->stream));
    *out = c->stage[slot].p;
    return PPPM_OK;
}

int stageOut(pppm_ctx* c, void* dst, size_t bytes, int slot, void** out) {
    if (dst == nullptr) {
        *out = nullptr;
        return PPPM_OK;
    }
    if (bytes == 0 || isDevicePtr(dst)) {
        *out = dst;
        return PPPM_OK;
    }
    PPPM_CUDA(c, c->stage[slot].ensure(bytes));
    *out = c->stage[slot].p;
    return PPPM_OK;
}

int finishOut(pppm_ctx* c, void* dst, const void* staged, size_t bytes) {
    if (dst == nullptr || dst == staged || bytes == 0) return PPPM_OK;
    PPPM_CUDA(c, cudaMemcpyAsync(dst, staged, bytes, cudaMemcpyDeviceToHost, c->stream));
    return PPPM_OK;
}

DipoleDev dipoleFrom(const pppm_material& mat) {
    DipoleDev d;
    std::memset(&d, 0, sizeof(d));
    // BSSRDFBase::Fdr (bssrdf.cc:33-42) and the DipoleBSSRDF ctor
    // (bssrdf.cc:48-63) in double
    const double eta = mat.eta, eta2 = eta * eta, eta3 = eta2 * eta;
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

static DevMaterial toDevMaterial(const pppm_material& m) {
    DevMaterial d;
    std::memset(&d, 0, sizeof(d));
    d.type = m.type | (m.has_bssrdf ? PPPM_BSDF_BSSRDF : 0);
    for (int k = 0; k < 3; k++) d.refl[k] = m.refl[k];
    d.phong_n = m.phong_n;
    d.roulette = std::fmax(m.refl[0], std::fmax(m.refl[1], m.refl[2]));
    d.rr_photon = ((double)m.refl[0] + (double)m.refl[1] + (double)m.refl[2]) / 3.0;
    // integer forms of the draw comparisons (x * 2^-32 is exact in double)
    d.rrCeil = (unsigned long long)std::ceil(d.rr_photon * 4294967296.0);
    d.roulFloor = (unsigned long long)std::floor((double)d.roulette * 4294967296.0);
    d.invRr = (float)(1.0 / d.rr_photon);
    if (m.has_bssrdf) d.dip = dipoleFrom(m);
    return d;
}

int envFluxScale(pppm_ctx* c, double numPhotons) {
    if (c->envScaleFor == numPhotons) return PPPM_OK;
    // Envmap::samplePhoton: area / (pdf * numPhotons) (envmap.cc:80-83)
    const double area = ((double)((unsigned)c->envW * (unsigned)c->envH)) / (4.0 * 3.14159265358979323846 * 64 * 64);
    std::vector<float> s(4096);
    for (int i = 0; i < 4096; i++) s[i] = (float)(area / (c->envPdf[i] * numPhotons));
    PPPM_CUDA(c, cudaMemcpy(c->envScaleD.p, s.data(), 4096 * 4, cudaMemcpyHostToDevice));
    c->envScaleFor = numPhotons;
    return PPPM_OK;
}

}  // namespace pppm

using namespace pppm;

extern "C" {

int pppm_create(int device, pppm_ctx** out) {
    if (!out) return PPPM_E_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return PPPM_E_CUDA;
    }
    pppm_ctx* c = new (std::nothrow) pppm_ctx();
    if (!c) return PPPM_E_CAPACITY;
    c->device = device;
    // the main stream (photon pass, grid, gather: the critical path of a
    // pass) outranks the side stream's eye trace when both have blocks
    // waiting for an SM
    int leastPrio = 0, greatestPrio = 0;
    if (cudaSetDevice(device) != cudaSuccess || cudaDeviceGetStreamPriorityRange(&leastPrio, &greatestPrio) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, greatestPrio) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return PPPM_E_CUDA;
    }
    for (auto& e : c->ev) cudaEventCreate(&e);
    // the octree build's short level kernels on the aux stream interleave
    // with the photon pass instead of waiting behind it
    cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, greatestPrio);
    cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, leastPrio);
    cudaEventCreateWithFlags(&c->rs.sss.done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->rs.sss.octDone, cudaEventDisableTiming);
    {
        XorShift x;
        x.seed(0u);
        for (int k = 0; k < 4; k++) c->poissonRng[k] = x.s[k];
    }
    *out = c;
    return PPPM_OK;
}

int pppm_destroy(pppm_ctx* c) {
    if (!c) return PPPM_E_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->graphEvents) cudaEventDestroy(e);
    if (c->rs.sss.done) cudaEventDestroy(c->rs.sss.done);
    if (c->rs.sss.octDone) cudaEventDestroy(c->rs.sss.octDone);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    cudaStreamDestroy(c->stream);
    delete c;
    return PPPM_OK;
}

const char* pppm_last_error(const pppm_ctx* c) { return c ? c->err.c_str() : "null context"; }

int pppm_sync(pppm_ctx* c) {
    if (!c) return PPPM_E_ARG;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    PPPM_CUDA(c, cudaGetLastError());
    return PPPM_OK;
}

void* pppm_stream(pppm_ctx* c) { return c ? (void*)c->stream : nullptr; }

int pppm_scene_set(pppm_ctx* c, const float* tri, int64_t ntri, const int32_t* matId, const pppm_material* mats,
                   int32_t nmat) {
    if (!c || ntri < 0 || (ntri > 0 && (!tri || !matId)) || nmat < 0 || (nmat > 0 && !mats))
        return fail(c, PPPM_E_ARG, "scene_set: bad arguments");
    if (isDevicePtr(tri) || isDevicePtr(matId) || isDevicePtr(mats))
        return fail(c, PPPM_E_ARG, "scene_set: scene arrays must be host memory");
    for (int i = 0; i < nmat; i++) {
        const int t = mats[i].type;
        if (t != PPPM_BSDF_LAMBERTIAN && t != PPPM_BSDF_SPECULAR && t != PPPM_BSDF_PHONG && t != PPPM_BSDF_REFRACTION)
            return fail(c, PPPM_E_ARG, "scene_set: material type must be one BSDF bit");
    }
    for (int64_t i = 0; i < ntri; i++)
        if (matId[i] < 0 || matId[i] >= nmat) return fail(c, PPPM_E_ARG, "scene_set: material id out of range");
    cudaSetDevice(c->device);
    HostBvh bvh;
    std::string err;
    if (!buildQbvh(tri, ntri, &bvh, &err)) return fail(c, PPPM_E_CAPACITY, "scene_set: " + err);
    c->hasScene = false;
    c->rs.active = false;
    const size_t nodeBytes = bvh.nodes.size() * sizeof(QNode);
    PPPM_CUDA(c, c->nodes.ensure(nodeBytes));
    if (nodeBytes) {
        std::vector<QNode> dn(bvh.nodes.size());
        for (size_t k = 0; k < dn.size(); k++) {
            const HostQNode& h = bvh.nodes[k];
            for (int d = 0; d < 3; d++) {
                dn[k].bmin[d] = make_float4(h.bmin[d][0], h.bmin[d][1], h.bmin[d][2], h.bmin[d][3]);
                dn[k].bmax[d] = make_float4(h.bmax[d][0], h.bmax[d][1], h.bmax[d][2], h.bmax[d][3]);
            }
            dn[k].child = make_int4(h.child[0], h.child[1], h.child[2], h.child[3]);
            dn[k].meta = make_int4(h.sep, 0, 0, 0);
        }
        PPPM_CUDA(c, cudaMemcpy(c->nodes.p, dn.data(), nodeBytes, cudaMemcpyHostToDevice));
    }
    PPPM_CUDA(c, c->tris.ensure(bvh.tris.size() * sizeof(float)));
    if (!bvh.tris.empty())
        PPPM_CUDA(c, cudaMemcpy(c->tris.p, bvh.tris.data(), bvh.tris.size() * sizeof(float), cudaMemcpyHostToDevice));
    {
        // per slot the exact test's double vertex and edges, with the
        // device's operations: p0 = (double)a, e1 = (double)b - p0, e2 = (double)c - p0
        const size_t slots = bvh.tris.size() / 12;
        std::unique_ptr<double[]> te(new double[std::max<size_t>(slots, 1) * 10]);
        slotEdges(bvh.tris.data(), (int64_t)slots, te.get());
        PPPM_CUDA(c, c->triE.ensure(std::max<size_t>(slots, 1) * 10 * sizeof(double)));
        if (slots)
            PPPM_CUDA(c, cudaMemcpy(c->triE.p, te.get(), slots * 10 * sizeof(double), cudaMemcpyHostToDevice));
    }
    PPPM_CUDA(c, c->matId.ensure((size_t)ntri * 4));
    if (ntri) PPPM_CUDA(c, cudaMemcpy(c->matId.p, matId, (size_t)ntri * 4, cudaMemcpyHostToDevice));
    std::vector<DevMaterial> dm(nmat);
    c->anyBssrdf = false;
    for (int i = 0; i < nmat; i++) {
        dm[i] = toDevMaterial(mats[i]);
        c->anyBssrdf |= mats[i].has_bssrdf != 0;
    }
    PPPM_CUDA(c, c->devMats.ensure(dm.size() * sizeof(DevMaterial)));
    if (nmat) PPPM_CUDA(c, cudaMemcpy(c->devMats.p, dm.data(), dm.size() * sizeof(DevMaterial), cudaMemcpyHostToDevice));
    c->mats.assign(mats, mats + nmat);
    c->lambertArea = 0.0;
    for (int64_t i = 0; i < ntri; i++) {
        if (mats[matId[i]].type != PPPM_BSDF_LAMBERTIAN) continue;
        const float* p = tri + 9 * i;
        const double e1[3] = {(double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2]};
        const double e2[3] = {(double)p[6] - p[0], (double)p[7] - p[1], (double)p[8] - p[2]};
        const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
        c->lambertArea += 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
    }
    c->hostTri.assign(tri, tri + 9 * ntri);
    c->hostMatId.assign(matId, matId + ntri);
    c->matEmit.assign((size_t)nmat * 3, 0.0f);
    c->numLights = 0;
    c->lightArea = 0.0;
    c->bssrdfTris.clear();
    c->bssrdfArea = 0.0;
    for (int64_t i = 0; i < ntri; i++) {
        if (!mats[matId[i]].has_bssrdf) continue;
        c->bssrdfTris.push_back(i);
        // Triangle::area: 0.5 |(p1 - p0) x (p2 - p1)| (triangle.cc:80-84)
        const float* p = tri + 9 * i;
        const double e1[3] = {(double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2]};
        const double e2[3] = {(double)p[6] - p[3], (double)p[7] - p[4], (double)p[8] - p[5]};
        const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
        c->bssrdfArea += 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
    }
    c->ntri = ntri;
    c->rootCode = bvh.rootCode;
    c->numNodes = (int)bvh.nodes.size();
    c->bvhDepth = bvh.depth;
    // BBox over all triangles (ppm_probabilistic.cc:50-54)
    for (int d = 0; d < 3; d++) { c->bbmin[d] = 1e20; c->bbmax[d] = -1e20; }
    for (int64_t i = 0; i < ntri * 3; i++)
        for (int d = 0; d < 3; d++) {
            const double v = tri[3 * i + d];
            c->bbmin[d] = v < c->bbmin[d] ? v : c->bbmin[d];
            c->bbmax[d] = v > c->bbmax[d] ? v : c->bbmax[d];
        }
    c->hasScene = true;
    return PPPM_OK;
}

static int uploadEnvTables(pppm_ctx* c);

int pppm_material_emission(pppm_ctx* c, int32_t mat_id, const float* rgb) {
    if (!c || !rgb) return fail(c, PPPM_E_ARG, "material_emission: bad arguments");
    if (!c->hasScene) return fail(c, PPPM_E_STATE, "material_emission: no scene");
    if (mat_id < 0 || (size_t)mat_id >= c->mats.size()) return fail(c, PPPM_E_ARG, "material_emission: bad material id");
    for (int k = 0; k < 3; k++)
        if (!(rgb[k] >= 0.0f) || !std::isfinite(rgb[k]))
            return fail(c, PPPM_E_ARG, "material_emission: emission must be finite and >= 0");
    cudaSetDevice(c->device);
    c->rs.active = false;
    for (int k = 0; k < 3; k++) c->matEmit[3 * (size_t)mat_id + k] = rgb[k];
    DevMaterial d = toDevMaterial(c->mats[(size_t)mat_id]);
    for (int k = 0; k < 3; k++) d.emit[k] = rgb[k];
    d.emissive = (rgb[0] > 0.0f || rgb[1] > 0.0f || rgb[2] > 0.0f) ? 1 : 0;
    PPPM_CUDA(c, cudaMemcpy(c->devMats.as<DevMaterial>() + mat_id, &d, sizeof(d), cudaMemcpyHostToDevice));
    // the emitter list: triangles of emissive materials in scene order, with
    // their areas 0.5 |e1 x e2| in double
    std::vector<float> tri;
    std::vector<float> le;
    std::vector<double> cdf;
    double total = 0.0;
    for (size_t i = 0; i < c->hostMatId.size(); i++) {
        const float* e = &c->matEmit[3 * (size_t)c->hostMatId[i]];
        if (!(e[0] > 0.0f || e[1] > 0.0f || e[2] > 0.0f)) continue;
        const float* p = &c->hostTri[9 * i];
        const float e1[3] = {p[3] - p[0], p[4] - p[1], p[5] - p[2]};
        const float e2[3] = {p[6] - p[0], p[7] - p[1], p[8] - p[2]};
        float idBits;
        std::memcpy(&idBits, &c->hostMatId[i], 4);
        const float row[12] = {p[0], p[1], p[2], idBits, e1[0], e1[1], e1[2], 0.0f, e2[0], e2[1], e2[2], 0.0f};
        tri.insert(tri.end(), row, row + 12);
        le.insert(le.end(), e, e + 3);
        const double cx = (double)e1[1] * e2[2] - (double)e1[2] * e2[1];
        const double cy = (double)e1[2] * e2[0] - (double)e1[0] * e2[2];
        const double cz = (double)e1[0] * e2[1] - (double)e1[1] * e2[0];
        total += 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
        cdf.push_back(total);
    }
    c->numLights = (int)cdf.size();
    c->lightArea = total;
    if (c->numLights == 0) return PPPM_OK;
    if (!(total > 0.0)) return fail(c, PPPM_E_ARG, "material_emission: the emitting triangles have zero area");
    std::vector<unsigned long long> u(cdf.size());
    for (size_t i = 0; i < cdf.size(); i++) {
        cdf[i] /= total;
        u[i] = (unsigned long long)std::floor(cdf[i] * 4294967296.0);
    }
    cdf.back() = 1.0;
    u.back() = 4294967296ull;  // every draw x < 2^32 selects an emitter
    PPPM_CUDA(c, c->lightTri.ensure(tri.size() * 4));
    PPPM_CUDA(c, c->lightLe.ensure(le.size() * 4));
    PPPM_CUDA(c, c->lightCdf.ensure(cdf.size() * 8));
    PPPM_CUDA(c, c->lightUcdf.ensure(u.size() * 8));
    PPPM_CUDA(c, cudaMemcpy(c->lightTri.p, tri.data(), tri.size() * 4, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(c->lightLe.p, le.data(), le.size() * 4, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(c->lightCdf.p, cdf.data(), cdf.size() * 8, cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(c->lightUcdf.p, u.data(), u.size() * 8, cudaMemcpyHostToDevice));
    return PPPM_OK;
}

int pppm_env_set(pppm_ctx* c, const float* rgb, int32_t w, int32_t h) {
    if (c && !rgb && w == 0 && h == 0) {
        // no environment map: rays that leave the scene see black (the
        // reference's default Envmap, scene.cc:11-12)
        c->hasEnv = false;
        c->envExponent = 2.0;
        return PPPM_OK;
    }
    if (!c || !rgb || w <= 0 || h <= 0) return fail(c, PPPM_E_ARG, "env_set: bad arguments");
    // The 64x64 importance map divides by the texel area of each cell
    // (envmap.cc:104-113); below 64 texels per axis that area is zero and
    // the reference aborts.
    if (w < 64 || h < 64) return fail(c, PPPM_E_UNDEFINED, "env_set: env map must be at least 64x64");
    if (isDevicePtr(rgb)) return fail(c, PPPM_E_ARG, "env_set: rgb must be host memory");
    cudaSetDevice(c->device);
    envImportance(rgb, w, h, &c->envPdf, &c->envCdf);
    const size_t bytes = (size_t)w * h * 3 * sizeof(float);
    PPPM_CUDA(c, c->envRgb.ensure(bytes));
    PPPM_CUDA(c, cudaMemcpy(c->envRgb.p, rgb, bytes, cudaMemcpyHostToDevice));
    c->envW = w;
    c->envH = h;
    const int r = uploadEnvTables(c);
    if (r != PPPM_OK) return r;
    c->hasEnv = true;
    c->envExponent = 2.0;
    return PPPM_OK;
}

int pppm_env_importance(pppm_ctx* c, double exponent) {
    if (!c || !(exponent >= 0.0 && exponent <= 8.0)) return fail(c, PPPM_E_ARG, "env_importance: bad exponent");
    if (!c->hasEnv) return fail(c, PPPM_E_STATE, "env_importance: no env map");
    if (exponent == c->envExponent) return PPPM_OK;
    cudaSetDevice(c->device);
    std::vector<float> rgb((size_t)c->envW * c->envH * 3);
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    PPPM_CUDA(c, cudaMemcpy(rgb.data(), c->envRgb.p, rgb.size() * sizeof(float), cudaMemcpyDeviceToHost));
    envImportance(rgb.data(), c->envW, c->envH, &c->envPdf, &c->envCdf, exponent);
    const int r = uploadEnvTables(c);
    if (r != PPPM_OK) return r;
    c->envExponent = exponent;
    return PPPM_OK;
}

// Device copies of the importance tables in c->envPdf / c->envCdf: pdf, cdf,
// the integer cdf of the draw comparison, and a fresh flux-scale table.
static int uploadEnvTables(pppm_ctx* c) {
    PPPM_CUDA(c, c->envPdfD.ensure(4096 * sizeof(double)));
    PPPM_CUDA(c, c->envCdfD.ensure(4096 * sizeof(double)));
    PPPM_CUDA(c, cudaMemcpy(c->envPdfD.p, c->envPdf.data(), 4096 * sizeof(double), cudaMemcpyHostToDevice));
    PPPM_CUDA(c, cudaMemcpy(c->envCdfD.p, c->envCdf.data(), 4096 * sizeof(double), cudaMemcpyHostToDevice));
    {
        // lower_bound(cdf, x * 2^-32) == first i with x <= floor(cdf[i] * 2^32)
        std::vector<unsigned long long> u(4096);
        for (int i = 0; i < 4096; i++) u[i] = (unsigned long long)std::floor(c->envCdf[i] * 4294967296.0);
        PPPM_CUDA(c, c->envUcdfD.ensure(4096 * 8));
        PPPM_CUDA(c, cudaMemcpy(c->envUcdfD.p, u.data(), 4096 * 8, cudaMemcpyHostToDevice));
    }
    PPPM_CUDA(c, c->envScaleD.ensure(4096 * 4));
    c->envScaleFor = -1.0;
    return PPPM_OK;
}

int pppm_env_tables(pppm_ctx* c, double* pdf, double* cdf) {
    if (!c || !pdf || !cdf) return fail(c, PPPM_E_ARG, "env_tables: bad arguments");
    if (!c->hasEnv) return fail(c, PPPM_E_STATE, "env_tables: no env map");
    std::memcpy(pdf, c->envPdf.data(), 4096 * sizeof(double));
    std::memcpy(cdf, c->envCdf.data(), 4096 * sizeof(double));
    return PPPM_OK;
}

int pppm_hdr_decode(const uint8_t* bytes, int64_t n, float* rgb, int64_t cap, int32_t* w, int32_t* h) {
    if (!bytes || n <= 0 || !w || !h) return PPPM_E_ARG;
    int ww = 0, hh = 0;
    const int r = decodeHdr(bytes, n, rgb, cap, &ww, &hh);
    *w = ww;
    *h = hh;
    if (r == -4) return PPPM_E_CAPACITY;
    return r == 0 ? PPPM_OK : PPPM_E_ARG;
}

int pppm_intersect(pppm_ctx* c, const float* rays, int64_t n, int32_t* tri, double* t, float* pos, float* nrm) {
    if (!c || n < 0 || (n > 0 && (!rays || !tri || !t))) return fail(c, PPPM_E_ARG, "intersect: bad arguments");
    if (!c->hasScene) return fail(c, PPPM_E_STATE, "intersect: no scene");
    if (n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    const void* dr;
    void *dtri, *dt, *dpos, *dnrm;
    int r;
    if ((r = stageIn(c, rays, (size_t)n * 24, 0, &dr))) return r;
    if ((r = stageOut(c, tri, (size_t)n * 4, 1, &dtri))) return r;
    if ((r = stageOut(c, t, (size_t)n * 8, 2, &dt))) return r;
    if ((r = stageOut(c, pos, (size_t)n * 12, 3, &dpos))) return r;
    if ((r = stageOut(c, nrm, (size_t)n * 12, 4, &dnrm))) return r;
    PPPM_CUDA(c, launchIntersect(sceneView(c), (const float*)dr, n, (int32_t*)dtri, (double*)dt, (float*)dpos,
                                 (float*)dnrm, c->stream, true));
    const bool host = dr != rays || dtri != tri || dt != t || (pos && dpos != pos) || (nrm && dnrm != nrm);
    if ((r = finishOut(c, tri, dtri, (size_t)n * 4))) return r;
    if ((r = finishOut(c, t, dt, (size_t)n * 8))) return r;
    if ((r = finishOut(c, pos, dpos, (size_t)n * 12))) return r;
    if ((r = finishOut(c, nrm, dnrm, (size_t)n * 12))) return r;
    if (host) PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_env_lookup(pppm_ctx* c, const float* dirs, int64_t n, float* rgb) {
    if (!c || n < 0 || (n > 0 && (!dirs || !rgb))) return fail(c, PPPM_E_ARG, "env_lookup: bad arguments");
    if (!c->hasEnv) return fail(c, PPPM_E_STATE, "env_lookup: no env map");
    if (n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    const void* dd;
    void* dout;
    int r;
    if ((r = stageIn(c, dirs, (size_t)n * 12, 0, &dd))) return r;
    if ((r = stageOut(c, rgb, (size_t)n * 12, 1, &dout))) return r;
    PPPM_CUDA(c, launchEnvLookup(envView(c), (const float*)dd, n, (float*)dout, c->stream));
    if ((r = finishOut(c, rgb, dout, (size_t)n * 12))) return r;
    if (dd != dirs || dout != rgb) PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_emit_photons(pppm_ctx* c, const double* tapes, int64_t n, int64_t numPhotons, float* pos, float* dir,
                      float* flux, int32_t* defined) {
    if (!c || n < 0 || numPhotons < 1 || (n > 0 && (!tapes || !pos || !dir || !flux || !defined)))
        return fail(c, PPPM_E_ARG, "emit_photons: bad arguments");
    if (!c->hasEnv) return fail(c, PPPM_E_STATE, "emit_photons: no env map");
    if (n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    const void* dt;
    void *dp, *dd, *df, *dk;
    int r;
    if ((r = stageIn(c, tapes, (size_t)n * 40, 0, &dt))) return r;
    if ((r = stageOut(c, pos, (size_t)n * 12, 1, &dp))) return r;
    if ((r = stageOut(c, dir, (size_t)n * 12, 2, &dd))) return r;
    if ((r = stageOut(c, flux, (size_t)n * 12, 3, &df))) return r;
    if ((r = stageOut(c, defined, (size_t)n * 4, 4, &dk))) return r;
    int rs_;
    if ((rs_ = envFluxScale(c, (double)numPhotons))) return rs_;
    PPPM_CUDA(c, launchEmit(envView(c), (const double*)dt, n, (double)numPhotons, (float*)dp, (float*)dd, (float*)df,
                            (int*)dk, c->stream));
    if ((r = finishOut(c, pos, dp, (size_t)n * 12))) return r;
    if ((r = finishOut(c, dir, dd, (size_t)n * 12))) return r;
    if ((r = finishOut(c, flux, df, (size_t)n * 12))) return r;
    if ((r = finishOut(c, defined, dk, (size_t)n * 4))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_hash_points(pppm_ctx* c, const float* pts, int64_t n, int32_t size, double scale, const double* bbmin,
                     uint32_t* out) {
    if (!c || n < 0 || size <= 0 || !bbmin || (n > 0 && (!pts || !out)))
        return fail(c, PPPM_E_ARG, "hash_points: bad arguments");
    if (n == 0) return PPPM_OK;
    cudaSetDevice(c->device);
    const void* dp;
    void* dout;
    int r;
    if ((r = stageIn(c, pts, (size_t)n * 12, 0, &dp))) return r;
    if ((r = stageOut(c, out, (size_t)n * 4, 1, &dout))) return r;
    PPPM_CUDA(c, launchHashPoints((const float*)dp, n, (uint32_t)size, scale, bbmin, (uint32_t*)dout, c->stream));
    if ((r = finishOut(c, out, dout, (size_t)n * 4))) return r;
    if (dp != pts || dout != out) PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

}  // extern "C"
