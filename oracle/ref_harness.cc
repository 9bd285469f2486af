// Test-only harness around the UNMODIFIED tatsy-pppm reference library.
//
// This file is part of the oracle (test infrastructure). It is linked with
// the reference's own object files (oracle/Makefile) and is called through
// ctypes by tests/golden/make_golden.py and by the CPU tests that pin the
// C++ port (oracle/pppm_port.cc) against the reference. Nothing in the
// product links or loads it.
//
// The stage methods of the reference are private; the harness reaches them
// by redefining `private` before including the reference headers, so no
// reference file is edited. Every function below calls reference code; the
// harness adds only marshalling between flat arrays and reference objects.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <algorithm>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <queue>
#include <stack>
#include <string>
#include <vector>
#include <xmmintrin.h>
#include <immintrin.h>
#include <omp.h>

#define private public
#define protected public
#include "renderer.h"
#include "random.h"
#include "random_queue.h"
#include "sampler.h"
#include "hash_grid.h"
#include "kdtree.h"
#include "subsurface_integrator.h"
#undef private
#undef protected

// `enabler` is declared (common.h:41, size.h:6) but never defined by the
// reference; the default template argument of clamp()/Size<> needs a symbol.
void* enabler = nullptr;

// time(NULL) as seen by subsurface_integrator.cc (oracle/fake_time.h).
static time_t gFakeTime = 0;
extern "C" time_t rh_fake_time(time_t* t) {
    if (t) *t = gFakeTime;
    return gFakeTime;
}

namespace {

// Triangle soup geometry: lets the harness add an arbitrary triangle list
// through the reference's own Scene::add<T> (scene.h:38-50).
class TriSoup : public IGeometry {
public:
    std::vector<Triangle> tris;
    bool intersect(const Ray&, Hitpoint*) const override { return false; }
    double area() const override { return 0.0; }
    IGeometry* clone() const override { return new TriSoup(*this); }
    std::vector<Triangle> triangulate() const override { return tris; }
};

struct HarnessScene {
    Scene scene;
};

// Material record shared with the Python side (same layout as pppm_material
// in include/pppm_c.h).
struct Mat {
    int32_t type;        // BsdfType bitmask without the BSSRDF bit
    int32_t has_bssrdf;  // 1 -> attach DipoleBSSRDF
    float refl[3];
    float phong_n;
    float sigma_a[3];
    float sigmap_s[3];
    float eta;
    float scale;
};

BSDF makeBsdf(const Mat& m) {
    const Vector3D refl(m.refl[0], m.refl[1], m.refl[2]);
    BSDF b;
    switch (m.type) {
    case BSDF_TYPE_LAMBERTIAN_BRDF: b = LambertianBRDF::factory(refl); break;
    case BSDF_TYPE_SPECULAR_BRDF:   b = SpecularBRDF::factory(refl); break;
    case BSDF_TYPE_PHONG_BRDF:      b = PhongBRDF::factory(refl, m.phong_n); break;
    case BSDF_TYPE_REFRACTION:      b = RefractionBSDF::factory(refl); break;
    default: std::abort();
    }
    if (m.has_bssrdf) {
        BSSRDF s = DipoleBSSRDF::factory(Vector3D(m.sigma_a[0], m.sigma_a[1], m.sigma_a[2]),
                                         Vector3D(m.sigmap_s[0], m.sigmap_s[1], m.sigmap_s[2]),
                                         m.eta, m.scale);
        b.setBssrdf(s);
    }
    return b;
}

Vector3D v3(const float* p) { return Vector3D(p[0], p[1], p[2]); }
void put3(double* o, const Vector3D& v) { o[0] = v.x(); o[1] = v.y(); o[2] = v.z(); }

}  // namespace

extern "C" {

int rh_num_threads() { return OMP_NUM_CORE; }

// ---------------------------------------------------------------- scene
void* rh_scene_create() { return new HarnessScene(); }
void rh_scene_destroy(void* s) { delete static_cast<HarnessScene*>(s); }

// Adds `ntri` triangles (9 floats each) sharing one material.
void rh_scene_add(void* s, const float* v9, int ntri, const Mat* m) {
    TriSoup soup;
    soup.tris.reserve(ntri);
    for (int i = 0; i < ntri; i++) {
        soup.tris.push_back(Triangle(v3(v9 + 9 * i), v3(v9 + 9 * i + 3), v3(v9 + 9 * i + 6)));
    }
    static_cast<HarnessScene*>(s)->scene.add(soup, makeBsdf(*m));
}

// Adds a PLY mesh through the reference loader (trimesh.cc:139-217).
int rh_scene_add_ply(void* s, const char* path, const Mat* m) {
    Trimesh mesh;
    mesh.load(path);
    static_cast<HarnessScene*>(s)->scene.add(mesh, makeBsdf(*m));
    return (int)mesh.numFaces();
}

void rh_scene_finalize(void* s) { static_cast<HarnessScene*>(s)->scene.setAccelerator(); }

// Loads a PLY through Trimesh::load (trimesh.cc:125-217) and places it the
// way the reference's demo driver does (main/appmain.cc:38-40): fitToBBox
// when fit != 0, scale(scaleAll) when scaleAll != 1, putOnPlane when
// onPlane != 0, then translate(move). Writes the double vertices and faces;
// returns the face count (vertex count in *nv), or -1 when a buffer is short.
int rh_mesh_place(const char* path, int fit, const double* bmin, const double* bmax, double scaleAll, int onPlane,
                  double planeDist, const double* planeN, const double* move, double* verts, int vcap, int* faces,
                  int fcap, int* nv) {
    Trimesh mesh;
    mesh.load(path);
    if (fit) mesh.fitToBBox(BBox(bmin[0], bmin[1], bmin[2], bmax[0], bmax[1], bmax[2]));
    if (scaleAll != 1.0) mesh.scale(scaleAll);
    if (onPlane) mesh.putOnPlane(Plane(planeDist, Vector3D(planeN[0], planeN[1], planeN[2])));
    mesh.translate(Vector3D(move[0], move[1], move[2]));
    *nv = (int)mesh.numVerts();
    if (mesh.numVerts() > vcap || mesh.numFaces() > fcap) return -1;
    for (int i = 0; i < (int)mesh.numVerts(); i++) {
        const Vector3D v = mesh.getVertex(i);
        verts[3 * i] = v.x();
        verts[3 * i + 1] = v.y();
        verts[3 * i + 2] = v.z();
    }
    const std::vector<Triplet> ids = mesh.getIndices();
    for (int i = 0; i < (int)ids.size(); i++)
        for (int k = 0; k < 3; k++) faces[3 * i + k] = ids[i][k];
    return (int)mesh.numFaces();
}

// Writes an RGB float image as Radiance HDR with the reference writer
// (image.cc:436-482) so the env map goes through its own RGBE round trip.
void rh_write_hdr(const char* path, const float* rgb, int w, int h) {
    Image img(w, h);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const float* p = rgb + 3 * (y * w + x);
            img.pixel(x, y) = Vector3D(p[0], p[1], p[2]);
        }
    img.save(path);
}

// Loads an HDR with the reference loader (image.cc:296-434) into doubles.
int rh_load_hdr(const char* path, double* rgb_out, int cap_pixels, int* w, int* h) {
    Image img;
    img.load(path);
    *w = img.width();
    *h = img.height();
    if ((int)(img.width() * img.height()) > cap_pixels) return -1;
    for (unsigned y = 0; y < img.height(); y++)
        for (unsigned x = 0; x < img.width(); x++) put3(rgb_out + 3 * (y * img.width() + x), img(x, y));
    return 0;
}

void rh_scene_set_envmap(void* s, const char* hdr_path) {
    Envmap env(hdr_path);
    static_cast<HarnessScene*>(s)->scene.setEnvmap(env);
}

// Envmap importance arrays (envmap.cc:88-163), 64*64 entries each.
void rh_envmap_tables(void* s, double* pdf, double* cdf) {
    const Envmap& e = static_cast<HarnessScene*>(s)->scene.envmap();
    for (size_t i = 0; i < e._pdf.size(); i++) { pdf[i] = e._pdf[i]; cdf[i] = e._cdf[i]; }
}

// Envmap::sampleFromDir (envmap.cc:47-60) for unit directions.
void rh_envmap_lookup(void* s, const double* dirs, int n, double* out) {
    const Envmap& e = static_cast<HarnessScene*>(s)->scene.envmap();
    for (int i = 0; i < n; i++) put3(out + 3 * i, e.sampleFromDir(Vector3D(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2])));
}

// Envmap::samplePhoton + sampler::onHemisphere on explicit random tapes
// (ppm_probabilistic.cc:137-144). tapes: n x 5 doubles.
void rh_emit(void* s, const double* tapes, int n, int numPhotons, double* pos, double* dir, double* flux) {
    const Envmap& e = static_cast<HarnessScene*>(s)->scene.envmap();
    for (int i = 0; i < n; i++) {
        RandomSequence rseq;
        rseq.resize(5);
        for (int k = 0; k < 5; k++) rseq.set(k, tapes[5 * i + k]);
        rseq.reset();
        const Photon ph = e.samplePhoton(rseq, numPhotons);
        Vector3D nextDir;
        sampler::onHemisphere(ph.normal(), &nextDir, rseq.pop(), rseq.pop());
        put3(pos + 3 * i, static_cast<Vector3D>(ph));
        put3(dir + 3 * i, nextDir);
        put3(flux + 3 * i, ph.flux());
    }
}

// ---------------------------------------------------------------- geometry
// Scene::intersect (scene.cc:40-47) for rays given as 6 floats (o, d).
void rh_intersect(void* s, const float* rays, int n, int32_t* tri, double* t, double* pos, double* nrm) {
    const Scene& sc = static_cast<HarnessScene*>(s)->scene;
    for (int i = 0; i < n; i++) {
        Ray ray(v3(rays + 6 * i), v3(rays + 6 * i + 3));
        Intersection isect;
        const bool hit = sc.intersect(ray, isect);
        tri[i] = hit ? isect.objectID() : -1;
        t[i] = isect.hitpoint().distance();
        put3(pos + 3 * i, isect.hitpoint().position());
        put3(nrm + 3 * i, isect.hitpoint().normal());
    }
}

// ---------------------------------------------------------------- RNG
void rh_xorshift(uint32_t seed, int n, uint32_t* out) {
    XorShift x(seed);
    for (int i = 0; i < n; i++) out[i] = x.next();
}

// Random::nextReal tape of n doubles (random.h:45-55).
void rh_xorshift_reals(uint32_t seed, int skip, int n, double* out) {
    XorShift x(seed);
    for (int i = 0; i < skip; i++) x.next();
    for (int i = 0; i < n; i++) out[i] = x.nextReal();
}

// ---------------------------------------------------------------- sampling / BSDF
void rh_on_hemisphere(const double* normals, const double* r, int n, double* out) {
    for (int i = 0; i < n; i++) {
        Vector3D d;
        sampler::onHemisphere(Vector3D(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]), &d, r[2 * i], r[2 * i + 1]);
        put3(out + 3 * i, d);
    }
}

// BSDF::sample for one material over n (in, normal, r1, r2) tuples.
void rh_bsdf_sample(const Mat* m, const double* in, const double* nrm, const double* r, int n, double* out, double* pdf) {
    BSDF b = makeBsdf(*m);
    for (int i = 0; i < n; i++) {
        Vector3D o;
        double p = 1.0;
        b.sample(Vector3D(in[3 * i], in[3 * i + 1], in[3 * i + 2]), Vector3D(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]),
                 r[2 * i], r[2 * i + 1], &o, &p);
        put3(out + 3 * i, o);
        pdf[i] = p;
    }
}

// PerspectiveCamera::getRay (perspective_camera.cc:42-46).
void rh_camera_rays(const double* eye, const double* dir, const double* up, double fov, int w, int h,
                    const double* pxy, int n, double* org, double* d) {
    PerspectiveCamera cam(Vector3D(eye[0], eye[1], eye[2]), Vector3D(dir[0], dir[1], dir[2]),
                          Vector3D(up[0], up[1], up[2]), fov, w, h, 1.0);
    for (int i = 0; i < n; i++) {
        Ray r = cam.getRay(pxy[2 * i], pxy[2 * i + 1]);
        put3(org + 3 * i, r.origin());
        put3(d + 3 * i, r.direction());
    }
}

// ---------------------------------------------------------------- hash grid
// HashGrid<int>::operator[] bucket index (hash_grid_detail.h:60-72).
void rh_hash_points(int hashSize, double scale, const double* bbmin, const double* bbmax, const float* pts, int n,
                    uint32_t* out) {
    HashGrid<int> g;
    g.init(hashSize, scale, BBox(Vector3D(bbmin[0], bbmin[1], bbmin[2]), Vector3D(bbmax[0], bbmax[1], bbmax[2])));
    for (int i = 0; i < n; i++) out[i] = (uint32_t)(&g[v3(pts + 3 * i)] - &g._data[0]);
}

// HashGrid<int>::add (hash_grid_detail.h:34-52): items inserted per bucket.
// Returns, for every bucket, the item ids in insertion order (CSR layout).
int rh_hash_add_boxes(int hashSize, double scale, const double* bbmin, const double* bbmax, const double* boxmin,
                      const double* boxmax, int n, int32_t* start, int32_t* items, int cap) {
    HashGrid<int> g;
    g.init(hashSize, scale, BBox(Vector3D(bbmin[0], bbmin[1], bbmin[2]), Vector3D(bbmax[0], bbmax[1], bbmax[2])));
    for (int i = 0; i < n; i++)
        g.add(i, Vector3D(boxmin[3 * i], boxmin[3 * i + 1], boxmin[3 * i + 2]),
              Vector3D(boxmax[3 * i], boxmax[3 * i + 1], boxmax[3 * i + 2]));
    int k = 0;
    for (int b = 0; b < hashSize; b++) {
        start[b] = k;
        for (int id : g._data[b]) {
            if (k >= cap) return -1;
            items[k++] = id;
        }
    }
    start[hashSize] = k;
    return k;
}

// ---------------------------------------------------------------- kNN
// PhotonMap::findKNN (photon_map.cc:24-26) with the reference's argument
// order. Photon ids travel in the (unused by the query) direction field.
// out_idx: m x cap ids in the reference's result order (farthest first).
int rh_knn(const float* ppos, int n, const float* q, int m, int numTargetPhotons, double targetRadius,
           int32_t* out_idx, int32_t* out_cnt, int cap) {
    std::vector<Photon> photons(n);
    for (int i = 0; i < n; i++) photons[i] = Photon(v3(ppos + 3 * i), Vector3D(), Vector3D(i, 0, 0), Vector3D());
    PhotonMap pm;
    pm.construct(photons);
    int overflow = 0;
    for (int j = 0; j < m; j++) {
        std::vector<Photon> res;
        pm.findKNN(Photon(v3(q + 3 * j), Vector3D(), Vector3D(), Vector3D()), &res, numTargetPhotons, targetRadius);
        out_cnt[j] = (int)res.size();
        for (size_t i = 0; i < res.size(); i++) {
            if ((int)i < cap) out_idx[j * cap + i] = (int32_t)res[i].direction().x();
            else overflow = 1;
        }
    }
    return overflow ? -1 : 0;
}

// KdTree<Photon>::knnSearch (kdtree_detail.h:88-132) with KnnQuery(type,
// epsilon, k) as given; ids travel in the direction field as in rh_knn.
int rh_kdtree_knn(const float* ppos, int n, const float* q, int m, int type, double epsilon, int k, int32_t* out_idx,
                  int32_t* out_cnt, int cap) {
    std::vector<Photon> photons(n);
    for (int i = 0; i < n; i++) photons[i] = Photon(v3(ppos + 3 * i), Vector3D(), Vector3D(i, 0, 0), Vector3D());
    KdTree<Photon> tree;
    tree.construct(photons);
    int overflow = 0;
    for (int j = 0; j < m; j++) {
        std::vector<Photon> res;
        tree.knnSearch(Photon(v3(q + 3 * j), Vector3D(), Vector3D(), Vector3D()), KnnQuery(type, epsilon, k), &res);
        out_cnt[j] = (int)res.size();
        for (size_t i = 0; i < res.size(); i++) {
            if ((int)i < cap) out_idx[j * cap + i] = (int32_t)res[i].direction().x();
            else overflow = 1;
        }
    }
    return overflow ? -1 : 0;
}

// ---------------------------------------------------------------- gather
// ProgressivePhotonMappingProb::radiance (ppm_probabilistic.cc:246-344) at
// bounce 0 for rays hitting Lambertian surfaces, with the photon map built
// from the given photons and the global radius forced to `radius`.
// Photon records: pos(3) flux(3) dir(3) normal(3) floats.
void rh_gather(void* s, const float* photons, int n, double radius, int gatherPhotons, const float* rays, int m,
               double* out) {
    const Scene& sc = static_cast<HarnessScene*>(s)->scene;
    std::vector<Photon> ph(n);
    for (int i = 0; i < n; i++) {
        const float* p = photons + 12 * i;
        ph[i] = Photon(v3(p), v3(p + 3), v3(p + 6), v3(p + 9));
    }
    ProgressivePhotonMappingProb ppm;
    ppm._photonMap.construct(ph);
    ppm._radius = radius;
    RenderParameters params(1000, 1, gatherPhotons, 16.0);
    for (int j = 0; j < m; j++) {
        RandomSequence rseq;
        rseq.resize(200);
        for (int k = 0; k < 200; k++) rseq.set(k, 0.5);
        rseq.reset();
        Ray ray(v3(rays + 6 * j), v3(rays + 6 * j + 3));
        put3(out + 3 * j, ppm.radiance(sc, ray, params, rseq, 0));
    }
}

// ---------------------------------------------------------------- whole pass
// Runs passes 1..npasses of ProgressivePhotonMappingProb::render's loop
// (ppm_probabilistic.cc:24-121) by calling the reference's own
// tracePhotons / traceRays and radius update, without the PNG side effects.
// accum: w*h*3 doubles of the linear buffer after the last pass (not divided
// by t). radii: radius used in each pass. photons_out (optional): the photon
// multiset of the last pass read back from the kd-tree, 12 doubles each.
struct PassJob {
    double eye[3], dir[3], up[3];
    double fov;
    int w, h;
    int photons;
    int gatherPhotons;
    double gatherRadius;
    int npasses;
    unsigned int sssTime;  // time(NULL) seen by pass t's subsurface photon map: sssTime + t - 1
    int sampler;           // rh_render_passes: 0 RANDOM_SAMPLER_PSEUDO_RANDOM, 1 RANDOM_SAMPLER_QUASI_MONTE_CARLO
};

static void collectKd(const KdTree<Photon>::KdTreeNode* node, std::vector<Photon>* out) {
    if (!node) return;
    out->push_back(node->point);
    collectKd(node->left, out);
    collectKd(node->right, out);
}

int rh_render_passes(void* s, const PassJob* job, double* accum, double* radii, double* photons_out, int photon_cap,
                     int* photon_count) {
    const Scene& sc = static_cast<HarnessScene*>(s)->scene;
    PerspectiveCamera cam(Vector3D(job->eye[0], job->eye[1], job->eye[2]), Vector3D(job->dir[0], job->dir[1], job->dir[2]),
                          Vector3D(job->up[0], job->up[1], job->up[2]), job->fov, job->w, job->h, 1.0);
    RenderParameters params(job->photons, job->npasses, job->gatherPhotons, job->gatherRadius);
    ProgressivePhotonMappingProb ppm;

    BBox bbox;
    for (int i = 0; i < (int)sc.numTriangles(); i++) bbox.merge(sc.getTriangle(i));
    ppm._radius = (bbox.posMax() - bbox.posMin()).norm() * 0.1;

    // subsurface set-up as render() does it (ppm_probabilistic.cc:33-47)
    bool enableBssrdf = false;
    double avgArea = 0.0;
    for (int i = 0; i < sc.numTriangles(); i++) {
        if (sc.getBsdf(i).type() & BSDF_TYPE_BSSRDF) {
            enableBssrdf = true;
            avgArea += sc.getTriangle(i).area();
        }
    }
    avgArea /= sc.numTriangles();
    double areaRadius = 0.0;
    if (enableBssrdf) {
        areaRadius = sqrt(avgArea) * 1.0;
        ppm._integrator = new SubsurfaceIntegrator();
    }

    // the samplers of render() (ppm_probabilistic.cc:58-73)
    RandomSampler* rs = new RandomSampler[OMP_NUM_CORE];
    for (int i = 0; i < OMP_NUM_CORE; i++)
        rs[i] = job->sampler == 1 ? Halton::generateSampler(200, true, i) : Random::generateSampler(i);
    Image buffer(job->w, job->h);
    buffer.fill(Vector3D(0.0, 0.0, 0.0));
    std::streambuf* old = std::cout.rdbuf(nullptr);  // silence progress output
    for (int t = 1; t <= job->npasses; t++) {
        radii[t - 1] = ppm._radius;
        if (enableBssrdf) {
            gFakeTime = (time_t)(job->sssTime + (unsigned int)(t - 1));
            ppm._integrator->initialize(sc, params, areaRadius, 0.05);
        }
        ppm.tracePhotons(sc, cam, params, rs);
        ppm.traceRays(&buffer, sc, cam, params, rs);
        ppm._radius = (t + 1.0) / (t + ProgressivePhotonMappingProb::ALPHA) * ppm._radius;
    }
    std::cout.rdbuf(old);
    for (int y = 0; y < job->h; y++)
        for (int x = 0; x < job->w; x++) put3(accum + 3 * (y * job->w + x), buffer(x, y));
    if (photons_out && photon_count) {
        std::vector<Photon> all;
        collectKd(&ppm._photonMap._kdtree._nodes[0], &all);
        *photon_count = (int)all.size();
        for (int i = 0; i < (int)all.size() && i < photon_cap; i++) {
            put3(photons_out + 12 * i, static_cast<Vector3D>(all[i]));
            put3(photons_out + 12 * i + 3, all[i].flux());
            put3(photons_out + 12 * i + 6, all[i].direction());
            put3(photons_out + 12 * i + 9, all[i].normal());
        }
    }
    delete[] rs;
    return 0;
}

// SubsurfaceIntegrator::buildPhotonMap (subsurface_integrator.cc:240-327)
// with time(NULL) = sssTime: the photon map's records (12 doubles each,
// read back from its kd-tree as rh_render_passes does).
int rh_sss_photons(void* s, int photons, unsigned int sssTime, double* out, int cap, int* count) {
    const Scene& sc = static_cast<HarnessScene*>(s)->scene;
    SubsurfaceIntegrator integ;
    gFakeTime = (time_t)sssTime;
    std::streambuf* old = std::cout.rdbuf(nullptr);
    integ.buildPhotonMap(sc, photons, 64);
    std::cout.rdbuf(old);
    std::vector<Photon> all;
    if (integ.photonMap._kdtree._nodes) collectKd(&integ.photonMap._kdtree._nodes[0], &all);
    *count = (int)all.size();
    for (int i = 0; i < (int)all.size() && i < cap; i++) {
        put3(out + 12 * i, static_cast<Vector3D>(all[i]));
        put3(out + 12 * i + 3, all[i].flux());
        put3(out + 12 * i + 6, all[i].direction());
        put3(out + 12 * i + 9, all[i].normal());
    }
    return 0;
}

// PathTracing::render (path_tracing.cc:23-127) with the pseudo-random
// sampler and without its PNG side effects: npasses samples per pixel, rows
// y to stream y % N, a 200-number tape per pixel (path_tracing.cc:82-90),
// bounceLimit 64. With a BSSRDF in the scene, sample t's subsurface photon
// streams see time(NULL) = sssTime + t - 1. accum: w*h*3 doubles with row
// y = camera row y (the reference's buffer holds pixel (x, y) at
// (x, H - 1 - y)).
int rh_path_trace(void* s, const PassJob* job, double* accum) {
    const Scene& sc = static_cast<HarnessScene*>(s)->scene;
    PerspectiveCamera cam(Vector3D(job->eye[0], job->eye[1], job->eye[2]), Vector3D(job->dir[0], job->dir[1], job->dir[2]),
                          Vector3D(job->up[0], job->up[1], job->up[2]), job->fov, job->w, job->h, 1.0);
    RenderParameters params(job->photons, job->npasses, job->gatherPhotons, job->gatherRadius);
    PathTracing pt;
    bool enableBssrdf = false;
    double avgArea = 0.0;
    for (int i = 0; i < sc.numTriangles(); i++) {
        if (sc.getBsdf(i).type() & BSDF_TYPE_BSSRDF) {
            enableBssrdf = true;
            avgArea += sc.getTriangle(i).area();
        }
    }
    avgArea /= sc.numTriangles();
    double areaRadius = 0.0;
    if (enableBssrdf) {
        areaRadius = sqrt(avgArea) * 1.0;
        pt._integrator = new SubsurfaceIntegrator();
    }
    RandomSampler* rs = new RandomSampler[OMP_NUM_CORE];
    for (int i = 0; i < OMP_NUM_CORE; i++) rs[i] = Random::generateSampler(i);
    const int w = job->w, h = job->h;
    const int taskPerThread = (h + OMP_NUM_CORE - 1) / OMP_NUM_CORE;
    std::vector<std::vector<int> > tasks(OMP_NUM_CORE);
    for (int y = 0; y < h; y++) tasks[y % OMP_NUM_CORE].push_back(y);
    Image buffer(w, h);
    buffer.fill(Vector3D(0.0, 0.0, 0.0));
    std::streambuf* old = std::cout.rdbuf(nullptr);
    for (int i = 0; i < job->npasses; i++) {
        if (enableBssrdf) {
            gFakeTime = (time_t)(job->sssTime + (unsigned int)i);
            pt._integrator->initialize(sc, params, areaRadius, 0.05);
        }
        for (int t = 0; t < taskPerThread; t++) {
#pragma omp parallel for
            for (int threadID = 0; threadID < OMP_NUM_CORE; threadID++) {
                RandomSequence rseq;
                if (t < (int)tasks[threadID].size()) {
                    const int y = tasks[threadID][t];
                    for (int x = 0; x < w; x++) {
                        rs[threadID].request(200, &rseq);
                        buffer.pixel(x, h - y - 1) += pt.executePathTracing(sc, cam, params, x, y, rseq);
                    }
                }
            }
        }
    }
    std::cout.rdbuf(old);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) put3(accum + 3 * (y * w + x), buffer(x, h - 1 - y));
    delete[] rs;
    return 0;
}

// ProgressivePhotonMapping (classic PPM, progressive_photon_mapping.cc:31-345)
// without its PNG side effects: render points, Halton samplers, then per
// pass traceRays (+ constructHashGrid) and tracePhotons, as render() does.
// image: per pixel (emission + flux / (pi r2)) * coeff, NOT divided by the
// pass count (row y = camera row y).
int rh_classic_passes(void* s, const PassJob* job, double* image) {
    const Scene& sc = static_cast<HarnessScene*>(s)->scene;
    PerspectiveCamera cam(Vector3D(job->eye[0], job->eye[1], job->eye[2]), Vector3D(job->dir[0], job->dir[1], job->dir[2]),
                          Vector3D(job->up[0], job->up[1], job->up[2]), job->fov, job->w, job->h, 1.0);
    ProgressivePhotonMapping ppm;
    const int np = job->w * job->h;
    std::vector<ProgressivePhotonMapping::RenderPoint> rpoints(np);
    for (int y = 0; y < job->h; y++)
        for (int x = 0; x < job->w; x++) {
            rpoints[y * job->w + x].pixelX = x;
            rpoints[y * job->w + x].pixelY = y;
            rpoints[y * job->w + x].n = 0;
        }
    Halton* hals = new Halton[OMP_NUM_CORE];
    for (int i = 0; i < OMP_NUM_CORE; i++) hals[i] = Halton(200, true, i);
    std::streambuf* old = std::cout.rdbuf(nullptr);
    for (int t = 0; t < job->npasses; t++) {
        ppm.traceRays(sc, cam, hals, &rpoints);
        ppm.tracePhotons(sc, hals, job->photons);
    }
    std::cout.rdbuf(old);
    for (int i = 0; i < np; i++) {
        const ProgressivePhotonMapping::RenderPoint& rp = rpoints[i];
        put3(image + 3 * i, (rp.emission + rp.flux / (PI * rp.r2)) * rp.coeff);
    }
    delete[] hals;
    return 0;
}

// The bytes a pass writes (ppm_probabilistic.cc:96-106) from an
// accumulation buffer (w*h*3 doubles, row y = camera row y, not divided):
// result.pixel(x, h - y - 1) = buffer(x, y) / t, optionally Image::tonemap
// (image.cc:498-524), Image::gamma(2.2, true) (image.cc:202-213), then
// Image::toByte per channel as Image::savePng does (image.cc:484-495).
// vals (optional, w*h*3): the doubles toByte receives.
void rh_image_bytes(const double* buffer, int w, int h, int t, int tonemap, unsigned char* out, double* vals) {
    Image result(w, h);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const double* b = buffer + 3 * ((size_t)y * w + x);
            result.pixel(x, h - y - 1) = Vector3D(b[0], b[1], b[2]) / t;
        }
    if (tonemap) result.tonemap();
    result.gamma(2.2, true);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const Vector3D& c = result(x, y);
            unsigned char* o = out + 3 * ((size_t)y * w + x);
            o[0] = Image::toByte(c.x());
            o[1] = Image::toByte(c.y());
            o[2] = Image::toByte(c.z());
            if (vals) {
                double* v = vals + 3 * ((size_t)y * w + x);
                v[0] = c.x(); v[1] = c.y(); v[2] = c.z();
            }
        }
}

// Halton::request (halton.cc:123-133): n numbers of `count` consecutive
// requests of the sampler Halton(200, true, seed).
void rh_halton(unsigned int seed, int count, int n, double* out) {
    Halton h(200, true, seed);
    for (int k = 0; k < count; k++) {
        RandomSequence rs;
        h.request(n, &rs);
        for (int i = 0; i < n; i++) out[(size_t)k * n + i] = rs.pop();
    }
}

// ---------------------------------------------------------------- dipole
void rh_dipole_rd(const Mat* m, const double* d2, int n, double* out) {
    BSDF b = makeBsdf(*m);
    for (int i = 0; i < n; i++) put3(out + 3 * i, (*b._bssrdf)(d2[i]));
}

double rh_dipole_fdr(const Mat* m) {
    BSDF b = makeBsdf(*m);
    return b._bssrdf->Fdr();
}

// SubsurfaceIntegrator::irradiance (subsurface_integrator.cc:234-238) over an
// octree built (subsurface_integrator.cc:67-145) from injected irradiance
// points: pos(3) normal(3) area(1) irad(3) doubles each.
void rh_dipole_irradiance(const Mat* m, const double* ipts, int n, double maxError, const double* q, int nq,
                          double* out) {
    BSDF b = makeBsdf(*m);
    SubsurfaceIntegrator integ;
    integ._maxError = maxError;
    std::vector<IrradiancePoint> pts(n);
    for (int i = 0; i < n; i++) {
        const double* p = ipts + 10 * i;
        pts[i] = IrradiancePoint(Vector3D(p[0], p[1], p[2]), Vector3D(p[3], p[4], p[5]), p[6], Vector3D(p[7], p[8], p[9]));
    }
    integ.octree.construct(&integ, pts);
    for (int j = 0; j < nq; j++) put3(out + 3 * j, integ.irradiance(Vector3D(q[3 * j], q[3 * j + 1], q[3 * j + 2]), b));
}

// SubsurfaceIntegrator::irradianceWithPM (subsurface_integrator.cc:329-365)
// over an injected photon map: photons are 8 doubles each (pos, flux, 2
// unused), points 6 doubles each (pos, normal).
void rh_irradiance_pm(const double* photons, int n, const double* points, int m, int numPhotons, int gatherPhotons,
                      double gatherRadius, double* out) {
    SubsurfaceIntegrator integ;
    std::vector<Photon> ph;
    ph.reserve(n);
    for (int i = 0; i < n; i++) {
        const double* p = photons + 8 * i;
        ph.push_back(Photon(Vector3D(p[0], p[1], p[2]), Vector3D(p[3], p[4], p[5]), Vector3D(), Vector3D()));
    }
    integ.photonMap.construct(ph);
    RenderParameters params(numPhotons, 1, gatherPhotons, gatherRadius);
    for (int j = 0; j < m; j++) {
        const double* q = points + 6 * j;
        put3(out + 3 * j, integ.irradianceWithPM(Vector3D(q[0], q[1], q[2]), Vector3D(q[3], q[4], q[5]), params));
    }
}

// sampler::poissonDisk (sampler.cc:36-101). Uses the reference's static RNG,
// so only the first call in a fresh process is reproducible.
int rh_poisson_disk(const float* v9, int ntri, double minDist, double* pts, double* nrms, int cap) {
    std::vector<Triangle> tris;
    for (int i = 0; i < ntri; i++) tris.push_back(Triangle(v3(v9 + 9 * i), v3(v9 + 9 * i + 3), v3(v9 + 9 * i + 6)));
    std::vector<Vector3D> p, nn;
    sampler::poissonDisk(tris, minDist, &p, &nn);
    for (int i = 0; i < (int)p.size() && i < cap; i++) { put3(pts + 3 * i, p[i]); put3(nrms + 3 * i, nn[i]); }
    return (int)p.size();
}

}  // extern "C"
