// C++ host mirror of the tatsy-pppm interface over the GB300 C ABI.
//
// Same class names and argument meanings as the reference, so a driver
// written against the reference (appmain.cc:11-26 shape) switches to the GPU
// by including this header instead of renderer.h and linking
// libpppm_gb300.so:
//
//   Scene scene;                      scene.h:23-56
//   scene.add(mesh, LambertianBRDF::factory(Vector3D(0.7, 0.3, 0.3)));
//   scene.setEnvmap(Envmap("sky.hdr"));
//   scene.setAccelerator();
//   Camera camera(eye, dir, up, 45.0, w, h, 1.0);
//   RenderParameters params(2000000, spp, 128, 16.0);
//   ProgressivePhotonMappingProb ppm;     // or ProgressivePhotonMapping, PathTracing
//   ppm.render(scene, camera, params);
//
// Where the reference aborts (Assertion, common.h:24-35) the mirror throws
// pppm::Error carrying the C ABI status and message; uncaught, it ends the
// program as the reference's abort does. Header-only.
#pragma once

#include <cmath>
#include <cstdint>
#include <ctime>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pppm_c.h"

namespace pppm {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int r, const pppm_ctx* c, const char* what) {
    if (r != PPPM_OK) throw Error(r, std::string(what) + ": " + (c ? pppm_last_error(c) : "no context"));
}

// One context per thread of the calling program; created on first use.
inline pppm_ctx* context() {
    thread_local std::unique_ptr<pppm_ctx, int (*)(pppm_ctx*)> ctx(nullptr, pppm_destroy);
    if (!ctx) {
        pppm_ctx* c = nullptr;
        check(pppm_create(0, &c), nullptr, "pppm_create");
        ctx.reset(c);
    }
    return ctx.get();
}

// The current pass's image as the reference saves it (flip, gamma 1/2.2,
// toByte; ppm_probabilistic.cc:96-106) written to a PNG file.
inline void savePassPng(pppm_ctx* c, int w, int h, const std::string& filename) {
    std::vector<uint8_t> rgb((size_t)w * h * 3);
    check(pppm_render_image(c, 0, rgb.data()), c, "savePng");
    int64_t n = 0;
    check(pppm_png_encode(rgb.data(), w, h, nullptr, 0, &n), nullptr, "savePng");
    std::vector<uint8_t> png((size_t)n);
    check(pppm_png_encode(rgb.data(), w, h, png.data(), n, &n), nullptr, "savePng");
    FILE* f = std::fopen(filename.c_str(), "wb");
    if (!f) throw Error(PPPM_E_ARG, "cannot write " + filename);
    const size_t wrote = std::fwrite(png.data(), 1, png.size(), f);
    std::fclose(f);
    if (wrote != png.size()) throw Error(PPPM_E_ARG, "short write to " + filename);
}

inline std::string passFile(const std::string& dir, const char* pattern, int t) {
    char name[64];
    std::snprintf(name, sizeof(name), pattern, t);
    return dir + name;
}

}  // namespace pppm

// --------------------------------------------------------------- math
class Vector3D {  // vector3d.h:21-98 (double x3)
    double v_[3];

public:
    Vector3D() : v_{0, 0, 0} {}
    Vector3D(double x, double y, double z) : v_{x, y, z} {}
    double x() const { return v_[0]; }
    double y() const { return v_[1]; }
    double z() const { return v_[2]; }
    double operator[](int d) const { return v_[d]; }
    double norm() const { return std::sqrt(dot(*this, *this)); }
    Vector3D normalized() const { return *this / (norm() + 1e-12); }
    static double dot(const Vector3D& a, const Vector3D& b) { return a.x() * b.x() + a.y() * b.y() + a.z() * b.z(); }
    static Vector3D cross(const Vector3D& u, const Vector3D& v) {
        return Vector3D(u.y() * v.z() - u.z() * v.y(), u.z() * v.x() - u.x() * v.z(), u.x() * v.y() - u.y() * v.x());
    }
    friend Vector3D operator+(const Vector3D& a, const Vector3D& b) { return Vector3D(a.x() + b.x(), a.y() + b.y(), a.z() + b.z()); }
    friend Vector3D operator-(const Vector3D& a, const Vector3D& b) { return Vector3D(a.x() - b.x(), a.y() - b.y(), a.z() - b.z()); }
    friend Vector3D operator*(const Vector3D& a, double s) { return Vector3D(a.x() * s, a.y() * s, a.z() * s); }
    friend Vector3D operator*(double s, const Vector3D& a) { return a * s; }
    friend Vector3D operator/(const Vector3D& a, double s) { return a * (1.0 / s); }
    Vector3D operator-() const { return Vector3D(-v_[0], -v_[1], -v_[2]); }
};

// --------------------------------------------------------------- geometry
class Triangle {  // triangle.h:16-45
    Vector3D p_[3];

public:
    Triangle() = default;
    Triangle(const Vector3D& a, const Vector3D& b, const Vector3D& c) : p_{a, b, c} {}
    Vector3D p(int i) const { return p_[i]; }
    std::vector<Triangle> triangulate() const { return {*this}; }
};

class Plane {  // plane.h: distance and normal, as Plane(double, const Vector3D&) takes them
    double d_ = 0.0;
    Vector3D n_;

public:
    Plane() = default;
    Plane(double distance, const Vector3D& normal) : d_(distance), n_(normal) {}
    double distance() const { return d_; }
    const Vector3D& normal() const { return n_; }
};

class BBox {  // bbox.h: BBox(minX, minY, minZ, maxX, maxY, maxZ)
    Vector3D lo_, hi_;

public:
    BBox(double minX, double minY, double minZ, double maxX, double maxY, double maxZ)
        : lo_(minX, minY, minZ), hi_(maxX, maxY, maxZ) {}
    BBox(const Vector3D& posMin, const Vector3D& posMax) : lo_(posMin), hi_(posMax) {}
    const Vector3D& posMin() const { return lo_; }
    const Vector3D& posMax() const { return hi_; }
};

class Trimesh {  // trimesh.h:68-166: binary little-endian PLY through pppm_ply_decode
    std::vector<double> verts_;  // 3 per vertex, double like the reference's Vector3D
    std::vector<int> faces_;

public:
    Trimesh() = default;
    explicit Trimesh(const std::string& filename) { load(filename); }
    Trimesh(const std::vector<Vector3D>& v, const std::vector<int>& f) : faces_(f) {
        for (const Vector3D& x : v)
            for (int d = 0; d < 3; d++) verts_.push_back(x[d]);
    }
    void load(const std::string& filename) {  // trimesh.cc:125-217
        std::ifstream in(filename, std::ios::binary);
        if (!in) throw pppm::Error(PPPM_E_ARG, "Failed to open mesh file: " + filename);
        const std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        int64_t nv = 0, nf = 0;
        int r = pppm_ply_decode(bytes.data(), (int64_t)bytes.size(), nullptr, 0, nullptr, 0, &nv, &nf);
        if (r) throw pppm::Error(r, "Invalid PLY file: " + filename);
        std::vector<float> v((size_t)(3 * nv));
        faces_.assign((size_t)(3 * nf), 0);
        if (nv > 0) {
            r = pppm_ply_decode(bytes.data(), (int64_t)bytes.size(), v.data(), 3 * nv, faces_.data(), 3 * nf, &nv,
                                &nf);
            if (r) throw pppm::Error(r, "Invalid PLY file: " + filename);
        }
        verts_.assign(v.begin(), v.end());
    }
    // placement before Scene::add, with the reference's arithmetic
    void translate(const Vector3D& move) {  // trimesh.cc:272-276
        const double m[3] = {move.x(), move.y(), move.z()};
        pppm_mesh_translate(verts_.data(), (int64_t)numVerts(), m);
    }
    void scale(double sx, double sy, double sz) { pppm_mesh_scale(verts_.data(), (int64_t)numVerts(), sx, sy, sz); }
    void scale(double s) { scale(s, s, s); }  // trimesh.cc:286-288
    void putOnPlane(const Plane& plane) {  // trimesh.cc:290-300
        const double n[3] = {plane.normal().x(), plane.normal().y(), plane.normal().z()};
        pppm_mesh_put_on_plane(verts_.data(), (int64_t)numVerts(), plane.distance(), n);
    }
    void fitToBBox(const BBox& box) {  // trimesh.cc:302-320
        const double lo[3] = {box.posMin().x(), box.posMin().y(), box.posMin().z()};
        const double hi[3] = {box.posMax().x(), box.posMax().y(), box.posMax().z()};
        pppm_mesh_fit_bbox(verts_.data(), (int64_t)numVerts(), lo, hi);
    }
    size_t numVerts() const { return verts_.size() / 3; }
    size_t numFaces() const { return faces_.size() / 3; }
    Vector3D getVertex(int id) const {
        if (id < 0 || (size_t)id >= numVerts()) throw pppm::Error(PPPM_E_ARG, "Vertex index out of bounds");
        return Vector3D(verts_[3 * id], verts_[3 * id + 1], verts_[3 * id + 2]);
    }
    std::vector<Triangle> triangulate() const {
        std::vector<Triangle> out;
        out.reserve(numFaces());
        for (size_t i = 0; i < numFaces(); i++)
            out.emplace_back(getVertex(faces_[3 * i]), getVertex(faces_[3 * i + 1]), getVertex(faces_[3 * i + 2]));
        return out;
    }
};

// --------------------------------------------------------------- materials
enum BsdfType {  // bsdf.h:19-26
    BSDF_TYPE_NONE = 0x00,
    BSDF_TYPE_LAMBERTIAN_BRDF = PPPM_BSDF_LAMBERTIAN,
    BSDF_TYPE_SPECULAR_BRDF = PPPM_BSDF_SPECULAR,
    BSDF_TYPE_PHONG_BRDF = PPPM_BSDF_PHONG,
    BSDF_TYPE_REFRACTION = PPPM_BSDF_REFRACTION,
    BSDF_TYPE_BSSRDF = PPPM_BSDF_BSSRDF
};

class BSSRDF {
public:
    pppm_material dipole{};
};

class DipoleBSSRDF {  // bssrdf.h:47-66
public:
    static BSSRDF factory(const Vector3D& sigma_a, const Vector3D& sigmap_s, double eta = 1.3, double scale = 1.0) {
        BSSRDF b;
        for (int k = 0; k < 3; k++) {
            b.dipole.sigma_a[k] = (float)sigma_a[k];
            b.dipole.sigmap_s[k] = (float)sigmap_s[k];
        }
        b.dipole.eta = (float)eta;
        b.dipole.scale = (float)scale;
        return b;
    }
};

class BSDF {  // bsdf.h:32-59
public:
    pppm_material m{};
    BsdfType type() const { return (BsdfType)(m.type | (m.has_bssrdf ? PPPM_BSDF_BSSRDF : 0)); }
    Vector3D reflectance() const { return Vector3D(m.refl[0], m.refl[1], m.refl[2]); }
    void setBssrdf(const BSSRDF& b) {
        m.has_bssrdf = 1;
        for (int k = 0; k < 3; k++) {
            m.sigma_a[k] = b.dipole.sigma_a[k];
            m.sigmap_s[k] = b.dipole.sigmap_s[k];
        }
        m.eta = b.dipole.eta;
        m.scale = b.dipole.scale;
    }
    static BSDF make(int type, const Vector3D& r, double n = 0.0) {
        BSDF b;
        b.m.type = type;
        for (int k = 0; k < 3; k++) b.m.refl[k] = (float)r[k];
        b.m.phong_n = (float)n;
        return b;
    }
};

struct LambertianBRDF {
    static BSDF factory(const Vector3D& r) { return BSDF::make(PPPM_BSDF_LAMBERTIAN, r); }
};
struct SpecularBRDF {
    static BSDF factory(const Vector3D& r) { return BSDF::make(PPPM_BSDF_SPECULAR, r); }
};
struct PhongBRDF {
    static BSDF factory(const Vector3D& r, double n) { return BSDF::make(PPPM_BSDF_PHONG, r, n); }
};
struct RefractionBSDF {
    static BSDF factory(const Vector3D& r) { return BSDF::make(PPPM_BSDF_REFRACTION, r); }
};

// --------------------------------------------------------------- env map
class Envmap {  // envmap.h:21-47
public:
    int width = 0, height = 0;
    std::vector<float> rgb;  // row 0 = top, as Image stores it
    Envmap() = default;
    explicit Envmap(const std::string& filename) {  // Radiance HDR via Image::loadHdr semantics
        std::ifstream in(filename, std::ios::binary);
        if (!in) throw pppm::Error(PPPM_E_ARG, "Failed to load file \"" + filename + "\"");
        std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        int32_t w = 0, h = 0;
        pppm::check(pppm_hdr_decode(bytes.data(), (int64_t)bytes.size(), nullptr, 0, &w, &h), nullptr, "Envmap");
        rgb.resize((size_t)w * h * 3);
        pppm::check(pppm_hdr_decode(bytes.data(), (int64_t)bytes.size(), rgb.data(), (int64_t)rgb.size(), &w, &h),
                    nullptr, "Envmap");
        width = w;
        height = h;
    }
    Envmap(int w, int h, std::vector<float> data) : width(w), height(h), rgb(std::move(data)) {}
};

// --------------------------------------------------------------- rays / scene
class Ray {  // ray.h:20-38
    Vector3D o_, d_;

public:
    Ray(const Vector3D& o, const Vector3D& d) : o_(o), d_(d) {}
    Vector3D origin() const { return o_; }
    Vector3D direction() const { return d_; }
};

class Hitpoint {  // ray.h:40-60
public:
    double distance_ = 1e20;
    Vector3D position_, normal_;
    double distance() const { return distance_; }
    Vector3D position() const { return position_; }
    Vector3D normal() const { return normal_; }
};

class Intersection {  // ray.h:62-80
public:
    Hitpoint hp;
    int id = -1;
    int objectID() const { return id; }
    const Hitpoint& hitpoint() const { return hp; }
};

namespace pppm {
// A context of its own (device memory, stream, render state), released
// with the last owner.
inline std::shared_ptr<pppm_ctx> newContext() {
    pppm_ctx* c = nullptr;
    check(pppm_create(0, &c), nullptr, "pppm_create");
    return std::shared_ptr<pppm_ctx>(c, [](pppm_ctx* x) { pppm_destroy(x); });
}
}  // namespace pppm

class Scene {  // scene.h:23-56, scene.cc
    std::vector<float> tris_;
    std::vector<int32_t> matId_;
    std::vector<pppm_material> mats_;
    Envmap env_;
    bool accel_ = false;
    // every Scene owns its GPU context: its triangles, BVH and env map live
    // there, and integrators render a scene in the scene's own context, so
    // several scenes coexist in one program (copies share the context)
    std::shared_ptr<pppm_ctx> ctx_;

public:
    template <class T>
    void add(const T& geom, const BSDF& bsdf) {
        const int id = (int)mats_.size();
        mats_.push_back(bsdf.m);
        for (const Triangle& t : geom.triangulate()) {
            for (int k = 0; k < 3; k++)
                for (int d = 0; d < 3; d++) tris_.push_back((float)t.p(k)[d]);
            matId_.push_back(id);
        }
        accel_ = false;
    }
    void setEnvmap(const Envmap& e) { env_ = e; }
    void setAccelerator() {
        if (!ctx_) ctx_ = pppm::newContext();
        pppm_ctx* c = ctx_.get();
        pppm::check(pppm_scene_set(c, tris_.data(), (int64_t)matId_.size(), matId_.data(), mats_.data(),
                                   (int32_t)mats_.size()), c, "Scene::setAccelerator");
        if (!env_.rgb.empty())
            pppm::check(pppm_env_set(c, env_.rgb.data(), env_.width, env_.height), c, "Scene::setEnvmap");
        accel_ = true;
    }
    // The scene's context (after setAccelerator; integrators render there).
    pppm_ctx* context() const {
        if (!accel_) throw pppm::Error(PPPM_E_STATE, "the scene has no accelerator: call setAccelerator first");
        return ctx_.get();
    }
    size_t numTriangles() const { return matId_.size(); }
    Triangle getTriangle(int id) const {  // scene.h:52
        const float* t = &tris_[9 * (size_t)id];
        return Triangle(Vector3D(t[0], t[1], t[2]), Vector3D(t[3], t[4], t[5]), Vector3D(t[6], t[7], t[8]));
    }
    BSDF getBsdf(int id) const {  // scene.h:53
        BSDF b;
        b.m = mats_[(size_t)matId_[(size_t)id]];
        return b;
    }
    // Scene::intersect -> QBVHAccel::intersect (scene.cc:40-47)
    bool intersect(const Ray& ray, Intersection& isect) const {
        if (!accel_) throw pppm::Error(PPPM_E_STATE, "Scene::intersect before setAccelerator");
        const float r[6] = {(float)ray.origin().x(), (float)ray.origin().y(), (float)ray.origin().z(),
                            (float)ray.direction().x(), (float)ray.direction().y(), (float)ray.direction().z()};
        int32_t tri;
        double t;
        float pos[3], nrm[3];
        pppm_ctx* c = context();
        pppm::check(pppm_intersect(c, r, 1, &tri, &t, pos, nrm), c, "Scene::intersect");
        isect.id = tri;
        isect.hp.distance_ = t;
        isect.hp.position_ = Vector3D(pos[0], pos[1], pos[2]);
        isect.hp.normal_ = Vector3D(nrm[0], nrm[1], nrm[2]);
        return tri != -1;
    }
    // Many rays in one GPU call (the single-ray form waits for the GPU per ray).
    void intersect(const std::vector<Ray>& rays, std::vector<Intersection>* out) const {
        std::vector<float> r(rays.size() * 6);
        for (size_t i = 0; i < rays.size(); i++)
            for (int d = 0; d < 3; d++) {
                r[6 * i + d] = (float)rays[i].origin()[d];
                r[6 * i + 3 + d] = (float)rays[i].direction()[d];
            }
        std::vector<int32_t> tri(rays.size());
        std::vector<double> t(rays.size());
        std::vector<float> pos(rays.size() * 3), nrm(rays.size() * 3);
        pppm_ctx* c = context();
        pppm::check(pppm_intersect(c, r.data(), (int64_t)rays.size(), tri.data(), t.data(), pos.data(), nrm.data()), c,
                    "Scene::intersect");
        out->resize(rays.size());
        for (size_t i = 0; i < rays.size(); i++) {
            Intersection& x = (*out)[i];
            x.id = tri[i];
            x.hp.distance_ = t[i];
            x.hp.position_ = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
            x.hp.normal_ = Vector3D(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        }
    }
};

// --------------------------------------------------------------- QBVH
class QBVHAccel {  // qbvh_accel.h:24-67: construct + closest hit, on the GPU
    std::shared_ptr<pppm_ctx> ctx_;
    bool built_ = false;

public:
    // QBVHAccel::construct (qbvh_accel.cc:139-203): the reference's 4-wide
    // topology, built on the host and uploaded to this accelerator's context.
    void construct(const std::vector<Triangle>& triangles) {
        if (!ctx_) ctx_ = pppm::newContext();
        std::vector<float> tri(triangles.size() * 9);
        for (size_t i = 0; i < triangles.size(); i++)
            for (int k = 0; k < 3; k++)
                for (int d = 0; d < 3; d++) tri[9 * i + 3 * k + d] = (float)triangles[i].p(k)[d];
        const std::vector<int32_t> mid(triangles.size(), 0);
        const pppm_material m = LambertianBRDF::factory(Vector3D(0.5, 0.5, 0.5)).m;
        pppm::check(pppm_scene_set(ctx_.get(), tri.data(), (int64_t)triangles.size(), mid.data(), &m, 1), ctx_.get(),
                    "QBVHAccel::construct");
        built_ = true;
    }
    // QBVHAccel::intersect (qbvh_accel.cc:205-285): the closest triangle's
    // index, or -1; hitpoint receives distance, position and normal.
    int intersect(const Ray& ray, Hitpoint* hitpoint) const {
        if (!built_) throw pppm::Error(PPPM_E_STATE, "QBVHAccel::intersect before construct");
        const float r[6] = {(float)ray.origin().x(), (float)ray.origin().y(), (float)ray.origin().z(),
                            (float)ray.direction().x(), (float)ray.direction().y(), (float)ray.direction().z()};
        int32_t tri;
        double t;
        float pos[3], nrm[3];
        pppm::check(pppm_intersect(ctx_.get(), r, 1, &tri, &t, pos, nrm), ctx_.get(), "QBVHAccel::intersect");
        if (tri >= 0 && hitpoint) {
            hitpoint->distance_ = t;
            hitpoint->position_ = Vector3D(pos[0], pos[1], pos[2]);
            hitpoint->normal_ = Vector3D(nrm[0], nrm[1], nrm[2]);
        }
        return tri;
    }
};

// --------------------------------------------------------------- camera / params
class PerspectiveCamera {  // perspective_camera.h:16-32
public:
    pppm_camera c{};
    PerspectiveCamera() = default;
    PerspectiveCamera(const Vector3D& center, const Vector3D& direction, const Vector3D& up, double fov, int w, int h,
                      double /*sensitivity*/) {
        for (int d = 0; d < 3; d++) {
            c.eye[d] = (float)center[d];
            c.dir[d] = (float)direction[d];
            c.up[d] = (float)up[d];
        }
        c.fov = (float)fov;
        c.width = w;
        c.height = h;
    }
};
typedef PerspectiveCamera Camera;

class RenderParameters {  // render_parameters.h:4-37
    int photons_, spp_, gatherPhotons_;
    double gatherRadius_;

public:
    explicit RenderParameters(int photons = 1000000, int spp = 16, int gatherPhotons = 16, double gatherRadius = 16.0)
        : photons_(photons), spp_(spp), gatherPhotons_(gatherPhotons), gatherRadius_(gatherRadius) {}
    int photons() const { return photons_; }
    int spp() const { return spp_; }
    int gatherPhotons() const { return gatherPhotons_; }
    double gatherRadius() const { return gatherRadius_; }
};

// --------------------------------------------------------------- integrator
enum RandomSamplerType {  // random_sampler.h
    RANDOM_SAMPLER_PSEUDO_RANDOM = 0,
    RANDOM_SAMPLER_QUASI_MONTE_CARLO = 1
};

class ProgressivePhotonMappingProb {  // ppm_probabilistic.h:23-42
    std::vector<float> result_;
    int w_ = 0, h_ = 0, passes_ = 0;

public:
    // Reference semantics by default; `mode` selects PPPM_MODE_CANONICAL.
    // numStreams is the reference's OMP_NUM_CORE (its RNG stream count).
    int mode = PPPM_MODE_COMPAT;
    int numStreams = 8;
    // Non-empty: after every pass the image is written to
    // resultDirectory + "%03d.png", as the reference does with RESULT_DIRECTORY.
    std::string resultDirectory;

    // ProgressivePhotonMappingProb::render (ppm_probabilistic.cc:24-121) in
    // the scene's context: the reference writes a PNG per pass; here the
    // linear buffer stays on the GPU and result() returns buffer / passes
    // after the call. randomSamplerType as the reference's (:58-73): the
    // quasi-Monte Carlo type gives stream i the sampler Halton(200, true, i)
    // (compat mode only, as the reference has no canonical mode).
    void render(const Scene& scene, const Camera& camera, const RenderParameters& params,
                RandomSamplerType randomSamplerType = RANDOM_SAMPLER_PSEUDO_RANDOM) {
        pppm_ctx* ctx = scene.context();
        pppm_params p{};
        p.mode = mode;
        if (randomSamplerType == RANDOM_SAMPLER_QUASI_MONTE_CARLO) p.flags |= PPPM_FLAG_SAMPLER_QMC;
        p.num_streams = numStreams;
        p.photons = params.photons();
        p.gather_photons = params.gatherPhotons();
        p.gather_radius = params.gatherRadius();
        p.max_bounce_photon = 64;
        p.max_bounce_eye = 64;
        p.alpha = 0.7;
        p.radius_scale = mode == PPPM_MODE_COMPAT ? 0.1 : 1.0 / 64.0;
        p.cell_factor = 1.0f;
        p.seed = 1;
        // the subsurface photon streams of the reference are seeded with
        // time(NULL) + thread (subsurface_integrator.cc:248)
        p.sss_time = (uint32_t)std::time(nullptr);
        pppm::check(pppm_render_begin(ctx, &camera.c, &p), ctx, "render");
        for (int t = 1; t <= params.spp(); t++) {
            pppm::check(pppm_render_pass(ctx, t, nullptr), ctx, "render");
            if (!resultDirectory.empty())
                pppm::savePassPng(ctx, camera.c.width, camera.c.height, pppm::passFile(resultDirectory, "%03d.png", t));
        }
        w_ = camera.c.width;
        h_ = camera.c.height;
        passes_ = params.spp();
        result_.assign((size_t)w_ * h_ * 3, 0.0f);
        pppm::check(pppm_render_read(ctx, result_.data()), ctx, "render");
    }
    // Linear radiance per pixel (row y = camera row y, not flipped), divided
    // by the pass count like the reference's per-pass image (:97-100).
    std::vector<float> result() const {
        std::vector<float> r(result_);
        for (auto& v : r) v /= (float)(passes_ > 0 ? passes_ : 1);
        return r;
    }
    int width() const { return w_; }
    int height() const { return h_; }
};

class ProgressivePhotonMapping {  // progressive_photon_mapping.h:26-110 (classic PPM)
    std::vector<float> result_;
    int w_ = 0, h_ = 0, passes_ = 0;

public:
    // numStreams is the reference's OMP_NUM_CORE: its Halton sampler count
    // (with more than one, the reference's update order varies per run).
    int numStreams = 8;
    // Non-empty: after every pass the image is written to resultDirectory +
    // "progressive_photonmap_%03d.png" (progressive_photon_mapping.cc:103).
    std::string resultDirectory;

    // ProgressivePhotonMapping::render (progressive_photon_mapping.cc:31-119):
    // result() returns the last pass's image.
    void render(const Scene& scene, const Camera& camera, const RenderParameters& params) {
        pppm_ctx* ctx = scene.context();
        pppm_params p{};
        p.mode = PPPM_MODE_CLASSIC;
        p.num_streams = numStreams;
        p.photons = params.photons();
        p.gather_photons = params.gatherPhotons();
        p.gather_radius = params.gatherRadius();
        p.max_bounce_photon = 64;
        p.max_bounce_eye = 64;
        p.alpha = 0.7;  // ProgressivePhotonMapping::ALPHA
        p.radius_scale = 1.0;
        p.cell_factor = 1.0f;
        pppm::check(pppm_render_begin(ctx, &camera.c, &p), ctx, "render");
        for (int t = 1; t <= params.spp(); t++) {
            pppm::check(pppm_render_pass(ctx, t, nullptr), ctx, "render");
            if (!resultDirectory.empty())
                pppm::savePassPng(ctx, camera.c.width, camera.c.height,
                                  pppm::passFile(resultDirectory, "progressive_photonmap_%03d.png", t));
        }
        w_ = camera.c.width;
        h_ = camera.c.height;
        passes_ = params.spp();
        result_.assign((size_t)w_ * h_ * 3, 0.0f);
        pppm::check(pppm_render_read(ctx, result_.data()), ctx, "render");
    }
    // (emission + flux / (pi r^2)) * coeff / passes per pixel (:98-103), not flipped.
    std::vector<float> result() const {
        std::vector<float> r(result_);
        for (auto& v : r) v /= (float)(passes_ > 0 ? passes_ : 1);
        return r;
    }
    int width() const { return w_; }
    int height() const { return h_; }
};

class PathTracing {  // path_tracing.h:20-37
    std::vector<float> result_;
    int w_ = 0, h_ = 0, passes_ = 0;

public:
    // numStreams is the reference's OMP_NUM_CORE (its RNG stream count).
    int numStreams = 8;
    // Non-empty: after every sample the image is written to
    // resultDirectory + "%03d.png" (path_tracing.cc:107-110).
    std::string resultDirectory;

    // PathTracing::render (path_tracing.cc:23-127) with the pseudo-random
    // sampler (the quasi-Monte Carlo one is not provided: PPPM_E_ARG);
    // bounceLimit 64 as executePathTracing's default.
    void render(const Scene& scene, const Camera& camera, const RenderParameters& params,
                RandomSamplerType randomSamplerType = RANDOM_SAMPLER_PSEUDO_RANDOM) {
        if (randomSamplerType != RANDOM_SAMPLER_PSEUDO_RANDOM)
            throw pppm::Error(PPPM_E_ARG, "PathTracing: only the pseudo-random sampler");
        pppm_ctx* ctx = scene.context();
        pppm_params p{};
        p.mode = PPPM_MODE_PATH_TRACING;
        p.num_streams = numStreams;
        p.photons = params.photons();
        p.gather_photons = params.gatherPhotons();
        p.gather_radius = params.gatherRadius();
        p.max_bounce_photon = 64;
        p.max_bounce_eye = 64;
        p.alpha = 0.7;
        p.radius_scale = 0.1;
        p.cell_factor = 1.0f;
        p.sss_time = (uint32_t)std::time(nullptr);
        pppm::check(pppm_render_begin(ctx, &camera.c, &p), ctx, "render");
        for (int t = 1; t <= params.spp(); t++) {
            pppm::check(pppm_render_pass(ctx, t, nullptr), ctx, "render");
            if (!resultDirectory.empty())
                pppm::savePassPng(ctx, camera.c.width, camera.c.height, pppm::passFile(resultDirectory, "%03d.png", t));
        }
        w_ = camera.c.width;
        h_ = camera.c.height;
        passes_ = params.spp();
        result_.assign((size_t)w_ * h_ * 3, 0.0f);
        pppm::check(pppm_render_read(ctx, result_.data()), ctx, "render");
    }
    // Linear radiance per pixel (row y = camera row y, not flipped) / samples.
    std::vector<float> result() const {
        std::vector<float> r(result_);
        for (auto& v : r) v /= (float)(passes_ > 0 ? passes_ : 1);
        return r;
    }
    int width() const { return w_; }
    int height() const { return h_; }
};

// --------------------------------------------------------------- subsurface
namespace pppm {
// The state of sampler::poissonDisk's process-wide XorShift (sampler.cc:
// its static Random), XorShift(0) at program start (random.h:23-31).
inline uint32_t* poissonRngState() {
    static uint32_t st[4] = {0, 0, 0, 0};
    static bool init = false;
    if (!init) {
        uint32_t v = 0;
        for (int i = 1; i <= 4; i++) {
            v = 1812433253u * (v ^ (v >> 30)) + (uint32_t)i;
            st[i - 1] = v;
        }
        init = true;
    }
    return st;
}
}  // namespace pppm

class SubsurfaceIntegrator {  // subsurface_integrator.h:40-130
    std::vector<float> ipts_;  // per irradiance point: position, normal, area, irradiance (10 floats)
    double maxError_ = 0.05;

public:
    // numStreams is the reference's OMP_NUM_CORE (the subsurface photon
    // streams XorShift(time(NULL) + i)); sssTime, when non-zero, stands for
    // time(NULL) so that a run can be repeated.
    int numStreams = 8;
    uint32_t sssTime = 0;

    // SubsurfaceIntegrator::initialize (subsurface_integrator.cc:179-204) in
    // the scene's context: Poisson-disc points on the BSSRDF triangles with
    // the process-wide sampler state (sampler.cc:36-101), the subsurface
    // photon map (buildPhotonMap, :240-327, streams seeded time(NULL) + i),
    // the irradiance at the points (irradianceWithPM, :329-365). The octree
    // over the points is built where irradiance() is evaluated. Resets any
    // render active in the scene's context.
    void initialize(const Scene& scene, const RenderParameters& params, double areaRadius, double maxError = 0.05) {
        pppm_ctx* c = scene.context();
        std::vector<float> tri;
        double area4 = 0.0;
        for (int i = 0; i < (int)scene.numTriangles(); i++) {
            if (!(scene.getBsdf(i).type() & BSDF_TYPE_BSSRDF)) continue;
            const Triangle t = scene.getTriangle(i);
            for (int k = 0; k < 3; k++)
                for (int d = 0; d < 3; d++) tri.push_back((float)t.p(k)[d]);
            const Vector3D cr = Vector3D::cross(t.p(1) - t.p(0), t.p(2) - t.p(1));
            area4 += std::ceil(4.0 * 0.5 * cr.norm() / (areaRadius * areaRadius));
        }
        if (tri.empty()) throw pppm::Error(PPPM_E_STATE, "The scene does not have subsurface scattering object!!");
        const int64_t ntri = (int64_t)tri.size() / 9;
        const int64_t cap = (int64_t)area4 + ntri + 16;
        std::vector<float> pts((size_t)cap * 3), nrm((size_t)cap * 3);
        int64_t m = 0;
        pppm::check(pppm_poisson_disk(c, tri.data(), ntri, areaRadius, pppm::poissonRngState(), pts.data(), nrm.data(),
                                      cap, &m), c, "SubsurfaceIntegrator::initialize");
        maxError_ = maxError;
        pppm_params p{};
        p.mode = PPPM_MODE_COMPAT;
        p.num_streams = numStreams;
        p.photons = params.photons();
        p.gather_photons = params.gatherPhotons();
        p.gather_radius = params.gatherRadius();
        p.max_bounce_photon = 64;
        p.max_bounce_eye = 64;
        p.alpha = 0.7;
        p.radius_scale = 0.1;
        p.cell_factor = 1.0f;
        p.sss_time = sssTime ? sssTime : (uint32_t)std::time(nullptr);
        int64_t np = 0;
        pppm::check(pppm_subsurface_photons(c, &p, 1, nullptr, 0, &np), c, "SubsurfaceIntegrator::initialize");
        std::vector<float> ph((size_t)std::max<int64_t>(np, 1) * 8);
        pppm::check(pppm_subsurface_photons(c, &p, 1, ph.data(), np, &np), c, "SubsurfaceIntegrator::initialize");
        std::vector<float> q6((size_t)m * 6), irad((size_t)m * 3);
        for (int64_t i = 0; i < m; i++)
            for (int d = 0; d < 3; d++) {
                q6[6 * i + d] = pts[3 * i + d];
                q6[6 * i + 3 + d] = nrm[3 * i + d];
            }
        if (m > 0)
            pppm::check(pppm_subsurface_photon_irradiance(c, ph.data(), np, q6.data(), m, params.photons(),
                                                          params.gatherRadius(), params.gatherPhotons(), irad.data()),
                        c, "SubsurfaceIntegrator::initialize");
        const double dA = (0.5 * areaRadius) * (0.5 * areaRadius) * 3.14159265358979323846;  // :199
        ipts_.assign((size_t)m * 10, 0.0f);
        for (int64_t i = 0; i < m; i++) {
            float* o = &ipts_[10 * (size_t)i];
            for (int d = 0; d < 3; d++) {
                o[d] = pts[3 * i + d];
                o[3 + d] = nrm[3 * i + d];
                o[7 + d] = irad[3 * i + d];
            }
            o[6] = (float)dA;
        }
    }
    size_t numPoints() const { return ipts_.size() / 10; }
    // SubsurfaceIntegrator::irradiance (:234-238): (1/pi)(1 - Fdr) times the
    // octree sum of Rd(d^2) E A (subsurface_integrator.cc:147-167).
    Vector3D irradiance(const Vector3D& p, const BSDF& bsdf) const { return irradiance(std::vector<Vector3D>{p}, bsdf)[0]; }
    std::vector<Vector3D> irradiance(const std::vector<Vector3D>& ps, const BSDF& bsdf) const {
        if (!bsdf.m.has_bssrdf) throw pppm::Error(PPPM_E_ARG, "Specified object does not have BSSRDF!!");
        std::vector<float> q(ps.size() * 3), rgb(ps.size() * 3);
        for (size_t i = 0; i < ps.size(); i++)
            for (int d = 0; d < 3; d++) q[3 * i + d] = (float)ps[i][d];
        pppm_ctx* c = pppm::context();
        pppm::check(pppm_dipole_irradiance(c, &bsdf.m, ipts_.data(), (int64_t)numPoints(), maxError_, q.data(),
                                           (int64_t)ps.size(), rgb.data()), c, "SubsurfaceIntegrator::irradiance");
        std::vector<Vector3D> out;
        for (size_t i = 0; i < ps.size(); i++) out.emplace_back(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
        return out;
    }
};

// --------------------------------------------------------------- photon map / hash grid
class Photon : public Vector3D {  // photon.h:6-44
public:
    Vector3D flux_;
    using Vector3D::Vector3D;
    Photon(const Vector3D& p, const Vector3D& flux) : Vector3D(p), flux_(flux) {}
    Vector3D flux() const { return flux_; }
};

class PhotonMap {  // photon_map.h:18-29
    std::vector<Photon> photons_;
    std::vector<float> pos_;

public:
    void construct(const std::vector<Photon>& photons) {
        photons_ = photons;
        pos_.clear();
        for (const Photon& p : photons)
            for (int d = 0; d < 3; d++) pos_.push_back((float)p[d]);
    }
    // PhotonMap::findKNN (photon_map.cc:24-26), reference argument order and
    // result order (farthest first).
    void findKNN(const Photon& query, std::vector<Photon>* out, int numTargetPhotons, double targetRadius) const {
        const float q[3] = {(float)query.x(), (float)query.y(), (float)query.z()};
        const int cap = 64;
        std::vector<int32_t> idx(cap);
        int32_t cnt = 0;
        pppm_ctx* c = pppm::context();
        pppm::check(pppm_knn(c, pos_.data(), (int64_t)photons_.size(), q, 1, numTargetPhotons, targetRadius,
                             idx.data(), &cnt, cap), c, "PhotonMap::findKNN");
        for (int i = 0; i < cnt && i < cap; i++) out->push_back(photons_[idx[i]]);
    }
};

enum KnnSearchType {  // kdtree.h:8-11
    EPSILON_BALL = PPPM_KNN_EPSILON_BALL,
    K_NEAREST = PPPM_KNN_K_NEAREST
};

struct KnnQuery {  // kdtree.h:13-24
    KnnSearchType type;
    double epsilon;
    int k;
    KnnQuery(int type_, double epsilon_, int k_) : type(static_cast<KnnSearchType>(type_)), epsilon(epsilon_), k(k_) {}
};

template <class T>
class KdTree {  // kdtree.h:26-88: the search runs on the GPU over the hash grid
    std::vector<T> points_;
    std::vector<float> pos_;

public:
    void construct(const std::vector<T>& points) {  // kdtree_detail.h:53-87
        points_ = points;
        pos_.clear();
        pos_.reserve(points.size() * 3);
        for (const T& p : points)
            for (int d = 0; d < 3; d++) pos_.push_back((float)p[d]);
    }
    void release() {
        points_.clear();
        pos_.clear();
    }
    // KdTree::knnSearch (kdtree_detail.h:88-132): the reference's result
    // order (farthest first). At most 64 results per query; an
    // EPSILON_BALL-only query with more points in its ball throws
    // (PPPM_E_CAPACITY) instead of returning a partial set.
    void knnSearch(const T& point, const KnnQuery& query, std::vector<T>* results) const {
        const float q[3] = {(float)point[0], (float)point[1], (float)point[2]};
        const int cap = 64;
        std::vector<int32_t> idx(cap);
        int32_t cnt = 0;
        pppm_ctx* c = pppm::context();
        pppm::check(pppm_kdtree_knn(c, pos_.data(), (int64_t)points_.size(), q, 1, (int32_t)query.type, query.epsilon,
                                    query.k, idx.data(), &cnt, cap), c, "KdTree::knnSearch");
        for (int i = 0; i < cnt && i < cap; i++) results->push_back(points_[(size_t)idx[i]]);
    }
};

template <class T>
class HashGrid {  // hash_grid.h:8-37; buckets built on the GPU (pppm_hashgrid_build)
    int size_ = -1;
    double scale_ = 0.0;
    double bbmin_[3] = {0, 0, 0};
    std::vector<T> items_;
    std::vector<double> lo_, hi_;
    std::vector<std::vector<T>> data_;
    bool built_ = false;

    void build() {
        pppm_ctx* c = pppm::context();
        const int64_t n = (int64_t)items_.size();
        int64_t cnt = 0;
        pppm::check(pppm_hashgrid_build(c, lo_.data(), hi_.data(), n, size_, scale_, bbmin_, nullptr, nullptr, 0, &cnt),
                    c, "HashGrid::add");
        std::vector<uint32_t> start((size_t)size_ + 1);
        std::vector<int32_t> ids((size_t)std::max<int64_t>(cnt, 1));
        pppm::check(pppm_hashgrid_build(c, lo_.data(), hi_.data(), n, size_, scale_, bbmin_, start.data(), ids.data(),
                                        cnt, &cnt), c, "HashGrid::add");
        data_.assign((size_t)size_, {});
        for (int b = 0; b < size_; b++)
            for (uint32_t k = start[b]; k < start[(size_t)b + 1]; k++) data_[(size_t)b].push_back(items_[(size_t)ids[k]]);
        built_ = true;
    }

public:
    // HashGrid::init (hash_grid_detail.h:26-31)
    void init(int hashSize, double hashScale, const BBox& bbox) {
        size_ = hashSize;
        scale_ = hashScale;
        for (int d = 0; d < 3; d++) bbmin_[d] = bbox.posMin()[d];
        clear();
    }
    // HashGrid::add (hash_grid_detail.h:34-52): p enters every bucket of the
    // cells the box covers; the buckets are formed on the GPU at the next
    // operator[] after adds.
    void add(const T& p, const Vector3D& boxMin, const Vector3D& boxMax) {
        items_.push_back(p);
        for (int d = 0; d < 3; d++) {
            lo_.push_back(boxMin[d]);
            hi_.push_back(boxMax[d]);
        }
        built_ = false;
    }
    void clear() {  // hash_grid_detail.h:54-57
        items_.clear();
        lo_.clear();
        hi_.clear();
        data_.clear();
        built_ = false;
    }
    // HashGrid::operator[] (hash_grid_detail.h:65-72): the bucket of v's cell,
    // items in the reference's insertion order
    std::vector<T>& operator[](const Vector3D& v) {
        if (size_ <= 0) throw pppm::Error(PPPM_E_STATE, "hash size is not initialized");
        if (!built_) build();
        return data_[(size_t)bucket(v)];
    }
    // The bucket of v's cell: |(int)((v - bbMin) * scale)| per axis and the
    // reference's hash, in double like operator[] (hash_grid_detail.h:60-72).
    uint32_t bucket(const Vector3D& v) const {
        int c[3];
        for (int d = 0; d < 3; d++) c[d] = std::abs(static_cast<int>((v[d] - bbmin_[d]) * scale_));
        return ((uint32_t)c[0] * 73856093u ^ (uint32_t)c[1] * 19349663u ^ (uint32_t)c[2] * 83492791u) % (uint32_t)size_;
    }
    // buckets of many points (rounded to FP32) in one GPU call
    std::vector<uint32_t> buckets(const std::vector<Vector3D>& pts) const {
        std::vector<float> p;
        for (const auto& v : pts)
            for (int d = 0; d < 3; d++) p.push_back((float)v[d]);
        std::vector<uint32_t> out(pts.size());
        pppm_ctx* c = pppm::context();
        pppm::check(pppm_hash_points(c, p.data(), (int64_t)pts.size(), size_, scale_, bbmin_, out.data()), c,
                    "HashGrid");
        return out;
    }
};
