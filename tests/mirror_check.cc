// Exercise of the C++ host mirror (tatsy-pppm_gb300/host/pppm.hpp) with the
// reference's class names, compiled and run by tests/test_host_mirror.py:
//
//   mirror_check <dir>
//
// <dir> holds a.ply/a.hdr, b.ply/b.hdr (two scenes) and c.ply/c.hdr (a
// BSSRDF mesh). The program renders scene A, scene B and scene A again in
// one process (each Scene owns its GPU context), intersects rays through
// QBVHAccel and Scene, searches a KdTree, fills a HashGrid through add, and
// initializes a SubsurfaceIntegrator; every input it generates and every
// result is written to <dir> as raw little-endian arrays for the test to
// recompute through the Python binding.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "pppm.hpp"

namespace {

std::string gDir;

template <class T>
void save(const char* name, const std::vector<T>& v) {
    FILE* f = std::fopen((gDir + "/" + name).c_str(), "wb");
    if (!f) throw pppm::Error(PPPM_E_ARG, std::string("cannot write ") + name);
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

// deterministic inputs: a 64-bit LCG
uint64_t gState = 0x9E3779B97F4A7C15ull;
double uniform(double lo, double hi) {
    gState = gState * 6364136223846793005ull + 1442695040888963407ull;
    return lo + (hi - lo) * (double)(gState >> 11) * (1.0 / 9007199254740992.0);
}

struct Point {  // a KdTree element: coordinates by operator[], an id
    double v[3];
    int id;
    double operator[](int d) const { return v[d]; }
};

std::vector<float> render(const Scene& scene, int w, int h, RandomSamplerType type) {
    Camera camera(Vector3D(0.0, 4.0, -24.0), Vector3D(0.0, -0.15, 1.0).normalized(), Vector3D(0.0, 1.0, 0.0), 0.8, w,
                  h, 1.0);
    RenderParameters params(20000, 2, 128, 16.0);
    ProgressivePhotonMappingProb ppm;
    ppm.render(scene, camera, params, type);
    return ppm.result();
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s dir\n", argv[0]);
        return 2;
    }
    gDir = argv[1];
    try {
        Scene a, b, c;
        a.add(Trimesh(gDir + "/a.ply"), LambertianBRDF::factory(Vector3D(0.7, 0.6, 0.5)));
        a.setEnvmap(Envmap(gDir + "/a.hdr"));
        a.setAccelerator();
        b.add(Trimesh(gDir + "/b.ply"), SpecularBRDF::factory(Vector3D(0.9, 0.9, 0.9)));
        b.add(Trimesh(gDir + "/a.ply"), LambertianBRDF::factory(Vector3D(0.3, 0.5, 0.7)));
        b.setEnvmap(Envmap(gDir + "/b.hdr"));
        b.setAccelerator();
        // two scenes in one program: A, B, A again (compat mode, as the reference)
        save("render_a1.f32", render(a, 48, 32, RANDOM_SAMPLER_PSEUDO_RANDOM));
        save("render_b.f32", render(b, 48, 32, RANDOM_SAMPLER_PSEUDO_RANDOM));
        save("render_a2.f32", render(a, 48, 32, RANDOM_SAMPLER_PSEUDO_RANDOM));
        save("render_a_qmc.f32", render(a, 48, 32, RANDOM_SAMPLER_QUASI_MONTE_CARLO));

        // QBVHAccel over scene A's triangles, and Scene::intersect on the same rays
        const Trimesh mesh(gDir + "/a.ply");
        QBVHAccel accel;
        accel.construct(mesh.triangulate());
        std::vector<float> rays;
        std::vector<Ray> rv;
        std::vector<int32_t> ids, sids;
        std::vector<double> dist;
        for (int i = 0; i < 2000; i++) {
            const Vector3D o(uniform(-12, 12), uniform(-2, 12), uniform(-30, -15));
            const Vector3D d = (Vector3D(uniform(-4, 4), uniform(-6, 2), uniform(-4, 4)) - o).normalized();
            const float r[6] = {(float)o.x(), (float)o.y(), (float)o.z(), (float)d.x(), (float)d.y(), (float)d.z()};
            rays.insert(rays.end(), r, r + 6);
            // the mirror rounds a Ray to FP32 like every other caller of the C ABI
            rv.emplace_back(Vector3D(r[0], r[1], r[2]), Vector3D(r[3], r[4], r[5]));
            Hitpoint hp;
            ids.push_back(accel.intersect(rv.back(), &hp));
            dist.push_back(ids.back() >= 0 ? hp.distance() : 1e20);
        }
        std::vector<Intersection> isect;
        a.intersect(rv, &isect);
        for (const Intersection& x : isect) sids.push_back(x.objectID());
        save("rays.f32", rays);
        save("qbvh_ids.i32", ids);
        save("qbvh_dist.f64", dist);
        save("scene_ids.i32", sids);

        // KdTree with each KnnQuery type
        std::vector<Point> pts;
        std::vector<float> pf;
        for (int i = 0; i < 20000; i++) {
            Point p{{uniform(-10, 10), uniform(-10, 10), uniform(-10, 10)}, i};
            pts.push_back(p);
            for (int d = 0; d < 3; d++) pf.push_back((float)p.v[d]);
        }
        KdTree<Point> tree;
        tree.construct(pts);
        std::vector<float> qf;
        std::vector<int32_t> knn;
        const KnnQuery queries[3] = {KnnQuery(K_NEAREST | EPSILON_BALL, 1.5, 10), KnnQuery(K_NEAREST, 0.0, 16),
                                     KnnQuery(EPSILON_BALL, 0.9, 0)};
        for (int i = 0; i < 300; i++) {
            Point q{{uniform(-10, 10), uniform(-10, 10), uniform(-10, 10)}, -1};
            for (int d = 0; d < 3; d++) qf.push_back((float)q.v[d]);
            for (const KnnQuery& kq : queries) {
                std::vector<Point> res;
                tree.knnSearch(q, kq, &res);
                knn.push_back((int32_t)res.size());
                for (const Point& p : res) knn.push_back(p.id);
            }
        }
        save("kd_points.f32", pf);
        save("kd_queries.f32", qf);
        save("kd_results.i32", knn);

        // HashGrid<int>: add over boxes, operator[] at points
        HashGrid<int> grid;
        grid.init(4093, 1.0 / 0.7, BBox(-12.0, -12.0, -12.0, 12.0, 12.0, 12.0));
        std::vector<double> boxes;
        for (int i = 0; i < 3000; i++) {
            const Vector3D ctr(uniform(-13, 12), uniform(-13, 12), uniform(-13, 12));
            const double hx = uniform(0.0, 0.8), hy = uniform(0.0, 0.8), hz = uniform(0.0, 0.8);
            const Vector3D lo = ctr - Vector3D(hx, hy, hz), hi = ctr + Vector3D(hx, hy, hz);
            grid.add(i, lo, hi);
            const double bx[6] = {lo.x(), lo.y(), lo.z(), hi.x(), hi.y(), hi.z()};
            boxes.insert(boxes.end(), bx, bx + 6);
        }
        std::vector<double> hq;
        std::vector<int32_t> buckets;
        for (int i = 0; i < 500; i++) {
            const Vector3D v(uniform(-12, 12), uniform(-12, 12), uniform(-12, 12));
            const double xyz[3] = {v.x(), v.y(), v.z()};
            hq.insert(hq.end(), xyz, xyz + 3);
            const std::vector<int>& bucket = grid[v];
            buckets.push_back((int32_t)bucket.size());
            buckets.insert(buckets.end(), bucket.begin(), bucket.end());
        }
        save("hash_boxes.f64", boxes);
        save("hash_points.f64", hq);
        save("hash_buckets.i32", buckets);

        // SubsurfaceIntegrator on a BSSRDF mesh over a ground quad
        c.add(Trimesh(gDir + "/c.ply"), [] {
            BSDF s = LambertianBRDF::factory(Vector3D(0.6, 0.55, 0.5));
            s.setBssrdf(DipoleBSSRDF::factory(Vector3D(0.01, 0.02, 0.03), Vector3D(1.0, 1.5, 2.0), 1.3, 1.0));
            return s;
        }());
        c.add(Trimesh(gDir + "/a.ply"), LambertianBRDF::factory(Vector3D(0.5, 0.5, 0.5)));
        c.setEnvmap(Envmap(gDir + "/c.hdr"));
        c.setAccelerator();
        SubsurfaceIntegrator integ;
        integ.sssTime = 424242;
        RenderParameters sp(20000, 1, 128, 16.0);
        integ.initialize(c, sp, 0.6, 0.05);
        std::vector<Vector3D> at;
        std::vector<double> atf;
        for (int i = 0; i < 64; i++) {
            const Vector3D v(uniform(-3, 3), uniform(-4.5, 0.5), uniform(-12, -6));
            at.push_back(v);
            const double xyz[3] = {v.x(), v.y(), v.z()};
            atf.insert(atf.end(), xyz, xyz + 3);
        }
        const std::vector<Vector3D> irr = integ.irradiance(at, c.getBsdf(0));
        std::vector<double> irrf;
        for (const Vector3D& v : irr) irrf.insert(irrf.end(), {v.x(), v.y(), v.z()});
        save("sss_at.f64", atf);
        save("sss_irradiance.f64", irrf);
        save("sss_points.i64", std::vector<int64_t>{(int64_t)integ.numPoints()});
    } catch (const pppm::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 1;
    }
    std::printf("mirror check done\n");
    return 0;
}
