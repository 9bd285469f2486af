// CPU restatement of tatsy-pppm's PPM-APA pass (the oracle port).
//
// TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load this library, as the checker or as the timed CPU
// baseline. The product never links or calls it.
//
// It restates the reference algorithm in double precision, following its
// operation order so results are bit-identical to the reference built with
// the same compiler flags on the same machine (pinned against the compiled
// reference by tests/test_oracle_port.py):
//   - XorShift streams, 200-number tapes   random.h:16-62, random_sequence.h
//   - QBVH build/traversal                 qbvh_accel.cc:139-285
//   - Moller-Trumbore                      triangle.cc:53-78
//   - Envmap importance + photon emission  envmap.cc:47-163
//   - BSDF sampling                        brdf.cc:23-142, reflectance.h:7-34
//   - tracePhotons / traceRays / radiance  ppm_probabilistic.cc:123-344
//   - kd-tree + kNN (max-heap)             kdtree_detail.h:53-132
// and adds the canonical Knaus-Zwicker variant of the GPU library
// (radius-ball gather, r^2 *= (t+alpha)/(t+1), counter-seeded RNG).
// The OpenMP structure of the reference is kept (one fork per round of N
// photons, rows distributed y % N) so its speed stands in for the reference.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <queue>
#include <stack>
#include <string>
#include <vector>

#include "../include/pppm_c.h"

namespace port {

const double kEps = 1.0e-12;
const double kInf = 1.0e20;
const double kPi = 4.0 * std::atan(1.0);
const double kInvPi = 1.0 / kPi;

struct V {
    double x, y, z;
    V() : x(0), y(0), z(0) {}
    V(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int d) const { return d == 0 ? x : (d == 1 ? y : z); }
};
// Vector3D semantics (vector3d.cc): binary ops component-wise, division by a
// scalar multiplies by its reciprocal.
inline V operator+(V a, V b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V operator-(V a, V b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V operator-(V a) { return V(-a.x, -a.y, -a.z); }
inline V operator*(V a, V b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V operator*(V a, double s) { return V(a.x * s, a.y * s, a.z * s); }
inline V operator*(double s, V a) { return V(a.x * s, a.y * s, a.z * s); }
inline V operator/(V a, double s) {
    const double d = 1.0 / s;
    return V(a.x * d, a.y * d, a.z * d);
}
inline double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(V u, V v) { return V(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x); }
inline double norm(V v) { return std::sqrt(dot(v, v)); }
inline V normalized(V v) { return v / (norm(v) + kEps); }
inline V reflect(V v, V n) { return v - n * (2.0 * dot(n, v)); }
inline double lum(V v) { return dot(v, V(0.2126, 0.7152, 0.0722)); }

// ------------------------------------------------------------------ RNG
struct XorShift {
    uint32_t s[4];
    explicit XorShift(uint32_t init = 0) {
        uint32_t v = init;
        for (int i = 1; i <= 4; i++) { v = 1812433253u * (v ^ (v >> 30)) + (uint32_t)i; s[i - 1] = v; }
    }
    uint32_t next() {
        const uint32_t t = s[0] ^ (s[0] << 11);
        s[0] = s[1]; s[1] = s[2]; s[2] = s[3];
        return s[3] = (s[3] ^ (s[3] >> 19)) ^ (t ^ (t >> 8));
    }
    double real() { return (double)next() * (double)(1.0f / 4294967295u); }
};

// Murmur3's 32-bit finaliser (a nonlinear bijection of 32-bit words).
inline uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}

struct Tape {
    double v[200];
    int pos = 0;
    // scramble (canonical mode): every output through mix32 before it
    // becomes a real, as the GPU library's canonical tapes do
    void fill(XorShift& x, bool scramble = false) {
        for (int i = 0; i < 200; i++)
            v[i] = scramble ? (double)mix32(x.next()) * (double)(1.0f / 4294967295u) : x.real();
        pos = 0;
    }
    double pop() { return v[pos++]; }
};

// Canonical mode: the same per-path seeding as the GPU library.
inline XorShift seedCanonical(uint32_t seed, int pass, uint64_t id) {
    XorShift x;
    const uint32_t a = mix32(seed ^ 0x9e3779b9u * (uint32_t)(pass + 1));
    const uint32_t b = mix32((uint32_t)id ^ mix32((uint32_t)(id >> 32) + a));
    x.s[0] = mix32(a ^ b) | 1u;
    x.s[1] = mix32(b + 0x632be59bu);
    x.s[2] = mix32(a + 0x85157af5u + b);
    x.s[3] = mix32(b ^ 0xa54ff53au);
    return x;
}

// ------------------------------------------------------------------ geometry
struct Tri {
    V p0, p1, p2;
    V gravity() const { return (p0 + p1 + p2) / 3.0; }
    V normal() const { return normalized(cross(p1 - p0, p2 - p0)); }
    bool hit(V o, V d, double* t) const {
        const V e1 = p1 - p0, e2 = p2 - p0;
        const V pv = cross(d, e2);
        const double det = dot(e1, pv);
        if (det > -kEps && det < kEps) return false;
        const double inv = 1.0 / det;
        const V tv = o - p0;
        const double u = dot(tv, pv) * inv;
        if (u < 0.0 || u > 1.0) return false;
        const V qv = cross(tv, e1);
        const double v = dot(d, qv) * inv;
        if (v < 0.0 || u + v > 1.0) return false;
        const double tt = dot(e2, qv) * inv;
        if (tt > kEps) { *t = tt; return true; }
        return false;
    }
};

// 4-wide BVH with the reference's construction and traversal.
class Qbvh {
    struct Node {
        float box[2][3][4];
        Node* child[4] = {nullptr, nullptr, nullptr, nullptr};
        std::vector<std::pair<int, int>> tris;  // (slot in tris_, id)
        int sep[3] = {0, 0, 0};
        bool leaf = false;
    };
    std::vector<std::unique_ptr<Node>> pool_;
    Node* root_ = nullptr;
    const std::vector<Tri>* tris_ = nullptr;

    static const int* order() {
        static const int t[128] = {
            0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44444, 0x44440, 0x44440, 0x44440, 0x44440,
            0x44440, 0x44440, 0x44440, 0x44440, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441, 0x44441,
            0x44401, 0x44401, 0x44410, 0x44410, 0x44401, 0x44401, 0x44410, 0x44410, 0x44442, 0x44442, 0x44442, 0x44442,
            0x44442, 0x44442, 0x44442, 0x44442, 0x44402, 0x44402, 0x44402, 0x44402, 0x44420, 0x44420, 0x44420, 0x44420,
            0x44412, 0x44412, 0x44412, 0x44412, 0x44421, 0x44421, 0x44421, 0x44421, 0x44012, 0x44012, 0x44102, 0x44102,
            0x44201, 0x44201, 0x44210, 0x44210, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443, 0x44443,
            0x44403, 0x44403, 0x44403, 0x44403, 0x44430, 0x44430, 0x44430, 0x44430, 0x44413, 0x44413, 0x44413, 0x44413,
            0x44431, 0x44431, 0x44431, 0x44431, 0x44013, 0x44013, 0x44103, 0x44103, 0x44301, 0x44301, 0x44310, 0x44310,
            0x44423, 0x44432, 0x44423, 0x44432, 0x44423, 0x44432, 0x44423, 0x44432, 0x44023, 0x44032, 0x44023, 0x44032,
            0x44230, 0x44320, 0x44230, 0x44320, 0x44123, 0x44132, 0x44123, 0x44132, 0x44231, 0x44321, 0x44231, 0x44321,
            0x40123, 0x40132, 0x41023, 0x41032, 0x42301, 0x43201, 0x42310, 0x43210};
        return t;
    }

    struct Item {
        V g;
        int id;
    };

    Node* rec(std::vector<Item>& v, int dim) {
        pool_.emplace_back(new Node());
        Node* nd = pool_.back().get();
        const int n = (int)v.size();
        if (n <= 3) {
            nd->leaf = true;
            for (auto& it : v) nd->tris.push_back({it.id, it.id});
            return nd;
        }
        auto cmp = [](int d) { return [d](const Item& a, const Item& b) { return a.g[d] < b.g[d]; }; };
        std::sort(v.begin(), v.end(), cmp(dim));
        const int mid = n / 2;
        std::sort(v.begin(), v.begin() + mid, cmp((dim + 1) % 3));
        std::sort(v.begin() + mid, v.end(), cmp((dim + 1) % 3));
        std::vector<Item> c[4] = {std::vector<Item>(v.begin(), v.begin() + mid / 2),
                                  std::vector<Item>(v.begin() + mid / 2, v.begin() + mid),
                                  std::vector<Item>(v.begin() + mid, v.begin() + mid + mid / 2),
                                  std::vector<Item>(v.begin() + mid + mid / 2, v.end())};
        for (int i = 0; i < 4; i++) {
            V mn(kInf, kInf, kInf), mx(-kInf, -kInf, -kInf);
            for (auto& it : c[i]) {
                const Tri& t = (*tris_)[it.id];
                for (const V& p : {t.p0, t.p1, t.p2}) {
                    mn = V(std::min(mn.x, p.x), std::min(mn.y, p.y), std::min(mn.z, p.z));
                    mx = V(std::max(mx.x, p.x), std::max(mx.y, p.y), std::max(mx.z, p.z));
                }
            }
            for (int d = 0; d < 3; d++) {
                nd->box[0][d][i] = (float)mn[d];
                nd->box[1][d][i] = (float)mx[d];
            }
        }
        for (int i = 0; i < 4; i++) nd->child[i] = rec(c[i], (dim + 2) % 3);
        nd->sep[0] = dim;
        nd->sep[1] = (dim + 1) % 3;
        nd->sep[2] = (dim + 1) % 3;
        return nd;
    }

public:
    void build(const std::vector<Tri>& tris) {
        tris_ = &tris;
        pool_.clear();
        std::vector<Item> v(tris.size());
        for (size_t i = 0; i < tris.size(); i++) v[i] = {tris[i].gravity(), (int)i};
        root_ = rec(v, 0);
    }

    // Returns the triangle id or -1; *t is the hit distance (kInf on a miss).
    int intersect(V o, V d, double* tOut) const {
        const float o3[3] = {(float)o.x, (float)o.y, (float)o.z};
        const float id3[3] = {d.x == 0.0 ? 1.0e20f : (float)(1.0 / d.x), d.y == 0.0 ? 1.0e20f : (float)(1.0 / d.y),
                              d.z == 0.0 ? 1.0e20f : (float)(1.0 / d.z)};
        int sgn[3];
        for (int k = 0; k < 3; k++) sgn[k] = id3[k] > 0.0f ? 0 : 1;
        int hit = -1;
        double best = kInf;
        Node* stack[64];
        int sp = 0;
        stack[sp++] = root_;
        const int* ord = order();
        while (sp > 0) {
            Node* nd = stack[--sp];
            if (nd->leaf) {
                for (auto& tr : nd->tris) {
                    double t;
                    if ((*tris_)[tr.second].hit(o, d, &t) && best > t) {
                        best = t;
                        hit = tr.second;
                    }
                }
                continue;
            }
            const float hd = (float)best;
            float tmin[4] = {0, 0, 0, 0}, tmax[4] = {hd, hd, hd, hd};
            for (int k = 0; k < 3; k++)
                for (int i = 0; i < 4; i++) {
                    const float a = (nd->box[sgn[k]][k][i] - o3[k]) * id3[k];
                    const float b = (nd->box[1 - sgn[k]][k][i] - o3[k]) * id3[k];
                    tmin[i] = tmin[i] > a ? tmin[i] : a;
                    tmax[i] = tmax[i] < b ? tmax[i] : b;
                }
            int mask = 0;
            for (int i = 0; i < 4; i++) mask |= (tmax[i] >= tmin[i]) ? (1 << i) : 0;
            if (mask) {
                const int sep = (sgn[nd->sep[0]] << 2) | (sgn[nd->sep[1]] << 1) | sgn[nd->sep[2]];
                int om = ord[mask * 8 + sep];
                for (int i = 0; i < 4; i++) {
                    if (om & 0x04) break;
                    stack[sp++] = nd->child[om & 0x03];
                    om >>= 4;
                }
            }
        }
        *tOut = best;
        return hit;
    }
};

// ------------------------------------------------------------------ materials, env, camera
struct Mat {
    int type;
    bool bssrdf;
    V refl;
    double phongN;
};

inline void onHemisphere(V w, double r1, double r2, V* out) {
    V u = std::abs(w.x) > kEps ? normalized(cross(V(0, 1, 0), w)) : normalized(cross(V(1, 0, 0), w));
    const V v = cross(w, u);
    const double t = 2.0 * kPi * r1;
    const double z2s = std::sqrt(r2);
    *out = normalized(u * std::cos(t) * z2s + v * std::sin(t) * z2s + w * std::sqrt(1.0 - r2));
}

inline bool totalReflection(bool into, V in, V n, V on, V* rd, V* td, double* fre, double* ftr) {
    *rd = reflect(in, n);
    const double nnt = into ? 1.0 / 1.5 : 1.5 / 1.0;
    const double ddn = dot(in, on);
    const double cos2t = 1.0 - nnt * nnt * (1.0 - ddn * ddn);
    if (cos2t < 0.0) { *td = V(); *fre = 1.0; *ftr = 0.0; return true; }
    *td = normalized(in * nnt - n * (into ? 1.0 : -1.0) * (ddn * nnt + std::sqrt(cos2t)));
    const double a = 1.5 - 1.0, b = 1.5 + 1.0, R0 = (a * a) / (b * b);
    const double c = 1.0 - (into ? -ddn : dot(*td, -on));
    *fre = R0 + (1.0 - R0) * (c * c * c * c * c);
    *ftr = 1.0 - *fre;
    return false;
}

inline void bsdfSample(const Mat& m, V in, V n, double r1, double r2, V* out, double* pdf) {
    if (m.type == PPPM_BSDF_LAMBERTIAN) {
        onHemisphere(dot(in, n) < 0.0 ? n : -n, r1, r2, out);
    } else if (m.type == PPPM_BSDF_SPECULAR) {
        *out = reflect(in, dot(in, n) < 0.0 ? n : -n);
    } else if (m.type == PPPM_BSDF_PHONG) {
        const V w = reflect(in, dot(in, n) < 0.0 ? n : -n);
        V u = std::abs(w.x) > kEps ? normalized(cross(V(0, 1, 0), w)) : normalized(cross(V(1, 0, 0), w));
        const V v = cross(w, u);
        const double th = std::acos(std::pow(r1, 1.0 / (m.phongN + 1.0)));
        const double ph = 2.0 * kPi * r2;
        *out = u * std::sin(th) * std::cos(ph) + w * std::cos(th) + v * std::sin(th) * std::sin(ph);
    } else {
        bool into = true;
        V on = n;
        if (dot(in, n) >= 0.0) { into = false; on = on * -1.0; }
        V rd, td;
        double fre, ftr;
        if (totalReflection(into, in, n, on, &rd, &td, &fre, &ftr)) {
            *out = rd;
            *pdf = 1.0;
        } else {
            const double p = 0.25 + 0.5 * 0.5;
            if (r1 < p) { *out = rd; *pdf = p / fre; } else { *out = td; *pdf = (1.0 - p) / ftr; }
        }
    }
}

struct Env {
    int w = 0, h = 0;
    std::vector<V> img;
    std::vector<double> pdf, cdf;
    V lookup(V d) const {
        if (w == 0) return V();  // no environment map
        const double th = std::acos(d.y);
        double ph = std::atan2(d.z, d.x);
        if (ph < 0.0) ph += 2.0 * kPi;
        const double u = ph / (2.0 * kPi), v = th / kPi;
        int ix = (int)(u * w), iy = (int)(v * h);
        ix = ix < 0 ? 0 : (ix > w - 1 ? w - 1 : ix);
        iy = iy < 0 ? 0 : (iy > h - 1 ? h - 1 : iy);
        return img[(size_t)iy * w + ix];
    }
    void build() {
        const int W = 64, H = 64, sx = w / W, sy = h / H;
        pdf.assign(W * H, 0.0);
        cdf.assign(W * H, 0.0);
        double total = 0.0;
        for (int iy = 0; iy < H; iy++)
            for (int ix = 0; ix < W; ix++) {
                V acc;
                for (int y = 0; y < sy; y++)
                    for (int x = 0; x < sx; x++) {
                        const double u = (ix + static_cast<double>(x) / sx) / W;
                        const double v = (iy + static_cast<double>(y) / sy) / H;
                        const double phi = u * 2.0 * kPi;
                        const double yy = (1.0 - v) * 2.0 - 1.0;
                        acc = acc + lookup(V(std::sqrt(1.0 - yy * yy) * std::cos(phi), yy,
                                             std::sqrt(1.0 - yy * yy) * std::sin(phi))) / (sx * sy);
                    }
                const double l = lum(acc);
                pdf[iy * W + ix] = l * l;
                total += pdf[iy * W + ix];
            }
        pdf[0] /= (total + kEps);
        cdf[0] = pdf[0];
        for (int i = 1; i < W * H; i++) {
            pdf[i] /= (total + kEps);
            cdf[i] = pdf[i] + cdf[i - 1];
        }
    }
    // Envmap::samplePhoton + onHemisphere. Returns false past the CDF end.
    bool emit(Tape& tp, double numPhotons, V* pos, V* dir, V* flux) const {
        const double r = tp.pop();
        const int index = (int)(std::lower_bound(cdf.begin(), cdf.end(), r) - cdf.begin());
        if (index >= (int)cdf.size()) return false;
        const int ix = index % 64, iy = index / 64;
        const double u = (ix + tp.pop()) / 64;
        const double v = (iy + tp.pop()) / 64;
        const double phi = u * kPi * 2.0;
        const double y = (1.0 - v) * 2.0 - 1.0;
        const V d(std::sqrt(1.0 - y * y) * std::cos(phi), y, std::sqrt(1.0 - y * y) * std::sin(phi));
        const double area = ((double)((unsigned)w * (unsigned)h)) / (4.0 * kPi * 64 * 64);
        *flux = lookup(d) * (area / (pdf[index] * numPhotons));
        *pos = 50.0 * d;
        // the reference build evaluates onHemisphere's two pop() arguments right to left
        const double r2 = tp.pop();
        const double r1 = tp.pop();
        onHemisphere(-d, r1, r2, dir);
        return true;
    }
};

struct Camera {
    V center, dir, U, Vv;
    double halfTan, aspect;
    int w, h;
    V ray(double px, double py) const {
        const V d = dir + halfTan * aspect * (2.0 * px / w - 1.0) * U + halfTan * (2.0 * py / h - 1.0) * Vv;
        return normalized(d);
    }
};

// ------------------------------------------------------------------ photon map
struct Photon {
    V p, flux, dir, n;
    int64_t path = -1;  // emitted path index (the GPU library's numbering: s * T + i in compat mode)
};

class KdTree {
    struct Node {
        Photon pt;
        Node* l = nullptr;
        Node* r = nullptr;
        int axis = 0;
    };
    std::vector<Node> nodes_;

    Node* rec(std::vector<const Photon*>& v, int id, int s, int e, int dim) {
        if (s >= e) return nullptr;
        std::sort(v.begin() + s, v.begin() + e, [dim](const Photon* a, const Photon* b) { return a->p[dim] < b->p[dim]; });
        const int mid = (s + e) / 2;
        Node* nd = &nodes_[id];
        nd->axis = dim;
        nd->pt = *v[mid];
        nd->l = rec(v, id * 2 + 1, s, mid, (dim + 1) % 3);
        nd->r = rec(v, id * 2 + 2, mid + 1, e, (dim + 1) % 3);
        return nd;
    }

    struct Ord {
        double d;
        const Photon* p;
        bool operator<(const Ord& o) const { return d < o.d; }
    };

    void knnRec(const Node* nd, V q, bool knn, int k, double& eps, std::priority_queue<Ord>& pq) const {
        if (!nd) return;
        const double dist = norm(nd->pt.p - q);
        if (dist < eps) {
            pq.push({dist, &nd->pt});
            if (knn && (int)pq.size() > k) {
                pq.pop();
                eps = norm(pq.top().p->p - q);
            }
        }
        const double delta = q[nd->axis] - nd->pt.p[nd->axis];
        if (delta < 0.0) {
            knnRec(nd->l, q, knn, k, eps, pq);
            if (std::abs(delta) <= eps) knnRec(nd->r, q, knn, k, eps, pq);
        } else {
            knnRec(nd->r, q, knn, k, eps, pq);
            if (std::abs(delta) <= eps) knnRec(nd->l, q, knn, k, eps, pq);
        }
    }

public:
    void build(const std::vector<Photon>& pts) {
        int nn = 1;
        while (nn < (int)pts.size()) nn <<= 1;
        nodes_.assign(nn, Node());
        std::vector<const Photon*> v(pts.size());
        for (size_t i = 0; i < pts.size(); i++) v[i] = &pts[i];
        if (!pts.empty()) rec(v, 0, 0, (int)pts.size(), 0);
    }
    // Canonical gather: the flux of every photon strictly inside the ball of
    // radius r around q whose stored normal faces `on`. Same tree and the
    // same pruning as knnRec (a subtree is visited when |delta| <= r), but
    // the fluxes are summed in visiting order with no heap: the reference
    // has no ball-only gather, and a heap of ~10^3 photons per query would
    // make the CPU timing a measure of std::priority_queue.
    V ballSum(V q, double r, V on) const {
        V tot;
        if (nodes_.empty()) return tot;
        const Node* stack[64];
        int sp = 0;
        stack[sp++] = &nodes_[0];
        while (sp > 0) {
            const Node* nd = stack[--sp];
            const V diff = nd->pt.p - q;
            if (norm(diff) < r && dot(nd->pt.n, on) > 0.0) tot = tot + nd->pt.flux;
            const double delta = q[nd->axis] - nd->pt.p[nd->axis];
            const Node* nearC = delta < 0.0 ? nd->l : nd->r;
            const Node* farC = delta < 0.0 ? nd->r : nd->l;
            if (farC && std::abs(delta) <= r) stack[sp++] = farC;
            if (nearC) stack[sp++] = nearC;
        }
        return tot;
    }
    // Calls f(photon, |p - q|) for every photon strictly inside radius r of q
    // (same traversal as ballSum).
    template <class F>
    void forBall(V q, double r, F&& f) const {
        if (nodes_.empty()) return;
        const Node* stack[64];
        int sp = 0;
        stack[sp++] = &nodes_[0];
        while (sp > 0) {
            const Node* nd = stack[--sp];
            const double d = norm(nd->pt.p - q);
            if (d < r) f(nd->pt, d);
            const double delta = q[nd->axis] - nd->pt.p[nd->axis];
            const Node* nearC = delta < 0.0 ? nd->l : nd->r;
            const Node* farC = delta < 0.0 ? nd->r : nd->l;
            if (farC && std::abs(delta) <= r) stack[sp++] = farC;
            if (nearC) stack[sp++] = nearC;
        }
    }
    // knn: K_NEAREST | EPSILON_BALL with (epsilon, k); else EPSILON_BALL only.
    // Results farthest first (the max-heap's pop order).
    void query(V q, bool knn, int k, double eps, std::vector<const Photon*>* out) const {
        out->clear();
        if (nodes_.empty()) return;
        std::priority_queue<Ord> pq;
        knnRec(&nodes_[0], q, knn, k, eps, pq);
        while (!pq.empty()) {
            out->push_back(pq.top().p);
            pq.pop();
        }
    }
};

// ------------------------------------------------------------------ renderer
struct Scene {
    std::vector<Tri> tris;
    std::vector<int> matId;
    std::vector<Mat> mats;
    Env env;
    Qbvh bvh;
    double bmin[3], bmax[3];
    // emissive materials (the GPU library's pppm_material_emission; the
    // reference has none): emission per material, the emitting triangles,
    // their area CDF (last entry 1) and summed area
    std::vector<V> emit;
    std::vector<int> lightTris;
    std::vector<double> lightCdf;
    double lightArea = 0.0;
    bool emissive(int mat) const { return emit[mat].x > 0.0 || emit[mat].y > 0.0 || emit[mat].z > 0.0; }
};

struct Renderer {
    const Scene* sc;
    Camera cam;
    pppm_params par;
    bool compat;
    double radius = 0.0;
    int N;
    std::vector<XorShift> streams;
    KdTree kd;
    std::vector<double> buffer;
    std::vector<double> queries;  // per pixel, 12 doubles (radiance's rec), when requested
    std::vector<Photon> lastPhotons;
    int64_t stored = 0, phantoms = 0;
    double msPhoton = 0.0, msEye = 0.0;

    V envLookup(V d) const { return sc->env.lookup(d); }

    // tracePhotons (ppm_probabilistic.cc:123-208) for one path.
    // A photon from the emissive triangles, in the GPU library's draw order:
    // the emitter by area (first CDF entry >= the draw), u = sqrt(r1) and
    // barycentrics (1 - u, u (1 - r2), u r2), a cosine direction about the
    // normal e1 x e2, flux Le * pi * area / photons.
    bool lightEmit(Tape& tp, V* pos, V* dir, V* flux) const {
        const double r = tp.pop();
        const int k = (int)(std::lower_bound(sc->lightCdf.begin(), sc->lightCdf.end(), r) - sc->lightCdf.begin());
        if (k >= (int)sc->lightCdf.size()) return false;
        const Tri& t = sc->tris[sc->lightTris[k]];
        const double r1 = tp.pop(), r2 = tp.pop();
        const double su = std::sqrt(r1);
        const V e1 = t.p1 - t.p0, e2 = t.p2 - t.p0;
        *pos = t.p0 + (su * (1.0 - r2)) * e1 + (su * r2) * e2;
        const V n = normalized(cross(e1, e2));
        const double a0 = tp.pop(), a1 = tp.pop();
        onHemisphere(n, a0, a1, dir);
        *flux = sc->emit[sc->matId[sc->lightTris[k]]] * (kPi * sc->lightArea / (double)par.photons);
        return true;
    }

    void tracePath(Tape& tp, std::vector<Photon>* out, int pass, int64_t pathId) {
        V pos, d, flux;
        if (!sc->lightTris.empty()) {
            if (!lightEmit(tp, &pos, &d, &flux)) return;
        } else if (!sc->env.emit(tp, (double)par.photons, &pos, &d, &flux)) {
            return;
        }
        V o = pos;
        for (int b = 0;; b++) {
            if (b >= par.max_bounce_photon || std::max(flux.x, std::max(flux.y, flux.z)) <= 0.0) break;
            double t;
            const int id = sc->bvh.intersect(o, d, &t);
            if (id < 0) break;
            const double r0 = tp.pop(), r1 = tp.pop(), r2 = tp.pop();
            const Mat& m = sc->mats[sc->matId[id]];
            const V hp = o + t * d;
            const V n = sc->tris[id].normal();
            const V on = dot(n, d) < 0.0 ? n : -n;
            V nd;
            double pdf = 1.0;
            if (m.type == PPPM_BSDF_LAMBERTIAN) {
                out->push_back({hp, flux, d, compat ? n : on, pathId});
                const double prob = (m.refl.x + m.refl.y + m.refl.z) / 3.0;
                if (r0 < prob) {
                    bsdfSample(m, d, on, r1, r2, &nd, &pdf);
                    flux = flux * m.refl / prob;
                } else {
                    break;
                }
            } else {
                bsdfSample(m, d, on, r0, r1, &nd, &pdf);
                flux = flux * m.refl / pdf;
            }
            o = hp;
            d = nd;
        }
        (void)pass;
    }

    // The Lambertian gather of radiance (ppm_probabilistic.cc:300-335).
    V gatherCompat(V q, V n, V refl, double roulette) const {
        std::vector<const Photon*> ph;
        kd.query(q, true, (int)radius, (double)par.gather_photons, &ph);
        const int np = (int)ph.size();
        std::vector<double> dist;
        double maxd = 0.0;
        for (int i = 0; i < np; i++) {
            const V diff = q - ph[i]->p;
            const double dd = norm(diff);
            if (std::abs(dot(n, diff) / dd) < radius * radius * 0.01) {
                dist.push_back(dd);
                maxd = std::max(maxd, dd);
            }
        }
        const double k = 1.1;
        V tot;
        for (size_t i = 0; i < dist.size(); i++) {
            const double w = 1.0 - (dist[i] / (k * maxd));
            const V v = refl * ph[i]->flux * kInvPi;
            tot = tot + w * v;
        }
        tot = tot / (1.0 - 2.0 / (3.0 * k));
        if (maxd > kEps) return tot / (kPi * maxd * maxd * roulette);
        return V();
    }

    V gatherCanonical(V q, V on, V refl, double roulette) const {
        const V tot = kd.ballSum(q, radius, on);
        return refl * tot * kInvPi / (kPi * radius * radius * roulette);
    }

    // radiance (ppm_probabilistic.cc:246-344) without BSSRDF. The recursion
    // is unrolled into a loop; the per-bounce factors are applied innermost
    // first, (refl * L) / (pdf * roulette), as the recursive calls return.
    // rec (optional, 12 doubles): the gather query of this path, as the GPU
    // library's eye kernel writes it: hit point, triangle id, oriented
    // normal, specular bounces before the hit, path weight * refl /
    // roulette, and rec[11] = 1 when the path gathered.
    V radiance(V o, V d, Tape& tp, double* rec = nullptr) const {
        std::vector<std::pair<V, double>> stack;
        V inner;
        // emitters met on the way (none in the reference's scenes), weighted
        // by the path throughput so far
        V emitted, wfwd(1.0, 1.0, 1.0);
        for (int b = 0;; b++) {
            double t;
            const int id = b >= par.max_bounce_eye ? -1 : sc->bvh.intersect(o, d, &t);
            if (id < 0) {
                inner = envLookup(d);
                break;
            }
            const double r0 = tp.pop(), r1 = tp.pop(), r2 = tp.pop();
            const Mat& m = sc->mats[sc->matId[id]];
            const V hp = o + t * d;
            const V n = sc->tris[id].normal();
            if (!sc->lightTris.empty() && sc->emissive(sc->matId[id]) && dot(n, d) < 0.0)
                emitted = emitted + wfwd * sc->emit[sc->matId[id]];
            double roul = std::max(m.refl.x, std::max(m.refl.y, m.refl.z));
            if (b >= 3) {
                if (r0 > roul) {
                    inner = V();
                    break;
                }
            } else {
                roul = 1.0;
            }
            if (m.type == PPPM_BSDF_LAMBERTIAN) {
                const V on = dot(n, d) < 0.0 ? n : -n;
                inner = compat ? gatherCompat(hp, n, m.refl, roul) : gatherCanonical(hp, on, m.refl, roul);
                if (rec) {
                    V w(1.0, 1.0, 1.0);
                    for (const auto& f : stack) w = w * f.first / f.second;
                    w = w * m.refl / roul;
                    const double v[12] = {hp.x, hp.y, hp.z, (double)id, on.x, on.y, on.z, (double)stack.size(),
                                          w.x, w.y, w.z, 1.0};
                    std::memcpy(rec, v, sizeof(v));
                }
                break;
            }
            double pdf = 1.0;
            V nd;
            bsdfSample(m, d, n, r1, r2, &nd, &pdf);
            stack.push_back({m.refl, pdf * roul});
            wfwd = wfwd * m.refl / (pdf * roul);
            o = hp;
            d = nd;
        }
        for (size_t j = stack.size(); j-- > 0;) inner = stack[j].first * inner / stack[j].second;
        return sc->lightTris.empty() ? inner : inner + emitted;
    }

    int pass(int t) {
        const auto t0 = std::chrono::steady_clock::now();
        const int64_t T = compat ? (par.photons + N - 1) / N : par.photons;
        std::vector<std::vector<Photon>> ph(compat ? N : 1);
        if (compat) {
            // one OpenMP fork per round of N photons, like the reference
            for (int64_t i = 0; i < T; i++) {
#pragma omp parallel for num_threads(N)
                for (int s = 0; s < N; s++) {
                    Tape tp;
                    tp.fill(streams[s]);
                    tracePath(tp, &ph[s], t, (int64_t)s * T + i);
                }
            }
        } else {
            const int nt = omp_get_max_threads();
            std::vector<std::vector<Photon>> loc(nt);
#pragma omp parallel for schedule(dynamic, 1024)
            for (int64_t g = 0; g < T; g++) {
                Tape tp;
                XorShift x = seedCanonical(par.seed, t, (uint64_t)g);
                tp.fill(x, true);
                tracePath(tp, &loc[omp_get_thread_num()], t, g);
            }
            for (auto& v : loc) ph[0].insert(ph[0].end(), v.begin(), v.end());
        }
        std::vector<Photon> all;
        stored = 0;
        phantoms = 0;
        if (compat) {
            all.assign((size_t)(T * N), Photon());
            for (int s = 0; s < N; s++) {
                if ((int64_t)ph[s].size() > T) return PPPM_E_UNDEFINED;
                std::copy(ph[s].begin(), ph[s].end(), all.begin() + s * T);
                stored += (int64_t)ph[s].size();
            }
            phantoms = T * N - stored;
        } else {
            all.swap(ph[0]);
            stored = (int64_t)all.size();
        }
        kd.build(all);
        lastPhotons.swap(all);
        const auto t1 = std::chrono::steady_clock::now();
        const int W = cam.w, H = cam.h;
        if (compat) {
            const int64_t rounds = (H + N - 1) / N;
            for (int64_t i = 0; i < rounds; i++) {
#pragma omp parallel for num_threads(N)
                for (int s = 0; s < N; s++) {
                    const int64_t y = (int64_t)s + i * N;
                    if (y >= H) continue;
                    for (int x = 0; x < W; x++) {
                        Tape tp;
                        tp.fill(streams[s]);
                        const double px = x + tp.pop() - 0.5;
                        const double py = y + tp.pop() - 0.5;
                        double* rec = queries.empty() ? nullptr : &queries[12 * ((size_t)y * W + x)];
                        if (rec) rec[11] = 0.0;
                        const V L = radiance(cam.center, cam.ray(px, py), tp, rec);
                        double* p = &buffer[3 * ((size_t)y * W + x)];
                        p[0] += L.x; p[1] += L.y; p[2] += L.z;
                    }
                }
            }
        } else {
#pragma omp parallel for schedule(dynamic, 16)
            for (int64_t pix = 0; pix < (int64_t)W * H; pix++) {
                Tape tp;
                XorShift x = seedCanonical(par.seed, t, (uint64_t)T + (uint64_t)pix);
                tp.fill(x, true);
                const double px = (pix % W) + tp.pop() - 0.5;
                const double py = (pix / W) + tp.pop() - 0.5;
                double* rec = queries.empty() ? nullptr : &queries[12 * (size_t)pix];
                if (rec) rec[11] = 0.0;
                const V L = radiance(cam.center, cam.ray(px, py), tp, rec);
                double* p = &buffer[3 * pix];
                p[0] += L.x; p[1] += L.y; p[2] += L.z;
            }
        }
        const auto t2 = std::chrono::steady_clock::now();
        msPhoton = std::chrono::duration<double, std::milli>(t1 - t0).count();
        msEye = std::chrono::duration<double, std::milli>(t2 - t1).count();
        if (compat) radius = (t + 1.0) / (t + par.alpha) * radius;
        else radius = radius * std::sqrt((t + par.alpha) / (t + 1.0));
        return PPPM_OK;
    }
};

}  // namespace port

using namespace port;

extern "C" {

struct port_pass_stats {
    double radius;
    int64_t stored;
    int64_t phantoms;
    double ms_photon;  // photon trace + photon map build
    double ms_eye;     // eye paths + gather
};

// Loads a scene: triangles, materials, env map (decoded floats, >= 64x64).
void* port_scene_create(const float* tri9, int64_t ntri, const int32_t* matId, const pppm_material* mats, int32_t nmat,
                        const float* env, int32_t ew, int32_t eh) {
    Scene* s = new Scene();
    s->tris.resize((size_t)ntri);
    for (int d = 0; d < 3; d++) { s->bmin[d] = kInf; s->bmax[d] = -kInf; }
    for (int64_t i = 0; i < ntri; i++) {
        const float* p = tri9 + 9 * i;
        s->tris[i] = {V(p[0], p[1], p[2]), V(p[3], p[4], p[5]), V(p[6], p[7], p[8])};
        for (int k = 0; k < 9; k++) {
            s->bmin[k % 3] = std::min(s->bmin[k % 3], (double)p[k]);
            s->bmax[k % 3] = std::max(s->bmax[k % 3], (double)p[k]);
        }
    }
    s->matId.assign(matId, matId + ntri);
    for (int i = 0; i < nmat; i++)
        s->mats.push_back({mats[i].type, mats[i].has_bssrdf != 0, V(mats[i].refl[0], mats[i].refl[1], mats[i].refl[2]),
                           (double)mats[i].phong_n});
    if (env && ew >= 64 && eh >= 64) {
        s->env.w = ew;
        s->env.h = eh;
        s->env.img.resize((size_t)ew * eh);
        for (size_t i = 0; i < s->env.img.size(); i++) s->env.img[i] = V(env[3 * i], env[3 * i + 1], env[3 * i + 2]);
        s->env.build();
    }
    s->bvh.build(s->tris);
    s->emit.assign((size_t)nmat, V());
    return s;
}

// Material mat emits rgb from the front side of its triangles; rebuilds the
// emitter list (scene order) and its area CDF as the GPU library does (edges
// subtracted in float, the cross product in double).
void port_scene_emission(void* sp, int32_t mat, const float* rgb) {
    Scene* s = static_cast<Scene*>(sp);
    s->emit[mat] = V(rgb[0], rgb[1], rgb[2]);
    s->lightTris.clear();
    s->lightCdf.clear();
    double total = 0.0;
    for (size_t i = 0; i < s->tris.size(); i++) {
        if (!s->emissive(s->matId[i])) continue;
        const Tri& t = s->tris[i];
        const float e1[3] = {(float)t.p1.x - (float)t.p0.x, (float)t.p1.y - (float)t.p0.y, (float)t.p1.z - (float)t.p0.z};
        const float e2[3] = {(float)t.p2.x - (float)t.p0.x, (float)t.p2.y - (float)t.p0.y, (float)t.p2.z - (float)t.p0.z};
        const double cx = (double)e1[1] * e2[2] - (double)e1[2] * e2[1];
        const double cy = (double)e1[2] * e2[0] - (double)e1[0] * e2[2];
        const double cz = (double)e1[0] * e2[1] - (double)e1[1] * e2[0];
        total += 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
        s->lightTris.push_back((int)i);
        s->lightCdf.push_back(total);
    }
    s->lightArea = total;
    for (double& c : s->lightCdf) c /= total;
    if (!s->lightCdf.empty()) s->lightCdf.back() = 1.0;
}

void port_scene_destroy(void* s) { delete static_cast<Scene*>(s); }

void port_env_tables(void* s, double* pdf, double* cdf) {
    const Scene* sc = static_cast<Scene*>(s);
    std::memcpy(pdf, sc->env.pdf.data(), 4096 * 8);
    std::memcpy(cdf, sc->env.cdf.data(), 4096 * 8);
}

void port_intersect(void* s, const float* rays, int64_t n, int32_t* tri, double* t) {
    const Scene* sc = static_cast<Scene*>(s);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
        const float* r = rays + 6 * i;
        tri[i] = sc->bvh.intersect(V(r[0], r[1], r[2]), V(r[3], r[4], r[5]), &t[i]);
    }
}

// Renders `passes` passes; accum: W*H*3 doubles (sum over passes), stats
// per pass. photons (optional, cap records of 13 doubles: position, flux,
// direction, normal, emitted path index or -1 for a phantom slot) receives
// the photon map of the last pass (each path's records in bounce order);
// returns the record count in *nphotons.
// queries (optional, W*H records of 12 doubles) receives each pixel's gather
// query of the last pass (radiance's rec; rec[11] = 0 where none).
int port_render(void* s, const pppm_camera* cam, const pppm_params* par, int32_t passes, double* accum,
                port_pass_stats* stats, double* photons, int64_t cap, int64_t* nphotons, double* queries) {
    const Scene* sc = static_cast<Scene*>(s);
    if (sc->env.w == 0 && sc->lightTris.empty()) return PPPM_E_STATE;
    Renderer R;
    R.sc = sc;
    R.par = *par;
    R.compat = par->mode == PPPM_MODE_COMPAT;
    R.N = par->num_streams;
    const double dx = sc->bmax[0] - sc->bmin[0], dy = sc->bmax[1] - sc->bmin[1], dz = sc->bmax[2] - sc->bmin[2];
    R.radius = norm(V(dx, dy, dz)) * par->radius_scale;
    for (int i = 0; i < R.N; i++) R.streams.push_back(XorShift((uint32_t)i));
    R.cam.center = V(cam->eye[0], cam->eye[1], cam->eye[2]);
    R.cam.dir = V(cam->dir[0], cam->dir[1], cam->dir[2]);
    const V up(cam->up[0], cam->up[1], cam->up[2]);
    R.cam.U = cross(R.cam.dir, up);
    R.cam.Vv = cross(R.cam.U, R.cam.dir);
    R.cam.halfTan = std::tan((double)cam->fov * 0.5);
    R.cam.aspect = (double)cam->width / (double)cam->height;
    R.cam.w = cam->width;
    R.cam.h = cam->height;
    R.buffer.assign((size_t)cam->width * cam->height * 3, 0.0);
    for (int t = 1; t <= passes; t++) {
        if (queries && t == passes) R.queries.assign((size_t)cam->width * cam->height * 12, 0.0);
        if (R.compat && (int)R.radius < 1) return PPPM_E_UNDEFINED;
        const double r = R.radius;
        const int rc = R.pass(t);
        if (rc) return rc;
        if (stats) stats[t - 1] = {r, R.stored, R.phantoms, R.msPhoton, R.msEye};
    }
    std::memcpy(accum, R.buffer.data(), R.buffer.size() * 8);
    if (queries && !R.queries.empty()) std::memcpy(queries, R.queries.data(), R.queries.size() * 8);
    if (nphotons) {
        *nphotons = (int64_t)R.lastPhotons.size();
        for (int64_t i = 0; i < std::min<int64_t>(cap, *nphotons); i++) {
            const Photon& p = R.lastPhotons[i];
            const double v[13] = {p.p.x, p.p.y, p.p.z, p.flux.x, p.flux.y, p.flux.z,
                                  p.dir.x, p.dir.y, p.dir.z, p.n.x, p.n.y, p.n.z, (double)p.path};
            std::memcpy(photons + 13 * i, v, sizeof(v));
        }
    }
    return PPPM_OK;
}

// Stage checks: kNN and gathers on explicit photons.
void port_knn(const float* pos, int64_t n, const float* q, int64_t m, int32_t numTarget, double targetRadius,
              int32_t* idx, int32_t* cnt, int32_t cap) {
    std::vector<Photon> ph((size_t)n);
    for (int64_t i = 0; i < n; i++) ph[i] = {V(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), V(), V((double)i, 0, 0), V()};
    KdTree kd;
    kd.build(ph);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t j = 0; j < m; j++) {
        std::vector<const Photon*> out;
        kd.query(V(q[3 * j], q[3 * j + 1], q[3 * j + 2]), true, (int)targetRadius, (double)numTarget, &out);
        cnt[j] = (int32_t)out.size();
        for (int t = 0; t < cap; t++) idx[j * cap + t] = t < (int)out.size() ? (int32_t)out[t]->dir.x : -1;
    }
}

// Canonical gather on explicit photons (pos, flux, oriented normal: 9
// doubles) and queries (pos, oriented normal, refl, weight: 12 doubles).
void port_gather_canonical(const double* ph9, int64_t n, const double* q12, int64_t m, double radius, double* out) {
    std::vector<Photon> ph((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const double* p = ph9 + 9 * i;
        ph[i] = {V(p[0], p[1], p[2]), V(p[3], p[4], p[5]), V(), V(p[6], p[7], p[8])};
    }
    KdTree kd;
    kd.build(ph);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t j = 0; j < m; j++) {
        const double* q = q12 + 12 * j;
        const V tot = kd.ballSum(V(q[0], q[1], q[2]), radius, V(q[3], q[4], q[5]));
        const V L = V(q[6], q[7], q[8]) * V(q[9], q[10], q[11]) * tot * kInvPi / (kPi * radius * radius);
        out[3 * j] = L.x;
        out[3 * j + 1] = L.y;
        out[3 * j + 2] = L.z;
    }
}

// Canonical gather bounds on explicit photons (9 doubles: pos, flux,
// normal) and queries (12 doubles: pos, oriented normal, weight, as
// port_gather_canonical with refl folded into the weight: refl = 1). A
// photon is ambiguous when a float32 implementation may decide it the
// other way: squared distance within d2band * r^2 of r^2, or normal dot
// within nband of zero. lo sums the photons inside for certain, hi adds the
// ambiguous ones, ref is the exact float64 gather; amb counts ambiguous
// photons, inside the photons ref sums. All m x 3 (amb, inside m) and divided
// by pi^2 r^2.
void port_gather_bounds(const double* ph9, int64_t n, const double* q12, int64_t m, double radius, double d2band,
                        double nband, double* lo, double* hi, double* ref, int64_t* amb, int64_t* inside) {
    std::vector<Photon> ph((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        const double* p = ph9 + 9 * i;
        ph[i] = {V(p[0], p[1], p[2]), V(p[3], p[4], p[5]), V(), V(p[6], p[7], p[8])};
    }
    KdTree kd;
    kd.build(ph);
    const double r2 = radius * radius;
    const double rq = radius * std::sqrt(1.0 + d2band);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t j = 0; j < m; j++) {
        const double* q = q12 + 12 * j;
        const V qp(q[0], q[1], q[2]), qn(q[3], q[4], q[5]);
        V sure, maybe, exact;
        int64_t na = 0, ni = 0;
        kd.forBall(qp, rq, [&](const Photon& p, double d) {
            const double d2 = d * d;
            const double c = dot(p.n, qn);
            const bool in = d2 < r2 * (1.0 - d2band) && c > nband;
            const bool amb = !in && ((std::abs(d2 - r2) <= d2band * r2 && c > -nband) || std::abs(c) <= nband);
            if (in) sure = sure + p.flux;
            if (amb) {
                maybe = maybe + p.flux;
                na++;
            }
            if (d < radius && c > 0.0) {
                exact = exact + p.flux;
                ni++;
            }
        });
        const V w = V(q[6], q[7], q[8]) * V(q[9], q[10], q[11]) * (1.0 / (kPi * kPi * r2));
        const V a = w * sure, b = a + w * maybe, e = w * exact;
        lo[3 * j] = a.x; lo[3 * j + 1] = a.y; lo[3 * j + 2] = a.z;
        hi[3 * j] = b.x; hi[3 * j + 1] = b.y; hi[3 * j + 2] = b.z;
        ref[3 * j] = e.x; ref[3 * j + 1] = e.y; ref[3 * j + 2] = e.z;
        amb[j] = na;
        inside[j] = ni;
    }
}

}  // extern "C"
