// Host side of the subsurface stage: Poisson-disc sampling of the BSSRDF
// surfaces as sampler::poissonDisk does it (sampler.cc:36-101). The dart
// throwing is sequential in a random order and its result depends on the
// reference's hash-grid buckets (including the |(int)x| folding of cells
// below the box minimum, hash_grid_detail.h:34-52), so it is reproduced
// here exactly; the candidates' random numbers come from an explicit
// XorShift state (the reference's is a process-wide static seeded 0).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <utility>
#include <vector>

#include "host_build.h"
#include "pppm_device.cuh"

namespace pppm {

namespace {

struct D3 {
    double x, y, z;
};
inline D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 mul(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline D3 cross(D3 u, D3 v) { return {u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

double realOf(XorShift& x) { return (double)x.next() * (double)(1.0f / 4294967295u); }

struct RefHashGrid {  // HashGrid<int> (hash_grid_detail.h)
    int size;
    double scale;
    D3 bmin;
    std::vector<std::vector<int>> data;
    uint32_t hash(int ix, int iy, int iz) const { return refHash(ix, iy, iz, (uint32_t)size); }
    std::vector<int>& at(D3 v) {
        const D3 b = mul(sub(v, bmin), scale);
        return data[hash(std::abs((int)b.x), std::abs((int)b.y), std::abs((int)b.z))];
    }
    void add(int id, D3 lo, D3 hi) {
        const D3 a = mul(sub(lo, bmin), scale), b = mul(sub(hi, bmin), scale);
        const int minZ = std::abs((int)a.z), maxZ = std::abs((int)b.z);
        const int minY = std::abs((int)a.y), maxY = std::abs((int)b.y);
        const int minX = std::abs((int)a.x), maxX = std::abs((int)b.x);
        for (int iz = minZ; iz <= maxZ; iz++)
            for (int iy = minY; iy <= maxY; iy++)
                for (int ix = minX; ix <= maxX; ix++) data[hash(ix, iy, iz)].push_back(id);
    }
};

}  // namespace

int64_t poissonDisk(const float* tri9, const std::vector<int64_t>& tris, double minDist, uint32_t rng[4],
                    std::vector<float>* points, std::vector<float>* normals) {
    XorShift x;
    for (int k = 0; k < 4; k++) x.s[k] = rng[k];
    std::vector<D3> cand, candN;
    D3 bmin = {1e20, 1e20, 1e20}, bmax = {-1e20, -1e20, -1e20};
    for (int64_t t : tris) {
        const float* p = tri9 + 9 * t;
        const D3 p0 = {p[0], p[1], p[2]}, p1 = {p[3], p[4], p[5]}, p2 = {p[6], p[7], p[8]};
        // Triangle::area uses p1-p0 and p2-p1 (triangle.cc:80-84)
        const D3 c = cross(sub(p1, p0), sub(p2, p1));
        const double A = 0.5 * std::sqrt(dot(c, c));
        const int nSample = (int)std::ceil(4.0 * A / (minDist * minDist));
        const D3 nc = cross(sub(p1, p0), sub(p2, p0));
        const D3 n = mul(nc, 1.0 / (std::sqrt(dot(nc, nc)) + 1e-12));
        for (int k = 0; k < nSample; k++) {
            double u = realOf(x), v = realOf(x);
            if (u + v >= 1.0) {
                u = 1.0 - u;
                v = 1.0 - v;
            }
            const D3 q = add(add(p0, mul(sub(p1, p0), u)), mul(sub(p2, p0), v));
            cand.push_back(q);
            candN.push_back(n);
            bmin = {std::min(bmin.x, q.x), std::min(bmin.y, q.y), std::min(bmin.z, q.z)};
            bmax = {std::max(bmax.x, q.x), std::max(bmax.y, q.y), std::max(bmax.z, q.z)};
        }
    }
    for (int k = 0; k < 4; k++) rng[k] = x.s[k];
    const int n = (int)cand.size();
    points->clear();
    normals->clear();
    if (n == 0) return 0;
    RefHashGrid grid;
    grid.size = n;
    grid.scale = 1.0 / (2.0 * minDist);
    grid.bmin = bmin;
    grid.data.assign(n, std::vector<int>());
    // RandomQueue<int> with seed -1 (random_queue.h:20,66-73)
    XorShift q;
    q.seed((uint32_t)-1);
    std::vector<int> que(n);
    for (int i = 0; i < n; i++) que[i] = i;
    size_t pos = (size_t)n;
    const D3 margin = {2.0 * minDist, 2.0 * minDist, 2.0 * minDist};
    const double d2 = minDist * minDist;
    while (pos != 0) {
        const int r = std::abs((int)q.next()) % (int)pos;  // XorShift::nextInt
        pos--;
        std::swap(que[r], que[pos]);
        const int id = que[pos];
        const D3 v = cand[id];
        std::vector<int>& cell = grid.at(v);
        bool accept = true;
        for (int k : cell) {
            const D3 d = sub(cand[k], v);
            if (dot(d, d) <= d2) {
                accept = false;
                break;
            }
        }
        if (accept) {
            grid.add(id, sub(v, margin), add(v, margin));
            points->insert(points->end(), {(float)v.x, (float)v.y, (float)v.z});
            normals->insert(normals->end(), {(float)candN[id].x, (float)candN[id].y, (float)candN[id].z});
        }
    }
    return (int64_t)(points->size() / 3);
}

}  // namespace pppm
