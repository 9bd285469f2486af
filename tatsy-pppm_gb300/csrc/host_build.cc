// Host preprocessing: QBVH with the reference topology, env importance
// tables, RGBE decoding. Compiled with -ffp-contract=off so the double
// arithmetic that mirrors the reference is rounded step by step.
#include "host_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>

namespace pppm {
namespace {

// A triangle as the builder sorts it: the reference's gravity()
// (triangle.cc:41-43) = (p0 + p1 + p2) / 3.0, where Vector3D's division by a
// scalar multiplies by 1.0 / s (vector3d.cc:145-152).
struct Item {
    double g[3];
    int id;
};

struct TempNode {
    float bmin[3][4], bmax[3][4];
    int child[4];  // >= 0: temp node index; < 0: leaf code
    int sep;
};

// The construction splits a range of n > 3 triangles into quarters of
// fixed sizes (half, then half of each half), so the number of inner nodes
// of a subtree depends on n alone. With those counts every subtree's place
// in the serial depth-first layout is known before it is built: a node's
// children follow it in child order, and a leaf's slots are its triangles'
// positions in the sorted item array. Subtrees of at least kTaskTris
// triangles, above kTaskDepth, are built as OpenMP tasks writing straight
// into their places, which gives the serial layout exactly (the sorts of
// disjoint ranges are independent; each range is sorted by the same
// std::sort call).
constexpr int kTaskTris = 1 << 14;
constexpr int kTaskDepth = 6;

void quarterSizes(int n, int* sz) {
    const int mid = n / 2;
    sz[0] = mid / 2;
    sz[1] = mid - mid / 2;
    sz[2] = mid / 2;
    sz[3] = n - mid - mid / 2;
}

struct Builder {
    const float* tri9;
    std::vector<Item> items;
    std::vector<TempNode> nodes;  // serial depth-first layout
    float* slots = nullptr;       // 12 floats per triangle, in leaf order
    std::map<int, int> innerNodes;  // inner nodes of a subtree of n triangles (read-only while building)

    int countInner(int n) {
        if (n <= 3) return 0;
        const auto it = innerNodes.find(n);
        if (it != innerNodes.end()) return it->second;
        int sz[4];
        quarterSizes(n, sz);
        int c = 1;
        for (int k = 0; k < 4; k++) c += countInner(sz[k]);
        innerNodes[n] = c;
        return c;
    }

    int makeLeaf(int lo, int hi) const {
        for (int i = lo; i < hi; i++) {
            const float* t = tri9 + 9 * (int64_t)items[i].id;
            float idbits;
            const int id = items[i].id;
            std::memcpy(&idbits, &id, 4);
            const float rec[12] = {t[0], t[1], t[2], idbits, t[3], t[4], t[5], 0.0f, t[6], t[7], t[8], 0.0f};
            std::memcpy(slots + 12 * (int64_t)i, rec, sizeof(rec));
        }
        return ~((lo << 2) | (hi - lo));
    }

    void box(int lo, int hi, float* mn, float* mx) const {
        double a[3] = {1e20, 1e20, 1e20}, b[3] = {-1e20, -1e20, -1e20};  // INFTY init (qbvh_accel.cc:55-56)
        for (int i = lo; i < hi; i++) {
            const float* t = tri9 + 9 * (int64_t)items[i].id;
            for (int j = 0; j < 3; j++)
                for (int d = 0; d < 3; d++) {
                    const double v = t[3 * j + d];
                    a[d] = std::min(a[d], v);
                    b[d] = std::max(b[d], v);
                }
        }
        for (int d = 0; d < 3; d++) { mn[d] = (float)a[d]; mx[d] = (float)b[d]; }
    }

    void sortRange(int lo, int hi, int dim) {
        std::sort(items.begin() + lo, items.begin() + hi,
                  [dim](const Item& x, const Item& y) { return x.g[dim] < y.g[dim]; });
    }

    // constructRec (qbvh_accel.cc:150-203) on items[lo, hi): its node at
    // nodes[at] (when inner); returns the subtree's code and, in *depthOut,
    // the deepest inner node's depth + 1 (0 for a leaf).
    int rec(int lo, int hi, int dim, int depth, int at, int* depthOut) {
        const int n = hi - lo;
        *depthOut = 0;
        if (n <= 3) return makeLeaf(lo, hi);
        sortRange(lo, hi, dim);
        const int mid = n / 2;
        const bool par = n >= kTaskTris && depth < kTaskDepth;
        if (par) {
#pragma omp task default(shared)
            sortRange(lo, lo + mid, (dim + 1) % 3);
#pragma omp task default(shared)
            sortRange(lo + mid, hi, (dim + 1) % 3);
#pragma omp taskwait
        } else {
            sortRange(lo, lo + mid, (dim + 1) % 3);
            sortRange(lo + mid, hi, (dim + 1) % 3);
        }
        const int cut[5] = {lo, lo + mid / 2, lo + mid, lo + mid + mid / 2, hi};
        float mn[4][3], mx[4][3];
        if (par) {
            for (int c = 0; c < 4; c++) {
#pragma omp task default(shared) firstprivate(c)
                box(cut[c], cut[c + 1], mn[c], mx[c]);
            }
#pragma omp taskwait
        } else {
            for (int c = 0; c < 4; c++) box(cut[c], cut[c + 1], mn[c], mx[c]);
        }
        TempNode nd;
        for (int c = 0; c < 4; c++)
            for (int d = 0; d < 3; d++) { nd.bmin[d][c] = mn[c][d]; nd.bmax[d][c] = mx[c][d]; }
        nd.sep = dim | (((dim + 1) % 3) << 2) | (((dim + 1) % 3) << 4);
        int start[4], depths[4];
        int next = at + 1;
        for (int c = 0; c < 4; c++) {
            start[c] = next;
            next += innerNodes.at(cut[c + 1] - cut[c]) ;
        }
        if (par) {
            for (int c = 0; c < 4; c++) {
#pragma omp task default(shared) firstprivate(c)
                nd.child[c] = rec(cut[c], cut[c + 1], (dim + 2) % 3, depth + 1, start[c], &depths[c]);
            }
#pragma omp taskwait
        } else {
            for (int c = 0; c < 4; c++)
                nd.child[c] = rec(cut[c], cut[c + 1], (dim + 2) % 3, depth + 1, start[c], &depths[c]);
        }
        nodes[at] = nd;
        int md = depth + 1;
        for (int c = 0; c < 4; c++) md = std::max(md, depths[c]);
        *depthOut = md;
        return at;
    }
};

}  // namespace

bool buildQbvh(const float* tri9, int64_t ntri, HostBvh* out, std::string* err) {
    if (ntri > (int64_t)(1 << 28)) {
        *err = "too many triangles (limit 2^28)";
        return false;
    }
    Builder b;
    b.tri9 = tri9;
    b.items.resize((size_t)ntri);
    const double third = 1.0 / 3.0;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < ntri; i++) {
        const float* t = tri9 + 9 * i;
        for (int d = 0; d < 3; d++) {
            const double s = ((double)t[d] + (double)t[3 + d]) + (double)t[6 + d];
            b.items[i].g[d] = s * third;
        }
        b.items[i].id = (int)i;
    }
    // inner-node counts of every subtree size the construction meets
    b.innerNodes[0] = 0;
    for (int k = 1; k <= 3; k++) b.innerNodes[k] = 0;
    b.nodes.resize((size_t)b.countInner((int)ntri));
    out->tris.resize((size_t)ntri * 12);
    b.slots = out->tris.data();
    int rootTemp = 0, depth = 0;
#pragma omp parallel
#pragma omp single
    rootTemp = b.rec(0, (int)ntri, 0, 0, 0, &depth);
    if (depth > 20) {
        *err = "QBVH deeper than 20 levels";
        return false;
    }
    out->depth = depth;
    out->nodes.clear();
    if (rootTemp < 0) {
        out->rootCode = rootTemp;
        return true;
    }
    const std::vector<TempNode>& allNodes = b.nodes;
    // BFS renumbering: top levels become contiguous from index 0 (the order
    // list is its own queue)
    std::vector<int> newIndex(allNodes.size(), -1);
    std::vector<int> order;
    order.reserve(allNodes.size());
    order.push_back(rootTemp);
    for (size_t head = 0; head < order.size(); head++) {
        const int v = order[head];
        newIndex[v] = (int)head;
        for (int c = 0; c < 4; c++)
            if (allNodes[v].child[c] >= 0) order.push_back(allNodes[v].child[c]);
    }
    out->nodes.resize(order.size());
    for (size_t k = 0; k < order.size(); k++) {
        const TempNode& t = allNodes[order[k]];
        HostQNode& h = out->nodes[k];
        std::memcpy(h.bmin, t.bmin, sizeof(h.bmin));
        std::memcpy(h.bmax, t.bmax, sizeof(h.bmax));
        for (int c = 0; c < 4; c++) h.child[c] = t.child[c] >= 0 ? newIndex[t.child[c]] : t.child[c];
        h.sep = t.sep;
    }
    out->rootCode = 0;
    return true;
}

void slotEdges(const float* slots, int64_t nslots, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nslots; k++) {
        const float* t = slots + 12 * k;
        double* e = out + 10 * k;
        for (int d = 0; d < 3; d++) {
            const double p0 = (double)t[d];
            e[d] = p0;
            e[3 + d] = (double)t[4 + d] - p0;
            e[6 + d] = (double)t[8 + d] - p0;
        }
        e[9] = 0.0;
    }
}

namespace {
const double kPi = 4.0 * std::atan(1.0);  // PI (common.h:14)

// Envmap::sampleFromDir (envmap.cc:47-60) in double.
void lookup(const float* rgb, int w, int h, double dx, double dy, double dz, double* out) {
    const double theta = std::acos(dy);
    double phi = std::atan2(dz, dx);
    if (phi < 0.0) phi += 2.0 * kPi;
    const double iblv = theta / kPi;
    const double iblu = phi / (2.0 * kPi);
    const double iblx = iblu * w;
    const double ibly = iblv * h;
    int ix = (int)iblx, iy = (int)ibly;
    ix = ix < 0 ? 0 : (ix > w - 1 ? w - 1 : ix);
    iy = iy < 0 ? 0 : (iy > h - 1 ? h - 1 : iy);
    const float* p = rgb + 3 * ((size_t)iy * w + ix);
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
}
}  // namespace

void envImportance(const float* rgb, int w, int h, std::vector<double>* pdf, std::vector<double>* cdf,
                   double exponent) {
    const int W = 64, H = 64;
    pdf->assign(W * H, 0.0);
    cdf->assign(W * H, 0.0);
    const int superX = w / W, superY = h / H;
    const double inv = 1.0 / (double)(superX * superY);
    // cells in parallel (each computed exactly as alone), then the total in
    // the reference's cell order
#pragma omp parallel for schedule(dynamic, 1)
    for (int iy = 0; iy < H; iy++) {
        for (int ix = 0; ix < W; ix++) {
            double acc[3] = {0.0, 0.0, 0.0};
            for (int sy = 0; sy < superY; sy++) {
                for (int sx = 0; sx < superX; sx++) {
                    const double u = (ix + static_cast<double>(sx) / superX) / W;
                    const double v = (iy + static_cast<double>(sy) / superY) / H;
                    const double phi = u * 2.0 * kPi;
                    const double y = (1.0 - v) * 2.0 - 1.0;
                    const double s = std::sqrt(1.0 - y * y);
                    double c[3];
                    lookup(rgb, w, h, s * std::cos(phi), y, s * std::sin(phi), c);
                    acc[0] += c[0] * inv;
                    acc[1] += c[1] * inv;
                    acc[2] += c[2] * inv;
                }
            }
            const double l = acc[0] * 0.2126 + acc[1] * 0.7152 + acc[2] * 0.0722;
            const double wgt = exponent == 2.0 ? l * l : std::pow(l, exponent);
            (*pdf)[iy * W + ix] = wgt;
        }
    }
    double total = 0.0;
    for (int i = 0; i < W * H; i++) total += (*pdf)[i];
    const double eps = 1.0e-12;
    (*pdf)[0] /= (total + eps);
    (*cdf)[0] = (*pdf)[0];
    for (int i = 1; i < W * H; i++) {
        (*pdf)[i] /= (total + eps);
        (*cdf)[i] = (*pdf)[i] + (*cdf)[i - 1];
    }
}

int decodeHdr(const uint8_t* bytes, int64_t n, float* rgb, int64_t capFloats, int* wOut, int* hOut) {
    int64_t pos = 0;
    auto getline = [&](std::string* line) -> bool {
        if (pos >= n) return false;
        line->clear();
        while (pos < n && line->size() < 4095) {
            const char c = (char)bytes[pos++];
            line->push_back(c);
            if (c == '\n') break;
        }
        return true;
    };
    std::string line;
    bool valid = false, rle = false;
    for (;;) {
        if (!getline(&line)) return -1;
        if (line[0] == '#') {
            if (line == "#?RADIANCE\n") valid = true;
        } else if (line.compare(0, 7, "FORMAT=") == 0) {
            if (line.compare(7, 15, "32-bit_rle_rgbe") == 0) rle = true;
        }
        if (line[0] == '\n') break;
    }
    if (!valid || !rle) return -1;
    if (!getline(&line)) return -1;
    char by[64] = {0}, bx[64] = {0};
    int w = 0, h = 0;
    if (std::sscanf(line.c_str(), "%63s %d %63s %d", by, &h, bx, &w) != 4) return -1;
    if (std::strcmp(by, "-Y") != 0 || std::strcmp(bx, "+X") != 0 || w <= 0 || h <= 0 || w > 65535 ||
        (int64_t)w * h > (int64_t)1 << 30)
        return -1;
    *wOut = w;
    *hOut = h;
    if (rgb == nullptr) return 0;
    if (capFloats < (int64_t)w * h * 3) return -4;
    std::vector<uint8_t> tmp((size_t)w * h * 4, 0);
    for (int y = 0; y < h; y++) {
        if (pos + 4 > n) return -1;
        if (bytes[pos] != 0x02 || bytes[pos + 1] != 0x02) return -1;  // only new-style RLE scanlines
        const int sw = (bytes[pos + 2] << 8) | bytes[pos + 3];
        pos += 4;
        if (sw != w) return -1;
        for (int ch = 0; ch < 4; ch++) {
            int x = 0;
            while (x < w) {
                if (pos >= n) return -1;
                const int info = bytes[pos++];
                if (info <= 128) {
                    if (x + info > w || pos + info > n) return -1;
                    for (int i = 0; i < info; i++) tmp[((size_t)y * w + x++) * 4 + ch] = bytes[pos++];
                } else {
                    const int cnt = info - 128;
                    if (x + cnt > w || pos >= n) return -1;
                    const uint8_t v = bytes[pos++];
                    for (int i = 0; i < cnt; i++) tmp[((size_t)y * w + x++) * 4 + ch] = v;
                }
            }
        }
    }
    for (size_t i = 0; i < (size_t)w * h; i++) {
        const int e = tmp[4 * i + 3];
        const double f = std::pow(2.0, e - 128.0) / 256.0;
        for (int c = 0; c < 3; c++) rgb[3 * i + c] = (float)(tmp[4 * i + c] * f);
    }
    return 0;
}

}  // namespace pppm
