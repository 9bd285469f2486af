// Host preprocessing: QBVH with the reference topology, env importance
// tables, RGBE decoding. Compiled with -ffp-contract=off so the double
// arithmetic that mirrors the reference is rounded step by step.
#include "host_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>

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

// Nodes and leaf slots of a subtree, as the serial construction would lay
// them out: the subtree's root first, then its children's subtrees in
// child order (depth-first); leaf slots in the same order.
struct Part {
    std::vector<TempNode> nodes;
    std::vector<float> slots;
    int maxDepth = 0;
};

// Subtrees of at least this many triangles, above this depth, are built as
// OpenMP tasks into parts of their own and appended in child order, which
// reproduces the serial layout exactly (the sorts of disjoint ranges are
// independent; each range is sorted by the same std::sort call).
constexpr int kTaskTris = 1 << 14;
constexpr int kTaskDepth = 6;

struct Builder {
    const float* tri9;
    std::vector<Item> items;

    int makeLeaf(Part& P, int lo, int hi) const {
        const int first = (int)(P.slots.size() / 12);
        for (int i = lo; i < hi; i++) {
            const float* t = tri9 + 9 * (int64_t)items[i].id;
            float idbits;
            const int id = items[i].id;
            std::memcpy(&idbits, &id, 4);
            const float rec[12] = {t[0], t[1], t[2], idbits, t[3], t[4], t[5], 0.0f, t[6], t[7], t[8], 0.0f};
            P.slots.insert(P.slots.end(), rec, rec + 12);
        }
        return ~((first << 2) | (hi - lo));
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

    // a child code of a part appended at (nodeOff, slotOff) of another
    static int shift(int code, int nodeOff, int slotOff) {
        if (code >= 0) return code + nodeOff;
        const int lc = ~code;
        return ~((((lc >> 2) + slotOff) << 2) | (lc & 3));
    }

    // constructRec (qbvh_accel.cc:150-203) on items[lo, hi), into P.
    int rec(Part& P, int lo, int hi, int dim, int depth) {
        const int n = hi - lo;
        if (n <= 3) return makeLeaf(P, lo, hi);
        P.maxDepth = std::max(P.maxDepth, depth + 1);
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
        TempNode nd;
        for (int c = 0; c < 4; c++) {
            float mn[3], mx[3];
            box(cut[c], cut[c + 1], mn, mx);
            for (int d = 0; d < 3; d++) { nd.bmin[d][c] = mn[d]; nd.bmax[d][c] = mx[d]; }
        }
        nd.sep = dim | (((dim + 1) % 3) << 2) | (((dim + 1) % 3) << 4);
        const int self = (int)P.nodes.size();
        P.nodes.push_back(nd);
        if (!par) {
            for (int c = 0; c < 4; c++) {
                const int code = rec(P, cut[c], cut[c + 1], (dim + 2) % 3, depth + 1);
                P.nodes[self].child[c] = code;
            }
            return self;
        }
        Part sub[4];
        int code[4];
        for (int c = 0; c < 4; c++) {
#pragma omp task default(shared) firstprivate(c)
            code[c] = rec(sub[c], cut[c], cut[c + 1], (dim + 2) % 3, depth + 1);
        }
#pragma omp taskwait
        for (int c = 0; c < 4; c++) {
            const int nodeOff = (int)P.nodes.size(), slotOff = (int)(P.slots.size() / 12);
            for (TempNode t : sub[c].nodes) {
                for (int k = 0; k < 4; k++) t.child[k] = shift(t.child[k], nodeOff, slotOff);
                P.nodes.push_back(t);
            }
            P.slots.insert(P.slots.end(), sub[c].slots.begin(), sub[c].slots.end());
            P.nodes[self].child[c] = shift(code[c], nodeOff, slotOff);
            P.maxDepth = std::max(P.maxDepth, sub[c].maxDepth);
        }
        return self;
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
    for (int64_t i = 0; i < ntri; i++) {
        const float* t = tri9 + 9 * i;
        for (int d = 0; d < 3; d++) {
            const double s = ((double)t[d] + (double)t[3 + d]) + (double)t[6 + d];
            b.items[i].g[d] = s * third;
        }
        b.items[i].id = (int)i;
    }
    Part all;
    int rootTemp = 0;
#pragma omp parallel
#pragma omp single
    rootTemp = b.rec(all, 0, (int)ntri, 0, 0);
    if (all.maxDepth > 20) {
        *err = "QBVH deeper than 20 levels";
        return false;
    }
    out->tris.swap(all.slots);
    out->depth = all.maxDepth;
    out->nodes.clear();
    if (rootTemp < 0) {
        out->rootCode = rootTemp;
        return true;
    }
    // BFS renumbering: top levels become contiguous from index 0.
    std::vector<int> newIndex(all.nodes.size(), -1);
    std::deque<int> q;
    q.push_back(rootTemp);
    int next = 0;
    std::vector<int> order;
    order.reserve(all.nodes.size());
    while (!q.empty()) {
        const int v = q.front();
        q.pop_front();
        newIndex[v] = next++;
        order.push_back(v);
        for (int c = 0; c < 4; c++)
            if (all.nodes[v].child[c] >= 0) q.push_back(all.nodes[v].child[c]);
    }
    out->nodes.resize(order.size());
    for (size_t k = 0; k < order.size(); k++) {
        const TempNode& t = all.nodes[order[k]];
        HostQNode& h = out->nodes[k];
        std::memcpy(h.bmin, t.bmin, sizeof(h.bmin));
        std::memcpy(h.bmax, t.bmax, sizeof(h.bmax));
        for (int c = 0; c < 4; c++) h.child[c] = t.child[c] >= 0 ? newIndex[t.child[c]] : t.child[c];
        h.sep = t.sep;
    }
    out->rootCode = 0;
    return true;
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
