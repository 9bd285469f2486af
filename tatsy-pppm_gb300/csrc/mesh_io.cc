// Mesh input of the reference's scenes: the binary PLY reader of
// Trimesh::loadPly (trimesh.cc:139-217) and the placement helpers that the
// reference's drivers apply before Scene::add (Trimesh::translate, scale,
// putOnPlane, fitToBBox, trimesh.cc:272-320). Host code, no CUDA.
//
// The placement helpers work on double vertices with the reference's
// operations in its order (Vector3D arithmetic, std::min / std::max
// selection, no fused multiply-add), so the vertices equal the reference's
// bit for bit.
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/pppm_c.h"

namespace {

constexpr double kInfty = 1.0e20;  // INFTY (common.h:12)

// std::min / std::max as the reference calls them
inline double refMin(double a, double b) { return (b < a) ? b : a; }
inline double refMax(double a, double b) { return (a < b) ? b : a; }

// Splits off the next whitespace-separated token of [p, end), as
// `stringstream >> std::string` does; returns false when there is none.
bool token(const char*& p, const char* end, std::string* out) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
    if (p >= end) return false;
    const char* s = p;
    while (p < end && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
    out->assign(s, p);
    return true;
}

bool parseCount(const char*& p, const char* end, int64_t* v) {
    std::string t;
    if (!token(p, end, &t) || t.empty()) return false;
    int64_t x = 0;
    for (char ch : t) {
        if (ch < '0' || ch > '9') return false;
        x = x * 10 + (ch - '0');
        if (x > ((int64_t)1 << 40)) return false;
    }
    *v = x;
    return true;
}

}  // namespace

extern "C" {

int pppm_ply_decode(const uint8_t* bytes, int64_t nbytes, float* verts, int64_t vcap_floats, int32_t* faces,
                    int64_t fcap_ints, int64_t* nverts, int64_t* nfaces) {
    if (!bytes || nbytes <= 0 || !nverts || !nfaces) return PPPM_E_ARG;
    *nverts = 0;
    *nfaces = 0;
    const char* p = reinterpret_cast<const char*>(bytes);
    const char* end = p + nbytes;
    auto nextLine = [&](const char** ls, const char** le) -> bool {
        if (p >= end) return false;
        *ls = p;
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        *le = nl ? nl : end;
        p = nl ? nl + 1 : end;
        return true;
    };
    const char *ls, *le;
    // the identifier line must be exactly "ply"
    if (!nextLine(&ls, &le) || std::string(ls, le) != "ply") return PPPM_E_ARG;
    int64_t nv = 0, nf = 0;
    bool body = false;
    while (!body && nextLine(&ls, &le)) {
        const char* q = ls;
        std::string key, name;
        if (!token(q, le, &key)) continue;
        if (key == "format") {
            if (!token(q, le, &name) || name != "binary_little_endian") return PPPM_E_ARG;
        } else if (key == "element") {
            if (!token(q, le, &name)) return PPPM_E_ARG;
            if (name == "vertex") {
                if (!parseCount(q, le, &nv)) return PPPM_E_ARG;
            } else if (name == "face") {
                if (!parseCount(q, le, &nf)) return PPPM_E_ARG;
            } else {
                return PPPM_E_ARG;  // "Invalid element identifier"
            }
        } else if (key == "end_header") {
            body = true;
        }
        // "property", "comment" and anything else: ignored
    }
    // a header without end_header leaves the reference's mesh empty
    if (!body) return PPPM_OK;
    if (nv <= 0 || nf <= 0) return PPPM_E_ARG;
    // the reference reads 3 floats per vertex whatever properties the header
    // declares, then per face one uchar count and 3 ints
    const int64_t need = nv * 12 + nf * 13;
    if (end - p < need) return PPPM_E_ARG;
    *nverts = nv;
    *nfaces = nf;
    if (!verts && !faces) return PPPM_OK;
    if (!verts || !faces || vcap_floats < 3 * nv || fcap_ints < 3 * nf) return PPPM_E_CAPACITY;
    std::memcpy(verts, p, (size_t)nv * 12);
    p += nv * 12;
    for (int64_t i = 0; i < nf; i++) {
        const uint8_t count = (uint8_t)*p++;
        int32_t ii[3];
        std::memcpy(ii, p, 12);
        p += 12;
        // a polygon with more vertices ends the reference's program
        if (count > 3) return PPPM_E_ARG;
        for (int k = 0; k < 3; k++) {
            if (ii[k] < 0 || ii[k] >= nv) return PPPM_E_ARG;
            faces[3 * i + k] = ii[k];
        }
    }
    return PPPM_OK;
}

int pppm_mesh_translate(double* v, int64_t n, const double move[3]) {
    if ((n > 0 && (!v || !move)) || n < 0) return PPPM_E_ARG;
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) v[3 * i + d] = v[3 * i + d] + move[d];
    return PPPM_OK;
}

int pppm_mesh_scale(double* v, int64_t n, double sx, double sy, double sz) {
    if ((n > 0 && !v) || n < 0) return PPPM_E_ARG;
    for (int64_t i = 0; i < n; i++) {
        v[3 * i] = v[3 * i] * sx;
        v[3 * i + 1] = v[3 * i + 1] * sy;
        v[3 * i + 2] = v[3 * i + 2] * sz;
    }
    return PPPM_OK;
}

int pppm_mesh_put_on_plane(double* v, int64_t n, double distance, const double normal[3]) {
    if ((n > 0 && (!v || !normal)) || n < 0) return PPPM_E_ARG;
    double minval = kInfty;
    for (int64_t i = 0; i < n; i++) {
        const double d = normal[0] * v[3 * i] + normal[1] * v[3 * i + 1] + normal[2] * v[3 * i + 2];
        minval = refMin(minval, d);
    }
    const double s = minval + distance;
    const double m[3] = {normal[0] * s, normal[1] * s, normal[2] * s};
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) v[3 * i + d] = v[3 * i + d] - m[d];
    return PPPM_OK;
}

int pppm_mesh_fit_bbox(double* v, int64_t n, const double bmin[3], const double bmax[3]) {
    if ((n > 0 && (!v || !bmin || !bmax)) || n < 0) return PPPM_E_ARG;
    double lo[3] = {kInfty, kInfty, kInfty}, hi[3] = {-kInfty, -kInfty, -kInfty};
    for (int64_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = refMin(lo[d], v[3 * i + d]);
            hi[d] = refMax(hi[d], v[3 * i + d]);
        }
    double sc[3];
    for (int d = 0; d < 3; d++) sc[d] = (bmax[d] - bmin[d]) / (hi[d] - lo[d]);
    const double all = refMin(sc[0], refMin(sc[1], sc[2]));
    pppm_mesh_scale(v, n, all, all, all);
    const double half = 0.5 * all;
    double move[3];
    for (int d = 0; d < 3; d++) move[d] = (bmin[d] + bmax[d]) * 0.5 - (lo[d] + hi[d]) * half;
    return pppm_mesh_translate(v, n, move);
}

}  // extern "C"
