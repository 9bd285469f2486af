// Host-side preprocessing for the device layouts: QBVH construction with the
// reference's topology, env-map importance tables, RGBE decoding.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pppm {

struct HostQNode {
    float bmin[3][4];
    float bmax[3][4];
    int child[4];
    int sep;  // sep0 | sep1 << 2 | sep2 << 4
};

struct HostBvh {
    std::vector<HostQNode> nodes;  // BFS order, nodes[0] = root when root is inner
    std::vector<float> tris;       // slot-ordered triangles, 12 floats each (3 x float4, p0.w = id bits)
    int rootCode = 0;              // node index (>= 0) or leaf code (< 0)
    int depth = 0;                 // inner-node levels
};

// QBVHAccel::construct / constructRec (qbvh_accel.cc:139-203). Returns false
// with `err` set when the tree would exceed the device stack bound.
bool buildQbvh(const float* tri9, int64_t ntri, HostBvh* out, std::string* err);

// The exact triangle test's operands of each 12-float slot of
// HostBvh::tris: the double vertex p0 = (double)a and the edges
// e1 = (double)b - p0, e2 = (double)c - p0, 10 doubles per slot (the last 0),
// the operations the device test would otherwise repeat per ray.
void slotEdges(const float* slots, int64_t nslots, double* out);

// Envmap::createImportanceMap (envmap.cc:88-163): 64x64 cell pdf/cdf over
// super-sampled directions, cell weight luminance^exponent (2 in the
// reference: l * l).
void envImportance(const float* rgb, int w, int h, std::vector<double>* pdf, std::vector<double>* cdf,
                   double exponent = 2.0);

// Image::loadHdr (image.cc:296-434) on an in-memory file. Returns 0 or a
// negative code; with rgb == nullptr only reports the size.
int decodeHdr(const uint8_t* bytes, int64_t n, float* rgb, int64_t capFloats, int* w, int* h);

}  // namespace pppm
