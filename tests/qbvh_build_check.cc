// Builds QBVHs of seeded random triangle soups (with repeated centroids, so
// the sorts meet ties) and prints a hash of each build's nodes, leaf slots,
// root and depth, one line per size. tests/test_host_build.py runs it with
// one and with several OpenMP threads: the parallel construction must lay
// the tree out exactly as the serial one. The slots' double edges
// (slotEdges) are checked against the serial formula bit for bit; a
// mismatch prints an error line.
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "host_build.h"

namespace {
unsigned long long fnv(const void* p, size_t n, unsigned long long h) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}
}  // namespace

int main() {
    for (int n : {1, 3, 4, 17, 1000, 16384, 70000, 200000}) {
        std::vector<float> t(9 * (size_t)n);
        std::mt19937 rng(n);
        std::uniform_real_distribution<float> u(-10.0f, 10.0f);
        for (int i = 0; i < n; i++) {
            const float c[3] = {u(rng), u(rng), u(rng)};
            for (int j = 0; j < 9; j++)
                t[9 * (size_t)i + j] = (i % 7 == 3) ? t[9 * (size_t)(i - 1) + j] : c[j % 3] + 0.01f * u(rng);
        }
        pppm::HostBvh b;
        std::string err;
        if (!pppm::buildQbvh(t.data(), n, &b, &err)) {
            std::printf("%d error %s\n", n, err.c_str());
            continue;
        }
        const size_t slots = b.tris.size() / 12;
        std::vector<double> edges(slots * 10 + 1, -1.0);
        pppm::slotEdges(b.tris.data(), (int64_t)slots, edges.data());
        bool same = edges[slots * 10] == -1.0;  // nothing past the last slot
        for (size_t k = 0; k < slots && same; k++) {
            const float* t = &b.tris[12 * k];
            for (int d = 0; d < 3; d++) {
                const double p0 = (double)t[d];
                const double want[3] = {p0, (double)t[4 + d] - p0, (double)t[8 + d] - p0};
                for (int j = 0; j < 3; j++)
                    same = same && std::memcmp(&edges[10 * k + 3 * j + d], &want[j], sizeof(double)) == 0;
            }
            same = same && edges[10 * k + 9] == 0.0;
        }
        if (!same) std::printf("%d error slot edges\n", n);
        unsigned long long h = 1469598103934665603ull;
        h = fnv(b.nodes.data(), b.nodes.size() * sizeof(pppm::HostQNode), h);
        h = fnv(b.tris.data(), b.tris.size() * sizeof(float), h);
        h = fnv(&b.rootCode, sizeof(b.rootCode), h);
        h = fnv(&b.depth, sizeof(b.depth), h);
        std::printf("%d %zu %016llx\n", n, b.nodes.size(), h);
    }
    return 0;
}
