// Launchers shared between the C-ABI files.
#pragma once

#include "context.h"
#include "grid.cuh"

namespace pppm {

constexpr int kMaxKnn = 64;  // largest k of the compat kNN gather

// Query record of the gather: q0 = (pos, pixel bits), q1 = (normal, 0),
// q2 = (weight = path throughput * refl / roulette, 0).
struct QueryView {
    const float4* q;      // 3 float4 per query
    const uint32_t* count;  // device count (nullptr: use n)
    int64_t n;
};

cudaError_t exclusiveScan(uint32_t* data, int64_t n, uint32_t* cursor, uint32_t* tmp, cudaStream_t st);
int64_t scanTmpWords(int64_t n);
cudaError_t gridLayout(GridBufs& g, const double* bbmin, const double* bbmax, double cell, int64_t nPhotons);
GridDev gridView(const GridBufs& g, const double* bbmin, const double* bbmax);
// Origin, cell edge and cells per axis of the grid gridLayout would give.
GridDev gridGeometry(const double* bbmin, const double* bbmax, double cell);
cudaError_t gridBuild(GridBufs& g, const GridDev& view, const float4* rec, const uint64_t* dCount, int64_t capacity,
                      cudaStream_t st, bool withOwner = false);

// Canonical gather with shared-memory staging of cell neighbourhoods
// (queries counting-sorted by cell first). work: optional 2 counters.
cudaError_t querySortLayout(QuerySortBufs& qs, int64_t maxQueries);
cudaError_t launchGatherTiled(const GridDev& g, QueryView q, QuerySortBufs& qs, float radius, float* out,
                              bool accumulate, unsigned long long* work, cudaStream_t st);
// The two halves of launchGatherTiled: the query sort needs only the grid's
// geometry (gridGeometry), so it can run as soon as the queries exist; the
// gather then reads the sorted queries.
cudaError_t querySort(const GridDev& geometry, QueryView q, QuerySortBufs& qs, cudaStream_t st);
cudaError_t launchGatherSorted(const GridDev& g, QueryView q, QuerySortBufs& qs, float radius, float* out,
                               bool accumulate, unsigned long long* work, cudaStream_t st);
// Compat kNN gather (ppm_probabilistic.cc:300-335; irradianceWithPM,
// subsurface_integrator.cc:329-365): k nearest within eps, normal filter
// |n.(q-p)|/|q-p| < rlim, cone filter, output scaled by the query weight.
cudaError_t launchGatherCompat(const GridDev& g, QueryView q, int k, float eps, float rlim, int64_t phantoms,
                               float* out, bool accumulate, cudaStream_t st);
// kNN only (PhotonMap::findKNN): idx in farthest-first order.
cudaError_t launchKnn(const GridDev& g, const float* queries, int64_t m, int k, float eps, int32_t* idx, int32_t* cnt,
                      int cap, cudaStream_t st);

// Photon records from plain arrays (pos xyz, flux xyz, normal bits, id).
cudaError_t launchPackPhotons(const float* in8, int64_t n, float4* rec, uint64_t* count, cudaStream_t st);
cudaError_t launchPackPositions(const float* pos3, int64_t n, float4* rec, uint64_t* count, cudaStream_t st);
cudaError_t launchPackQueries(const float* in12, int64_t m, float4* q, cudaStream_t st);
cudaError_t launchUnpackRecords(const float4* rec, int64_t n, float* out, cudaStream_t st);

}  // namespace pppm
