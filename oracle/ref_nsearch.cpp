/*
 * ref_nsearch.cpp — runs cuNSearch's own neighbour kernels on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY: compiled by oracle/build_ref.py into
 * oracle/_ref/ from the sources under the reference tree; never shipped.
 *
 * The kernels (kComputeMinMax, kInsertParticles_Morton, kCountingSortIndices,
 * kComputeCounts, kNeighborhoodQueryWithCounts) are the reference's,
 * included verbatim from src/cuNSearch/src/cuNSearchKernels.cu.  This file
 * only restates the host glue of cuNSearchDeviceData.cu:27-293 (grid set-up,
 * scans, gather) and launches each kernel as a sequential loop over its
 * thread index.  Run sequentially, kInsertParticles_Morton's atomicAdd hands
 * out in-cell slots in ascending particle order, so the neighbour order is
 * the deterministic one the oracle uses.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "cuda_host_shim.h"
#include "cuNSearchKernels.cu"

template <class F>
static void launch_seq(uint32_t n, F&& f) {
  blockDim = dim3(1, 1, 1);
  blockIdx = make_uint3(0, 0, 0);
  for (uint32_t t = 0; t < n; t++) {
    threadIdx = make_uint3(t, 0, 0);
    f();
  }
}

extern "C" int wfr_neighbors(const double* x, int64_t n64, double h_glob, int32_t* counts,
                             int32_t* lists /* n*70 */) {
  const uint32_t n = (uint32_t)n64;
  if (n == 0) return 0;
  /* SolverFraser.cu:72-82: radius = 2*h_glob, stored as Real (float). */
  double radius = 2.0 * h_glob;
  float searchRadius = (float)radius;
  std::vector<float3> pts(n);
  for (uint32_t i = 0; i < n; i++)                   /* SolverFraser.cu:63-69 */
    pts[i] = make_float3((float)x[3 * i], (float)x[3 * i + 1], (float)x[3 * i + 2]);

  /* computeMinMax (cuNSearchDeviceData.cu:27-60) */
  int3 mm[2];
  mm[0] = make_int3(std::numeric_limits<int>().max(), std::numeric_limits<int>().max(),
                    std::numeric_limits<int>().max());
  mm[1] = make_int3(std::numeric_limits<int>().min(), std::numeric_limits<int>().min(),
                    std::numeric_limits<int>().min());
  launch_seq(n, [&] { kComputeMinMax(pts.data(), n, searchRadius, &mm[0], &mm[1]); });
  float3 Min = make_float3(mm[0].x * searchRadius, mm[0].y * searchRadius, mm[0].z * searchRadius);
  float3 Max = make_float3(mm[1].x * searchRadius, mm[1].y * searchRadius, mm[1].z * searchRadius);

  /* computeCellInformation (cuNSearchDeviceData.cu:80-174) */
  GridInfo gi;
  gi.ParticleCount = n;
  gi.SquaredSearchRadius = searchRadius * searchRadius;
  gi.GridMin = Min;
  float cellSize = searchRadius;
  float3 gridSize = Max - Min;
  gi.GridDimension.x = static_cast<unsigned int>(ceil(gridSize.x / cellSize));
  gi.GridDimension.y = static_cast<unsigned int>(ceil(gridSize.y / cellSize));
  gi.GridDimension.z = static_cast<unsigned int>(ceil(gridSize.z / cellSize));
  gi.GridDimension.x += 4;
  gi.GridDimension.y += 4;
  gi.GridDimension.z += 4;
  gi.GridMin -= make_float3(cellSize, cellSize, cellSize) * (float)2;
  gi.MetaGridDimension.x = static_cast<unsigned int>(ceil(gi.GridDimension.x / (float)CUDA_META_GRID_GROUP_SIZE));
  gi.MetaGridDimension.y = static_cast<unsigned int>(ceil(gi.GridDimension.y / (float)CUDA_META_GRID_GROUP_SIZE));
  gi.MetaGridDimension.z = static_cast<unsigned int>(ceil(gi.GridDimension.z / (float)CUDA_META_GRID_GROUP_SIZE));
  gridSize.x = gi.GridDimension.x * cellSize;
  gridSize.y = gi.GridDimension.y * cellSize;
  gridSize.z = gi.GridDimension.z * cellSize;
  gi.GridDelta.x = gi.GridDimension.x / gridSize.x;
  gi.GridDelta.y = gi.GridDimension.y / gridSize.y;
  gi.GridDelta.z = gi.GridDimension.z / gridSize.z;
  uint64_t numberOfCells = (uint64_t)(gi.MetaGridDimension.x * gi.MetaGridDimension.y *
                                      gi.MetaGridDimension.z) * CUDA_META_GRID_BLOCK_SIZE;

  std::vector<uint> cellIdx(n), tempSort(n), sortIdx(n), revSort(n);
  std::vector<uint> cellCounts(numberOfCells, 0u), cellOffsets(numberOfCells, 0u);
  launch_seq(n, [&] {
    kInsertParticles_Morton(gi, pts.data(), cellIdx.data(), cellCounts.data(), tempSort.data());
  });
  uint acc = 0;                                       /* thrust::exclusive_scan */
  for (uint64_t c = 0; c < numberOfCells; c++) { cellOffsets[c] = acc; acc += cellCounts[c]; }
  launch_seq(n, [&] {
    kCountingSortIndices(gi, cellIdx.data(), cellOffsets.data(), tempSort.data(), sortIdx.data());
  });
  for (uint32_t k = 0; k < n; k++) revSort[k] = sortIdx[k];  /* gather of a sequence */

  /* computeNeighborhood (cuNSearchDeviceData.cu:176-247) */
  std::vector<uint> nbCounts(n), nbOffsets(n);
  launch_seq(n, [&] {
    kComputeCounts(pts.data(), n, gi, pts.data(), cellOffsets.data(), cellCounts.data(),
                   nbCounts.data(), revSort.data());
  });
  uint total = 0;
  for (uint32_t i = 0; i < n; i++) { nbOffsets[i] = total; total += nbCounts[i]; }
  std::vector<uint> nbs(total ? total : 1);
  launch_seq(n, [&] {
    kNeighborhoodQueryWithCounts(pts.data(), n, gi, pts.data(), cellOffsets.data(),
                                 cellCounts.data(), nbOffsets.data(), nbs.data(), revSort.data());
  });
  for (uint32_t i = 0; i < n; i++) {
    counts[i] = (int32_t)nbCounts[i];
    for (uint k = 0; k < nbCounts[i]; k++) lists[(size_t)i * 70 + k] = (int32_t)nbs[nbOffsets[i] + k];
  }
  return 0;
}
