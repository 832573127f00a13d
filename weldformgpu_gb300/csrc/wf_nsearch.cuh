// wf_nsearch.cuh — neighbour-search launchers (wf_nsearch.cu).
#pragma once
#include <climits>
#include "wf_common.cuh"

struct GridDev {
  float gmin[3], gdelta[3], r2;
  int dim[3];
};

void grid_from_minmax(const int mm[6], float r, GridDev* g);
void device_exclusive_scan(uint32_t* data, int64_t n, uint32_t* tmp, cudaStream_t s);
int64_t scan_tmp_words(int64_t n);
void launch_prep_positions(int64_t n, const Fields& F, int use_current, float4* pf,
                           cudaStream_t s);
void launch_minmax(int64_t n, const float4* pf, float r, int* mm, cudaStream_t s);
void launch_cell_count(int64_t n, const float4* pf, const GridDev& g, uint32_t* cellid,
                       uint32_t* count, int* status, cudaStream_t s);
void launch_cell_scatter(int64_t n, const uint32_t* cellid, const uint32_t* start,
                         uint32_t* cursor, const int32_t* perm, int32_t* s_src, int32_t* s_orig,
                         cudaStream_t s);
void launch_cell_sort(int64_t ncell, const uint32_t* start, int32_t* s_src, int32_t* s_orig,
                      cudaStream_t s);
void launch_reorder(int64_t n, const int32_t* s_src, const Fields& A, const Fields& B,
                    const float4* pf, float4* pf2, int32_t* inv, cudaStream_t s);
void launch_nblist(int64_t n, int64_t npad, const float4* pf, const GridDev& g,
                   const uint32_t* start, const int32_t* slot_of, int32_t* nb, int32_t* cnt,
                   int* status, cudaStream_t s);
void launch_gather_pf(int64_t n, const int32_t* s_src, const float4* pf, float4* pf2,
                      cudaStream_t s);
void launch_snapshot(int64_t n, const Fields& F, cudaStream_t s);
