// wf_noalloc.cu — neighbour search that allocates no device memory.
//
// wf_find_neighbors_static() gives the same lists as wf_find_neighbors()
// followed by wf_get_neighbors() (cuNSearch's float32 rule, candidates in the
// z, y, x cell order, ascending particle index inside a cell, at most 70 per
// particle), for callers that cannot call cudaMalloc: hosts whose framework
// owns every device allocation through its own pool or allocator, hosts that
// run under a fixed device-memory budget reserved up front, and code that must
// not allocate while other work runs on the device.  The caller passes device
// buffers for the positions and the output lists; the temporaries of the
// search (cell ids, cell counts and offsets, sorted indices and positions, the
// grid bounds, the scan's block sums) live in one file-scope device array,
// `g_static_scratch`, of fixed size.  Loading the library reserves it on every
// GPU the process uses, until the process exits.
//
// Sharing rules, stated in the header too: every call uses the same array and
// leaves its contents behind; each call clears what must start at zero (the
// grid bounds, the status word, the per-cell counters).  Two calls whose GPU
// work overlaps on one device (two streams, or two host threads at once) race
// on the array and give wrong lists; callers serialise them.
#include <climits>
#include <cstdio>
#include <mutex>

#include "wf_common.cuh"
#include "wf_nsearch.cuh"

namespace {

constexpr int64_t kMaxParticles = WF_STATIC_MAX_PARTICLES;
constexpr int64_t kMaxCells = WF_STATIC_MAX_CELLS;
constexpr int64_t kScanWords = 1024;   // block sums of a scan over kMaxCells + 1 entries

constexpr int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }
// byte offsets inside the scratch array
constexpr int64_t kOffHeader = 0;                                     // int[64]: bounds, status
constexpr int64_t kOffPos = kOffHeader + 256;                         // float4[n] positions
constexpr int64_t kOffSorted = kOffPos + align256(16 * kMaxParticles);   // float4[n] cell order
constexpr int64_t kOffCellId = kOffSorted + align256(16 * kMaxParticles);  // uint32[n]
constexpr int64_t kOffOrder = kOffCellId + align256(4 * kMaxParticles);    // int32[n] index
constexpr int64_t kOffStart = kOffOrder + align256(4 * kMaxParticles);     // uint32[cells + 1]
constexpr int64_t kOffCursor = kOffStart + align256(4 * (kMaxCells + 1));  // uint32[cells]
constexpr int64_t kOffScan = kOffCursor + align256(4 * kMaxCells);         // uint32[kScanWords]
constexpr int64_t kScratchBytes = kOffScan + align256(4 * kScanWords);
static_assert(kScratchBytes == WF_STATIC_SCRATCH_BYTES, "header and layout disagree");

// header words
constexpr int kHdrBounds = 0;   // int[6]: min cell x, y, z, max cell x, y, z
constexpr int kHdrStatus = 8;   // int: WF_STATUS_* bits

}  // namespace

// The device scratch.  In host code `g_static_scratch` names a host-side
// stand-in for the symbol, not a device address; the device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

namespace {

__device__ __forceinline__ int static_cell(float p, float gmin, float gdelta) {
  return (int)floorf(__fmul_rn(__fsub_rn(p, gmin), gdelta));
}

// resets the grid bounds and the status word left by the previous call; a
// launch of its own, so that it is ordered (by the stream) before every block
// of k_static_prep, whose blocks may flag a non-finite position in any order
__global__ void k_static_clear(int* __restrict__ hdr) {
  hdr[kHdrBounds + 0] = hdr[kHdrBounds + 1] = hdr[kHdrBounds + 2] = INT_MAX;
  hdr[kHdrBounds + 3] = hdr[kHdrBounds + 4] = hdr[kHdrBounds + 5] = INT_MIN;
  hdr[kHdrStatus] = 0;
}

// float positions from the caller's double3 array; flags non-finite ones
__global__ void k_static_prep(int64_t n, const double* __restrict__ x, float4* __restrict__ pf,
                              int* __restrict__ hdr) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x0 = x[3 * i], x1 = x[3 * i + 1], x2 = x[3 * i + 2];
  if (!isfinite(x0) || !isfinite(x1) || !isfinite(x2)) atomicOr(hdr + kHdrStatus, WF_STATUS_GRID);
  pf[i] = make_float4(__double2float_rn(x0), __double2float_rn(x1), __double2float_rn(x2), 0.0f);
}

__global__ void k_static_scatter(int64_t n, const uint32_t* __restrict__ cellid,
                                 const uint32_t* __restrict__ start, uint32_t* __restrict__ cursor,
                                 int32_t* __restrict__ order) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = cellid[i];
  order[start[c] + atomicAdd(cursor + c, 1u)] = (int32_t)i;
}

// ascending particle index inside each cell (insertion sort; a cell holds a
// few tens of particles at most)
__global__ void k_static_cell_sort(int64_t ncell, const uint32_t* __restrict__ start,
                                   int32_t* __restrict__ order) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const uint32_t b = start[c], e = start[c + 1];
  for (uint32_t k = b + 1; k < e; k++) {
    const int32_t v = order[k];
    uint32_t m = k;
    while (m > b && order[m - 1] > v) {
      order[m] = order[m - 1];
      m--;
    }
    order[m] = v;
  }
}

__global__ void k_static_gather(int64_t n, const int32_t* __restrict__ order,
                                const float4* __restrict__ pf, float4* __restrict__ sorted) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  sorted[k] = pf[order[k]];
}

// one thread per particle in cell order; writes row order[k] of the caller's
// row-major lists, neighbour indices in the caller's numbering
__global__ void __launch_bounds__(128) k_static_query(
    int64_t n, const float4* __restrict__ sorted, GridDev g, const uint32_t* __restrict__ start,
    const int32_t* __restrict__ order, int32_t* __restrict__ counts, int32_t* __restrict__ lists,
    int* status) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float4 p = sorted[k];
  const int cx = static_cell(p.x, g.gmin[0], g.gdelta[0]);
  const int cy = static_cell(p.y, g.gmin[1], g.gdelta[1]);
  const int cz = static_cell(p.z, g.gmin[2], g.gdelta[2]);
  const int64_t row = order[k];
  int32_t* out = lists + row * WF_MAX_NEIGHBORS;
  int count = 0;
  const int x0 = max(cx - 1, 0), x1 = min(cx + 1, g.dim[0] - 1);
  for (int z = -1; z < 2; z++) {
    const int fz = cz + z;
    if (fz < 0 || fz >= g.dim[2]) continue;
    for (int y = -1; y < 2; y++) {
      const int fy = cy + y;
      if (fy < 0 || fy >= g.dim[1] || x0 > x1) continue;
      const uint32_t rowc = ((uint32_t)fz * g.dim[1] + fy) * g.dim[0];
      const uint32_t b = start[rowc + x0], e = start[rowc + x1 + 1];
      for (uint32_t s = b; s < e; s++) {
        const float4 q = sorted[s];
        const float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
        const float sq =
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        if (sq < g.r2 && sq > 0.0f) {
          out[count++] = order[s];
          if (count == WF_MAX_NEIGHBORS) {
            counts[row] = count;
            atomicOr(status, WF_STATUS_NB_CAP);
            return;
          }
        }
      }
    }
  }
  counts[row] = count;
}

inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

void set_message(char* err, int64_t err_len, const char* msg) {
  if (err && err_len > 0) snprintf(err, (size_t)err_len, "%s", msg);
}

int fail(char* err, int64_t err_len, int code, const char* fmt, long long a = 0,
         long long b = 0) {
  char buf[256];
  snprintf(buf, sizeof buf, fmt, a, b);
  set_message(err, err_len, buf);
  return code;
}

int cuda_fail(char* err, int64_t err_len, cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  set_message(err, err_len, buf);
  return WF_ERR_CUDA;
}

// Device address of the scratch array on the current device.  The first call
// on each device looks it up with cudaGetSymbolAddress and caches it.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

cudaError_t scratch_on_current_device(unsigned char** out, int* dev_out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  *dev_out = dev;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// a pointer the kernels may dereference: device, managed or mapped host memory
bool device_accessible(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeHost && a.devicePointer != nullptr;
}

}  // namespace

extern "C" int wf_find_neighbors_static(const double* x, int64_t n, double h, int32_t* counts,
                                        int32_t* lists, void* stream, char* err,
                                        int64_t err_len) {
  set_message(err, err_len, "");
  if (n < 0) return fail(err, err_len, WF_ERR_ARG, "particle count %lld is negative", n);
  if (n > kMaxParticles)
    return fail(err, err_len, WF_ERR_ARG,
                "particle count %lld exceeds the static scratch limit of %lld particles "
                "(WF_STATIC_MAX_PARTICLES)",
                n, kMaxParticles);
  if (!(h > 0.0) || !(h < 1.0e30))
    return fail(err, err_len, WF_ERR_ARG, "smoothing length must be positive and finite");
  if (n == 0) return WF_OK;
  if (!x || !counts || !lists)
    return fail(err, err_len, WF_ERR_ARG, "null positions, counts or lists pointer");
  if (!device_accessible(x) || !device_accessible(counts) || !device_accessible(lists))
    return fail(err, err_len, WF_ERR_ARG,
                "positions, counts and lists must be device-accessible memory");

  unsigned char* base = nullptr;
  int dev = -1;
  cudaError_t e = scratch_on_current_device(&base, &dev);
  if (e != cudaSuccess) return cuda_fail(err, err_len, e, "scratch address (cudaGetSymbolAddress)");

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* hdr = reinterpret_cast<int*>(base + kOffHeader);
  float4* pf = reinterpret_cast<float4*>(base + kOffPos);
  float4* sorted = reinterpret_cast<float4*>(base + kOffSorted);
  uint32_t* cellid = reinterpret_cast<uint32_t*>(base + kOffCellId);
  int32_t* order = reinterpret_cast<int32_t*>(base + kOffOrder);
  uint32_t* start = reinterpret_cast<uint32_t*>(base + kOffStart);
  uint32_t* cursor = reinterpret_cast<uint32_t*>(base + kOffCursor);
  uint32_t* scan = reinterpret_cast<uint32_t*>(base + kOffScan);

  // grid bounds (cuNSearch kComputeMinMax, cuNSearchKernels.cu:41-71), read
  // back to size the cell arrays as computeCellInformation does
  const float r = (float)(2.0 * h);
  k_static_clear<<<1, 1, 0, s>>>(hdr);
  k_static_prep<<<blocks_for(n, 256), 256, 0, s>>>(n, x, pf, hdr);
  launch_minmax(n, pf, r, hdr + kHdrBounds, s);
  int head[kHdrStatus + 1];
  e = cudaMemcpyAsync(head, hdr, sizeof head, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(err, err_len, e, "grid bounds");
  if (head[kHdrStatus] & WF_STATUS_GRID)
    return fail(err, err_len, WF_ERR_ARG, "a position is not finite");
  const int* mm = head + kHdrBounds;
  for (int a = 0; a < 3; a++) {
    const int64_t span = (int64_t)mm[3 + a] - (int64_t)mm[a];
    if (span < 0 || span + 5 > kMaxCells)
      return fail(err, err_len, WF_ERR_ARG,
                  "positions span %lld search radii (2h) along an axis; the static scratch "
                  "holds %lld cells (WF_STATIC_MAX_CELLS)",
                  span, kMaxCells);
  }
  GridDev g;
  grid_from_minmax(mm, r, &g);
  int64_t ncell = 1;
  for (int a = 0; a < 3; a++) {
    if (g.dim[a] <= 0 || g.dim[a] > kMaxCells)
      return fail(err, err_len, WF_ERR_ARG,
                  "search grid needs %lld cells along an axis; the static scratch holds "
                  "%lld cells (WF_STATIC_MAX_CELLS)",
                  (long long)g.dim[a], kMaxCells);
    ncell *= g.dim[a];
    if (ncell > kMaxCells)
      return fail(err, err_len, WF_ERR_ARG,
                  "search grid needs more than %lld cells (positions span too many radii "
                  "2h); the static scratch holds %lld cells (WF_STATIC_MAX_CELLS)",
                  ncell, kMaxCells);
  }
  if (scan_tmp_words(ncell + 1) > kScanWords)
    return fail(err, err_len, WF_ERR_ARG, "scan of %lld cells exceeds the scratch", ncell);

  // counting sort by cell, ascending index inside a cell, then the queries
  e = cudaMemsetAsync(start, 0, sizeof(uint32_t) * (ncell + 1), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * ncell, s);
  if (e != cudaSuccess) return cuda_fail(err, err_len, e, "clear cell counters");
  launch_cell_count(n, pf, g, cellid, start, hdr + kHdrStatus, s);
  device_exclusive_scan(start, ncell + 1, scan, s);
  k_static_scatter<<<blocks_for(n, 256), 256, 0, s>>>(n, cellid, start, cursor, order);
  k_static_cell_sort<<<blocks_for(ncell, 256), 256, 0, s>>>(ncell, start, order);
  k_static_gather<<<blocks_for(n, 256), 256, 0, s>>>(n, order, pf, sorted);
  k_static_query<<<blocks_for(n, 128), 128, 0, s>>>(n, sorted, g, start, order, counts, lists,
                                                     hdr + kHdrStatus);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(err, err_len, e, "neighbour search launch");
  int status = 0;
  e = cudaMemcpyAsync(&status, hdr + kHdrStatus, sizeof status, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(err, err_len, e, "neighbour search");
  if (status & WF_STATUS_GRID)
    return fail(err, err_len, WF_ERR_NUMERIC,
                "a position is not finite or lies outside the search grid");
  return WF_OK;
}
