// wf_tiles.cu — builds the neighbour halos of the slot tiles (wf_tiles.cuh).
//
// One block per tile, one thread per slot.  The tile's list entries (and its
// own slots) lie in a window [lo, hi] of slots: with cell-sorted slots that
// window is about two cell layers wide, while the halo itself is a few times
// the tile.  The block marks every entry in a shared-memory bitmap of the
// window, an exclusive scan of the words' popcounts numbers the marked slots
// in ascending order, the numbered slots become the halo, and each entry is
// rewritten as its slot's number (its rank in the bitmap).  Rebuilt with the
// lists, every neighbour rebuild.
#include <climits>

#include "wf_common.cuh"
#include "wf_tiles.cuh"

namespace {

constexpr int kT = WF_TILE;
constexpr int kWarps = kT / 32;

__global__ void __launch_bounds__(kT) k_tile_halo(int64_t n, int64_t npad,
                                                  const int32_t* __restrict__ nb,
                                                  const int32_t* __restrict__ cnt,
                                                  int32_t* __restrict__ hoff,
                                                  int32_t* __restrict__ hcnt,
                                                  int32_t* __restrict__ halo, int64_t halo_cap,
                                                  uint16_t* __restrict__ nbl, int cap,
                                                  unsigned* __restrict__ halo_used,
                                                  int* __restrict__ hmax) {
  extern __shared__ uint32_t sm[];
  uint32_t* bits = sm;                       // [WF_TILE_WIN_WORDS]
  uint32_t* pre = sm + WF_TILE_WIN_WORDS;    // [WF_TILE_WIN_WORDS]
  __shared__ int s_lo[kWarps], s_hi[kWarps];
  __shared__ uint32_t s_sum[kWarps];
  __shared__ int s_base;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tile = blockIdx.x;
  const int64_t i = tile * kT + tid;
  const bool valid = i < n;
  const int c = valid ? cnt[i] : 0;
  // the window of slots the tile's lists name
  int lo = valid ? (int)i : INT_MAX, hi = valid ? (int)i : INT_MIN;
  for (int k = 0; k < c; k++) {
    const int s = nb[nb_at(npad, i, k)];
    lo = min(lo, s);
    hi = max(hi, s);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) { s_lo[warp] = lo; s_hi[warp] = hi; }
  __syncthreads();
  lo = s_lo[0];
  hi = s_hi[0];
  for (int w = 1; w < kWarps; w++) { lo = min(lo, s_lo[w]); hi = max(hi, s_hi[w]); }
  if (lo > hi) {                             // a tile past the last particle
    if (tid == 0) { hcnt[tile] = 0; hoff[tile] = 0; }
    return;
  }
  const int64_t span = (int64_t)hi - lo + 1;
  const int words = (int)((span + 31) >> 5);
  if (words > WF_TILE_WIN_WORDS) {           // uniform: the window does not fit
    if (tid == 0) { hcnt[tile] = -1; hoff[tile] = 0; }
    return;
  }
  for (int w = tid; w < words; w += kT) bits[w] = 0u;
  __syncthreads();
  if (valid) {
    const int o = (int)i - lo;
    atomicOr(bits + (o >> 5), 1u << (o & 31));
    for (int k = 0; k < c; k++) {
      const int q = nb[nb_at(npad, i, k)] - lo;
      atomicOr(bits + (q >> 5), 1u << (q & 31));
    }
  }
  __syncthreads();
  // exclusive scan of the words' popcounts: thread t takes words [t per, (t+1) per)
  const int per = (words + kT - 1) / kT;
  const int w0 = min(words, tid * per), w1 = min(words, w0 + per);
  uint32_t own = 0;
  for (int w = w0; w < w1; w++) own += __popc(bits[w]);
  uint32_t incl = own;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_sum[warp] = incl;
  __syncthreads();
  uint32_t before = 0, total = 0;
  for (int w = 0; w < kWarps; w++) {
    if (w < warp) before += s_sum[w];
    total += s_sum[w];
  }
  uint32_t run = before + incl - own;
  for (int w = w0; w < w1; w++) {
    pre[w] = run;
    run += __popc(bits[w]);
  }
  const int H = (int)total;
  if (tid == 0) {
    atomicMax(hmax, H);
    int base = -1;
    if (H <= cap) {
      const unsigned want = ((unsigned)H + 3u) & ~3u;
      const unsigned at = atomicAdd(halo_used, want);
      if ((int64_t)at + want <= halo_cap) base = (int)at;
    }
    s_base = base;
    hoff[tile] = base < 0 ? 0 : base;
    hcnt[tile] = base < 0 ? -1 : H;
  }
  __syncthreads();
  const int base = s_base;
  if (base < 0) return;                      // uniform: too large, or no room left
  // the halo: marked slots in ascending order
  for (int w = tid; w < words; w += kT) {
    uint32_t m = bits[w];
    int at = base + (int)pre[w];
    while (m) {
      const int b = __ffs(m) - 1;
      halo[at++] = lo + 32 * w + b;
      m &= m - 1u;
    }
  }
  // the local lists: each entry's rank in the bitmap (padding: the own slot)
  if (valid) {
    const int cend = (c + WF_NB_BLK - 1) & ~(WF_NB_BLK - 1);
    for (int k = 0; k < cend; k++) {
      const int s = k < c ? nb[nb_at(npad, i, k)] : (int)i;
      const int q = s - lo;
      const uint32_t wv = bits[q >> 5];
      const int r = (int)pre[q >> 5] + __popc(wv & ((1u << (q & 31)) - 1u));
      nbl[nb_at(npad, i, k)] = (uint16_t)r;
    }
  }
}

// 16-bit lists: the tile's window [lo, hi] of named slots; when it spans at
// most 65,536 slots every entry (padding included) becomes slot - lo.
__global__ void __launch_bounds__(kT) k_list16(int64_t n, int64_t npad,
                                               const int32_t* __restrict__ nb,
                                               const int32_t* __restrict__ cnt,
                                               int32_t* __restrict__ base,
                                               uint16_t* __restrict__ off) {
  __shared__ int s_lo[kWarps], s_hi[kWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tile = blockIdx.x;
  const int64_t i = tile * kT + tid;
  const bool valid = i < n;
  const int c = valid ? cnt[i] : 0;
  int lo = valid ? (int)i : INT_MAX, hi = valid ? (int)i : INT_MIN;
  for (int k = 0; k < c; k++) {
    const int s = nb[nb_at(npad, i, k)];
    lo = min(lo, s);
    hi = max(hi, s);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) { s_lo[warp] = lo; s_hi[warp] = hi; }
  __syncthreads();
  lo = s_lo[0];
  hi = s_hi[0];
  for (int w = 1; w < kWarps; w++) { lo = min(lo, s_lo[w]); hi = max(hi, s_hi[w]); }
  const bool fits = lo <= hi && (int64_t)hi - lo < 65536;
  if (tid == 0) base[tile] = fits ? lo : -1;
  if (!fits || !valid) return;
  const int cend = (c + WF_NB_BLK - 1) & ~(WF_NB_BLK - 1);
  for (int k = 0; k < cend; k++) {
    const int s = k < c ? nb[nb_at(npad, i, k)] : (int)i;
    off[nb_at(npad, i, k)] = (uint16_t)(s - lo);
  }
}

}  // namespace

void launch_list16(int64_t n, int64_t npad, const int32_t* nb, const int32_t* cnt, int32_t* base,
                   uint16_t* off, cudaStream_t s) {
  k_list16<<<(unsigned)(npad / WF_TILE), WF_TILE, 0, s>>>(n, npad, nb, cnt, base, off);
}

void launch_tile_halo(int64_t n, int64_t npad, const int32_t* nb, const int32_t* cnt,
                      int32_t* hoff, int32_t* hcnt, int32_t* halo, int64_t halo_cap,
                      uint16_t* nbl, int cap, unsigned* halo_used, int* hmax, cudaStream_t s) {
  const int64_t tiles = npad / WF_TILE;
  const size_t smem = 2 * sizeof(uint32_t) * WF_TILE_WIN_WORDS;
  static size_t opted[64] = {};
  opt_in_smem(k_tile_halo, smem, opted);
  k_tile_halo<<<(unsigned)tiles, WF_TILE, smem, s>>>(n, npad, nb, cnt, hoff, hcnt, halo,
                                                     halo_cap, nbl, cap, halo_used, hmax);
}
