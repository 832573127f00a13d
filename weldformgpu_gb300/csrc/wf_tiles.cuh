// wf_tiles.cuh — neighbour halos of slot tiles, for the staged pair passes.
//
// A tile is WF_TILE consecutive slots, the particles of one block of a mixed
// pair pass.  Its halo is the ascending list of distinct slots that its
// particles' neighbour lists name (its own slots included).  The block copies
// the halo's gathered records (positions, velocities, ...) into shared memory
// once, with asynchronous 16-byte copies, and its threads then read their
// neighbours from shared memory through local lists: 16-bit indices into the
// halo, stored like the slot lists (blocks of 8 entries, nb_at).  The
// neighbours are the same, in the same order, so the FP32 sums are those of
// the unstaged passes bit for bit.
#pragma once
#include "wf_common.cuh"

#define WF_TILE 128                 // slots per tile
#define WF_TILE_HALO_MAX 2048       // largest halo a pass stages (records in shared memory)
#define WF_TILE_WIN_WORDS 8192      // bitmap words of the builder: a window of 262,144 slots

struct TileHalo {
  const int32_t* hoff;    // [tiles] offset of the tile's halo in `halo` (a multiple of 4)
  const int32_t* hcnt;    // [tiles] halo size; -1: not staged (the pass gathers from global)
  const int32_t* halo;    // halo slots, ascending per tile
  const uint16_t* nbl;    // local lists, layout of nb (nb_at)
  int cap;                // halo size the passes' shared memory holds (0: staging off)
};

// Builds the halos and local lists of every tile from the slot lists (nb,
// cnt) for halos of at most `cap` slots; tiles whose halo is larger, or whose
// slots span more than the builder's window, get hcnt = -1.  The largest halo
// found (staged or not) is atomicMax-ed into *hmax.  `halo` holds
// `halo_cap` entries; tiles that find it full are not staged.
void launch_tile_halo(int64_t n, int64_t npad, const int32_t* nb, const int32_t* cnt,
                      int32_t* hoff, int32_t* hcnt, int32_t* halo, int64_t halo_cap,
                      uint16_t* nbl, int cap, unsigned* halo_used, int* hmax, cudaStream_t s);

// 16-bit neighbour lists for the global gather path: per tile of WF_TILE
// slots a base slot (the smallest slot its lists name, or -1 when they span
// more than 65,536 slots: the tile then keeps the 32-bit lists), and entries
// stored as slot - base in the layout of nb (nb_at).
struct List16 {
  const int32_t* base;    // [tiles]
  const uint16_t* off;    // offsets, layout of nb
};
void launch_list16(int64_t n, int64_t npad, const int32_t* nb, const int32_t* cnt, int32_t* base,
                   uint16_t* off, cudaStream_t s);

// Lets `kernel` use `bytes` of dynamic shared memory on the current device
// (the attribute is per device; set once per device and larger size).
template <class K>
inline void opt_in_smem(K kernel, size_t bytes, size_t* opted /* [64] */) {
  if (bytes <= 48 * 1024) return;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (bytes <= opted[dev]) return;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
      cudaSuccess)
    opted[dev] = bytes;
}

// asynchronous global -> shared copies (cp.async; both addresses aligned to the size)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// A staged tile's local lists in shared memory: block b of the tile's t-th
// slot at sl[(b * WF_TILE + t) * 8] (the global layout with WF_TILE as stride)
#define WF_TILE_LIST_BYTES (WF_NB_BLOCKS * WF_TILE * WF_NB_BLK * 2)

// Copies the tile's local lists (all WF_NB_BLOCKS blocks, 2 KB each,
// contiguous in global memory) into shared memory with 16-byte cp.async;
// the caller waits (cp_async_wait_all + barrier).
__device__ __forceinline__ void stage_lists(const uint16_t* __restrict__ nbl, int64_t npad,
                                            int tile, uint16_t* sl);

// block b (entries 8b .. 8b+7) of slot t's local list in shared memory
__device__ __forceinline__ void nbl_block_s(const uint16_t* sl, int t, int b, int js[8]) {
  const uint4 q = *reinterpret_cast<const uint4*>(sl + (b * WF_TILE + t) * WF_NB_BLK);
  js[0] = (int)(q.x & 0xffffu); js[1] = (int)(q.x >> 16);
  js[2] = (int)(q.y & 0xffffu); js[3] = (int)(q.y >> 16);
  js[4] = (int)(q.z & 0xffffu); js[5] = (int)(q.z >> 16);
  js[6] = (int)(q.w & 0xffffu); js[7] = (int)(q.w >> 16);
}

// block b (entries 8b .. 8b+7) of slot i's local list as one 16-byte load
__device__ __forceinline__ void nbl_block(const uint16_t* __restrict__ nbl, int64_t npad,
                                          int64_t i, int b, int js[8]) {
  const uint4 q = __ldg(reinterpret_cast<const uint4*>(nbl + ((int64_t)b * npad + i) * WF_NB_BLK));
  js[0] = (int)(q.x & 0xffffu); js[1] = (int)(q.x >> 16);
  js[2] = (int)(q.y & 0xffffu); js[3] = (int)(q.y >> 16);
  js[4] = (int)(q.z & 0xffffu); js[5] = (int)(q.z >> 16);
  js[6] = (int)(q.w & 0xffffu); js[7] = (int)(q.w >> 16);
}

__device__ __forceinline__ void stage_lists(const uint16_t* __restrict__ nbl, int64_t npad,
                                            int tile, uint16_t* sl) {
  constexpr int kChunks = WF_NB_BLOCKS * WF_TILE;   // 16-byte pieces
  for (int k = threadIdx.x; k < kChunks; k += blockDim.x) {
    const int b = k / WF_TILE, t = k - b * WF_TILE;
    cp_async16(sl + (int64_t)k * WF_NB_BLK,
               nbl + ((int64_t)b * npad + (int64_t)tile * WF_TILE + t) * WF_NB_BLK);
  }
}

// ---- neighbour-list readers of the mixed pair passes ----------------------
// block(b, js): entries 8b .. 8b+7 of the particle's list; sub<W>(b, g, js):
// the W entries of lane g of a lane group (W = 8 / lanes); prefetch(b):
// brings block b towards L2 two blocks ahead of use.  `kSlots` tells whether
// the entries are slots (global arrays) or halo ranks (shared memory).
struct NbList32 {                 // 32-bit slot lists
  static constexpr bool kSlots = true;
  const int32_t* nb;
  int64_t npad, i;
  __device__ __forceinline__ void block(int b, int* js) const {
    const int4* q = reinterpret_cast<const int4*>(nb + ((int64_t)b * npad + i) * WF_NB_BLK);
    const int4 lo = __ldg(q), hi = __ldg(q + 1);
    js[0] = lo.x; js[1] = lo.y; js[2] = lo.z; js[3] = lo.w;
    js[4] = hi.x; js[5] = hi.y; js[6] = hi.z; js[7] = hi.w;
  }
  template <int W>
  __device__ __forceinline__ void sub(int b, int g, int* js) const {
    const int32_t* q = nb + ((int64_t)b * npad + i) * WF_NB_BLK + g * W;
    if constexpr (W == 8) {
      block(b, js);
    } else if constexpr (W == 4) {
      const int4 v = __ldg(reinterpret_cast<const int4*>(q));
      js[0] = v.x; js[1] = v.y; js[2] = v.z; js[3] = v.w;
    } else {
      static_assert(W == 2, "list sub-block of 2, 4 or 8 entries");
      const int2 v = __ldg(reinterpret_cast<const int2*>(q));
      js[0] = v.x; js[1] = v.y;
    }
  }
  // a 128-byte line holds one block of 4 consecutive slots
  __device__ __forceinline__ void prefetch(int b, int lanes) const {
    nb_prefetch(nb, npad, i, b, 4 * lanes);
  }
};

struct NbList16 {                 // 16-bit offsets from the tile's base slot
  static constexpr bool kSlots = true;
  const uint16_t* off;
  int64_t npad, i;
  int base;
  __device__ __forceinline__ void block(int b, int* js) const {
    const uint4 q = __ldg(reinterpret_cast<const uint4*>(off + ((int64_t)b * npad + i) * WF_NB_BLK));
    js[0] = base + (int)(q.x & 0xffffu); js[1] = base + (int)(q.x >> 16);
    js[2] = base + (int)(q.y & 0xffffu); js[3] = base + (int)(q.y >> 16);
    js[4] = base + (int)(q.z & 0xffffu); js[5] = base + (int)(q.z >> 16);
    js[6] = base + (int)(q.w & 0xffffu); js[7] = base + (int)(q.w >> 16);
  }
  template <int W>
  __device__ __forceinline__ void sub(int b, int g, int* js) const {
    if constexpr (W == 8) {
      block(b, js);
    } else {
      static_assert(W == 4, "16-bit sub-blocks of 4 entries");
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(
          off + ((int64_t)b * npad + i) * WF_NB_BLK + g * W));
      js[0] = base + (int)(v.x & 0xffffu); js[1] = base + (int)(v.x >> 16);
      js[2] = base + (int)(v.y & 0xffffu); js[3] = base + (int)(v.y >> 16);
    }
  }
  // a 128-byte line holds one block of 8 consecutive slots
  __device__ __forceinline__ void prefetch(int b, int lanes) const {
    if ((threadIdx.x & (8 * lanes - 1)) == 0)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(off + ((int64_t)b * npad + i) * WF_NB_BLK));
  }
};

struct NbListS {                  // a staged tile's local lists in shared memory
  static constexpr bool kSlots = false;
  const uint16_t* sl;
  int t;                          // the slot's place in its tile
  __device__ __forceinline__ void block(int b, int* js) const { nbl_block_s(sl, t, b, js); }
  template <int W>
  __device__ __forceinline__ void sub(int b, int g, int* js) const {
    if constexpr (W == 8) {
      block(b, js);
    } else {
      static_assert(W == 4, "local sub-blocks of 4 entries");
      const uint2 v = *reinterpret_cast<const uint2*>(sl + (b * WF_TILE + t) * WF_NB_BLK + g * W);
      js[0] = (int)(v.x & 0xffffu); js[1] = (int)(v.x >> 16);
      js[2] = (int)(v.y & 0xffffu); js[3] = (int)(v.y >> 16);
    }
  }
  __device__ __forceinline__ void prefetch(int, int) const {}
};
