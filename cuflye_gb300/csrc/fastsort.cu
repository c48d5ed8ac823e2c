// fastsort.cu — exact fast paths for Flye's sort points on segments whose
// keys are all distinct.
//
// Flye sorts with std::sort, so where a segment holds equal keys their final
// order is the one libstdc++'s introsort leaves them in, and sort.cu
// reproduces that order.  A segment whose keys are all distinct has exactly
// one sorted order, so any correct sort gives Flye's result there.  Two fast
// paths use that; segments that may hold equal keys still go to sort.cu.
//
// * KmerMatch sort of a query's hits by (ext id, cur pos)
//   (patches/flye/2.9.6/0001-cuflye-candidate-match-dump.patch:86-92).  Hits
//   are generated window by window, so the hits on one ext id already come
//   in cur-pos order.  Two hits share (ext id, cur pos) only when one window's
//   bucket lists a target id twice; the index marks such buckets (kDupIdsBit)
//   and hit counting flags the queries that look one up (q_tie).  An
//   unflagged query's keys are distinct, and its sort is a stable sort by ext
//   id: a least-significant-digit radix sort over the ext id bits, 8 bits per
//   pass, in tiles of kMatchTile hits that never straddle two queries.
// * Ext-pos re-sort of ext-sorted groups
//   (tools/replay_read_to_graph_source_pack.py:396-397) that are not already
//   in strict ext-pos order.  One block sorts the group, in shared memory up
//   to kGroupCap elements when (ext pos - min, index) packs in 32 bits, else in
//   device scratch (the same radix sort on separate key and index arrays),
//   and compares neighbours; a group with equal ext positions is written out
//   in the layout sort.cu expects and listed for it.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

// ---------------------------------------------------------------- KmerMatch tiles

constexpr int kTileBlock = 512;
constexpr int kTileWarps = kTileBlock / 32;
constexpr int kTileItems = static_cast<int>(kMatchTile / kTileBlock);  // per thread
constexpr uint32_t kPerWarp = kMatchTile / kTileWarps;               // consecutive hits

// Hit pairs as the hit arrays hold them: key = (ext id << 32) | cur pos.
struct PairsAoS {
  uint64_t* k;
  uint32_t* v;
  __device__ __forceinline__ uint32_t hi(uint64_t i) const {
    return static_cast<uint32_t>(k[i] >> 32);
  }
  __device__ __forceinline__ void load(uint64_t i, uint32_t& h, uint32_t& l, uint32_t& x) const {
    const uint64_t kk = k[i];
    h = static_cast<uint32_t>(kk >> 32);
    l = static_cast<uint32_t>(kk);
    x = v[i];
  }
  __device__ __forceinline__ void store(uint64_t i, uint32_t h, uint32_t l, uint32_t x) const {
    k[i] = (static_cast<uint64_t>(h) << 32) | l;
    v[i] = x;
  }
};

__global__ void match_plan_kernel(const uint64_t* __restrict__ q_off,
                                  const uint32_t* __restrict__ q_tie, uint32_t nq,
                                  uint32_t* __restrict__ ntiles, uint64_t* __restrict__ emu_begin,
                                  uint64_t* __restrict__ emu_end, uint32_t* __restrict__ emu_count,
                                  bool tile_flagged) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    const uint64_t b = q_off[q], e = q_off[q + 1];
    uint32_t t = 0;
    if (tile_flagged) {
      // the flagged queries only, all by radix tiles
      if (e - b > 1 && q_tie[q]) t = static_cast<uint32_t>((e - b + kMatchTile - 1) / kMatchTile);
    } else if (e - b > 1) {
      if (q_tie[q]) {
        const uint32_t s = atomicAdd(emu_count, 1u);
        emu_begin[s] = b;
        emu_end[s] = e;
      } else {
        t = static_cast<uint32_t>((e - b + kMatchTile - 1) / kMatchTile);
      }
    }
    ntiles[q] = t;
  }
}

__global__ void match_tiles_kernel(const uint64_t* __restrict__ q_off,
                                   const uint32_t* __restrict__ ntiles,
                                   const uint64_t* __restrict__ tile_off, uint32_t nq,
                                   MatchTile* __restrict__ tiles) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    const uint32_t nt = ntiles[q];
    const uint64_t t0 = tile_off[q], b = q_off[q], e = q_off[q + 1];
    for (uint32_t t = 0; t < nt; ++t) {
      const uint64_t s = b + static_cast<uint64_t>(t) * kMatchTile;
      MatchTile tl;
      tl.begin = s;
      tl.n = static_cast<uint32_t>(e - s < kMatchTile ? e - s : kMatchTile);
      tl.query = q;
      tiles[t0 + t] = tl;
    }
  }
}

template <class Src>
__global__ void __launch_bounds__(256) match_hist_kernel(Src src,
                                                         const MatchTile* __restrict__ tiles,
                                                         uint32_t ntile, int shift,
                                                         uint32_t* __restrict__ counts) {
  __shared__ uint32_t h[256];
  for (uint32_t t = blockIdx.x; t < ntile; t += gridDim.x) {
    h[threadIdx.x] = 0;
    __syncthreads();
    const MatchTile tl = tiles[t];
    // eight keys in flight per thread before their counts
    for (uint32_t j0 = 0; j0 < tl.n; j0 += 8 * 256) {
      uint32_t d[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const uint32_t j = j0 + u * 256 + threadIdx.x;
        d[u] = j < tl.n ? (src.hi(tl.begin + j) >> shift) & 0xffu : 256u;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (d[u] < 256u) atomicAdd(&h[d[u]], 1u);
    }
    __syncthreads();
    counts[static_cast<uint64_t>(t) * 256 + threadIdx.x] = h[threadIdx.x];
    __syncthreads();
  }
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block256_exclusive(uint32_t v, uint32_t* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += ws[w];
  __syncthreads();
  return before + inc - v;
}

// Per query: counts[tile][digit] -> destination of the tile's first hit of
// that digit, relative to the query's first hit (digit-major, tile-minor).
__global__ void __launch_bounds__(256) match_offsets_kernel(const uint32_t* __restrict__ ntiles,
                                                            const uint64_t* __restrict__ tile_off,
                                                            uint32_t nq,
                                                            uint32_t* __restrict__ counts) {
  __shared__ uint32_t ws[8];
  const uint32_t d = threadIdx.x;
  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const uint32_t nt = ntiles[q];
    if (nt == 0) continue;
    const uint64_t t0 = tile_off[q];
    uint32_t tot = 0;
#pragma unroll 8
    for (uint32_t t = 0; t < nt; ++t) tot += counts[(t0 + t) * 256 + d];
    uint32_t run = block256_exclusive(tot, ws);
    // eight tiles' counts in flight, then their offsets
    for (uint32_t t8 = 0; t8 < nt; t8 += 8) {
      uint32_t c[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        c[u] = t8 + u < nt ? counts[(t0 + t8 + u) * 256 + d] : 0u;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (t8 + u < nt) {
          counts[(t0 + t8 + u) * 256 + d] = run;
          run += c[u];
        }
      }
    }
  }
}

struct TileSmem {
  uint64_t key[kMatchTile];  // staged pairs in digit order: (ext id << 32) | cur pos
  uint32_t val[kMatchTile];
  uint32_t wc[kTileWarps][256];  // per-warp digit counts, then offsets
  uint32_t dbase[256];           // tile-local start of each digit
  uint32_t gbase[256];           // query-relative destination of each digit
  uint32_t ws[kTileWarps];
};

// One stable radix pass over a tile: hits keep their order within a digit.
// Warp w owns the tile's hits [w * kPerWarp, (w + 1) * kPerWarp), visited in
// rounds of 32 consecutive hits; match_any ranks a round, per-warp counters
// carry the ranks across rounds, and a digit-major scan over warps places
// each hit.  The tile is staged in shared memory in digit order so that each
// digit's hits leave as one coalesced run.
template <class Src, class Dst>
__global__ void __launch_bounds__(kTileBlock, 2)
    match_scatter_kernel(Src src, Dst dst, const MatchTile* __restrict__ tiles, uint32_t ntile,
                         const uint64_t* __restrict__ q_off, int shift,
                         const uint32_t* __restrict__ counts) {
  extern __shared__ __align__(16) unsigned char tile_raw[];
  TileSmem& sm = *reinterpret_cast<TileSmem*>(tile_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t t = blockIdx.x; t < ntile; t += gridDim.x) {
    const MatchTile tl = tiles[t];
    for (int i = threadIdx.x; i < kTileWarps * 256; i += kTileBlock) (&sm.wc[0][0])[i] = 0;
    if (threadIdx.x < 256) sm.gbase[threadIdx.x] = counts[static_cast<uint64_t>(t) * 256 + threadIdx.x];
    __syncthreads();
    uint32_t hi[kTileItems], lo[kTileItems], va[kTileItems], rk[kTileItems];
#pragma unroll
    for (int r = 0; r < kTileItems; ++r) {
      const uint32_t j = warp * kPerWarp + r * 32 + lane;
      const bool valid = j < tl.n;
      uint32_t d = 256;  // no digit: invalid lanes never touch a counter
      hi[r] = lo[r] = va[r] = 0;
      if (valid) {
        src.load(tl.begin + j, hi[r], lo[r], va[r]);
        d = (hi[r] >> shift) & 0xffu;
      }
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const int leader = __ffs(peers) - 1;
      uint32_t base = 0;
      if (valid && lane == leader) {
        base = sm.wc[warp][d];
        sm.wc[warp][d] = base + __popc(peers);
      }
      base = __shfl_sync(0xffffffffu, base, leader);
      rk[r] = base + __popc(peers & lt);
    }
    __syncthreads();
    uint32_t tot = 0;
    if (threadIdx.x < 256) {
      const int d = threadIdx.x;
      for (int w = 0; w < kTileWarps; ++w) {
        const uint32_t c = sm.wc[w][d];
        sm.wc[w][d] = tot;
        tot += c;
      }
    }
    {
      uint32_t inc = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
      }
      if (lane == 31 && warp < 8) sm.ws[warp] = inc;
      __syncthreads();
      if (threadIdx.x < 256) {
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += sm.ws[w];
        sm.dbase[threadIdx.x] = before + inc - tot;
      }
      __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < kTileItems; ++r) {
      const uint32_t j = warp * kPerWarp + r * 32 + lane;
      if (j < tl.n) {
        const uint32_t d = (hi[r] >> shift) & 0xffu;
        const uint32_t p = sm.dbase[d] + sm.wc[warp][d] + rk[r];
        sm.key[p] = (static_cast<uint64_t>(hi[r]) << 32) | lo[r];
        sm.val[p] = va[r];
      }
    }
    __syncthreads();
    const uint64_t qb = q_off[tl.query];
    for (uint32_t j = threadIdx.x; j < tl.n; j += kTileBlock) {
      const uint64_t x = sm.key[j];
      const uint32_t h = static_cast<uint32_t>(x >> 32);
      const uint32_t d = (h >> shift) & 0xffu;
      dst.store(qb + sm.gbase[d] + (j - sm.dbase[d]), h, static_cast<uint32_t>(x), sm.val[j]);
    }
    __syncthreads();
  }
}

template <class Src, class Dst>
__global__ void match_copy_kernel(Src src, Dst dst, const MatchTile* __restrict__ tiles,
                                  uint32_t ntile) {
  for (uint32_t t = blockIdx.x; t < ntile; t += gridDim.x) {
    const MatchTile tl = tiles[t];
    for (uint32_t j = threadIdx.x; j < tl.n; j += blockDim.x) {
      uint32_t h, l, v;
      src.load(tl.begin + j, h, l, v);
      dst.store(tl.begin + j, h, l, v);
    }
  }
}

// ---------------------------------------------------------------- group sorts

constexpr int kGroupBlock = 1024;
constexpr int kGroupWarps = kGroupBlock / 32;

struct GroupSmem {
  uint32_t a[kGroupCap];  // packed (key - min) << ib | index
  uint32_t b[kGroupCap];
  uint16_t rank[kGroupCap];
  uint32_t wc[kGroupWarps][256];
  uint32_t dbase[256];
  uint32_t ws[kGroupWarps];
  uint32_t kmin, kmax;
  uint32_t item;
};

// Rewrites the group as (key = ext pos, val = cur pos) for sort.cu and lists it there.
__device__ void group_to_emulation(uint64_t* keys, uint32_t* vals, const GroupInfo& g,
                                   uint64_t* emu_begin, uint64_t* emu_end, uint32_t* emu_count) {
  for (uint32_t j = threadIdx.x; j < g.n; j += blockDim.x) {
    const uint64_t i = g.start + j;
    const uint64_t kk = keys[i];
    keys[i] = static_cast<uint64_t>(vals[i]);
    vals[i] = static_cast<uint32_t>(kk & 0xffffffffu);
  }
  if (threadIdx.x == 0) {
    const uint32_t s = atomicAdd(emu_count, 1u);
    emu_begin[s] = g.start;
    emu_end[s] = g.start + g.n;
  }
}

// Turns the per-warp digit counts in sm.wc into each warp's first output slot
// per digit: digits in order, warps in order within a digit.
__device__ void group_digit_bases(GroupSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t tot = 0;
  if (threadIdx.x < 256) {
    for (int w = 0; w < kGroupWarps; ++w) {
      const uint32_t c = sm.wc[w][threadIdx.x];
      sm.wc[w][threadIdx.x] = tot;
      tot += c;
    }
  }
  uint32_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31 && warp < 8) sm.ws[warp] = inc;
  __syncthreads();
  if (threadIdx.x < 256) {
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += sm.ws[w];
    sm.dbase[threadIdx.x] = before + inc - tot;
  }
  __syncthreads();
}

// Key and index arrays of the device-scratch sort, indexed like the hits.
struct GroupScratch {
  uint32_t* k0;
  uint32_t* i0;
  uint32_t* k1;
  uint32_t* i1;
};

// A group beyond shared memory: LSD radix sort of (ext pos - min, index) by
// 8-bit digits in device scratch; each warp owns a contiguous slice, counts
// its digits, then scatters the slice in order (stable).  Equal ext
// positions send the group to sort.cu untouched; otherwise the group is
// rewritten as (key = ext pos, val = cur pos) in ext-pos order.
__device__ void group_sort_global(uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                  const GroupInfo& g, GroupScratch sc, GroupSmem& sm,
                                  uint64_t* emu_begin, uint64_t* emu_end, uint32_t* emu_count) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t n = g.n;
  const uint64_t b = g.start;
  if (threadIdx.x == 0) {
    sm.kmin = 0xffffffffu;
    sm.kmax = 0;
  }
  __syncthreads();
  uint32_t lmin = 0xffffffffu, lmax = 0;
  for (uint32_t j = threadIdx.x; j < n; j += kGroupBlock) {
    const uint32_t key = vals[b + j];
    lmin = min(lmin, key);
    lmax = max(lmax, key);
  }
  atomicMin(&sm.kmin, lmin);
  atomicMax(&sm.kmax, lmax);
  __syncthreads();
  const uint32_t kmin = sm.kmin, range = sm.kmax - sm.kmin;
  const int kb = range ? 32 - __clz(range) : 0;
  uint32_t* sk = sc.k0 + b;
  uint32_t* si = sc.i0 + b;
  uint32_t* dk = sc.k1 + b;
  uint32_t* di = sc.i1 + b;
  for (uint32_t j = threadIdx.x; j < n; j += kGroupBlock) {
    sk[j] = vals[b + j] - kmin;
    si[j] = j;
  }
  const uint32_t per_warp = (((n + 31) / 32 + kGroupWarps - 1) / kGroupWarps) * 32;
  const uint32_t w0 = min(n, warp * per_warp);
  const uint32_t w1 = min(n, w0 + per_warp);
  for (int shift = 0; shift < kb; shift += 8) {
    for (int i = threadIdx.x; i < kGroupWarps * 256; i += kGroupBlock) (&sm.wc[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
      const uint32_t j = r0 + lane;
      const bool valid = j < w1;
      const uint32_t d = valid ? (sk[j] >> shift) & 0xffu : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      if (valid && lane == __ffs(peers) - 1) sm.wc[warp][d] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    group_digit_bases(sm);
    for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
      const uint32_t j = r0 + lane;
      const bool valid = j < w1;
      const uint32_t x = valid ? sk[j] : 0u;
      const uint32_t d = valid ? (x >> shift) & 0xffu : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t base = valid ? sm.dbase[d] + sm.wc[warp][d] : 0u;
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) sm.wc[warp][d] += __popc(peers);
      __syncwarp();
      if (valid) {
        const uint32_t o = base + __popc(peers & lt);
        dk[o] = x;
        di[o] = si[j];
      }
    }
    __syncthreads();
    uint32_t* t = sk;
    sk = dk;
    dk = t;
    t = si;
    si = di;
    di = t;
  }
  bool tie = false;
  for (uint32_t j = threadIdx.x + 1; j < n && !tie; j += kGroupBlock) tie = sk[j] == sk[j - 1];
  if (__syncthreads_or(tie)) {
    group_to_emulation(keys, vals, g, emu_begin, emu_end, emu_count);
    return;
  }
  // gather the cur positions before any write: the group is rewritten in place
  for (uint32_t i = threadIdx.x; i < n; i += kGroupBlock)
    dk[i] = static_cast<uint32_t>(keys[b + si[i]] & 0xffffffffu);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += kGroupBlock) {
    keys[b + i] = static_cast<uint64_t>(sk[i] + kmin);
    vals[b + i] = dk[i];
  }
}

// In (key = (ext id << 32) | cur pos, val = ext pos), out (key = ext pos,
// val = cur pos) in ext-pos order.
__global__ void __launch_bounds__(kGroupBlock, 1)
    group_sort_kernel(uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                      const GroupInfo* __restrict__ groups, const uint32_t* __restrict__ list,
                      const uint32_t* __restrict__ list_count, uint64_t* __restrict__ emu_begin,
                      uint64_t* __restrict__ emu_end, uint32_t* __restrict__ emu_count,
                      GroupScratch sc, uint32_t* __restrict__ work) {
  extern __shared__ __align__(16) unsigned char group_raw[];
  GroupSmem& sm = *reinterpret_cast<GroupSmem*>(group_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t cnt = *list_count;
  for (;;) {
    // blocks take groups from a shared counter (group lengths vary widely)
    __syncthreads();
    if (threadIdx.x == 0) sm.item = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t li = sm.item;
    if (li >= cnt) break;
    const uint32_t gidx = list[li];
    const GroupInfo g = groups[gidx];
    const uint32_t n = g.n;
    const uint64_t b = g.start;
    if (n == 0) continue;
    if (n > kGroupCap) {
      group_sort_global(keys, vals, g, sc, sm, emu_begin, emu_end, emu_count);
      __syncthreads();
      continue;
    }
    if (threadIdx.x == 0) {
      sm.kmin = 0xffffffffu;
      sm.kmax = 0;
    }
    __syncthreads();
    uint32_t lmin = 0xffffffffu, lmax = 0;
    for (uint32_t j = threadIdx.x; j < n; j += kGroupBlock) {
      const uint32_t key = vals[b + j];
      sm.a[j] = key;
      lmin = min(lmin, key);
      lmax = max(lmax, key);
    }
    atomicMin(&sm.kmin, lmin);
    atomicMax(&sm.kmax, lmax);
    __syncthreads();
    const uint32_t kmin = sm.kmin, range = sm.kmax - sm.kmin;
    const int kb = range ? 32 - __clz(range) : 0;
    const int ib = n > 1 ? 32 - __clz(n - 1) : 0;
    if (kb + ib > 32) {  // the packed form does not fit: separate keys and indices
      __syncthreads();     // every thread has read kmin / kmax before they are reset
      group_sort_global(keys, vals, g, sc, sm, emu_begin, emu_end, emu_count);
      __syncthreads();
      continue;
    }
    for (uint32_t j = threadIdx.x; j < n; j += kGroupBlock)
      sm.a[j] = ib ? (((sm.a[j] - kmin) << ib) | j) : 0u;
    __syncthreads();
    uint32_t* src = sm.a;
    uint32_t* dst = sm.b;
    const uint32_t per_warp = (((n + 31) / 32 + kGroupWarps - 1) / kGroupWarps) * 32;
    const uint32_t w0 = warp * per_warp;
    const uint32_t w1 = min(n, w0 + per_warp);
    for (int sh = 0; sh < kb; sh += 8) {
      const int shift = ib + sh;
      for (int i = threadIdx.x; i < kGroupWarps * 256; i += kGroupBlock) (&sm.wc[0][0])[i] = 0;
      __syncthreads();
      for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
        const uint32_t j = r0 + lane;
        const bool valid = j < w1;
        const uint32_t d = valid ? (src[j] >> shift) & 0xffu : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) {
          base = sm.wc[warp][d];
          sm.wc[warp][d] = base + __popc(peers);
        }
        base = __shfl_sync(0xffffffffu, base, leader);
        if (valid) sm.rank[j] = static_cast<uint16_t>(base + __popc(peers & lt));
      }
      __syncthreads();
      group_digit_bases(sm);
      for (uint32_t j = w0 + lane; j < w1; j += 32) {
        const uint32_t x = src[j];
        const uint32_t d = (x >> shift) & 0xffu;
        dst[sm.dbase[d] + sm.wc[warp][d] + sm.rank[j]] = x;
      }
      __syncthreads();
      uint32_t* tmp = src;
      src = dst;
      dst = tmp;
    }
    // Equal ext positions?
    bool tie = false;
    for (uint32_t j = threadIdx.x + 1; j < n && !tie; j += kGroupBlock)
      tie = (src[j] >> ib) == (src[j - 1] >> ib);
    if (__syncthreads_or(tie)) {
      group_to_emulation(keys, vals, g, emu_begin, emu_end, emu_count);
      __syncthreads();
      continue;
    }
    const uint32_t imask = ib ? ((1u << ib) - 1u) : 0u;
    // gather the cur positions before any write: the group is rewritten in place
    for (uint32_t i = threadIdx.x; i < n; i += kGroupBlock)
      dst[i] = static_cast<uint32_t>(keys[b + (src[i] & imask)] & 0xffffffffu);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += kGroupBlock) {
      keys[b + i] = static_cast<uint64_t>((ib ? (src[i] >> ib) : 0u) + kmin);
      vals[b + i] = dst[i];
    }
    __syncthreads();
  }
}

__global__ void sort_stats_kernel(uint64_t* stats, int i_plain, int i_emul,
                                  const uint32_t* total_dev, uint32_t total_host,
                                  const uint32_t* emul) {
  const uint32_t e = *emul;
  const uint32_t t = total_dev ? *total_dev : total_host;
  stats[i_emul] += e;
  if (i_plain >= 0) stats[i_plain] += t - e;
}

template <class T>
void allow_smem(T* kernel, size_t bytes) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(bytes));
}

}  // namespace

cudaError_t match_plan(const uint64_t* q_off, const uint32_t* q_tie, uint32_t nq, uint32_t* ntiles,
                       uint64_t* emu_begin, uint64_t* emu_end, uint32_t* emu_count,
                       cudaStream_t s, bool tile_flagged) {
  cudaError_t e = tile_flagged ? cudaSuccess : cudaMemsetAsync(emu_count, 0, 4, s);
  if (e != cudaSuccess || nq == 0) return e;
  count_launch();
  match_plan_kernel<<<(nq + 255) / 256, 256, 0, s>>>(q_off, q_tie, nq, ntiles, emu_begin, emu_end,
                                                     emu_count, tile_flagged);
  return cudaGetLastError();
}

cudaError_t match_tiles(const uint64_t* q_off, const uint32_t* ntiles, const uint64_t* tile_off,
                        uint32_t nq, MatchTile* tiles, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  match_tiles_kernel<<<(nq + 255) / 256, 256, 0, s>>>(q_off, ntiles, tile_off, nq, tiles);
  return cudaGetLastError();
}

cudaError_t match_radix(uint64_t* keys, uint32_t* vals, uint64_t* alt_keys, uint32_t* alt_vals,
                        const MatchTile* tiles, uint32_t ntile,
                        const uint64_t* q_off, const uint32_t* ntiles, const uint64_t* tile_off,
                        uint32_t nq, int id_bits, uint32_t* counts, int num_sms,
                        int scatter_per_sm, cudaStream_t s) {
  if (ntile == 0 || id_bits <= 0) return cudaSuccess;
  const PairsAoS aos{keys, vals};
  const PairsAoS alt{alt_keys, alt_vals};
  allow_smem(match_scatter_kernel<PairsAoS, PairsAoS>, sizeof(TileSmem));
  const unsigned tgrid = static_cast<unsigned>(std::min<uint64_t>(ntile, 2ull * num_sms * 8));
  // tiles are taken grid-stride: the scatter's grid (scatter_per_sm blocks
  // per SM, 1-2, 0: 2) changes no result
  const uint64_t per_sm = scatter_per_sm > 0 ? std::min(scatter_per_sm, 2) : 2;
  const unsigned sgrid = static_cast<unsigned>(std::min<uint64_t>(ntile, per_sm * num_sms));
  const unsigned qgrid = static_cast<unsigned>(std::min<uint64_t>(nq, 4ull * num_sms));
  bool in_aos = true;
  for (int sh = 0; sh < id_bits; sh += 8) {
    const PairsAoS src = in_aos ? aos : alt, dst = in_aos ? alt : aos;
    count_launch();
    match_hist_kernel<<<tgrid, 256, 0, s>>>(src, tiles, ntile, sh, counts);
    count_launch();
    match_offsets_kernel<<<qgrid, 256, 0, s>>>(ntiles, tile_off, nq, counts);
    count_launch();
    match_scatter_kernel<<<sgrid, kTileBlock, sizeof(TileSmem), s>>>(src, dst, tiles, ntile, q_off,
                                                                     sh, counts);
    in_aos = !in_aos;
  }
  if (!in_aos) {
    count_launch();
    match_copy_kernel<<<tgrid, 256, 0, s>>>(alt, aos, tiles, ntile);
  }
  return cudaGetLastError();
}

cudaError_t group_ext_sort(uint64_t* keys, uint32_t* vals, const GroupInfo* groups,
                           const uint32_t* list, const uint32_t* list_count, uint32_t max_groups,
                           uint64_t* emu_begin, uint64_t* emu_end, uint32_t* emu_count,
                           uint32_t* scratch_a, uint32_t* scratch_b, uint32_t* scratch_c,
                           uint64_t nhits, uint32_t* work, int num_sms, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(emu_count, 0, 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(work, 0, 4, s);
  if (e != cudaSuccess || max_groups == 0) return e;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(max_groups, num_sms));
  allow_smem(group_sort_kernel, sizeof(GroupSmem));
  count_launch();
  group_sort_kernel<<<grid, kGroupBlock, sizeof(GroupSmem), s>>>(
      keys, vals, groups, list, list_count, emu_begin, emu_end, emu_count,
      GroupScratch{scratch_a, scratch_b, scratch_c, scratch_c + nhits}, work);
  return cudaGetLastError();
}

cudaError_t sort_stats_add(uint64_t* stats, int i_plain, int i_emul, const uint32_t* total_dev,
                           uint32_t total_host, const uint32_t* emul, cudaStream_t s) {
  count_launch();
  sort_stats_kernel<<<1, 1, 0, s>>>(stats, i_plain, i_emul, total_dev, total_host, emul);
  return cudaGetLastError();
}

}  // namespace cuflye
