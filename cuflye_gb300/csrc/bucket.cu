// bucket.cu — hits of tie-free queries written straight into Flye's
// KmerMatch order.
//
// Within a query Flye sorts its KmerMatches by (ext id, cur pos)
// (patches/flye/2.9.6/0001-cuflye-candidate-match-dump.patch:86-92).  When no
// window yields two hits on one ext id (hits_count leaves q_tie = 0) the keys
// are distinct, the sorted order is unique, and it is a counting sort by ext
// id of the hits in window order.  One block per query:
//   1. counts the query's hits per distinct ext id and per warp chunk of its
//      windows, with the ext ids in a shared-memory hash (dense ids in
//      arrival order);
//   2. sorts the distinct ext ids and turns the counts into each warp's first
//      position per ext id;
//   3. walks each warp's chunk of windows in order and writes every hit at its
//      final position, so each ext id's hits stay in window (cur pos) order.
// A query with more distinct ext ids than the dictionary holds, or ext ids
// beyond its packing, is written in window order instead and marked q_tie = 2
// for the radix path of the KmerMatch sort.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr int kDsWarps = 8;
constexpr int kDsBlock = kDsWarps * 32;
constexpr uint32_t kDsCap = 1024;   // distinct ext ids per query
constexpr uint32_t kDsHash = 2048;  // hash slots (power of two)
constexpr int kDsHashBits = 11;
constexpr uint32_t kDsIdBits = 20;  // ext ids packed above a 12-bit dense id
constexpr uint32_t kDsDense = 0xfffu;
constexpr int kDsBatch = 4;         // windows whose bucket loads are issued together
constexpr uint32_t kDsEmpty = 0xffffffffu;
constexpr uint32_t kDsSpin = 1u << 16;  // bound on waiting for a slot's dense id

struct DsSmem {
  uint32_t hash[kDsHash];          // (ext id << 12) | dense id; dense 0xfff = being claimed
  uint32_t sorted[kDsCap];         // packed entries sorted by ext id
  uint32_t cnt[kDsWarps][kDsCap];  // per-warp hit counts by dense id, then cursors
  uint32_t part[kDsBlock];
  uint32_t ndense;
  uint32_t item;
  int overflow;
};

__device__ __forceinline__ uint32_t ds_slot(uint32_t e) {
  return (e * 0x9E3779B1u) >> (32 - kDsHashBits);
}

// Dense id of ext id e, inserting it if new; kDsEmpty when the dictionary
// is full (or a claim did not resolve within kDsSpin reads).
__device__ uint32_t ds_insert(DsSmem& sm, uint32_t e) {
  uint32_t slot = ds_slot(e);
  for (uint32_t probes = 0; probes < kDsHash; ++probes) {
    uint32_t v = sm.hash[slot];
    if (v == kDsEmpty) {
      const uint32_t claim = (e << 12) | kDsDense;
      v = atomicCAS(&sm.hash[slot], kDsEmpty, claim);
      if (v == kDsEmpty) {
        const uint32_t d = atomicAdd(&sm.ndense, 1u);
        if (d >= kDsCap) {
          sm.overflow = 1;
          atomicExch(&sm.hash[slot], (e << 12) | 0u);  // resolve waiters; results unused
          return kDsEmpty;
        }
        atomicExch(&sm.hash[slot], (e << 12) | d);
        return d;
      }
    }
    if ((v >> 12) == e) {
      for (uint32_t spin = 0; (v & kDsDense) == kDsDense && spin < kDsSpin; ++spin)
        v = atomicAdd(&sm.hash[slot], 0u);
      if ((v & kDsDense) == kDsDense) {
        sm.overflow = 1;
        return kDsEmpty;
      }
      return v & kDsDense;
    }
    slot = (slot + 1) & (kDsHash - 1);
  }
  sm.overflow = 1;
  return kDsEmpty;
}

// Dense id of an ext id already in the dictionary.
__device__ __forceinline__ uint32_t ds_find(const DsSmem& sm, uint32_t e) {
  uint32_t slot = ds_slot(e);
  for (uint32_t probes = 0; probes < kDsHash; ++probes) {
    const uint32_t v = sm.hash[slot];
    if ((v >> 12) == e) return v & kDsDense;
    slot = (slot + 1) & (kDsHash - 1);
  }
  return 0;  // not reached: every ext id of the query was inserted
}

// Bucket entry e of a window as the hit it yields (flipped to the other
// strand when the query k-mer is not in standard form); false for the self
// hit, which Flye skips.
__device__ __forceinline__ bool hit_of(const DeviceIndex& idx, uint64_t off, uint32_t e,
                                       bool flip, int32_t qdi, uint32_t p, uint32_t& id,
                                       int32_t& pos) {
  const uint64_t sv = __ldg(idx.pos + off + e);
  id = static_cast<uint32_t>(sv >> 32);
  pos = static_cast<int32_t>(sv & 0xffffffffu);
  if (flip) {
    pos = idx.slot_len[id >> 1] - pos - idx.k;
    id ^= 1u;
  }
  return !(static_cast<int32_t>(id) == qdi && pos == static_cast<int32_t>(p));
}

__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) part[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += part[w];
  __syncthreads();
  return before + inc - v;
}

// Walks windows [c0, c1) of a query in order with the calling warp, calling
// op(id, v, p) on each lane for each of the window's hits (lanes over the
// window's bucket entries, __syncwarp between windows): id is the hit's ext
// id and v the raw stored entry, from which hit_pos() gives the ext pos.  The
// first kDsPre * 32 bucket entries of kDsBatch windows are loaded together.
constexpr int kDsPre = 3;

__device__ __forceinline__ int32_t hit_pos(const DeviceIndex& idx, uint64_t v, bool flip) {
  const int32_t pos = static_cast<int32_t>(v & 0xffffffffu);
  return flip ? idx.slot_len[static_cast<uint32_t>(v >> 33)] - pos - idx.k : pos;
}

template <class Op>
__device__ __forceinline__ void walk_windows(const DeviceIndex& idx, const QueryBatch& q,
                                             const uint64_t* __restrict__ hit_off,
                                             const uint64_t* __restrict__ wmeta,
                                             const uint8_t* __restrict__ wflags, uint64_t w0,
                                             uint64_t c0, uint64_t c1, int32_t qdi, Op op) {
  const int lane = threadIdx.x & 31;
  for (uint64_t wb = c0; wb < c1; wb += 32) {
    uint8_t fl = 0;
    uint64_t meta = 0;
    bool has = false;
    if (wb + lane < c1) {
      fl = wflags[wb + lane];
      has = !(fl & kWinFiltered) && hit_off[wb + lane + 1] != hit_off[wb + lane];
      if (has) meta = wmeta[wb + lane];
    }
    unsigned todo = __ballot_sync(0xffffffffu, has);
    while (todo) {
      int src[kDsBatch];
      uint64_t sv[kDsBatch][kDsPre];
#pragma unroll
      for (int u = 0; u < kDsBatch; ++u) {
        src[u] = todo ? __ffs(todo) - 1 : -1;
        if (todo) todo &= todo - 1;
      }
#pragma unroll
      for (int u = 0; u < kDsBatch; ++u) {
        const uint64_t wm = __shfl_sync(0xffffffffu, meta, src[u] < 0 ? 0 : src[u]);
        const uint32_t c = src[u] < 0 ? 0u
                                      : static_cast<uint32_t>((wm >> 40) &
                                                              ((1ULL << kCountBits) - 1));
        const uint64_t* base = idx.pos + (wm & kOffsetMask);
#pragma unroll
        for (int j = 0; j < kDsPre; ++j)
          sv[u][j] = static_cast<uint32_t>(lane + 32 * j) < c ? __ldg(base + lane + 32 * j) : 0;
      }
#pragma unroll
      for (int u = 0; u < kDsBatch; ++u) {
        if (src[u] < 0) continue;
        const uint64_t wm = __shfl_sync(0xffffffffu, meta, src[u]);
        const uint32_t wf = __shfl_sync(0xffffffffu, static_cast<uint32_t>(fl), src[u]);
        const uint64_t off = wm & kOffsetMask;
        const uint32_t c = static_cast<uint32_t>((wm >> 40) & ((1ULL << kCountBits) - 1));
        const bool flip = idx.transform && (wf & kWinRev);
        const uint32_t p = static_cast<uint32_t>(wb + src[u] - w0);
#pragma unroll
        for (int j = 0; j < kDsPre; ++j) {
          const uint32_t e = lane + 32 * j;
          if (e < c) {
            const uint64_t v = sv[u][j];
            const uint32_t id = static_cast<uint32_t>(v >> 32) ^ (flip ? 1u : 0u);
            if (static_cast<int32_t>(id) != qdi || hit_pos(idx, v, flip) != static_cast<int32_t>(p))
              op(id, v, flip, p);
          }
        }
        for (uint32_t e = lane + 32 * kDsPre; e < c; e += 32) {
          const uint64_t v = __ldg(idx.pos + off + e);
          const uint32_t id = static_cast<uint32_t>(v >> 32) ^ (flip ? 1u : 0u);
          if (static_cast<int32_t>(id) != qdi || hit_pos(idx, v, flip) != static_cast<int32_t>(p))
            op(id, v, flip, p);
        }
        __syncwarp();
      }
    }
  }
}

__global__ void __launch_bounds__(kDsBlock) bucket_kernel(
    DeviceIndex idx, QueryBatch q, const uint64_t* __restrict__ hit_off,
    const uint64_t* __restrict__ wmeta, const uint8_t* __restrict__ wflags,
    uint32_t* __restrict__ q_tie, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
    uint32_t* __restrict__ work) {
  extern __shared__ __align__(16) unsigned char ds_raw[];
  DsSmem& sm = *reinterpret_cast<DsSmem*>(ds_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sm.item = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t qi = sm.item;
    if (qi >= q.nq) break;
    const uint64_t w0 = q.win_off[qi], w1 = q.win_off[qi + 1];
    const uint64_t qbase = hit_off[w0];
    if (q_tie[qi] != 0 || hit_off[w1] == qbase) continue;
    const int32_t qdi = q.qdi[qi];
    const uint64_t nw = w1 - w0;
    // warp k owns windows [c0, c1) of the query
    const uint64_t c0 = w0 + nw * warp / kDsWarps, c1 = w0 + nw * (warp + 1) / kDsWarps;
    for (uint32_t i = threadIdx.x; i < kDsHash; i += kDsBlock) sm.hash[i] = kDsEmpty;
    for (uint32_t i = threadIdx.x; i < kDsWarps * kDsCap; i += kDsBlock) (&sm.cnt[0][0])[i] = 0;
    if (threadIdx.x == 0) {
      sm.ndense = 0;
      sm.overflow = 0;
    }
    __syncthreads();
    // 1. count: each warp walks its chunk a window at a time (lanes over the
    // bucket entries: distinct ext ids, so counter updates never collide)
    walk_windows(idx, q, hit_off, wmeta, wflags, w0, c0, c1, qdi,
                 [&](uint32_t id, uint64_t, bool, uint32_t) {
                   if (id >> kDsIdBits) {
                     sm.overflow = 1;
                     return;
                   }
                   const uint32_t d = ds_insert(sm, id);
                   if (d != kDsEmpty) ++sm.cnt[warp][d];
                 });
    __syncthreads();
    if (sm.overflow) {
      // window order, like hits_emit; the radix path sorts it later
      for (uint64_t w = w0 + warp; w < w1; w += kDsWarps) {
        const uint8_t fl = wflags[w];
        uint64_t out = hit_off[w];
        if ((fl & kWinFiltered) || hit_off[w + 1] == out) continue;
        const uint64_t meta = wmeta[w];
        const uint64_t off = meta & kOffsetMask;
        const uint32_t c = static_cast<uint32_t>((meta >> 40) & ((1ULL << kCountBits) - 1));
        const bool flip = idx.transform && (fl & kWinRev);
        const uint32_t p = static_cast<uint32_t>(w - w0);
        for (uint32_t e0 = 0; e0 < c; e0 += 32) {
          uint32_t id = 0;
          int32_t pos = 0;
          const bool keep = e0 + lane < c && hit_of(idx, off, e0 + lane, flip, qdi, p, id, pos);
          const unsigned km = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            const uint64_t dpos = out + __popc(km & lt);
            keys[dpos] = (static_cast<uint64_t>(id) << 32) | p;
            vals[dpos] = static_cast<uint32_t>(pos);
          }
          out += __popc(km);
        }
      }
      if (threadIdx.x == 0) q_tie[qi] = 2;
      continue;
    }
    // 2. dictionary in ext-id order, per-warp cursors
    const uint32_t nd = sm.ndense;
    uint32_t np2 = 1;
    while (np2 < nd) np2 <<= 1;
    for (uint32_t i = threadIdx.x; i < np2; i += kDsBlock) sm.sorted[i] = kDsEmpty;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kDsHash; i += kDsBlock) {
      const uint32_t v = sm.hash[i];
      if (v != kDsEmpty) sm.sorted[v & kDsDense] = v;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= np2; size <<= 1) {
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = threadIdx.x; i < np2 / 2; i += kDsBlock) {
          const uint32_t lo = 2 * i - (i & (stride - 1));
          const uint32_t hi = lo + stride;
          const bool up = (lo & size) == 0;
          const uint32_t a = sm.sorted[lo], b = sm.sorted[hi];
          if ((a > b) == up) {
            sm.sorted[lo] = b;
            sm.sorted[hi] = a;
          }
        }
        __syncthreads();
      }
    }
    // totals in ext-id order: thread t owns ranks [t * per, (t + 1) * per)
    const uint32_t per = (nd + kDsBlock - 1) / kDsBlock;
    const uint32_t r0 = threadIdx.x * per, r1 = min(nd, r0 + per);
    uint32_t local = 0;
    for (uint32_t r = r0; r < r1; ++r) {
      const uint32_t d = sm.sorted[r] & kDsDense;
      for (int k = 0; k < kDsWarps; ++k) local += sm.cnt[k][d];
    }
    uint32_t base = block_exclusive(local, sm.part);
    for (uint32_t r = r0; r < r1; ++r) {
      const uint32_t d = sm.sorted[r] & kDsDense;
      for (int k = 0; k < kDsWarps; ++k) {
        const uint32_t t = sm.cnt[k][d];
        sm.cnt[k][d] = base;
        base += t;
      }
    }
    __syncthreads();
    // 3. emit: each warp walks its windows in order; a window's hits have
    // distinct ext ids, so their cursors never collide
    walk_windows(idx, q, hit_off, wmeta, wflags, w0, c0, c1, qdi,
                 [&](uint32_t id, uint64_t v, bool flip, uint32_t p) {
                   const uint32_t at = sm.cnt[warp][ds_find(sm, id)]++;
                   keys[qbase + at] = (static_cast<uint64_t>(id) << 32) | p;
                   vals[qbase + at] = static_cast<uint32_t>(hit_pos(idx, v, flip));
                 });
  }
}

}  // namespace

cudaError_t hits_emit_sorted(const DeviceIndex& idx, const QueryBatch& q, const uint64_t* hit_off,
                             const uint64_t* wmeta, const uint8_t* wflags, uint32_t* q_tie,
                             uint64_t* keys, uint32_t* vals, uint32_t* work, int num_sms,
                             cudaStream_t s) {
  if (q.nq == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(work, 0, 4, s);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(bucket_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(sizeof(DsSmem)));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bucket_kernel, kDsBlock,
                                                    sizeof(DsSmem));
  if (e != cudaSuccess) return e;
  const uint64_t grid = std::min<uint64_t>(q.nq, static_cast<uint64_t>(num_sms) * std::max(per_sm, 1));
  count_launch();
  bucket_kernel<<<static_cast<unsigned>(grid), kDsBlock, sizeof(DsSmem), s>>>(
      idx, q, hit_off, wmeta, wflags, q_tie, keys, vals, work);
  return cudaGetLastError();
}

}  // namespace cuflye
