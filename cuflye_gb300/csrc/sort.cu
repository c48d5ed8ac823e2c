// sort.cu — segmented sort of (u64 key, u32 value) pairs in libstdc++ std::sort
// order (see introsort.cuh for why and for the parallel partition).
//
// Segments are classified by size and sorted by four kernels:
//   * <= kTiny elements:      one thread runs the serial algorithm;
//   * <= kWarpSeg elements:   one warp, segment staged in its own shared-memory
//                             slice, partitions by warp ballots, leaves per lane;
//   * <= kCap elements:       one CTA, segment in shared memory; block-wide
//                             partitions while tasks exceed kWarpMax, then all
//                             16 warps partition different tasks concurrently
//                             (level by level), then one thread per leaf task;
//   * larger:                 one CTA partitions in global memory until its
//                             tasks fit kCap, then finishes each in shared memory.
// Every partition is a single pass: L stoppers get ranks from the left, R
// stoppers left ranks too (the k-th R stopper from the right is the
// (TR - k)-th from the left), so a partition reads its keys once.
#include <cstdint>

#include "common.cuh"
#include "introsort.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr int kBlock = 512;
constexpr int kWarps = kBlock / 32;
constexpr uint32_t kCap = 8192;       // CTA shared-memory segment capacity
constexpr uint32_t kWarpMax = 2048;   // tasks up to this size go to single warps
constexpr uint32_t kSerial = 32;      // tasks up to this size go to single threads
constexpr uint32_t kTiny = 64;        // segments up to this size: thread kernel
constexpr uint32_t kWarpSeg = 2048;   // segments up to this size: warp kernel
constexpr int kWarpSegWarps = 6;      // warps per CTA in the warp kernel
constexpr int kMaxWarpTasks = 256;    // disjoint tasks > kSerial in kCap elements
constexpr int kMaxSerial = 1024;
constexpr int kSerialFlush = 512;

// ---------------------------------------------------------------- partitions

// Warp-wide unguarded partition of [f, l) (l - f > 16).  Rank maps: the k-th L
// stopper (k >= 1) at Lr[f + k - 1], the j-th R stopper from the left (j >= 0)
// at Rr[f + j]; both stay inside [f, l).
template <typename RT>
__device__ uint32_t warp_partition(uint64_t* K, uint32_t* V, RT* Lr, RT* Rr, uint32_t f,
                                   uint32_t l) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) isort::median_to_first(K, V, f, f + 1, f + (l - f) / 2, l - 1);
  __syncwarp();
  const uint64_t p = K[f];
  const unsigned lt = (1u << lane) - 1u;
  uint32_t tl = 0, tr = 0;
  for (uint32_t base = f; base < l; base += 32) {
    const uint32_t i = base + lane;
    const bool valid = i < l;
    const uint64_t k = valid ? K[i] : 0;
    const bool isL = valid && i > f && !(k < p);
    const bool isR = valid && !(p < k);
    const unsigned bl = __ballot_sync(0xffffffffu, isL);
    const unsigned br = __ballot_sync(0xffffffffu, isR);
    if (isL) Lr[f + tl + __popc(bl & lt)] = static_cast<RT>(i);
    if (isR) Rr[f + tr + __popc(br & lt)] = static_cast<RT>(i);
    tl += __popc(bl);
    tr += __popc(br);
  }
  __syncwarp();
  // m = largest k with l_k < r_k, l_k = Lr[f + k - 1], r_k = Rr[f + tr - k]
  uint32_t lo = 0, hi = tl < tr ? tl : tr;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (static_cast<uint32_t>(Lr[f + mid - 1]) < static_cast<uint32_t>(Rr[f + tr - mid]))
      lo = mid;
    else
      hi = mid - 1;
  }
  const uint32_t m = lo;
  uint32_t cut;
  if (m == 0) {
    cut = Lr[f];
  } else {
    cut = Rr[f + tr - m];
    if (m + 1 <= tl && static_cast<uint32_t>(Lr[f + m]) < cut) cut = Lr[f + m];
  }
  __syncwarp();
  for (uint32_t k = 1 + lane; k <= m; k += 32) isort::swap_kv(K, V, Lr[f + k - 1], Rr[f + tr - k]);
  __syncwarp();
  return cut;
}

struct BlockScratch {
  uint64_t warp_sums[kWarps + 1];
  uint32_t scalar[4];
};

__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, BlockScratch& bs,
                                                         uint64_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint64_t o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) bs.warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint64_t w = lane < kWarps ? bs.warp_sums[lane] : 0;
    uint64_t wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t o = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += o;
    }
    if (lane < kWarps) bs.warp_sums[lane] = wi - w;
    if (lane == kWarps - 1) bs.warp_sums[kWarps] = wi;
  }
  __syncthreads();
  const uint64_t r = bs.warp_sums[warp] + inc - v;
  *total = bs.warp_sums[kWarps];
  __syncthreads();
  return r;
}

// Block-wide unguarded partition of [f, l), one pass over the keys in tiles
// of kBlock * 16 (each thread owns 16 consecutive positions of a tile).
template <typename RT>
__device__ uint32_t block_partition(uint64_t* K, uint32_t* V, RT* Lr, RT* Rr, uint32_t f,
                                    uint32_t l, BlockScratch& bs) {
  if (threadIdx.x == 0) isort::median_to_first(K, V, f, f + 1, f + (l - f) / 2, l - 1);
  __syncthreads();
  const uint64_t p = K[f];
  uint64_t carry = 0;  // (L count << 32) | R count before the tile
  for (uint32_t t0 = f; t0 < l; t0 += kBlock * 16u) {
    const uint32_t a = t0 + threadIdx.x * 16u;
    uint32_t cl = 0, cr = 0;
    for (uint32_t i = a; i < a + 16u && i < l; ++i) {
      const uint64_t k = K[i];
      cl += (i > f) && !(k < p);
      cr += !(p < k);
    }
    uint64_t tile_tot;
    const uint64_t ex = carry + block_exclusive_scan((static_cast<uint64_t>(cl) << 32) | cr, bs,
                                                     &tile_tot);
    uint32_t rl = static_cast<uint32_t>(ex >> 32);
    uint32_t rr = static_cast<uint32_t>(ex & 0xffffffffu);
    for (uint32_t i = a; i < a + 16u && i < l; ++i) {
      const uint64_t k = K[i];
      if ((i > f) && !(k < p)) Lr[f + rl++] = static_cast<RT>(i);
      if (!(p < k)) Rr[f + rr++] = static_cast<RT>(i);
    }
    carry += tile_tot;
  }
  __syncthreads();
  const uint32_t tl = static_cast<uint32_t>(carry >> 32);
  const uint32_t tr = static_cast<uint32_t>(carry & 0xffffffffu);
  if (threadIdx.x == 0) {
    uint32_t lo = 0, hi = tl < tr ? tl : tr;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (static_cast<uint32_t>(Lr[f + mid - 1]) < static_cast<uint32_t>(Rr[f + tr - mid]))
        lo = mid;
      else
        hi = mid - 1;
    }
    const uint32_t m = lo;
    uint32_t cut;
    if (m == 0) {
      cut = Lr[f];
    } else {
      cut = Rr[f + tr - m];
      if (m + 1 <= tl && static_cast<uint32_t>(Lr[f + m]) < cut) cut = Lr[f + m];
    }
    bs.scalar[0] = m;
    bs.scalar[1] = cut;
  }
  __syncthreads();
  const uint32_t m = bs.scalar[0], cut = bs.scalar[1];
  for (uint32_t k = 1 + threadIdx.x; k <= m; k += kBlock)
    isort::swap_kv(K, V, Lr[f + k - 1], Rr[f + tr - k]);
  __syncthreads();
  return cut;
}

// ---------------------------------------------------------------- CTA sort

struct CtaSmem {
  uint64_t K[kCap];
  uint32_t V[kCap];
  uint16_t Lr[kCap];
  uint16_t Rr[kCap];
  uint32_t bf[64], bl[64];
  int bd[64];
  uint32_t wf[2][kMaxWarpTasks], wl[2][kMaxWarpTasks];
  int wd[2][kMaxWarpTasks];
  uint32_t sf[kMaxSerial], sl[kMaxSerial];
  int sd[kMaxSerial];
  int nb, wn[2], ns;
  BlockScratch bs;
};

// Routes a task to the serial list, the next warp round or the block stack.
// Called by one thread (block phase) or one lane (warp phase); lists are
// appended with atomics because several warps add concurrently.
__device__ __forceinline__ void route_task(CtaSmem& sm, int next, uint32_t f, uint32_t l, int d) {
  const uint32_t n = l - f;
  if (n <= 1) return;
  if (n <= kSerial || d == 0) {
    const int s = atomicAdd(&sm.ns, 1);
    sm.sf[s] = f;
    sm.sl[s] = l;
    sm.sd[s] = d;
  } else if (n <= kWarpMax) {
    const int s = atomicAdd(&sm.wn[next], 1);
    sm.wf[next][s] = f;
    sm.wl[next][s] = l;
    sm.wd[next][s] = d;
  } else {
    const int s = atomicAdd(&sm.nb, 1);
    sm.bf[s] = f;
    sm.bl[s] = l;
    sm.bd[s] = d;
  }
}

__device__ __forceinline__ void flush_serial(CtaSmem& sm) {
  for (int s = threadIdx.x; s < sm.ns; s += kBlock)
    isort::serial_introsort(sm.K, sm.V, sm.sf[s], sm.sl[s], sm.sd[s]);
  __syncthreads();
  if (threadIdx.x == 0) sm.ns = 0;
  __syncthreads();
}

// Sorts sm.K/sm.V[0, n) from recursion budget depth0.
__device__ void cta_sort(CtaSmem& sm, uint32_t n, int depth0) {
  if (threadIdx.x == 0) {
    sm.nb = 0;
    sm.wn[0] = 0;
    sm.wn[1] = 0;
    sm.ns = 0;
    route_task(sm, 0, 0, n, depth0);
  }
  __syncthreads();
  // block phase: tasks larger than kWarpMax, one at a time
  for (;;) {
    const int nb = sm.nb;
    if (nb == 0) break;
    const uint32_t f = sm.bf[nb - 1], l = sm.bl[nb - 1];
    const int d = sm.bd[nb - 1];
    __syncthreads();
    if (threadIdx.x == 0) sm.nb = nb - 1;
    const uint32_t cut = block_partition<uint16_t>(sm.K, sm.V, sm.Lr, sm.Rr, f, l, sm.bs);
    if (threadIdx.x == 0) {
      route_task(sm, 0, f, cut, d - 1);
      route_task(sm, 0, cut, l, d - 1);
    }
    __syncthreads();
    if (sm.ns > kSerialFlush) flush_serial(sm);
  }
  // warp phase: level by level, every warp takes different tasks
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int cur = 0;
  for (;;) {
    const int cnt = sm.wn[cur];
    if (cnt == 0) break;
    if (threadIdx.x == 0) sm.wn[cur ^ 1] = 0;
    __syncthreads();
    for (int t = warp; t < cnt; t += kWarps) {
      const uint32_t f = sm.wf[cur][t], l = sm.wl[cur][t];
      const int d = sm.wd[cur][t];
      const uint32_t cut = warp_partition<uint16_t>(sm.K, sm.V, sm.Lr, sm.Rr, f, l);
      if (lane == 0) {
        route_task(sm, cur ^ 1, f, cut, d - 1);
        route_task(sm, cur ^ 1, cut, l, d - 1);
      }
      __syncwarp();
    }
    __syncthreads();
    if (sm.ns > kSerialFlush) flush_serial(sm);
    cur ^= 1;
  }
  flush_serial(sm);
}

__device__ void cta_load_sort_store(uint64_t* K, uint32_t* V, uint64_t begin, uint32_t n,
                                    int depth, CtaSmem& sm) {
  for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
    sm.K[i] = K[begin + i];
    sm.V[i] = V[begin + i];
  }
  __syncthreads();
  cta_sort(sm, n, depth);
  for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
    K[begin + i] = sm.K[i];
    V[begin + i] = sm.V[i];
  }
  __syncthreads();
}

// ---------------------------------------------------------------- kernels

__global__ void classify_segments(const uint64_t* __restrict__ begin,
                                  const uint64_t* __restrict__ end, uint32_t nseg,
                                  const uint32_t* __restrict__ nseg_dev, uint32_t* lists,
                                  uint32_t* counts) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || (nseg_dev && s >= *nseg_dev)) return;
  const uint64_t n = end[s] - begin[s];
  if (n <= 1) return;
  int c;
  if (n <= kTiny)
    c = 0;
  else if (n <= kWarpSeg)
    c = 1;
  else if (n <= kCap)
    c = 2;
  else
    c = 3;
  lists[static_cast<size_t>(c) * nseg + atomicAdd(&counts[c], 1u)] = s;
}

__global__ void sort_tiny(uint64_t* K, uint32_t* V, const uint64_t* __restrict__ begin,
                          const uint64_t* __restrict__ end, const uint32_t* __restrict__ list,
                          const uint32_t* __restrict__ counts) {
  const uint32_t cnt = counts[0];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
       i += gridDim.x * blockDim.x) {
    const uint32_t s = list[i];
    const uint64_t b = begin[s];
    const uint32_t n = static_cast<uint32_t>(end[s] - b);
    isort::serial_introsort(K + b, V + b, 0, n, isort::depth_limit(n));
  }
}

struct WarpSlice {
  uint64_t K[kWarpSeg];
  uint32_t V[kWarpSeg];
  uint16_t Lr[kWarpSeg];
  uint16_t Rr[kWarpSeg];
  uint32_t sf[64], sl[64];
  int sd[64];
};

// One warp per segment of (kTiny, kWarpSeg] elements.
__global__ void __launch_bounds__(kWarpSegWarps * 32) sort_warp(
    uint64_t* K, uint32_t* V, const uint64_t* __restrict__ begin,
    const uint64_t* __restrict__ end, const uint32_t* __restrict__ list,
    const uint32_t* __restrict__ counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSlice& ws = reinterpret_cast<WarpSlice*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const uint32_t cnt = counts[1];
  const uint32_t nwarps = gridDim.x * kWarpSegWarps;
  for (uint32_t li = blockIdx.x * kWarpSegWarps + (threadIdx.x >> 5); li < cnt; li += nwarps) {
    const uint32_t s = list[li];
    const uint64_t b = begin[s];
    const uint32_t n = static_cast<uint32_t>(end[s] - b);
    for (uint32_t i = lane; i < n; i += 32) {
      ws.K[i] = K[b + i];
      ws.V[i] = V[b + i];
    }
    __syncwarp();
    // task stack (identical in every lane) and a per-warp leaf list
    uint32_t tf[40], tl[40];
    int td[40];
    int top = 0, ns = 0;
    tf[0] = 0;
    tl[0] = n;
    td[0] = isort::depth_limit(n);
    top = 1;
    while (top > 0) {
      --top;
      const uint32_t f = tf[top], l = tl[top];
      const int d = td[top];
      if (l - f <= kSerial || d == 0) {
        if (lane == 0) {
          ws.sf[ns] = f;
          ws.sl[ns] = l;
          ws.sd[ns] = d;
        }
        ++ns;
        if (ns == 64) {
          __syncwarp();
          for (int t = lane; t < ns; t += 32)
            isort::serial_introsort(ws.K, ws.V, ws.sf[t], ws.sl[t], ws.sd[t]);
          __syncwarp();
          ns = 0;
        }
        continue;
      }
      const uint32_t cut = warp_partition<uint16_t>(ws.K, ws.V, ws.Lr, ws.Rr, f, l);
      if (cut - f > 1) {
        tf[top] = f;
        tl[top] = cut;
        td[top] = d - 1;
        ++top;
      }
      if (l - cut > 1) {
        tf[top] = cut;
        tl[top] = l;
        td[top] = d - 1;
        ++top;
      }
    }
    __syncwarp();
    for (int t = lane; t < ns; t += 32)
      isort::serial_introsort(ws.K, ws.V, ws.sf[t], ws.sl[t], ws.sd[t]);
    __syncwarp();
    for (uint32_t i = lane; i < n; i += 32) {
      K[b + i] = ws.K[i];
      V[b + i] = ws.V[i];
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kBlock) sort_cta(uint64_t* K, uint32_t* V,
                                                   const uint64_t* __restrict__ begin,
                                                   const uint64_t* __restrict__ end,
                                                   const uint32_t* __restrict__ list,
                                                   const uint32_t* __restrict__ counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CtaSmem& sm = *reinterpret_cast<CtaSmem*>(smem_raw);
  const uint32_t cnt = counts[2];
  for (uint32_t i = blockIdx.x; i < cnt; i += gridDim.x) {
    const uint32_t s = list[i];
    const uint64_t b = begin[s];
    const uint32_t n = static_cast<uint32_t>(end[s] - b);
    cta_load_sort_store(K, V, b, n, isort::depth_limit(n), sm);
  }
}

// ---------------------------------------------------------------- large segments
//
// Global phase: one CTA of kBigBlock threads per segment partitions in global
// memory until every task fits kCap, and appends the final tasks to a list
// that sort_tasks finishes in shared memory.  A tile holds kRounds rounds of
// kBigBlock consecutive positions; in round r thread t owns position
// r * kBigBlock + t, so loads are coalesced and independent, and the
// (round, warp, lane) order equals position order, which gives the ranks.

constexpr int kBigBlock = 256;
constexpr int kBigWarps = kBigBlock / 32;
constexpr int kRounds = 16;
constexpr uint32_t kBigTile = kBigBlock * kRounds;

struct BigSmem {
  uint32_t cl[kRounds * kBigWarps], cr[kRounds * kBigWarps];  // counts, then offsets
  uint32_t tot[2];
  uint32_t scalar[2];
  uint32_t gf[96], gl[96];
  int gd[96];
  int gn;
};

// Exclusive scan of sm.cl / sm.cr (kRounds * kBigWarps = 128 entries each) by
// the first four warps; totals to sm.tot.
__device__ __forceinline__ void scan_round_counts(BigSmem& sm) {
  static_assert(kRounds * kBigWarps == 128, "scan below covers 128 entries");
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  __shared__ uint32_t wsum[2][4];
  uint32_t vl = 0, vr = 0, il = 0, ir = 0;
  if (t < 128) {
    vl = sm.cl[t];
    vr = sm.cr[t];
    il = vl;
    ir = vr;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t a = __shfl_up_sync(0xffffffffu, il, d);
      const uint32_t b = __shfl_up_sync(0xffffffffu, ir, d);
      if (lane >= d) {
        il += a;
        ir += b;
      }
    }
    if (lane == 31) {
      wsum[0][warp] = il;
      wsum[1][warp] = ir;
    }
  }
  __syncthreads();
  if (t < 128) {
    uint32_t bl = 0, br = 0;
    for (int w = 0; w < warp; ++w) {
      bl += wsum[0][w];
      br += wsum[1][w];
    }
    sm.cl[t] = bl + il - vl;
    sm.cr[t] = br + ir - vr;
    if (t == 127) {
      sm.tot[0] = bl + il;
      sm.tot[1] = br + ir;
    }
  }
  __syncthreads();
}

__device__ uint32_t big_partition_task(uint64_t* K, uint32_t* V, uint32_t* Lr, uint32_t* Rr,
                                       uint32_t f, uint32_t l, BigSmem& sm) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned lt = (1u << lane) - 1u;
  if (t == 0) isort::median_to_first(K, V, f, f + 1, f + (l - f) / 2, l - 1);
  __syncthreads();
  const uint64_t p = K[f];
  uint32_t carry_l = 0, carry_r = 0;
  for (uint32_t t0 = f; t0 < l; t0 += kBigTile) {
    uint64_t k[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const uint32_t i = t0 + r * kBigBlock + t;
      k[r] = i < l ? K[i] : 0;
    }
    unsigned bl[kRounds], br[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const uint32_t i = t0 + r * kBigBlock + t;
      const bool valid = i < l;
      bl[r] = __ballot_sync(0xffffffffu, valid && i > f && !(k[r] < p));
      br[r] = __ballot_sync(0xffffffffu, valid && !(p < k[r]));
      if (lane == 0) {
        sm.cl[r * kBigWarps + warp] = __popc(bl[r]);
        sm.cr[r * kBigWarps + warp] = __popc(br[r]);
      }
    }
    __syncthreads();
    scan_round_counts(sm);
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const uint32_t i = t0 + r * kBigBlock + t;
      if ((bl[r] >> lane) & 1u)
        Lr[f + carry_l + sm.cl[r * kBigWarps + warp] + __popc(bl[r] & lt)] = i;
      if ((br[r] >> lane) & 1u)
        Rr[f + carry_r + sm.cr[r * kBigWarps + warp] + __popc(br[r] & lt)] = i;
    }
    carry_l += sm.tot[0];
    carry_r += sm.tot[1];
    __syncthreads();
  }
  const uint32_t tl = carry_l, tr = carry_r;
  __syncthreads();
  if (t == 0) {
    uint32_t lo = 0, hi = tl < tr ? tl : tr;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (Lr[f + mid - 1] < Rr[f + tr - mid])
        lo = mid;
      else
        hi = mid - 1;
    }
    const uint32_t m = lo;
    uint32_t cut;
    if (m == 0) {
      cut = Lr[f];
    } else {
      cut = Rr[f + tr - m];
      if (m + 1 <= tl && Lr[f + m] < cut) cut = Lr[f + m];
    }
    sm.scalar[0] = m;
    sm.scalar[1] = cut;
  }
  __syncthreads();
  const uint32_t m = sm.scalar[0], cut = sm.scalar[1];
  for (uint32_t q = 1 + t; q <= m; q += kBigBlock) isort::swap_kv(K, V, Lr[f + q - 1], Rr[f + tr - q]);
  __syncthreads();
  return cut;
}

__global__ void __launch_bounds__(kBigBlock) sort_big(uint64_t* K, uint32_t* V, uint32_t* Lg,
                                                      uint32_t* Rg,
                                                      const uint64_t* __restrict__ begin,
                                                      const uint64_t* __restrict__ end,
                                                      const uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ counts,
                                                      uint64_t* task_f, uint32_t* task_n,
                                                      int* task_d, uint32_t* task_count) {
  __shared__ BigSmem sm;
  const uint32_t cnt = counts[3];
  for (uint32_t i = blockIdx.x; i < cnt; i += gridDim.x) {
    const uint32_t s = list[i];
    const uint64_t b = begin[s];
    const uint32_t n = static_cast<uint32_t>(end[s] - b);
    uint64_t* Ks = K + b;
    uint32_t* Vs = V + b;
    uint32_t* Ls = Lg + b;  // rank maps share the segment's index range
    uint32_t* Rs = Rg + b;
    if (threadIdx.x == 0) {
      sm.gf[0] = 0;
      sm.gl[0] = n;
      sm.gd[0] = isort::depth_limit(n);
      sm.gn = 1;
    }
    __syncthreads();
    for (;;) {
      const int nt = sm.gn;
      if (nt == 0) break;
      const uint32_t f = sm.gf[nt - 1], l = sm.gl[nt - 1];
      const int d = sm.gd[nt - 1];
      __syncthreads();
      if (l - f <= kCap) {
        if (threadIdx.x == 0) {
          sm.gn = nt - 1;
          if (l - f > 1) {
            const uint32_t slot = atomicAdd(task_count, 1u);
            task_f[slot] = b + f;
            task_n[slot] = l - f;
            task_d[slot] = d;
          }
        }
        __syncthreads();
        continue;
      }
      if (d == 0) {
        if (threadIdx.x == 0) {
          isort::heap_sort(Ks, Vs, f, l);
          sm.gn = nt - 1;
        }
        __syncthreads();
        continue;
      }
      const uint32_t cut = big_partition_task(Ks, Vs, Ls, Rs, f, l, sm);
      if (threadIdx.x == 0) {
        sm.gf[nt - 1] = cut;
        sm.gl[nt - 1] = l;
        sm.gd[nt - 1] = d - 1;
        sm.gf[nt] = f;
        sm.gl[nt] = cut;
        sm.gd[nt] = d - 1;
        sm.gn = nt + 1;
      }
      __syncthreads();
    }
  }
}

// Finishes the <= kCap tasks left by sort_big, one CTA per task.
__global__ void __launch_bounds__(kBlock) sort_tasks(uint64_t* K, uint32_t* V,
                                                     const uint64_t* __restrict__ task_f,
                                                     const uint32_t* __restrict__ task_n,
                                                     const int* __restrict__ task_d,
                                                     const uint32_t* __restrict__ task_count) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CtaSmem& sm = *reinterpret_cast<CtaSmem*>(smem_raw);
  const uint32_t cnt = *task_count;
  for (uint32_t i = blockIdx.x; i < cnt; i += gridDim.x)
    cta_load_sort_store(K, V, task_f[i], task_n[i], task_d[i], sm);
}

}  // namespace

size_t segsort_smem_bytes() { return sizeof(CtaSmem); }

size_t segsort_task_words(uint64_t nelems, uint32_t nseg) {
  // final tasks of the global phase are disjoint and come from partitions of
  // tasks larger than kCap (at most depth_limit levels of them)
  return nseg + 2 * (nelems / kCap + 1) * 64;
}

cudaError_t segmented_std_sort(uint64_t* keys, uint32_t* vals, uint32_t* lscratch,
                               uint32_t* rscratch, const uint64_t* begin, const uint64_t* end,
                               uint32_t nseg, const uint32_t* nseg_dev, uint32_t* lists,
                               uint32_t* counts, int num_sms, cudaStream_t stream,
                               SortTasks tasks) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(sort_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(CtaSmem)));
    cudaFuncSetAttribute(sort_tasks, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(CtaSmem)));
    cudaFuncSetAttribute(sort_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(WarpSlice) * kWarpSegWarps));
    attr = true;
  }
  if (nseg == 0) return cudaSuccess;
  cudaMemsetAsync(counts, 0, 5 * sizeof(uint32_t), stream);
  count_launch();
  classify_segments<<<(nseg + 255) / 256, 256, 0, stream>>>(begin, end, nseg, nseg_dev, lists,
                                                            counts);
  count_launch();
  sort_tiny<<<num_sms * 4, 128, 0, stream>>>(keys, vals, begin, end, lists, counts);
  count_launch();
  sort_warp<<<num_sms, kWarpSegWarps * 32, sizeof(WarpSlice) * kWarpSegWarps, stream>>>(
      keys, vals, begin, end, lists + nseg, counts);
  count_launch();
  sort_cta<<<num_sms, kBlock, sizeof(CtaSmem), stream>>>(keys, vals, begin, end,
                                                         lists + 2 * static_cast<size_t>(nseg),
                                                         counts);
  count_launch();
  sort_big<<<num_sms * 4, kBigBlock, 0, stream>>>(keys, vals, lscratch, rscratch, begin, end,
                                                  lists + 3 * static_cast<size_t>(nseg), counts,
                                                  tasks.f, tasks.n, tasks.d, counts + 4);
  count_launch();
  sort_tasks<<<num_sms, kBlock, sizeof(CtaSmem), stream>>>(keys, vals, tasks.f, tasks.n, tasks.d,
                                                           counts + 4);
  return cudaGetLastError();
}

}  // namespace cuflye
