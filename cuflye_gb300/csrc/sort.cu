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
//   * larger:                 partitions in global memory, in rounds over all
//                             such ranges (one CTA per range), until the ranges
//                             fit kCap; each is then finished in shared memory.
// Every partition is a single pass: L stoppers get ranks from the left, R
// stoppers left ranks too (the k-th R stopper from the right is the
// (TR - k)-th from the left), so a partition reads its keys once.
// A range sorted in shared memory first tries a radix sort: when its keys
// turn out distinct, that is libstdc++'s result too (the sorted order of
// distinct keys is unique), and only ranges with equal keys are emulated.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "introsort.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
constexpr uint32_t kCap = 4096;       // CTA shared-memory segment capacity
constexpr uint32_t kWarpMax = 512;    // tasks up to this size become warp subtrees
constexpr uint32_t kTiny = 64;        // segments up to this size: thread kernel
constexpr uint32_t kWarpSeg = 2048;   // segments up to this size: warp kernel
constexpr int kWarpSegWarps = 6;      // warps per CTA in the warp kernel
constexpr int kMaxWarpTasks = 256;    // warp subtrees per CTA task (<= 2 per partition)

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

// Block-wide unguarded partition of [f, l) by BLOCK threads, one pass over
// the keys in tiles of kRounds rounds: in round r thread t owns position
// t0 + r * BLOCK + t, so loads are coalesced (and bank-conflict free in
// shared memory) and independent; (round, warp, lane) order is position
// order, so per-(round, warp) ballot counts scanned in that order give ranks.
constexpr int kRounds = 16;

template <int BLOCK, int ROUNDS = kRounds>
struct RoundScratch {
  static constexpr int kW = BLOCK / 32;
  static constexpr int kR = ROUNDS;
  static constexpr int kN = ROUNDS * kW;
  uint32_t cl[kN], cr[kN];  // counts, then exclusive offsets
  uint32_t wsum[2][kN / 32];
  uint32_t tot[2];
  uint32_t scalar[2];
};

template <class RS>
__device__ __forceinline__ void round_scan(RS& rs) {
  constexpr int kN = RS::kN;
  static_assert(kN % 32 == 0 && kN <= RS::kW * 32, "one entry per thread");
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t vl = 0, vr = 0, il = 0, ir = 0;
  if (t < kN) {
    vl = rs.cl[t];
    vr = rs.cr[t];
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
      rs.wsum[0][warp] = il;
      rs.wsum[1][warp] = ir;
    }
  }
  __syncthreads();
  if (t < kN) {
    uint32_t bl = 0, br = 0;
    for (int w = 0; w < warp; ++w) {
      bl += rs.wsum[0][w];
      br += rs.wsum[1][w];
    }
    rs.cl[t] = bl + il - vl;
    rs.cr[t] = br + ir - vr;
    if (t == kN - 1) {
      rs.tot[0] = bl + il;
      rs.tot[1] = br + ir;
    }
  }
  __syncthreads();
}

template <int BLOCK, typename RT, class RS>
__device__ uint32_t round_partition(uint64_t* K, uint32_t* V, RT* Lr, RT* Rr, uint32_t f,
                                    uint32_t l, RS& rs) {
  constexpr int kW = RS::kW;
  constexpr int kRounds = RS::kR;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned lt = (1u << lane) - 1u;
  if (t == 0) isort::median_to_first(K, V, f, f + 1, f + (l - f) / 2, l - 1);
  __syncthreads();
  const uint64_t p = K[f];
  uint32_t carry_l = 0, carry_r = 0;
  for (uint32_t t0 = f; t0 < l; t0 += BLOCK * kRounds) {
    // rounds this tile actually covers (uniform across the block)
    const uint32_t nr = (l - t0 + BLOCK - 1) / BLOCK;
    uint64_t k[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const uint32_t i = t0 + r * BLOCK + t;
      k[r] = (static_cast<uint32_t>(r) < nr && i < l) ? K[i] : 0;
    }
    unsigned bl[kRounds], br[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      bl[r] = 0;
      br[r] = 0;
      if (static_cast<uint32_t>(r) < nr) {
        const uint32_t i = t0 + r * BLOCK + t;
        const bool valid = i < l;
        bl[r] = __ballot_sync(0xffffffffu, valid && i > f && !(k[r] < p));
        br[r] = __ballot_sync(0xffffffffu, valid && !(p < k[r]));
      }
      if (lane == 0) {
        rs.cl[r * kW + warp] = __popc(bl[r]);
        rs.cr[r * kW + warp] = __popc(br[r]);
      }
    }
    __syncthreads();
    round_scan(rs);
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      if (static_cast<uint32_t>(r) >= nr) continue;
      const uint32_t i = t0 + r * BLOCK + t;
      if ((bl[r] >> lane) & 1u)
        Lr[f + carry_l + rs.cl[r * kW + warp] + __popc(bl[r] & lt)] = static_cast<RT>(i);
      if ((br[r] >> lane) & 1u)
        Rr[f + carry_r + rs.cr[r * kW + warp] + __popc(br[r] & lt)] = static_cast<RT>(i);
    }
    carry_l += rs.tot[0];
    carry_r += rs.tot[1];
    __syncthreads();
  }
  const uint32_t tl = carry_l, tr = carry_r;
  if (warp == 0) {
    // m = largest k in [0, min(tl, tr)] with l_k < r_k (true for k = 0 and
    // monotone): 32-way search, each lane probing one candidate per round.
    uint32_t lo = 0, hi = tl < tr ? tl : tr;
    while (lo < hi) {
      const uint32_t step = (hi - lo + 31) / 32;
      const uint32_t k = lo + (lane + 1) * step;
      bool ok = false;
      if (k <= hi)
        ok = static_cast<uint32_t>(Lr[f + k - 1]) < static_cast<uint32_t>(Rr[f + tr - k]);
      const unsigned mask = __ballot_sync(0xffffffffu, ok);
      if (mask == 0) {
        hi = lo + step - 1;
      } else {
        const uint32_t j = 31u - __clz(mask);
        const uint32_t nlo = lo + (j + 1) * step;
        hi = (nlo + step - 1 < hi) ? nlo + step - 1 : hi;
        lo = nlo;
      }
    }
    if (lane == 0) {
      const uint32_t m = lo;
      uint32_t cut;
      if (m == 0) {
        cut = Lr[f];
      } else {
        cut = Rr[f + tr - m];
        if (m + 1 <= tl && static_cast<uint32_t>(Lr[f + m]) < cut) cut = Lr[f + m];
      }
      rs.scalar[0] = m;
      rs.scalar[1] = cut;
    }
  }
  __syncthreads();
  const uint32_t m = rs.scalar[0], cut = rs.scalar[1];
  // swaps, four per thread per iteration so their loads overlap
  for (uint32_t q0 = 1 + t; q0 <= m; q0 += 4 * BLOCK) {
    uint32_t a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t q = q0 + u * BLOCK;
      if (q <= m) {
        a[u] = Lr[f + q - 1];
        b[u] = Rr[f + tr - q];
      }
    }
    uint64_t ka[4], kb[4];
    uint32_t va[4], vb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (q0 + u * BLOCK <= m) {
        ka[u] = K[a[u]];
        kb[u] = K[b[u]];
        va[u] = V[a[u]];
        vb[u] = V[b[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (q0 + u * BLOCK <= m) {
        K[a[u]] = kb[u];
        K[b[u]] = ka[u];
        V[a[u]] = vb[u];
        V[b[u]] = va[u];
      }
    }
  }
  __syncthreads();
  return cut;
}

// ---------------------------------------------------------------- CTA sort

// Leaves: libstdc++ finishes every block of <= 16 elements with a stable
// insertion sort, i.e. the stable sorted order.  Each half-warp sorts one leaf
// in registers: element i moves to (number of smaller keys) + (number of equal
// keys before it).  Lanes read consecutive positions, so shared-memory banks
// do not conflict.
constexpr uint32_t kLeafMax = isort::kLeaf;  // 16
constexpr int kLeafBuf = 64;

struct LeafBuf {
  uint32_t f[kLeafBuf], l[kLeafBuf];
};

__device__ void flush_leaves(uint64_t* K, uint32_t* V, const LeafBuf& lb, int ns) {
  const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
  for (int t0 = 0; t0 < ns; t0 += 2) {
    const int t = t0 + half;
    const bool live = t < ns;
    const uint32_t f = live ? lb.f[t] : 0;
    const uint32_t n = live ? lb.l[t] - f : 0;
    const bool valid = static_cast<uint32_t>(hl) < n;
    const uint64_t k = valid ? K[f + hl] : 0;
    const uint32_t v = valid ? V[f + hl] : 0;
    uint32_t rank = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const uint64_t kj = __shfl_sync(0xffffffffu, k, (half << 4) + j);
      if (static_cast<uint32_t>(j) < n) rank += (kj < k) || (kj == k && j < hl);
    }
    __syncwarp();
    if (valid) {
      K[f + rank] = k;
      V[f + rank] = v;
    }
    __syncwarp();
  }
}

// A warp sorts the subtree of task [f, l) on its own: warp partitions while a
// task exceeds 16 elements (heapsort by one lane once the recursion budget is
// spent), leaves collected in the warp's list and finished two at a time.
// The task stack is identical in every lane; rank maps live in the task's own
// index range of Lr / Rr.
__device__ void warp_subtree_sort(uint64_t* K, uint32_t* V, uint16_t* Lr, uint16_t* Rr,
                                  uint32_t f0, uint32_t l0, int d0, LeafBuf& lb) {
  const int lane = threadIdx.x & 31;
  uint32_t tf[40], tl[40];
  int td[40];
  int top = 0, ns = 0;
  tf[0] = f0;
  tl[0] = l0;
  td[0] = d0;
  top = 1;
  while (top > 0) {
    --top;
    const uint32_t f = tf[top], l = tl[top];
    const int d = td[top];
    if (l - f <= kLeafMax) {
      if (l - f > 1) {
        if (lane == 0) {
          lb.f[ns] = f;
          lb.l[ns] = l;
        }
        ++ns;
        if (ns == kLeafBuf) {
          __syncwarp();
          flush_leaves(K, V, lb, ns);
          ns = 0;
        }
      }
      continue;
    }
    if (d == 0) {
      if (lane == 0) isort::heap_sort(K, V, f, l);
      __syncwarp();
      continue;
    }
    const uint32_t cut = warp_partition<uint16_t>(K, V, Lr, Rr, f, l);
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
  flush_leaves(K, V, lb, ns);
}

struct CtaSmem {
  uint64_t K[kCap];
  uint32_t V[kCap];
  uint16_t Lr[kCap];
  uint16_t Rr[kCap];
  uint32_t bf[64], bl[64];
  int bd[64];
  uint32_t tf[kMaxWarpTasks], tl[kMaxWarpTasks];
  int td[kMaxWarpTasks];
  LeafBuf leaves[kWarps];
  int nb, nt, next;
  RoundScratch<kBlock> rs;
};

// Block phase routing: tasks above kWarpMax stay on the block stack, every
// other task (> 1 element) becomes a warp subtree.
__device__ __forceinline__ void route_task(CtaSmem& sm, uint32_t f, uint32_t l, int d) {
  const uint32_t n = l - f;
  if (n <= 1) return;
  if (n > kWarpMax && d > 0) {
    sm.bf[sm.nb] = f;
    sm.bl[sm.nb] = l;
    sm.bd[sm.nb] = d;
    ++sm.nb;
  } else {
    sm.tf[sm.nt] = f;
    sm.tl[sm.nt] = l;
    sm.td[sm.nt] = d;
    ++sm.nt;
  }
}

// Sorts sm.K/sm.V[0, n) from recursion budget depth0: block-wide partitions
// while tasks exceed kWarpMax, then warps take whole subtrees from the list.
__device__ void cta_sort(CtaSmem& sm, uint32_t n, int depth0) {
  if (threadIdx.x == 0) {
    sm.nb = 0;
    sm.nt = 0;
    sm.next = 0;
    route_task(sm, 0, n, depth0);
  }
  __syncthreads();
  for (;;) {
    const int nb = sm.nb;
    if (nb == 0) break;
    const uint32_t f = sm.bf[nb - 1], l = sm.bl[nb - 1];
    const int d = sm.bd[nb - 1];
    __syncthreads();
    if (threadIdx.x == 0) sm.nb = nb - 1;
    const uint32_t cut = round_partition<kBlock, uint16_t>(sm.K, sm.V, sm.Lr, sm.Rr, f, l, sm.rs);
    if (threadIdx.x == 0) {
      route_task(sm, f, cut, d - 1);
      route_task(sm, cut, l, d - 1);
    }
    __syncthreads();
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nt = sm.nt;
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&sm.next, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= nt) break;
    // a spent budget heap-sorts only ranges above 16 elements; shorter ones
    // are leaves, as in libstdc++'s loop (warp_subtree_sort checks in that order)
    warp_subtree_sort(sm.K, sm.V, sm.Lr, sm.Rr, sm.tf[t], sm.tl[t], sm.td[t], sm.leaves[warp]);
  }
  __syncthreads();
}

// A range whose keys are all distinct has one sorted order, whatever
// libstdc++'s introsort would do with it.  So a range in shared memory first
// takes an LSD radix sort of its positions (16-bit, ping-ponging between the
// two rank maps) by 7-bit digits of key - min, stable per warp-owned slice,
// and a check of neighbours in that order.  It returns the sorted positions
// when no two keys are equal, else null; the keys and values stay as loaded
// either way.  The digit counters overlay the emulation's task-stack fields,
// unused until then.
constexpr int kRadixBits = 7;
constexpr int kRadixBins = 1 << kRadixBits;

struct CtaRadix {
  uint32_t wc[kWarps][kRadixBins];
  uint32_t dbase[kRadixBins];
  uint32_t ws[kWarps];
  uint32_t lo[kWarps], hi[kWarps], lo2[kWarps], hi2[kWarps];
};

__device__ const uint16_t* cta_radix_distinct(CtaSmem& sm, uint32_t n) {
  static_assert(sizeof(CtaRadix) <= sizeof(sm.tf) + sizeof(sm.tl) + sizeof(sm.td) +
                                        sizeof(sm.leaves),
                "radix counters fit the task-stack fields");
  CtaRadix& rx = *reinterpret_cast<CtaRadix*>(sm.tf);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  // smallest and largest key (64-bit, by warp shuffles)
  uint64_t mn = ~0ull, mx = 0;
  for (uint32_t i = t; i < n; i += kBlock) {
    mn = min(mn, sm.K[i]);
    mx = max(mx, sm.K[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, static_cast<uint64_t>(__shfl_xor_sync(0xffffffffu, mn, o)));
    mx = max(mx, static_cast<uint64_t>(__shfl_xor_sync(0xffffffffu, mx, o)));
  }
  if (lane == 0) {
    rx.lo[warp] = static_cast<uint32_t>(mn);
    rx.hi[warp] = static_cast<uint32_t>(mn >> 32);
    rx.lo2[warp] = static_cast<uint32_t>(mx);
    rx.hi2[warp] = static_cast<uint32_t>(mx >> 32);
  }
  __syncthreads();
  uint64_t kmin = ~0ull, kmax = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) {
    kmin = min(kmin, (static_cast<uint64_t>(rx.hi[w]) << 32) | rx.lo[w]);
    kmax = max(kmax, (static_cast<uint64_t>(rx.hi2[w]) << 32) | rx.lo2[w]);
  }
  const uint64_t span = kmax - kmin;
  const int kb = span ? 64 - __clzll(span) : 0;
  if (kb == 0 && n > 1) return nullptr;  // all keys equal: emulate
  uint16_t* src = sm.Lr;
  uint16_t* dst = sm.Rr;
  for (uint32_t i = t; i < n; i += kBlock) src[i] = static_cast<uint16_t>(i);
  const uint32_t per_warp = (((n + 31) / 32 + kWarps - 1) / kWarps) * 32;
  const uint32_t w0 = min(n, warp * per_warp);
  const uint32_t w1 = min(n, w0 + per_warp);
  for (int shift = 0; shift < kb; shift += kRadixBits) {
    for (int i = t; i < kWarps * kRadixBins; i += kBlock) (&rx.wc[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
      const uint32_t j = r0 + lane;
      const bool valid = j < w1;
      const uint32_t d =
          valid ? static_cast<uint32_t>((sm.K[src[j]] - kmin) >> shift) & (kRadixBins - 1)
                : kRadixBins;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      if (valid && lane == __ffs(peers) - 1) rx.wc[warp][d] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // bases: digits in order, warps in order within a digit
    uint32_t tot = 0;
    if (t < kRadixBins) {
      for (int w = 0; w < kWarps; ++w) {
        const uint32_t c = rx.wc[w][t];
        rx.wc[w][t] = tot;
        tot += c;
      }
    }
    uint32_t inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31 && t < kRadixBins) rx.ws[warp] = inc;
    __syncthreads();
    if (t < kRadixBins) {
      uint32_t before = 0;
      for (int w = 0; w < warp; ++w) before += rx.ws[w];
      rx.dbase[t] = before + inc - tot;
    }
    __syncthreads();
    for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
      const uint32_t j = r0 + lane;
      const bool valid = j < w1;
      const uint16_t x = valid ? src[j] : 0;
      const uint32_t d = valid ? static_cast<uint32_t>((sm.K[x] - kmin) >> shift) &
                                     (kRadixBins - 1)
                               : kRadixBins;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t base = valid ? rx.dbase[d] + rx.wc[warp][d] : 0u;
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) rx.wc[warp][d] += __popc(peers);
      __syncwarp();
      if (valid) dst[base + __popc(peers & lt)] = x;
    }
    __syncthreads();
    uint16_t* tmp = src;
    src = dst;
    dst = tmp;
  }
  bool tie = false;
  for (uint32_t i = t + 1; i < n; i += kBlock) tie |= sm.K[src[i]] == sm.K[src[i - 1]];
  return __syncthreads_or(tie) ? nullptr : src;
}

__device__ void cta_load_sort_store(uint64_t* K, uint32_t* V, uint64_t begin, uint32_t n,
                                    int depth, CtaSmem& sm) {
  for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
    sm.K[i] = K[begin + i];
    sm.V[i] = V[begin + i];
  }
  __syncthreads();
  const uint16_t* perm = cta_radix_distinct(sm, n);
  if (perm) {
    for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
      K[begin + i] = sm.K[perm[i]];
      V[begin + i] = sm.V[perm[i]];
    }
    __syncthreads();
    return;
  }
  // equal keys: libstdc++'s order, from the range as loaded
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
  LeafBuf leaves;
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
    warp_subtree_sort(ws.K, ws.V, ws.Lr, ws.Rr, 0, n, isort::depth_limit(n), ws.leaves);
    for (uint32_t i = lane; i < n; i += 32) {
      K[b + i] = ws.K[i];
      V[b + i] = ws.V[i];
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kBlock, 3) sort_cta(uint64_t* K, uint32_t* V,
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
// Global phase, in rounds: each launch partitions every range of its round's
// list (ranges longer than kCap with recursion budget left) in global memory
// (round_partition), one CTA per range, CTAs taking ranges from a counter.
// Children longer than kCap with budget left go to the next round's list,
// shorter ones to the task list that sort_tasks finishes in shared memory,
// and children whose budget ran out to the heap lists.  A range's partition
// depends on its own elements only, so the rounds give libstdc++'s result in
// a breadth-first order, and every CTA has work while ranges remain.

constexpr int kBigBlock = 512;
constexpr int kBigPerSm = 2;

// A range of a round: its elements [f, f + n), depth budget d, segment seg,
// and the key interval [lo, hi] its elements lie in (the pivots above it).
struct RoundItem {
  uint64_t f;
  uint64_t lo, hi;
  uint32_t n;
  int d;
  uint32_t seg;
  uint32_t pad;
};
static_assert(sizeof(RoundItem) == kRoundItemBytes, "round item size");

struct PruneLists {
  const uint64_t* keys;
  const uint32_t* off;
};

// Whether segment seg's list holds a key in [lo, hi] (always, without lists).
__device__ __forceinline__ bool holds_listed_key(const PruneLists& pl, uint32_t seg, uint64_t lo,
                                                 uint64_t hi) {
  if (!pl.off) return true;
  uint32_t a = pl.off[seg], b = pl.off[seg + 1];
  while (a < b) {  // first key >= lo
    const uint32_t m = (a + b) >> 1;
    if (pl.keys[m] < lo)
      a = m + 1;
    else
      b = m;
  }
  return a < pl.off[seg + 1] && pl.keys[a] <= hi;
}

// Where a child range of a global-phase partition goes.
__device__ __forceinline__ void place_range(const RoundItem& r, RoundItem* out,
                                            uint32_t* out_count, uint64_t* task_f,
                                            uint32_t* task_n, int* task_d, uint32_t* task_count,
                                            uint32_t* heap_count, uint32_t* pair_count,
                                            uint32_t task_cap, uint32_t pair_reserve,
                                            const PruneLists& pl) {
  const uint64_t f = r.f;
  const uint32_t n = r.n;
  const int d = r.d;
  if (n > 1 && !holds_listed_key(pl, r.seg, r.lo, r.hi)) return;  // distinct keys: dropped
  if (n <= kCap) {
    if (n > 1) {
      const uint32_t slot = atomicAdd(task_count, 1u);
      task_f[slot] = f;
      task_n[slot] = n;
      task_d[slot] = d;
    }
  } else if (d == 0) {
    // depth exhausted: libstdc++ heap-sorts the range; sort_heaps does it
    // (listed from the top of the task arrays: ranges beyond one block's
    // shared memory first, then the others)
    const uint32_t slot = n > kHeapPackCap
                              ? task_cap - 1u - atomicAdd(pair_count, 1u)
                              : task_cap - 1u - pair_reserve - atomicAdd(heap_count, 1u);
    task_f[slot] = f;
    task_n[slot] = n;
    task_d[slot] = 0;
  } else {
    out[atomicAdd(out_count, 1u)] = r;
  }
}

// The round-0 list: the segments longer than kCap with libstdc++'s budget.
__global__ void round_seed(const uint64_t* __restrict__ begin, const uint64_t* __restrict__ end,
                           const uint32_t* __restrict__ list, const uint32_t* __restrict__ counts,
                           RoundItem* __restrict__ out) {
  const uint32_t cnt = counts[3];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const uint32_t s = list[i];
    const uint32_t n = static_cast<uint32_t>(end[s] - begin[s]);
    out[i] = RoundItem{begin[s], 0ull, ~0ull, n, isort::depth_limit(n), s, 0u};
  }
}

__global__ void __launch_bounds__(kBigBlock, kBigPerSm)
    sort_round(uint64_t* K, uint32_t* V, uint32_t* Lg, uint32_t* Rg,
               const RoundItem* __restrict__ in, const uint32_t* __restrict__ in_count,
               uint32_t* work, RoundItem* out, uint32_t* out_count, uint64_t* task_f,
               uint32_t* task_n, int* task_d, uint32_t* task_count, uint32_t* heap_count,
               uint32_t* pair_count, uint32_t task_cap, uint32_t pair_reserve, PruneLists pl) {
  __shared__ RoundScratch<kBigBlock, 8> rs;
  __shared__ uint32_t item;
  const uint32_t cnt = *in_count;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t i = item;
    __syncthreads();
    if (i >= cnt) break;
    const RoundItem r = in[i];
    // rank maps share the range's index range
    const uint32_t cut =
        round_partition<kBigBlock, uint32_t>(K + r.f, V + r.f, Lg + r.f, Rg + r.f, 0, r.n, rs);
    if (threadIdx.x == 0) {
      // the pivot stays at the range's first slot: the left part holds keys
      // <= it, the right part keys >= it
      const uint64_t p = K[r.f];
      const RoundItem left{r.f, r.lo, p, cut, r.d - 1, r.seg, 0u};
      const RoundItem right{r.f + cut, p, r.hi, r.n - cut, r.d - 1, r.seg, 0u};
      place_range(left, out, out_count, task_f, task_n, task_d, task_count, heap_count,
                  pair_count, task_cap, pair_reserve, pl);
      place_range(right, out, out_count, task_f, task_n, task_d, task_count, heap_count,
                  pair_count, task_cap, pair_reserve, pl);
    }
    __syncthreads();
  }
}

// Finishes the <= kCap tasks left by the global phase, one CTA per task.
__global__ void __launch_bounds__(kBlock, 3) sort_tasks(uint64_t* K, uint32_t* V,
                                                     const uint64_t* __restrict__ task_f,
                                                     const uint32_t* __restrict__ task_n,
                                                     const int* __restrict__ task_d,
                                                     const uint32_t* __restrict__ task_count,
                                                     uint32_t* work) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CtaSmem& sm = *reinterpret_cast<CtaSmem*>(smem_raw);
  __shared__ uint32_t item;
  const uint32_t cnt = *task_count;
  // blocks claim tasks from a counter: a task with equal keys runs the whole
  // emulation and costs far more than one the radix check finishes
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(work, 1u);
    __syncthreads();
    const uint32_t i = item;
    __syncthreads();
    if (i >= cnt) break;
    if (task_n[i] <= kCap) cta_load_sort_store(K, V, task_f[i], task_n[i], task_d[i], sm);
  }
}

// Heapsorts the tasks longer than kCap (ranges whose introsort depth ran out
// in the global phase), as libstdc++'s make_heap and sort_heap do: the heap is
// built level by level (sibling subtrees are disjoint, so building a level in
// parallel equals libstdc++'s right-to-left order), then one thread pops it.
//
// The heap only compares keys, so each key is replaced by its dense rank among
// the range's keys, found by an LSD radix sort of (key - min) << s | position
// in the range's own key slots and the two scratch maps.  Heap entries are
// 4-byte words holding the rank in the high bits:
//   * own form (ranges of up to kPackCap elements): rank << 16 | position, in
//     the block's shared memory;
//   * pair form (up to kPairCap elements): rank << 15 | index within the run
//     of equal keys, in the shared memory of a block pair (a cluster of two;
//     the second block lends its shared memory for the deeper nodes); a run's
//     start in sorted order maps an entry back to its position.
// A node's two children are one 8-byte word, its four grandchildren one
// 16-byte word.  The sorted keys are the radix sort's; the heap gives the
// order of the positions, so the values are gathered by it.  Ranges whose
// keys span too many bits: 12-byte entries in shared memory up to kHeapCap,
// beyond that in place in device memory.
constexpr uint32_t kHeapCap = 18432;
constexpr uint32_t kPackCap = kHeapPackCap;
constexpr uint32_t kPairCap = 2 * kPackCap - 1;
constexpr int kHeapBlock = 512;
constexpr int kHeapWarps = kHeapBlock / 32;
constexpr size_t kHeapSmem =
    std::max<size_t>(kHeapCap * (sizeof(uint64_t) + sizeof(uint32_t)), (kPackCap + 2) * 4);

// key(a) < key(b) for entries rank << SH | low bits: a's rank is below b's
// exactly when a < (b with its low bits cleared)
template <int SH>
__device__ __forceinline__ bool rank_less(uint32_t a, uint32_t b) {
  constexpr uint32_t hi = ~((1u << SH) - 1u);
  return a < (b & hi);
}

// Node x lives at word x + 1, so the children 2x + 1 and 2x + 2 of x share
// one 8-byte word and the grandchildren one 16-byte word.
struct OwnHeap {
  uint32_t* E;
  __device__ __forceinline__ uint32_t* at(uint32_t i) const { return E + i; }
  __device__ __forceinline__ uint32_t ld(uint32_t w) const { return E[w]; }
  __device__ __forceinline__ uint2 ld2(uint32_t w) const {
    return *reinterpret_cast<const uint2*>(E + w);
  }
  __device__ __forceinline__ uint4 ld4(uint32_t w) const {
    return *reinterpret_cast<const uint4*>(E + w);
  }
  __device__ __forceinline__ void st(uint32_t w, uint32_t x) const { E[w] = x; }
};
// Words from kPackCap on live in the partner block (a multiple of 8, so no
// aligned 8- or 16-byte word straddles the two).  The heap's own loads and
// stores address both blocks in the cluster's shared window (lb: this
// block's word 0, rb: the partner's, which holds word kPackCap).
struct PairHeap {
  uint32_t* E;
  uint32_t* E1;
  uint32_t lb, rb;
  __device__ __forceinline__ uint32_t* at(uint32_t i) const {
    return i < kPackCap ? E + i : E1 + (i - kPackCap);
  }
  __device__ __forceinline__ uint32_t addr(uint32_t w) const {
    return w < kPackCap ? lb + 4u * w : rb + 4u * (w - kPackCap);
  }
  __device__ __forceinline__ uint32_t ld(uint32_t w) const {
    uint32_t x;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(x) : "r"(addr(w)));
    return x;
  }
  __device__ __forceinline__ uint2 ld2(uint32_t w) const {
    uint2 x;
    asm volatile("ld.shared::cluster.v2.u32 {%0, %1}, [%2];" : "=r"(x.x), "=r"(x.y) : "r"(addr(w)));
    return x;
  }
  __device__ __forceinline__ uint4 ld4(uint32_t w) const {
    uint4 x;
    asm volatile("ld.shared::cluster.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(x.x), "=r"(x.y), "=r"(x.z), "=r"(x.w)
                 : "r"(addr(w)));
    return x;
  }
  __device__ __forceinline__ void st(uint32_t w, uint32_t x) const {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr(w)), "r"(x) : "memory");
  }
};

// libstdc++ __adjust_heap on packed entries.
template <int SH, class H>
__device__ __forceinline__ void packed_adjust(H h, uint32_t hole, uint32_t len, uint32_t v) {
  const uint32_t top = hole;
  uint32_t child = hole;
  const uint32_t lim = len > 2 ? (len - 1) / 2 : 0;
  // three of libstdc++'s steps at once while every node two levels below the
  // hole has two children: the 2 + 4 + 8 candidate nodes load together
  while (4 * child + 6 < lim) {
    const uint2 a = h.ld2(2 * (child + 1));
    const uint4 b = h.ld4(4 * (child + 1));
    const uint4 c0 = h.ld4(8 * (child + 1));
    const uint4 c1 = h.ld4(8 * (child + 1) + 4);
    const bool s1 = !rank_less<SH>(a.y, a.x);  // the right child unless right < left
    const uint32_t v1 = s1 ? a.y : a.x;
    const uint32_t l2 = s1 ? b.z : b.x, r2 = s1 ? b.w : b.y;
    const bool s2 = !rank_less<SH>(r2, l2);
    const uint32_t v2 = s2 ? r2 : l2;
    const uint4 cc = s1 ? c1 : c0;
    const uint32_t l3 = s2 ? cc.z : cc.x, r3 = s2 ? cc.w : cc.y;
    const bool s3 = !rank_less<SH>(r3, l3);
    const uint32_t v3 = s3 ? r3 : l3;
    const uint32_t n1 = 2 * child + 1 + s1;
    const uint32_t n2 = 2 * n1 + 1 + s2;
    h.st(child + 1, v1);
    h.st(n1 + 1, v2);
    h.st(n2 + 1, v3);
    child = 2 * n2 + 1 + s3;
  }
  hole = child;
  while (child < lim) {
    child = 2 * (child + 1);
    const uint2 pr = h.ld2(child);  // nodes child - 1, child
    uint32_t c = pr.y;
    if (rank_less<SH>(pr.y, pr.x)) {
      --child;
      c = pr.x;
    }
    h.st(hole + 1, c);
    hole = child;
  }
  if ((len & 1u) == 0 && len >= 2 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    h.st(hole + 1, h.ld(child));
    hole = child - 1;
  }
  while (hole > top) {
    const uint32_t parent = (hole - 1) / 2;
    const uint32_t pv = h.ld(parent + 1);
    if (!rank_less<SH>(pv, v)) break;
    h.st(hole + 1, pv);
    hole = parent;
  }
  h.st(hole + 1, v);
}

// make_heap by levels (all threads), then sort_heap (thread 0).
template <int SH, class H>
__device__ void packed_heap_run(H h, uint32_t n) {
  const uint32_t last_parent = (n - 2) / 2;
  for (int lv = 31 - __clz(last_parent + 1); lv >= 0; --lv) {
    const uint32_t lo = (1u << lv) - 1u;
    const uint32_t hi = min((2u << lv) - 2u, last_parent);
    for (uint32_t p = lo + threadIdx.x; p <= hi; p += kHeapBlock)
      packed_adjust<SH>(h, p, n, h.ld(p + 1));
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (uint32_t last = n - 1; last >= 1; --last) {
      const uint32_t v = h.ld(last + 1);
      h.st(last + 1, h.ld(1));
      packed_adjust<SH>(h, 0, last, v);
    }
  }
  __syncthreads();
}

struct HeapShared {
  uint32_t kmin_hi, kmin_lo, kmax_hi, kmax_lo;
  uint32_t carry, cstart, item;
  uint32_t ws[kHeapWarps];
  uint32_t wm[kHeapWarps];
};

__device__ __forceinline__ uint64_t heap_pair_load(const uint64_t* K, const uint32_t* hi,
                                                   const uint32_t* lo, bool in_keys, uint64_t i) {
  return in_keys ? K[i] : ((static_cast<uint64_t>(hi[i]) << 32) | lo[i]);
}

__device__ __forceinline__ void heap_pair_store(uint64_t* K, uint32_t* hi, uint32_t* lo,
                                                bool in_keys, uint64_t i, uint64_t x) {
  if (in_keys) {
    K[i] = x;
  } else {
    hi[i] = static_cast<uint32_t>(x >> 32);
    lo[i] = static_cast<uint32_t>(x);
  }
}

// Smallest key and the bit span of (key - smallest) over K[f, f + n).
__device__ void heap_key_span(const uint64_t* K, uint64_t f, uint32_t n, HeapShared& hs,
                              uint64_t& kmin, int& kb) {
  if (threadIdx.x == 0) {
    hs.kmin_hi = hs.kmin_lo = 0xffffffffu;
    hs.kmax_hi = hs.kmax_lo = 0;
  }
  __syncthreads();
  uint64_t lmin = ~0ull, lmax = 0;
  for (uint32_t j = threadIdx.x; j < n; j += kHeapBlock) {
    const uint64_t k = K[f + j];
    lmin = min(lmin, k);
    lmax = max(lmax, k);
  }
  // 64-bit min / max as (hi, lo): hi first, then lo among the threads holding
  // the extreme hi
  atomicMin(&hs.kmin_hi, static_cast<uint32_t>(lmin >> 32));
  atomicMax(&hs.kmax_hi, static_cast<uint32_t>(lmax >> 32));
  __syncthreads();
  if (static_cast<uint32_t>(lmin >> 32) == hs.kmin_hi)
    atomicMin(&hs.kmin_lo, static_cast<uint32_t>(lmin));
  if (static_cast<uint32_t>(lmax >> 32) == hs.kmax_hi)
    atomicMax(&hs.kmax_lo, static_cast<uint32_t>(lmax));
  __syncthreads();
  kmin = (static_cast<uint64_t>(hs.kmin_hi) << 32) | hs.kmin_lo;
  const uint64_t kmax = (static_cast<uint64_t>(hs.kmax_hi) << 32) | hs.kmax_lo;
  const uint64_t span = kmax - kmin;
  kb = span ? 64 - __clzll(span) : 0;
  __syncthreads();
}

// K[f + j] = (K[f + j] - kmin) << sh | j, then an LSD radix sort on the key
// bits [sh, sh + kb) (8 per pass, stable), ping-ponging with the (Rg, Lg)
// pairs; ends with the sorted words in K.  Counters live in `scratch` (the
// heap's shared memory, unused until the heap is built).
__device__ void heap_radix(uint64_t* K, uint32_t* Lg, uint32_t* Rg, uint64_t f, uint32_t n,
                           uint64_t kmin, int sh, int kb, uint32_t* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t j = threadIdx.x; j < n; j += kHeapBlock)
    K[f + j] = ((K[f + j] - kmin) << sh) | j;
  uint32_t (*wc)[256] = reinterpret_cast<uint32_t (*)[256]>(scratch);
  uint32_t* dbase = scratch + kHeapWarps * 256;
  uint32_t* dws = dbase + 256;
  const uint32_t per_warp = (((n + 31) / 32 + kHeapWarps - 1) / kHeapWarps) * 32;
  const uint32_t w0 = min(n, warp * per_warp);
  const uint32_t w1 = min(n, w0 + per_warp);
  bool in_keys = true;
  for (int shift = sh; shift < sh + kb; shift += 8) {
    for (int i = threadIdx.x; i < kHeapWarps * 256; i += kHeapBlock) (&wc[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
      const uint32_t j = r0 + lane;
      const bool valid = j < w1;
      const uint32_t d =
          valid ? static_cast<uint32_t>(heap_pair_load(K, Rg, Lg, in_keys, f + j) >> shift) & 0xffu
                : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      if (valid && lane == __ffs(peers) - 1) wc[warp][d] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // warp-major prefix within each digit, then digit bases
    uint32_t tot = 0;
    if (threadIdx.x < 256) {
      for (int w = 0; w < kHeapWarps; ++w) {
        const uint32_t c = wc[w][threadIdx.x];
        wc[w][threadIdx.x] = tot;
        tot += c;
      }
    }
    uint32_t inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += u;
    }
    if (lane == 31 && warp < 8) dws[warp] = inc;
    __syncthreads();
    if (threadIdx.x < 256) {
      uint32_t before = 0;
      for (int w = 0; w < warp; ++w) before += dws[w];
      dbase[threadIdx.x] = before + inc - tot;
    }
    __syncthreads();
    for (uint32_t r0 = w0; r0 < w1; r0 += 32) {
      const uint32_t j = r0 + lane;
      const bool valid = j < w1;
      const uint64_t x = valid ? heap_pair_load(K, Rg, Lg, in_keys, f + j) : 0;
      const uint32_t d = valid ? static_cast<uint32_t>(x >> shift) & 0xffu : 256u;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t base = valid ? dbase[d] + wc[warp][d] : 0u;
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) wc[warp][d] += __popc(peers);
      __syncwarp();
      if (valid) heap_pair_store(K, Rg, Lg, !in_keys, f + base + __popc(peers & lt), x);
    }
    __syncthreads();
    in_keys = !in_keys;
  }
  if (!in_keys) {
    for (uint32_t j = threadIdx.x; j < n; j += kHeapBlock)
      K[f + j] = heap_pair_load(K, Rg, Lg, false, f + j);
  }
  __syncthreads();
}

// Runs of equal keys over the sorted words K[f, f + n) (key bits from sh
// up): for each sorted index i its dense rank and the index where its run
// starts; `act(i, word, rank, start, first)` is called for every i.
template <class Act>
__device__ void heap_runs(const uint64_t* K, uint64_t f, uint32_t n, int sh, HeapShared& hs,
                          Act act) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t le = (2u << lane) - 1u;
  if (threadIdx.x == 0) {
    hs.carry = 0;
    hs.cstart = 0;
  }
  __syncthreads();
  for (uint32_t c0 = 0; c0 < n; c0 += kHeapBlock) {
    const uint32_t i = c0 + threadIdx.x;
    const bool valid = i < n;
    const uint64_t w = valid ? K[f + i] : 0;
    const bool first = valid && (i == 0 || (w >> sh) != (K[f + i - 1] >> sh));
    const unsigned bal = __ballot_sync(0xffffffffu, first);
    uint32_t st = first ? i : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, st, o);
      if (lane >= o) st = max(st, y);
    }
    if (lane == 31) {
      hs.ws[warp] = __popc(bal);
      hs.wm[warp] = st;
    }
    __syncthreads();
    uint32_t count = hs.carry, start = max(hs.cstart, st);
    for (int v = 0; v < warp; ++v) {
      count += hs.ws[v];
      start = max(start, hs.wm[v]);
    }
    count += __popc(bal & le);
    if (valid) act(i, w, count - 1u, start, first);
    __syncthreads();
    if (threadIdx.x == kHeapBlock - 1) {
      hs.carry = count;
      hs.cstart = start;
    }
    __syncthreads();
  }
}

// Own form: ranges of up to kPackCap elements whose keys span at most 47 bits.
__device__ void own_heap_sort(uint64_t* K, uint32_t* V, uint32_t* Lg, uint32_t* Rg, uint64_t f,
                              uint32_t n, uint64_t kmin, int kb, uint32_t* E, HeapShared& hs) {
  heap_radix(K, Lg, Rg, f, n, kmin, 16, kb, E);
  const OwnHeap h{E};
  heap_runs(K, f, n, 16, hs, [&](uint32_t, uint64_t w, uint32_t rank, uint32_t, bool) {
    const uint32_t pos = static_cast<uint32_t>(w & 0xffffu);
    *h.at(pos + 1) = (rank << 16) | pos;
  });
  packed_heap_run<16>(h, n);
  for (uint32_t i = threadIdx.x; i < n; i += kHeapBlock) {
    K[f + i] = kmin + (K[f + i] >> 16);
    Lg[f + i] = V[f + (*h.at(i + 1) & 0xffffu)];
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += kHeapBlock) V[f + i] = Lg[f + i];
  __syncthreads();
}

// Pair form: ranges of up to kPairCap elements whose keys span at most 46
// bits and whose runs of equal keys are shorter than 32,768.  Returns false,
// with K as it was, when a run is longer.
__device__ bool pair_heap_sort(uint64_t* K, uint32_t* V, uint32_t* Lg, uint32_t* Rg, uint64_t f,
                               uint32_t n, uint64_t kmin, int kb, PairHeap h, HeapShared& hs) {
  heap_radix(K, Lg, Rg, f, n, kmin, 17, kb, h.E);
  bool long_run = false;
  heap_runs(K, f, n, 17, hs, [&](uint32_t i, uint64_t, uint32_t, uint32_t start, bool) {
    long_run |= i - start >= 32768u;
  });
  if (__syncthreads_or(long_run)) {
    // put the keys back in position order
    for (uint32_t i = threadIdx.x; i < n; i += kHeapBlock) {
      const uint64_t w = K[f + i];
      heap_pair_store(K, Rg, Lg, false, f + (w & 0x1ffffu), kmin + (w >> 17));
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < n; j += kHeapBlock)
      K[f + j] = heap_pair_load(K, Rg, Lg, false, f + j);
    __syncthreads();
    return false;
  }
  heap_runs(K, f, n, 17, hs, [&](uint32_t i, uint64_t w, uint32_t rank, uint32_t start, bool first) {
    if (first) Rg[f + rank] = i;
    *h.at(static_cast<uint32_t>(w & 0x1ffffu) + 1) = (rank << 15) | (i - start);
  });
  packed_heap_run<15>(h, n);
  for (uint32_t i = threadIdx.x; i < n; i += kHeapBlock) {
    const uint32_t e = *h.at(i + 1);
    const uint32_t s = Rg[f + (e >> 15)] + (e & 0x7fffu);
    Lg[f + i] = V[f + static_cast<uint32_t>(K[f + s] & 0x1ffffu)];
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += kHeapBlock) K[f + i] = kmin + (K[f + i] >> 17);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += kHeapBlock) V[f + i] = Lg[f + i];
  __syncthreads();
  return true;
}

// 12-byte entries in shared memory (ranges of up to kHeapCap elements).
__device__ void wide_heap_sort(uint64_t* K, uint32_t* V, uint64_t f, uint32_t n,
                               unsigned char* raw) {
  uint64_t* hk = reinterpret_cast<uint64_t*>(raw);
  uint32_t* hv = reinterpret_cast<uint32_t*>(hk + kHeapCap);
  for (uint32_t j = threadIdx.x; j < n; j += kHeapBlock) {
    hk[j] = K[f + j];
    hv[j] = V[f + j];
  }
  __syncthreads();
  const uint32_t last_parent = (n - 2) / 2;
  for (int lv = 31 - __clz(last_parent + 1); lv >= 0; --lv) {
    const uint32_t lo = (1u << lv) - 1u;
    const uint32_t hi = min((2u << lv) - 2u, last_parent);
    for (uint32_t p = lo + threadIdx.x; p <= hi; p += kHeapBlock)
      isort::heap_adjust(hk, hv, 0, p, n, hk[p], hv[p]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (uint32_t last = n; last > 1;) {
      --last;
      const uint64_t vk = hk[last];
      const uint32_t vv = hv[last];
      hk[last] = hk[0];
      hv[last] = hv[0];
      isort::heap_adjust(hk, hv, 0, 0, last, vk, vv);
    }
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < n; j += kHeapBlock) {
    K[f + j] = hk[j];
    V[f + j] = hv[j];
  }
  __syncthreads();
}

// Heap tasks sit at the top of the task arrays: tasks longer than kPackCap
// (pair tasks) at slot task_cap - 1 - j, the others below the pair reserve.
// Each block pair first takes pair tasks together (the first block works,
// the second lends its shared memory), then both blocks take the other tasks
// one at a time from a counter (their lengths vary).
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kHeapBlock, 1)
    sort_heaps(uint64_t* K, uint32_t* V, uint32_t* Lg, uint32_t* Rg,
               const uint64_t* __restrict__ task_f, const uint32_t* __restrict__ task_n,
               const uint32_t* __restrict__ heap_count, uint32_t* heap_work,
               const uint32_t* __restrict__ pair_count, uint32_t* pair_work, uint32_t task_cap,
               uint32_t pair_reserve) {
  extern __shared__ __align__(16) unsigned char heap_raw[];
  __shared__ HeapShared hs;
  uint32_t* E = reinterpret_cast<uint32_t*>(heap_raw);
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned crank = cluster.block_rank();
  const uint32_t npair = *pair_count;
  for (;;) {
    if (crank == 0 && threadIdx.x == 0) {
      const uint32_t it = atomicAdd(pair_work, 1u);
      hs.item = it;
      *cluster.map_shared_rank(&hs.item, 1) = it;
    }
    cluster.sync();
    const uint32_t item = hs.item;
    if (item >= npair) break;
    if (crank == 0) {
      const uint32_t i = task_cap - 1u - item;
      const uint32_t n = task_n[i];
      const uint64_t f = task_f[i];
      uint64_t kmin = 0;
      int kb = 0;
      heap_key_span(K, f, n, hs, kmin, kb);
      const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(E));
      uint32_t lb, rb;
      asm("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(lb) : "r"(sa));
      asm("mapa.shared::cluster.u32 %0, %1, 1;" : "=r"(rb) : "r"(sa));
      const PairHeap h{E, cluster.map_shared_rank(E, 1), lb, rb};
      const bool done = n <= kPairCap && kb <= 46 && pair_heap_sort(K, V, Lg, Rg, f, n, kmin, kb, h, hs);
      if (!done) {
        if (threadIdx.x == 0) isort::heap_sort(K + f, V + f, 0, n);
        __syncthreads();
      }
    }
    cluster.sync();
  }
  const uint32_t cnt = *heap_count;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) hs.item = atomicAdd(heap_work, 1u);
    __syncthreads();
    const uint32_t item = hs.item;
    if (item >= cnt) break;
    const uint32_t i = task_cap - 1u - pair_reserve - item;
    const uint32_t n = task_n[i];
    const uint64_t f = task_f[i];
    uint64_t kmin = 0;
    int kb = 0;
    heap_key_span(K, f, n, hs, kmin, kb);
    if (kb <= 47) {
      own_heap_sort(K, V, Lg, Rg, f, n, kmin, kb, E, hs);
    } else if (n <= kHeapCap) {
      wide_heap_sort(K, V, f, n, heap_raw);
    } else {
      if (threadIdx.x == 0) isort::heap_sort(K + f, V + f, 0, n);
      __syncthreads();
    }
  }
}

}  // namespace

// Blocks over fixed chunks of the compact copy (its ranges ascending in
// cbeg, end to end): each element finds its range by a search of cbeg.
constexpr uint32_t kGatherChunk = 4096;

__global__ void gather_ranges_kernel(const uint64_t* __restrict__ keys,
                                     const uint32_t* __restrict__ vals,
                                     const uint64_t* __restrict__ begin,
                                     const uint64_t* __restrict__ cbeg, uint32_t nseg,
                                     uint64_t total, uint64_t* __restrict__ ck,
                                     uint32_t* __restrict__ cv) {
  const uint64_t nchunk = (total + kGatherChunk - 1) / kGatherChunk;
  for (uint64_t ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
    const uint64_t c0 = ch * kGatherChunk;
    // the range holding the chunk's first element
    uint32_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
      const uint32_t m = (lo + hi) >> 1;
      if (cbeg[m] <= c0)
        lo = m;
      else
        hi = m;
    }
    const uint64_t c1 = c0 + kGatherChunk < total ? c0 + kGatherChunk : total;
    for (uint64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
      uint32_t s = lo;
      while (s + 1 < nseg && cbeg[s + 1] <= c) ++s;
      const uint64_t src = begin[s] + (c - cbeg[s]);
      ck[c] = keys[src];
      cv[c] = vals[src];
    }
  }
}

// Sorted ranges of the pruned sort: items [0, nseg) are the segments (copied
// when they have at most kCap elements), then the tasks, the block-pair heaps
// and the own-block heaps.
__global__ void copy_sorted_kernel(const uint64_t* __restrict__ ck, const uint32_t* __restrict__ cv,
                                   const uint64_t* __restrict__ cbeg,
                                   const uint64_t* __restrict__ cend,
                                   const uint64_t* __restrict__ begin, uint32_t nseg,
                                   const uint32_t* __restrict__ counts,
                                   const uint64_t* __restrict__ task_f,
                                   const uint32_t* __restrict__ task_n, uint32_t task_cap,
                                   uint32_t pair_reserve, uint64_t* __restrict__ keys,
                                   uint32_t* __restrict__ vals) {
  const uint32_t ntask = counts[4], nheap = counts[5], npair = counts[7];
  const uint64_t items = static_cast<uint64_t>(nseg) + ntask + npair + nheap;
  for (uint64_t it = blockIdx.x; it < items; it += gridDim.x) {
    uint64_t f = 0, n = 0;
    if (it < nseg) {
      f = cbeg[it];
      n = cend[it] - f;
      if (n > kCap) continue;  // the global phase's ranges come below
    } else {
      uint64_t j = it - nseg;
      uint32_t slot;
      if (j < ntask) {
        slot = static_cast<uint32_t>(j);
      } else if ((j -= ntask) < npair) {
        slot = task_cap - 1u - static_cast<uint32_t>(j);
      } else {
        j -= npair;
        slot = task_cap - 1u - pair_reserve - static_cast<uint32_t>(j);
      }
      f = task_f[slot];
      n = task_n[slot];
    }
    // the segment holding f: the last s with cbeg[s] <= f
    uint32_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
      const uint32_t m = (lo + hi) >> 1;
      if (cbeg[m] <= f)
        lo = m;
      else
        hi = m;
    }
    const uint64_t dst = begin[lo] + (f - cbeg[lo]);
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
      keys[dst + i] = ck[f + i];
      vals[dst + i] = cv[f + i];
    }
  }
}

size_t segsort_smem_bytes() { return sizeof(CtaSmem); }

cudaError_t gather_ranges(const uint64_t* keys, const uint32_t* vals, const uint64_t* begin,
                          const uint64_t* cbeg, uint32_t nseg, uint64_t total, uint64_t* ck,
                          uint32_t* cv, int num_sms, cudaStream_t s) {
  if (nseg == 0 || total == 0) return cudaSuccess;
  count_launch();
  const uint64_t nchunk = (total + kGatherChunk - 1) / kGatherChunk;
  gather_ranges_kernel<<<static_cast<unsigned>(std::min<uint64_t>(nchunk, 16ull * num_sms)), 512,
                         0, s>>>(keys, vals, begin, cbeg, nseg, total, ck, cv);
  return cudaGetLastError();
}

cudaError_t copy_sorted_ranges(const uint64_t* ck, const uint32_t* cv, const uint64_t* cbeg,
                               const uint64_t* cend, const uint64_t* begin, uint32_t nseg,
                               const uint32_t* counts, const SortTasks& tasks, uint64_t* keys,
                               uint32_t* vals, int num_sms, cudaStream_t s) {
  if (nseg == 0) return cudaSuccess;
  count_launch();
  copy_sorted_kernel<<<8u * num_sms, 256, 0, s>>>(ck, cv, cbeg, cend, begin, nseg, counts, tasks.f,
                                                  tasks.n, tasks.cap, tasks.pair_reserve, keys,
                                                  vals);
  return cudaGetLastError();
}

uint32_t segsort_pair_reserve(uint64_t nelems) {
  return static_cast<uint32_t>(nelems / kHeapPackCap + 1);
}

size_t segsort_round_bytes(uint64_t nelems) { return (nelems / kCap + 1) * sizeof(RoundItem); }

size_t segsort_task_words(uint64_t nelems, uint32_t nseg) {
  // final tasks of the global phase are disjoint and come from partitions of
  // tasks larger than kCap (at most depth_limit levels of them); heap tasks
  // beyond kHeapPackCap get a reserve of their own at the top
  return nseg + 2 * (nelems / kCap + 1) * 64 + segsort_pair_reserve(nelems);
}

cudaError_t segmented_std_sort(uint64_t* keys, uint32_t* vals, uint32_t* lscratch,
                               uint32_t* rscratch, const uint64_t* begin, const uint64_t* end,
                               uint32_t nseg, const uint32_t* nseg_dev, uint32_t* lists,
                               uint32_t* counts, int num_sms, cudaStream_t stream,
                               SortTasks tasks) {
  // The shared-memory limits are attributes of the current device: set them
  // on every call (cheap), so a later call on another device, or from
  // another host thread, finds them set too.
  {
    cudaError_t e = cudaFuncSetAttribute(sort_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sizeof(CtaSmem)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(sort_tasks, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(sizeof(CtaSmem)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(sort_warp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(sizeof(WarpSlice) * kWarpSegWarps));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(sort_heaps, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(kHeapSmem));
    if (e != cudaSuccess) return e;
  }
  if (nseg == 0) return cudaSuccess;
  const bool split = tasks.side && tasks.side2 && tasks.fork && tasks.rounds_done && tasks.join &&
                     tasks.join2;
  cudaStream_t side = split ? tasks.side : stream;
  cudaStream_t side2 = split ? tasks.side2 : stream;
  cudaMemsetAsync(counts, 0, 10 * sizeof(uint32_t), stream);
  count_launch();
  classify_segments<<<(nseg + 255) / 256, 256, 0, stream>>>(begin, end, nseg, nseg_dev, lists,
                                                            counts);
  if (split) {
    cudaError_t e = cudaEventRecord(tasks.fork, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side, tasks.fork, 0);
    if (e != cudaSuccess) return e;
  }
  count_launch();
  sort_tiny<<<num_sms * 4, 128, 0, side>>>(keys, vals, begin, end, lists, counts);
  count_launch();
  sort_warp<<<num_sms, kWarpSegWarps * 32, sizeof(WarpSlice) * kWarpSegWarps, side>>>(
      keys, vals, begin, end, lists + nseg, counts);
  count_launch();
  sort_cta<<<num_sms * 3, kBlock, sizeof(CtaSmem), side>>>(keys, vals, begin, end,
                                                       lists + 2 * static_cast<size_t>(nseg),
                                                       counts);
  if (tasks.nelems > kCap) {
    // global phase in rounds; the host looks at the next round's list after
    // rounds 0, 1, 3, 7, ... and stops when it is empty (every range's budget
    // runs out by round 62)
    RoundItem* rl[2] = {static_cast<RoundItem*>(tasks.round[0]),
                        static_cast<RoundItem*>(tasks.round[1])};
    uint32_t* rcount = tasks.round_counts;                  // list size of round r
    uint32_t* rwork = tasks.round_counts + kSortRounds + 1;  // claims of round r
    cudaMemsetAsync(tasks.round_counts, 0, 2 * (kSortRounds + 1) * sizeof(uint32_t), stream);
    count_launch();
    round_seed<<<std::min((nseg + 255) / 256, 1024u), 256, 0, stream>>>(
        begin, end, lists + 3 * static_cast<size_t>(nseg), counts, rl[0]);
    // blocks claim ranges from a counter: the grid (round_per_sm blocks per
    // SM, 1-2) changes no result
    const int round_blocks =
        tasks.round_per_sm > 0 ? std::min(tasks.round_per_sm, kBigPerSm) : kBigPerSm;
    for (int r = 0; r < kSortRounds; ++r) {
      count_launch();
      sort_round<<<num_sms * round_blocks, kBigBlock, 0, stream>>>(
          keys, vals, lscratch, rscratch, rl[r & 1], r == 0 ? counts + 3 : rcount + r, rwork + r,
          rl[(r + 1) & 1], rcount + r + 1, tasks.f, tasks.n, tasks.d, counts + 4, counts + 5,
          counts + 7, tasks.cap, tasks.pair_reserve, PruneLists{tasks.prune_keys, tasks.prune_off});
      if (((r + 1) & r) == 0) {
        uint32_t next = 0;
        cudaError_t e = cudaMemcpyAsync(&next, rcount + r + 1, sizeof(next),
                                        cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return e;
        if (next == 0) break;
      }
    }
  }
  if (split) {
    cudaError_t e = cudaEventRecord(tasks.rounds_done, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side2, tasks.rounds_done, 0);
    if (e != cudaSuccess) return e;
  }
  // the heap ranges first: their serial pops are the longest chains
  count_launch();
  sort_heaps<<<(num_sms + 1) / 2 * 2, kHeapBlock, kHeapSmem, side2>>>(
      keys, vals, lscratch, rscratch, tasks.f, tasks.n, counts + 5, counts + 6, counts + 7,
      counts + 8, tasks.cap, tasks.pair_reserve);
  count_launch();
  sort_tasks<<<num_sms * 3, kBlock, sizeof(CtaSmem), stream>>>(keys, vals, tasks.f, tasks.n, tasks.d,
                                                           counts + 4, counts + 9);
  if (split) {
    cudaError_t e = cudaEventRecord(tasks.join, side);
    if (e == cudaSuccess) e = cudaEventRecord(tasks.join2, side2);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, tasks.join, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, tasks.join2, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace cuflye
