// sort.cu — segmented libstdc++-order sort and stable LSD radix sort.
//
// segmented_std_sort(): every segment [begin[s], end[s]) of (key, value)
// pairs is put in exactly the order libstdc++'s std::sort with `key < key`
// gives (introsort.cuh explains the parallel formulation).  Segments are
// classified by size:
//   * <= kSerialMax elements: one thread runs the serial algorithm;
//   * <= kSmemCap: one CTA loads the segment into shared memory, partitions
//     block-wide while tasks are large and finishes small tasks per thread;
//   * larger: one CTA partitions in global memory (prefix counts tiled over
//     the task) until tasks fit in shared memory.
//
// radix_sort_pairs(): stable least-significant-digit radix sort of
// (u64 key, u64 value) on a digit range, 8 bits per pass; used to build the
// k-mer index with entries in (key, stored id, stored position) order.
#include <cstdint>
#include <cstdio>

#include "common.cuh"
#include "introsort.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr int kBlock = 512;
constexpr uint32_t kSmemCap = 8192;
constexpr uint32_t kSerialMax = 128;
constexpr int kMaxTasks = 96;
constexpr int kMaxSerial = 256;

struct SortSmem {
  uint64_t K[kSmemCap];
  uint32_t V[kSmemCap];
  uint32_t L[kSmemCap + 1];
  uint32_t R[kSmemCap + 1];
  uint32_t tf[kMaxTasks], tl[kMaxTasks];
  int td[kMaxTasks];
  uint32_t sf[kMaxSerial], sl[kMaxSerial];
  int sd[kMaxSerial];
  uint64_t warp_sums[kBlock / 32 + 1];
  int ntask, nserial;
  uint32_t scalar[4];
};

// Exclusive block scan of a packed pair of 32-bit counters; returns the
// exclusive prefix and the block total (to every thread).
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t* warp_sums,
                                                         uint64_t* total) {
  constexpr int kWarps = kBlock / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t inc = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint64_t o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint64_t w = lane < kWarps ? warp_sums[lane] : 0;
    uint64_t wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t o = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += o;
    }
    if (lane < kWarps) warp_sums[lane] = wi - w;
    if (lane == kWarps - 1) warp_sums[kWarps] = wi;
  }
  __syncthreads();
  const uint64_t r = warp_sums[warp] + inc - v;
  *total = warp_sums[kWarps];
  __syncthreads();
  return r;
}

// Largest m in [0, hi] with L[m] < R[m] (L[0] = 0 < R[0] = inf by convention).
__device__ __forceinline__ uint32_t find_swaps(const uint32_t* L, const uint32_t* R,
                                               uint32_t hi) {
  uint32_t lo = 0;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (L[mid] < R[mid])
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Block-wide unguarded partition of [f, l) (shared or global arrays; L and R
// are 1-based rank -> position maps with room for l - f + 1 entries).
__device__ uint32_t block_partition(uint64_t* K, uint32_t* V, uint32_t* L, uint32_t* R,
                                    uint32_t f, uint32_t l, SortSmem& sm) {
  if (threadIdx.x == 0) isort::median_to_first(K, V, f, f + 1, f + (l - f) / 2, l - 1);
  __syncthreads();
  const uint64_t p = K[f];
  const uint32_t n = l - f;
  const uint32_t tile = kBlock * 16u;
  // pass 1: totals
  {
    uint32_t cl = 0, cr = 0;
    for (uint32_t i = f + threadIdx.x; i < l; i += kBlock) {
      const uint64_t k = K[i];
      cl += (i > f) && !(k < p);
      cr += !(p < k);
    }
    uint64_t tot;
    block_exclusive_scan((static_cast<uint64_t>(cl) << 32) | cr, sm.warp_sums, &tot);
    if (threadIdx.x == 0) {
      sm.scalar[0] = static_cast<uint32_t>(tot >> 32);
      sm.scalar[1] = static_cast<uint32_t>(tot & 0xffffffffu);
    }
    __syncthreads();
  }
  const uint32_t TL = sm.scalar[0], TR = sm.scalar[1];
  // pass 2: ranks, tile by tile, each thread owning 16 consecutive items
  uint64_t carry = 0;
  for (uint32_t t0 = f; t0 < l; t0 += tile) {
    const uint32_t a = t0 + threadIdx.x * 16u;
    uint32_t cl = 0, cr = 0;
    for (uint32_t i = a; i < a + 16u && i < l; ++i) {
      const uint64_t k = K[i];
      cl += (i > f) && !(k < p);
      cr += !(p < k);
    }
    uint64_t tile_tot;
    const uint64_t ex = block_exclusive_scan((static_cast<uint64_t>(cl) << 32) | cr,
                                             sm.warp_sums, &tile_tot);
    if (threadIdx.x == 0) {
      sm.scalar[2] = static_cast<uint32_t>(tile_tot >> 32);
      sm.scalar[3] = static_cast<uint32_t>(tile_tot & 0xffffffffu);
    }
    uint32_t rl = static_cast<uint32_t>((carry + ex) >> 32);
    uint32_t rr = static_cast<uint32_t>((carry + ex) & 0xffffffffu);
    for (uint32_t i = a; i < a + 16u && i < l; ++i) {
      const uint64_t k = K[i];
      if ((i > f) && !(k < p)) L[++rl] = i;
      if (!(p < k)) {
        R[TR - rr] = i;
        ++rr;
      }
    }
    __syncthreads();
    carry += (static_cast<uint64_t>(sm.scalar[2]) << 32) | sm.scalar[3];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const uint32_t hi = TL < TR ? TL : TR;
    const uint32_t m = find_swaps(L, R, hi);
    uint32_t cut;
    if (m == 0) {
      cut = L[1];
    } else {
      cut = R[m];
      if (m + 1 <= TL && L[m + 1] < cut) cut = L[m + 1];
    }
    sm.scalar[0] = m;
    sm.scalar[1] = cut;
  }
  __syncthreads();
  const uint32_t m = sm.scalar[0], cut = sm.scalar[1];
  for (uint32_t k = 1 + threadIdx.x; k <= m; k += kBlock) isort::swap_kv(K, V, L[k], R[k]);
  __syncthreads();
  (void)n;
  return cut;
}

// Sorts [0, n) held in shared memory starting at recursion budget depth0.
__device__ void smem_sort(SortSmem& sm, uint32_t n, int depth0) {
  if (threadIdx.x == 0) {
    sm.ntask = 0;
    sm.nserial = 0;
    sm.tf[0] = 0;
    sm.tl[0] = n;
    sm.td[0] = depth0;
    sm.ntask = 1;
  }
  __syncthreads();
  for (;;) {
    const int nt = sm.ntask;
    if (nt == 0) break;
    const uint32_t f = sm.tf[nt - 1], l = sm.tl[nt - 1];
    const int d = sm.td[nt - 1];
    __syncthreads();
    if (l - f <= kSerialMax || d == 0) {
      if (threadIdx.x == 0) {
        sm.ntask = nt - 1;
        sm.sf[sm.nserial] = f;
        sm.sl[sm.nserial] = l;
        sm.sd[sm.nserial] = d;
        ++sm.nserial;
      }
      __syncthreads();
      if (sm.nserial == kMaxSerial) {
        // the ranges are disjoint, so finishing them early changes nothing
        for (int s = threadIdx.x; s < kMaxSerial; s += kBlock)
          isort::serial_introsort(sm.K, sm.V, sm.sf[s], sm.sl[s], sm.sd[s]);
        __syncthreads();
        if (threadIdx.x == 0) sm.nserial = 0;
        __syncthreads();
      }
      continue;
    }
    const uint32_t cut = block_partition(sm.K, sm.V, sm.L, sm.R, f, l, sm);
    if (threadIdx.x == 0) {
      sm.tf[nt - 1] = cut;
      sm.tl[nt - 1] = l;
      sm.td[nt - 1] = d - 1;
      sm.tf[nt] = f;
      sm.tl[nt] = cut;
      sm.td[nt] = d - 1;
      sm.ntask = nt + 1;
    }
    __syncthreads();
  }
  for (int s = threadIdx.x; s < sm.nserial; s += kBlock)
    isort::serial_introsort(sm.K, sm.V, sm.sf[s], sm.sl[s], sm.sd[s]);
  __syncthreads();
}

__device__ void load_sort_store(uint64_t* K, uint32_t* V, uint64_t begin, uint32_t n, int depth,
                                SortSmem& sm) {
  for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
    sm.K[i] = K[begin + i];
    sm.V[i] = V[begin + i];
  }
  __syncthreads();
  smem_sort(sm, n, depth);
  for (uint32_t i = threadIdx.x; i < n; i += kBlock) {
    K[begin + i] = sm.K[i];
    V[begin + i] = sm.V[i];
  }
  __syncthreads();
}

__global__ void classify_segments(const uint64_t* __restrict__ begin,
                                  const uint64_t* __restrict__ end, uint32_t nseg,
                                  const uint32_t* __restrict__ nseg_dev, uint32_t* tiny,
                                  uint32_t* mid, uint32_t* big, uint32_t* counts) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || (nseg_dev && s >= *nseg_dev)) return;
  const uint64_t n = end[s] - begin[s];
  if (n <= 1) return;
  if (n <= kSerialMax) {
    tiny[atomicAdd(&counts[0], 1u)] = s;
  } else if (n <= kSmemCap) {
    mid[atomicAdd(&counts[1], 1u)] = s;
  } else {
    big[atomicAdd(&counts[2], 1u)] = s;
  }
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

__global__ void __launch_bounds__(kBlock) sort_mid(uint64_t* K, uint32_t* V,
                                                   const uint64_t* __restrict__ begin,
                                                   const uint64_t* __restrict__ end,
                                                   const uint32_t* __restrict__ list,
                                                   const uint32_t* __restrict__ counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmem& sm = *reinterpret_cast<SortSmem*>(smem_raw);
  const uint32_t cnt = counts[1];
  for (uint32_t i = blockIdx.x; i < cnt; i += gridDim.x) {
    const uint32_t s = list[i];
    const uint64_t b = begin[s];
    const uint32_t n = static_cast<uint32_t>(end[s] - b);
    load_sort_store(K, V, b, n, isort::depth_limit(n), sm);
  }
}

__global__ void __launch_bounds__(kBlock) sort_big(uint64_t* K, uint32_t* V, uint32_t* Lg,
                                                   uint32_t* Rg,
                                                   const uint64_t* __restrict__ begin,
                                                   const uint64_t* __restrict__ end,
                                                   const uint32_t* __restrict__ list,
                                                   const uint32_t* __restrict__ counts) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SortSmem& sm = *reinterpret_cast<SortSmem*>(smem_raw);
  __shared__ uint32_t gf[kMaxTasks], gl[kMaxTasks];
  __shared__ int gd[kMaxTasks];
  __shared__ int gn;
  const uint32_t cnt = counts[2];
  for (uint32_t i = blockIdx.x; i < cnt; i += gridDim.x) {
    const uint32_t s = list[i];
    const uint64_t b = begin[s];
    const uint32_t n = static_cast<uint32_t>(end[s] - b);
    uint64_t* Ks = K + b;
    uint32_t* Vs = V + b;
    // rank maps share the segment's index range in the scratch arrays
    uint32_t* Ls = Lg + b;
    uint32_t* Rs = Rg + b;
    if (threadIdx.x == 0) {
      gf[0] = 0;
      gl[0] = n;
      gd[0] = isort::depth_limit(n);
      gn = 1;
    }
    __syncthreads();
    for (;;) {
      const int nt = gn;
      if (nt == 0) break;
      const uint32_t f = gf[nt - 1], l = gl[nt - 1];
      const int d = gd[nt - 1];
      __syncthreads();
      if (l - f <= kSmemCap) {
        if (threadIdx.x == 0) gn = nt - 1;
        __syncthreads();
        if (l - f > 1) load_sort_store(Ks, Vs, f, l - f, d, sm);
        continue;
      }
      if (d == 0) {
        if (threadIdx.x == 0) {
          isort::heap_sort(Ks, Vs, f, l);
          gn = nt - 1;
        }
        __syncthreads();
        continue;
      }
      // rank maps are indexed from the task start
      // rank k of this task lives at index f - 1 + k, inside [f, l)
      const int64_t rb = static_cast<int64_t>(f) - 1;
      const uint32_t cut = block_partition(Ks, Vs, Ls + rb, Rs + rb, f, l, sm);
      if (threadIdx.x == 0) {
        gf[nt - 1] = cut;
        gl[nt - 1] = l;
        gd[nt - 1] = d - 1;
        gf[nt] = f;
        gl[nt] = cut;
        gd[nt] = d - 1;
        gn = nt + 1;
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------- radix sort

constexpr int kRadixBlock = 256;
constexpr int kRadixItems = 16;  // items per thread per tile
constexpr uint32_t kRadixTile = kRadixBlock * kRadixItems;

__device__ __forceinline__ uint32_t digit_of(uint64_t key, uint64_t val, int d) {
  // digits 0..7: value bytes (least significant first); 8..15: key bytes
  return d < 8 ? static_cast<uint32_t>((val >> (8 * d)) & 0xffu)
               : static_cast<uint32_t>((key >> (8 * (d - 8))) & 0xffu);
}

__global__ void radix_histogram(const uint64_t* __restrict__ keys,
                                const uint64_t* __restrict__ vals, uint64_t n, int d,
                                uint32_t* __restrict__ hist, uint32_t ntiles) {
  __shared__ uint32_t h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const uint64_t t0 = static_cast<uint64_t>(blockIdx.x) * kRadixTile;
  for (uint32_t j = threadIdx.x; j < kRadixTile; j += blockDim.x) {
    const uint64_t i = t0 + j;
    if (i < n) atomicAdd(&h[digit_of(keys[i], vals[i], d)], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b * ntiles + blockIdx.x] = h[b];
}

// Exclusive scan over the digit-major histogram (256 * ntiles counters) by
// one block; counts fit 32 bits because a pass covers < 2^32 elements.
__global__ void radix_scan(uint32_t* hist, uint32_t total) {
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < total; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < total ? hist[i] : 0;
    uint32_t inc = v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int dd = 1; dd < 32; dd <<= 1) {
      const uint32_t o = __shfl_up_sync(0xffffffffu, inc, dd);
      if (lane >= dd) inc += o;
    }
    __shared__ uint32_t ws[32];
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      const uint32_t nw = blockDim.x / 32;
      uint32_t w = lane < static_cast<int>(nw) ? ws[lane] : 0;
      uint32_t wi = w;
      for (int dd = 1; dd < 32; dd <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, wi, dd);
        if (lane >= dd) wi += o;
      }
      if (lane < static_cast<int>(nw)) ws[lane] = wi - w;
    }
    __syncthreads();
    const uint32_t ex = carry + ws[warp] + inc - v;
    if (i < total) hist[i] = ex;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = ex + v;
    __syncthreads();
  }
}

// Stable scatter: within a tile, elements keep their order per digit.  Each
// warp ranks its 32-element chunks with match_any, chunks are visited in
// order, and per-digit running offsets live in shared memory.
__global__ void radix_scatter(const uint64_t* __restrict__ keys_in,
                              const uint64_t* __restrict__ vals_in, uint64_t* __restrict__ keys_out,
                              uint64_t* __restrict__ vals_out, uint64_t n, int d,
                              const uint32_t* __restrict__ hist, uint32_t ntiles) {
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcount[kRadixBlock / 32][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nwarps = kRadixBlock / 32;
  for (int b = threadIdx.x; b < 256; b += blockDim.x) base[b] = hist[b * ntiles + blockIdx.x];
  const uint64_t t0 = static_cast<uint64_t>(blockIdx.x) * kRadixTile;
  // The tile is processed in rounds of nwarps*32 consecutive elements;
  // within a round warp w owns elements [w*32, w*32+32).
  for (uint32_t r0 = 0; r0 < kRadixTile; r0 += nwarps * 32) {
    for (int b = threadIdx.x; b < 256 * nwarps; b += blockDim.x)
      wcount[b / 256][b % 256] = 0;
    __syncthreads();
    const uint64_t i = t0 + r0 + warp * 32 + lane;
    const bool valid = i < n;
    uint64_t k = 0, v = 0;
    uint32_t dig = 0xffffffffu;
    if (valid) {
      k = keys_in[i];
      v = vals_in[i];
      dig = digit_of(k, v, d);
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, dig);
    const uint32_t rank_in_warp = __popc(peers & ((1u << lane) - 1u));
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) wcount[warp][dig] = __popc(peers);
    __syncthreads();
    // exclusive prefix over warps for this element's digit
    uint32_t before = 0;
    if (valid)
      for (int w = 0; w < warp; ++w) before += wcount[w][dig];
    if (valid) {
      const uint32_t dst = base[dig] + before + rank_in_warp;
      keys_out[dst] = k;
      vals_out[dst] = v;
    }
    __syncthreads();
    // advance per-digit bases by this round's totals
    for (int b = threadIdx.x; b < 256; b += blockDim.x) {
      uint32_t s = 0;
      for (int w = 0; w < nwarps; ++w) s += wcount[w][b];
      base[b] += s;
    }
    __syncthreads();
  }
}

}  // namespace

size_t segsort_smem_bytes() { return sizeof(SortSmem); }

cudaError_t segmented_std_sort(uint64_t* keys, uint32_t* vals, uint32_t* lscratch,
                               uint32_t* rscratch, const uint64_t* begin, const uint64_t* end,
                               uint32_t nseg, const uint32_t* nseg_dev, uint32_t* lists,
                               uint32_t* counts, int num_sms, cudaStream_t stream) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(sort_mid, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(SortSmem)));
    cudaFuncSetAttribute(sort_big, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(SortSmem)));
    attr = true;
  }
  if (nseg == 0) return cudaSuccess;
  cudaMemsetAsync(counts, 0, 3 * sizeof(uint32_t), stream);
  uint32_t* tiny = lists;
  uint32_t* mid = lists + nseg;
  uint32_t* big = lists + 2 * static_cast<size_t>(nseg);
  count_launch();
  classify_segments<<<(nseg + 255) / 256, 256, 0, stream>>>(begin, end, nseg, nseg_dev, tiny,
                                                            mid, big, counts);
  count_launch();
  sort_tiny<<<num_sms * 4, 128, 0, stream>>>(keys, vals, begin, end, tiny, counts);
  count_launch();
  sort_mid<<<num_sms, kBlock, sizeof(SortSmem), stream>>>(keys, vals, begin, end, mid, counts);
  count_launch();
  sort_big<<<num_sms, kBlock, sizeof(SortSmem), stream>>>(keys, vals, lscratch, rscratch, begin,
                                                          end, big, counts);
  return cudaGetLastError();
}

cudaError_t radix_sort_pairs(uint64_t* keys, uint64_t* vals, uint64_t* keys_alt,
                             uint64_t* vals_alt, uint64_t n, const int* digits, int ndigits,
                             uint32_t* hist, int* result_in_alt, cudaStream_t stream) {
  const uint32_t ntiles = static_cast<uint32_t>((n + kRadixTile - 1) / kRadixTile);
  uint64_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
  for (int p = 0; p < ndigits; ++p) {
    const int d = digits[p];
    count_launch();
    radix_histogram<<<ntiles, kRadixBlock, 0, stream>>>(ki, vi, n, d, hist, ntiles);
    count_launch();
    radix_scan<<<1, 1024, 0, stream>>>(hist, 256u * ntiles);
    count_launch();
    radix_scatter<<<ntiles, kRadixBlock, 0, stream>>>(ki, vi, ko, vo, n, d, hist, ntiles);
    uint64_t* t = ki;
    ki = ko;
    ko = t;
    t = vi;
    vi = vo;
    vo = t;
  }
  *result_in_alt = (ki == keys_alt);
  return cudaGetLastError();
}

size_t radix_hist_words(uint64_t n) {
  return 256 * ((n + kRadixTile - 1) / kRadixTile);
}

}  // namespace cuflye
