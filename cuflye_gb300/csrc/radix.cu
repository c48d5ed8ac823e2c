// radix.cu — stable least-significant-digit radix sort of (u64 key, u64 value)
// pairs, 8 bits per pass, over a chosen list of digits (value bytes 0-7 are
// digits 0-7, key bytes are digits 8-15).  Builds the k-mer index with its
// entries in (key, stored id, stored position) order.
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

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
