// util.cu — exclusive prefix sums and 2-bit packing.
#include <atomic>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launches_total() { return g_launches.load(std::memory_order_relaxed); }

namespace {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr uint64_t kScanTile = kScanBlock * kScanItems;

template <typename In>
__global__ void scan_tile_sums(const In* __restrict__ in, uint64_t n, uint64_t* __restrict__ sums) {
  __shared__ uint64_t ws[kScanBlock / 32];
  const uint64_t t0 = static_cast<uint64_t>(blockIdx.x) * kScanTile;
  uint64_t s = 0;
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = t0 + static_cast<uint64_t>(j) * kScanBlock + threadIdx.x;
    if (i < n) s += static_cast<uint64_t>(in[i]);
  }
  for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t = 0;
    for (int w = 0; w < kScanBlock / 32; ++w) t += ws[w];
    sums[blockIdx.x] = t;
  }
}

// Single-block exclusive scan of the tile sums (sums[ntiles] = grand total).
__global__ void scan_sums(uint64_t* sums, uint64_t ntiles) {
  __shared__ uint64_t ws[32];
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x / 32;
  for (uint64_t base = 0; base < ntiles; base += blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const uint64_t v = i < ntiles ? sums[i] : 0;
    uint64_t inc = v;
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t o = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += o;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      const uint64_t w = lane < nw ? ws[lane] : 0;
      uint64_t wi = w;
      for (int d = 1; d < 32; d <<= 1) {
        const uint64_t o = __shfl_up_sync(0xffffffffu, wi, d);
        if (lane >= d) wi += o;
      }
      if (lane < nw) ws[lane] = wi - w;
    }
    __syncthreads();
    const uint64_t ex = carry + ws[warp] + inc - v;
    if (i < ntiles) sums[i] = ex;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = ex + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[ntiles] = carry;
}

template <typename In>
__global__ void scan_downsweep(const In* __restrict__ in, uint64_t* __restrict__ out, uint64_t n,
                               const uint64_t* __restrict__ sums) {
  __shared__ uint64_t ws[kScanBlock / 32 + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t t0 = static_cast<uint64_t>(blockIdx.x) * kScanTile;
  // each thread owns kScanItems consecutive elements
  const uint64_t a = t0 + static_cast<uint64_t>(threadIdx.x) * kScanItems;
  uint64_t v[kScanItems];
  uint64_t s = 0;
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = a + j;
    v[j] = i < n ? static_cast<uint64_t>(in[i]) : 0;
    s += v[j];
  }
  uint64_t inc = s;
  for (int d = 1; d < 32; d <<= 1) {
    const uint64_t o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t c = 0;
    for (int w = 0; w < kScanBlock / 32; ++w) {
      const uint64_t t = ws[w];
      ws[w] = c;
      c += t;
    }
  }
  __syncthreads();
  uint64_t run = sums[blockIdx.x] + ws[warp] + inc - s;
  for (int j = 0; j < kScanItems; ++j) {
    const uint64_t i = a + j;
    if (i < n) out[i] = run;
    run += v[j];
  }
}

__global__ void pack_kernel(const uint8_t* __restrict__ ascii, uint64_t nbases,
                            uint64_t* __restrict__ words, uint64_t nwords) {
  const uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  const uint64_t b0 = w * 32;
  uint64_t x = 0;
  if (b0 + 32 <= nbases) {
    const uint4* p = reinterpret_cast<const uint4*>(ascii + b0);
    uint4 c[2];
    if ((reinterpret_cast<uintptr_t>(ascii + b0) & 15u) == 0) {
      c[0] = p[0];
      c[1] = p[1];
    } else {
      uint8_t* cb = reinterpret_cast<uint8_t*>(c);
      for (int i = 0; i < 32; ++i) cb[i] = ascii[b0 + i];
    }
    const uint8_t* cb = reinterpret_cast<const uint8_t*>(c);
#pragma unroll
    for (int i = 0; i < 32; ++i) x = (x << 2) | base_code(cb[i]);
  } else {
    for (int i = 0; i < 32; ++i) {
      const uint64_t b = b0 + i;
      x = (x << 2) | (b < nbases ? base_code(ascii[b]) : 0u);
    }
  }
  words[w] = x;
}

}  // namespace

size_t scan_temp_words(uint64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

template <typename In>
static cudaError_t run_scan(const In* in, uint64_t* out, uint64_t n, uint64_t* temp,
                            cudaStream_t s) {
  if (n == 0) {
    cudaMemsetAsync(temp, 0, sizeof(uint64_t), s);
    return cudaGetLastError();
  }
  const uint64_t ntiles = (n + kScanTile - 1) / kScanTile;
  count_launch();
  scan_tile_sums<In><<<static_cast<unsigned>(ntiles), kScanBlock, 0, s>>>(in, n, temp);
  count_launch();
  scan_sums<<<1, 1024, 0, s>>>(temp, ntiles);
  count_launch();
  scan_downsweep<In><<<static_cast<unsigned>(ntiles), kScanBlock, 0, s>>>(in, out, n, temp);
  return cudaGetLastError();
}

cudaError_t exclusive_scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n,
                                      uint64_t* temp, cudaStream_t s) {
  return run_scan<uint32_t>(in, out, n, temp, s);
}

cudaError_t exclusive_scan_u64(const uint64_t* in, uint64_t* out, uint64_t n, uint64_t* temp,
                               cudaStream_t s) {
  return run_scan<uint64_t>(in, out, n, temp, s);
}

cudaError_t pack_bases(const uint8_t* ascii, uint64_t nbases, uint64_t* words, cudaStream_t s) {
  const uint64_t nwords = (nbases + 31) / 32 + 1;
  count_launch();
  pack_kernel<<<static_cast<unsigned>((nwords + 255) / 256), 256, 0, s>>>(ascii, nbases, words,
                                                                         nwords);
  return cudaGetLastError();
}

}  // namespace cuflye
