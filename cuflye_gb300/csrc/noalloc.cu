// noalloc.cu — the allocation-free variant of the libstdc++-order segmented
// sort (cuflye_std_sort_segments_noalloc).
//
// Some callers cannot allocate device memory at all: a host process whose
// device memory is owned end to end by another allocator (a serving runtime
// that reserves the whole GPU for its own pool and forbids any other
// cudaMalloc), or a worker that must keep a fixed, pre-declared footprint.
// This entry point lets them use the sort with the buffers they already own:
// keys and values are the caller's device memory, segment offsets come from
// the host, and every scratch byte the sort needs (its rank maps, segment
// lists, counters and task list) lives in one file-scope device array of
// fixed size, g_noalloc_scratch, which every GPU that loads the library holds
// until the process exits.  The call itself makes no cudaMalloc, cudaFree or
// other allocating call.
//
// Host code cannot use g_noalloc_scratch's name as a device address; the
// first call on each device, with that device current, asks the runtime for
// the array's device address (cudaGetSymbolAddress) and caches it.  The
// cache assumes the device's primary context lives as long as the process:
// after a cudaDeviceReset the cached address is stale and the call must not
// be used again in that process.  A call over more than 4,096 elements
// reads its round counts back between sort rounds and so waits on `stream`
// before it returns; smaller calls return once the work is queued.  Calls
// share the array and it keeps the previous call's contents: the counters
// that must start at zero are cleared by every call, and calls whose work
// overlaps on the GPU (different streams, or different host threads on one
// device) race on the scratch and must not be issued.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/cuflye.h"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

constexpr size_t kMaxElems = CUFLYE_NOALLOC_MAX_ELEMENTS;
constexpr size_t kMaxSegs = CUFLYE_NOALLOC_MAX_SEGMENTS;
constexpr size_t kTaskCap = size_t(1) << 18;  // task-list entries reserved

constexpr size_t kOffL = 0;
constexpr size_t kOffR = align256(kOffL + 4 * (kMaxElems + 1));
constexpr size_t kOffLists = align256(kOffR + 4 * (kMaxElems + 1));
constexpr size_t kOffCounts = align256(kOffLists + 4 * 4 * kMaxSegs);
constexpr size_t kOffSegs = align256(kOffCounts + 4 * 16);
constexpr size_t kOffTf = align256(kOffSegs + 8 * (kMaxSegs + 1));
constexpr size_t kOffTn = align256(kOffTf + 8 * kTaskCap);
constexpr size_t kOffTd = align256(kOffTn + 4 * kTaskCap);
constexpr size_t kRoundBytes = (kMaxElems / 4096 + 1) * kRoundItemBytes;  // segsort_round_bytes(kMaxElems)
constexpr size_t kOffR0 = align256(kOffTd + 4 * kTaskCap);
constexpr size_t kOffR1 = align256(kOffR0 + kRoundBytes);
constexpr size_t kOffRc = align256(kOffR1 + kRoundBytes);
constexpr size_t kScratchBytes = align256(kOffRc + 4 * 2 * (kSortRounds + 1));

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

}  // namespace

// Fixed scratch of the allocation-free sort (about 13.6 MiB per device).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// Device address of g_noalloc_scratch on the current device (set up once per
// device, under a lock, with that device current).
cuflye_status scratch_address(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return CUFLYE_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return CUFLYE_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return CUFLYE_ERR_CUDA;
    }
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_addr[dev];
  return CUFLYE_OK;
}

}  // namespace
}  // namespace cuflye

extern "C" cuflye_status cuflye_std_sort_segments_noalloc(uint64_t* keys, uint32_t* values,
                                                          const uint64_t* seg_offsets,
                                                          size_t n_segments, size_t n_elements,
                                                          void* stream) {
  using namespace cuflye;
  if (!seg_offsets) return CUFLYE_ERR_INVALID;
  if (n_elements > kMaxElems || n_segments > kMaxSegs) return CUFLYE_ERR_UNSUPPORTED;
  if (n_segments == 0) return CUFLYE_OK;
  if (n_elements && (!keys || !values)) return CUFLYE_ERR_INVALID;
  for (size_t s = 0; s < n_segments; ++s)
    if (seg_offsets[s + 1] < seg_offsets[s]) return CUFLYE_ERR_INVALID;
  if (seg_offsets[n_segments] > n_elements) return CUFLYE_ERR_INVALID;
  if (segsort_task_words(n_elements, static_cast<uint32_t>(n_segments)) > kTaskCap)
    return CUFLYE_ERR_UNSUPPORTED;
  if (segsort_round_bytes(n_elements) > kRoundBytes) return CUFLYE_ERR_UNSUPPORTED;
  // every size check is above this line: a refused request queues nothing
  unsigned char* base = nullptr;
  const cuflye_status st = scratch_address(&base);
  if (st != CUFLYE_OK) return st;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return CUFLYE_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint64_t* segs = reinterpret_cast<uint64_t*>(base + kOffSegs);
  // the offsets travel with the work, in stream order
  if (cudaMemcpyAsync(segs, seg_offsets, (n_segments + 1) * sizeof(uint64_t),
                      cudaMemcpyHostToDevice, s) != cudaSuccess) {
    cudaGetLastError();
    return CUFLYE_ERR_CUDA;
  }
  SortTasks tasks{reinterpret_cast<uint64_t*>(base + kOffTf),
                  reinterpret_cast<uint32_t*>(base + kOffTn), reinterpret_cast<int*>(base + kOffTd),
                  static_cast<uint32_t>(kTaskCap), segsort_pair_reserve(n_elements),
                  n_elements, {base + kOffR0, base + kOffR1},
                  reinterpret_cast<uint32_t*>(base + kOffRc)};
  // segmented_std_sort clears its counters (the task count included) itself
  const cudaError_t e = segmented_std_sort(
      keys, values, reinterpret_cast<uint32_t*>(base + kOffL),
      reinterpret_cast<uint32_t*>(base + kOffR), segs, segs + 1,
      static_cast<uint32_t>(n_segments), nullptr, reinterpret_cast<uint32_t*>(base + kOffLists),
      reinterpret_cast<uint32_t*>(base + kOffCounts), sms, s, tasks);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return CUFLYE_ERR_CUDA;
  }
  return CUFLYE_OK;
}
