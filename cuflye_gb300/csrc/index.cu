// index.cu — device construction of the k-mer index (Flye VertexIndex equivalent).
//
// Definition (Flye's VertexIndex sources are not in the reference; the CPU
// oracle defines the same): every window of every target's forward strand
// is keyed by its standard form min(x, revcomp(x)); a window whose k-mer is
// not in standard form is stored on the reverse strand at
// (len - pos - k).  freq(key) is the number of windows.  Keys with
// freq > max_freq are repetitive; keys with min_freq <= freq <= max_freq are
// solid and keep their entries, in ascending (stored id, stored position)
// order.  Lookups serve isRepetitive / kmerFreq / iterKmerPos as called at
// patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:55-80.
//
// Construction: enumerate windows -> stable LSD radix sort of
// (key | stored id | stored position) -> run detection -> solid positions
// copied in run order -> open-addressing insert (linear probing, load <= 1/2,
// the table sized at twice its entries).
// When the windows do not fit the memory budget at once, the same steps run
// per contiguous key range (ranges cut from a histogram of key prefixes), in
// two passes: the first counts each prefix's solid positions and table
// entries, the second writes every range's positions at its prefix's offset
// in the final array and inserts its runs into the final table.  The
// position array is then the same as one range's.
// A standard form never equals ~0 (the all-T k-mer's standard form is the
// all-A k-mer, 0), so ~0 marks an empty slot.
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

__device__ __forceinline__ uint32_t find_segment(const uint64_t* __restrict__ off, uint32_t n,
                                                 uint64_t x) {
  // largest s with off[s] <= x, s in [0, n)
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

struct Windows {
  const uint64_t* __restrict__ words;
  const uint64_t* __restrict__ base_off;
  const uint64_t* __restrict__ win_off;
  const int32_t* __restrict__ slot_len;
  uint32_t nslots;
  uint64_t nwin;
  int k;

  // Window w's standard-form key and (stored id << 32) | stored position.
  __device__ __forceinline__ void entry(uint64_t w, uint64_t& key, uint64_t& val) const {
    const uint32_t t = find_segment(win_off, nslots, w);
    const uint64_t p = w - win_off[t];
    const uint64_t x = kmer_at(words, base_off[t] + p, k);
    const uint64_t rc = revcomp(x, k);
    if (rc < x) {
      key = rc;
      val = (static_cast<uint64_t>(2u * t + 1u) << 32) |
            static_cast<uint32_t>(slot_len[t] - static_cast<int32_t>(p) - k);
    } else {
      key = x;
      val = (static_cast<uint64_t>(2u * t) << 32) | static_cast<uint32_t>(p);
    }
  }
};

__global__ void enumerate_kernel(Windows win, uint64_t* __restrict__ keys,
                                 uint64_t* __restrict__ vals) {
  const uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= win.nwin) return;
  win.entry(w, keys[w], vals[w]);
}

// Windows per key prefix (key >> shift), counted in shared memory per block.
__global__ void __launch_bounds__(1024) prefix_hist_kernel(Windows win, int shift, int nbins,
                                                           unsigned long long* __restrict__ hist) {
  extern __shared__ uint32_t bins[];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) bins[i] = 0;
  __syncthreads();
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < win.nwin;
       w += stride) {
    uint64_t key, val;
    win.entry(w, key, val);
    atomicAdd(&bins[key >> shift], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (bins[i]) atomicAdd(&hist[i], static_cast<unsigned long long>(bins[i]));
}

// Appends (warp-aggregated) the windows whose key lies in [lo, hi).  The
// order of the appended entries does not matter: the radix sort that
// follows orders them by (key, stored id, stored position), which is
// distinct per window.
__device__ __forceinline__ uint64_t warp_append(bool take, unsigned long long* count) {
  const uint32_t m = __ballot_sync(0xffffffffu, take);
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (m) {
    const int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(count, static_cast<unsigned long long>(__popc(m)));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  return base + __popc(m & ((1u << lane) - 1u));
}

__global__ void enumerate_range_kernel(Windows win, uint64_t lo, uint64_t hi,
                                       uint64_t* __restrict__ keys, uint64_t* __restrict__ vals,
                                       unsigned long long* count, uint64_t cap) {
  // every warp is full (block 256, grid rounded up): lanes past the end take nothing
  const uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  uint64_t key = 0, val = 0;
  bool take = false;
  if (w < win.nwin) {
    win.entry(w, key, val);
    take = key >= lo && key < hi;
  }
  const uint64_t i = warp_append(take, count);
  if (take && i < cap) {
    keys[i] = key;
    vals[i] = val;
  }
}

__global__ void mark_runs_kernel(const uint64_t* __restrict__ keys, uint64_t n,
                                 uint32_t* __restrict__ flags) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void run_starts_kernel(const uint32_t* __restrict__ flags,
                                  const uint64_t* __restrict__ run_id, uint64_t n,
                                  uint64_t nruns, uint64_t* __restrict__ run_start) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && flags[i]) run_start[run_id[i]] = i;
  if (i == 0) run_start[nruns] = n;
}

// tally (optional): [0] += solid runs, [1] += repetitive runs.
__global__ void classify_runs_kernel(const uint64_t* __restrict__ run_start, uint64_t nruns,
                                     uint32_t min_freq, uint32_t max_freq,
                                     uint32_t* __restrict__ kept, uint8_t* __restrict__ cls,
                                     unsigned long long* tally) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  uint8_t c = 0;
  if (r < nruns) {
    const uint64_t freq = run_start[r + 1] - run_start[r];
    if (freq > max_freq)
      c = 2;
    else if (freq >= min_freq)
      c = 1;
    cls[r] = c;
    kept[r] = c == 1 ? static_cast<uint32_t>(freq) : 0u;
  }
  if (tally) {  // uniform over the launch: every lane of the warp is here
    const uint32_t solid = __popc(__ballot_sync(0xffffffffu, c == 1));
    const uint32_t rep = __popc(__ballot_sync(0xffffffffu, c == 2));
    if ((threadIdx.x & 31) == 0) {
      if (solid) atomicAdd(&tally[0], static_cast<unsigned long long>(solid));
      if (rep) atomicAdd(&tally[1], static_cast<unsigned long long>(rep));
    }
  }
}

__global__ void copy_positions_kernel(const uint64_t* __restrict__ vals,
                                      const uint64_t* __restrict__ flags_scan,
                                      const uint64_t* __restrict__ run_start,
                                      const uint8_t* __restrict__ cls,
                                      const uint64_t* __restrict__ kept_off, uint64_t n,
                                      uint64_t* __restrict__ pos, uint32_t* __restrict__ self_at,
                                      const uint64_t* __restrict__ win_off,
                                      const int32_t* __restrict__ slot_len, int k) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // flags_scan holds the exclusive scan of run-start flags: the run of
  // element i is the number of run starts at or before i, minus one.
  uint64_t r = flags_scan[i];
  if (r >= 1 && run_start[r] > i) r -= 1;
  while (run_start[r] > i) --r;
  if (cls[r] != 1) return;
  const uint64_t v = vals[i];
  pos[kept_off[r] + (i - run_start[r])] = v;
  if (self_at) {
    // the window this entry came from: its forward position in its target
    const uint32_t sid = static_cast<uint32_t>(v >> 32);
    const uint32_t slot = sid >> 1;
    const int64_t sp = static_cast<int64_t>(v & 0xffffffffu);
    const int64_t p = (sid & 1u) ? static_cast<int64_t>(slot_len[slot]) - sp - k : sp;
    const uint64_t w = win_off[slot] + static_cast<uint64_t>(p);
    if (p >= 0 && w < win_off[slot + 1]) self_at[w] = static_cast<uint32_t>(i - run_start[r]);
  }
}

__device__ bool table_insert(TableEntry* table, uint64_t cap, uint64_t key, uint64_t meta,
                             bool merge_rep) {
  uint64_t slot = table_slot(key, cap);
  for (uint64_t step = 0; step < cap; ++step) {
    unsigned long long* kp = reinterpret_cast<unsigned long long*>(&table[slot].key);
    const unsigned long long prev = atomicCAS(kp, kEmptyKey, key);
    if (prev == kEmptyKey) {
      table[slot].meta = meta;
      return true;
    }
    if (prev == key) {
      if (merge_rep)
        atomicOr(reinterpret_cast<unsigned long long*>(&table[slot].meta), kRepetitiveBit);
      return true;
    }
    slot = table_next(slot, cap);
  }
  return false;
}

// Table word of run r (class 1 solid or 2 repetitive) whose positions start
// at pos_off in the position array.  vals: the run's entries, (stored id <<
// 32) | stored position.  With sorted_ids the entries of a run are in (id,
// position) order and a repeated id shows as two neighbours; otherwise
// (explicit entries in input order) every run of two or more entries is
// marked.
__device__ __forceinline__ uint64_t run_meta(const uint64_t* __restrict__ vals, uint64_t r0,
                                             uint64_t freq, uint8_t cls, uint64_t pos_off,
                                             bool sorted_ids) {
  if (cls == 2) {
    const uint64_t c = freq < ((1ULL << kCountBits) - 1) ? freq : ((1ULL << kCountBits) - 1);
    return kRepetitiveBit | (c << 40);
  }
  uint64_t meta = (pos_off & kOffsetMask) | (freq << 40);
  bool dup = !sorted_ids && freq > 1;
  for (uint64_t e = 1; sorted_ids && e < freq && !dup; ++e)
    dup = (vals[r0 + e] >> 32) == (vals[r0 + e - 1] >> 32);
  if (dup) meta |= kDupIdsBit;
  return meta;
}

__global__ void insert_kernel(const uint64_t* __restrict__ keys,
                              const uint64_t* __restrict__ vals,
                              const uint64_t* __restrict__ run_start,
                              const uint8_t* __restrict__ cls,
                              const uint64_t* __restrict__ kept_off, uint64_t nruns,
                              uint64_t pos_base, bool sorted_ids, TableEntry* table,
                              uint64_t cap, DeviceStatus* st) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= nruns || cls[r] == 0) return;
  const uint64_t r0 = run_start[r];
  const uint64_t meta =
      run_meta(vals, r0, run_start[r + 1] - r0, cls[r], pos_base + kept_off[r], sorted_ids);
  if (!table_insert(table, cap, keys[r0], meta, false)) raise_status(st, kDevTableFull, 0, r);
}

// Per key prefix (key >> shift): solid positions and table entries (solid
// and repetitive runs).  Runs arrive in key order, so a warp's runs share
// few prefixes: each distinct prefix of the warp takes one atomic per count.
__global__ void bin_totals_kernel(const uint64_t* __restrict__ keys,
                                  const uint64_t* __restrict__ run_start,
                                  const uint8_t* __restrict__ cls, uint64_t nruns, int shift,
                                  unsigned long long* __restrict__ npos_bin,
                                  unsigned long long* __restrict__ nent_bin) {
  // every warp is full (block 256, grid rounded up): lanes past the end count nothing
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  bool live = false;
  uint64_t bin = 0;
  uint32_t npos = 0;
  if (r < nruns && cls[r] != 0) {
    const uint64_t r0 = run_start[r];
    live = true;
    bin = keys[r0] >> shift;
    npos = cls[r] == 1 ? static_cast<uint32_t>(run_start[r + 1] - r0) : 0u;  // < 2^22
  }
  uint32_t left = __ballot_sync(0xffffffffu, live);
  while (left) {  // at most 32 rounds: each removes the leader's prefix
    const int leader = __ffs(left) - 1;
    const uint64_t b = __shfl_sync(0xffffffffu, bin, leader);
    const bool mine = live && bin == b;
    const uint32_t same = __ballot_sync(0xffffffffu, mine);
    const uint32_t sum = __reduce_add_sync(0xffffffffu, mine ? npos : 0u);
    if (lane == leader) {
      atomicAdd(&nent_bin[b], static_cast<unsigned long long>(__popc(same)));
      if (sum) atomicAdd(&npos_bin[b], static_cast<unsigned long long>(sum));
    }
    left &= ~same;
    if (mine) live = false;
  }
}

__global__ void insert_rep_kernel(const uint64_t* __restrict__ rep, uint64_t n, TableEntry* table,
                                  uint64_t cap, DeviceStatus* st) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!table_insert(table, cap, rep[i], kRepetitiveBit, true))
    raise_status(st, kDevTableFull, 1, i);
}

inline unsigned grid(uint64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

cudaError_t index_enumerate(const uint64_t* words, const uint64_t* base_off,
                            const uint64_t* win_off, const int32_t* slot_len, uint32_t nslots,
                            uint64_t nwin, int k, uint64_t* keys, uint64_t* vals,
                            cudaStream_t s) {
  if (nwin == 0) return cudaSuccess;
  count_launch();
  enumerate_kernel<<<grid(nwin, 256), 256, 0, s>>>(
      Windows{words, base_off, win_off, slot_len, nslots, nwin, k}, keys, vals);
  return cudaGetLastError();
}

cudaError_t index_prefix_hist(const uint64_t* words, const uint64_t* base_off,
                              const uint64_t* win_off, const int32_t* slot_len, uint32_t nslots,
                              uint64_t nwin, int k, int shift, int nbins,
                              unsigned long long* hist, int num_sms, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * nbins, s);
  if (e != cudaSuccess || nwin == 0) return e;
  const size_t smem = sizeof(uint32_t) * static_cast<size_t>(nbins);
  e = cudaFuncSetAttribute(prefix_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  count_launch();
  prefix_hist_kernel<<<static_cast<unsigned>(num_sms), 1024, smem, s>>>(
      Windows{words, base_off, win_off, slot_len, nslots, nwin, k}, shift, nbins, hist);
  return cudaGetLastError();
}

cudaError_t index_enumerate_range(const uint64_t* words, const uint64_t* base_off,
                                  const uint64_t* win_off, const int32_t* slot_len,
                                  uint32_t nslots, uint64_t nwin, int k, uint64_t lo,
                                  uint64_t hi, uint64_t* keys, uint64_t* vals,
                                  unsigned long long* count, uint64_t cap, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess || nwin == 0) return e;
  count_launch();
  enumerate_range_kernel<<<grid(nwin, 256), 256, 0, s>>>(
      Windows{words, base_off, win_off, slot_len, nslots, nwin, k}, lo, hi, keys, vals, count,
      cap);
  return cudaGetLastError();
}

cudaError_t index_mark_runs(const uint64_t* keys, uint64_t n, uint32_t* flags, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  mark_runs_kernel<<<grid(n, 256), 256, 0, s>>>(keys, n, flags);
  return cudaGetLastError();
}

cudaError_t index_run_starts(const uint32_t* flags, const uint64_t* run_id, uint64_t n,
                             uint64_t nruns, uint64_t* run_start, cudaStream_t s) {
  count_launch();
  run_starts_kernel<<<grid(n > 0 ? n : 1, 256), 256, 0, s>>>(flags, run_id, n, nruns,
                                                             run_start);
  return cudaGetLastError();
}

cudaError_t index_classify_runs(const uint64_t* run_start, uint64_t nruns, uint32_t min_freq,
                                uint32_t max_freq, uint32_t* kept, uint8_t* cls,
                                unsigned long long* tally, cudaStream_t s) {
  if (tally) {
    const cudaError_t e = cudaMemsetAsync(tally, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
  }
  if (nruns == 0) return cudaSuccess;
  count_launch();
  classify_runs_kernel<<<grid(nruns, 256), 256, 0, s>>>(run_start, nruns, min_freq, max_freq,
                                                        kept, cls, tally);
  return cudaGetLastError();
}

cudaError_t index_copy_positions(const uint64_t* vals, const uint64_t* run_id,
                                 const uint64_t* run_start, const uint8_t* cls,
                                 const uint64_t* kept_off, uint64_t n, uint64_t* pos,
                                 cudaStream_t s, uint32_t* self_at, const uint64_t* win_off,
                                 const int32_t* slot_len, int k) {
  if (n == 0) return cudaSuccess;
  count_launch();
  copy_positions_kernel<<<grid(n, 256), 256, 0, s>>>(vals, run_id, run_start, cls, kept_off, n,
                                                     pos, self_at, win_off, slot_len, k);
  return cudaGetLastError();
}

cudaError_t index_insert(const uint64_t* keys, const uint64_t* vals, const uint64_t* run_start,
                         const uint8_t* cls, const uint64_t* kept_off, uint64_t nruns,
                         uint64_t pos_base, bool sorted_ids, TableEntry* table, uint64_t cap,
                         DeviceStatus* st, cudaStream_t s) {
  if (nruns == 0) return cudaSuccess;
  count_launch();
  insert_kernel<<<grid(nruns, 256), 256, 0, s>>>(keys, vals, run_start, cls, kept_off, nruns,
                                                 pos_base, sorted_ids, table, cap, st);
  return cudaGetLastError();
}

cudaError_t index_bin_totals(const uint64_t* keys, const uint64_t* run_start, const uint8_t* cls,
                             uint64_t nruns, int shift, unsigned long long* npos_bin,
                             unsigned long long* nent_bin, cudaStream_t s) {
  if (nruns == 0) return cudaSuccess;
  count_launch();
  bin_totals_kernel<<<grid(nruns, 256), 256, 0, s>>>(keys, run_start, cls, nruns, shift,
                                                     npos_bin, nent_bin);
  return cudaGetLastError();
}

cudaError_t index_insert_repetitive(const uint64_t* rep_keys, uint64_t n, TableEntry* table,
                                    uint64_t cap, DeviceStatus* st, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  insert_rep_kernel<<<grid(n, 256), 256, 0, s>>>(rep_keys, n, table, cap, st);
  return cudaGetLastError();
}

}  // namespace cuflye
