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
// copied in run order -> open-addressing insert (linear probing, load <= 1/2).
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

__global__ void enumerate_kernel(const uint64_t* __restrict__ words,
                                 const uint64_t* __restrict__ base_off,
                                 const uint64_t* __restrict__ win_off,
                                 const int32_t* __restrict__ slot_len, uint32_t nslots,
                                 uint64_t nwin, int k, uint64_t* __restrict__ keys,
                                 uint64_t* __restrict__ vals) {
  const uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= nwin) return;
  const uint32_t t = find_segment(win_off, nslots, w);
  const uint64_t p = w - win_off[t];
  const uint64_t x = kmer_at(words, base_off[t] + p, k);
  const uint64_t rc = revcomp(x, k);
  if (rc < x) {
    keys[w] = rc;
    vals[w] = (static_cast<uint64_t>(2u * t + 1u) << 32) |
              static_cast<uint32_t>(slot_len[t] - static_cast<int32_t>(p) - k);
  } else {
    keys[w] = x;
    vals[w] = (static_cast<uint64_t>(2u * t) << 32) | static_cast<uint32_t>(p);
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

__global__ void classify_runs_kernel(const uint64_t* __restrict__ run_start, uint64_t nruns,
                                     uint32_t min_freq, uint32_t max_freq,
                                     uint32_t* __restrict__ kept, uint8_t* __restrict__ cls) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= nruns) return;
  const uint64_t freq = run_start[r + 1] - run_start[r];
  uint8_t c = 0;
  if (freq > max_freq)
    c = 2;
  else if (freq >= min_freq)
    c = 1;
  cls[r] = c;
  kept[r] = c == 1 ? static_cast<uint32_t>(freq) : 0u;
}

__global__ void copy_positions_kernel(const uint64_t* __restrict__ vals,
                                      const uint64_t* __restrict__ flags_scan,
                                      const uint64_t* __restrict__ run_start,
                                      const uint8_t* __restrict__ cls,
                                      const uint64_t* __restrict__ kept_off, uint64_t n,
                                      uint64_t* __restrict__ pos) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // flags_scan holds the exclusive scan of run-start flags: the run of
  // element i is the number of run starts at or before i, minus one.
  uint64_t r = flags_scan[i];
  if (r >= 1 && run_start[r] > i) r -= 1;
  while (run_start[r] > i) --r;
  if (cls[r] != 1) return;
  pos[kept_off[r] + (i - run_start[r])] = vals[i];
}

__device__ bool table_insert(TableEntry* table, uint64_t mask, uint64_t key, uint64_t meta,
                             bool merge_rep) {
  uint64_t slot = mix64(key) & mask;
  for (uint64_t step = 0; step <= mask; ++step) {
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
    slot = (slot + 1) & mask;
  }
  return false;
}

// vals: the run's entries, (stored id << 32) | stored position.  With
// sorted_ids the entries of a run are in (id, position) order and a repeated
// id shows as two neighbours; otherwise (explicit entries in input order)
// every run of two or more entries is marked.
__global__ void insert_kernel(const uint64_t* __restrict__ keys,
                              const uint64_t* __restrict__ vals,
                              const uint64_t* __restrict__ run_start,
                              const uint8_t* __restrict__ cls,
                              const uint64_t* __restrict__ kept_off, uint64_t nruns,
                              bool sorted_ids, TableEntry* table, uint64_t mask,
                              DeviceStatus* st) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= nruns || cls[r] == 0) return;
  const uint64_t r0 = run_start[r];
  const uint64_t key = keys[r0];
  const uint64_t freq = run_start[r + 1] - r0;
  uint64_t meta;
  if (cls[r] == 2) {
    const uint64_t c = freq < ((1ULL << kCountBits) - 1) ? freq : ((1ULL << kCountBits) - 1);
    meta = kRepetitiveBit | (c << 40);
  } else {
    meta = (kept_off[r] & kOffsetMask) | (freq << 40);
    bool dup = !sorted_ids && freq > 1;
    for (uint64_t e = 1; sorted_ids && e < freq && !dup; ++e)
      dup = (vals[r0 + e] >> 32) == (vals[r0 + e - 1] >> 32);
    if (dup) meta |= kDupIdsBit;
  }
  if (!table_insert(table, mask, key, meta, false)) raise_status(st, kDevTableFull, 0, r);
}

__global__ void insert_rep_kernel(const uint64_t* __restrict__ rep, uint64_t n, TableEntry* table,
                                  uint64_t mask, DeviceStatus* st) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!table_insert(table, mask, rep[i], kRepetitiveBit, true))
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
  enumerate_kernel<<<grid(nwin, 256), 256, 0, s>>>(words, base_off, win_off, slot_len, nslots,
                                                   nwin, k, keys, vals);
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
                                cudaStream_t s) {
  if (nruns == 0) return cudaSuccess;
  count_launch();
  classify_runs_kernel<<<grid(nruns, 256), 256, 0, s>>>(run_start, nruns, min_freq, max_freq,
                                                        kept, cls);
  return cudaGetLastError();
}

cudaError_t index_copy_positions(const uint64_t* vals, const uint64_t* run_id,
                                 const uint64_t* run_start, const uint8_t* cls,
                                 const uint64_t* kept_off, uint64_t n, uint64_t* pos,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  copy_positions_kernel<<<grid(n, 256), 256, 0, s>>>(vals, run_id, run_start, cls, kept_off, n,
                                                     pos);
  return cudaGetLastError();
}

cudaError_t index_insert(const uint64_t* keys, const uint64_t* vals, const uint64_t* run_start,
                         const uint8_t* cls, const uint64_t* kept_off, uint64_t nruns,
                         bool sorted_ids, TableEntry* table, uint64_t mask, DeviceStatus* st,
                         cudaStream_t s) {
  if (nruns == 0) return cudaSuccess;
  count_launch();
  insert_kernel<<<grid(nruns, 256), 256, 0, s>>>(keys, vals, run_start, cls, kept_off, nruns,
                                                 sorted_ids, table, mask, st);
  return cudaGetLastError();
}

cudaError_t index_insert_repetitive(const uint64_t* rep_keys, uint64_t n, TableEntry* table,
                                    uint64_t mask, DeviceStatus* st, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  insert_rep_kernel<<<grid(n, 256), 256, 0, s>>>(rep_keys, n, table, mask, st);
  return cudaGetLastError();
}

}  // namespace cuflye
