// introsort.cuh — libstdc++-order segmented sort of (u64 key, u32 value) pairs.
//
// Flye orders KmerMatches, ext-sorted groups, chain starts, overlap proposals
// and read-to-graph alignments with libstdc++'s std::sort, which is not
// stable: equal keys end in an order fixed by the algorithm (introsort =
// median-of-three quicksort with Hoare's unguarded partition, a heapsort
// once the recursion depth 2*floor(log2 n) runs out, and a final insertion
// sort over blocks of at most 16 elements).  The reference's replay closes
// its last mismatch only by emulating that order
// (tools/replay_read_to_graph_source_pack.py:95-181).  These routines give
// the same order on the GPU.
//
// Parallel partition.  With pivot value P at position f, the left scan of
// the unguarded partition stops at "L stoppers" (K[i] >= P, i > f) and the
// right scan at "R stoppers" (K[i] <= P, i >= f).  Let l_k be the k-th L
// stopper from the left and r_k the k-th R stopper from the right.  The
// partition swaps l_k with r_k for every k with l_k < r_k (k = 1..m, a prefix
// since l_k rises and r_k falls) and returns cut = min(l_{m+1}, r_m), or l_1
// when m = 0: positions between the two scan fronts are never modified
// before the fronts reach them, so each scan meets exactly the original
// stoppers.  Ranks come from one prefix count, so a block (or a grid) can
// partition n elements in O(n) work and O(log n) depth.
//
// Leaves.  After the partitions every element of a block of <= 16 elements
// is >= every element of the blocks to its left, so libstdc++'s final
// insertion sort never moves an element across a block boundary: it equals a
// stable insertion sort inside each block.
#pragma once

#include <cstdint>

namespace cuflye {
namespace isort {

constexpr uint32_t kLeaf = 16;

__device__ __forceinline__ void swap_kv(uint64_t* K, uint32_t* V, uint32_t a, uint32_t b) {
  const uint64_t tk = K[a];
  K[a] = K[b];
  K[b] = tk;
  const uint32_t tv = V[a];
  V[a] = V[b];
  V[b] = tv;
}

// Median of K[a], K[b], K[c] moved to `res` (std::sort's pivot choice with
// a = f + 1, b = f + (l - f) / 2, c = l - 1).
__device__ __forceinline__ void median_to_first(uint64_t* K, uint32_t* V, uint32_t res,
                                                uint32_t a, uint32_t b, uint32_t c) {
  const uint64_t ka = K[a], kb = K[b], kc = K[c];
  uint32_t pick;
  if (ka < kb) {
    if (kb < kc)
      pick = b;
    else if (ka < kc)
      pick = c;
    else
      pick = a;
  } else if (ka < kc) {
    pick = a;
  } else if (kb < kc) {
    pick = c;
  } else {
    pick = b;
  }
  swap_kv(K, V, res, pick);
}

// Stable insertion sort of [f, l).
__device__ __forceinline__ void leaf_sort(uint64_t* K, uint32_t* V, uint32_t f, uint32_t l) {
  for (uint32_t i = f + 1; i < l; ++i) {
    const uint64_t k = K[i];
    const uint32_t v = V[i];
    uint32_t j = i;
    while (j > f && k < K[j - 1]) {
      K[j] = K[j - 1];
      V[j] = V[j - 1];
      --j;
    }
    K[j] = k;
    V[j] = v;
  }
}

// Binary heap with the hole technique: the hole walks down to a leaf along
// the larger child (the left one when the right is not larger), then the
// saved value climbs back up while its parent is smaller.
__device__ __forceinline__ void heap_adjust(uint64_t* K, uint32_t* V, uint32_t base,
                                            uint32_t hole, uint32_t len, uint64_t vk,
                                            uint32_t vv) {
  const uint32_t top = hole;
  uint32_t child = hole;
  while (len > 2 && child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (K[base + child] < K[base + child - 1]) --child;
    K[base + hole] = K[base + child];
    V[base + hole] = V[base + child];
    hole = child;
  }
  if ((len & 1u) == 0 && len >= 2 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    K[base + hole] = K[base + child - 1];
    V[base + hole] = V[base + child - 1];
    hole = child - 1;
  }
  while (hole > top) {
    const uint32_t parent = (hole - 1) / 2;
    if (!(K[base + parent] < vk)) break;
    K[base + hole] = K[base + parent];
    V[base + hole] = V[base + parent];
    hole = parent;
  }
  K[base + hole] = vk;
  V[base + hole] = vv;
}

// Heapsort of [f, l): build the heap from the last parent down, then pop the
// maximum to the back repeatedly.
__device__ inline void heap_sort(uint64_t* K, uint32_t* V, uint32_t f, uint32_t l) {
  const uint32_t len = l - f;
  if (len < 2) return;
  for (uint32_t parent = (len - 2) / 2;; --parent) {
    heap_adjust(K, V, f, parent, len, K[f + parent], V[f + parent]);
    if (parent == 0) break;
  }
  for (uint32_t last = len; last > 1;) {
    --last;
    const uint64_t vk = K[f + last];
    const uint32_t vv = V[f + last];
    K[f + last] = K[f];
    V[f + last] = V[f];
    heap_adjust(K, V, f, 0, last, vk, vv);
  }
}

// One unguarded partition of [f, l) (l - f > kLeaf), pivot moved to f.
__device__ __forceinline__ uint32_t serial_partition(uint64_t* K, uint32_t* V, uint32_t f,
                                                     uint32_t l) {
  median_to_first(K, V, f, f + 1, f + (l - f) / 2, l - 1);
  const uint64_t p = K[f];
  uint32_t lo = f + 1, hi = l;
  for (;;) {
    while (K[lo] < p) ++lo;
    --hi;
    while (p < K[hi]) --hi;
    if (!(lo < hi)) return lo;
    swap_kv(K, V, lo, hi);
    ++lo;
  }
}

__host__ __device__ __forceinline__ int depth_limit(uint32_t n) {
  int lg = 0;
  while ((n >> (lg + 1)) != 0) ++lg;
  return 2 * lg;
}

// Whole libstdc++ sort of [f, l) starting at recursion budget `depth`, by one
// thread.  Pending right halves wait on a small explicit stack.
__device__ inline void serial_introsort(uint64_t* K, uint32_t* V, uint32_t f, uint32_t l,
                                        int depth) {
  uint32_t sf[64], sl[64];
  int sd[64];
  int top = 0;
  for (;;) {
    while (l - f > kLeaf) {
      if (depth == 0) {
        heap_sort(K, V, f, l);
        f = l;
        break;
      }
      --depth;
      const uint32_t cut = serial_partition(K, V, f, l);
      sf[top] = cut;
      sl[top] = l;
      sd[top] = depth;
      ++top;
      l = cut;
    }
    if (l > f) leaf_sort(K, V, f, l);
    if (top == 0) return;
    --top;
    f = sf[top];
    l = sl[top];
    depth = sd[top];
  }
}

}  // namespace isort
}  // namespace cuflye
