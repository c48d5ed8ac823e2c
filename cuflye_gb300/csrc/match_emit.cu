// match_emit.cu — candidate hits written straight into Flye's KmerMatch order,
// with the target groups and their prefilter decided on the way.
//
// Flye collects a query's KmerMatches window by window and bucket entry by
// bucket entry (patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:55-89),
// then std::sorts them by (ext id, cur pos)
// (patches/flye/2.9.6/0001-cuflye-candidate-match-dump.patch:86-92) and chains
// each run of one ext id (tools/replay_overlap_chains.py:228-270).  When no
// window's bucket lists a target twice (the query is not flagged in q_tie),
// the keys are distinct, so the sorted order is the only one: the hits of
// each ext id in window order, ext ids ascending.  Two kernels produce it
// without ever storing the hits in generation order:
//
//   match_dict_kernel  one block per query reads every bucket entry of the
//                      query's windows and counts the hits per ext id in a
//                      shared-memory hash table; the distinct ext ids, sorted,
//                      with their counts are the query's groups (the
//                      dictionary);
//   match_emit_kernel  one block per query reads the entries again in batches
//                      of up to 128 windows.  A window hits an ext id at most
//                      once, so a hit's place in its group is the group's
//                      running count plus the number of earlier windows of
//                      the batch that hit the same ext id (a 128-bit mask per
//                      group, set in a first phase, read in a second).  The
//                      hits are stored there directly: a group's hits of one
//                      batch fill consecutive slots, which the L2 cache merges
//                      into whole sectors.  Each group's least and greatest
//                      ext pos are kept on the way (shared-memory atomics), so
//                      every group's prefilter (survival, spans, overhangs) is
//                      decided here.
//
// A flagged query's hits are written in generation order instead (its equal
// keys need the libstdc++-order sort), and its groups are listed for the
// prefilter after that sort.  Both kernels visit a window's entries in the
// order hits_count / hits_emit do: the bucket's stored entries, flipped to
// the other strand when the window's k-mer is not in standard form, less the
// query's own position (its index in the bucket is wself).
//
// Work split: each thread takes kSePer consecutive entries of the batch (one
// search for its first window, then a forward walk), and issues all of its
// loads before using any.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr int kSeBlock = 512;
constexpr int kSeWarps = kSeBlock / 32;
constexpr int kSeWin = 128;           // windows per batch (bits of the group masks)
constexpr int kSeMaskWords = kSeWin / 64;
constexpr uint32_t kSePer = 8;        // consecutive entries per thread
constexpr uint32_t kSeBatch = kSePer * kSeBlock;  // bucket entries per batch
constexpr int kHashBits = 12;
constexpr uint32_t kHashSlots = 1u << kHashBits;  // load 1/2 at kMatchDictCap ids
constexpr uint32_t kNone = 0xffffffffu;

static_assert(kHashSlots == 2 * kMatchDictCap, "hash slots: twice the dictionary");
static_assert(kMatchDictCap % kSeBlock == 0, "dictionary ranks per thread");
static_assert(kMatchDictCap <= 65536, "ranks fit 16 bits");
static_assert(kSeWin <= kSeBlock, "one thread per batch window");
static_assert(kHashSlots % kSeBlock == 0, "hash slots per thread");

// Fibonacci hashing of a dense target id onto the table's slots.
__device__ __forceinline__ uint32_t hash_slot(uint32_t id) {
  return (id * 0x9E3779B1u) >> (32 - kHashBits);
}

// The windows of one batch, in shared memory.  Entry j of the batch (its
// visited entries numbered in window order) belongs to window wl_of[j]; its
// bucket entry is idx.pos[jbase[wl] + j], its generation-order slot
// hbase[wl] + j (less one past the self hit), and it is the query's own
// position when j == self_j[wl].
struct BatchWin {
  uint64_t jbase[kSeWin];    // ebase + first - cum (modulo 2^64)
  uint64_t hbase[kSeWin];    // hoff + first - cum (modulo 2^64)
  int32_t self_j[kSeWin];    // batch-local index of the self entry (may be < 0), or INT_MAX
  uint32_t prev[kSeWin];     // cur pos | rev << 31
  uint32_t cum[kSeWin + 1];  // batch-local index of each window's first visited entry
  uint8_t wl_of[kSeBatch];
  uint32_t wsum[kSeWin / 32];
  uint32_t nw, total;
  uint64_t next_w;
  uint32_t next_e;
};

struct EmitQuery {
  uint64_t w0, w1;  // the query's windows [w0, w1) in the pass
  uint64_t h0, h1;  // its hits [h0, h1) in the pass
};

// A window's fields as the batch setup reads them, all four loads issued at
// once (wself holds a value only for trivial windows; it is read anyway and
// used only then).
struct WinLoad {
  uint64_t meta = 0, hoff = 0;
  uint32_t self = 0;
  uint8_t fl = 0;
  bool in = false;
};

__device__ __forceinline__ WinLoad load_window(const MatchEmitArgs& a, const EmitQuery& eq,
                                               uint64_t wi) {
  WinLoad x;
  if (threadIdx.x < kSeWin && wi < eq.w1) {
    x.in = true;
    x.fl = a.wflags[wi];
    x.meta = a.wmeta[wi];
    x.self = a.wself[wi];
    x.hoff = a.hit_off[wi];
  }
  return x;
}

// Sets up the batch that starts at window w (bucket entry e0 of it): as many
// windows as fit kSeBatch entries and kSeWin windows, or kSeBatch entries of
// one window that has more.  win: thread t's load of window w + t (issued
// ahead, while the previous batch ran).  Writes the filtered positions of the
// batch's windows when fpos is given.  Every thread of the block calls it.
__device__ void batch_setup(BatchWin& b, const MatchEmitArgs& a, const EmitQuery& eq, uint64_t w,
                            uint32_t e0, const WinLoad& win) {
  const int t = threadIdx.x;
  uint32_t raw = 0;
  uint64_t ebase = 0, hoff = 0;
  uint32_t self = kNone, prev = 0;
  if (t < kSeWin) {
    const uint64_t wi = w + t;
    if (win.in) {
      const uint8_t fl = win.fl;
      if (!(fl & kWinFiltered)) {
        raw = static_cast<uint32_t>((win.meta >> 40) & ((1ULL << kCountBits) - 1));
        ebase = win.meta & kOffsetMask;
      }
      if (fl & kWinTrivial) self = win.self;
      hoff = win.hoff;
      prev = static_cast<uint32_t>(wi - eq.w0) | ((fl & kWinRev) ? 0x80000000u : 0u);
    }
    raw -= t == 0 ? e0 : 0u;
    uint32_t inc = raw;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if ((t & 31) >= o) inc += u;
    }
    if ((t & 31) == 31) b.wsum[t >> 5] = inc;
    raw = inc;  // inclusive within the warp
  }
  __syncthreads();
  if (t < kSeWin) {
    uint32_t before = 0;
#pragma unroll
    for (int k = 0; k < kSeWin / 32; ++k) before += k < (t >> 5) ? b.wsum[k] : 0u;
    raw += before;  // inclusive over the batch's windows
    b.cum[t + 1] = raw;
    if (t == 0) b.cum[0] = 0;
  }
  // windows whose entries all fit the batch (the cumulative counts rise)
  const int m = __syncthreads_count(t < kSeWin && raw <= kSeBatch);
  if (t < kSeWin) {
    const uint32_t first = t == 0 ? e0 : 0u;
    const uint32_t start = b.cum[t];
    b.jbase[t] = ebase + first - start;
    b.hbase[t] = hoff + first - start;
    b.self_j[t] = self == kNone ? INT_MAX
                                : static_cast<int32_t>(self) - static_cast<int32_t>(first) +
                                      static_cast<int32_t>(start);
    b.prev[t] = prev;
  }
  if (t == 0) {
    if (m == 0) {  // the first window alone holds more than a batch
      b.nw = 1;
      b.total = kSeBatch;
      b.next_w = w;
      b.next_e = e0 + kSeBatch;
    } else {
      b.nw = static_cast<uint32_t>(m);
      b.total = b.cum[m];
      b.next_w = w + static_cast<uint64_t>(m);
      b.next_e = 0;
    }
  }
  __syncthreads();
  // filtered positions of the windows this batch covers: a filtered window
  // has no entries, so it lies in exactly one batch
  if (a.fpos && t < static_cast<int>(b.nw) && win.in && (win.fl & kWinFiltered)) {
    const uint64_t wi = w + t;
    a.fpos[a.filt_off[wi]] = static_cast<int32_t>(wi - eq.w0);
  }
  // entry -> window table: each thread its kSePer consecutive entries (one
  // search, then a forward walk over windows without entries)
  const uint32_t j0 = static_cast<uint32_t>(t) * kSePer;
  if (j0 < b.total) {
    int lo = 0, hi = static_cast<int>(b.nw) - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (b.cum[mid] <= j0)
        lo = mid;
      else
        hi = mid - 1;
    }
#pragma unroll
    for (uint32_t u = 0; u < kSePer; ++u) {
      const uint32_t j = j0 + u;
      if (j < b.total) {
        while (b.cum[lo + 1] <= j) ++lo;
        b.wl_of[j] = static_cast<uint8_t>(lo);
      }
    }
  }
  __syncthreads();
}

// The thread's entries of the batch, j = threadIdx.x + u * kSeBlock (a warp
// takes 32 consecutive entries, mostly of one window), all loads issued
// before any use.  Bit u of valid marks entry u as present.
struct Entries {
  uint64_t sv[kSePer];
  uint8_t wl[kSePer];
  uint32_t valid;
};

__device__ __forceinline__ void load_entries(const BatchWin& b, const MatchEmitArgs& a,
                                             Entries& x) {
  x.valid = 0;
#pragma unroll
  for (uint32_t u = 0; u < kSePer; ++u) {
    const uint32_t j = threadIdx.x + u * kSeBlock;
    if (j < b.total) {
      x.wl[u] = b.wl_of[j];
      x.valid |= 1u << u;
    }
  }
#pragma unroll
  for (uint32_t u = 0; u < kSePer; ++u) {
    if (x.valid & (1u << u)) {
      const uint32_t j = threadIdx.x + u * kSeBlock;
      x.sv[u] = __ldg(a.idx.pos + (b.jbase[x.wl[u]] + j));
    }
  }
}

// Entry u after the strand transform: (target dense id, position); false for
// the query's own position.
__device__ __forceinline__ bool entry_hit(const BatchWin& b, const MatchEmitArgs& a,
                                          const Entries& x, uint32_t u, uint32_t& id,
                                          uint32_t& pos) {
  const int wl = x.wl[u];
  const int32_t j = static_cast<int32_t>(threadIdx.x + u * kSeBlock);
  id = static_cast<uint32_t>(x.sv[u] >> 32);
  pos = static_cast<uint32_t>(x.sv[u] & 0xffffffffu);
  if (b.prev[wl] & 0x80000000u) {
    pos = static_cast<uint32_t>(__ldg(a.idx.slot_len + (id >> 1)) - static_cast<int32_t>(pos) -
                                a.idx.k);
    id ^= 1u;
  }
  return j != b.self_j[wl];
}

// Next query of the block from the launch's counter.
__device__ __forceinline__ uint32_t next_query(uint32_t* counter, uint32_t* slot) {
  if (threadIdx.x == 0) *slot = atomicAdd(counter, 1u);
  __syncthreads();
  const uint32_t q = *slot;
  __syncthreads();
  return q;
}

// ------------------------------------------------------------ dictionary

struct DictSmem {
  // the hash table; once counted, its slots are compacted into list (which
  // takes the place of key: kMatchDictCap words of 8 bytes)
  union {
    uint32_t key[kHashSlots];
    uint64_t list[kMatchDictCap];
  };
  uint32_t cnt[kHashSlots];
  BatchWin b;
  unsigned long long dslot;  // the query's first word in dict
  uint32_t nkeys, nlist, qslot;
};

__global__ void __launch_bounds__(kSeBlock, 3) match_dict_kernel(MatchEmitArgs a, uint64_t* dict,
                                                               unsigned long long* dict_cursor,
                                                               uint32_t* q_ng, uint64_t* q_dbase,
                                                               uint32_t* overflow,
                                                               uint32_t* counter) {
  extern __shared__ __align__(16) unsigned char dict_raw[];
  DictSmem& sm = *reinterpret_cast<DictSmem*>(dict_raw);
  const int t = threadIdx.x;
  for (;;) {
    const uint32_t q = next_query(counter, &sm.qslot);
    if (q >= a.nq) return;
    for (uint32_t s = t; s < kHashSlots; s += kSeBlock) {
      sm.key[s] = kNone;
      sm.cnt[s] = 0;
    }
    if (t == 0) {
      sm.nkeys = 0;
      sm.nlist = 0;
    }
    const EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q], a.q_off[q + 1]};
    __syncthreads();
    uint64_t w = eq.w0;
    uint32_t e0 = 0;
    bool over = false;
    WinLoad win = load_window(a, eq, w + t);
    while (w < eq.w1 && !over) {
      batch_setup(sm.b, a, eq, w, e0, win);
      // the next batch's windows load while this one runs
      win = load_window(a, eq, sm.b.next_w + t);
      Entries x;
      load_entries(sm.b, a, x);
#pragma unroll
      for (uint32_t u = 0; u < kSePer; ++u) {
        uint32_t id, pos;
        if (!(x.valid & (1u << u)) || !entry_hit(sm.b, a, x, u, id, pos)) continue;
        uint32_t s = hash_slot(id);
        for (uint32_t probe = 0; probe < kHashSlots; ++probe) {
          uint32_t k = sm.key[s];
          if (k == kNone) {
            k = atomicCAS(&sm.key[s], kNone, id);
            if (k == kNone) {
              atomicAdd(&sm.nkeys, 1u);
              k = id;
            }
          }
          if (k == id) {
            atomicAdd(&sm.cnt[s], 1u);
            break;
          }
          s = (s + 1) & (kHashSlots - 1);
        }
      }
      w = sm.b.next_w;
      e0 = sm.b.next_e;
      __syncthreads();
      over = sm.nkeys > kMatchDictCap;  // block-uniform (read after the barrier)
    }
    if (over) {
      if (t == 0) {
        q_ng[q] = 0;
        q_dbase[q] = 0;
        atomicAdd(overflow, 1u);
      }
      __syncthreads();
      continue;
    }
    const uint32_t n = sm.nkeys;
    constexpr uint32_t kSlotsPer = kHashSlots / kSeBlock;
    uint64_t kc[kSlotsPer];
#pragma unroll
    for (uint32_t u = 0; u < kSlotsPer; ++u) {
      const uint32_t s = t + u * kSeBlock;
      kc[u] = (static_cast<uint64_t>(sm.key[s]) << 32) | sm.cnt[s];
    }
    __syncthreads();  // list overwrites key from here on
#pragma unroll
    for (uint32_t u = 0; u < kSlotsPer; ++u) {
      if ((kc[u] >> 32) != kNone) sm.list[atomicAdd(&sm.nlist, 1u)] = kc[u];
    }
    __syncthreads();
    // bitonic sort of the (ext id, count) words by ext id, padded to a power of two
    uint32_t n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (uint32_t i = n + t; i < n2; i += kSeBlock) sm.list[i] = ~0ULL;
    __syncthreads();
    for (uint32_t size = 2; size <= n2; size <<= 1) {
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = t; i < n2 / 2; i += kSeBlock) {
          const uint32_t lo = 2 * i - (i & (stride - 1));
          const uint32_t hi = lo + stride;
          const bool up = (lo & size) == 0;
          const uint64_t x0 = sm.list[lo], x1 = sm.list[hi];
          if ((x0 > x1) == up) {
            sm.list[lo] = x1;
            sm.list[hi] = x0;
          }
        }
        __syncthreads();
      }
    }
    if (t == 0) {
      sm.dslot = n ? atomicAdd(dict_cursor, static_cast<unsigned long long>(n)) : 0ULL;
      q_ng[q] = n;
    }
    __syncthreads();
    const uint64_t base = sm.dslot;
    if (t == 0) q_dbase[q] = base;
    for (uint32_t i = t; i < n; i += kSeBlock) dict[base + i] = sm.list[i];
    __syncthreads();
  }
}

// ------------------------------------------------------------ emission

struct EmitSmem {
  unsigned long long hent[kHashSlots];  // rank << 32 | ext id (kNone: free)
  uint32_t cursor[kMatchDictCap];  // the group's next hit, counted from the query's first
  unsigned long long mask[kSeMaskWords][kMatchDictCap];  // batch windows that hit the group
  int32_t mnx[kMatchDictCap];      // least ext pos of the group's hits
  int32_t mxx[kMatchDictCap];      // greatest
  BatchWin b;
  uint32_t ws[kSeWarps];
  uint32_t qslot;
};

// Exclusive scan of v over the block's threads (thread order).
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
#pragma unroll
  for (int w = 0; w < kSeWarps; ++w) before += w < warp ? ws[w] : 0u;
  __syncthreads();
  return before + inc - v;
}

// Rank of ext id `id` in its query's dictionary.  Every hit's id is there
// (the dictionary counted the same entries); the probe is still bounded, and
// a miss is reported through the status word and the hit dropped (kNone).
__device__ __forceinline__ uint32_t rank_of(const EmitSmem& sm, uint32_t id, DeviceStatus* st) {
  uint32_t s = hash_slot(id);
  for (uint32_t probe = 0; probe < kHashSlots; ++probe) {
    const unsigned long long e = sm.hent[s];
    const uint32_t k = static_cast<uint32_t>(e);
    if (k == id) return static_cast<uint32_t>(e >> 32);
    if (k == kNone) break;
    s = (s + 1) & (kHashSlots - 1);
  }
  raise_status(st, kDevMatchDict, 0, id);
  return kNone;
}

// Hits of group r in the batch's windows before wl.
__device__ __forceinline__ uint32_t earlier_hits(const EmitSmem& sm, uint32_t r, int wl) {
  const unsigned long long m0 = sm.mask[0][r];
  if (wl < 64) return static_cast<uint32_t>(__popcll(m0 & ((1ULL << wl) - 1)));
  const unsigned long long m1 = sm.mask[1][r];
  return static_cast<uint32_t>(__popcll(m0) + __popcll(m1 & ((1ULL << (wl - 64)) - 1)));
}

__global__ void __launch_bounds__(kSeBlock, 2) match_emit_kernel(
    MatchEmitArgs a, const uint64_t* __restrict__ dict, const uint32_t* __restrict__ q_ng,
    const uint64_t* __restrict__ q_dbase, const uint64_t* __restrict__ q_goff,
    const uint32_t* __restrict__ q_tie, const QueryInfo* __restrict__ qinfo, ChainParams p,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, GroupInfo* __restrict__ groups,
    MatchEmitLists lists, uint32_t* counter) {
  static_assert(kSeMaskWords == 2, "two mask words per group");
  extern __shared__ __align__(16) unsigned char emit_raw[];
  EmitSmem& sm = *reinterpret_cast<EmitSmem*>(emit_raw);
  const int t = threadIdx.x;
  constexpr uint32_t kPer = kMatchDictCap / kSeBlock;  // ranks per thread in scans
  for (;;) {
    const uint32_t q = next_query(counter, &sm.qslot);
    if (q >= a.nq) return;
    const EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q], a.q_off[q + 1]};
    const uint32_t ng = min(q_ng[q], kMatchDictCap);
    const uint64_t dbase = q_dbase[q];
    const bool flagged = q_tie[q] != 0;
    // dictionary -> hash of ext id to rank, and each group's first hit
    for (uint32_t s = t; s < kHashSlots; s += kSeBlock) sm.hent[s] = kNone;
    __syncthreads();
    uint32_t c[kPer], sum = 0;
#pragma unroll
    for (uint32_t u = 0; u < kPer; ++u) {
      const uint32_t r = t * kPer + u;
      c[u] = 0;
      if (r < ng) {
        const uint64_t d = dict[dbase + r];
        const uint32_t id = static_cast<uint32_t>(d >> 32);
        c[u] = static_cast<uint32_t>(d);
        // ng <= kMatchDictCap distinct ids in 2 * kMatchDictCap slots: a free
        // slot is always found within the table
        uint32_t s = hash_slot(id);
        for (uint32_t probe = 0; probe < kHashSlots; ++probe) {
          if (atomicCAS(&sm.hent[s], static_cast<unsigned long long>(kNone),
                        (static_cast<unsigned long long>(r) << 32) | id) == kNone)
            break;
          s = (s + 1) & (kHashSlots - 1);
        }
      }
      sum += c[u];
    }
    uint32_t run = block_exclusive(sum, sm.ws);
#pragma unroll
    for (uint32_t u = 0; u < kPer; ++u) {
      const uint32_t r = t * kPer + u;
      if (r < ng) {
        sm.cursor[r] = run;
        sm.mask[0][r] = 0;
        sm.mask[1][r] = 0;
        sm.mnx[r] = INT_MAX;
        sm.mxx[r] = INT_MIN;
      }
      run += c[u];
    }
    __syncthreads();
    uint64_t w = eq.w0;
    uint32_t e0 = 0;
    WinLoad win = load_window(a, eq, w + t);
    while (w < eq.w1) {
      batch_setup(sm.b, a, eq, w, e0, win);
      // the next batch's windows load while this one runs
      win = load_window(a, eq, sm.b.next_w + t);
      Entries x;
      load_entries(sm.b, a, x);
      if (flagged) {
        // generation order: the window's first hit plus the entry's index
        // among the window's hits
#pragma unroll
        for (uint32_t u = 0; u < kSePer; ++u) {
          uint32_t id, pos;
          if (!(x.valid & (1u << u)) || !entry_hit(sm.b, a, x, u, id, pos)) continue;
          const int wl = x.wl[u];
          const int32_t j = static_cast<int32_t>(t + u * kSeBlock);
          const uint64_t d = sm.b.hbase[wl] + static_cast<uint64_t>(j) -
                             (sm.b.self_j[wl] < j ? 1u : 0u);
          const uint64_t key = (static_cast<uint64_t>(id) << 32) | (sm.b.prev[wl] & 0x7fffffffu);
          if (d >= eq.h0 && d < eq.h1) {  // always: the window's hits lie in the query's range
            keys[d] = key;
            vals[d] = pos;
          }
          // equal keys come only from a bucket listing one target twice, at
          // neighbouring entries: record the key when the entry before this
          // one (in the bucket) has the same target
          if (lists.tie_count &&
              (j > static_cast<int32_t>(sm.b.cum[wl]) || (wl == 0 && e0 > 0))) {
            const uint64_t before = __ldg(a.idx.pos + (sm.b.jbase[wl] + static_cast<uint64_t>(j) - 1u));
            if ((before >> 32) == (x.sv[u] >> 32)) {
              const uint32_t slot = atomicAdd(lists.tie_count, 1u);
              if (slot < lists.tie_cap) {
                lists.tie_h0[slot] = eq.h0;
                lists.tie_key[slot] = key;
              }
            }
          }
        }
      } else {
        // first phase: each hit's group rank and transformed entry (id << 32
        // | pos, in sv); the group masks and ext-pos extremes
        uint32_t rk[kSePer];
#pragma unroll
        for (uint32_t u = 0; u < kSePer; ++u) {
          uint32_t id, pos, r = kNone;
          if ((x.valid & (1u << u)) && entry_hit(sm.b, a, x, u, id, pos)) {
            r = rank_of(sm, id, a.status);
            x.sv[u] = (static_cast<uint64_t>(id) << 32) | pos;
            if (r != kNone) {
              const int wl = x.wl[u];
              atomicOr(reinterpret_cast<unsigned*>(&sm.mask[wl >> 6][r]) + ((wl >> 5) & 1),
                       1u << (wl & 31));
              atomicMin(&sm.mnx[r], static_cast<int32_t>(pos));
              atomicMax(&sm.mxx[r], static_cast<int32_t>(pos));
            }
          }
          rk[u] = r;
        }
        __syncthreads();
        // second phase: each hit at its group's place
#pragma unroll
        for (uint32_t u = 0; u < kSePer; ++u) {
          const uint32_t r = rk[u];
          if (r == kNone) continue;
          const int wl = x.wl[u];
          const uint64_t d = eq.h0 + sm.cursor[r] + earlier_hits(sm, r, wl);
          if (d < eq.h1) {  // always, with the dictionary's counts
            keys[d] = (x.sv[u] & 0xffffffff00000000ULL) | (sm.b.prev[wl] & 0x7fffffffu);
            vals[d] = static_cast<uint32_t>(x.sv[u]);
          } else {
            raise_status(a.status, kDevMatchDict, 1, static_cast<int64_t>(q));
          }
        }
        __syncthreads();
#pragma unroll
        for (uint32_t u = 0; u < kPer; ++u) {
          const uint32_t r = t * kPer + u;
          if (r < ng) {
            const unsigned long long m0 = sm.mask[0][r], m1 = sm.mask[1][r];
            if (m0 | m1) {
              sm.cursor[r] += static_cast<uint32_t>(__popcll(m0) + __popcll(m1));
              sm.mask[0][r] = 0;
              sm.mask[1][r] = 0;
            }
          }
        }
      }
      w = sm.b.next_w;
      e0 = sm.b.next_e;
      __syncthreads();
    }
    // the query's groups: GroupInfo and the prefilter; flagged queries' groups
    // wait for their libstdc++-order sort
    const int32_t cur_len = qinfo[q].len;
    const uint64_t g0 = q_goff[q];
    for (uint32_t r = t; r < ng; r += kSeBlock) {
      const uint64_t d = dict[dbase + r];
      const uint32_t ext = static_cast<uint32_t>(d >> 32);
      const uint32_t n = static_cast<uint32_t>(d);
      GroupInfo gi{};
      gi.start = eq.h0 + (flagged ? sm.cursor[r] : sm.cursor[r] - n);
      gi.n = n;
      gi.query = q;
      gi.ext_di = ext;
      gi.ext_len = __ldg(a.idx.slot_len + (ext >> 1));
      gi.survive = 0;
      gi.ext_sorted = 0;
      const uint32_t g = static_cast<uint32_t>(g0 + r);
      if (!flagged) {
        // in KmerMatch order the group's cur positions rise, each once: its
        // first and last hits hold the least and greatest
        const int32_t min_cur = static_cast<int32_t>(keys[gi.start] & 0xffffffffu);
        const int32_t max_cur = static_cast<int32_t>(keys[gi.start + n - 1] & 0xffffffffu);
        const uint32_t uniq = n - (min_cur == 0 ? 1u : 0u);
        gi.ext_sorted = gi.ext_len > cur_len ? 1 : 0;
        if (prefilter_keeps(uniq, min_cur, max_cur, sm.mnx[r], sm.mxx[r], cur_len, gi.ext_len,
                            p)) {
          gi.survive = 1;
          lists.dp_list[atomicAdd(lists.counts + 1, 1u)] = g;
          if (gi.ext_sorted) lists.ext_list[atomicAdd(lists.counts + 0, 1u)] = g;
        }
      } else {
        lists.pf_list[atomicAdd(lists.counts + 2, 1u)] = g;
        atomicAdd(lists.tally + 1, static_cast<unsigned long long>(n));
      }
      groups[g] = gi;
    }
    if (flagged && t == 0 && eq.h0 + 1 < eq.h1) {
      const uint32_t s = atomicAdd(lists.emu_count, 1u);
      lists.emu_begin[s] = eq.h0;
      lists.emu_end[s] = eq.h1;
      atomicAdd(lists.tally, static_cast<unsigned long long>(eq.h1 - eq.h0));
    }
    __syncthreads();
  }
}

// Blocks of a kernel resident per SM, at least one.
template <class K>
int resident(K kernel, size_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kSeBlock, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return std::max(per_sm, 1);
}

}  // namespace

size_t match_dict_smem_bytes() { return sizeof(DictSmem); }
size_t match_emit_smem_bytes() { return sizeof(EmitSmem); }

cudaError_t match_dict(const MatchEmitArgs& a, uint64_t* dict, unsigned long long* dict_cursor,
                       uint32_t* q_ng, uint64_t* q_dbase, uint32_t* overflow, uint32_t* counter,
                       int num_sms, cudaStream_t s) {
  if (a.nq == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(match_dict_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(DictSmem)));
  // all of the SM's shared memory, so that four blocks fit
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(match_dict_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             100);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(
      static_cast<uint64_t>(resident(match_dict_kernel, sizeof(DictSmem))) * num_sms, a.nq));
  MatchEmitArgs da = a;
  da.fpos = nullptr;  // the filtered positions are match_emit's to write
  count_launch();
  match_dict_kernel<<<grid, kSeBlock, sizeof(DictSmem), s>>>(da, dict, dict_cursor, q_ng, q_dbase,
                                                             overflow, counter);
  return cudaGetLastError();
}

cudaError_t match_emit(const MatchEmitArgs& a, const uint64_t* dict, const uint32_t* q_ng,
                       const uint64_t* q_dbase, const uint64_t* q_goff, const uint32_t* q_tie,
                       const QueryInfo* qinfo, const ChainParams& p, uint64_t* keys,
                       uint32_t* vals, GroupInfo* groups, const MatchEmitLists& lists,
                       uint32_t* counter, int num_sms, cudaStream_t s) {
  if (a.nq == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(match_emit_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(EmitSmem)));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(match_emit_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             100);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(
      static_cast<uint64_t>(resident(match_emit_kernel, sizeof(EmitSmem))) * num_sms, a.nq));
  count_launch();
  match_emit_kernel<<<grid, kSeBlock, sizeof(EmitSmem), s>>>(a, dict, q_ng, q_dbase, q_goff, q_tie,
                                                             qinfo, p, keys, vals, groups, lists,
                                                             counter);
  return cudaGetLastError();
}

}  // namespace cuflye
