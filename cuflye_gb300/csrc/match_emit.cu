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

// Sets up the batch that starts at window w (bucket entry e0 of it): as many
// windows as fit kSeBatch entries and kSeWin windows, or kSeBatch entries of
// one window that has more.  Writes the filtered positions of the batch's
// windows when fpos is given.  Every thread of the block calls it.
__device__ void batch_setup(BatchWin& b, const MatchEmitArgs& a, const EmitQuery& eq, uint64_t w,
                            uint32_t e0) {
  const int t = threadIdx.x;
  uint32_t raw = 0;
  uint64_t ebase = 0, hoff = 0;
  uint32_t self = kNone, prev = 0;
  if (t < kSeWin) {
    const uint64_t wi = w + t;
    if (wi < eq.w1) {
      const uint8_t fl = a.wflags[wi];
      if (!(fl & kWinFiltered)) {
        const uint64_t meta = a.wmeta[wi];
        raw = static_cast<uint32_t>((meta >> 40) & ((1ULL << kCountBits) - 1));
        ebase = meta & kOffsetMask;
      }
      if (fl & kWinTrivial) self = a.wself[wi];
      hoff = a.hit_off[wi];
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
  if (a.fpos && t < static_cast<int>(b.nw)) {
    const uint64_t wi = w + t;
    if (wi < eq.w1 && (a.wflags[wi] & kWinFiltered))
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

// The queries qlist[0 .. *qcount) (those the warp kernel found to hit more
// than kWarpDictCap targets), one block each.
__global__ void __launch_bounds__(kSeBlock, 3) match_dict_kernel(MatchEmitArgs a, uint64_t* dict,
                                                               unsigned long long* dict_cursor,
                                                               uint32_t* q_ng, uint64_t* q_dbase,
                                                               uint32_t* overflow,
                                                               const uint32_t* qlist,
                                                               const uint32_t* qcount,
                                                               uint32_t* counter) {
  extern __shared__ __align__(16) unsigned char dict_raw[];
  DictSmem& sm = *reinterpret_cast<DictSmem*>(dict_raw);
  const int t = threadIdx.x;
  const uint32_t nlisted = *qcount;
  for (;;) {
    const uint32_t qi = next_query(counter, &sm.qslot);
    if (qi >= nlisted) return;
    const uint32_t q = qlist[qi];
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
    while (w < eq.w1 && !over) {
      batch_setup(sm.b, a, eq, w, e0);
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
  uint32_t hkey[kHashSlots];
  uint16_t hrank[kHashSlots];
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
    const uint32_t k = sm.hkey[s];
    if (k == id) return sm.hrank[s];
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

// The query's groups: their GroupInfo, and the prefilter of an unflagged
// query's groups (cursor[r]: the group's end, counted from the query's first
// hit; mnx / mxx its ext-pos extremes).  A flagged query's groups (cursor[r]:
// the group's start) wait for its libstdc++-order sort in pf_list.  Threads
// lane0, lane0 + step, ... take the ranks.
__device__ __forceinline__ void finish_query(const MatchEmitArgs& a, const uint64_t* dict,
                                             uint64_t dbase, uint32_t ng, const uint64_t* q_goff,
                                             const QueryInfo* qinfo, const ChainParams& p,
                                             const uint64_t* keys, GroupInfo* groups,
                                             const MatchEmitLists& lists, uint32_t q,
                                             const EmitQuery& eq, bool flagged,
                                             const uint32_t* cursor, const int32_t* mnx,
                                             const int32_t* mxx, uint32_t lane0, uint32_t step) {
  const int32_t cur_len = qinfo[q].len;
  const uint64_t g0 = q_goff[q];
  for (uint32_t r = lane0; r < ng; r += step) {
    const uint64_t d = dict[dbase + r];
    const uint32_t ext = static_cast<uint32_t>(d >> 32);
    const uint32_t n = static_cast<uint32_t>(d);
    GroupInfo gi{};
    gi.start = eq.h0 + (flagged ? cursor[r] : cursor[r] - n);
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
      if (prefilter_keeps(uniq, min_cur, max_cur, mnx[r], mxx[r], cur_len, gi.ext_len, p)) {
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
  if (flagged && lane0 == 0 && eq.h0 + 1 < eq.h1) {
    const uint32_t s = atomicAdd(lists.emu_count, 1u);
    lists.emu_begin[s] = eq.h0;
    lists.emu_end[s] = eq.h1;
    atomicAdd(lists.tally, static_cast<unsigned long long>(eq.h1 - eq.h0));
  }
}

__global__ void __launch_bounds__(kSeBlock, 2) match_emit_kernel(
    MatchEmitArgs a, const uint64_t* __restrict__ dict, const uint32_t* __restrict__ q_ng,
    const uint64_t* __restrict__ q_dbase, const uint64_t* __restrict__ q_goff,
    const uint32_t* __restrict__ q_tie, const QueryInfo* __restrict__ qinfo, ChainParams p,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, GroupInfo* __restrict__ groups,
    MatchEmitLists lists, const uint32_t* qlist, const uint32_t* qcount, uint32_t* counter) {
  static_assert(kSeMaskWords == 2, "two mask words per group");
  extern __shared__ __align__(16) unsigned char emit_raw[];
  EmitSmem& sm = *reinterpret_cast<EmitSmem*>(emit_raw);
  const int t = threadIdx.x;
  constexpr uint32_t kPer = kMatchDictCap / kSeBlock;  // ranks per thread in scans
  const uint32_t nlisted = *qcount;
  for (;;) {
    const uint32_t qi = next_query(counter, &sm.qslot);
    if (qi >= nlisted) return;
    const uint32_t q = qlist[qi];
    const EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q], a.q_off[q + 1]};
    const uint32_t ng = min(q_ng[q], kMatchDictCap);
    const uint64_t dbase = q_dbase[q];
    const bool flagged = q_tie[q] != 0;
    // dictionary -> hash of ext id to rank, and each group's first hit
    for (uint32_t s = t; s < kHashSlots; s += kSeBlock) sm.hkey[s] = kNone;
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
          if (atomicCAS(&sm.hkey[s], kNone, id) == kNone) {
            sm.hrank[s] = static_cast<uint16_t>(r);
            break;
          }
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
    while (w < eq.w1) {
      batch_setup(sm.b, a, eq, w, e0);
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
          if (d >= eq.h0 && d < eq.h1) {  // always: the window's hits lie in the query's range
            keys[d] = (static_cast<uint64_t>(id) << 32) | (sm.b.prev[wl] & 0x7fffffffu);
            vals[d] = pos;
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
    finish_query(a, dict, dbase, ng, q_goff, qinfo, p, keys, groups, lists, q, eq, flagged,
                 sm.cursor, sm.mnx, sm.mxx, t, kSeBlock);
    __syncthreads();
  }
}

// ------------------------------------------------------------ one warp per query
//
// Most queries hit a few hundred targets at most; a warp takes each of them,
// with a dictionary of up to kWarpDictCap ext ids in its own slice of shared
// memory and no block barriers.  The warp visits its query's windows 32 at a
// time: lane l reads window l's table meta, a warp scan numbers their entries,
// and the entries go through in rows of 32 (lane l takes entries l, l + 32,
// ...), kWRows rows' loads in flight at once.  A row's lanes are in entry
// order, so hits of one group within a row are in window order: __match_any
// gives each its rank among them, and the rows go through one after another.

constexpr int kWarpDictCap = 512;
constexpr int kWHashBits = 10;
constexpr uint32_t kWHashSlots = 1u << kWHashBits;  // load 1/2 at kWarpDictCap ids
constexpr int kWWarps = 8;                          // warps per block
constexpr int kWRows = 4;                           // rows of 32 entries in flight
static_assert(kWHashSlots == 2 * kWarpDictCap, "warp hash: twice the dictionary");

__device__ __forceinline__ uint32_t whash_slot(uint32_t id) {
  return (id * 0x9E3779B1u) >> (32 - kWHashBits);
}

// 32 consecutive windows of a query, numbered entries (warp-local): entry j of
// window l is idx.pos[jbase[l] + j], its generation-order slot hbase[l] + j
// (less one past the self hit), and the query's own position when j ==
// self_j[l]; window l's entries end at incl[l].
struct WarpWin {
  uint64_t jbase[32];
  uint64_t hbase[32];
  uint32_t incl[32];
  int32_t self_j[32];
  uint32_t prev[32];  // cur pos | rev << 31
};

// Lane l reads window wg + l; returns the windows' entries.  Writes the
// filtered positions when fpos is given.
__device__ __forceinline__ uint32_t warp_windows(WarpWin& ww, const MatchEmitArgs& a,
                                                 const EmitQuery& eq, uint64_t wg) {
  const int lane = threadIdx.x & 31;
  const uint64_t wi = wg + lane;
  uint32_t raw = 0, self = kNone, prev = 0;
  uint64_t ebase = 0, hoff = 0;
  if (wi < eq.w1) {
    const uint8_t fl = a.wflags[wi];
    if (!(fl & kWinFiltered)) {
      const uint64_t meta = a.wmeta[wi];
      raw = static_cast<uint32_t>((meta >> 40) & ((1ULL << kCountBits) - 1));
      ebase = meta & kOffsetMask;
    } else if (a.fpos) {
      a.fpos[a.filt_off[wi]] = static_cast<int32_t>(wi - eq.w0);
    }
    if (fl & kWinTrivial) self = a.wself[wi];
    hoff = a.hit_off[wi];
    prev = static_cast<uint32_t>(wi - eq.w0) | ((fl & kWinRev) ? 0x80000000u : 0u);
  }
  uint32_t inc = raw;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  const uint32_t excl = inc - raw;
  __syncwarp();  // the previous window group's readers are done
  ww.jbase[lane] = ebase - excl;
  ww.hbase[lane] = hoff - excl;
  ww.incl[lane] = inc;
  ww.self_j[lane] = self == kNone ? INT_MAX : static_cast<int32_t>(excl + self);
  ww.prev[lane] = prev;
  __syncwarp();
  return __shfl_sync(0xffffffffu, inc, 31);
}

// The lane's entries j0, j0 + 32, ... (kWRows rows): windows, then loads.
struct WRow {
  uint64_t sv[kWRows];
  uint32_t j[kWRows];
  uint8_t wl[kWRows];
};

__device__ __forceinline__ void warp_rows(const WarpWin& ww, const MatchEmitArgs& a, uint32_t j0,
                                          uint32_t total, int& wl, WRow& x) {
#pragma unroll
  for (int r = 0; r < kWRows; ++r) {
    const uint32_t j = j0 + 32u * r;
    x.j[r] = j;
    if (j < total) {
      while (ww.incl[wl] <= j) ++wl;  // forward only: j rises
      x.wl[r] = static_cast<uint8_t>(wl);
    }
  }
#pragma unroll
  for (int r = 0; r < kWRows; ++r)
    if (x.j[r] < total) x.sv[r] = __ldg(a.idx.pos + (ww.jbase[x.wl[r]] + x.j[r]));
}

// Row r's entry after the strand transform; false when absent or the query's
// own position.
__device__ __forceinline__ bool wrow_hit(const WarpWin& ww, const MatchEmitArgs& a, const WRow& x,
                                         int r, uint32_t total, uint32_t& id, uint32_t& pos) {
  if (x.j[r] >= total) return false;
  const int wl = x.wl[r];
  id = static_cast<uint32_t>(x.sv[r] >> 32);
  pos = static_cast<uint32_t>(x.sv[r] & 0xffffffffu);
  if (ww.prev[wl] & 0x80000000u) {
    pos = static_cast<uint32_t>(__ldg(a.idx.slot_len + (id >> 1)) - static_cast<int32_t>(pos) -
                                a.idx.k);
    id ^= 1u;
  }
  return static_cast<int32_t>(x.j[r]) != ww.self_j[wl];
}

struct DictWarp {
  uint32_t key[kWHashSlots];
  uint32_t cnt[kWHashSlots];
  uint64_t list[kWarpDictCap];  // the counted ids, (id << 32 | count), then sorted
  WarpWin ww;
  uint32_t nkeys;
};

// Dictionaries of every query (one warp each); a query with more than
// kWarpDictCap ext ids goes to heavy_list for the block kernel.
__global__ void __launch_bounds__(kWWarps * 32, 2) match_dict_warp_kernel(
    MatchEmitArgs a, uint64_t* dict, unsigned long long* dict_cursor, uint32_t* q_ng,
    uint64_t* q_dbase, uint32_t* heavy_list, uint32_t* heavy_count, uint32_t* counter) {
  extern __shared__ __align__(16) unsigned char dw_raw[];
  DictWarp& sm = reinterpret_cast<DictWarp*>(dw_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  uint64_t* list = sm.list;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(counter, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= a.nq) return;
    for (uint32_t s = lane; s < kWHashSlots; s += 32) {
      sm.key[s] = kNone;
      sm.cnt[s] = 0;
    }
    if (lane == 0) sm.nkeys = 0;
    __syncwarp();
    const EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q], a.q_off[q + 1]};
    bool over = false;
    for (uint64_t wg = eq.w0; wg < eq.w1 && !over; wg += 32) {
      const uint32_t total = warp_windows(sm.ww, a, eq, wg);
      int wl = 0;
      for (uint32_t j0 = lane; j0 - lane < total && !over; j0 += 32u * kWRows) {
        WRow x;
        warp_rows(sm.ww, a, j0, total, wl, x);
#pragma unroll
        for (int r = 0; r < kWRows; ++r) {
          uint32_t id, pos;
          if (!wrow_hit(sm.ww, a, x, r, total, id, pos)) continue;
          uint32_t s = whash_slot(id);
          for (uint32_t probe = 0; probe < kWHashSlots; ++probe) {
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
            s = (s + 1) & (kWHashSlots - 1);
          }
        }
        __syncwarp();
        over = sm.nkeys > kWarpDictCap;  // warp-uniform after the sync
      }
    }
    if (over) {
      if (lane == 0) {
        q_ng[q] = 0;
        q_dbase[q] = 0;
        heavy_list[atomicAdd(heavy_count, 1u)] = q;
      }
      __syncwarp();
      continue;
    }
    // compact, sort by ext id, write out
    const uint32_t n = sm.nkeys;
    uint32_t at = 0;
    for (uint32_t s0 = 0; s0 < kWHashSlots; s0 += 32) {
      const uint32_t k = sm.key[s0 + lane];
      const bool keep = k != kNone;
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep)
        list[at + __popc(m & ((1u << lane) - 1u))] = (static_cast<uint64_t>(k) << 32) |
                                                     sm.cnt[s0 + lane];
      at += __popc(m);
    }
    uint32_t n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (uint32_t i = n + lane; i < n2; i += 32) list[i] = ~0ULL;
    __syncwarp();
    for (uint32_t size = 2; size <= n2; size <<= 1) {
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = lane; i < n2 / 2; i += 32) {
          const uint32_t lo = 2 * i - (i & (stride - 1));
          const uint32_t hi = lo + stride;
          const bool up = (lo & size) == 0;
          const uint64_t x0 = list[lo], x1 = list[hi];
          if ((x0 > x1) == up) {
            list[lo] = x1;
            list[hi] = x0;
          }
        }
        __syncwarp();
      }
    }
    unsigned long long base = 0;
    if (lane == 0 && n) base = atomicAdd(dict_cursor, static_cast<unsigned long long>(n));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (lane == 0) {
      q_ng[q] = n;
      q_dbase[q] = base;
    }
    for (uint32_t i = lane; i < n; i += 32) dict[base + i] = list[i];
    __syncwarp();
  }
}

struct EmitWarp {
  uint32_t hkey[kWHashSlots];
  uint16_t hrank[kWHashSlots];
  uint32_t cursor[kWarpDictCap];
  int32_t mnx[kWarpDictCap];
  int32_t mxx[kWarpDictCap];
  WarpWin ww;
};

__device__ __forceinline__ uint32_t wrank_of(const EmitWarp& sm, uint32_t id, DeviceStatus* st) {
  uint32_t s = whash_slot(id);
  for (uint32_t probe = 0; probe < kWHashSlots; ++probe) {
    const uint32_t k = sm.hkey[s];
    if (k == id) return sm.hrank[s];
    if (k == kNone) break;
    s = (s + 1) & (kWHashSlots - 1);
  }
  raise_status(st, kDevMatchDict, 2, id);
  return kNone;
}

// Emission of every query with at most kWarpDictCap groups (one warp each).
__global__ void __launch_bounds__(kWWarps * 32, 2) match_emit_warp_kernel(
    MatchEmitArgs a, const uint64_t* __restrict__ dict, const uint32_t* __restrict__ q_ng,
    const uint64_t* __restrict__ q_dbase, const uint64_t* __restrict__ q_goff,
    const uint32_t* __restrict__ q_tie, const QueryInfo* __restrict__ qinfo, ChainParams p,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, GroupInfo* __restrict__ groups,
    MatchEmitLists lists, uint32_t* counter) {
  extern __shared__ __align__(16) unsigned char ew_raw[];
  EmitWarp& sm = reinterpret_cast<EmitWarp*>(ew_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(counter, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= a.nq) return;
    const uint32_t ng = q_ng[q];
    if (ng > kWarpDictCap) continue;  // the block kernel's
    const EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q], a.q_off[q + 1]};
    const uint64_t dbase = q_dbase[q];
    const bool flagged = q_tie[q] != 0;
    for (uint32_t s = lane; s < kWHashSlots; s += 32) sm.hkey[s] = kNone;
    __syncwarp();
    // ranks, and each group's first slot (warp scan of the counts in rank order)
    uint32_t run = 0;
    for (uint32_t r0 = 0; r0 < ng; r0 += 32) {
      const uint32_t r = r0 + lane;
      uint32_t c = 0;
      if (r < ng) {
        const uint64_t d = dict[dbase + r];
        const uint32_t id = static_cast<uint32_t>(d >> 32);
        c = static_cast<uint32_t>(d);
        uint32_t s = whash_slot(id);
        for (uint32_t probe = 0; probe < kWHashSlots; ++probe) {
          if (atomicCAS(&sm.hkey[s], kNone, id) == kNone) {
            sm.hrank[s] = static_cast<uint16_t>(r);
            break;
          }
          s = (s + 1) & (kWHashSlots - 1);
        }
      }
      uint32_t inc = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
      }
      if (r < ng) {
        sm.cursor[r] = run + inc - c;
        sm.mnx[r] = INT_MAX;
        sm.mxx[r] = INT_MIN;
      }
      run += __shfl_sync(0xffffffffu, inc, 31);
    }
    __syncwarp();
    for (uint64_t wg = eq.w0; wg < eq.w1; wg += 32) {
      const uint32_t total = warp_windows(sm.ww, a, eq, wg);
      int wl = 0;
      for (uint32_t j0 = lane; j0 - lane < total; j0 += 32u * kWRows) {
        WRow x;
        warp_rows(sm.ww, a, j0, total, wl, x);
        if (flagged) {
#pragma unroll
          for (int r = 0; r < kWRows; ++r) {
            uint32_t id, pos;
            if (!wrow_hit(sm.ww, a, x, r, total, id, pos)) continue;
            const int w = x.wl[r];
            const int32_t j = static_cast<int32_t>(x.j[r]);
            const uint64_t d = sm.ww.hbase[w] + static_cast<uint64_t>(j) -
                               (sm.ww.self_j[w] < j ? 1u : 0u);
            if (d >= eq.h0 && d < eq.h1) {  // always: the window's hits lie in the query's range
              keys[d] = (static_cast<uint64_t>(id) << 32) | (sm.ww.prev[w] & 0x7fffffffu);
              vals[d] = pos;
            }
          }
        } else {
#pragma unroll
          for (int r = 0; r < kWRows; ++r) {
            uint32_t id, pos, rk = kNone;
            if (wrow_hit(sm.ww, a, x, r, total, id, pos)) rk = wrank_of(sm, id, a.status);
            // a row's hits of one group come from distinct windows, in lane order
            const unsigned peers = __match_any_sync(0xffffffffu, rk);
            uint32_t slot = 0;
            if (rk != kNone) slot = sm.cursor[rk] + __popc(peers & lt);
            __syncwarp();
            if (rk != kNone) {
              if ((peers >> lane) == 1u) sm.cursor[rk] = slot + 1;  // the group's last in the row
              atomicMin(&sm.mnx[rk], static_cast<int32_t>(pos));
              atomicMax(&sm.mxx[rk], static_cast<int32_t>(pos));
              const uint64_t d = eq.h0 + slot;
              if (d < eq.h1) {  // always, with the dictionary's counts
                keys[d] = (static_cast<uint64_t>(id) << 32) | (sm.ww.prev[x.wl[r]] & 0x7fffffffu);
                vals[d] = pos;
              } else {
                raise_status(a.status, kDevMatchDict, 3, static_cast<int64_t>(q));
              }
            }
            __syncwarp();
          }
        }
      }
    }
    finish_query(a, dict, dbase, ng, q_goff, qinfo, p, keys, groups, lists, q, eq, flagged,
                 sm.cursor, sm.mnx, sm.mxx, lane, 32);
    __syncwarp();
  }
}

}  // namespace

size_t match_dict_smem_bytes() { return sizeof(DictSmem); }
size_t match_emit_smem_bytes() { return sizeof(EmitSmem); }

namespace {
template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(bytes));
  // all of the SM's shared memory for the carve-out, so that more blocks fit
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  return e;
}

template <class K>
int resident_of(K kernel, int threads, size_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return std::max(per_sm, 1);
}
}  // namespace

cudaError_t match_dict(const MatchEmitArgs& a, uint64_t* dict, unsigned long long* dict_cursor,
                       uint32_t* q_ng, uint64_t* q_dbase, uint32_t* overflow,
                       uint32_t* heavy_list, uint32_t* heavy_count, uint32_t* counters,
                       int num_sms, cudaStream_t s) {
  if (a.nq == 0) return cudaSuccess;
  const size_t wsm = kWWarps * sizeof(DictWarp);
  cudaError_t e = allow_smem(match_dict_warp_kernel, wsm);
  if (e == cudaSuccess) e = allow_smem(match_dict_kernel, sizeof(DictSmem));
  if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 2 * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(heavy_count, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  MatchEmitArgs da = a;
  da.fpos = nullptr;  // the filtered positions are match_emit's to write
  const uint64_t wblocks = (a.nq + kWWarps - 1) / kWWarps;
  const unsigned wgrid = static_cast<unsigned>(std::min<uint64_t>(
      static_cast<uint64_t>(resident_of(match_dict_warp_kernel, kWWarps * 32, wsm)) * num_sms,
      wblocks));
  count_launch();
  match_dict_warp_kernel<<<wgrid, kWWarps * 32, wsm, s>>>(da, dict, dict_cursor, q_ng, q_dbase,
                                                          heavy_list, heavy_count, counters);
  // the heavy queries, one block each (the grid idles when there are none)
  const unsigned bgrid = static_cast<unsigned>(std::min<uint64_t>(
      static_cast<uint64_t>(resident_of(match_dict_kernel, kSeBlock, sizeof(DictSmem))) * num_sms,
      a.nq));
  count_launch();
  match_dict_kernel<<<bgrid, kSeBlock, sizeof(DictSmem), s>>>(
      da, dict, dict_cursor, q_ng, q_dbase, overflow, heavy_list, heavy_count, counters + 1);
  return cudaGetLastError();
}

cudaError_t match_emit(const MatchEmitArgs& a, const uint64_t* dict, const uint32_t* q_ng,
                       const uint64_t* q_dbase, const uint64_t* q_goff, const uint32_t* q_tie,
                       const QueryInfo* qinfo, const ChainParams& p, uint64_t* keys,
                       uint32_t* vals, GroupInfo* groups, const MatchEmitLists& lists,
                       const uint32_t* heavy_list, const uint32_t* heavy_count,
                       uint32_t* counters, int num_sms, cudaStream_t s) {
  if (a.nq == 0) return cudaSuccess;
  const size_t wsm = kWWarps * sizeof(EmitWarp);
  cudaError_t e = allow_smem(match_emit_warp_kernel, wsm);
  if (e == cudaSuccess) e = allow_smem(match_emit_kernel, sizeof(EmitSmem));
  if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 2 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const uint64_t wblocks = (a.nq + kWWarps - 1) / kWWarps;
  const unsigned wgrid = static_cast<unsigned>(std::min<uint64_t>(
      static_cast<uint64_t>(resident_of(match_emit_warp_kernel, kWWarps * 32, wsm)) * num_sms,
      wblocks));
  count_launch();
  match_emit_warp_kernel<<<wgrid, kWWarps * 32, wsm, s>>>(a, dict, q_ng, q_dbase, q_goff, q_tie,
                                                          qinfo, p, keys, vals, groups, lists,
                                                          counters);
  const unsigned bgrid = static_cast<unsigned>(std::min<uint64_t>(
      static_cast<uint64_t>(resident_of(match_emit_kernel, kSeBlock, sizeof(EmitSmem))) * num_sms,
      a.nq));
  count_launch();
  match_emit_kernel<<<bgrid, kSeBlock, sizeof(EmitSmem), s>>>(a, dict, q_ng, q_dbase, q_goff,
                                                              q_tie, qinfo, p, keys, vals, groups,
                                                              lists, heavy_list, heavy_count,
                                                              counters + 1);
  return cudaGetLastError();
}

}  // namespace cuflye
