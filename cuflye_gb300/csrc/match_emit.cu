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
//                      of up to 64 windows.  A hit's place in its group is the
//                      group's running count plus the number of earlier windows
//                      of the batch that hit the same ext id (a 64-bit mask per
//                      group), so the batch is staged in shared memory in
//                      group order and leaves in coalesced runs.  Each group's
//                      first and last ext pos and whether its ext positions
//                      rise strictly in cur-pos order are tracked on the way, so
//                      the group's prefilter (survival, spans, overhangs) is
//                      decided here for every group whose ext positions rise;
//                      the others are listed for the prefilter kernel.
//
// A flagged query's hits are written in generation order instead (its equal
// keys need the libstdc++-order sort), and all its groups are listed for the
// prefilter after that sort.  Both kernels visit a window's entries in the
// same order as hits_count / hits_emit: the bucket's stored entries, flipped
// to the other strand when the window's k-mer is not in standard form, less
// the query's own position (its index in the bucket is wself).
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

constexpr int kSeBlock = 512;
constexpr int kSeWarps = kSeBlock / 32;
constexpr uint32_t kSeBatch = 2048;  // bucket entries per batch
constexpr int kSeWin = 64;           // windows per batch (one 64-bit mask bit each)
constexpr uint32_t kSePerThread = kSeBatch / kSeBlock;
constexpr int kHashBits = 12;
constexpr uint32_t kHashSlots = 1u << kHashBits;  // load 1/2 at kMatchDictCap ids
constexpr uint32_t kNone = 0xffffffffu;

static_assert(kSeBatch % kSeBlock == 0, "batch entries per thread");
static_assert(kHashSlots == 2 * kMatchDictCap, "hash slots: twice the dictionary");
static_assert(kMatchDictCap % kSeBlock == 0, "dictionary ranks per thread");
static_assert(kMatchDictCap <= 65536, "ranks fit 16 bits");

// Fibonacci hashing of a dense target id onto the table's slots.
__device__ __forceinline__ uint32_t hash_slot(uint32_t id) {
  return (id * 0x9E3779B1u) >> (32 - kHashBits);
}

// The windows of one batch, in shared memory.
struct BatchWin {
  uint64_t ebase[kSeWin];    // index of the window's first bucket entry in idx.pos
  uint32_t cum[kSeWin + 1];  // batch-local index of each window's first visited entry
  uint32_t first[kSeWin];    // first visited entry of the window (e0 for a split window)
  uint32_t self[kSeWin];     // bucket index of the query's own position, or kNone
  uint32_t p[kSeWin];        // window position in the query (cur pos)
  uint64_t hoff[kSeWin];     // hit offset of the window (generation order)
  uint8_t rev[kSeWin];       // the window's k-mer is not in standard form
  uint32_t nw, total;
  uint64_t next_w;
  uint32_t next_e;
  uint32_t wsum[2];
};

struct EmitQuery {
  uint64_t w0, w1;  // the query's windows [w0, w1) in the pass
  uint64_t h0;      // the query's first hit in the pass
};

// Sets up the batch that starts at window w (entry e0 of it): as many
// windows as fit kSeBatch entries and kSeWin windows, or kSeBatch entries of
// one window that has more.  Writes the filtered positions of the batch's
// windows when fpos is given.  Every thread of the block calls it.
__device__ void batch_setup(BatchWin& b, const MatchEmitArgs& a, const EmitQuery& eq, uint64_t w,
                            uint32_t e0) {
  const int t = threadIdx.x;
  uint32_t raw = 0;
  if (t < kSeWin) {
    const uint64_t wi = w + t;
    uint64_t ebase = 0;
    uint32_t self = kNone;
    uint8_t rev = 0;
    uint64_t hoff = 0;
    if (wi < eq.w1) {
      const uint8_t fl = a.wflags[wi];
      rev = (fl & kWinRev) ? 1 : 0;
      if (!(fl & kWinFiltered)) {
        const uint64_t meta = a.wmeta[wi];
        raw = static_cast<uint32_t>((meta >> 40) & ((1ULL << kCountBits) - 1));
        ebase = meta & kOffsetMask;
      }
      if (fl & kWinTrivial) self = a.wself[wi];
      hoff = a.hit_off[wi];
    }
    const uint32_t f = t == 0 ? e0 : 0u;
    raw -= f;
    b.ebase[t] = ebase;
    b.first[t] = f;
    b.self[t] = self;
    b.rev[t] = rev;
    b.hoff[t] = hoff;
    b.p[t] = static_cast<uint32_t>(wi - eq.w0);
    // inclusive scan of the raw counts over the 64 windows (two warps)
    uint32_t inc = raw;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
      if ((t & 31) >= o) inc += u;
    }
    if ((t & 31) == 31) b.wsum[t >> 5] = inc;
    raw = inc;  // inclusive, warp-local for now
  }
  __syncthreads();
  if (t < kSeWin) {
    const uint32_t inc = raw + (t >= 32 ? b.wsum[0] : 0u);
    b.cum[t + 1] = inc;
    if (t == 0) b.cum[0] = 0;
    raw = inc;
  }
  const int m = __syncthreads_count(t < kSeWin && raw <= kSeBatch);
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
  // filtered positions of the windows this batch covers (each window once:
  // a window that spans batches has entries, so it is not filtered)
  if (a.fpos && t < static_cast<int>(b.nw)) {
    const uint64_t wi = w + t;
    if (wi < eq.w1 && (a.wflags[wi] & kWinFiltered))
      a.fpos[a.filt_off[wi]] = static_cast<int32_t>(wi - eq.w0);
  }
}

// Batch-local window of visited entry j: the last window whose first entry
// is at or before j (windows without entries are skipped that way).
__device__ __forceinline__ int entry_window(const BatchWin& b, uint32_t j) {
  int lo = 0, hi = static_cast<int>(b.nw) - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (b.cum[mid] <= j)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// One visited entry: its target (dense internal id) and position after the
// strand transform, its bucket index, and whether it is a hit (not the
// query's own position).
struct Entry {
  uint32_t id;
  uint32_t pos;
  uint32_t e;
  int wl;
  bool hit;
};

__device__ __forceinline__ Entry load_entry(const BatchWin& b, const MatchEmitArgs& a, uint32_t j) {
  Entry x;
  x.wl = entry_window(b, j);
  x.e = b.first[x.wl] + (j - b.cum[x.wl]);
  const uint64_t sv = __ldg(a.idx.pos + b.ebase[x.wl] + x.e);
  x.id = static_cast<uint32_t>(sv >> 32);
  x.pos = static_cast<uint32_t>(sv & 0xffffffffu);
  if (b.rev[x.wl]) {
    x.pos = static_cast<uint32_t>(__ldg(a.idx.slot_len + (x.id >> 1)) - static_cast<int32_t>(x.pos) -
                                  a.idx.k);
    x.id ^= 1u;
  }
  x.hit = x.e != b.self[x.wl];
  return x;
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
  uint32_t key[kHashSlots];
  uint32_t cnt[kHashSlots];
  uint64_t list[kMatchDictCap];
  BatchWin b;
  unsigned long long dslot;  // the query's first word in dict
  uint32_t nkeys, nlist, qslot;
};

__global__ void __launch_bounds__(kSeBlock) match_dict_kernel(MatchEmitArgs a, uint64_t* dict,
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
    EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q]};
    __syncthreads();
    uint64_t w = eq.w0;
    uint32_t e0 = 0;
    bool over = false;
    while (w < eq.w1 && !over) {
      batch_setup(sm.b, a, eq, w, e0);
      for (uint32_t j = t; j < sm.b.total; j += kSeBlock) {
        const Entry x = load_entry(sm.b, a, j);
        if (!x.hit) continue;
        uint32_t s = hash_slot(x.id);
        for (uint32_t probe = 0; probe < kHashSlots; ++probe) {
          uint32_t k = sm.key[s];
          if (k == kNone) {
            k = atomicCAS(&sm.key[s], kNone, x.id);
            if (k == kNone) {
              atomicAdd(&sm.nkeys, 1u);
              k = x.id;
            }
          }
          if (k == x.id) {
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
    for (uint32_t s = t; s < kHashSlots; s += kSeBlock) {
      if (sm.key[s] != kNone) {
        const uint32_t i = atomicAdd(&sm.nlist, 1u);
        sm.list[i] = (static_cast<uint64_t>(sm.key[s]) << 32) | sm.cnt[s];
      }
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
          const uint64_t x = sm.list[lo], y = sm.list[hi];
          if ((x > y) == up) {
            sm.list[lo] = y;
            sm.list[hi] = x;
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
  uint32_t cursor[kMatchDictCap];  // the group's next hit, relative to the query's first
  uint64_t mask[kMatchDictCap];    // windows of the batch that hit the group
  uint32_t sbase[kMatchDictCap];   // the group's first slot in the staged batch
  uint32_t firstx[kMatchDictCap];  // ext pos of the group's first hit (kNone: none yet)
  uint32_t lastx[kMatchDictCap];   // ext pos of its latest hit
  uint8_t notinc[kMatchDictCap];   // ext positions do not rise strictly in cur-pos order
  uint64_t skey[kSeBatch];         // the batch's hits in group order
  uint32_t sval[kSeBatch];
  uint16_t srank[kSeBatch];
  BatchWin b;
  uint32_t ws[kSeWarps];
  uint32_t qslot, nkept;
};

// Exclusive scan of v over the block's threads (thread order); returns the
// prefix and writes the total to *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* ws, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < kSeWarps; ++w) {
    const uint32_t c = ws[w];
    before += w < warp ? c : 0u;
    all += c;
  }
  __syncthreads();
  *total = all;
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

__global__ void __launch_bounds__(kSeBlock, 2) match_emit_kernel(
    MatchEmitArgs a, const uint64_t* __restrict__ dict, const uint32_t* __restrict__ q_ng,
    const uint64_t* __restrict__ q_dbase, const uint64_t* __restrict__ q_goff,
    const uint32_t* __restrict__ q_tie, const QueryInfo* __restrict__ qinfo, ChainParams p,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, GroupInfo* __restrict__ groups,
    MatchEmitLists lists, uint32_t* counter) {
  extern __shared__ __align__(16) unsigned char emit_raw[];
  EmitSmem& sm = *reinterpret_cast<EmitSmem*>(emit_raw);
  const int t = threadIdx.x;
  constexpr uint32_t kPer = kMatchDictCap / kSeBlock;  // ranks per thread in scans
  for (;;) {
    const uint32_t q = next_query(counter, &sm.qslot);
    if (q >= a.nq) return;
    const EmitQuery eq{a.win_off[q], a.win_off[q + 1], a.q_off[q]};
    const uint64_t h1 = a.q_off[q + 1];
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
    uint32_t all;
    uint32_t run = block_exclusive(sum, sm.ws, &all);
#pragma unroll
    for (uint32_t u = 0; u < kPer; ++u) {
      const uint32_t r = t * kPer + u;
      if (r < ng) {
        sm.cursor[r] = run;
        sm.mask[r] = 0;
        sm.firstx[r] = kNone;
        sm.lastx[r] = kNone;
        sm.notinc[r] = 0;
      }
      run += c[u];
    }
    __syncthreads();
    uint64_t w = eq.w0;
    uint32_t e0 = 0;
    while (w < eq.w1) {
      batch_setup(sm.b, a, eq, w, e0);
      const uint32_t total = sm.b.total;
      if (flagged) {
        // generation order: the window's hit offset plus the entry's index
        // among the window's hits
        for (uint32_t j = t; j < total; j += kSeBlock) {
          const Entry x = load_entry(sm.b, a, j);
          if (!x.hit) continue;
          const uint32_t self = sm.b.self[x.wl];
          const uint64_t d = sm.b.hoff[x.wl] + x.e - (self != kNone && self < x.e ? 1u : 0u);
          if (d < h1) {  // always: the window's hits lie in the query's range
            keys[d] = (static_cast<uint64_t>(x.id) << 32) | sm.b.p[x.wl];
            vals[d] = x.pos;
          }
        }
      } else {
        uint32_t rk[kSePerThread], ps[kSePerThread], id[kSePerThread];
        int wl[kSePerThread];
#pragma unroll
        for (uint32_t u = 0; u < kSePerThread; ++u) {
          const uint32_t j = t + u * kSeBlock;
          rk[u] = kNone;
          if (j < total) {
            const Entry x = load_entry(sm.b, a, j);
            if (x.hit) {
              rk[u] = rank_of(sm, x.id, a.status);
              ps[u] = x.pos;
              id[u] = x.id;
              wl[u] = x.wl;
              if (rk[u] != kNone)
                atomicOr(reinterpret_cast<unsigned long long*>(&sm.mask[rk[u]]), 1ULL << x.wl);
            }
          }
        }
        __syncthreads();
        // staging slots: groups in rank order, windows in order within a group
        uint32_t cc[kPer], csum = 0;
#pragma unroll
        for (uint32_t u = 0; u < kPer; ++u) {
          const uint32_t r = t * kPer + u;
          cc[u] = r < ng ? static_cast<uint32_t>(__popcll(sm.mask[r])) : 0u;
          csum += cc[u];
        }
        uint32_t kept;
        uint32_t sb = block_exclusive(csum, sm.ws, &kept);
#pragma unroll
        for (uint32_t u = 0; u < kPer; ++u) {
          const uint32_t r = t * kPer + u;
          if (r < ng) sm.sbase[r] = sb;
          sb += cc[u];
        }
        __syncthreads();
#pragma unroll
        for (uint32_t u = 0; u < kSePerThread; ++u) {
          if (rk[u] != kNone) {
            const uint32_t r = rk[u];
            const uint32_t slot =
                sm.sbase[r] + static_cast<uint32_t>(__popcll(sm.mask[r] & ((1ULL << wl[u]) - 1)));
            sm.skey[slot] = (static_cast<uint64_t>(id[u]) << 32) | sm.b.p[wl[u]];
            sm.sval[slot] = ps[u];
            sm.srank[slot] = static_cast<uint16_t>(r);
          }
        }
        __syncthreads();
        // out in group runs; each hit's ext pos against its group predecessor
        for (uint32_t j = t; j < kept; j += kSeBlock) {
          const uint32_t r = sm.srank[j];
          const uint32_t x = sm.sval[j];
          const uint32_t local = j - sm.sbase[r];
          const uint64_t d = eq.h0 + sm.cursor[r] + local;
          if (d < h1) {  // always, with the dictionary's counts
            keys[d] = sm.skey[j];
            vals[d] = x;
          } else {
            raise_status(a.status, kDevMatchDict, 1, static_cast<int64_t>(q));
          }
          const uint32_t prev = local ? sm.sval[j - 1] : sm.lastx[r];
          if ((local || sm.firstx[r] != kNone) && x <= prev) sm.notinc[r] = 1;
        }
        __syncthreads();
#pragma unroll
        for (uint32_t u = 0; u < kPer; ++u) {
          const uint32_t r = t * kPer + u;
          if (r < ng && cc[u]) {
            const uint32_t sbr = sm.sbase[r];
            if (sm.firstx[r] == kNone) sm.firstx[r] = sm.sval[sbr];
            sm.lastx[r] = sm.sval[sbr + cc[u] - 1];
            sm.cursor[r] += cc[u];
            sm.mask[r] = 0;
          }
        }
      }
      w = sm.b.next_w;
      e0 = sm.b.next_e;
      __syncthreads();
    }
    // the query's groups: GroupInfo, and the prefilter where the group's ext
    // positions rose strictly (first and last ext pos are its extremes)
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
      const uint64_t g = g0 + r;
      if (!flagged && !sm.notinc[r]) {
        const int32_t min_cur = static_cast<int32_t>(keys[gi.start] & 0xffffffffu);
        const int32_t max_cur = static_cast<int32_t>(keys[gi.start + n - 1] & 0xffffffffu);
        const uint32_t uniq = n - (min_cur == 0 ? 1u : 0u);
        const bool ok = prefilter_keeps(uniq, min_cur, max_cur, static_cast<int32_t>(sm.firstx[r]),
                                        static_cast<int32_t>(sm.lastx[r]), cur_len, gi.ext_len, p);
        if (ok) {
          gi.survive = 1;
          gi.ext_sorted = gi.ext_len > cur_len ? 2 : 0;  // already in ext-pos order
          lists.dp_list[atomicAdd(lists.counts + 1, 1u)] = static_cast<uint32_t>(g);
        }
      } else {
        lists.pf_list[atomicAdd(lists.counts + 2, 1u)] = static_cast<uint32_t>(g);
        atomicAdd(lists.tally + 1, static_cast<unsigned long long>(n));
      }
      groups[g] = gi;
    }
    if (flagged && t == 0 && eq.h0 + 1 < a.q_off[q + 1]) {
      const uint32_t s = atomicAdd(lists.emu_count, 1u);
      lists.emu_begin[s] = eq.h0;
      lists.emu_end[s] = a.q_off[q + 1];
      atomicAdd(lists.tally, static_cast<unsigned long long>(a.q_off[q + 1] - eq.h0));
    }
    __syncthreads();
  }
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
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, match_dict_kernel, kSeBlock,
                                                    sizeof(DictSmem));
  if (e != cudaSuccess) return e;
  const unsigned grid = static_cast<unsigned>(
      std::min<uint64_t>(static_cast<uint64_t>(std::max(per_sm, 1)) * num_sms, a.nq));
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
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, match_emit_kernel, kSeBlock,
                                                    sizeof(EmitSmem));
  if (e != cudaSuccess) return e;
  const unsigned grid = static_cast<unsigned>(
      std::min<uint64_t>(static_cast<uint64_t>(std::max(per_sm, 1)) * num_sms, a.nq));
  count_launch();
  match_emit_kernel<<<grid, kSeBlock, sizeof(EmitSmem), s>>>(a, dict, q_ng, q_dbase, q_goff, q_tie,
                                                             qinfo, p, keys, vals, groups, lists,
                                                             counter);
  return cudaGetLastError();
}

}  // namespace cuflye
