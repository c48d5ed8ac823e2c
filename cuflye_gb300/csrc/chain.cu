// chain.cu — per-target chaining of sorted KmerMatches (getSeqOverlaps after
// the candidate loop), following tools/replay_overlap_chains.py:228-422 and
// cuda/cuflye_cuda_overlap_chain_replay.cu:977-1015, 1493-1719.
//
// A group is a run of equal ext ids inside one query's sorted matches.
//   groups_*       : group bounds, the survival / span / overhang prefilter,
//                    and which ext-sorted groups are already in ext order;
//   chain_dp       : the DP over the sorted pairs, one warp per group (see
//                    dp_kernel);
//   chain_backtrack: score-ordered backtrack (starts picked by score, or the
//                    libstdc++-order sort of the scores), overlapTest, k-mer
//                    divergence, proposal sort, primary selection and the
//                    divergence filter, one warp per group;
//   rows_*         : max_overlaps cutoff per query and order-preserving
//                    compaction of the rows.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "introsort.cuh"
#include "kernels.h"

namespace cuflye {
namespace {

inline unsigned grid(uint64_t n, int b) {
  return static_cast<unsigned>((n + b - 1) / b > 0 ? (n + b - 1) / b : 1);
}

__device__ __forceinline__ uint32_t upper_query(const uint64_t* __restrict__ q_off, uint32_t nq,
                                                uint64_t i) {
  // query q with q_off[q] <= i < q_off[q + 1]
  uint32_t lo = 0, hi = nq - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (q_off[mid] <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// A tile's hits are visited in kGroupTile / kGroupBlock rounds of
// consecutive hits (coalesced); a group starts where the ext id changes or a
// query starts (the tile's query starts are marked in a bitmap first).
constexpr int kGroupBlock = 256;
constexpr int kGroupRounds = static_cast<int>(kGroupTile / kGroupBlock);

template <bool WRITE>
__global__ void __launch_bounds__(kGroupBlock) group_tiles_kernel(
    const uint64_t* __restrict__ keys, const uint64_t* __restrict__ q_off, uint32_t nq,
    uint64_t n, uint32_t* __restrict__ tile_counts, const uint64_t* __restrict__ tile_off,
    GroupInfo* __restrict__ groups) {
  __shared__ uint32_t qbits[kGroupTile / 32];
  __shared__ uint32_t wsum[kGroupBlock / 32];
  __shared__ uint32_t qfirst;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t t0 = static_cast<uint64_t>(blockIdx.x) * kGroupTile;
  const uint32_t tn = static_cast<uint32_t>(n - t0 < kGroupTile ? n - t0 : kGroupTile);
  for (uint32_t w = threadIdx.x; w < kGroupTile / 32; w += kGroupBlock) qbits[w] = 0;
  if (threadIdx.x == 0) {
    // first query starting at or after t0
    uint32_t lo = 0, hi = nq;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (q_off[mid] < t0)
        lo = mid + 1;
      else
        hi = mid;
    }
    qfirst = lo;
  }
  __syncthreads();
  for (uint32_t q = qfirst + threadIdx.x; q < nq && q_off[q] < t0 + tn; q += kGroupBlock) {
    const uint32_t j = static_cast<uint32_t>(q_off[q] - t0);
    atomicOr(&qbits[j >> 5], 1u << (j & 31));
  }
  __syncthreads();
  // counting: every round's ext ids (and their predecessors') in flight
  // before any use; writing: one round at a time (fewer registers)
  uint32_t ex[kGroupRounds], pe[kGroupRounds];
  if (!WRITE) {
#pragma unroll
    for (int r = 0; r < kGroupRounds; ++r) {
      const uint32_t j = static_cast<uint32_t>(r) * kGroupBlock + threadIdx.x;
      const uint64_t i = t0 + j;
      ex[r] = j < tn ? static_cast<uint32_t>(keys[i] >> 32) : 0u;
      pe[r] = j < tn && i > 0 ? static_cast<uint32_t>(keys[i - 1] >> 32) : 0u;
    }
  }
  uint64_t g = WRITE ? tile_off[blockIdx.x] : 0;
  uint32_t total = 0;
#pragma unroll
  for (int r = 0; r < kGroupRounds; ++r) {
    const uint32_t j = static_cast<uint32_t>(r) * kGroupBlock + threadIdx.x;
    const uint64_t i = t0 + j;
    uint32_t e, prev;
    if (!WRITE) {
      e = ex[r];
      prev = pe[r];
    } else {
      e = j < tn ? static_cast<uint32_t>(keys[i] >> 32) : 0u;
      prev = j < tn && i > 0 ? static_cast<uint32_t>(keys[i - 1] >> 32) : 0u;
    }
    const bool start =
        j < tn && (i == 0 || ((qbits[j >> 5] >> (j & 31)) & 1u) || e != prev);
    if (!WRITE) {
      total += start;
      continue;
    }
    const unsigned m = __ballot_sync(0xffffffffu, start);
    if (lane == 0) wsum[warp] = __popc(m);
    __syncthreads();
    uint32_t before = 0, round_total = 0;
    for (int w = 0; w < kGroupBlock / 32; ++w) {
      const uint32_t c = wsum[w];
      if (w < warp) before += c;
      round_total += c;
    }
    if (start) {
      GroupInfo gi{};
      gi.start = i;
      gi.ext_di = e;
      gi.query = upper_query(q_off, nq, i);
      groups[g + before + __popc(m & ((1u << lane) - 1u))] = gi;
    }
    g += round_total;
    __syncthreads();
  }
  if (!WRITE) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
    if (lane == 0) wsum[warp] = total;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int w = 0; w < kGroupBlock / 32; ++w) t += wsum[w];
      tile_counts[blockIdx.x] = t;
    }
  }
}

// The prefilter of one group by one warp: unique query positions (changes
// of curPos, starting from prevPos = 0), the ext-pos extremes, then
// prefilter_keeps.  Writes n, ext_len, ext_sorted and survive into gi.
__device__ __forceinline__ bool prefilter_group(const uint64_t* __restrict__ keys,
                                                const uint32_t* __restrict__ vals, GroupInfo& gi,
                                                uint32_t n, const QueryInfo* __restrict__ qinfo,
                                                const int32_t* __restrict__ slot_len,
                                                const ChainParams& p) {
  const int lane = threadIdx.x & 31;
  uint32_t uniq = 0;
  int32_t mn = INT_MAX, mx = INT_MIN;
  // four rounds of loads in flight per lane
  for (uint32_t j0 = lane; j0 < n; j0 += 4 * 32) {
    int32_t c[4], pc[4], e[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t j = j0 + 32 * u;
      const uint64_t i = gi.start + j;
      const bool ok = j < n;
      c[u] = ok ? static_cast<int32_t>(keys[i] & 0xffffffffu) : 0;
      pc[u] = ok && j > 0 ? static_cast<int32_t>(keys[i - 1] & 0xffffffffu) : 0;
      e[u] = ok ? static_cast<int32_t>(vals[i]) : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (j0 + 32 * u < n) {
        uniq += c[u] != pc[u];
        mn = min(mn, e[u]);
        mx = max(mx, e[u]);
      }
    }
  }
  for (int d = 16; d > 0; d >>= 1) {
    uniq += __shfl_down_sync(0xffffffffu, uniq, d);
    mn = min(mn, __shfl_down_sync(0xffffffffu, mn, d));
    mx = max(mx, __shfl_down_sync(0xffffffffu, mx, d));
  }
  if (lane != 0) return false;
  const int32_t cur_len = qinfo[gi.query].len;
  const int32_t ext_len = slot_len[gi.ext_di >> 1];
  const int32_t min_cur = static_cast<int32_t>(keys[gi.start] & 0xffffffffu);
  const int32_t max_cur = static_cast<int32_t>(keys[gi.start + n - 1] & 0xffffffffu);
  gi.n = n;
  gi.ext_len = ext_len;
  gi.ext_sorted = ext_len > cur_len;
  const bool ok = prefilter_keeps(uniq, min_cur, max_cur, mn, mx, cur_len, ext_len, p);
  gi.survive = ok;
  return ok;
}

__global__ void prefilter_kernel(const uint64_t* __restrict__ keys,
                                 const uint32_t* __restrict__ vals, GroupInfo* __restrict__ groups,
                                 uint64_t ngroups, uint64_t nhits,
                                 const QueryInfo* __restrict__ qinfo,
                                 const int32_t* __restrict__ slot_len, ChainParams p,
                                 uint32_t* __restrict__ ext_list, uint32_t* __restrict__ dp_list,
                                 uint32_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const uint64_t g = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (g >= ngroups) return;
  GroupInfo gi = groups[g];
  const uint64_t end = g + 1 < ngroups ? groups[g + 1].start : nhits;
  const bool ok = prefilter_group(keys, vals, gi, static_cast<uint32_t>(end - gi.start), qinfo,
                                  slot_len, p);
  if (lane != 0) return;
  groups[g] = gi;
  if (ok) {
    dp_list[atomicAdd(&counts[1], 1u)] = static_cast<uint32_t>(g);
    if (gi.ext_sorted) ext_list[atomicAdd(&counts[0], 1u)] = static_cast<uint32_t>(g);
  }
}

// The same over a list of groups whose GroupInfo already holds start and n.
__global__ void prefilter_list_kernel(const uint64_t* __restrict__ keys,
                                      const uint32_t* __restrict__ vals,
                                      GroupInfo* __restrict__ groups,
                                      const uint32_t* __restrict__ list,
                                      const QueryInfo* __restrict__ qinfo,
                                      const int32_t* __restrict__ slot_len, ChainParams p,
                                      uint32_t* __restrict__ ext_list,
                                      uint32_t* __restrict__ dp_list,
                                      uint32_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const uint32_t cnt = counts[2];
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < cnt; li += nwarps) {
    const uint32_t g = list[li];
    GroupInfo gi = groups[g];
    const bool ok = prefilter_group(keys, vals, gi, gi.n, qinfo, slot_len, p);
    if (lane == 0) {
      groups[g] = gi;
      if (ok) {
        dp_list[atomicAdd(&counts[1], 1u)] = g;
        if (gi.ext_sorted) ext_list[atomicAdd(&counts[0], 1u)] = g;
      }
    }
  }
}

__global__ void prepare_ext_sort_kernel(uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                        const GroupInfo* __restrict__ groups,
                                        const uint32_t* __restrict__ ext_list,
                                        const uint32_t* __restrict__ counts,
                                        uint64_t* __restrict__ sb, uint64_t* __restrict__ se) {
  const uint32_t cnt = counts[0];
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < cnt; li += nwarps) {
    const GroupInfo g = groups[ext_list[li]];
    for (uint32_t j = lane; j < g.n; j += 32) {
      const uint64_t i = g.start + j;
      const uint64_t k = keys[i];
      keys[i] = static_cast<uint64_t>(vals[i]);
      vals[i] = static_cast<uint32_t>(k & 0xffffffffu);
    }
    if (lane == 0) {
      sb[li] = g.start;
      se[li] = g.start + g.n;
    }
  }
}

// An ext-sorted group whose ext positions already increase strictly in
// cur-pos order is in its only ext-pos order: it is marked ext_sorted = 2 and
// read in place; the others are listed for the re-sort.
__global__ void ext_presorted_kernel(const uint32_t* __restrict__ vals,
                                     GroupInfo* __restrict__ groups,
                                     const uint32_t* __restrict__ ext_list,
                                     const uint32_t* __restrict__ counts,
                                     uint32_t* __restrict__ out, uint32_t* __restrict__ out_count) {
  const uint32_t cnt = counts[0];
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < cnt; li += nwarps) {
    const uint32_t gid = ext_list[li];
    const GroupInfo g = groups[gid];
    bool up = true;
    for (uint32_t j0 = lane + 1; j0 < g.n && up; j0 += 4 * 32) {
      uint32_t a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t j = j0 + 32 * u;
        a[u] = j < g.n ? vals[g.start + j] : 1u;
        b[u] = j < g.n ? vals[g.start + j - 1] : 0u;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) up &= a[u] > b[u];
    }
    up = __all_sync(0xffffffffu, up);
    if (lane == 0) {
      if (up)
        groups[gid].ext_sorted = 2;
      else
        out[atomicAdd(out_count, 1u)] = gid;
    }
  }
}

// ---------------------------------------------------------------- DP
//
// Flye's DP visits predecessors j = i-1, i-2, ... and keeps the first j (in
// visit order) that strictly beats the running maximum, which starts at 0; it
// stops right after an update with jumpDiv == 0 && curDelta < k, and right
// after the first j whose sort-axis delta exceeds maxJump.  A warp evaluates
// 32 predecessors at once (lane L <-> j = i-1-32c-L): an inclusive prefix
// max over lanes gives each lane the running maximum before it, a ballot
// finds the first lane that ends the scan, and the winner is the first lane
// at or before it that attains the maximum (later equal scores do not update).
//
// Most elements end the scan at j = i-1: it updates (its score is at least 0,
// and the match adds at least 1) and breaks when 0 < curDelta = extDelta < k
// (both under maxJump).  That test needs positions only, so the warp marks
// such "step" elements for 32 elements at once.  Along a run of steps the
// score is a prefix sum: S[i] = max(S[i-1] + curDelta, k), which is
// S[i-1] + curDelta whenever S[i-1] >= k (every element but the first has
// S >= k), and the link is i-1 whenever that sum exceeds k.  The warp scores
// each run with one prefix sum over lanes and scans predecessors only for the
// other elements.

constexpr int kDpWarps = 8;

__device__ __forceinline__ void eval_chunk(bool valid, int32_t cj, int32_t ej, int32_t sj,
                                           int32_t j, int32_t ci, int32_t ei, bool es,
                                           const ChainParams& p, int32_t& best, int32_t& bestj,
                                           bool& done) {
  const int lane = threadIdx.x & 31;
  const int32_t cd = ci - cj, ed = ei - ej;
  const int32_t jd = abs(cd - ed);
  const bool acc = valid && cd > 0 && cd < p.max_jump && ed > 0 && ed < p.max_jump &&
                   jd <= p.max_gap;
  int32_t sc = INT_MIN;
  if (acc) {
    const int32_t ms = min(min(cd, ed), p.k);
    const float pen = jd > p.gap_jump_threshold ? p.large_gap_penalty : p.small_gap_penalty;
    const int32_t gc = __float2int_rz(__fmul_rn(pen, static_cast<float>(jd)));
    sc = sj + ms - gc;
  }
  const bool stop = !valid || (es ? ed > p.max_jump : cd > p.max_jump);
  if (__ballot_sync(0xffffffffu, acc) == 0) {  // no candidate: only a stop matters
    done = __ballot_sync(0xffffffffu, stop) != 0;
    return;
  }
  int32_t incl = sc;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl = max(incl, o);
  }
  int32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) excl = INT_MIN;
  const bool upd = acc && sc > max(best, excl);
  const bool brk = (upd && jd == 0 && cd < p.k) || stop;
  const unsigned bm = __ballot_sync(0xffffffffu, brk);
  const int bl = bm ? __ffs(bm) - 1 : 31;
  const int32_t nb = max(best, __shfl_sync(0xffffffffu, incl, bl));
  if (nb > best) {
    const unsigned um = __ballot_sync(0xffffffffu, upd && lane <= bl && sc == nb);
    bestj = __shfl_sync(0xffffffffu, j, __ffs(um) - 1);
    best = nb;
  }
  done = bm != 0;
}

// Warps take groups from a shared counter (groups differ a lot in length).
__device__ __forceinline__ uint32_t next_item(uint32_t* counter) {
  uint32_t v = 0;
  if ((threadIdx.x & 31) == 0) v = atomicAdd(counter, 1u);
  return __shfl_sync(0xffffffffu, v, 0);
}

// Positions of match i of a group: the sorted pairs hold key = (ext id << 32)
// | cur pos, val = ext pos, or key = ext pos, val = cur pos in groups
// re-sorted by ext pos (swapped).
__device__ __forceinline__ void load_match(const uint64_t* __restrict__ keys,
                                           const uint32_t* __restrict__ vals, bool swapped,
                                           uint64_t i, int32_t& c, int32_t& e) {
  const uint32_t lo = static_cast<uint32_t>(__ldg(keys + i));
  const uint32_t v = __ldg(vals + i);
  c = static_cast<int32_t>(swapped ? v : lo);
  e = static_cast<int32_t>(swapped ? lo : v);
}

__global__ void __launch_bounds__(kDpWarps * 32, 8) dp_kernel(
    const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, int32_t* score,
    int32_t* bt, const GroupInfo* __restrict__ groups, const uint32_t* __restrict__ list,
    const uint32_t* __restrict__ counts, ChainParams p, GroupTop* __restrict__ top,
    int32_t* pmc, uint32_t* __restrict__ work) {
  const int lane = threadIdx.x & 31;
  const uint32_t cnt = counts[1];
  for (uint32_t li = next_item(work); li < cnt; li = next_item(work)) {
    const uint32_t gidx = list[li];
    const GroupInfo g = groups[gidx];
    // this lane's highest score, its first element and how many elements have it
    int32_t top_s = INT_MIN;
    uint32_t top_i = 0, top_c = 0;
    const uint64_t b = g.start;
    const uint32_t n = g.n;
    const bool es = g.ext_sorted != 0;
    const bool swapped = g.ext_sorted == 1;
    int32_t s_prev = 0;        // score of the element before the next one to score
    int32_t pc = 0, pe = 0;    // positions of the element before this chunk
    // Highest score so far, and per 32-element chunk t of the group the
    // highest score over elements [0, 32t + 31] in pmc[pbase + t].  A
    // predecessor j scores at most S[j] + k, so a scan stops once that bound
    // over every j still to visit cannot beat the best found.
    int32_t run_max = 0;
    const uint64_t pbase = (b >> 5) + gidx;
    for (uint32_t i0 = 0; i0 < n; i0 += 32) {
      const uint32_t i = i0 + lane;
      const uint32_t len = min(32u, n - i0);
      int32_t ci = 0, ei = 0;
      if (i < n) load_match(keys, vals, swapped, b + i, ci, ei);
      int32_t cp = __shfl_up_sync(0xffffffffu, ci, 1);
      int32_t ep = __shfl_up_sync(0xffffffffu, ei, 1);
      if (lane == 0) {
        cp = pc;
        ep = pe;
      }
      const int32_t cd = ci - cp, ed = ei - ep;
      const bool step = i < n && i > 0 && cd > 0 && cd < p.max_jump && cd == ed && cd < p.k;
      const unsigned smask = __ballot_sync(0xffffffffu, step);
      int32_t s_mine = 0;
      uint32_t t = 0;
      if (i0 == 0) {
        if (lane == 0) {
          score[b] = 0;
          bt[b] = -1;
          top_s = 0;
          top_i = 0;
          top_c = 1;
        }
        t = 1;
      }
      while (t < len) {
        // run of step elements [t, u)
        const unsigned rest = ~smask & (0xffffffffu << t);
        const uint32_t u = min(rest ? static_cast<uint32_t>(__ffs(rest) - 1) : 32u, len);
        if (u > t) {
          const bool in = lane >= static_cast<int>(t) && lane < static_cast<int>(u);
          int32_t x = in ? cd : 0;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
          }
          const int32_t dt = __shfl_sync(0xffffffffu, cd, t);
          const int32_t first = max(s_prev + dt, p.k);
          if (in) {
            s_mine = first + (x - dt);
            score[b + i] = s_mine;
            if (s_mine > top_s) {
              top_s = s_mine;
              top_i = i;
              top_c = 1;
            } else if (s_mine == top_s) {
              ++top_c;
            }
            bt[b + i] = (lane > static_cast<int>(t) || s_prev + dt > p.k)
                            ? static_cast<int32_t>(i) - 1
                            : -1;
          }
          s_prev = __shfl_sync(0xffffffffu, s_mine, u - 1);
          run_max = max(run_max, s_prev);  // scores rise along a run
          t = u;
        }
        if (t < len) {
          // predecessor scan for element i0 + t
          __syncwarp();
          const int32_t cit = __shfl_sync(0xffffffffu, ci, t);
          const int32_t eit = __shfl_sync(0xffffffffu, ei, t);
          const int32_t it = static_cast<int32_t>(i0 + t);
          int32_t best = 0, bestj = 0;
          bool done = false;
          for (int32_t c0 = it - 1; !done && c0 >= 0; c0 -= 32) {
            const int32_t bound =
                c0 >= static_cast<int32_t>(i0) ? run_max : __ldcg(pmc + pbase + (c0 >> 5));
            if (bound + p.k <= best) break;
            const int32_t j = c0 - lane;
            const bool valid = j >= 0;
            int32_t cj = 0, ej = 0, sj = 0;
            if (valid) {
              load_match(keys, vals, swapped, b + j, cj, ej);
              sj = __ldcg(score + b + j);
            }
            eval_chunk(valid, cj, ej, sj, j, cit, eit, es, p, best, bestj, done);
          }
          const int32_t si = max(best, p.k);
          if (lane == static_cast<int>(t)) {
            s_mine = si;
            score[b + it] = si;
            bt[b + it] = best > p.k ? bestj : -1;
            if (si > top_s) {
              top_s = si;
              top_i = static_cast<uint32_t>(it);
              top_c = 1;
            } else if (si == top_s) {
              ++top_c;
            }
          }
          s_prev = si;
          run_max = max(run_max, si);
          ++t;
        }
        __syncwarp();
      }
      if (lane == 0) pmc[pbase + (i0 >> 5)] = run_max;
      __syncwarp();
      pc = __shfl_sync(0xffffffffu, ci, 31);
      pe = __shfl_sync(0xffffffffu, ei, 31);
    }
    int32_t ms = top_s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ms = max(ms, __shfl_xor_sync(0xffffffffu, ms, o));
    uint32_t mc = top_s == ms ? top_c : 0u;
    uint32_t mi = top_s == ms ? top_i : 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mc += __shfl_xor_sync(0xffffffffu, mc, o);
      mi = min(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    }
    if (lane == 0) top[gidx] = GroupTop{ms, mi, mc, 0u};
  }
}

__global__ void prepare_order_kernel(const int32_t* __restrict__ score, uint64_t* __restrict__ keys,
                                     uint32_t* __restrict__ vals,
                                     const GroupInfo* __restrict__ groups,
                                     const uint32_t* __restrict__ dp_list,
                                     const uint32_t* __restrict__ list_count,
                                     uint64_t* __restrict__ sb, uint64_t* __restrict__ se) {
  const uint32_t cnt = *list_count;
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < cnt; li += nwarps) {
    const GroupInfo g = groups[dp_list[li]];
    for (uint32_t j = lane; j < g.n; j += 32) {
      const uint64_t i = g.start + j;
      keys[i] = static_cast<uint64_t>(static_cast<uint32_t>(INT_MAX - score[i]));
      vals[i] = j;
    }
    if (lane == 0) {
      sb[li] = g.start;
      se[li] = g.start + g.n;
    }
  }
}

// ---------------------------------------------------------------- backtrack

constexpr int kMaxProposals = 64;

struct Prop {
  int32_t cb, ce, eb, ee, score, clen;
  float div;
};

__device__ __forceinline__ bool overlap_test(const Prop& o, int64_t cur_id, int64_t ext_id,
                                             int32_t cur_len, int32_t ext_len,
                                             const ChainParams& p) {
  const int32_t cr = o.ce - o.cb, er = o.ee - o.eb;
  if (cr < p.min_overlap || er < p.min_overlap) return false;
  const int32_t diff = abs(cr - er);
  if (static_cast<float>(diff) > fmul(0.5f, static_cast<float>(min(cr, er)))) return false;
  if (cur_id == ext_id) {
    const int32_t inter = min(o.ce, o.ee) - max(o.cb, o.eb);
    if (static_cast<float>(inter) > fdiv(static_cast<float>(cr), 2.0f)) return false;
  }
  if (cur_id == -ext_id) {
    const int32_t inter = min(o.ce, ext_len - o.eb) - max(o.cb, ext_len - o.ee);
    if (static_cast<float>(inter) > fdiv(static_cast<float>(cr), 2.0f)) return false;
  }
  if (!p.force_local && p.check_overhang) {
    const int32_t lr = max(min(o.cb, o.eb), min(cur_len - o.ce, ext_len - o.ee));
    if (lr > p.max_overhang) return false;
  }
  return true;
}

__device__ __forceinline__ uint32_t lower_bound_i32(const int32_t* a, uint32_t n, int32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Flye walks chains in score order: from each start whose backtrack entry is
// still set it follows the links, clearing every entry it visits, and the
// chain ends at the first node whose entry is -1 (never linked, or cleared
// by an earlier walk).  One warp per group keeps three bitmaps in place of
// the table: linked (entry != -1 at the start), step (entry == i - 1) and
// cleared; in shared memory for groups of up to kBtCap elements, else in
// device memory.  A walk crosses a run of step links in one 32-word search
// per 1,024 nodes (the next node that is not a step or is cleared) and
// clears the run word by word; only links that are not steps are read from
// the table, which stays unchanged.  The warp counts linked nodes not yet
// cleared and stops when none is left: no later start could begin a chain.
// A fourth map marks the nodes cleared while several starts share the top
// score (a tie round), to tell whether their walks touch one another.

constexpr uint32_t kBtCap = kBacktrackCap;
constexpr uint32_t kBtWords = kBtCap / 32;
constexpr int kBtWarps = 8;

struct BtMaps {
  uint32_t link[kBtWords];
  uint32_t step[kBtWords];
  uint32_t done[kBtWords];
  uint32_t round[kBtWords];
};

__device__ __forceinline__ uint32_t bits_upto(int32_t pos) {
  const int r = pos & 31;
  return r == 31 ? 0xffffffffu : ((2u << r) - 1u);
}

__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Walk from s0 (linked, not cleared) with the whole warp: first node and
// chain length as Flye's walk counts them; visited nodes become cleared and
// `remaining` drops by the linked ones among them.  With `round`, visited
// nodes are marked there too, and `met` tells whether the walk ended on a
// linked node marked earlier.
__device__ void walk_maps(const uint32_t* link, const uint32_t* step, uint32_t* done,
                          const int32_t* __restrict__ btg, int32_t s0, int32_t& first,
                          int32_t& clen, uint32_t& remaining, uint32_t* round, bool& met) {
  const int lane = threadIdx.x & 31;
  int32_t pos = s0;
  clen = 0;
  for (;;) {
    // z: the highest node <= pos that is not an uncleared step
    int32_t z = -1;
    for (int32_t w0 = pos >> 5; z < 0; w0 -= 32) {
      const int32_t w = w0 - lane;
      uint32_t bits = 0;
      if (w >= 0) {
        bits = ~step[w] | done[w];
        if (w == (pos >> 5)) bits &= bits_upto(pos);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, bits != 0);
      if (bal) {
        const int l = __ffs(bal) - 1;
        const uint32_t wb = __shfl_sync(0xffffffffu, bits, l);
        z = (w0 - l) * 32 + 31 - __clz(wb);
      }
    }
    const bool stop = ((done[z >> 5] >> (z & 31)) & 1u) || !((link[z >> 5] >> (z & 31)) & 1u);
    // an unlinked node ends every walk that reaches it, whichever comes first
    if (round && stop) met = ((round[z >> 5] & link[z >> 5]) >> (z & 31)) & 1u;
    __syncwarp();
    uint32_t newly = 0;
    for (int32_t w = (z >> 5) + lane; w <= (pos >> 5); w += 32) {
      uint32_t mask = 0xffffffffu;
      if (w == (z >> 5)) mask &= 0xffffffffu << (z & 31);
      if (w == (pos >> 5)) mask &= bits_upto(pos);
      newly += __popc(link[w] & ~done[w] & mask);
      done[w] |= mask;
      if (round) round[w] |= mask;
    }
    remaining -= warp_sum_u32(newly);
    clen += pos - z + 1;
    __syncwarp();
    if (stop) {
      first = z;
      return;
    }
    pos = btg[z];  // a link to a node other than z - 1
  }
}

// The overlap of one walked chain (start s0 back to first): overlapTest,
// then the k-mer divergence; kept proposals are appended to props.
__device__ __forceinline__ void add_proposal(
    const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
    const int32_t* __restrict__ score, uint64_t b, uint32_t s0, int32_t first, int32_t clen,
    const QueryInfo& qi, int64_t ext_signed, const GroupInfo& g, const int32_t* fq, uint32_t nf,
    const LogfTable& logt, const ChainParams& p, DeviceStatus* st, uint32_t gidx, Prop* props,
    int& np, bool& overflow) {
  const int32_t k = p.k;
  const bool swapped = g.ext_sorted == 1;
  int32_t c0, e0, c1, e1;
  load_match(keys, vals, swapped, b + first, c0, e0);
  load_match(keys, vals, swapped, b + s0, c1, e1);
  Prop o;
  o.cb = c0;
  o.ce = c1 + k - 1;
  o.eb = e0;
  o.ee = e1 + k - 1;
  o.score = score[b + s0] - score[b + first] + k - 1;
  o.clen = clen;
  bool keep = overlap_test(o, qi.signed_id, ext_signed, qi.len, g.ext_len, p);
  if (keep) {
    const uint32_t lo = lower_bound_i32(fq, nf, o.cb);
    const uint32_t hi = lower_bound_i32(fq, nf, o.ce + 1);
    const int32_t norm = max(o.ce - o.cb, o.ee - o.eb) - static_cast<int32_t>(hi - lo);
    keep = norm > 0;
    if (keep) {
      float rate = fdiv(fmul(static_cast<float>(clen), p.sample_rate), static_cast<float>(norm));
      rate = rate < 1.0f ? rate : 1.0f;
      const float x = fdiv(1.0f, rate);
      if (!(x < 16777216.0f)) raise_status(st, kDevLogDomain, 0, static_cast<int64_t>(gidx));
      o.div = fdiv(flye_logf(x, logt), static_cast<float>(k));
    }
  }
  if (keep) {
    if (np == kMaxProposals) {
      raise_status(st, kDevProposalOverflow, 0, static_cast<int64_t>(gidx));
      overflow = true;
    } else {
      props[np++] = o;
    }
  }
}

__global__ void __launch_bounds__(kBtWarps * 32, 4) backtrack_kernel(
    const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
    const int32_t* __restrict__ score, int32_t* bt, const uint32_t* __restrict__ order,
    const GroupInfo* __restrict__ groups, const uint32_t* __restrict__ dp_list,
    const uint32_t* __restrict__ list_count, const GroupTop* __restrict__ top,
    uint32_t* __restrict__ redo_list, uint32_t* __restrict__ redo_count,
    const QueryInfo* __restrict__ qinfo,
    const uint64_t* __restrict__ f_off, const int32_t* __restrict__ fpos,
    const int64_t* __restrict__ slot_signed, LogfTable logt, ChainParams p,
    OverlapRow* __restrict__ pool, uint64_t pool_cap, uint32_t* __restrict__ pool_count,
    uint32_t* __restrict__ group_rows, DeviceStatus* st, uint32_t* gmaps, uint64_t gmap_words,
    uint32_t* __restrict__ work) {
  extern __shared__ __align__(16) unsigned char bt_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  BtMaps& m = reinterpret_cast<BtMaps*>(bt_raw)[wib];
  const uint32_t cnt = *list_count;
  for (uint32_t li = next_item(work); li < cnt; li = next_item(work)) {
  const uint32_t gidx = dp_list[li];
  const GroupInfo g = groups[gidx];
  const uint64_t b = g.start;
  const int32_t k = p.k;
  const QueryInfo qi = qinfo[g.query];
  const int64_t ext_signed = (g.ext_di & 1u) ? -slot_signed[g.ext_di >> 1]
                                             : slot_signed[g.ext_di >> 1];
  const int32_t* fq = fpos + f_off[g.query];
  const uint32_t nf = static_cast<uint32_t>(f_off[g.query + 1] - f_off[g.query]);
  // the maps: shared memory up to kBtCap nodes, else device memory at the
  // group's own word range
  uint32_t *lk = m.link, *sp = m.step, *dn = m.done, *rn = m.round;
  if (g.n > kBtCap) {
    const uint64_t pb = (b >> 5) + gidx;
    lk = gmaps + pb;
    sp = gmaps + gmap_words + pb;
    dn = gmaps + 2 * gmap_words + pb;
    rn = gmaps + 3 * gmap_words + pb;
  }
  // the first run picks its starts itself; the second follows `order`
  // (Flye's order)
  const bool pick = top != nullptr;
  bool ambiguous = false;
  uint32_t remaining = 0;
  const uint32_t nw = (g.n + 31) / 32;
  for (uint32_t w = 0; w < nw; ++w) {
    const uint32_t j = w * 32 + lane;
    const int32_t v = j < g.n ? bt[b + j] : -1;
    const unsigned lkw = __ballot_sync(0xffffffffu, v != -1);
    const unsigned spw = __ballot_sync(0xffffffffu, j >= 1 && v == static_cast<int32_t>(j) - 1);
    if (lane == 0) {
      lk[w] = lkw;
      sp[w] = spw;
      dn[w] = 0;
      rn[w] = 0;
    }
    remaining += __popc(lkw);
  }
  __syncwarp();
  Prop props[kMaxProposals];
  int np = 0;
  bool overflow = false;
  // Starts by score: the live node of the highest score next (the DP's top
  // first, when it is linked and no other node shares its score).  Live
  // nodes sharing the top score are walked in index order; Flye's order
  // among them (libstdc++'s) gives the same result unless a walk clears
  // another tied start or ends on a node another tied walk cleared, two
  // proposals they keep share a score, or they keep two or more proposals
  // and the group's proposals end up more than 16 (libstdc++ then sorts them
  // unstably).  In those cases the group goes back for Flye's order.
  bool multi = false;
  for (bool first_pick = true; pick && remaining > 0; first_pick = false) {
    int32_t ms = INT_MIN;
    uint32_t mi = 0xffffffffu, mc = 0;
    bool scan = true;
    if (first_pick) {
      const GroupTop t = top[gidx];
      if (t.count == 1 && ((lk[t.first >> 5] >> (t.first & 31)) & 1u)) {
        ms = t.score;
        mi = t.first;
        mc = 1;
        scan = false;
      }
    }
    if (scan) {
      int32_t bs = INT_MIN;
      uint32_t bi = 0xffffffffu, bc = 0;
      for (uint32_t w = 0; w < nw; ++w) {
        const uint32_t lv = lk[w] & ~dn[w];
        if (!lv) continue;
        if ((lv >> lane) & 1u) {
          const int32_t sv = score[b + w * 32 + lane];
          if (sv > bs) {
            bs = sv;
            bi = w * 32 + lane;
            bc = 1;
          } else if (sv == bs) {
            ++bc;
          }
        }
      }
      ms = bs;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) ms = max(ms, __shfl_xor_sync(0xffffffffu, ms, o));
      mc = bs == ms ? bc : 0u;
      mi = bs == ms ? bi : 0xffffffffu;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        mc += __shfl_xor_sync(0xffffffffu, mc, o);
        mi = min(mi, __shfl_xor_sync(0xffffffffu, mi, o));
      }
    }
    if (mc == 0) break;  // no live node (remaining counts them; kept as a guard)
    if (mc == 1) {
      int32_t first = 0, clen = 0;
      bool met = false;
      walk_maps(lk, sp, dn, bt + b, static_cast<int32_t>(mi), first, clen, remaining, nullptr,
                met);
      if (lane == 0 && !overflow)
        add_proposal(keys, vals, score, b, mi, first, clen, qi, ext_signed, g, fq, nf, logt, p, st,
                     gidx, props, np, overflow);
      __syncwarp();
      continue;
    }
    // a tie round over the mc live nodes of score ms
    const int np0 = np;
    bool clash = false;
    uint32_t left = mc;
    for (uint32_t w = mi >> 5; w < nw && left > 0 && !clash; ++w) {
      const uint32_t lv = lk[w] & ~dn[w];
      unsigned tied = __ballot_sync(0xffffffffu,
                                    ((lv >> lane) & 1u) && score[b + w * 32 + lane] == ms);
      while (tied && !clash) {
        const int j = __ffs(tied) - 1;
        tied &= tied - 1;
        --left;
        if ((dn[w] >> j) & 1u) {  // cleared by an earlier walk of this round
          clash = true;
          break;
        }
        int32_t first = 0, clen = 0;
        bool met = false;
        const uint32_t s0 = w * 32 + j;
        walk_maps(lk, sp, dn, bt + b, static_cast<int32_t>(s0), first, clen, remaining, rn, met);
        if (met) {
          clash = true;
          break;
        }
        if (lane == 0 && !overflow)
          add_proposal(keys, vals, score, b, s0, first, clen, qi, ext_signed, g, fq, nf, logt, p,
                       st, gidx, props, np, overflow);
        __syncwarp();
      }
    }
    // a tied start cleared before its word was reached is never met above
    if (left > 0) clash = true;
    if (lane == 0 && !clash) {
      for (int i = np0; i < np && !clash; ++i)
        for (int j = i + 1; j < np; ++j)
          if (props[i].score == props[j].score) clash = true;
      if (np - np0 >= 2) multi = true;
    }
    clash = __shfl_sync(0xffffffffu, clash, 0);
    if (clash) {
      ambiguous = true;
      break;
    }
    for (uint32_t w = lane; w < nw; w += 32) rn[w] = 0;
    __syncwarp();
  }
  if (multi && np > 16) ambiguous = true;
  for (uint32_t o0 = 0; !pick && o0 < g.n && remaining > 0; o0 += 32) {
    const uint32_t oi = o0 + lane;
    const bool valid = oi < g.n;
    const uint32_t start = valid ? order[b + oi] : 0;
    unsigned mask = __ballot_sync(
        0xffffffffu,
        valid && (((lk[start >> 5] & ~dn[start >> 5]) >> (start & 31)) & 1u) != 0);
    while (mask) {
      const int j = __ffs(mask) - 1;
      const uint32_t s0 = __shfl_sync(0xffffffffu, start, j);
      int32_t first = 0, clen = 0;
      bool met = false;
      walk_maps(lk, sp, dn, bt + b, static_cast<int32_t>(s0), first, clen, remaining, nullptr,
                met);
      if (lane == 0 && !overflow)
        add_proposal(keys, vals, score, b, s0, first, clen, qi, ext_signed, g, fq, nf, logt, p, st,
                     gidx, props, np, overflow);
      __syncwarp();
      if (remaining == 0) break;
      mask = __ballot_sync(
          0xffffffffu,
          valid && lane > j &&
              (((lk[start >> 5] & ~dn[start >> 5]) >> (start & 31)) & 1u) != 0);
    }
  }
  __syncwarp();
  if (lane != 0) continue;
  if (ambiguous) {
    redo_list[atomicAdd(redo_count, 1u)] = gidx;
    continue;
  }
  if (overflow) {
    group_rows[gidx] = 0;
    continue;
  }
  // proposals by score descending, libstdc++ order
  uint64_t K[kMaxProposals];
  uint32_t V[kMaxProposals];
  for (int i = 0; i < np; ++i) {
    K[i] = static_cast<uint64_t>(static_cast<uint32_t>(INT_MAX - props[i].score));
    V[i] = static_cast<uint32_t>(i);
  }
  isort::serial_introsort(K, V, 0, static_cast<uint32_t>(np),
                          isort::depth_limit(static_cast<uint32_t>(np)));
  int prim[kMaxProposals];
  int nprim = 0;
  if (p.only_max_ext) {
    if (np > 0) prim[nprim++] = static_cast<int>(V[0]);
  } else {
    for (int s = 0; s < np; ++s) {
      const Prop& o = props[V[s]];
      bool contained = false;
      for (int t = 0; t < nprim && !contained; ++t) {
        const Prop& pr = props[prim[t]];
        contained = pr.cb <= o.cb && o.ce <= pr.ce && pr.eb <= o.eb && o.ee <= pr.ee &&
                    pr.score > o.score;
      }
      if (!contained) prim[nprim++] = static_cast<int>(V[s]);
    }
  }
  int keep[kMaxProposals];
  int nk = 0;
  for (int t = 0; t < nprim; ++t)
    if (props[prim[t]].div < p.max_divergence) keep[nk++] = prim[t];
  group_rows[gidx] = static_cast<uint32_t>(nk);
  if (nk == 0) continue;
  const uint32_t base = atomicAdd(pool_count, static_cast<uint32_t>(nk));
  if (base + nk > pool_cap) {
    raise_status(st, kDevProposalOverflow, 1, static_cast<int64_t>(gidx));
    continue;
  }
  for (int t = 0; t < nk; ++t) {
    const Prop& o = props[keep[t]];
    OverlapRow r;
    r.query = g.query;
    r.ext_di = g.ext_di;
    r.cur_begin = o.cb;
    r.cur_end = o.ce;
    r.cur_len = qi.len;
    r.ext_begin = o.eb;
    r.ext_end = o.ee;
    r.ext_len = g.ext_len;
    r.score = o.score;
    r.chain_len = o.clen;
    r.div = o.div;
    r.group = gidx;
    r.rank = static_cast<uint32_t>(t);
    pool[base + t] = r;
  }
  }
}

__global__ void query_group_off_kernel(const GroupInfo* __restrict__ groups, uint64_t ngroups,
                                       uint32_t nq, uint64_t* __restrict__ qg) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q > nq) return;
  uint64_t lo = 0, hi = ngroups;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (groups[mid].query < q)
      lo = mid + 1;
    else
      hi = mid;
  }
  qg[q] = lo;
}

__global__ void rows_limit_kernel(const uint32_t* __restrict__ group_rows,
                                  const uint64_t* __restrict__ q_group_off, uint32_t nq,
                                  int32_t max_overlaps, uint32_t* __restrict__ kept) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  uint64_t detected = 0;
  for (uint64_t g = q_group_off[q]; g < q_group_off[q + 1]; ++g) {
    if (max_overlaps > 0 && detected >= static_cast<uint64_t>(max_overlaps)) {
      kept[g] = 0;
      continue;
    }
    kept[g] = group_rows[g];
    detected += group_rows[g];
  }
}

__global__ void rows_scatter_kernel(const OverlapRow* __restrict__ pool, uint32_t npool,
                                    const uint32_t* __restrict__ kept,
                                    const uint64_t* __restrict__ kept_off,
                                    OverlapRow* __restrict__ rows) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npool) return;
  const OverlapRow r = pool[i];
  if (r.rank < kept[r.group]) rows[kept_off[r.group] + r.rank] = r;
}

}  // namespace

cudaError_t groups_count(const uint64_t* keys, const uint64_t* q_off, uint32_t nq, uint64_t nhits,
                         uint32_t* tile_counts, cudaStream_t s) {
  if (nhits == 0) return cudaSuccess;
  count_launch();
  group_tiles_kernel<false><<<static_cast<unsigned>((nhits + kGroupTile - 1) / kGroupTile),
                              kGroupBlock, 0, s>>>(keys, q_off, nq, nhits, tile_counts, nullptr,
                                                   nullptr);
  return cudaGetLastError();
}

cudaError_t groups_write(const uint64_t* keys, const uint64_t* q_off, uint32_t nq, uint64_t nhits,
                         const uint64_t* tile_off, GroupInfo* groups, cudaStream_t s) {
  if (nhits == 0) return cudaSuccess;
  count_launch();
  group_tiles_kernel<true><<<static_cast<unsigned>((nhits + kGroupTile - 1) / kGroupTile),
                             kGroupBlock, 0, s>>>(keys, q_off, nq, nhits, nullptr, tile_off,
                                                  groups);
  return cudaGetLastError();
}

cudaError_t groups_prefilter_n(const uint64_t* keys, const uint32_t* vals, GroupInfo* groups,
                               uint64_t ngroups, uint64_t nhits, const QueryInfo* qinfo,
                               const int32_t* slot_len, const ChainParams& p,
                               uint32_t* ext_list, uint32_t* dp_list, uint32_t* counts,
                               cudaStream_t s) {
  cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), s);
  if (ngroups == 0) return cudaGetLastError();
  count_launch();
  prefilter_kernel<<<grid(ngroups * 32, 256), 256, 0, s>>>(keys, vals, groups, ngroups, nhits,
                                                           qinfo, slot_len, p, ext_list, dp_list,
                                                           counts);
  return cudaGetLastError();
}

cudaError_t groups_prefilter_list(const uint64_t* keys, const uint32_t* vals, GroupInfo* groups,
                                  const uint32_t* list, const QueryInfo* qinfo,
                                  const int32_t* slot_len, const ChainParams& p,
                                  uint32_t* ext_list, uint32_t* dp_list, uint32_t* counts,
                                  uint32_t max_groups, cudaStream_t s) {
  if (max_groups == 0) return cudaSuccess;
  count_launch();
  prefilter_list_kernel<<<static_cast<unsigned>(std::min<uint64_t>(grid(max_groups * 32ull, 256),
                                                                    4096)),
                          256, 0, s>>>(keys, vals, groups, list, qinfo, slot_len, p,
                                       ext_list, dp_list, counts);
  return cudaGetLastError();
}

cudaError_t groups_prepare_ext_sort(uint64_t* keys, uint32_t* vals, const GroupInfo* groups,
                                    const uint32_t* ext_list, const uint32_t* counts,
                                    uint64_t* seg_begin, uint64_t* seg_end, cudaStream_t s) {
  count_launch();
  prepare_ext_sort_kernel<<<2048, 256, 0, s>>>(keys, vals, groups, ext_list, counts, seg_begin,
                                               seg_end);
  return cudaGetLastError();
}

cudaError_t groups_ext_presorted(const uint32_t* vals, GroupInfo* groups, const uint32_t* ext_list,
                                 const uint32_t* counts, uint32_t* out, uint32_t* out_count,
                                 cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out_count, 0, 4, s);
  if (e != cudaSuccess) return e;
  count_launch();
  ext_presorted_kernel<<<2048, 256, 0, s>>>(vals, groups, ext_list, counts, out, out_count);
  return cudaGetLastError();
}

namespace {
// Length buckets for the warp-per-group stages: groups of over 16,384,
// 4,096, 1,024 and 256 hits, then the rest, longest bucket first, so the
// longest groups start in the first wave and the short ones fill the tail.
constexpr int kLenBuckets = 5;
__device__ __forceinline__ int len_bucket(uint32_t n) {
  return n > 16384 ? 0 : n > 4096 ? 1 : n > 1024 ? 2 : n > 256 ? 3 : 4;
}

__global__ void bucket_count_kernel(const GroupInfo* __restrict__ groups,
                                    const uint32_t* __restrict__ list,
                                    const uint32_t* __restrict__ list_count,
                                    uint32_t* __restrict__ bcount) {
  __shared__ uint32_t h[kLenBuckets];
  if (threadIdx.x < kLenBuckets) h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t cnt = *list_count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
    atomicAdd(&h[len_bucket(groups[list[i]].n)], 1u);
  __syncthreads();
  if (threadIdx.x < kLenBuckets && h[threadIdx.x]) atomicAdd(&bcount[threadIdx.x], h[threadIdx.x]);
}

__global__ void bucket_scatter_kernel(const GroupInfo* __restrict__ groups,
                                      const uint32_t* __restrict__ list,
                                      const uint32_t* __restrict__ list_count,
                                      const uint32_t* __restrict__ bcount,
                                      uint32_t* __restrict__ bfill, uint32_t* __restrict__ out) {
  const uint32_t cnt = *list_count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const uint32_t g = list[i];
    const int b = len_bucket(groups[g].n);
    uint32_t base = 0;
    for (int c = 0; c < b; ++c) base += bcount[c];
    out[base + atomicAdd(&bfill[b], 1u)] = g;
  }
}
}  // namespace

cudaError_t groups_length_order(const GroupInfo* groups, const uint32_t* list,
                                const uint32_t* list_count, uint32_t max_groups,
                                uint32_t* scratch, uint32_t* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(scratch, 0, 2 * kLenBuckets * sizeof(uint32_t), s);
  if (e != cudaSuccess || max_groups == 0) return e;
  const unsigned g = static_cast<unsigned>(std::min<uint64_t>((max_groups + 255) / 256, 2048));
  count_launch();
  bucket_count_kernel<<<g, 256, 0, s>>>(groups, list, list_count, scratch);
  count_launch();
  bucket_scatter_kernel<<<g, 256, 0, s>>>(groups, list, list_count, scratch,
                                          scratch + kLenBuckets, out);
  return cudaGetLastError();
}

cudaError_t chain_dp(const uint64_t* keys, const uint32_t* vals, int32_t* score, int32_t* bt,
                     const GroupInfo* groups, const uint32_t* dp_list, const uint32_t* counts,
                     const ChainParams& p, GroupTop* top, int32_t* pmc, uint32_t* work,
                     int num_sms, int per_sm, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(work, 0, 4, s);
  if (e != cudaSuccess) return e;
  // one resident wave taking groups from a counter: any grid gives the same
  // result; per_sm (0: the occupancy limit) only sets how many warps share it
  int most = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&most, dp_kernel, kDpWarps * 32, 0);
  if (e != cudaSuccess) return e;
  most = std::max(most, 1);
  const int blocks = per_sm > 0 ? std::min(per_sm, most) : most;
  count_launch();
  dp_kernel<<<num_sms * blocks, kDpWarps * 32, 0, s>>>(keys, vals, score, bt, groups, dp_list,
                                                       counts, p, top, pmc, work);
  return cudaGetLastError();
}

namespace {
__global__ void query_rows_kernel(const uint64_t* __restrict__ q_group_off,
                                  const uint64_t* __restrict__ kept_off, uint32_t nq,
                                  uint64_t* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq) out[q] = kept_off[q_group_off[q + 1]] - kept_off[q_group_off[q]];
}
}  // namespace

cudaError_t query_row_counts(const uint64_t* q_group_off, const uint64_t* kept_off, uint32_t nq,
                             uint64_t* out, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  query_rows_kernel<<<grid(nq, 256), 256, 0, s>>>(q_group_off, kept_off, nq, out);
  return cudaGetLastError();
}

cudaError_t chain_prepare_order(const int32_t* score, uint64_t* keys, uint32_t* vals,
                                const GroupInfo* groups, const uint32_t* list,
                                const uint32_t* list_count, uint64_t* seg_begin,
                                uint64_t* seg_end, cudaStream_t s) {
  count_launch();
  prepare_order_kernel<<<2048, 256, 0, s>>>(score, keys, vals, groups, list, list_count,
                                            seg_begin, seg_end);
  return cudaGetLastError();
}

cudaError_t chain_backtrack(const uint64_t* keys, const uint32_t* vals, const int32_t* score,
                            int32_t* bt, const uint32_t* order, const GroupInfo* groups,
                            const uint32_t* list, const uint32_t* list_count,
                            const GroupTop* top, uint32_t* redo_list, uint32_t* redo_count,
                            const QueryInfo* qinfo, const uint64_t* f_off, const int32_t* fpos,
                            const int64_t* slot_signed, const LogfTable& logt,
                            const ChainParams& p, OverlapRow* pool, uint64_t pool_cap,
                            uint32_t* pool_count, uint32_t* group_rows, DeviceStatus* st,
                            uint32_t max_groups, uint32_t* gmaps, uint64_t gmap_words,
                            uint32_t* work, int per_sm, cudaStream_t s) {
  if (max_groups == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(work, 0, 4, s);
  if (e != cudaSuccess) return e;
  constexpr size_t smem = sizeof(BtMaps) * kBtWarps;
  cudaFuncSetAttribute(backtrack_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(smem));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  // blocks take groups from a counter: per_sm (1-4, 0: 4) sets only the wave
  const int blocks = per_sm > 0 ? std::min(per_sm, 4) : 4;
  count_launch();
  backtrack_kernel<<<sms * blocks, kBtWarps * 32, smem, s>>>(
      keys, vals, score, bt, order, groups, list, list_count, top, redo_list, redo_count,
      qinfo, f_off, fpos, slot_signed, logt,
      p, pool, pool_cap, pool_count, group_rows, st, gmaps, gmap_words, work);
  return cudaGetLastError();
}

cudaError_t query_group_offsets(const GroupInfo* groups, uint64_t ngroups, uint32_t nq,
                                uint64_t* q_group_off, cudaStream_t s) {
  count_launch();
  query_group_off_kernel<<<grid(nq + 1, 256), 256, 0, s>>>(groups, ngroups, nq, q_group_off);
  return cudaGetLastError();
}

cudaError_t rows_limit(const uint32_t* group_rows, const uint64_t* q_group_off, uint32_t nq,
                       int32_t max_overlaps, uint32_t* kept_rows, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  rows_limit_kernel<<<grid(nq, 128), 128, 0, s>>>(group_rows, q_group_off, nq, max_overlaps,
                                                  kept_rows);
  return cudaGetLastError();
}

cudaError_t rows_scatter(const OverlapRow* pool, uint32_t npool, const uint32_t* kept_rows,
                         const uint64_t* kept_off, OverlapRow* rows, cudaStream_t s) {
  if (npool == 0) return cudaSuccess;
  count_launch();
  rows_scatter_kernel<<<grid(npool, 256), 256, 0, s>>>(pool, npool, kept_rows, kept_off, rows);
  return cudaGetLastError();
}

}  // namespace cuflye
