// r2g.cu — read-to-graph chains: the per-read body of ReadAligner::alignReads
// after quickSeqOverlaps.
//
//   filter     : keep overlaps with extLen < LONG_EDGE or
//                min(curRange, extRange) > BIG_ALN
//                (patches/flye/2.9.6/0039-cuflye-read-to-graph-input-boundary-oracle.patch:72-76);
//   sort       : by curBegin with libstdc++ std::sort order (0039:249-251), done
//                by the segmented sort in sort.cu;
//   chain      : chainReadAlignments, one warp per read
//                (cuda/cuflye_cuda_read_alignment_chain_replay.cu:872-984): the
//                candidate chains before the divergence filter (Flye's
//                readChains), in acceptance order;
//   divergence : one value per candidate chain and the accept test
//                chainDivergence < read_align_ovlp_divergence
//                (patches/flye/2.9.6/0026-cuflye-read-alignment-replay-fixture-dump.patch:215-226).
//                Flye's getChainBaseDivergence is not in the reference; the
//                value is either supplied (a replay fixture's
//                chain-divergence.tsv) or this library's k-mer form, the
//                curRange-weighted mean of the segments' divergences, which the
//                CPU oracle shares;
//   emit       : good chains, then their complements with reversed segment
//                order (patches/flye/2.9.6/0037-cuflye-read-alignment-selected-cpu-bypass.patch:192-211),
//                or the candidate chains as chain records (the compact payload's
//                records, docs/abi/read-alignment-compact-binary-v0.md).
//
// Every stage reads a read's rows through a_off (first row of each read) and
// per-row metadata (graph nodes, edge ids, candidate id), so in-process reads
// and replay fixtures share the kernels.
#include <climits>
#include <cstdint>

#include "../../include/cuflye.h"
#include "common.cuh"
#include "kernels.h"
#include "r2g.h"

namespace cuflye {
namespace {

inline unsigned grid(uint64_t n, int b) {
  return static_cast<unsigned>((n + b - 1) / b > 0 ? (n + b - 1) / b : 1);
}

__global__ void filter_kernel(const OverlapRow* __restrict__ rows, uint64_t n, R2GParams rp,
                              uint32_t* __restrict__ keep) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const OverlapRow r = rows[i];
  const int32_t cr = r.cur_end - r.cur_begin, er = r.ext_end - r.ext_begin;
  keep[i] = (r.ext_len < rp.long_edge || min(cr, er) > rp.big_aln) ? 1u : 0u;
}

// Kept rows in order; src[j] = the kept row's index among all rows.
__global__ void compact_kernel(const OverlapRow* __restrict__ rows, uint64_t n,
                               const uint32_t* __restrict__ keep,
                               const uint64_t* __restrict__ pos, OverlapRow* __restrict__ out,
                               uint64_t* __restrict__ src) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  out[pos[i]] = rows[i];
  src[pos[i]] = i;
}

__global__ void sort_keys_kernel(const OverlapRow* __restrict__ a,
                                 const uint64_t* __restrict__ a_off, uint32_t nq,
                                 uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t q = blockIdx.x;
  if (q >= nq) return;
  const uint64_t b = a_off[q], e = a_off[q + 1];
  for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    keys[i] = static_cast<uint64_t>(static_cast<uint32_t>(a[i].cur_begin));
    vals[i] = static_cast<uint32_t>(i - b);
  }
}

// The sorted rows, and each one's metadata: graph nodes and ids from the
// edge sequence it aligns to, candidate id = its index among the read's
// quickSeqOverlaps rows before the filter.
__global__ void permute_kernel(const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off,
                               uint32_t nq, const uint32_t* __restrict__ vals,
                               const uint64_t* __restrict__ src,
                               const uint64_t* __restrict__ row_off, R2GGraph g,
                               OverlapRow* __restrict__ out, R2GRowMeta* __restrict__ meta) {
  const uint32_t q = blockIdx.x;
  if (q >= nq) return;
  const uint64_t b = a_off[q], e = a_off[q + 1];
  for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const uint64_t from = b + vals[i];
    const OverlapRow o = a[from];
    out[i] = o;
    const uint32_t slot = o.ext_di >> 1;
    const int64_t edge = g.edge_of_slot[slot];
    const int32_t l = g.left_of_slot[slot], r = g.right_of_slot[slot];
    const int64_t seq = g.slot_signed[slot];
    R2GRowMeta m;
    m.candidate_id = static_cast<int64_t>(src[from] - row_off[q]);
    if (o.ext_di & 1u) {  // the complement edge runs right^1 -> left^1
      m.edge_id = -edge;
      m.edge_seq_id = -seq;
      m.left = r ^ 1;
      m.right = l ^ 1;
    } else {
      m.edge_id = edge;
      m.edge_seq_id = seq;
      m.left = l;
      m.right = r;
    }
    meta[i] = m;
  }
}

// Replay fixtures: the caller's edge overlaps as rows and metadata.
__global__ void replay_rows_kernel(const cuflye_edge_overlap* __restrict__ in, uint64_t n,
                                   OverlapRow* __restrict__ out, R2GRowMeta* __restrict__ meta) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cuflye_edge_overlap x = in[i];
  OverlapRow o{};
  o.cur_begin = x.read_begin;
  o.cur_end = x.read_end;
  o.cur_len = x.read_len;
  o.ext_begin = x.edge_begin;
  o.ext_end = x.edge_end;
  o.ext_len = x.edge_len;
  o.score = x.score;
  o.div = x.seq_divergence;
  out[i] = o;
  R2GRowMeta m;
  m.candidate_id = x.candidate_id;
  m.edge_id = x.edge_id;
  m.edge_seq_id = x.edge_seq_id;
  m.left = x.edge_left;
  m.right = x.edge_right;
  meta[i] = m;
}

// Chain record: extending chain c appends a record whose parent is c's last
// record, so chains that share a prefix share records.
struct ChainRec {
  int32_t parent, idx, first, len, score;
};

// chainReadAlignments for one read per warp.  For each alignment in curBegin
// order the lanes score every active chain at once; the chain extended is the
// first (lowest position in the active list) with the highest score above 0,
// as the serial loop's strict '>' picks.  Outdated chains leave the active
// list (in order) when they outnumber half of it.  Then every chain, active
// before frozen, is ranked by score descending (stable), and accepted in that
// order when long enough and separated from the accepted ones.  Output:
// cand[b + t] = last record of candidate chain t, n_cand[q].
__global__ void __launch_bounds__(128) chain_kernel(const OverlapRow* __restrict__ a,
                                                    const uint64_t* __restrict__ a_off,
                                                    uint32_t nq,
                                                    const R2GRowMeta* __restrict__ meta,
                                                    R2GParams rp, ChainRec* __restrict__ recs,
                                                    int32_t* __restrict__ active,
                                                    int32_t* __restrict__ frozen,
                                                    int32_t* __restrict__ cand,
                                                    uint32_t* __restrict__ n_cand) {
  const int lane = threadIdx.x & 31;
  const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  const unsigned lt = (1u << lane) - 1u;
  const uint64_t b = a_off[q];
  const int32_t n = static_cast<int32_t>(a_off[q + 1] - b);
  const OverlapRow* A = a + b;
  const R2GRowMeta* M = meta + b;
  ChainRec* R = recs + b;
  int32_t* act = active + b;
  int32_t* frz = frozen + b;
  int32_t* cd = cand + b;
  int32_t na = 0, nf = 0, nr = 0;
  for (int32_t index = 0; index < n; ++index) {
    const OverlapRow cur = A[index];
    const int32_t cur_left = M[index].left;
    int32_t best = 0, best_c = INT_MAX;  // best score above 0, first position attaining it
    int32_t outdated = 0;
    const bool can_extend = cur.ext_begin < rp.max_jump;
    const bool can_be_extended = cur.ext_len - cur.ext_end < rp.max_jump;
    if (can_extend) {
      for (int32_t c = lane; c < na; c += 32) {
        const ChainRec ch = R[act[c]];
        const OverlapRow prev = A[ch.idx];
        const int32_t read_diff = cur.cur_begin - prev.cur_end;
        const int32_t gl = cur.ext_begin, gr = prev.ext_len - prev.ext_end;
        if (M[ch.idx].right == cur_left && rp.max_jump > read_diff &&
            read_diff > -rp.max_read_overlap && gl + gr < rp.max_jump) {
          const int32_t jd = abs(read_diff - (gl + gr));
          const int32_t gap = jd > 100 ? jd / 50 : 0;
          const int32_t sc = ch.score + cur.score - gap;
          if (sc > best) {  // lanes visit their positions in order: the first keeps ties
            best = sc;
            best_c = c;
          }
        }
        if (read_diff > rp.max_jump) ++outdated;
      }
      // highest score, then the first position attaining it
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int32_t ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int32_t oc = __shfl_xor_sync(0xffffffffu, best_c, o);
        if (ob > best || (ob == best && oc < best_c)) {
          best = ob;
          best_c = oc;
        }
        outdated += __shfl_xor_sync(0xffffffffu, outdated, o);
      }
    }
    const bool extends = best > 0;
    if (lane == 0) {
      ChainRec r;
      r.idx = index;
      if (extends) {
        const ChainRec pr = R[act[best_c]];
        r.parent = act[best_c];
        r.first = pr.first;
        r.len = pr.len + 1;
        r.score = best;
      } else {
        r.parent = -1;
        r.first = index;
        r.len = 1;
        r.score = cur.score;
      }
      R[nr] = r;
      if (extends || can_be_extended)
        act[na] = nr;
      else
        frz[nf] = nr;
    }
    if (extends || can_be_extended)
      ++na;
    else
      ++nf;
    ++nr;
    __syncwarp();
    if (outdated > na / 2) {
      // outdated chains to the frozen list, the others stay active, in order
      const int32_t na0 = na;
      int32_t w = 0;
      for (int32_t c0 = 0; c0 < na0; c0 += 32) {
        const int32_t c = c0 + lane;
        int32_t v = 0;
        bool old = false;
        if (c < na0) {
          v = act[c];
          old = cur.cur_begin - A[R[v].idx].cur_end > rp.max_jump;
        }
        const unsigned mo = __ballot_sync(0xffffffffu, c < na0 && old);
        const unsigned mk = __ballot_sync(0xffffffffu, c < na0 && !old);
        __syncwarp();  // every lane has read its entry before any is overwritten
        if (c < na0) {
          if (old)
            frz[nf + __popc(mo & lt)] = v;
          else
            act[w + __popc(mk & lt)] = v;
        }
        nf += __popc(mo);
        w += __popc(mk);
        __syncwarp();
      }
      na = w;
    }
  }
  // all = active ++ frozen, ranked by score descending, stable (into cand)
  const int32_t nall = na + nf;
  for (int32_t i = lane; i < nall; i += 32) {
    const int32_t vi = i < na ? act[i] : frz[i - na];
    const int32_t si = R[vi].score;
    int32_t rank = 0;
    for (int32_t j = 0; j < nall; ++j) {
      const int32_t sj = R[j < na ? act[j] : frz[j - na]].score;
      rank += (sj > si || (sj == si && j < i)) ? 1 : 0;
    }
    cd[rank] = vi;
  }
  __syncwarp();
  // acceptance: min overlap, and separation from the chains already accepted
  // (the active list holds them from here on)
  int32_t nacc = 0;
  for (int32_t i = 0; i < nall; ++i) {
    const ChainRec c = R[cd[i]];
    const OverlapRow first = A[c.first], last = A[c.idx];
    if (last.cur_end - first.cur_begin < rp.min_overlap) continue;
    bool overl = false;
    for (int32_t t = lane; t < nacc; t += 32) {
      const ChainRec e = R[act[t]];
      const OverlapRow ef = A[e.first], el = A[e.idx];
      const int32_t rate = min(last.cur_end, el.cur_end) - max(first.cur_begin, ef.cur_begin);
      overl |= rate > rp.max_separation;
    }
    overl = __any_sync(0xffffffffu, overl);
    if (!overl) {
      if (lane == 0) act[nacc] = cd[i];
      ++nacc;
      __syncwarp();
    }
  }
  for (int32_t t = lane; t < nacc; t += 32) cd[t] = act[t];
  if (lane == 0) n_cand[q] = static_cast<uint32_t>(nacc);
}

// Divergence of each candidate chain and the accept test, one warp per read,
// lanes over chains: supplied (div_in at div_off[q] + t) or the k-mer form
// (segments in chain order).  Accepted chains go to good (in order); per
// read n_good and the rows they emit (2 per segment) and, over all candidate
// chains, their segments (n_segs).
__global__ void __launch_bounds__(128) divergence_kernel(
    const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off, uint32_t nq,
    const ChainRec* __restrict__ recs, const int32_t* __restrict__ cand,
    const uint32_t* __restrict__ n_cand, const float* __restrict__ div_in,
    const uint64_t* __restrict__ div_off, R2GParams rp, float* __restrict__ div_out,
    uint8_t* __restrict__ acc_out, int32_t* __restrict__ good, uint32_t* __restrict__ n_good,
    uint32_t* __restrict__ n_rows, uint32_t* __restrict__ n_segs) {
  const int lane = threadIdx.x & 31;
  const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  const unsigned lt = (1u << lane) - 1u;
  const uint64_t b = a_off[q];
  const OverlapRow* A = a + b;
  const ChainRec* R = recs + b;
  const int32_t nc = static_cast<int32_t>(n_cand[q]);
  int32_t ngood = 0;
  uint32_t rows = 0, segs = 0;
  for (int32_t t0 = 0; t0 < nc; t0 += 32) {
    const int32_t t = t0 + lane;
    bool ok = false;
    int32_t last = 0, len = 0;
    if (t < nc) {
      last = cand[b + t];
      len = R[last].len;
      float d;
      if (div_in) {
        d = div_in[div_off[q] + t];
      } else {
        // curRange-weighted mean, summed in chain order (first segment first)
        float sum = 0.0f, total = 0.0f;
        for (int32_t s = 0; s < len; ++s) {
          int32_t r = last;
          for (int32_t k = len - 1; k > s; --k) r = R[r].parent;
          const OverlapRow o = A[R[r].idx];
          const float rr = static_cast<float>(o.cur_end - o.cur_begin);
          sum = fadd(sum, fmul(o.div, rr));
          total = fadd(total, rr);
        }
        d = fdiv(sum, total);
      }
      ok = d < rp.max_chain_divergence;
      if (div_out) div_out[b + t] = d;
      if (acc_out) acc_out[b + t] = ok ? 1 : 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok) good[b + ngood + __popc(m & lt)] = last;
    ngood += __popc(m);
    rows += ok ? 2u * static_cast<uint32_t>(len) : 0u;
    segs += t < nc ? static_cast<uint32_t>(len) : 0u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rows += __shfl_xor_sync(0xffffffffu, rows, o);
    segs += __shfl_xor_sync(0xffffffffu, segs, o);
  }
  if (lane == 0) {
    n_good[q] = static_cast<uint32_t>(ngood);
    n_rows[q] = rows;
    if (n_segs) n_segs[q] = segs;
  }
}

__device__ __forceinline__ void write_row(cuflye_read_alignment* out, int64_t chain,
                                          int64_t seg, const OverlapRow& o,
                                          const R2GRowMeta& m, int64_t read_id, bool comp) {
  cuflye_read_alignment r;
  r.chain_id = chain;
  r.segment_id = seg;
  r.score = o.score;
  r.seq_divergence = o.div;
  r.read_len = o.cur_len;
  r.edge_len = o.ext_len;
  if (!comp) {
    r.read_id = read_id;
    r.edge_id = m.edge_id;
    r.edge_seq_id = m.edge_seq_id;
    r.read_begin = o.cur_begin;
    r.read_end = o.cur_end;
    r.edge_begin = o.ext_begin;
    r.edge_end = o.ext_end;
  } else {
    r.read_id = -read_id;
    r.edge_id = -m.edge_id;
    r.edge_seq_id = -m.edge_seq_id;
    r.read_begin = o.cur_len - o.cur_end - 1;
    r.read_end = o.cur_len - o.cur_begin - 1;
    r.edge_begin = o.ext_len - o.ext_end - 1;
    r.edge_end = o.ext_len - o.ext_begin - 1;
  }
  *out = r;
}

// Segment s of the chain ending at record `last` (forward order).
__device__ __forceinline__ int32_t segment_row(const ChainRec* R, int32_t last, int32_t len,
                                               int32_t s) {
  int32_t r = last;
  for (int32_t k = len - 1; k > s; --k) r = R[r].parent;
  return R[r].idx;
}

// Good chains, then their complements (reversed segments); one thread per
// read, the chains' rows in order.
__global__ void emit_kernel(const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off,
                            uint32_t nq, const R2GRowMeta* __restrict__ meta,
                            const int64_t* __restrict__ read_ids,
                            const ChainRec* __restrict__ recs, const int32_t* __restrict__ good,
                            const uint32_t* __restrict__ n_good,
                            const uint64_t* __restrict__ chain_off,
                            const uint64_t* __restrict__ row_off, int32_t* __restrict__ tmp,
                            cuflye_read_alignment* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t b = a_off[q];
  const OverlapRow* A = a + b;
  const R2GRowMeta* M = meta + b;
  const ChainRec* R = recs + b;
  const int32_t* gd = good + b;
  int32_t* T = tmp + b;
  const int32_t ng = static_cast<int32_t>(n_good[q]);
  const int64_t read_id = read_ids[q];
  uint64_t w = row_off[q];
  const uint64_t c0 = chain_off[q];
  for (int pass = 0; pass < 2; ++pass) {
    for (int32_t t = 0; t < ng; ++t) {
      const int32_t last = gd[t];
      const int32_t len = R[last].len;
      int32_t r = last;
      for (int32_t s = len - 1; s >= 0; --s) {
        T[s] = R[r].idx;
        r = R[r].parent;
      }
      const int64_t chain = static_cast<int64_t>(c0) + pass * ng + t;
      for (int32_t s = 0; s < len; ++s) {
        const int32_t ai = pass == 0 ? T[s] : T[len - 1 - s];
        write_row(out + w, chain, s, A[ai], M[ai], read_id, pass == 1);
        ++w;
      }
    }
  }
}

// Candidate chains as chain records: per read, chains in acceptance order,
// segments in chain order; a warp per read, lanes over a chain's segments.
__global__ void __launch_bounds__(128) records_kernel(
    const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off, uint32_t nq,
    const R2GRowMeta* __restrict__ meta, const int64_t* __restrict__ query_ids,
    const int64_t* __restrict__ read_ids, const ChainRec* __restrict__ recs,
    const int32_t* __restrict__ cand, const uint32_t* __restrict__ n_cand,
    const uint64_t* __restrict__ rec_off, cuflye_chain_record* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  const uint64_t b = a_off[q];
  const OverlapRow* A = a + b;
  const R2GRowMeta* M = meta + b;
  const ChainRec* R = recs + b;
  const int32_t nc = static_cast<int32_t>(n_cand[q]);
  uint64_t w = rec_off[q];
  for (int32_t t = 0; t < nc; ++t) {
    const int32_t last = cand[b + t];
    const int32_t len = R[last].len;
    for (int32_t s = lane; s < len; s += 32) {
      const int32_t ai = segment_row(R, last, len, s);
      const OverlapRow o = A[ai];
      const R2GRowMeta m = M[ai];
      cuflye_chain_record x;
      x.query_id = query_ids[q];
      x.chain_id = t;
      x.segment_id = s;
      x.overlap_index = ai;
      x.reserved = 0;
      x.candidate_id = m.candidate_id;
      x.read_id = read_ids[q];
      x.read_begin = o.cur_begin;
      x.read_end = o.cur_end;
      x.read_len = o.cur_len;
      x.edge_left = m.left;
      x.edge_right = m.right;
      x.edge_id = m.edge_id;
      x.edge_seq_id = m.edge_seq_id;
      x.edge_begin = o.ext_begin;
      x.edge_end = o.ext_end;
      x.edge_len = o.ext_len;
      x.score = o.score;
      x.seq_divergence = o.div;
      out[w + s] = x;
    }
    w += static_cast<uint64_t>(len);
  }
}

}  // namespace

cudaError_t r2g_filter(const OverlapRow* rows, uint64_t n, const R2GParams& rp, uint32_t* keep,
                       cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  filter_kernel<<<grid(n, 256), 256, 0, s>>>(rows, n, rp, keep);
  return cudaGetLastError();
}

cudaError_t r2g_compact(const OverlapRow* rows, uint64_t n, const uint32_t* keep,
                        const uint64_t* pos, OverlapRow* out, uint64_t* src, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  compact_kernel<<<grid(n, 256), 256, 0, s>>>(rows, n, keep, pos, out, src);
  return cudaGetLastError();
}

cudaError_t r2g_sort_keys(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                          uint64_t* keys, uint32_t* vals, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  sort_keys_kernel<<<nq, 128, 0, s>>>(a, a_off, nq, keys, vals);
  return cudaGetLastError();
}

cudaError_t r2g_permute(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                        const uint32_t* vals, const uint64_t* src, const uint64_t* row_off,
                        const R2GGraph& g, OverlapRow* out, R2GRowMeta* meta, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  permute_kernel<<<nq, 128, 0, s>>>(a, a_off, nq, vals, src, row_off, g, out, meta);
  return cudaGetLastError();
}

cudaError_t r2g_replay_rows(const cuflye_edge_overlap* in, uint64_t n, OverlapRow* out,
                            R2GRowMeta* meta, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  replay_rows_kernel<<<grid(n, 256), 256, 0, s>>>(in, n, out, meta);
  return cudaGetLastError();
}

size_t r2g_rec_bytes() { return sizeof(ChainRec); }

cudaError_t r2g_chain(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                      const R2GRowMeta* meta, const R2GParams& rp, void* recs, int32_t* active,
                      int32_t* frozen, int32_t* cand, uint32_t* n_cand, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  chain_kernel<<<grid(32ull * nq, 128), 128, 0, s>>>(a, a_off, nq, meta, rp,
                                                    static_cast<ChainRec*>(recs), active, frozen,
                                                    cand, n_cand);
  return cudaGetLastError();
}

cudaError_t r2g_divergence(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                           const void* recs, const int32_t* cand, const uint32_t* n_cand,
                           const float* div_in, const uint64_t* div_off, const R2GParams& rp,
                           float* div_out, uint8_t* acc_out, int32_t* good, uint32_t* n_good,
                           uint32_t* n_rows, uint32_t* n_segs, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  divergence_kernel<<<grid(32ull * nq, 128), 128, 0, s>>>(
      a, a_off, nq, static_cast<const ChainRec*>(recs), cand, n_cand, div_in, div_off, rp,
      div_out, acc_out, good, n_good, n_rows, n_segs);
  return cudaGetLastError();
}

cudaError_t r2g_emit(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                     const R2GRowMeta* meta, const int64_t* read_ids, const void* recs,
                     const int32_t* good, const uint32_t* n_good, const uint64_t* chain_off,
                     const uint64_t* row_off, int32_t* tmp, cuflye_read_alignment* out,
                     cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  emit_kernel<<<grid(nq, 64), 64, 0, s>>>(a, a_off, nq, meta, read_ids,
                                          static_cast<const ChainRec*>(recs), good, n_good,
                                          chain_off, row_off, tmp, out);
  return cudaGetLastError();
}

cudaError_t r2g_records(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                        const R2GRowMeta* meta, const int64_t* query_ids, const int64_t* read_ids,
                        const void* recs, const int32_t* cand, const uint32_t* n_cand,
                        const uint64_t* rec_off, cuflye_chain_record* out, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  records_kernel<<<grid(32ull * nq, 128), 128, 0, s>>>(
      a, a_off, nq, meta, query_ids, read_ids, static_cast<const ChainRec*>(recs), cand, n_cand,
      rec_off, out);
  return cudaGetLastError();
}

}  // namespace cuflye
