// r2g.cu — read-to-graph chains: the per-read body of ReadAligner::alignReads
// after quickSeqOverlaps.
//
//   filter  : keep overlaps with extLen < LONG_EDGE or
//             min(curRange, extRange) > BIG_ALN
//             (patches/flye/2.9.6/0039-cuflye-read-to-graph-input-boundary-oracle.patch:72-76);
//   sort    : by curBegin with libstdc++ std::sort order (0039:249-251), done
//             by the segmented sort in sort.cu;
//   chain   : chainReadAlignments, one thread per read
//             (cuda/cuflye_cuda_read_alignment_chain_replay.cu:872-984);
//   accept  : chain divergence = curRange-weighted mean of segment
//             divergences (Flye's getChainBaseDivergence is not in the
//             reference; this is the definition the CPU oracle shares), kept
//             when below read_align_ovlp_divergence;
//   emit    : good chains, then their complements with reversed segment order
//             (patches/flye/2.9.6/0037-cuflye-read-alignment-selected-cpu-bypass.patch:192-211).
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

__global__ void compact_kernel(const OverlapRow* __restrict__ rows, uint64_t n,
                               const uint32_t* __restrict__ keep,
                               const uint64_t* __restrict__ pos, OverlapRow* __restrict__ out) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  out[pos[i]] = rows[i];
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

__global__ void permute_kernel(const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off,
                               uint32_t nq, const uint32_t* __restrict__ vals,
                               OverlapRow* __restrict__ out) {
  const uint32_t q = blockIdx.x;
  if (q >= nq) return;
  const uint64_t b = a_off[q], e = a_off[q + 1];
  for (uint64_t i = b + threadIdx.x; i < e; i += blockDim.x) out[i] = a[b + vals[i]];
}

struct EdgeView {
  int64_t edge;
  int32_t left, right;
};

__device__ __forceinline__ EdgeView edge_of(const R2GGraph& g, uint32_t ext_di) {
  const uint32_t slot = ext_di >> 1;
  const int64_t e = g.edge_of_slot[slot];
  const int32_t l = g.left_of_slot[slot], r = g.right_of_slot[slot];
  EdgeView v;
  if (ext_di & 1u) {
    v.edge = -e;
    v.left = r ^ 1;
    v.right = l ^ 1;
  } else {
    v.edge = e;
    v.left = l;
    v.right = r;
  }
  return v;
}

// Chain record: extending chain c appends a record whose parent is c's last
// record, so chains that share a prefix share records.
struct ChainRec {
  int32_t parent, idx, first, len, score;
};

__global__ void chain_kernel(const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off,
                             uint32_t nq, R2GGraph graph, R2GParams rp,
                             ChainRec* __restrict__ recs, int32_t* __restrict__ active,
                             int32_t* __restrict__ frozen, int32_t* __restrict__ good,
                             uint32_t* __restrict__ n_good, uint32_t* __restrict__ n_rows) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t b = a_off[q];
  const int32_t n = static_cast<int32_t>(a_off[q + 1] - b);
  const OverlapRow* A = a + b;
  ChainRec* R = recs + b;
  int32_t* act = active + b;
  int32_t* frz = frozen + b;
  int32_t* gd = good + b;
  int32_t na = 0, nf = 0, nr = 0;
  for (int32_t index = 0; index < n; ++index) {
    const OverlapRow cur = A[index];
    const EdgeView ce = edge_of(graph, cur.ext_di);
    int32_t max_score = 0, max_chain = -1;
    int32_t outdated = 0;
    const bool can_extend = cur.ext_begin < rp.max_jump;
    const bool can_be_extended = cur.ext_len - cur.ext_end < rp.max_jump;
    if (can_extend) {
      for (int32_t c = 0; c < na; ++c) {
        const ChainRec& ch = R[act[c]];
        const OverlapRow prev = A[ch.idx];
        const EdgeView pe = edge_of(graph, prev.ext_di);
        const int32_t read_diff = cur.cur_begin - prev.cur_end;
        const int32_t gl = cur.ext_begin, gr = prev.ext_len - prev.ext_end;
        if (pe.right == ce.left && rp.max_jump > read_diff && read_diff > -rp.max_read_overlap &&
            gl + gr < rp.max_jump) {
          const int32_t jd = abs(read_diff - (gl + gr));
          const int32_t gap = jd > 100 ? jd / 50 : 0;
          const int32_t sc = ch.score + cur.score - gap;
          if (sc > max_score) {
            max_score = sc;
            max_chain = c;
          }
        }
        if (read_diff > rp.max_jump) ++outdated;
      }
    }
    ChainRec r;
    r.idx = index;
    if (max_chain != -1) {
      const ChainRec& pr = R[act[max_chain]];
      r.parent = act[max_chain];
      r.first = pr.first;
      r.len = pr.len + 1;
      r.score = max_score;
      R[nr] = r;
      act[na++] = nr++;
    } else {
      r.parent = -1;
      r.first = index;
      r.len = 1;
      r.score = cur.score;
      R[nr] = r;
      if (can_be_extended)
        act[na++] = nr++;
      else
        frz[nf++] = nr++;
    }
    if (outdated > na / 2) {
      int32_t w = 0;
      for (int32_t c = 0; c < na; ++c) {
        const OverlapRow prev = A[R[act[c]].idx];
        if (cur.cur_begin - prev.cur_end > rp.max_jump)
          frz[nf++] = act[c];
        else
          act[w++] = act[c];
      }
      na = w;
    }
  }
  // all = active ++ frozen, stable by score descending (insertion sort into act)
  for (int32_t f = 0; f < nf; ++f) act[na + f] = frz[f];
  const int32_t nall = na + nf;
  for (int32_t i = 1; i < nall; ++i) {
    const int32_t v = act[i];
    const int32_t sv = R[v].score;
    int32_t j = i;
    while (j > 0 && R[act[j - 1]].score < sv) {
      act[j] = act[j - 1];
      --j;
    }
    act[j] = v;
  }
  // acceptance: min overlap and separation from already accepted chains
  int32_t nacc = 0;
  for (int32_t i = 0; i < nall; ++i) {
    const ChainRec& c = R[act[i]];
    const OverlapRow first = A[c.first], last = A[c.idx];
    if (last.cur_end - first.cur_begin < rp.min_overlap) continue;
    bool overl = false;
    for (int32_t t = 0; t < nacc && !overl; ++t) {
      const ChainRec& e = R[frz[t]];
      const OverlapRow ef = A[e.first], el = A[e.idx];
      const int32_t rate = min(last.cur_end, el.cur_end) - max(first.cur_begin, ef.cur_begin);
      overl = rate > rp.max_separation;
    }
    if (!overl) frz[nacc++] = act[i];  // frozen list is free now: reuse it
  }
  // chain divergence (segments in chain order) and the accept filter
  int32_t ngood = 0, segs = 0;
  for (int32_t t = 0; t < nacc; ++t) {
    const int32_t last = frz[t];
    const int32_t len = R[last].len;
    // walk back to fill the chain's segment list in forward order into act
    int32_t r = last;
    for (int32_t s = len - 1; s >= 0; --s) {
      act[s] = R[r].idx;
      r = R[r].parent;
    }
    float sum = 0.0f, total = 0.0f;
    for (int32_t s = 0; s < len; ++s) {
      const OverlapRow o = A[act[s]];
      const float rr = static_cast<float>(o.cur_end - o.cur_begin);
      sum = fadd(sum, fmul(o.div, rr));
      total = fadd(total, rr);
    }
    if (fdiv(sum, total) < rp.max_chain_divergence) {
      gd[ngood++] = last;
      segs += len;
    }
  }
  n_good[q] = static_cast<uint32_t>(ngood);
  n_rows[q] = static_cast<uint32_t>(2 * segs);
}

__device__ __forceinline__ void write_row(cuflye_read_alignment* out, int64_t chain,
                                          int64_t seg, const OverlapRow& o, int64_t read_id,
                                          int64_t edge, int64_t seq_signed, bool comp) {
  cuflye_read_alignment r;
  r.chain_id = chain;
  r.segment_id = seg;
  r.score = o.score;
  r.seq_divergence = o.div;
  r.read_len = o.cur_len;
  r.edge_len = o.ext_len;
  if (!comp) {
    r.read_id = read_id;
    r.edge_id = edge;
    r.edge_seq_id = seq_signed;
    r.read_begin = o.cur_begin;
    r.read_end = o.cur_end;
    r.edge_begin = o.ext_begin;
    r.edge_end = o.ext_end;
  } else {
    r.read_id = -read_id;
    r.edge_id = -edge;
    r.edge_seq_id = -seq_signed;
    r.read_begin = o.cur_len - o.cur_end - 1;
    r.read_end = o.cur_len - o.cur_begin - 1;
    r.edge_begin = o.ext_len - o.ext_end - 1;
    r.edge_end = o.ext_len - o.ext_begin - 1;
  }
  *out = r;
}

__global__ void emit_kernel(const OverlapRow* __restrict__ a, const uint64_t* __restrict__ a_off,
                            uint32_t nq, R2GGraph graph, const QueryInfo* __restrict__ qinfo,
                            const ChainRec* __restrict__ recs, const int32_t* __restrict__ good,
                            const uint32_t* __restrict__ n_good,
                            const uint64_t* __restrict__ chain_off,
                            const uint64_t* __restrict__ row_off, int32_t* __restrict__ tmp,
                            cuflye_read_alignment* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t b = a_off[q];
  const OverlapRow* A = a + b;
  const ChainRec* R = recs + b;
  const int32_t* gd = good + b;
  int32_t* T = tmp + b;
  const int32_t ng = static_cast<int32_t>(n_good[q]);
  const int64_t read_id = qinfo[q].signed_id;
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
        const OverlapRow o = A[ai];
        const EdgeView ev = edge_of(graph, o.ext_di);
        const int64_t seq = graph.slot_signed[o.ext_di >> 1];
        const int64_t seq_signed = (o.ext_di & 1u) ? -seq : seq;
        write_row(out + w, chain, s, o, read_id, ev.edge, seq_signed, pass == 1);
        ++w;
      }
    }
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
                        const uint64_t* pos, OverlapRow* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  compact_kernel<<<grid(n, 256), 256, 0, s>>>(rows, n, keep, pos, out);
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
                        const uint32_t* vals, OverlapRow* out, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  permute_kernel<<<nq, 128, 0, s>>>(a, a_off, nq, vals, out);
  return cudaGetLastError();
}

size_t r2g_rec_bytes() { return sizeof(ChainRec); }

cudaError_t r2g_chain(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                      const R2GGraph& g, const R2GParams& rp, void* recs, int32_t* active,
                      int32_t* frozen, int32_t* good, uint32_t* n_good, uint32_t* n_rows,
                      cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  chain_kernel<<<grid(nq, 64), 64, 0, s>>>(a, a_off, nq, g, rp, static_cast<ChainRec*>(recs),
                                           active, frozen, good, n_good, n_rows);
  return cudaGetLastError();
}

cudaError_t r2g_emit(const OverlapRow* a, const uint64_t* a_off, uint32_t nq, const R2GGraph& g,
                     const QueryInfo* qinfo, const void* recs, const int32_t* good,
                     const uint32_t* n_good, const uint64_t* chain_off, const uint64_t* row_off,
                     int32_t* tmp, cuflye_read_alignment* out, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  count_launch();
  emit_kernel<<<grid(nq, 64), 64, 0, s>>>(a, a_off, nq, g, qinfo,
                                          static_cast<const ChainRec*>(recs), good, n_good,
                                          chain_off, row_off, tmp, out);
  return cudaGetLastError();
}

}  // namespace cuflye
