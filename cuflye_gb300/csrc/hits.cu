// hits.cu — candidate hit generation (the candidate loop of getSeqOverlaps).
//
// Per query window, in the order of
// patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:55-89:
//   repetitive k-mer  -> the window position becomes a filtered position;
//   absent k-mer      -> nothing;
//   otherwise every bucket entry, flipped to the other strand when the query
//   k-mer is not in standard form, except the exact self hit.
// hits_count() probes the table once per window and records the bucket and
// the number of hits; an exclusive scan turns counts into offsets, and
// hits_emit() writes each window's hits at its offset, so the output is in
// Flye's generation order (window order, then bucket order) with no atomics.
#include <cstdint>

#include "common.cuh"
#include "kernels.h"

namespace cuflye {
namespace {


__device__ __forceinline__ uint32_t query_of(const uint64_t* __restrict__ win_off, uint32_t nq,
                                             uint64_t w) {
  uint32_t lo = 0, hi = nq - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (__ldg(win_off + mid) <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

struct WindowKmer {
  uint64_t x;    // forward k-mer (Kmer::numRepr)
  uint64_t key;  // standard form
  bool rev;      // x is not in standard form
};

__device__ __forceinline__ WindowKmer window_kmer(const QueryBatch& q, uint32_t qi, uint64_t p,
                                                  int k) {
  WindowKmer w;
  w.x = kmer_at(q.words, q.base_off[qi] + p, k);
  const uint64_t rc = revcomp(w.x, k);
  w.rev = rc < w.x;
  w.key = w.rev ? rc : w.x;
  return w;
}

__global__ void count_kernel(DeviceIndex idx, QueryBatch q, uint32_t* __restrict__ cnt,
                             uint32_t* __restrict__ filt, uint64_t* __restrict__ wmeta,
                             uint8_t* __restrict__ wflags, uint32_t* __restrict__ q_tie,
                             uint32_t* __restrict__ wself) {
  const uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= q.nwin) return;
  const uint32_t qi = query_of(q.win_off, q.nq, w);
  const uint64_t p = w - q.win_off[qi];
  const WindowKmer km = window_kmer(q, qi, p, idx.k);
  bool found;
  const uint64_t meta = table_probe(idx.table, idx.cap, km.key, &found);
  uint32_t c = 0;
  uint8_t fl = km.rev ? kWinRev : 0;
  if (found && (meta & kRepetitiveBit)) {
    fl |= kWinFiltered;
  } else if (found) {
    c = static_cast<uint32_t>((meta >> 40) & ((1ULL << kCountBits) - 1));
    if ((meta & kDupIdsBit) && q_tie[qi] == 0) atomicOr(q_tie + qi, 1u);
    const int32_t qdi = q.qdi[qi];
    if (c > 0 && qdi >= 0) {
      // Is the query's own window among the bucket entries?  Stored form of
      // the self hit: (qdi, p), or flipped when the lookup flips.
      uint64_t want;
      if (idx.transform && km.rev) {
        const uint32_t sid = static_cast<uint32_t>(qdi) ^ 1u;
        const int32_t slen = idx.slot_len[sid >> 1];
        const int64_t sp = static_cast<int64_t>(slen) - static_cast<int64_t>(p) - idx.k;
        want = sp >= 0 ? ((static_cast<uint64_t>(sid) << 32) | static_cast<uint32_t>(sp)) : ~0ULL;
      } else {
        want = (static_cast<uint64_t>(qdi) << 32) | static_cast<uint32_t>(p);
      }
      const uint64_t off = meta & kOffsetMask;
      uint32_t self_hits = 0;
      if (idx.transform) {
        // built buckets are sorted by (stored id, stored position), entries
        // unique.  A query that is an indexed target finds its own entry
        // where the index recorded it (checked: a query sequence that
        // differs from the indexed one searches as any other)
        bool known = false;
        uint32_t at = 0;
        if (idx.self_at && !(qdi & 1)) {
          const uint32_t slot = static_cast<uint32_t>(qdi) >> 1;
          const uint64_t w0 = idx.win_off[slot];
          if (w0 + p < idx.win_off[slot + 1]) {
            const uint32_t g = idx.self_at[w0 + p];
            if (g < c && __ldg(idx.pos + off + g) == want) {
              known = true;
              at = g;
            }
          }
        }
        if (!known) {
          uint32_t lo = 0, hi = c;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(idx.pos + off + mid) < want)
              lo = mid + 1;
            else
              hi = mid;
          }
          known = lo < c && __ldg(idx.pos + off + lo) == want;
          at = lo;
        }
        self_hits = known ? 1u : 0u;
        if (self_hits && wself) wself[w] = at;
      } else {
        // explicit entries keep input order and may repeat
        for (uint32_t e = 0; e < c; ++e) self_hits += __ldg(idx.pos + off + e) == want;
      }
      if (self_hits) {
        c -= self_hits;
        fl |= kWinTrivial;
      }
    }
  }
  cnt[w] = c;
  filt[w] = (fl & kWinFiltered) ? 1u : 0u;
  wmeta[w] = meta;
  wflags[w] = fl;
}

// A warp owns 32 consecutive windows (lane L <-> window w0 + L) and writes
// their hits one window at a time with all lanes, so that each store covers
// up to 32 consecutive records of one window.
__global__ void emit_kernel(DeviceIndex idx, QueryBatch q, const uint64_t* __restrict__ hit_off,
                            const uint64_t* __restrict__ filt_off,
                            const uint64_t* __restrict__ wmeta,
                            const uint8_t* __restrict__ wflags, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ vals, uint64_t* __restrict__ kmers,
                            int32_t* __restrict__ fpos) {
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  uint8_t fl = 0;
  uint32_t qi = 0, p = 0;
  uint64_t o = 0, end = 0, meta = 0;
  if (w < q.nwin) {
    fl = wflags[w];
    qi = query_of(q.win_off, q.nq, w);
    p = static_cast<uint32_t>(w - q.win_off[qi]);
    if (fl & kWinFiltered) {
      fpos[filt_off[w]] = static_cast<int32_t>(p);
    } else {
      o = hit_off[w];
      end = hit_off[w + 1];
      meta = wmeta[w];
    }
  }
  unsigned todo = __ballot_sync(0xffffffffu, end > o);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1;
    const uint64_t wo = __shfl_sync(0xffffffffu, o, src);
    const uint64_t wm = __shfl_sync(0xffffffffu, meta, src);
    const uint32_t wq = __shfl_sync(0xffffffffu, qi, src);
    const uint32_t wp = __shfl_sync(0xffffffffu, p, src);
    const uint32_t wf = __shfl_sync(0xffffffffu, static_cast<uint32_t>(fl), src);
    const uint64_t off = wm & kOffsetMask;
    const uint32_t c = static_cast<uint32_t>((wm >> 40) & ((1ULL << kCountBits) - 1));
    const bool flip = idx.transform && (wf & kWinRev);
    const int32_t qdi = q.qdi[wq];
    uint64_t x = 0;
    if (kmers) x = kmer_at(q.words, q.base_off[wq] + wp, idx.k);
    uint64_t out = wo;
    for (uint32_t e0 = 0; e0 < c; e0 += 32) {
      const uint32_t e = e0 + lane;
      bool keep = e < c;
      uint32_t id = 0;
      int32_t pos = 0;
      if (keep) {
        const uint64_t sv = __ldg(idx.pos + off + e);
        id = static_cast<uint32_t>(sv >> 32);
        pos = static_cast<int32_t>(sv & 0xffffffffu);
        if (flip) {
          pos = idx.slot_len[id >> 1] - pos - idx.k;
          id ^= 1u;
        }
        keep = !(static_cast<int32_t>(id) == qdi && pos == static_cast<int32_t>(wp));
      }
      const unsigned km = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const uint64_t d = out + __popc(km & lt);
        keys[d] = (static_cast<uint64_t>(id) << 32) | wp;
        vals[d] = static_cast<uint32_t>(pos);
        if (kmers) kmers[d] = x;
      }
      out += __popc(km);
    }
  }
}

__global__ void gather_kernel(const uint64_t* __restrict__ win_off,
                              const uint64_t* __restrict__ wl_off, uint32_t nq,
                              uint64_t* __restrict__ q_off) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nq) return;
  q_off[i] = wl_off[win_off[i]];
}

}  // namespace

cudaError_t hits_count(const DeviceIndex& idx, const QueryBatch& q, uint32_t* cnt,
                       uint32_t* filt, uint64_t* wmeta, uint8_t* wflags, uint32_t* q_tie,
                       uint32_t* wself, cudaStream_t s) {
  if (q.nwin == 0) return cudaSuccess;
  count_launch();
  count_kernel<<<static_cast<unsigned>((q.nwin + 255) / 256), 256, 0, s>>>(
      idx, q, cnt, filt, wmeta, wflags, q_tie, wself);
  return cudaGetLastError();
}

cudaError_t hits_emit(const DeviceIndex& idx, const QueryBatch& q, const uint64_t* hit_off,
                      const uint64_t* filt_off, const uint64_t* wmeta, const uint8_t* wflags,
                      uint64_t* keys, uint32_t* vals, uint64_t* kmers, int32_t* fpos,
                      cudaStream_t s) {
  if (q.nwin == 0) return cudaSuccess;
  count_launch();
  emit_kernel<<<static_cast<unsigned>((q.nwin + 255) / 256), 256, 0, s>>>(
      idx, q, hit_off, filt_off, wmeta, wflags, keys, vals, kmers, fpos);
  return cudaGetLastError();
}

cudaError_t gather_query_offsets(const uint64_t* win_off, const uint64_t* wl_off, uint32_t nq,
                                 uint64_t* q_off, cudaStream_t s) {
  count_launch();
  gather_kernel<<<(nq + 1 + 255) / 256, 256, 0, s>>>(win_off, wl_off, nq, q_off);
  return cudaGetLastError();
}

}  // namespace cuflye
