// cuflye_oracle.cpp — CPU restatement of the Flye overlap hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests compare the
// CUDA library against it, and the benchmark times it as the CPU baseline.  No
// product code path links, loads or calls it.
//
// It restates, in plain single-threaded C++ per query, the algorithm that the
// reference restates in its replay tools and CPU oracles:
//   * k-mer encoding / reverse complement / standard form
//       cuda/cuflye_cuda_read_window_smoke.cu:172-222
//   * candidate loop (repetitive -> filtered position, absent -> skip,
//     trivial self hit -> skip)
//       patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:53-95
//   * KmerMatch sort by (internal ext id, cur pos) with std::sort
//       patches/flye/2.9.6/0001-cuflye-candidate-dump.patch:86-92
//   * group prefilter, ext re-sort, chaining DP, score-ordered backtrack,
//     overlapTest, k-mer divergence, primary selection, max_overlaps
//       tools/replay_overlap_chains.py:196-422
//       tools/replay_read_to_graph_source_pack.py:95-181, 352-491
//       cuda/cuflye_cuda_overlap_chain_replay.cu:977-1015, 1493-1719
//   * read-to-graph input filter and curBegin sort
//       patches/flye/2.9.6/0039-cuflye-read-to-graph-input-boundary-oracle.patch:72-76, 226-251
//   * chainReadAlignments
//       cuda/cuflye_cuda_read_alignment_chain_replay.cu:872-984
//       tools/replay_read_alignment_chains.py:64-139
//   * complement chains appended after good chains
//       patches/flye/2.9.6/0037-cuflye-read-alignment-selected-cpu-bypass.patch:192-211
//
// Flye sorts with libstdc++ std::sort (not stable) at five places; the oracle
// calls std::sort itself at the same places, so equal keys land in the order
// libstdc++ gives them.  A "stable" mode swaps in std::stable_sort so the
// oracle can also be pinned against the reference's overlap replay, which
// uses Python's stable sort.  Each place can be switched on its own
// (orc_set_sort_mode), so the oracle can also reproduce the reference's C++
// CPU prototype, which re-sorts ext-sorted groups with std::sort but takes
// scores in stable order (cuda/cuflye_cuda_overlap_chain_replay.cu:905-911,
// 1587-1599, 1631-1635).
//
// Semantics the reference does not pin (Flye's VertexIndex is absent) and
// that this oracle defines, shared verbatim by the CUDA library:
//   * index: every k-mer window of every target's forward strand, keyed by
//     its standard form; a window whose k-mer is not standard is stored on the
//     reverse strand at (len - pos - k).  freq(key) = number of windows.
//     repetitive = freq > max_freq; solid = freq >= min_freq.  A bucket lists
//     its entries in ascending (stored internal id, stored pos).
//   * lookup with a non-standard query k-mer flips every entry to the other
//     strand: (id ^ 1, len - pos - k).
//   * chain base divergence = curRange-weighted mean of segment divergences.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// The five places Flye sorts, as bits of the stable-sort mask.
enum SortSite : unsigned {
  kSiteKmerMatch = 1,  // KmerMatch sort by (ext id, cur pos)
  kSiteExt = 2,        // ext-sorted group by ext pos
  kSiteScore = 4,      // backtrack starts by score
  kSitePrimary = 8,    // overlaps by score before primary selection
  kSiteChainIn = 16,   // read-to-graph alignments by cur begin
  kSiteAll = 31,
};
unsigned g_stable = 0;  // sites sorted with std::stable_sort; the rest std::sort (Flye)

template <class It, class Cmp>
void flyeSort(SortSite site, It first, It last, Cmp cmp) {
  if (g_stable & site)
    std::stable_sort(first, last, cmp);
  else
    std::sort(first, last, cmp);
}

inline uint64_t baseBits(char c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 0;
  }
}

inline uint64_t encodeKmer(const char* s, int k) {
  uint64_t r = 0;
  for (int i = 0; i < k; ++i) r = (r << 2) + baseBits(s[i]);
  return r;
}

inline uint64_t revComp(uint64_t x, int k) {
  uint64_t r = 0;
  for (int i = 0; i < k; ++i) {
    r = (r << 2) + (~x & 3ULL);
    x >>= 2;
  }
  return r;
}

inline uint32_t internalId(int64_t signedId) {
  return signedId > 0 ? static_cast<uint32_t>((signedId - 1) * 2)
                      : static_cast<uint32_t>((-signedId) * 2 - 1);
}

inline int64_t signedId(uint32_t internal) {
  return (internal & 1u) ? -static_cast<int64_t>((internal + 1) / 2)
                         : static_cast<int64_t>(internal / 2 + 1);
}

struct Bucket {
  uint64_t offset;
  uint32_t count;
  bool repetitive;
};

struct Index {
  int k = 0;
  bool transform = true;
  std::unordered_map<uint64_t, Bucket> table;
  std::vector<uint32_t> posId;
  std::vector<int32_t> posPos;
  std::unordered_map<uint32_t, int32_t> seqLen;  // forward internal id -> length
};

struct KmerMatch {
  int32_t curPos;
  int32_t extPos;
  uint32_t extId;
  uint64_t kmer;
};

struct Params {
  int32_t kmerSize;
  int32_t minOverlap;
  int32_t maxJump;
  int32_t maxGap;
  int32_t gapJumpThreshold;
  int32_t maxOverhang;
  int32_t checkOverhang;
  int32_t forceLocal;
  int32_t onlyMaxExt;
  int32_t maxOverlaps;
  float largeGapPenalty;
  float smallGapPenalty;
  float minKmerSurvivalRate;
  float maxDivergence;
  float sampleRate;
};

struct Overlap {
  int64_t curId;
  int32_t curBegin, curEnd, curLen;
  int64_t extId;
  int32_t extBegin, extEnd, extLen;
  int32_t score;
  int32_t chainLength;
  float seqDivergence;
};

// ---------------------------------------------------------------- index

Index* buildIndex(int k, int n, const int64_t* ids, const int64_t* offs,
                  const char* bases, uint32_t minFreq, uint32_t maxFreq) {
  struct Entry {
    uint64_t key;
    uint32_t id;
    int32_t pos;
  };
  Index* idx = new Index();
  idx->k = k;
  idx->transform = true;
  for (int t = 0; t < n; ++t) {
    uint32_t fid = internalId(ids[t]);
    int64_t len = offs[t + 1] - offs[t];
    idx->seqLen[fid] = static_cast<int32_t>(len);
    idx->seqLen[fid ^ 1u] = static_cast<int32_t>(len);
  }
  // Entries are unique, so (key, id, pos) is a total order and any correct
  // sort gives the same index: enumerate per thread, bucket by the key's top
  // bits, sort the buckets in parallel, concatenate in bucket order.
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 64) nt = 64;
  const int topBits = 2 * k >= 10 ? 10 : 2 * k;
  const size_t nb = size_t(1) << topBits;
  auto bucketOf = [&](uint64_t key) { return static_cast<size_t>(key >> (2 * k - topBits)); };
  std::vector<std::vector<Entry>> local(nt);
  {
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < nt; ++w)
      pool.emplace_back([&, w]() {
        for (int t = static_cast<int>(w); t < n; t += static_cast<int>(nt)) {
          uint32_t fid = internalId(ids[t]);
          int64_t len = offs[t + 1] - offs[t];
          const char* s = bases + offs[t];
          for (int64_t p = 0; p + k <= len; ++p) {
            uint64_t x = encodeKmer(s + p, k);
            uint64_t rc = revComp(x, k);
            if (rc < x)
              local[w].push_back({rc, fid ^ 1u, static_cast<int32_t>(len - p - k)});
            else
              local[w].push_back({x, fid, static_cast<int32_t>(p)});
          }
        }
      });
    for (auto& th : pool) th.join();
  }
  std::vector<size_t> bstart(nb + 1, 0);
  for (auto& v : local)
    for (const Entry& e : v) ++bstart[bucketOf(e.key) + 1];
  for (size_t b = 0; b < nb; ++b) bstart[b + 1] += bstart[b];
  std::vector<Entry> entries(bstart[nb]);
  {
    std::vector<size_t> fill(bstart.begin(), bstart.end() - 1);
    for (auto& v : local) {
      for (const Entry& e : v) entries[fill[bucketOf(e.key)]++] = e;
      std::vector<Entry>().swap(v);
    }
  }
  {
    std::atomic<size_t> next(0);
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < nt; ++w)
      pool.emplace_back([&]() {
        for (;;) {
          size_t b = next.fetch_add(1);
          if (b >= nb) break;
          std::sort(entries.begin() + bstart[b], entries.begin() + bstart[b + 1],
                    [](const Entry& a, const Entry& c) {
                      if (a.key != c.key) return a.key < c.key;
                      if (a.id != c.id) return a.id < c.id;
                      return a.pos < c.pos;
                    });
        }
      });
    for (auto& th : pool) th.join();
  }
  idx->table.reserve(bstart[nb] / 4 + 16);
  size_t i = 0;
  while (i < entries.size()) {
    size_t j = i;
    while (j < entries.size() && entries[j].key == entries[i].key) ++j;
    uint32_t freq = static_cast<uint32_t>(j - i);
    if (freq > maxFreq) {
      idx->table[entries[i].key] = {0, freq, true};
    } else if (freq >= minFreq) {
      idx->table[entries[i].key] = {idx->posId.size(), freq, false};
      for (size_t e = i; e < j; ++e) {
        idx->posId.push_back(entries[e].id);
        idx->posPos.push_back(entries[e].pos);
      }
    }
    i = j;
  }
  return idx;
}

// Explicit-entry index (the reference fixtures' flattened index.tsv): entries
// are already strand-resolved, so no transform is applied at lookup.
Index* indexFromEntries(int k, size_t n, const int64_t* targetIds,
                        const int64_t* pos, const uint64_t* keys, size_t nRep,
                        const uint64_t* repKeys) {
  Index* idx = new Index();
  idx->k = k;
  idx->transform = false;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return keys[a] < keys[b]; });
  size_t i = 0;
  while (i < n) {
    size_t j = i;
    while (j < n && keys[order[j]] == keys[order[i]]) ++j;
    idx->table[keys[order[i]]] = {idx->posId.size(), static_cast<uint32_t>(j - i), false};
    for (size_t e = i; e < j; ++e) {
      idx->posId.push_back(internalId(targetIds[order[e]]));
      idx->posPos.push_back(static_cast<int32_t>(pos[order[e]]));
    }
    i = j;
  }
  for (size_t r = 0; r < nRep; ++r) {
    auto it = idx->table.find(repKeys[r]);
    if (it == idx->table.end())
      idx->table[repKeys[r]] = {0, 0, true};
    else
      it->second.repetitive = true;
  }
  return idx;
}

// ---------------------------------------------------------------- candidates

// collectCandidateMatchesCpu: patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:53-95
void collectCandidates(const Index& idx, int64_t queryId, const char* seq,
                       int64_t len, std::vector<KmerMatch>& out,
                       std::vector<int32_t>& filtered) {
  const int k = idx.k;
  const uint32_t qid = internalId(queryId);
  for (int64_t p = 0; p + k <= len; ++p) {
    uint64_t x = encodeKmer(seq + p, k);
    uint64_t rc = revComp(x, k);
    bool revCmp = rc < x;
    uint64_t key = revCmp ? rc : x;
    auto it = idx.table.find(key);
    if (it != idx.table.end() && it->second.repetitive) {
      filtered.push_back(static_cast<int32_t>(p));
      continue;
    }
    if (it == idx.table.end() || it->second.count == 0) continue;
    const Bucket& b = it->second;
    for (uint64_t e = b.offset; e < b.offset + b.count; ++e) {
      uint32_t id = idx.posId[e];
      int32_t pos = idx.posPos[e];
      if (idx.transform && revCmp) {
        int32_t slen = idx.seqLen.at(id);
        id ^= 1u;
        pos = slen - pos - k;
      }
      if (id == qid && pos == p) continue;
      out.push_back({static_cast<int32_t>(p), pos, id, x});
    }
  }
}

void sortMatches(std::vector<KmerMatch>& m) {
  flyeSort(kSiteKmerMatch, m.begin(), m.end(), [](const KmerMatch& a, const KmerMatch& b) {
    return a.extId != b.extId ? a.extId < b.extId : a.curPos < b.curPos;
  });
}

// ---------------------------------------------------------------- chaining

int32_t lrOverhang(const Overlap& o) {
  return std::max(std::min(o.curBegin, o.extBegin),
                  std::min(o.curLen - o.curEnd, o.extLen - o.extEnd));
}

// overlapTest: tools/replay_overlap_chains.py:196-225
bool overlapTest(const Overlap& o, const Params& p) {
  int32_t cr = o.curEnd - o.curBegin, er = o.extEnd - o.extBegin;
  if (cr < p.minOverlap || er < p.minOverlap) return false;
  int32_t diff = std::abs(cr - er);
  if (static_cast<float>(diff) > 0.5f * static_cast<float>(std::min(cr, er))) return false;
  if (o.curId == o.extId) {
    int32_t inter = std::min(o.curEnd, o.extEnd) - std::max(o.curBegin, o.extBegin);
    if (static_cast<float>(inter) > static_cast<float>(cr) / 2.0f) return false;
  }
  if (o.curId == -o.extId) {
    int32_t inter = std::min(o.curEnd, o.extLen - o.extBegin) -
                    std::max(o.curBegin, o.extLen - o.extEnd);
    if (static_cast<float>(inter) > static_cast<float>(cr) / 2.0f) return false;
  }
  if (!p.forceLocal && p.checkOverhang && lrOverhang(o) > p.maxOverhang) return false;
  return true;
}

bool containedBy(const Overlap& a, const Overlap& b) {
  if (a.curId != b.curId || a.extId != b.extId) return false;
  return b.curBegin <= a.curBegin && a.curEnd <= b.curEnd &&
         b.extBegin <= a.extBegin && a.extEnd <= b.extEnd;
}

// k-mer divergence estimate: tools/replay_overlap_chains.py:348-360,
// cuda/cuflye_cuda_overlap_chain_replay.cu:1654-1670
float divergence(const Overlap& o, const std::vector<int32_t>& filtered, const Params& p,
                 bool* ok) {
  int32_t filteredCount = 0;
  auto lo = std::lower_bound(filtered.begin(), filtered.end(), o.curBegin);
  for (auto it = lo; it != filtered.end() && *it <= o.curEnd; ++it) ++filteredCount;
  int32_t norm = std::max(o.curEnd - o.curBegin, o.extEnd - o.extBegin) - filteredCount;
  *ok = norm > 0;
  float normLen = static_cast<float>(norm);
  float rate = static_cast<float>(o.chainLength) * p.sampleRate / normLen;
  rate = std::min(rate, 1.0f);
  return logf(1.0f / rate) / static_cast<float>(p.kmerSize);
}

// chain_target: tools/replay_overlap_chains.py:228-380 (std::sort at the
// ext re-sort, the score order and the ext-overlap order, as
// tools/replay_read_to_graph_source_pack.py:396, 440, 481 emulate).
void chainGroup(const KmerMatch* m, size_t n, int64_t queryId, int32_t curLen,
                int32_t extLen, const std::vector<int32_t>& filtered, const Params& p,
                std::vector<Overlap>& detected) {
  const int32_t k = p.kmerSize;
  uint32_t unique = 0;
  int32_t prev = 0;
  for (size_t i = 0; i < n; ++i)
    if (m[i].curPos != prev) {
      ++unique;
      prev = m[i].curPos;
    }
  if (static_cast<float>(unique) <
      p.minKmerSurvivalRate * static_cast<float>(p.minOverlap))
    return;
  int32_t minCur = m[0].curPos, maxCur = m[n - 1].curPos;
  int32_t minExt = m[0].extPos, maxExt = m[0].extPos;
  for (size_t i = 0; i < n; ++i) {
    minExt = std::min(minExt, m[i].extPos);
    maxExt = std::max(maxExt, m[i].extPos);
  }
  if (maxCur - minCur < p.minOverlap || maxExt - minExt < p.minOverlap) return;
  if (p.checkOverhang && !p.forceLocal) {
    if (std::min(minCur, minExt) > p.maxOverhang) return;
    if (std::min(curLen - maxCur, extLen - maxExt) > p.maxOverhang) return;
  }
  std::vector<KmerMatch> w(m, m + n);
  const bool extSorted = extLen > curLen;
  if (extSorted)
    flyeSort(kSiteExt, w.begin(), w.end(),
             [](const KmerMatch& a, const KmerMatch& b) { return a.extPos < b.extPos; });

  std::vector<int32_t> score(n, 0), bt(n, -1);
  for (size_t i = 1; i < n; ++i) {
    int32_t maxScore = 0, maxId = 0;
    const int32_t curNext = w[i].curPos, extNext = w[i].extPos;
    for (int64_t j = static_cast<int64_t>(i) - 1; j >= 0; --j) {
      const int32_t curDelta = curNext - w[j].curPos;
      const int32_t extDelta = extNext - w[j].extPos;
      const int32_t jumpDiv = std::abs(curDelta - extDelta);
      if (0 < curDelta && curDelta < p.maxJump && 0 < extDelta && extDelta < p.maxJump &&
          jumpDiv <= p.maxGap) {
        int32_t matchScore = std::min(std::min(curDelta, extDelta), k);
        float pen = jumpDiv > p.gapJumpThreshold ? p.largeGapPenalty : p.smallGapPenalty;
        int32_t gapCost = static_cast<int32_t>(pen * static_cast<float>(jumpDiv));
        int32_t next = score[j] + matchScore - gapCost;
        if (next > maxScore) {
          maxScore = next;
          maxId = static_cast<int32_t>(j);
          if (jumpDiv == 0 && curDelta < k) break;
        }
      }
      if (extSorted && extDelta > p.maxJump) break;
      if (!extSorted && curDelta > p.maxJump) break;
    }
    score[i] = std::max(maxScore, k);
    if (maxScore > k) bt[i] = maxId;
  }

  std::vector<int32_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = static_cast<int32_t>(i);
  flyeSort(kSiteScore, order.begin(), order.end(),
           [&](int32_t a, int32_t b) { return score[a] > score[b]; });

  std::vector<Overlap> ext;
  for (size_t oi = 0; oi < n; ++oi) {
    int32_t start = order[oi];
    if (bt[start] == -1) continue;
    int32_t last = start, first = 0, chainLen = 0, pos = start;
    while (pos != -1) {
      first = pos;
      ++chainLen;
      int32_t np = bt[pos];
      bt[pos] = -1;
      pos = np;
    }
    Overlap o;
    o.curId = queryId;
    o.curBegin = w[first].curPos;
    o.curEnd = w[last].curPos + k - 1;
    o.curLen = curLen;
    o.extId = signedId(w[0].extId);
    o.extBegin = w[first].extPos;
    o.extEnd = w[last].extPos + k - 1;
    o.extLen = extLen;
    o.score = score[last] - score[first] + k - 1;
    o.chainLength = chainLen;
    o.seqDivergence = 0.0f;
    if (!overlapTest(o, p)) continue;
    bool ok = true;
    o.seqDivergence = divergence(o, filtered, p, &ok);
    if (!ok) continue;
    ext.push_back(o);
  }
  flyeSort(kSitePrimary, ext.begin(), ext.end(),
           [](const Overlap& a, const Overlap& b) { return a.score > b.score; });
  std::vector<Overlap> primary;
  if (p.onlyMaxExt) {
    if (!ext.empty()) primary.push_back(ext[0]);
  } else {
    for (const Overlap& o : ext) {
      bool contained = false;
      for (const Overlap& pr : primary)
        if (containedBy(o, pr) && pr.score > o.score) {
          contained = true;
          break;
        }
      if (!contained) primary.push_back(o);
    }
  }
  for (const Overlap& o : primary)
    if (o.seqDivergence < p.maxDivergence) detected.push_back(o);
}

// Groups consecutive matches by ext id and applies the max_overlaps cutoff:
// tools/replay_overlap_chains.py:383-422.
void chainSorted(const std::vector<KmerMatch>& m, int64_t queryId, int32_t curLen,
                 const std::unordered_map<uint32_t, int32_t>& seqLen,
                 const std::vector<int32_t>& filtered, const Params& p,
                 std::vector<Overlap>& detected) {
  size_t s = 0;
  while (s < m.size()) {
    if (p.maxOverlaps && detected.size() >= static_cast<size_t>(p.maxOverlaps)) break;
    size_t e = s + 1;
    while (e < m.size() && m[e].extId == m[s].extId) ++e;
    int32_t extLen = seqLen.at(m[s].extId & ~1u);
    chainGroup(m.data() + s, e - s, queryId, curLen, extLen, filtered, p, detected);
    s = e;
  }
}

// ---------------------------------------------------------------- read-to-graph

struct EdgeAln {
  Overlap ovl;
  int64_t edgeId;
  int32_t leftNode, rightNode;
};

struct Chain {
  std::vector<int32_t> idx;
  int32_t score;
};

struct R2GParams {
  int32_t maxJump, maxReadOverlap, minOverlap, maxSeparation;
  int32_t longEdge, bigAln;
  float maxChainDivergence;
};

// cpuChainReadAlignments: cuda/cuflye_cuda_read_alignment_chain_replay.cu:872-984
std::vector<Chain> chainReadAlignments(const std::vector<EdgeAln>& a, const R2GParams& rp) {
  std::vector<Chain> active, frozen;
  for (size_t index = 0; index < a.size(); ++index) {
    const EdgeAln& cur = a[index];
    int32_t maxScore = 0, maxChain = -1;
    size_t numOutdated = 0;
    bool canExtend = cur.ovl.extBegin < rp.maxJump;
    bool canBeExtended = cur.ovl.extLen - cur.ovl.extEnd < rp.maxJump;
    if (canExtend) {
      for (size_t c = 0; c < active.size(); ++c) {
        const EdgeAln& prev = a[active[c].idx.back()];
        int32_t readDiff = cur.ovl.curBegin - prev.ovl.curEnd;
        int32_t gl = cur.ovl.extBegin, gr = prev.ovl.extLen - prev.ovl.extEnd;
        bool connected = prev.rightNode == cur.leftNode;
        if (connected && rp.maxJump > readDiff && readDiff > -rp.maxReadOverlap &&
            gl + gr < rp.maxJump) {
          int32_t jumpDiv = std::abs(readDiff - (gl + gr));
          int32_t gapCost = jumpDiv > 100 ? jumpDiv / 50 : 0;
          int32_t sc = active[c].score + cur.ovl.score - gapCost;
          if (sc > maxScore) {
            maxScore = sc;
            maxChain = static_cast<int32_t>(c);
          }
        }
        if (readDiff > rp.maxJump) ++numOutdated;
      }
    }
    if (maxChain != -1) {
      Chain next = active[maxChain];
      next.idx.push_back(static_cast<int32_t>(index));
      next.score = maxScore;
      active.push_back(next);
    } else if (canBeExtended) {
      active.push_back({{static_cast<int32_t>(index)}, cur.ovl.score});
    } else {
      frozen.push_back({{static_cast<int32_t>(index)}, cur.ovl.score});
    }
    if (numOutdated > active.size() / 2) {
      std::vector<Chain> na;
      for (const Chain& c : active) {
        const EdgeAln& prev = a[c.idx.back()];
        if (cur.ovl.curBegin - prev.ovl.curEnd > rp.maxJump)
          frozen.push_back(c);
        else
          na.push_back(c);
      }
      active.swap(na);
    }
  }
  active.insert(active.end(), frozen.begin(), frozen.end());
  std::stable_sort(active.begin(), active.end(),
                   [](const Chain& l, const Chain& r) { return l.score > r.score; });
  std::vector<Chain> accepted;
  for (const Chain& c : active) {
    const EdgeAln& f = a[c.idx.front()];
    const EdgeAln& l = a[c.idx.back()];
    if (l.ovl.curEnd - f.ovl.curBegin < rp.minOverlap) continue;
    bool overl = false;
    for (const Chain& e : accepted) {
      const EdgeAln& ef = a[e.idx.front()];
      const EdgeAln& el = a[e.idx.back()];
      int32_t rate = std::min(l.ovl.curEnd, el.ovl.curEnd) -
                     std::max(f.ovl.curBegin, ef.ovl.curBegin);
      if (rate > rp.maxSeparation) {
        overl = true;
        break;
      }
    }
    if (!overl) accepted.push_back(c);
  }
  return accepted;
}

float chainDivergence(const std::vector<EdgeAln>& a, const Chain& c) {
  float sum = 0.0f;
  float total = 0.0f;
  for (int32_t i : c.idx) {
    float r = static_cast<float>(a[i].ovl.curEnd - a[i].ovl.curBegin);
    sum = sum + a[i].ovl.seqDivergence * r;
    total = total + r;
  }
  return sum / total;
}

struct RaRow {
  int64_t chainId, segmentId, readId;
  int32_t readBegin, readEnd, readLen;
  int64_t edgeId, edgeSeqId;
  int32_t edgeBegin, edgeEnd, edgeLen, score;
  float div;
};

struct Graph {
  // keyed by forward edge-sequence internal id
  std::unordered_map<uint32_t, int64_t> seqToEdge;
  std::unordered_map<int64_t, std::pair<int32_t, int32_t>> edgeNodes;  // +e -> (L, R)
};

Overlap complementOverlap(const Overlap& o) {
  Overlap r = o;
  r.curBegin = o.curLen - o.curEnd - 1;
  r.curEnd = o.curLen - o.curBegin - 1;
  r.extBegin = o.extLen - o.extEnd - 1;
  r.extEnd = o.extLen - o.extBegin - 1;
  r.curId = -o.curId;
  r.extId = -o.extId;
  return r;
}

}  // namespace

// ================================================================ C interface

extern "C" {

struct orc_result {
  std::vector<KmerMatch> matches;   // generation order
  std::vector<int64_t> matchQuery;  // query signed id per match
  std::vector<int32_t> filtered;
  std::vector<int64_t> filteredQuery;
  std::vector<Overlap> overlaps;
  std::vector<RaRow> rows;
  std::vector<uint64_t> queryMatchCounts;
};

void orc_set_stable(int stable) { g_stable = stable ? kSiteAll : 0u; }

// mask: SortSite bits sorted stably (KmerMatch 1, ext 2, score 4, primary 8,
// read-to-graph input 16); the others use std::sort.
void orc_set_sort_mode(unsigned mask) { g_stable = mask & kSiteAll; }

void* orc_index_build(int k, int n, const int64_t* ids, const int64_t* offs,
                      const char* bases, uint32_t minFreq, uint32_t maxFreq) {
  return buildIndex(k, n, ids, offs, bases, minFreq, maxFreq);
}

void* orc_index_from_entries(int k, size_t n, const int64_t* targetIds, const int64_t* pos,
                             const uint64_t* keys, size_t nRep, const uint64_t* repKeys) {
  return indexFromEntries(k, n, targetIds, pos, keys, nRep, repKeys);
}

void orc_index_free(void* idx) { delete static_cast<Index*>(idx); }

uint64_t orc_index_positions(void* idx) { return static_cast<Index*>(idx)->posId.size(); }
uint64_t orc_index_keys(void* idx) { return static_cast<Index*>(idx)->table.size(); }

// Candidate records in generation order (before Flye's sort), plus filtered positions.
void* orc_candidates(void* vidx, int nq, const int64_t* qids, const int64_t* qoffs,
                     const char* qbases, int sorted) {
  const Index& idx = *static_cast<Index*>(vidx);
  orc_result* r = new orc_result();
  for (int q = 0; q < nq; ++q) {
    std::vector<KmerMatch> m;
    std::vector<int32_t> f;
    collectCandidates(idx, qids[q], qbases + qoffs[q], qoffs[q + 1] - qoffs[q], m, f);
    if (sorted) sortMatches(m);
    r->queryMatchCounts.push_back(m.size());
    for (auto& x : m) {
      r->matches.push_back(x);
      r->matchQuery.push_back(qids[q]);
    }
    for (auto x : f) {
      r->filtered.push_back(x);
      r->filteredQuery.push_back(qids[q]);
    }
  }
  return r;
}

// Explicit query windows (the kmer-join / kmer-encode fixture shape): each
// window carries its forward k-mer and its lookup key.
void* orc_candidates_windows(void* vidx, size_t n, const int64_t* qids, const int64_t* qpos,
                             const uint64_t* kmers, const uint64_t* keys) {
  const Index& idx = *static_cast<Index*>(vidx);
  orc_result* r = new orc_result();
  for (size_t w = 0; w < n; ++w) {
    auto it = idx.table.find(keys[w]);
    if (it != idx.table.end() && it->second.repetitive) {
      r->filtered.push_back(static_cast<int32_t>(qpos[w]));
      r->filteredQuery.push_back(qids[w]);
      continue;
    }
    if (it == idx.table.end() || it->second.count == 0) continue;
    uint32_t qid = internalId(qids[w]);
    for (uint64_t e = it->second.offset; e < it->second.offset + it->second.count; ++e) {
      if (idx.posId[e] == qid && idx.posPos[e] == qpos[w]) continue;
      r->matches.push_back({static_cast<int32_t>(qpos[w]), idx.posPos[e], idx.posId[e], kmers[w]});
      r->matchQuery.push_back(qids[w]);
    }
  }
  return r;
}

static void overlapsRange(const Index* idx, int q0, int q1, const int64_t* qids,
                          const int64_t* qoffs, const char* qbases, const Params* p,
                          std::vector<Overlap>* out) {
  for (int q = q0; q < q1; ++q) {
    std::vector<KmerMatch> m;
    std::vector<int32_t> f;
    int64_t len = qoffs[q + 1] - qoffs[q];
    collectCandidates(*idx, qids[q], qbases + qoffs[q], len, m, f);
    sortMatches(m);
    // detectedOverlaps is per getSeqOverlaps call, so max_overlaps counts per query
    std::vector<Overlap> detected;
    chainSorted(m, qids[q], static_cast<int32_t>(len), idx->seqLen, f, *p, detected);
    out->insert(out->end(), detected.begin(), detected.end());
  }
}

// Full overlap stage per query (getSeqOverlaps), optionally on several threads
// over queries.  Output order is query order, then Flye's emission order.
void* orc_overlaps(void* vidx, int nq, const int64_t* qids, const int64_t* qoffs,
                   const char* qbases, const Params* p, int threads) {
  const Index* idx = static_cast<Index*>(vidx);
  orc_result* r = new orc_result();
  if (threads <= 1) {
    overlapsRange(idx, 0, nq, qids, qoffs, qbases, p, &r->overlaps);
    return r;
  }
  std::vector<std::vector<Overlap>> parts(nq);
  std::vector<std::thread> pool;
  std::atomic_int cursor(0);
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      for (;;) {
        int q = cursor.fetch_add(1);
        if (q >= nq) break;
        overlapsRange(idx, q, q + 1, qids, qoffs, qbases, p, &parts[q]);
      }
    });
  for (auto& th : pool) th.join();
  for (auto& v : parts) r->overlaps.insert(r->overlaps.end(), v.begin(), v.end());
  return r;
}

// Chaining only, from candidate records already in Flye's sorted order (the
// overlap replay fixture shape).  targetLens is indexed by forward internal id.
void* orc_chain_sorted(size_t n, const int32_t* curPos, const int32_t* extPos,
                       const int64_t* extSigned, int64_t queryId, int32_t curLen,
                       size_t nt, const int64_t* targetIds, const int32_t* targetLens,
                       size_t nf, const int32_t* filteredPos, const Params* p) {
  std::vector<KmerMatch> m(n);
  for (size_t i = 0; i < n; ++i) m[i] = {curPos[i], extPos[i], internalId(extSigned[i]), 0};
  std::unordered_map<uint32_t, int32_t> lens;
  for (size_t t = 0; t < nt; ++t) lens[internalId(targetIds[t]) & ~1u] = targetLens[t];
  std::vector<int32_t> f(filteredPos, filteredPos + nf);
  std::sort(f.begin(), f.end());
  orc_result* r = new orc_result();
  chainSorted(m, queryId, curLen, lens, f, *p, r->overlaps);
  return r;
}

// Read-to-graph: quickSeqOverlaps -> input filter -> curBegin sort ->
// chainReadAlignments -> chain divergence -> good + complement chains.
// Edges: edgeIds[e] (> 0) owns edge sequence seqIds[e] (> 0) with nodes
// (left[e], right[e]); the complement edge -e runs right^1 -> left^1.
static void r2gRange(const Index* idx, const Graph* g, int q0, int q1, const int64_t* qids,
                     const int64_t* qoffs, const char* qbases, const Params* p,
                     const R2GParams* rp, std::vector<std::vector<RaRow>>* out) {
  for (int q = q0; q < q1; ++q) {
    std::vector<KmerMatch> m;
    std::vector<int32_t> f;
    int64_t len = qoffs[q + 1] - qoffs[q];
    collectCandidates(*idx, qids[q], qbases + qoffs[q], len, m, f);
    sortMatches(m);
    std::vector<Overlap> ovl;
    chainSorted(m, qids[q], static_cast<int32_t>(len), idx->seqLen, f, *p, ovl);
    std::vector<EdgeAln> alns;
    for (const Overlap& o : ovl) {
      if (!(o.extLen < rp->longEdge || std::min(o.curEnd - o.curBegin, o.extEnd - o.extBegin) > rp->bigAln))
        continue;
      uint32_t sid = internalId(o.extId);
      int64_t e = g->seqToEdge.at(sid & ~1u);
      auto nodes = g->edgeNodes.at(e);
      EdgeAln a;
      a.ovl = o;
      if (sid & 1u) {
        a.edgeId = -e;
        a.leftNode = nodes.second ^ 1;
        a.rightNode = nodes.first ^ 1;
      } else {
        a.edgeId = e;
        a.leftNode = nodes.first;
        a.rightNode = nodes.second;
      }
      alns.push_back(a);
    }
    flyeSort(kSiteChainIn, alns.begin(), alns.end(),
             [](const EdgeAln& x, const EdgeAln& y) { return x.ovl.curBegin < y.ovl.curBegin; });
    std::vector<Chain> chains = chainReadAlignments(alns, *rp);
    std::vector<const Chain*> good;
    for (const Chain& c : chains)
      if (chainDivergence(alns, c) < rp->maxChainDivergence) good.push_back(&c);
    std::vector<RaRow>& rows = (*out)[q];
    int64_t local = 0;
    for (const Chain* c : good) {
      int64_t seg = 0;
      for (int32_t i : c->idx) {
        const Overlap& o = alns[i].ovl;
        rows.push_back({local, seg++, o.curId, o.curBegin, o.curEnd, o.curLen, alns[i].edgeId,
                        o.extId, o.extBegin, o.extEnd, o.extLen, o.score, o.seqDivergence});
      }
      ++local;
    }
    for (const Chain* c : good) {
      int64_t seg = 0;
      for (auto it = c->idx.rbegin(); it != c->idx.rend(); ++it) {
        Overlap o = complementOverlap(alns[*it].ovl);
        rows.push_back({local, seg++, o.curId, o.curBegin, o.curEnd, o.curLen,
                        -alns[*it].edgeId, o.extId, o.extBegin, o.extEnd, o.extLen, o.score,
                        o.seqDivergence});
      }
      ++local;
    }
  }
}

void* orc_read_to_graph(void* vidx, int ne, const int64_t* edgeIds, const int64_t* seqIds,
                        const int32_t* left, const int32_t* right, int nq, const int64_t* qids,
                        const int64_t* qoffs, const char* qbases, const Params* p,
                        const R2GParams* rp, int threads) {
  const Index* idx = static_cast<Index*>(vidx);
  Graph g;
  for (int e = 0; e < ne; ++e) {
    g.seqToEdge[internalId(seqIds[e])] = edgeIds[e];
    g.edgeNodes[edgeIds[e]] = {left[e], right[e]};
  }
  std::vector<std::vector<RaRow>> parts(nq);
  if (threads <= 1) {
    r2gRange(idx, &g, 0, nq, qids, qoffs, qbases, p, rp, &parts);
  } else {
    std::atomic_int cursor(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
      pool.emplace_back([&]() {
        for (;;) {
          int q = cursor.fetch_add(1);
          if (q >= nq) break;
          r2gRange(idx, &g, q, q + 1, qids, qoffs, qbases, p, rp, &parts);
        }
      });
    for (auto& th : pool) th.join();
  }
  orc_result* r = new orc_result();
  int64_t base = 0;
  for (auto& v : parts) {
    int64_t maxLocal = -1;
    for (RaRow row : v) {
      maxLocal = std::max(maxLocal, row.chainId);
      row.chainId += base;
      r->rows.push_back(row);
    }
    base += maxLocal + 1;
  }
  return r;
}

// chainReadAlignments alone, on one read's EdgeOverlap rows (the reference
// read-alignment replay fixture shape).  Returns chains as flat
// (chain ordinal, overlap index) pairs in acceptance order.
size_t orc_chain_read_alignments(size_t n, const int32_t* readBegin, const int32_t* readEnd,
                                 const int32_t* edgeBegin, const int32_t* edgeEnd,
                                 const int32_t* edgeLen, const int32_t* score,
                                 const int32_t* leftNode, const int32_t* rightNode,
                                 const R2GParams* rp, int32_t* outChain, int32_t* outIndex,
                                 size_t cap) {
  std::vector<EdgeAln> a(n);
  for (size_t i = 0; i < n; ++i) {
    a[i].ovl = Overlap{};
    a[i].ovl.curBegin = readBegin[i];
    a[i].ovl.curEnd = readEnd[i];
    a[i].ovl.extBegin = edgeBegin[i];
    a[i].ovl.extEnd = edgeEnd[i];
    a[i].ovl.extLen = edgeLen[i];
    a[i].ovl.score = score[i];
    a[i].leftNode = leftNode[i];
    a[i].rightNode = rightNode[i];
  }
  std::vector<Chain> chains = chainReadAlignments(a, *rp);
  size_t w = 0;
  for (size_t c = 0; c < chains.size(); ++c)
    for (int32_t i : chains[c].idx) {
      if (w < cap) {
        outChain[w] = static_cast<int32_t>(c);
        outIndex[w] = i;
      }
      ++w;
    }
  return w;
}

// std::sort of plain (key, payload) pairs by key, to test the device sort.
void orc_std_sort_u64(size_t n, uint64_t* keys, uint32_t* payload) {
  std::vector<std::pair<uint64_t, uint32_t>> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = {keys[i], payload[i]};
  std::sort(v.begin(), v.end(), [](const std::pair<uint64_t, uint32_t>& a,
                                   const std::pair<uint64_t, uint32_t>& b) {
    return a.first < b.first;
  });
  for (size_t i = 0; i < n; ++i) {
    keys[i] = v[i].first;
    payload[i] = v[i].second;
  }
}

float orc_logf(float x) { return logf(x); }

// ---- result accessors
size_t orc_n_matches(void* r) { return static_cast<orc_result*>(r)->matches.size(); }
void orc_get_matches(void* vr, int64_t* qid, int32_t* cur, uint64_t* kmer, int64_t* ext,
                     int32_t* extPos) {
  orc_result* r = static_cast<orc_result*>(vr);
  for (size_t i = 0; i < r->matches.size(); ++i) {
    qid[i] = r->matchQuery[i];
    cur[i] = r->matches[i].curPos;
    kmer[i] = r->matches[i].kmer;
    ext[i] = signedId(r->matches[i].extId);
    extPos[i] = r->matches[i].extPos;
  }
}
size_t orc_n_filtered(void* r) { return static_cast<orc_result*>(r)->filtered.size(); }
void orc_get_filtered(void* vr, int64_t* qid, int32_t* pos) {
  orc_result* r = static_cast<orc_result*>(vr);
  for (size_t i = 0; i < r->filtered.size(); ++i) {
    qid[i] = r->filteredQuery[i];
    pos[i] = r->filtered[i];
  }
}
size_t orc_n_overlaps(void* r) { return static_cast<orc_result*>(r)->overlaps.size(); }
// 9 int64 columns + chain length + divergence
void orc_get_overlaps(void* vr, int64_t* cols, int32_t* chainLen, float* div) {
  orc_result* r = static_cast<orc_result*>(vr);
  for (size_t i = 0; i < r->overlaps.size(); ++i) {
    const Overlap& o = r->overlaps[i];
    int64_t* c = cols + 9 * i;
    c[0] = o.curId; c[1] = o.curBegin; c[2] = o.curEnd; c[3] = o.curLen;
    c[4] = o.extId; c[5] = o.extBegin; c[6] = o.extEnd; c[7] = o.extLen; c[8] = o.score;
    chainLen[i] = o.chainLength;
    div[i] = o.seqDivergence;
  }
}
size_t orc_n_rows(void* r) { return static_cast<orc_result*>(r)->rows.size(); }
// 12 int64 columns + divergence
void orc_get_rows(void* vr, int64_t* cols, float* div) {
  orc_result* r = static_cast<orc_result*>(vr);
  for (size_t i = 0; i < r->rows.size(); ++i) {
    const RaRow& w = r->rows[i];
    int64_t* c = cols + 12 * i;
    c[0] = w.chainId; c[1] = w.segmentId; c[2] = w.readId; c[3] = w.readBegin;
    c[4] = w.readEnd; c[5] = w.readLen; c[6] = w.edgeId; c[7] = w.edgeSeqId;
    c[8] = w.edgeBegin; c[9] = w.edgeEnd; c[10] = w.edgeLen; c[11] = w.score;
    div[i] = w.div;
  }
}
void orc_result_free(void* r) { delete static_cast<orc_result*>(r); }

}  // extern "C"
