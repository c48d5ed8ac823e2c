// cuflye_flye.hpp — the Flye-side adapter over the C ABI (include/cuflye.h).
//
// This header is what Flye's overlap code includes in place of the
// reference's CUDA adapter shell
// (patches/flye/2.9.6/0004-cuflye-cuda-adapter-shell.patch:117-300), which ran
// an external backend with std::system and parsed its TSV.  Here the
// candidate callee of patches/flye/2.9.6/0005-cuflye-real-data-pack-dump.patch:246-250
// calls libcuflye_gb300.so in process:
//
//   * Backend::instance() opens the device from CUFLYE_CUDA_DEVICE and
//     CUFLYE_CUDA_MEMORY_BUDGET_BYTES on first use (cuflye_open_from_env); a
//     failure throws std::runtime_error with the library's message, which
//     starts with the reference stub's fields (adapter=, CUFLYE_CUDA_DEVICE=,
//     CUFLYE_CUDA_MEMORY_BUDGET_BYTES=), so Flye fails fast as with the stub;
//   * Backend::buildIndex() uploads the reads once and builds the device
//     k-mer index (solid k-mers seen min_freq..max_freq times, repetitive
//     above max_freq);
//   * collectCandidateMatches() is the callee: it appends the query's
//     KmerMatches in Flye's generation order and its repetitive window
//     positions (curFilteredPos).  Flye runs it from many worker threads;
//     each thread gets a context of its own that shares the index
//     (cuflye_open_shared), so calls run side by side on the device;
//   * collectOverlaps() returns the whole of getSeqOverlaps for a query
//     (overlap-range-v1 rows) for callers that take the seam one level up.
//
// Output buffers grow on CUFLYE_ERR_CAPACITY and the call is repeated, the
// two-call pattern of the C ABI.  Nothing here falls back to the CPU: every
// failure throws.
//
// The header is templated on Flye's types (FastaRecord with .id.signedId()
// and .sequence.str(); a matches container with emplace_back(curPos, extPos,
// extId, kmerRepr)), so it compiles inside Flye and against the small stand-ins
// of the tests.
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "cuflye.h"

namespace cuflye_flye {

inline std::string last_error(const cuflye_ctx* c) {
  const char* m = cuflye_last_error(c);
  return m ? std::string(m) : std::string();
}

[[noreturn]] inline void fail(const std::string& what, cuflye_status st, const cuflye_ctx* c) {
  throw std::runtime_error(what + " failed (status " + std::to_string(static_cast<int>(st)) +
                           "): " + last_error(c));
}

// The device, the index over Flye's reads, and one context per calling thread.
class Backend {
 public:
  static Backend& instance() {
    static Backend b;
    return b;
  }

  Backend(const Backend&) = delete;
  Backend& operator=(const Backend&) = delete;

  // The index over the reads (ids as FastaRecord::Id::signedId(), forward
  // strands, ids > 0).  Call before any query; it closes the threads'
  // contexts of an earlier index.
  void buildIndex(int k, const std::vector<int64_t>& ids, const std::vector<std::string>& seqs,
                  uint32_t min_freq, uint32_t max_freq) {
    std::lock_guard<std::mutex> lock(mu_);
    closeThreadContexts();
    std::vector<int64_t> offs(ids.size() + 1, 0);
    std::string bases;
    for (size_t i = 0; i < seqs.size(); ++i) offs[i + 1] = offs[i] + seqs[i].size();
    bases.reserve(offs.back());
    for (const std::string& s : seqs) bases += s;
    const cuflye_status st = cuflye_index_build(owner_, k, ids.size(), ids.data(), offs.data(),
                                                bases.data(), min_freq, max_freq);
    if (st != CUFLYE_OK) fail("cuflye_index_build", st, owner_);
    k_ = k;
  }

  int k() const { return k_; }

  // The calling thread's context (shared index); opened on first use.
  cuflye_ctx* threadContext() {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = threads_.find(std::this_thread::get_id());
    if (it != threads_.end()) return it->second;
    cuflye_ctx* c = nullptr;
    const cuflye_status st = cuflye_open_shared(owner_, thread_budget_, &c);
    if (st != CUFLYE_OK) fail("cuflye_open_shared", st, c ? c : owner_);
    threads_[std::this_thread::get_id()] = c;
    return c;
  }

  // Device memory each thread's context may hold (0 = unbounded).
  void setThreadBudget(uint64_t bytes) { thread_budget_ = bytes; }

  ~Backend() {
    closeThreadContexts();
    cuflye_close(owner_);
  }

 private:
  Backend() {
    const cuflye_status st = cuflye_open_from_env(&owner_);
    if (st != CUFLYE_OK) throw std::runtime_error(last_error(nullptr));
  }

  void closeThreadContexts() {
    for (auto& kv : threads_) cuflye_close(kv.second);
    threads_.clear();
  }

  cuflye_ctx* owner_ = nullptr;
  std::mutex mu_;
  std::map<std::thread::id, cuflye_ctx*> threads_;
  uint64_t thread_budget_ = 0;
  int k_ = 0;
};

// Per-thread output buffers of the adapter, grown on demand.
struct Buffers {
  std::vector<cuflye_candidate> cand = std::vector<cuflye_candidate>(16);
  std::vector<cuflye_filtered_pos> filt = std::vector<cuflye_filtered_pos>(16);
  std::vector<cuflye_overlap_range> ovl = std::vector<cuflye_overlap_range>(16);
};

inline Buffers& threadBuffers() {
  static thread_local Buffers b;
  return b;
}

// The candidate callee: appends the query's KmerMatches (generation order:
// window order, then bucket order) and its repetitive window positions.
// idFromSigned turns a signed target id into Flye's FastaRecord::Id.
template <class FastaRecord, class Matches, class IdFromSigned>
void collectCandidateMatches(const FastaRecord& query, Matches& matches,
                             std::vector<int32_t>& curFilteredPos, IdFromSigned idFromSigned) {
  cuflye_ctx* c = Backend::instance().threadContext();
  Buffers& b = threadBuffers();
  const int64_t qid = query.id.signedId();
  const std::string seq = query.sequence.str();
  const int64_t offs[2] = {0, static_cast<int64_t>(seq.size())};
  size_t n = 0, nf = 0;
  for (;;) {
    const cuflye_status st = cuflye_candidates(c, 1, &qid, offs, seq.data(), b.cand.data(),
                                               b.cand.size(), &n, b.filt.data(), b.filt.size(),
                                               &nf);
    if (st == CUFLYE_ERR_CAPACITY) {
      if (n > b.cand.size()) b.cand.resize(n);
      if (nf > b.filt.size()) b.filt.resize(nf);
      continue;
    }
    if (st != CUFLYE_OK) fail("cuflye_candidates", st, c);
    break;
  }
  for (size_t i = 0; i < n; ++i) {
    const cuflye_candidate& r = b.cand[i];
    matches.emplace_back(r.query_pos, r.target_pos, idFromSigned(r.target_id),
                         static_cast<size_t>(r.kmer));
  }
  for (size_t i = 0; i < nf; ++i) curFilteredPos.push_back(b.filt[i].pos);
}

// getSeqOverlaps for one query: its overlap-range-v1 rows in Flye's order.
template <class FastaRecord>
std::vector<cuflye_overlap_range> collectOverlaps(const FastaRecord& query,
                                                  const cuflye_overlap_params& params) {
  cuflye_ctx* c = Backend::instance().threadContext();
  Buffers& b = threadBuffers();
  const int64_t qid = query.id.signedId();
  const std::string seq = query.sequence.str();
  const int64_t offs[2] = {0, static_cast<int64_t>(seq.size())};
  size_t n = 0;
  for (;;) {
    const cuflye_status st = cuflye_overlaps(c, 1, &qid, offs, seq.data(), &params, b.ovl.data(),
                                             b.ovl.size(), &n);
    if (st == CUFLYE_ERR_CAPACITY) {
      b.ovl.resize(n);
      continue;
    }
    if (st != CUFLYE_OK) fail("cuflye_overlaps", st, c);
    break;
  }
  return std::vector<cuflye_overlap_range>(b.ovl.begin(), b.ovl.begin() + n);
}

}  // namespace cuflye_flye
