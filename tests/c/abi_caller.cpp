// abi_caller.cpp — a compiled C++ caller of the C ABI through the Flye-side
// adapter (cuflye_gb300/flye/cuflye_flye.hpp), with small stand-ins for
// Flye's FastaRecord and KmerMatch.  Test infrastructure: the GPU tests run it
// and compare its output with the library's Python binding and the oracle.
//
//   abi_caller candidates READS.tsv K MIN_FREQ MAX_FREQ THREADS OUT.tsv
//       builds the index from the reads (id<TAB>sequence per line), then
//       THREADS worker threads take the reads as queries (read i goes to
//       thread i mod THREADS), each on its own context sharing the index, and
//       collect KmerMatches and filtered positions through the adapter's
//       callee.  Writes, read by read in input order,
//         C<TAB>query<TAB>query_pos<TAB>kmer<TAB>target<TAB>target_pos
//         F<TAB>query<TAB>pos
//   abi_caller overlaps READS.tsv K MIN_FREQ MAX_FREQ THREADS OUT.tsv
//       the same with the overlap rows of each query (overlap-range-v1
//       fields, the divergence as float bits)
//   abi_caller open
//       opens the device from the environment and prints OK or the error
//       (no GPU work; an invalid CUFLYE_CUDA_DEVICE fails before any call)
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "cuflye_flye.hpp"

namespace {

// Stand-ins for Flye's types: what the adapter uses of them.
struct Id {
  int64_t s = 0;
  int64_t signedId() const { return s; }
  bool strand() const { return s > 0; }
};
struct Sequence {
  std::string text;
  std::string str() const { return text; }
};
struct FastaRecord {
  Id id;
  Sequence sequence;
};
struct KmerMatch {
  KmerMatch(int32_t cur, int32_t ext, Id id, size_t kmer)
      : curPos(cur), extPos(ext), extId(id), kmerRepr(kmer) {}
  int32_t curPos;
  int32_t extPos;
  Id extId;
  size_t kmerRepr;
};

std::vector<FastaRecord> read_tsv(const char* path) {
  std::vector<FastaRecord> out;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty()) continue;
    const size_t tab = line.find('\t');
    if (tab == std::string::npos) throw std::runtime_error("bad reads line: " + line);
    FastaRecord r;
    r.id.s = std::stoll(line.substr(0, tab));
    r.sequence.text = line.substr(tab + 1);
    out.push_back(std::move(r));
  }
  return out;
}

uint32_t float_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, sizeof(u));
  return u;
}

int run(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "open") == 0) {
    cuflye_flye::Backend::instance();
    std::cout << "OK\n";
    return 0;
  }
  if (argc != 8) {
    std::cerr << "usage: abi_caller candidates|overlaps READS.tsv K MIN MAX THREADS OUT.tsv\n";
    return 2;
  }
  const std::string mode = argv[1];
  const std::vector<FastaRecord> reads = read_tsv(argv[2]);
  const int k = std::atoi(argv[3]);
  const uint32_t min_freq = static_cast<uint32_t>(std::atoi(argv[4]));
  const uint32_t max_freq = static_cast<uint32_t>(std::atoi(argv[5]));
  const int threads = std::max(1, std::atoi(argv[6]));
  std::vector<int64_t> ids;
  std::vector<std::string> seqs;
  for (const FastaRecord& r : reads) {
    ids.push_back(r.id.signedId());
    seqs.push_back(r.sequence.str());
  }
  cuflye_flye::Backend& be = cuflye_flye::Backend::instance();
  be.buildIndex(k, ids, seqs, min_freq, max_freq);
  cuflye_overlap_params params{};
  params.kmer_size = k;
  params.min_overlap = 1000;
  params.max_jump = 1500;
  params.max_gap = 500;
  params.gap_jump_threshold = 100;
  params.max_overhang = 1500;
  params.check_overhang = 1;
  params.force_local = 0;
  params.only_max_ext = 1;
  params.max_overlaps = 0;
  params.large_gap_penalty = 2.0f;
  params.small_gap_penalty = 0.5f;
  params.min_kmer_survival_rate = 0.01f;
  params.max_divergence = 1.0f;
  params.sample_rate = 1.0f;
  std::vector<std::string> text(reads.size());
  std::vector<std::string> errors(threads);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&, t]() {
      try {
        for (size_t i = static_cast<size_t>(t); i < reads.size(); i += threads) {
          std::ostringstream os;
          const FastaRecord& q = reads[i];
          if (mode == "candidates") {
            std::vector<KmerMatch> matches;
            std::vector<int32_t> filtered;
            cuflye_flye::collectCandidateMatches(q, matches, filtered,
                                                 [](int64_t s) { return Id{s}; });
            for (const KmerMatch& m : matches)
              os << "C\t" << q.id.signedId() << '\t' << m.curPos << '\t' << m.kmerRepr << '\t'
                 << m.extId.signedId() << '\t' << m.extPos << '\n';
            for (int32_t p : filtered) os << "F\t" << q.id.signedId() << '\t' << p << '\n';
          } else {
            for (const cuflye_overlap_range& r : cuflye_flye::collectOverlaps(q, params))
              os << r.cur_id << '\t' << r.cur_begin << '\t' << r.cur_end << '\t' << r.cur_len
                 << '\t' << r.ext_id << '\t' << r.ext_begin << '\t' << r.ext_end << '\t'
                 << r.ext_len << '\t' << r.score << '\t' << float_bits(r.seq_divergence) << '\n';
          }
          text[i] = os.str();
        }
      } catch (const std::exception& e) {
        errors[t] = e.what();
      }
    });
  }
  for (std::thread& th : pool) th.join();
  for (const std::string& e : errors)
    if (!e.empty()) throw std::runtime_error(e);
  std::ofstream out(argv[7]);
  for (const std::string& s : text) out << s;
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& e) {
    std::cout << "ERROR\t" << e.what() << '\n';
    return 1;
  }
}
