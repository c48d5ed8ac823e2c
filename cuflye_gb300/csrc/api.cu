// api.cu — host orchestration behind the C ABI (include/cuflye.h).
//
// One context = one device, one stream, one device arena (named buffers that
// grow and are reused across calls, like the reference's DeviceBuffer
// ensureCapacity arena in cuda/cuflye_cuda_raii.hpp:27-114), a resident
// k-mer index and an optional assembly graph.  Queries are processed in
// passes: every pass runs hit counting, an exclusive scan and hit emission
// for a contiguous run of queries, then the libstdc++-order match sort and
// the chaining stages, all on the context's stream; the host only reads back
// the sizes it needs to size the next stage's buffers.  A pass that would
// exceed the memory budget keeps the longest prefix of its queries whose hits
// fit, and a pass whose later stages do not fit runs again on half of its
// queries; a single query that does not fit fails with CUFLYE_ERR_BUDGET
// (records are never truncated, docs/abi/candidate-record-v1.md:105-118).
#include <dlfcn.h>

#include <algorithm>
#include <cerrno>
#include <climits>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/cuflye.h"
#include "kernels.h"
#include "r2g.h"

namespace cuflye {

struct Error : std::runtime_error {
  cuflye_status code;
  Error(cuflye_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CUFLYE_CHECK(call)                                                                \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      throw Error(CUFLYE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

}  // namespace cuflye

using namespace cuflye;

struct cuflye_ctx {
  int device = 0;
  uint64_t budget = 0;  // 0 = unbounded
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  std::mutex mu;
  std::string err;
  std::map<std::string, DevBuf> bufs;
  uint64_t in_use = 0, peak = 0;
  DeviceStatus* status = nullptr;
  // index
  bool has_index = false;
  DeviceIndex idx;
  std::unordered_map<int64_t, uint32_t> slot_of;  // |signed id| -> slot
  std::vector<int64_t> slot_signed_h;
  // graph
  bool has_graph = false;
  // logf exception table
  LogfTable logt{};
  size_t queries_per_pass = 0;
  // timing
  cudaEvent_t ev[8]{};
  // the segmented sort's side streams and its fork / rounds-done / join events
  cudaStream_t side = nullptr, side2 = nullptr;
  cudaEvent_t side_ev[4]{};
  double stage_ms[7]{};
  uint64_t stage_bytes[7]{};
  uint64_t sort_stats[8]{};  // see cuflye_last_sort_stats ([7]: emission fallbacks)
  // hits of the last call by path, for the stages' algorithmic bytes
  uint64_t hits_sorted_emission = 0, hits_flagged = 0, hits_prefiltered = 0, hits_emit_sort = 0;
  unsigned long long emit_tally[2]{};  // a pass's flagged and prefiltered hits, read back
  uint64_t passes = 0;       // see cuflye_last_passes
  uint64_t build_window_cap = 0;  // see cuflye_set_index_build_windows
  cuflye_launch_shape shape{0, 0, 0, 0};  // see cuflye_set_launch_shape (0: defaults)
  uint64_t build_ranges = 0;      // key ranges of the last index build
  int servers = 0;           // open serving loops and shared contexts borrowing this index
  cuflye_ctx* lender = nullptr;  // the context whose index this one borrows (cuflye_open_shared)
  int sorted_emission = 1;  // see cuflye_set_sorted_emission
  double other_per_hit = 0;  // a pass body's buffers beyond the per-hit ones, per hit
  std::map<std::string, uint64_t> pass_need;  // bytes each buffer was asked for in this pass
  uint64_t pass_retries = 0;   // passes of the last call run again on half their queries
  uint64_t pass_hit_cap = 0;   // hits a pass may take after a retry in this call (0: no cap)
  double alloc_ms = 0;         // host time of the last call in cudaMalloc / cudaFree
  uint64_t emission_fallbacks = 0;  // passes of the last call that fell back to emit + sort
};

namespace {

constexpr int kStages = 7;
constexpr int kSortStats = 7;

template <typename T>
T* buf(cuflye_ctx* c, const std::string& name, uint64_t count) {
  const size_t bytes = std::max<size_t>(static_cast<size_t>(count) * sizeof(T), 16);
  uint64_t& need = c->pass_need[name];
  need = std::max<uint64_t>(need, bytes);
  DevBuf& b = c->bufs[name];
  if (b.cap >= bytes) return static_cast<T*>(b.p);
  // grow by half, or under a budget that has no room for that, by an eighth
  // if there is room for that (fewer reallocations from pass to pass)
  size_t want = std::max(bytes, b.cap + b.cap / 2);
  if (c->budget && c->in_use - b.cap + want > c->budget) want = bytes + bytes / 8;
  if (c->budget && c->in_use - b.cap + want > c->budget) {
    if (c->in_use - b.cap + bytes > c->budget)
      throw Error(CUFLYE_ERR_BUDGET,
                  "device memory budget exceeded: buffer '" + name + "' needs " +
                      std::to_string(bytes) + " bytes; in use " + std::to_string(c->in_use) +
                      " of CUFLYE_CUDA_MEMORY_BUDGET_BYTES=" + std::to_string(c->budget));
  }
  const size_t alloc = (c->budget && c->in_use - b.cap + want > c->budget) ? bytes : want;
  const auto t0 = std::chrono::steady_clock::now();
  struct AllocTimer {
    cuflye_ctx* c;
    std::chrono::steady_clock::time_point t0;
    ~AllocTimer() {
      c->alloc_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                               t0).count();
    }
  } timer{c, t0};
  if (b.p) CUFLYE_CHECK(cudaFree(b.p));
  c->in_use -= b.cap;
  b.p = nullptr;
  b.cap = 0;
  cudaError_t e = cudaMalloc(&b.p, alloc);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(CUFLYE_ERR_BUDGET, "cudaMalloc of " + std::to_string(alloc) + " bytes for '" +
                                       name + "' failed: " + cudaGetErrorString(e));
  }
  b.cap = alloc;
  c->in_use += alloc;
  c->peak = std::max(c->peak, c->in_use);
  return static_cast<T*>(b.p);
}

void release(cuflye_ctx* c, const std::string& name) {
  auto it = c->bufs.find(name);
  if (it == c->bufs.end()) return;
  const auto t0 = std::chrono::steady_clock::now();
  if (it->second.p) cudaFree(it->second.p);
  c->alloc_ms +=
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  c->in_use -= it->second.cap;
  c->bufs.erase(it);
}

void sync(cuflye_ctx* c) { CUFLYE_CHECK(cudaStreamSynchronize(c->stream)); }

template <typename T>
T read_scalar(cuflye_ctx* c, const T* dev) {
  T v;
  CUFLYE_CHECK(cudaMemcpyAsync(&v, dev, sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  return v;
}

void check_device_status(cuflye_ctx* c) {
  DeviceStatus st;
  CUFLYE_CHECK(cudaMemcpyAsync(&st, c->status, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  if (st.code == kDevOk) return;
  CUFLYE_CHECK(cudaMemsetAsync(c->status, 0, sizeof(DeviceStatus), c->stream));
  switch (st.code) {
    case kDevProposalOverflow:
      throw Error(CUFLYE_ERR_UNSUPPORTED,
                  "unsupported shape: a target group produced more than 64 overlap proposals "
                  "(group " + std::to_string(st.detail) + ")");
    case kDevLogDomain:
      throw Error(CUFLYE_ERR_UNSUPPORTED,
                  "unsupported shape: divergence argument outside [1, 2^24)");
    case kDevTableFull:
      throw Error(CUFLYE_ERR_CUDA, "k-mer table insertion failed (table full)");
    case kDevMatchDict:
      throw Error(CUFLYE_ERR_CUDA, "sorted emission: a hit outside its query's dictionary "
                                   "(detail " + std::to_string(st.detail) + ")");
    default:
      throw Error(CUFLYE_ERR_CUDA, "device status " + std::to_string(st.code));
  }
}

// Exclusive scan with out[n] = total, left on the device.
void scan_u32_async(cuflye_ctx* c, const uint32_t* in, uint64_t* out, uint64_t n,
                    const char* temp_name) {
  uint64_t* temp = buf<uint64_t>(c, temp_name, scan_temp_words(n));
  CUFLYE_CHECK(exclusive_scan_u32_to_u64(in, out, n, temp, c->stream));
  const uint64_t ntiles = scan_temp_words(n) - 1;
  CUFLYE_CHECK(cudaMemcpyAsync(out + n, temp + (n ? ntiles : 0), sizeof(uint64_t),
                               cudaMemcpyDeviceToDevice, c->stream));
}

uint64_t scan_u32(cuflye_ctx* c, const uint32_t* in, uint64_t* out, uint64_t n,
                  const char* temp_name) {
  uint64_t* temp = buf<uint64_t>(c, temp_name, scan_temp_words(n));
  CUFLYE_CHECK(exclusive_scan_u32_to_u64(in, out, n, temp, c->stream));
  // out[n] = total
  const uint64_t ntiles = scan_temp_words(n) - 1;
  CUFLYE_CHECK(cudaMemcpyAsync(out + n, temp + (n ? ntiles : 0), sizeof(uint64_t),
                               cudaMemcpyDeviceToDevice, c->stream));
  return read_scalar(c, out + n);
}

std::string lib_dir() {
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&lib_dir), &info) && info.dli_fname) {
    std::string p = info.dli_fname;
    const size_t s = p.rfind('/');
    return s == std::string::npos ? "." : p.substr(0, s);
  }
  return ".";
}

void load_logf_table(cuflye_ctx* c) {
  const std::string path = lib_dir() + "/logf_exceptions.bin";
  std::ifstream in(path, std::ios::binary);
  if (!in)
    throw Error(CUFLYE_ERR_INVALID,
                "logf exception table missing: " + path + " (built by the package build step)");
  uint32_t n = 0;
  in.read(reinterpret_cast<char*>(&n), sizeof(n));
  std::vector<uint32_t> xy(2 * static_cast<size_t>(n));
  in.read(reinterpret_cast<char*>(xy.data()), static_cast<std::streamsize>(xy.size() * 4));
  if (!in) throw Error(CUFLYE_ERR_INVALID, "logf exception table truncated: " + path);
  std::vector<uint32_t> xs(n), ys(n);
  for (uint32_t i = 0; i < n; ++i) {
    xs[i] = xy[2 * i];
    ys[i] = xy[2 * i + 1];
  }
  uint32_t* dx = buf<uint32_t>(c, "logf_x", n);
  uint32_t* dy = buf<uint32_t>(c, "logf_y", n);
  CUFLYE_CHECK(cudaMemcpy(dx, xs.data(), n * 4ull, cudaMemcpyHostToDevice));
  CUFLYE_CHECK(cudaMemcpy(dy, ys.data(), n * 4ull, cudaMemcpyHostToDevice));
  c->logt = LogfTable{dx, dy, n};
}

int bits_for(uint64_t v) {
  int b = 0;
  while (b < 64 && (v >> b) != 0) ++b;
  return b;
}

// The memory budget, or the device's memory less an 8 GiB margin when unbounded.
uint64_t effective_budget(cuflye_ctx* c) {
  if (c->budget) return c->budget;
  size_t free_b = 0, total_b = 0;
  CUFLYE_CHECK(cudaMemGetInfo(&free_b, &total_b));
  const uint64_t cap = static_cast<uint64_t>(free_b) + c->in_use;
  const uint64_t margin = 8ull << 30;
  return cap > margin ? cap - margin : cap / 2;
}

// ---------------------------------------------------------------- index build

// The windows of the packed targets (device arrays).
struct WindowSet {
  const uint64_t* words;
  const uint64_t* base_off;
  const uint64_t* win_off;
  const int32_t* slot_len;
  uint32_t nslots;
  uint64_t nwin;
  int k;
};

struct BuiltIndex {
  TableEntry* table = nullptr;
  uint64_t cap = 0;
  uint64_t* pos = nullptr;
  uint64_t npos = 0, nsolid = 0, nrep = 0;
  uint32_t* self_at = nullptr;  // one-range builds, when memory allows
  uint64_t* win_off = nullptr;
};

// Scratch of one key range's build.
const char* const kBuildScratch[] = {"ib_keys", "ib_vals",  "ib_keys2",    "ib_vals2",
                                     "ib_hist", "ib_flags", "ib_runid",    "ib_runstart",
                                     "ib_kept", "ib_cls",   "ib_keptoff",  "ib_scan",
                                     "ib_count"};

void release_build_scratch(cuflye_ctx* c) {
  for (const char* t : kBuildScratch) release(c, t);
}

// Runs of nw windows sorted by (key, stored id, stored position).
struct KeyRuns {
  uint64_t* keys;
  uint64_t* vals;
  uint64_t* run_id;
  uint64_t* run_start;
  uint8_t* cls;
  uint64_t* kept_off;
  uint64_t nw, nruns, npos, nsolid, nrep;
};

// Sorts the windows in ib_keys / ib_vals (the alternates ib_keys2 / ib_vals2
// already sized), finds their runs and classifies them (solid, repetitive).
KeyRuns sort_and_classify(cuflye_ctx* c, uint64_t nw, const std::vector<int>& digits,
                          uint32_t min_freq, uint32_t max_freq) {
  cudaStream_t st = c->stream;
  uint64_t* keys = buf<uint64_t>(c, "ib_keys", nw);
  uint64_t* vals = buf<uint64_t>(c, "ib_vals", nw);
  uint64_t* keys2 = buf<uint64_t>(c, "ib_keys2", nw);
  uint64_t* vals2 = buf<uint64_t>(c, "ib_vals2", nw);
  uint32_t* hist = buf<uint32_t>(c, "ib_hist", radix_hist_words(nw));
  int in_alt = 0;
  if (nw)
    CUFLYE_CHECK(radix_sort_pairs(keys, vals, keys2, vals2, nw, digits.data(),
                                  static_cast<int>(digits.size()), hist, &in_alt, st));
  if (in_alt) {
    std::swap(keys, keys2);
    std::swap(vals, vals2);
  }
  uint32_t* flags = buf<uint32_t>(c, "ib_flags", nw);
  uint64_t* run_id = buf<uint64_t>(c, "ib_runid", nw + 1);
  CUFLYE_CHECK(index_mark_runs(keys, nw, flags, st));
  const uint64_t nruns = scan_u32(c, flags, run_id, nw, "ib_scan");
  uint64_t* run_start = buf<uint64_t>(c, "ib_runstart", nruns + 1);
  CUFLYE_CHECK(index_run_starts(flags, run_id, nw, nruns, run_start, st));
  uint32_t* kept = buf<uint32_t>(c, "ib_kept", nruns);
  uint8_t* cls = buf<uint8_t>(c, "ib_cls", nruns);
  unsigned long long* tally = buf<unsigned long long>(c, "ib_count", 4);
  CUFLYE_CHECK(index_classify_runs(run_start, nruns, min_freq, max_freq, kept, cls, tally, st));
  uint64_t* kept_off = buf<uint64_t>(c, "ib_keptoff", nruns + 1);
  const uint64_t npos = scan_u32(c, kept, kept_off, nruns, "ib_scan");
  unsigned long long t[2];
  CUFLYE_CHECK(cudaMemcpyAsync(t, tally, sizeof(t), cudaMemcpyDeviceToHost, st));
  sync(c);
  return KeyRuns{keys, vals, run_id, run_start, cls, kept_off, nw, nruns, npos, t[0], t[1]};
}

// Table slots for `entries` keys: twice as many (load 1/2), at least 16.
uint64_t table_capacity(uint64_t entries) { return std::max<uint64_t>(16, 2 * entries); }

// All windows at once.  This build fits the memory with room to spare, so
// its table takes the power of two at or above twice every run (solid,
// repetitive and absent): a load well under 1/2 keeps lookups short.
BuiltIndex build_one_range(cuflye_ctx* c, const WindowSet& w, const std::vector<int>& digits,
                           uint32_t min_freq, uint32_t max_freq) {
  cudaStream_t st = c->stream;
  // the four sort arrays first: a build that cannot hold them fails before any work
  uint64_t* keys = buf<uint64_t>(c, "ib_keys", w.nwin);
  uint64_t* vals = buf<uint64_t>(c, "ib_vals", w.nwin);
  buf<uint64_t>(c, "ib_keys2", w.nwin);
  buf<uint64_t>(c, "ib_vals2", w.nwin);
  CUFLYE_CHECK(index_enumerate(w.words, w.base_off, w.win_off, w.slot_len, w.nslots, w.nwin,
                               w.k, keys, vals, st));
  const KeyRuns r = sort_and_classify(c, w.nwin, digits, min_freq, max_freq);
  if (r.npos >= (1ull << 40)) throw Error(CUFLYE_ERR_UNSUPPORTED, "index larger than 2^40 entries");
  BuiltIndex bi;
  bi.pos = buf<uint64_t>(c, "ix_pos", r.npos);
  // each indexed window's own bucket entry (4 bytes a window), when memory
  // allows: hit counting then finds a query's own entry with one load
  uint32_t* self_at = nullptr;
  uint64_t* win_off = nullptr;
  try {
    self_at = buf<uint32_t>(c, "ix_selfat", w.nwin);
    win_off = buf<uint64_t>(c, "ix_winoff", static_cast<uint64_t>(w.nslots) + 1);
  } catch (const Error& e) {
    if (e.code != CUFLYE_ERR_BUDGET) throw;
    release(c, "ix_selfat");
    release(c, "ix_winoff");
    self_at = nullptr;
    win_off = nullptr;
  }
  if (win_off)
    CUFLYE_CHECK(cudaMemcpyAsync(win_off, w.win_off, (static_cast<uint64_t>(w.nslots) + 1) * 8,
                                 cudaMemcpyDeviceToDevice, st));
  CUFLYE_CHECK(index_copy_positions(r.vals, r.run_id, r.run_start, r.cls, r.kept_off, w.nwin,
                                    bi.pos, st, self_at, win_off, w.slot_len, w.k));
  bi.self_at = self_at;
  bi.win_off = win_off;
  bi.cap = 16;
  while (bi.cap < 2 * r.nruns) bi.cap <<= 1;
  bi.table = buf<TableEntry>(c, "ix_table", bi.cap);
  CUFLYE_CHECK(cudaMemsetAsync(bi.table, 0xff, bi.cap * sizeof(TableEntry), st));
  CUFLYE_CHECK(index_insert(r.keys, r.vals, r.run_start, r.cls, r.kept_off, r.nruns, 0, true,
                            bi.table, bi.cap, c->status, st));
  check_device_status(c);
  bi.npos = r.npos;
  bi.nsolid = r.nsolid;
  bi.nrep = r.nrep;
  return bi;
}

// Device bytes one window of a key range needs while the range is built:
// the radix sort's two key/value pairs (32), run flag and id (12) and the
// run tables (21, at most one run per window), with margin.
constexpr uint64_t kRangeBytesPerWindow = 72;
constexpr int kPrefixBits = 14;

// Cuts [0, nbins) into contiguous ranges of prefix bins, each holding as many
// windows as what the memory budget leaves allows (and at most the caller's
// window cap), and runs body(first bin, sorted runs) on each after enumerating,
// sorting and classifying its windows.  Returns the number of ranges.
template <typename Body>
uint64_t for_each_key_range(cuflye_ctx* c, const WindowSet& w, const std::vector<int>& digits,
                            uint32_t min_freq, uint32_t max_freq,
                            const std::vector<unsigned long long>& hist, int shift, Body body) {
  cudaStream_t st = c->stream;
  const int nbins = static_cast<int>(hist.size());
  uint64_t ranges = 0;
  int b = 0;
  while (b < nbins) {
    const uint64_t limit = effective_budget(c);
    const uint64_t avail = limit > c->in_use ? limit - c->in_use : 0;
    uint64_t cap = avail / kRangeBytesPerWindow;
    if (c->build_window_cap) cap = std::min(cap, c->build_window_cap);
    int e = b;
    uint64_t nw = 0;
    while (e < nbins && nw + hist[e] <= cap) nw += hist[e++];
    if (e == b)
      throw Error(CUFLYE_ERR_BUDGET,
                  "k-mer index build: " + std::to_string(hist[b]) +
                      " windows share one key prefix and need about " +
                      std::to_string(hist[b] * kRangeBytesPerWindow) + " bytes; " +
                      std::to_string(avail) + " bytes are left in the memory budget");
    const int first = b;
    const uint64_t lo = static_cast<uint64_t>(b) << shift;
    const uint64_t hi = static_cast<uint64_t>(e) << shift;
    b = e;
    if (nw == 0) continue;
    uint64_t* keys = buf<uint64_t>(c, "ib_keys", nw);
    uint64_t* vals = buf<uint64_t>(c, "ib_vals", nw);
    buf<uint64_t>(c, "ib_keys2", nw);
    buf<uint64_t>(c, "ib_vals2", nw);
    unsigned long long* count = buf<unsigned long long>(c, "ib_count", 4);
    CUFLYE_CHECK(index_enumerate_range(w.words, w.base_off, w.win_off, w.slot_len, w.nslots,
                                       w.nwin, w.k, lo, hi, keys, vals, count, nw, st));
    const unsigned long long got = read_scalar(c, count);
    if (got != nw)
      throw Error(CUFLYE_ERR_CUDA, "k-mer index build: key range [" + std::to_string(lo) + ", " +
                                       std::to_string(hi) + ") enumerated " +
                                       std::to_string(got) + " windows, the histogram " +
                                       std::to_string(nw));
    body(first, sort_and_classify(c, nw, digits, min_freq, max_freq));
    sync(c);
    release_build_scratch(c);
    ++ranges;
  }
  return ranges;
}

// The index built one contiguous key range at a time, in two passes over the
// ranges.  The first counts each key prefix's solid positions and table
// entries; the position array and the table are then allocated at their
// final sizes, and the second pass writes each range's positions at its
// first prefix's offset and inserts its runs.  The device holds the final
// index and one range's scratch at most, and the position array equals the
// one-range build's.
BuiltIndex build_key_ranges(cuflye_ctx* c, const WindowSet& w, const std::vector<int>& digits,
                            uint32_t min_freq, uint32_t max_freq) {
  cudaStream_t st = c->stream;
  const int bits = std::min(2 * w.k, kPrefixBits);
  const int shift = 2 * w.k - bits;
  const int nbins = 1 << bits;
  std::vector<unsigned long long> hist(nbins), npos_bin(nbins), nent_bin(nbins);
  unsigned long long* d_bins = buf<unsigned long long>(c, "ib_bins", 3ull * nbins);
  CUFLYE_CHECK(index_prefix_hist(w.words, w.base_off, w.win_off, w.slot_len, w.nslots, w.nwin,
                                 w.k, shift, nbins, d_bins, c->num_sms, st));
  CUFLYE_CHECK(cudaMemcpyAsync(hist.data(), d_bins, nbins * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st));
  CUFLYE_CHECK(cudaMemsetAsync(d_bins + nbins, 0, 2ull * nbins * sizeof(unsigned long long), st));
  sync(c);
  uint64_t nsolid = 0, nrep = 0;
  for_each_key_range(c, w, digits, min_freq, max_freq, hist, shift,
                     [&](int, const KeyRuns& r) {
                       CUFLYE_CHECK(index_bin_totals(r.keys, r.run_start, r.cls, r.nruns, shift,
                                                     d_bins + nbins, d_bins + 2 * nbins, st));
                       nsolid += r.nsolid;
                       nrep += r.nrep;
                     });
  CUFLYE_CHECK(cudaMemcpyAsync(npos_bin.data(), d_bins + nbins,
                               nbins * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  CUFLYE_CHECK(cudaMemcpyAsync(nent_bin.data(), d_bins + 2 * nbins,
                               nbins * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  sync(c);
  release(c, "ib_bins");
  std::vector<uint64_t> pos_start(nbins + 1, 0);
  uint64_t nent = 0;
  for (int i = 0; i < nbins; ++i) {
    pos_start[i + 1] = pos_start[i] + npos_bin[i];
    nent += nent_bin[i];
  }
  const uint64_t npos = pos_start[nbins];
  if (nent != nsolid + nrep)
    throw Error(CUFLYE_ERR_CUDA, "k-mer index build: " + std::to_string(nent) +
                                     " table entries by prefix, " +
                                     std::to_string(nsolid + nrep) + " by run class");
  if (npos >= (1ull << 40)) throw Error(CUFLYE_ERR_UNSUPPORTED, "index larger than 2^40 entries");
  BuiltIndex bi;
  bi.pos = buf<uint64_t>(c, "ix_pos", npos);
  bi.cap = table_capacity(nent);
  bi.table = buf<TableEntry>(c, "ix_table", bi.cap);
  CUFLYE_CHECK(cudaMemsetAsync(bi.table, 0xff, bi.cap * sizeof(TableEntry), st));
  uint64_t written = 0;
  c->build_ranges = for_each_key_range(
      c, w, digits, min_freq, max_freq, hist, shift, [&](int first, const KeyRuns& r) {
        const uint64_t base = pos_start[first];
        if (base + r.npos > npos)
          throw Error(CUFLYE_ERR_CUDA, "k-mer index build: a key range's positions overrun "
                                       "the counted total");
        CUFLYE_CHECK(index_copy_positions(r.vals, r.run_id, r.run_start, r.cls, r.kept_off, r.nw,
                                          bi.pos + base, st));
        CUFLYE_CHECK(index_insert(r.keys, r.vals, r.run_start, r.cls, r.kept_off, r.nruns, base,
                                  true, bi.table, bi.cap, c->status, st));
        written += r.npos;
      });
  if (written != npos)
    throw Error(CUFLYE_ERR_CUDA, "k-mer index build: the second pass wrote " +
                                     std::to_string(written) + " positions of " +
                                     std::to_string(npos));
  check_device_status(c);
  bi.npos = npos;
  bi.nsolid = nsolid;
  bi.nrep = nrep;
  return bi;
}

void build_index(cuflye_ctx* c, int k, size_t n, const int64_t* ids, const int64_t* offsets,
                 const char* bases, uint32_t min_freq, uint32_t max_freq) {
  c->other_per_hit = 0;  // a new workload: learned again
  if (k < 1 || k > 31) throw Error(CUFLYE_ERR_UNSUPPORTED, "k must be in [1, 31]");
  if (n == 0) throw Error(CUFLYE_ERR_INVALID, "index needs at least one target");
  if (max_freq >= (1u << kCountBits) - 1)
    throw Error(CUFLYE_ERR_UNSUPPORTED, "max_freq must be below 2^22 - 1");
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) {
    if (ids[i] <= 0) throw Error(CUFLYE_ERR_INVALID, "index target ids must be > 0");
    if (offsets[i + 1] < offsets[i]) throw Error(CUFLYE_ERR_INVALID, "offsets must not decrease");
    if (offsets[i + 1] - offsets[i] >= (1ll << 31))
      throw Error(CUFLYE_ERR_UNSUPPORTED, "target longer than 2^31");
    order[i] = i;
  }
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return ids[a] < ids[b]; });
  for (size_t i = 1; i < n; ++i)
    if (ids[order[i]] == ids[order[i - 1]])
      throw Error(CUFLYE_ERR_INVALID, "duplicate target id " + std::to_string(ids[order[i]]));
  if (2 * n >= (1ull << 31)) throw Error(CUFLYE_ERR_UNSUPPORTED, "too many targets");
  c->has_index = false;
  c->slot_of.clear();
  c->slot_signed_h.assign(n, 0);
  std::vector<int32_t> slot_len(n);
  std::vector<uint64_t> base_off(n), win_off(n + 1);
  win_off[0] = 0;
  int64_t maxlen = 0;
  for (size_t s = 0; s < n; ++s) {
    const size_t i = order[s];
    c->slot_of[ids[i]] = static_cast<uint32_t>(s);
    c->slot_signed_h[s] = ids[i];
    const int64_t len = offsets[i + 1] - offsets[i];
    slot_len[s] = static_cast<int32_t>(len);
    maxlen = std::max(maxlen, len);
    base_off[s] = static_cast<uint64_t>(offsets[i] - offsets[0]);
    win_off[s + 1] = win_off[s] + (len >= k ? static_cast<uint64_t>(len - k + 1) : 0);
  }
  const uint64_t nbases = static_cast<uint64_t>(offsets[n] - offsets[0]);
  const uint64_t nwin = win_off[n];
  cudaStream_t st = c->stream;
  // the previous index's arrays go first (has_index is false from here on)
  release(c, "ix_pos");
  release(c, "ix_table");
  release(c, "ix_selfat");
  release(c, "ix_winoff");
  c->idx.self_at = nullptr;
  c->idx.win_off = nullptr;
  // bases packed in chunks of 256 MiB (a multiple of 32 bases: chunks start on
  // word boundaries; each chunk's trailing pad word is overwritten by the next)
  uint64_t* words = buf<uint64_t>(c, "ib_words", (nbases + 31) / 32 + 2);
  {
    const uint64_t chunk = std::min<uint64_t>(nbases, 256ull << 20);
    uint8_t* d_ascii = buf<uint8_t>(c, "ib_ascii", chunk + 16);
    for (uint64_t b0 = 0; b0 < nbases; b0 += chunk) {
      const uint64_t len = std::min(chunk, nbases - b0);
      CUFLYE_CHECK(cudaMemcpyAsync(d_ascii, bases + offsets[0] + b0, len,
                                   cudaMemcpyHostToDevice, st));
      CUFLYE_CHECK(pack_bases(d_ascii, len, words + b0 / 32, st));
    }
    if (nbases == 0) CUFLYE_CHECK(cudaMemsetAsync(words, 0, 16, st));
    sync(c);
    release(c, "ib_ascii");
  }
  uint64_t* d_base = buf<uint64_t>(c, "ib_base", n);
  uint64_t* d_win = buf<uint64_t>(c, "ib_win", n + 1);
  int32_t* d_len = buf<int32_t>(c, "ix_slot_len", n);
  int64_t* d_signed = buf<int64_t>(c, "ix_slot_signed", n);
  CUFLYE_CHECK(cudaMemcpyAsync(d_base, base_off.data(), n * 8, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(d_win, win_off.data(), (n + 1) * 8, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(d_len, slot_len.data(), n * 4, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(d_signed, c->slot_signed_h.data(), n * 8, cudaMemcpyHostToDevice,
                               st));
  const WindowSet ws{words, d_base, d_win, d_len, static_cast<uint32_t>(n), nwin, k};
  // LSD digits: position bytes, stored-id bytes, key bytes
  std::vector<int> digits;
  const int pbytes = (bits_for(static_cast<uint64_t>(maxlen)) + 7) / 8;
  const int dbytes = (bits_for(2 * n) + 7) / 8;
  const int kbytes = (2 * k + 7) / 8;
  for (int d = 0; d < pbytes; ++d) digits.push_back(d);
  for (int d = 0; d < dbytes; ++d) digits.push_back(4 + d);
  for (int d = 0; d < kbytes; ++d) digits.push_back(8 + d);
  BuiltIndex bi;
  bool ranges = c->build_window_cap != 0 && nwin > c->build_window_cap;
  if (!ranges) {
    try {
      bi = build_one_range(c, ws, digits, min_freq, max_freq);
      c->build_ranges = 1;
    } catch (const Error& e) {
      if (e.code != CUFLYE_ERR_BUDGET) throw;
      sync(c);
      release_build_scratch(c);
      release(c, "ix_pos");
      release(c, "ix_table");
      release(c, "ix_selfat");
      release(c, "ix_winoff");
      ranges = true;
    }
  }
  if (ranges) bi = build_key_ranges(c, ws, digits, min_freq, max_freq);
  release_build_scratch(c);
  for (const char* t : {"ib_words", "ib_base", "ib_win", "ib_bins"}) release(c, t);
  c->idx.k = k;
  c->idx.transform = true;
  c->idx.table = bi.table;
  c->idx.cap = bi.cap;
  c->idx.pos = bi.pos;
  c->idx.npos = bi.npos;
  c->idx.slot_len = d_len;
  c->idx.slot_signed = d_signed;
  c->idx.nslots = static_cast<uint32_t>(n);
  c->idx.self_at = bi.self_at;
  c->idx.win_off = bi.win_off;
  c->idx.nkeys = bi.nsolid + bi.nrep;
  c->idx.nrep = bi.nrep;
  c->has_index = true;
}

void build_index_entries(cuflye_ctx* c, int k, size_t n, const int64_t* tids, const int64_t* tpos,
                         const uint64_t* keys_h, size_t nrep, const uint64_t* rep_h) {
  if (k < 1 || k > 31) throw Error(CUFLYE_ERR_UNSUPPORTED, "k must be in [1, 31]");
  c->has_index = false;
  std::vector<int64_t> absids;
  for (size_t i = 0; i < n; ++i) {
    if (tids[i] == 0) throw Error(CUFLYE_ERR_INVALID, "target id must not be zero");
    if (tpos[i] < 0 || tpos[i] >= (1ll << 31)) throw Error(CUFLYE_ERR_INVALID, "bad position");
    absids.push_back(tids[i] < 0 ? -tids[i] : tids[i]);
  }
  std::sort(absids.begin(), absids.end());
  absids.erase(std::unique(absids.begin(), absids.end()), absids.end());
  c->slot_of.clear();
  c->slot_signed_h = absids;
  for (size_t s = 0; s < absids.size(); ++s) c->slot_of[absids[s]] = static_cast<uint32_t>(s);
  const uint32_t nslots = static_cast<uint32_t>(std::max<size_t>(absids.size(), 1));
  std::vector<uint64_t> vals_h(n);
  for (size_t i = 0; i < n; ++i) {
    const int64_t a = tids[i] < 0 ? -tids[i] : tids[i];
    const uint32_t di = 2u * c->slot_of[a] + (tids[i] < 0 ? 1u : 0u);
    vals_h[i] = (static_cast<uint64_t>(di) << 32) | static_cast<uint32_t>(tpos[i]);
  }
  cudaStream_t st = c->stream;
  std::vector<int32_t> zero_len(nslots, 0);
  std::vector<int64_t> signed_h(nslots, 1);
  for (size_t s = 0; s < absids.size(); ++s) signed_h[s] = absids[s];
  int32_t* d_len = buf<int32_t>(c, "ix_slot_len", nslots);
  int64_t* d_signed = buf<int64_t>(c, "ix_slot_signed", nslots);
  CUFLYE_CHECK(cudaMemcpyAsync(d_len, zero_len.data(), nslots * 4ull, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(d_signed, signed_h.data(), nslots * 8ull, cudaMemcpyHostToDevice, st));
  const uint64_t nn = n;
  uint64_t* keys = buf<uint64_t>(c, "ib_keys", nn);
  uint64_t* vals = buf<uint64_t>(c, "ib_vals", nn);
  uint64_t* keys2 = buf<uint64_t>(c, "ib_keys2", nn);
  uint64_t* vals2 = buf<uint64_t>(c, "ib_vals2", nn);
  if (nn) {
    CUFLYE_CHECK(cudaMemcpyAsync(keys, keys_h, nn * 8, cudaMemcpyHostToDevice, st));
    CUFLYE_CHECK(cudaMemcpyAsync(vals, vals_h.data(), nn * 8, cudaMemcpyHostToDevice, st));
  }
  std::vector<int> digits;
  for (int d = 0; d < (2 * k + 7) / 8; ++d) digits.push_back(8 + d);
  uint32_t* hist = buf<uint32_t>(c, "ib_hist", radix_hist_words(nn));
  int in_alt = 0;
  if (nn)
    CUFLYE_CHECK(radix_sort_pairs(keys, vals, keys2, vals2, nn, digits.data(),
                                  static_cast<int>(digits.size()), hist, &in_alt, st));
  if (in_alt) {
    std::swap(keys, keys2);
    std::swap(vals, vals2);
  }
  uint32_t* flags = buf<uint32_t>(c, "ib_flags", nn);
  uint64_t* run_id = buf<uint64_t>(c, "ib_runid", nn + 1);
  CUFLYE_CHECK(index_mark_runs(keys, nn, flags, st));
  const uint64_t nruns = scan_u32(c, flags, run_id, nn, "ib_scan");
  uint64_t* run_start = buf<uint64_t>(c, "ib_runstart", nruns + 1);
  CUFLYE_CHECK(index_run_starts(flags, run_id, nn, nruns, run_start, st));
  uint32_t* kept = buf<uint32_t>(c, "ib_kept", nruns);
  uint8_t* cls = buf<uint8_t>(c, "ib_cls", nruns);
  CUFLYE_CHECK(index_classify_runs(run_start, nruns, 1, (1u << kCountBits) - 2, kept, cls,
                                    nullptr, st));
  uint64_t* kept_off = buf<uint64_t>(c, "ib_keptoff", nruns + 1);
  const uint64_t npos = scan_u32(c, kept, kept_off, nruns, "ib_scan");
  uint64_t* pos = buf<uint64_t>(c, "ix_pos", npos);
  CUFLYE_CHECK(index_copy_positions(vals, run_id, run_start, cls, kept_off, nn, pos, st));
  const uint64_t cap = table_capacity(nruns + nrep);
  TableEntry* table = buf<TableEntry>(c, "ix_table", cap);
  CUFLYE_CHECK(cudaMemsetAsync(table, 0xff, cap * sizeof(TableEntry), st));
  CUFLYE_CHECK(index_insert(keys, vals, run_start, cls, kept_off, nruns, 0, false, table, cap,
                            c->status, st));
  if (nrep) {
    uint64_t* d_rep = buf<uint64_t>(c, "ib_rep", nrep);
    CUFLYE_CHECK(cudaMemcpyAsync(d_rep, rep_h, nrep * 8, cudaMemcpyHostToDevice, st));
    CUFLYE_CHECK(index_insert_repetitive(d_rep, nrep, table, cap, c->status, st));
  }
  check_device_status(c);
  for (const char* t : {"ib_keys", "ib_vals", "ib_keys2", "ib_vals2", "ib_hist", "ib_flags",
                        "ib_runid", "ib_runstart", "ib_kept", "ib_cls", "ib_keptoff", "ib_scan",
                        "ib_rep"})
    release(c, t);
  c->idx.k = k;
  c->idx.transform = false;
  release(c, "ix_selfat");
  release(c, "ix_winoff");
  c->idx.self_at = nullptr;
  c->idx.win_off = nullptr;
  c->idx.table = table;
  c->idx.cap = cap;
  c->idx.pos = pos;
  c->idx.npos = npos;
  c->idx.slot_len = d_len;
  c->idx.slot_signed = d_signed;
  c->idx.nslots = nslots;
  c->idx.nkeys = nruns + nrep;
  c->idx.nrep = nrep;
  c->has_index = true;
}

// ---------------------------------------------------------------- passes

struct Queries {
  size_t n;
  const int64_t* ids;
  const int64_t* offsets;
  const char* bases;
};

struct PassState {
  uint32_t nq = 0;
  uint64_t nwin = 0, nhits = 0, nfilt = 0;
  uint64_t* keys = nullptr;
  uint32_t* vals = nullptr;
  uint64_t* kmers = nullptr;
  int32_t* fpos = nullptr;
  uint64_t* q_off = nullptr;  // nq + 1 hit offsets
  uint64_t* f_off = nullptr;  // nq + 1 filtered offsets
  QueryInfo* qinfo = nullptr;
  uint32_t* q_tie = nullptr;  // per query: its KmerMatch keys may repeat
  // false: the hits are not yet written (the sorted emission writes them
  // straight into KmerMatch order); the window tables below feed it
  bool emitted = true;
  QueryBatch qb;
  const uint64_t* hit_off = nullptr;
  const uint64_t* filt_off = nullptr;
  const uint64_t* wmeta = nullptr;
  const uint8_t* wflags = nullptr;
  const uint32_t* wself = nullptr;
  uint64_t fit_hits = 0;  // the hits the memory left could hold when the pass was cut
};

// Buffers sized by the hit count of a pass (reused by the next pass).
const char* const kPerHitBuffers[] = {"h_keys",  "h_vals",   "h_kmers", "s_l",     "s_r",
                                      "c_akeys", "c_avals",  "c_score", "c_bt",    "a_cand",
                                      "m_tiles", "m_counts", "c_pmc",   "o_maps",  "g_tcount",
                                      "g_toff"};


// The pass's hits in Flye's generation order (and the filtered positions).
void emit_generation_order(cuflye_ctx* c, PassState& ps) {
  CUFLYE_CHECK(hits_emit(c->idx, ps.qb, ps.hit_off, ps.filt_off, ps.wmeta, ps.wflags, ps.keys,
                         ps.vals, ps.kmers, ps.fpos, c->stream));
  ps.emitted = true;
}

// Upload a run of queries starting at q0 and produce the hits of the longest
// prefix of them that fits in device memory (ps.nq queries), in Flye's
// generation order.
// Device bytes per query window of a pass's run: bases (1), packed words
// (0.25), hit and filter counts (8), window metadata (8) and flags (1), the
// two offset arrays (16), rounded up.
constexpr uint64_t kRunBytesPerWindow = 40;
// Buffers sized by the windows of a pass's run (reused by the next pass).
const char* const kPerWindowBuffers[] = {"q_ascii", "q_words",  "w_cnt",     "w_filt", "w_meta",
                                         "w_flags", "w_hitoff", "w_filtoff", "w_scan", "w_self"};

// The end of the run of queries from q0 (at most q1) whose windows' buffers
// take at most a quarter of the memory the budget leaves; the rest is for
// the run's hits.  With the hits per window of the call's previous pass
// (hpw > 0), the run also stops about where its hits stop fitting, so that
// few of its queries are counted again by the next pass.  At least one query.
size_t run_end(cuflye_ctx* c, const Queries& Q, size_t q0, size_t q1, uint64_t bytes_per_hit,
               double hpw) {
  const uint64_t limit = effective_budget(c);
  uint64_t reusable = 0;
  auto held = [&](const char* name) {
    auto it = c->bufs.find(name);
    if (it != c->bufs.end()) reusable += it->second.cap;
  };
  for (const char* nm : kPerWindowBuffers) held(nm);
  for (const char* nm : kPerHitBuffers) held(nm);
  const uint64_t used = c->in_use > reusable ? c->in_use - reusable : 0;
  const uint64_t avail = limit > used ? limit - used : 0;
  uint64_t cap = avail / 4 / kRunBytesPerWindow;
  if (hpw > 0) {
    const double fit =
        1.1 * static_cast<double>(avail) / (static_cast<double>(bytes_per_hit) * hpw);
    if (fit < static_cast<double>(cap)) cap = std::max<uint64_t>(1, static_cast<uint64_t>(fit));
  }
  const int64_t k = c->idx.k;
  uint64_t nw = 0;
  size_t q = q0;
  while (q < q1) {
    const int64_t len = Q.offsets[q + 1] - Q.offsets[q];
    const uint64_t w = len >= k ? static_cast<uint64_t>(len - k + 1) : 0;
    if (q > q0 && nw + w > cap) break;
    nw += w;
    ++q;
  }
  return q;
}

// Hits per window below which a pass takes the emit + sort path.
constexpr uint64_t kSortedEmissionMinHitsPerWindow = 6;

// Whether a pass's hits may go straight into KmerMatch order (match_emit.cu):
// overlap and read-to-graph calls on a built index, unless switched off; the
// pass's hit density decides in the end.
bool sorted_emission(const cuflye_ctx* c, bool want_kmers) {
  return !want_kmers && c->idx.transform && c->sorted_emission != 0;
}

bool run_hits(cuflye_ctx* c, const Queries& Q, size_t q0, size_t q1, bool want_kmers,
              uint64_t bytes_per_hit, PassState& ps) {
  const int k = c->idx.k;
  const uint32_t nq = static_cast<uint32_t>(q1 - q0);
  ps.nq = nq;
  std::vector<uint64_t> base_off(nq + 1), win_off(nq + 1);
  std::vector<int32_t> qdi(nq);
  std::vector<QueryInfo> qinfo(nq);
  base_off[0] = 0;
  win_off[0] = 0;
  for (uint32_t i = 0; i < nq; ++i) {
    const int64_t id = Q.ids[q0 + i];
    if (id == 0) throw Error(CUFLYE_ERR_INVALID, "query id must not be zero");
    const int64_t len = Q.offsets[q0 + i + 1] - Q.offsets[q0 + i];
    if (len < 0) throw Error(CUFLYE_ERR_INVALID, "offsets must not decrease");
    if (len >= (1ll << 31)) throw Error(CUFLYE_ERR_UNSUPPORTED, "query longer than 2^31");
    base_off[i + 1] = base_off[i] + static_cast<uint64_t>(len);
    win_off[i + 1] = win_off[i] + (len >= k ? static_cast<uint64_t>(len - k + 1) : 0);
    const int64_t a = id < 0 ? -id : id;
    auto it = c->slot_of.find(a);
    qdi[i] = it == c->slot_of.end() ? -1 : static_cast<int32_t>(2u * it->second + (id < 0 ? 1u : 0u));
    qinfo[i] = QueryInfo{id, static_cast<int32_t>(len), 0};
  }
  const uint64_t nbases = base_off[nq];
  const uint64_t nwin = win_off[nq];
  ps.nwin = nwin;
  cudaStream_t st = c->stream;
  uint8_t* d_ascii = buf<uint8_t>(c, "q_ascii", nbases + 16);
  if (nbases)
    CUFLYE_CHECK(cudaMemcpyAsync(d_ascii, Q.bases + Q.offsets[q0], nbases, cudaMemcpyHostToDevice,
                                 st));
  uint64_t* words = buf<uint64_t>(c, "q_words", (nbases + 31) / 32 + 2);
  uint64_t* d_base = buf<uint64_t>(c, "q_base", nq + 1);
  uint64_t* d_win = buf<uint64_t>(c, "q_win", nq + 1);
  int32_t* d_qdi = buf<int32_t>(c, "q_qdi", nq);
  ps.qinfo = buf<QueryInfo>(c, "q_info", nq);
  CUFLYE_CHECK(cudaMemcpyAsync(d_base, base_off.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(d_win, win_off.data(), (nq + 1) * 8ull, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(d_qdi, qdi.data(), nq * 4ull, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(ps.qinfo, qinfo.data(), nq * sizeof(QueryInfo),
                               cudaMemcpyHostToDevice, st));
  // inputs are on the device from here on
  CUFLYE_CHECK(cudaEventRecord(c->ev[5], st));
  CUFLYE_CHECK(pack_bases(d_ascii, nbases, words, st));
  QueryBatch qb;
  qb.words = words;
  qb.base_off = d_base;
  qb.win_off = d_win;
  qb.qdi = d_qdi;
  qb.nq = nq;
  qb.nwin = nwin;
  uint32_t* cnt = buf<uint32_t>(c, "w_cnt", nwin);
  uint32_t* filt = buf<uint32_t>(c, "w_filt", nwin);
  uint64_t* wmeta = buf<uint64_t>(c, "w_meta", nwin);
  uint8_t* wflags = buf<uint8_t>(c, "w_flags", nwin);
  ps.q_tie = buf<uint32_t>(c, "q_tie", nq);
  CUFLYE_CHECK(cudaMemsetAsync(ps.q_tie, 0, std::max<uint64_t>(nq, 1) * 4ull, st));
  const bool fused = sorted_emission(c, want_kmers);
  uint32_t* wself = fused ? buf<uint32_t>(c, "w_self", nwin) : nullptr;
  CUFLYE_CHECK(hits_count(c->idx, qb, cnt, filt, wmeta, wflags, ps.q_tie, wself, st));
  uint64_t* hit_off = buf<uint64_t>(c, "w_hitoff", nwin + 1);
  uint64_t* filt_off = buf<uint64_t>(c, "w_filtoff", nwin + 1);
  ps.nhits = scan_u32(c, cnt, hit_off, nwin, "w_scan");
  ps.nfilt = scan_u32(c, filt, filt_off, nwin, "w_scan");
  ps.q_off = buf<uint64_t>(c, "q_hitoff", nq + 1);
  ps.f_off = buf<uint64_t>(c, "q_filtoff", nq + 1);
  CUFLYE_CHECK(gather_query_offsets(d_win, hit_off, nq, ps.q_off, st));
  CUFLYE_CHECK(gather_query_offsets(d_win, filt_off, nq, ps.f_off, st));
  // Keep the longest prefix of queries whose hits fit the memory left; the
  // per-hit buffers of an earlier pass are reused, so they count as free.
  const uint64_t limit = effective_budget(c);
  uint64_t reusable = 0;
  for (const char* nm : kPerHitBuffers) {
    auto it = c->bufs.find(nm);
    if (it != c->bufs.end()) reusable += it->second.cap;
  }
  const uint64_t used = c->in_use - reusable;
  // under a caller's budget an eighth stays free for the pass body's other
  // buffers (row pool, rows, per-group tables); without one, the device's
  // own margin covers them
  const uint64_t free_b = limit > used ? limit - used : 0;
  const uint64_t avail = c->budget ? free_b - free_b / 8 : free_b;
  // the pass body's other buffers, per hit, as earlier passes needed them
  const uint64_t fits = static_cast<uint64_t>(
      static_cast<double>(avail) / (static_cast<double>(bytes_per_hit) + c->other_per_hit));
  uint64_t hit_limit = fits;
  ps.fit_hits = fits;
  if (c->pass_hit_cap) hit_limit = std::min(hit_limit, c->pass_hit_cap);
  // Under a caller's budget a pass keeps to the per-hit buffers an earlier
  // pass grew when they hold at least 90 % of what fits: growing them frees
  // and reallocates them, and that synchronizes the device.
  if (c->budget) {
    auto it = c->bufs.find("h_keys");
    const uint64_t held = it == c->bufs.end() ? 0 : it->second.cap / sizeof(uint64_t);
    if (held < fits && held * 10 >= fits * 9) hit_limit = held;
  }
  if (ps.nhits > hit_limit) {
    std::vector<uint64_t> qoff(nq + 1);
    CUFLYE_CHECK(cudaMemcpyAsync(qoff.data(), ps.q_off, (nq + 1) * 8ull, cudaMemcpyDeviceToHost,
                                 st));
    sync(c);
    uint32_t m = 0;
    while (m < nq && qoff[m + 1] <= hit_limit) ++m;
    if (m == 0 && qoff[1] <= fits) m = 1;  // a first query beyond the held buffers
    if (m == 0)
      throw Error(CUFLYE_ERR_BUDGET,
                  "device memory budget exceeded: query " + std::to_string(Q.ids[q0]) + " has " +
                      std::to_string(qoff[1]) + " hits needing " +
                      std::to_string(qoff[1] * bytes_per_hit) + " bytes; " +
                      std::to_string(avail) + " available");
    ps.nq = m;
    ps.nhits = qoff[m];
    ps.nwin = win_off[m];
    qb.nq = m;
    qb.nwin = win_off[m];
    uint64_t fo = 0;
    CUFLYE_CHECK(cudaMemcpyAsync(&fo, ps.f_off + m, 8, cudaMemcpyDeviceToHost, st));
    sync(c);
    ps.nfilt = fo;
  }
  ps.keys = buf<uint64_t>(c, "h_keys", ps.nhits);
  ps.vals = buf<uint32_t>(c, "h_vals", ps.nhits);
  ps.kmers = want_kmers ? buf<uint64_t>(c, "h_kmers", ps.nhits) : nullptr;
  ps.fpos = buf<int32_t>(c, "h_fpos", ps.nfilt);
  ps.qb = qb;
  ps.hit_off = hit_off;
  ps.filt_off = filt_off;
  ps.wmeta = wmeta;
  ps.wflags = wflags;
  ps.wself = wself;
  // The sorted emission pays off where windows hit many targets and the
  // pass has queries for every SM (it runs a block per query); a pass of
  // sparse hits (reads against a genome or a graph) or of a few queries (the
  // one-read path) is cheaper to emit and sort.
  // A call whose passes overflowed the dictionary twice (queries hitting
  // more targets than it holds) emits the rest in generation order.
  ps.emitted = !(fused && (c->sorted_emission == 2 ||
                           (ps.nhits >= kSortedEmissionMinHitsPerWindow * ps.nwin &&
                            ps.nq >= 2ull * static_cast<uint64_t>(c->num_sms) &&
                            c->emission_fallbacks < 2)));
  if (ps.emitted) emit_generation_order(c, ps);
  return true;
}

ChainParams to_chain_params(const cuflye_overlap_params* p) {
  ChainParams cp;
  cp.k = p->kmer_size;
  cp.min_overlap = p->min_overlap;
  cp.max_jump = p->max_jump;
  cp.max_gap = p->max_gap;
  cp.gap_jump_threshold = p->gap_jump_threshold;
  cp.max_overhang = p->max_overhang;
  cp.check_overhang = p->check_overhang;
  cp.force_local = p->force_local;
  cp.only_max_ext = p->only_max_ext;
  cp.max_overlaps = p->max_overlaps;
  cp.large_gap_penalty = p->large_gap_penalty;
  cp.small_gap_penalty = p->small_gap_penalty;
  cp.min_kmer_survival_rate = p->min_kmer_survival_rate;
  cp.max_divergence = p->max_divergence;
  cp.sample_rate = p->sample_rate;
  return cp;
}

// Task-list buffers for the segmented sort, named by `prefix`.
SortTasks sort_tasks(cuflye_ctx* c, const std::string& prefix, uint64_t nelems, uint32_t nseg) {
  const uint64_t w = segsort_task_words(nelems, nseg);
  const size_t rb = segsort_round_bytes(nelems);
  SortTasks t{buf<uint64_t>(c, prefix + "_tf", w),
              buf<uint32_t>(c, prefix + "_tn", w),
              buf<int>(c, prefix + "_td", w),
              static_cast<uint32_t>(w),
              segsort_pair_reserve(nelems),
              nelems,
              {buf<uint8_t>(c, prefix + "_r0", rb), buf<uint8_t>(c, prefix + "_r1", rb)},
              buf<uint32_t>(c, prefix + "_rc", 2 * (kSortRounds + 1)),
              c->shape.round_blocks_per_sm};
  t.side = c->side;
  t.side2 = c->side2;
  t.fork = c->side_ev[0];
  t.rounds_done = c->side_ev[1];
  t.join = c->side_ev[2];
  t.join2 = c->side_ev[3];
  return t;
}

// The flagged queries' KmerMatch sort (their hits in generation order at
// [qb[s], qe[s]), *ecount of them) in libstdc++ order.  Their equal keys
// are few (a window whose bucket lists one target twice), and a range of
// the introsort whose key interval holds none of them has distinct keys, so
// its final order is its sorted order.  So the hits are radix-sorted in
// place (the sorted order up to the order among equal keys), and the
// introsort is emulated on a copy in generation order, pruned to the
// ranges that may hold equal keys; the ranges it sorted are copied back.
// Without the recorded keys (more than the list holds), or with more than
// one per 64 hits, the whole introsort is emulated in place.
void flagged_sort(cuflye_ctx* c, PassState& ps, const MatchEmitLists& L, uint64_t* qb,
                  uint64_t* qe, uint32_t* ecount, uint64_t* alt_keys, uint32_t* alt_vals,
                  uint32_t* lscr, uint32_t* rscr, uint32_t* lists, uint32_t* scounts) {
  cudaStream_t st = c->stream;
  const uint64_t H = ps.nhits;
  const uint32_t nq = ps.nq;
  uint32_t back[2] = {0, 0};
  CUFLYE_CHECK(cudaMemcpyAsync(&back[0], ecount, 4, cudaMemcpyDeviceToHost, st));
  CUFLYE_CHECK(cudaMemcpyAsync(&back[1], L.tie_count, 4, cudaMemcpyDeviceToHost, st));
  sync(c);
  const uint32_t E = back[0], T = back[1];
  if (E == 0) return;
  if (T > L.tie_cap) {
    CUFLYE_CHECK(segmented_std_sort(ps.keys, ps.vals, lscr, rscr, qb, qe, nq, ecount, lists,
                                    scounts, c->num_sms, st, sort_tasks(c, "s", H, nq)));
    return;
  }
  std::vector<uint64_t> b(E), e(E), th(T), tk(T);
  CUFLYE_CHECK(cudaMemcpyAsync(b.data(), qb, E * 8ull, cudaMemcpyDeviceToHost, st));
  CUFLYE_CHECK(cudaMemcpyAsync(e.data(), qe, E * 8ull, cudaMemcpyDeviceToHost, st));
  if (T) {
    CUFLYE_CHECK(cudaMemcpyAsync(th.data(), L.tie_h0, T * 8ull, cudaMemcpyDeviceToHost, st));
    CUFLYE_CHECK(cudaMemcpyAsync(tk.data(), L.tie_key, T * 8ull, cudaMemcpyDeviceToHost, st));
  }
  sync(c);
  // segments in hit order, their places in the compact copy
  std::vector<uint32_t> ord(E);
  for (uint32_t i = 0; i < E; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) { return b[x] < b[y]; });
  // host staging: begin, end, compact begin, compact end (4 E words), then
  // the keys' offsets (E + 1) and the keys
  std::vector<uint64_t> seg(4ull * E);
  uint64_t F = 0;
  for (uint32_t i = 0; i < E; ++i) {
    seg[i] = b[ord[i]];
    seg[E + i] = e[ord[i]];
    seg[2ull * E + i] = F;
    F += e[ord[i]] - b[ord[i]];
    seg[3ull * E + i] = F;
  }
  if (static_cast<uint64_t>(T) * 64u > F) {
    // equal keys everywhere: the pruning would keep most ranges
    CUFLYE_CHECK(segmented_std_sort(ps.keys, ps.vals, lscr, rscr, qb, qe, nq, ecount, lists,
                                    scounts, c->num_sms, st, sort_tasks(c, "s", H, nq)));
    return;
  }
  std::vector<std::pair<uint32_t, uint64_t>> ties(T);
  for (uint32_t i = 0; i < T; ++i) {
    const uint32_t s = static_cast<uint32_t>(
        std::upper_bound(seg.begin(), seg.begin() + E, th[i]) - seg.begin() - 1);
    ties[i] = {s, tk[i]};
  }
  std::sort(ties.begin(), ties.end());
  ties.erase(std::unique(ties.begin(), ties.end()), ties.end());
  std::vector<uint32_t> poff(E + 1, 0);
  std::vector<uint64_t> pkeys(ties.size());
  for (size_t i = 0; i < ties.size(); ++i) {
    ++poff[ties[i].first + 1];
    pkeys[i] = ties[i].second;
  }
  for (uint32_t i = 0; i < E; ++i) poff[i + 1] += poff[i];
  uint64_t* dseg = buf<uint64_t>(c, "f_seg", 4ull * E);
  uint32_t* dpoff = buf<uint32_t>(c, "f_poff", E + 1);
  uint64_t* dpkeys = buf<uint64_t>(c, "f_pkeys", std::max<size_t>(pkeys.size(), 1));
  uint64_t* gk = buf<uint64_t>(c, "f_gk", F);
  uint32_t* gv = buf<uint32_t>(c, "f_gv", F);
  CUFLYE_CHECK(cudaMemcpyAsync(dseg, seg.data(), seg.size() * 8ull, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(dpoff, poff.data(), poff.size() * 4ull, cudaMemcpyHostToDevice, st));
  if (!pkeys.empty())
    CUFLYE_CHECK(cudaMemcpyAsync(dpkeys, pkeys.data(), pkeys.size() * 8ull,
                                 cudaMemcpyHostToDevice, st));
  const uint64_t* sb = dseg;
  const uint64_t* cb = dseg + 2ull * E;
  const uint64_t* ce = dseg + 3ull * E;
  // the generation order, gathered
  CUFLYE_CHECK(gather_ranges(ps.keys, ps.vals, sb, cb, E, F, gk, gv, c->num_sms, st));
  // the sorted order in place: a stable radix sort by ext id of each
  // flagged query's hits (in cur-pos order as generated)
  uint32_t* ntiles = buf<uint32_t>(c, "m_ntiles", nq);
  uint64_t* tile_off = buf<uint64_t>(c, "m_tileoff", nq + 1);
  int id_bits = 0;
  while (id_bits < 32 && ((2ull * c->idx.nslots - 1) >> id_bits) != 0) ++id_bits;
  CUFLYE_CHECK(match_plan(ps.q_off, ps.q_tie, nq, ntiles, nullptr, nullptr, nullptr, st, true));
  const uint64_t NT = scan_u32(c, ntiles, tile_off, nq, "m_scan");
  MatchTile* tiles = buf<MatchTile>(c, "m_tiles", NT);
  uint32_t* mcounts = buf<uint32_t>(c, "m_counts", 256 * NT);
  CUFLYE_CHECK(match_tiles(ps.q_off, ntiles, tile_off, nq, tiles, st));
  SortTasks t = sort_tasks(c, "f", F, E);
  t.prune_keys = dpkeys;
  t.prune_off = dpoff;
  // The radix sort (in place, with the second buffer) and the emulation (on
  // the copy) touch disjoint buffers: the radix sort runs on the side stream
  // beside the emulation's global phase, and the emulation's side-stream
  // work queues behind it, so the emulation's join also waits for it.  Every
  // buffer is allocated before the fork: an allocation may fail, and a pass
  // that is run again must find no work of the failed one still running.
  CUFLYE_CHECK(cudaEventRecord(c->side_ev[0], st));
  CUFLYE_CHECK(cudaStreamWaitEvent(c->side, c->side_ev[0], 0));
  CUFLYE_CHECK(match_radix(ps.keys, ps.vals, alt_keys, alt_vals, tiles, static_cast<uint32_t>(NT),
                           ps.q_off, ntiles, tile_off, nq, id_bits, mcounts, c->num_sms,
                           c->shape.scatter_blocks_per_sm, c->side));
  // the pruned introsort on the copy, and the ranges it sorted copied back
  CUFLYE_CHECK(segmented_std_sort(gk, gv, lscr, rscr, cb, ce, E, nullptr, lists, scounts,
                                  c->num_sms, st, t));
  CUFLYE_CHECK(copy_sorted_ranges(gk, gv, cb, ce, sb, E, scounts, t, ps.keys, ps.vals, c->num_sms,
                                  st));
}

// Sort + chaining of the pass's hits; returns the number of overlap rows left
// on the device in "o_rows" (OverlapRow, query order, Flye emission order).
uint64_t run_chain(cuflye_ctx* c, PassState& ps, const ChainParams& cp,
                   uint64_t* rows_per_query = nullptr) {
  cudaStream_t st = c->stream;
  const uint64_t H = ps.nhits;
  const uint32_t nq = ps.nq;
  uint32_t* lscr = buf<uint32_t>(c, "s_l", H + 1);
  uint32_t* rscr = buf<uint32_t>(c, "s_r", H + 1);
  uint32_t* lists = buf<uint32_t>(c, "s_lists", 4ull * std::max<uint64_t>(nq, 1));
  uint32_t* scounts = buf<uint32_t>(c, "s_counts", 16);
  uint32_t* ecount = buf<uint32_t>(c, "s_ecount", 1);
  uint64_t* sstats = buf<uint64_t>(c, "x_sortstats", kSortStats);
  CUFLYE_CHECK(cudaMemsetAsync(sstats, 0, kSortStats * 8, st));
  uint64_t* qb = buf<uint64_t>(c, "s_qb", nq);
  uint64_t* qe = buf<uint64_t>(c, "s_qe", nq);
  // second buffer of the radix passes (or the sorted emission's dictionary);
  // later the exact score orders
  uint64_t* alt_keys = buf<uint64_t>(c, "c_akeys", H + 1);
  uint32_t* alt_vals = buf<uint32_t>(c, "c_avals", H + 1);
  const int* slot_len = c->idx.slot_len;
  GroupInfo* groups = nullptr;
  uint64_t G = 0;
  uint32_t* ext_list = nullptr;
  uint32_t* dp_list = nullptr;
  uint32_t* gcounts = buf<uint32_t>(c, "g_counts", 4);
  bool fused = !ps.emitted;
  bool tally_pending = false;
  if (fused) {
    // Sorted emission: each query's dictionary of ext ids, then its hits
    // written in KmerMatch order with their groups; flagged queries'
    // hits in generation order for the libstdc++-order sort.
    MatchEmitArgs a;
    a.idx = c->idx;
    a.win_off = ps.qb.win_off;
    a.q_off = ps.q_off;
    a.hit_off = ps.hit_off;
    a.wmeta = ps.wmeta;
    a.wflags = ps.wflags;
    a.wself = ps.wself;
    a.filt_off = ps.filt_off;
    a.fpos = ps.fpos;
    a.status = c->status;
    a.nq = nq;
    uint32_t* q_ng = buf<uint32_t>(c, "m_qng", nq);
    uint64_t* q_dbase = buf<uint64_t>(c, "m_qdbase", nq);
    uint64_t* q_goff = buf<uint64_t>(c, "m_qgoff", nq + 1);
    uint32_t* mwords = buf<uint32_t>(c, "m_words", 4);  // overflow, counter, tie count
    unsigned long long* dcur = buf<unsigned long long>(c, "m_dcur", 3);  // cursor, tallies
    CUFLYE_CHECK(cudaMemsetAsync(mwords, 0, 4 * sizeof(uint32_t), st));
    CUFLYE_CHECK(cudaMemsetAsync(dcur, 0, 3 * sizeof(unsigned long long), st));
    CUFLYE_CHECK(match_dict(a, alt_keys, dcur, q_ng, q_dbase, mwords, mwords + 1, c->num_sms, st));
    // the group count and the overflow count in one read back
    scan_u32_async(c, q_ng, q_goff, nq, "m_scan");
    uint64_t back[2] = {0, 0};
    CUFLYE_CHECK(cudaMemcpyAsync(&back[0], q_goff + nq, 8, cudaMemcpyDeviceToHost, st));
    CUFLYE_CHECK(cudaMemcpyAsync(&back[1], mwords, 4, cudaMemcpyDeviceToHost, st));
    sync(c);
    G = back[0];
    if (back[1] != 0) {
      // a query with more than kMatchDictCap ext ids: this pass takes the
      // generation-order emission and the sort instead
      ++c->emission_fallbacks;
      emit_generation_order(c, ps);
      fused = false;
    } else {
      if (G >= (1ull << 32)) throw Error(CUFLYE_ERR_UNSUPPORTED, "more than 2^32 target groups");
      groups = buf<GroupInfo>(c, "g_info", G);
      ext_list = buf<uint32_t>(c, "g_extlist", G);
      dp_list = buf<uint32_t>(c, "g_dplist", G);
      uint32_t* pf_list = buf<uint32_t>(c, "g_pflist", G);
      CUFLYE_CHECK(cudaMemsetAsync(gcounts, 0, 4 * sizeof(uint32_t), st));
      CUFLYE_CHECK(cudaMemsetAsync(ecount, 0, sizeof(uint32_t), st));
      MatchEmitLists L{dp_list, ext_list, pf_list, gcounts, qb, qe, ecount, dcur + 1};
      L.tie_cap = static_cast<uint32_t>(std::min<uint64_t>(H / 16 + 1024, 1u << 22));
      L.tie_h0 = buf<uint64_t>(c, "f_tieh0", L.tie_cap);
      L.tie_key = buf<uint64_t>(c, "f_tiekey", L.tie_cap);
      L.tie_count = mwords + 2;
      CUFLYE_CHECK(cudaMemsetAsync(L.tie_count, 0, sizeof(uint32_t), st));
      CUFLYE_CHECK(match_emit(a, alt_keys, q_ng, q_dbase, q_goff, ps.q_tie, ps.qinfo, cp, ps.keys,
                              ps.vals, groups, L, mwords + 1, c->num_sms, st));
      CUFLYE_CHECK(cudaEventRecord(c->ev[1], st));
      // 1. the flagged queries' KmerMatch sort in libstdc++ order
      CUFLYE_CHECK(sort_stats_add(sstats, 0, 1, nullptr, nq, ecount, st));
      flagged_sort(c, ps, L, qb, qe, ecount, alt_keys, alt_vals, lscr, rscr, lists, scounts);
      CUFLYE_CHECK(cudaEventRecord(c->ev[2], st));
      // 2. the prefilter of the groups the emission left open
      CUFLYE_CHECK(groups_prefilter_list(ps.keys, ps.vals, groups, pf_list, ps.qinfo, slot_len, cp,
                                         ext_list, dp_list, gcounts, static_cast<uint32_t>(G),
                                         st));
      // read back with the survivor count below (one stream sync)
      CUFLYE_CHECK(cudaMemcpyAsync(c->emit_tally, dcur + 1, sizeof(c->emit_tally),
                                   cudaMemcpyDeviceToHost, st));
      tally_pending = true;
      c->hits_sorted_emission += H;
    }
  }
  if (!fused) {
    // 1. KmerMatch sort per query by (ext id, cur pos) in libstdc++ order:
    // queries whose keys are distinct by a radix sort on the ext id, the
    // others by the emulated introsort
    uint32_t* ntiles = buf<uint32_t>(c, "m_ntiles", nq);
    uint64_t* tile_off = buf<uint64_t>(c, "m_tileoff", nq + 1);
    int id_bits = 0;
    while (id_bits < 32 && ((2ull * c->idx.nslots - 1) >> id_bits) != 0) ++id_bits;
    CUFLYE_CHECK(cudaEventRecord(c->ev[1], st));
    CUFLYE_CHECK(match_plan(ps.q_off, ps.q_tie, nq, ntiles, qb, qe, ecount, st));
    CUFLYE_CHECK(sort_stats_add(sstats, 0, 1, nullptr, nq, ecount, st));
    const uint64_t NT = scan_u32(c, ntiles, tile_off, nq, "m_scan");
    MatchTile* tiles = buf<MatchTile>(c, "m_tiles", NT);
    uint32_t* mcounts = buf<uint32_t>(c, "m_counts", 256 * NT);
    CUFLYE_CHECK(match_tiles(ps.q_off, ntiles, tile_off, nq, tiles, st));
    CUFLYE_CHECK(match_radix(ps.keys, ps.vals, alt_keys, alt_vals, tiles,
                             static_cast<uint32_t>(NT), ps.q_off, ntiles, tile_off, nq, id_bits,
                             mcounts, c->num_sms, c->shape.scatter_blocks_per_sm, st));
    CUFLYE_CHECK(segmented_std_sort(ps.keys, ps.vals, lscr, rscr, qb, qe, nq, ecount, lists,
                                    scounts, c->num_sms, st, sort_tasks(c, "s", H, nq)));
    CUFLYE_CHECK(cudaEventRecord(c->ev[2], st));
    // 2. groups: runs of one ext id within a query
    const uint64_t gtiles = (H + kGroupTile - 1) / kGroupTile;
    uint32_t* gtcount = buf<uint32_t>(c, "g_tcount", gtiles);
    uint64_t* gtoff = buf<uint64_t>(c, "g_toff", gtiles + 1);
    CUFLYE_CHECK(groups_count(ps.keys, ps.q_off, nq, H, gtcount, st));
    G = scan_u32(c, gtcount, gtoff, gtiles, "g_scan");
    if (G >= (1ull << 32)) throw Error(CUFLYE_ERR_UNSUPPORTED, "more than 2^32 target groups");
    groups = buf<GroupInfo>(c, "g_info", G);
    CUFLYE_CHECK(groups_write(ps.keys, ps.q_off, nq, H, gtoff, groups, st));
    ext_list = buf<uint32_t>(c, "g_extlist", G);
    dp_list = buf<uint32_t>(c, "g_dplist", G);
    CUFLYE_CHECK(groups_prefilter_n(ps.keys, ps.vals, groups, G, H, ps.qinfo, slot_len, cp,
                                    ext_list, dp_list, gcounts, st));
    c->hits_emit_sort += H;
  }
  uint64_t* sb = buf<uint64_t>(c, "g_sb", G);
  uint64_t* se = buf<uint64_t>(c, "g_se", G);
  uint32_t* glists = buf<uint32_t>(c, "g_lists", 4 * std::max<uint64_t>(G, 1));
  const uint32_t G32 = static_cast<uint32_t>(G);
  // 3. ext-sorted groups in ext-pos order: most already are (checked, read in
  // place); the rest are re-sorted in shared memory, or by the emulated
  // introsort where ext positions repeat
  uint32_t* work = buf<uint32_t>(c, "c_work", 1);
  uint32_t* resort = buf<uint32_t>(c, "g_resort", G);
  uint32_t* resort_count = buf<uint32_t>(c, "g_resortcount", 1);
  CUFLYE_CHECK(groups_ext_presorted(ps.vals, groups, ext_list, gcounts, resort, resort_count, st));
  CUFLYE_CHECK(group_ext_sort(ps.keys, ps.vals, groups, resort, resort_count, G32, sb, se, ecount,
                              lscr, rscr, reinterpret_cast<uint32_t*>(alt_keys), H, work,
                              c->num_sms, st));
  CUFLYE_CHECK(sort_stats_add(sstats, 2, 3, gcounts + 0, 0, ecount, st));
  CUFLYE_CHECK(segmented_std_sort(ps.keys, ps.vals, lscr, rscr, sb, se, G32, ecount, glists,
                                  scounts, c->num_sms, st, sort_tasks(c, "s", H, G32)));
  // 4. DP over the sorted pairs
  int32_t* score = buf<int32_t>(c, "c_score", H);
  int32_t* bt = buf<int32_t>(c, "c_bt", H);
  GroupTop* top = buf<GroupTop>(c, "c_top", G);
  // the surviving groups in length buckets, longest first, for the
  // warp-per-group stages (warps take them from a counter)
  uint32_t* blist = buf<uint32_t>(c, "g_lenlist", G);
  CUFLYE_CHECK(groups_length_order(groups, dp_list, gcounts + 1, G32,
                                   buf<uint32_t>(c, "g_lenscr", 10), blist, st));
  CUFLYE_CHECK(cudaEventRecord(c->ev[6], st));
  int32_t* pmc = buf<int32_t>(c, "c_pmc", chain_dp_pmc_words(H, G));
  CUFLYE_CHECK(chain_dp(ps.keys, ps.vals, score, bt, groups, blist, gcounts, cp, top, pmc, work,
                        c->num_sms, c->shape.dp_blocks_per_sm, st));
  CUFLYE_CHECK(cudaEventRecord(c->ev[7], st));
  // 5. the backtrack picks its chain starts by score itself; groups where
  // Flye's order among equal scores could matter get that order (libstdc++
  // order of indices by score descending) and run again.  The (key, index)
  // pairs of the order live in the radix sort's second buffer, free by now.
  uint64_t* okeys = alt_keys;
  uint32_t* order = alt_vals;
  const uint64_t gmap_words = chain_dp_pmc_words(H, G);
  uint32_t* gmaps = buf<uint32_t>(c, "o_maps", 4 * gmap_words);
  // 6. backtrack, proposals, primary selection; the row pool is sized by the
  // groups that survived the prefilter
  const uint32_t survivors = read_scalar(c, gcounts + 1);
  if (tally_pending) {
    c->hits_flagged += c->emit_tally[0];
    c->hits_prefiltered += c->emit_tally[1];
  }
  const uint64_t pool_cap = 8ull * survivors + 1024;
  OverlapRow* pool = buf<OverlapRow>(c, "o_pool", pool_cap);
  uint32_t* pool_count = buf<uint32_t>(c, "o_poolcount", 1);
  uint32_t* group_rows = buf<uint32_t>(c, "o_grows", G);
  CUFLYE_CHECK(cudaMemsetAsync(pool_count, 0, 4, st));
  CUFLYE_CHECK(cudaMemsetAsync(group_rows, 0, std::max<uint64_t>(G, 1) * 4, st));
  uint32_t* redo = buf<uint32_t>(c, "o_redo", G);
  uint32_t* redo_count = buf<uint32_t>(c, "o_redocount", 1);
  CUFLYE_CHECK(cudaMemsetAsync(redo_count, 0, 4, st));
  const int64_t* slot_signed = c->idx.slot_signed;
  CUFLYE_CHECK(chain_backtrack(ps.keys, ps.vals, score, bt, order, groups, blist, gcounts + 1, top,
                               redo, redo_count, ps.qinfo, ps.f_off, ps.fpos, slot_signed, c->logt,
                               cp, pool, pool_cap, pool_count, group_rows, c->status, G32, gmaps,
                               gmap_words, work, c->shape.backtrack_blocks_per_sm, st));
  CUFLYE_CHECK(sort_stats_add(sstats, 4, 6, gcounts + 1, 0, redo_count, st));
  // groups whose result could depend on the order among equal scores: again
  // with the libstdc++ order
  CUFLYE_CHECK(chain_prepare_order(score, okeys, order, groups, redo, redo_count, sb, se, st));
  CUFLYE_CHECK(segmented_std_sort(okeys, order, lscr, rscr, sb, se, G32, redo_count, glists,
                                  scounts, c->num_sms, st, sort_tasks(c, "s", H, G32)));
  CUFLYE_CHECK(chain_backtrack(ps.keys, ps.vals, score, bt, order, groups, redo, redo_count, nullptr,
                               nullptr, nullptr, ps.qinfo, ps.f_off, ps.fpos, slot_signed, c->logt,
                               cp, pool, pool_cap, pool_count, group_rows, c->status, G32, gmaps,
                               gmap_words, work, c->shape.backtrack_blocks_per_sm, st));
  check_device_status(c);
  // 7. max_overlaps + compaction in group order
  uint64_t* qg = buf<uint64_t>(c, "o_qg", nq + 1);
  CUFLYE_CHECK(query_group_offsets(groups, G, nq, qg, st));
  uint32_t* kept = buf<uint32_t>(c, "o_kept", G);
  if (cp.max_overlaps > 0) {
    CUFLYE_CHECK(rows_limit(group_rows, qg, nq, cp.max_overlaps, kept, st));
  } else {
    kept = group_rows;
  }
  uint64_t* kept_off = buf<uint64_t>(c, "o_keptoff", G + 1);
  const uint64_t R = scan_u32(c, kept, kept_off, G, "o_scan");
  const uint32_t npool = read_scalar(c, pool_count);
  OverlapRow* rows = buf<OverlapRow>(c, "o_rows", R);
  CUFLYE_CHECK(rows_scatter(pool, npool, kept, kept_off, rows, st));
  // each query's first row (rows are in query order)
  CUFLYE_CHECK(gather_query_offsets(qg, kept_off, nq, buf<uint64_t>(c, "o_qrowoff", nq + 1), st));
  if (rows_per_query) {
    uint64_t* qrows = buf<uint64_t>(c, "o_qrows", nq);
    CUFLYE_CHECK(query_row_counts(qg, kept_off, nq, qrows, st));
    CUFLYE_CHECK(cudaMemcpyAsync(rows_per_query, qrows, nq * sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, st));
  }
  CUFLYE_CHECK(cudaEventRecord(c->ev[3], st));
  return R;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return ms;
}

void reset_timing(cuflye_ctx* c) {
  c->passes = 0;
  c->pass_retries = 0;
  c->pass_hit_cap = 0;
  c->alloc_ms = 0;
  c->emission_fallbacks = 0;
  c->sort_stats[7] = 0;
  c->hits_sorted_emission = c->hits_flagged = c->hits_prefiltered = c->hits_emit_sort = 0;
  for (int i = 0; i < kStages; ++i) {
    c->stage_ms[i] = 0;
    c->stage_bytes[i] = 0;
    c->sort_stats[i] = 0;
  }
}

// Stages (see cuflye_last_timing): 0 hits, 1 match sort, 2 groups, 3 DP,
// 4 backtrack + rows, 5 output + D2H, 6 H2D.
void accumulate_timing(cuflye_ctx* c, bool chained) {
  sync(c);
  if (chained) {
    uint64_t st[kSortStats];
    CUFLYE_CHECK(cudaMemcpy(st, buf<uint64_t>(c, "x_sortstats", kSortStats), sizeof(st),
                            cudaMemcpyDeviceToHost));
    for (int i = 0; i < kSortStats; ++i) c->sort_stats[i] += st[i];
    c->sort_stats[7] = c->emission_fallbacks;
  }
  c->stage_ms[6] += elapsed(c->ev[0], c->ev[5]);
  c->stage_ms[0] += elapsed(c->ev[5], c->ev[1]);
  if (chained) {
    c->stage_ms[1] += elapsed(c->ev[1], c->ev[2]);
    c->stage_ms[2] += elapsed(c->ev[2], c->ev[6]);
    c->stage_ms[3] += elapsed(c->ev[6], c->ev[7]);
    c->stage_ms[4] += elapsed(c->ev[7], c->ev[3]);
    c->stage_ms[5] += elapsed(c->ev[3], c->ev[4]);
  }
}

// Compulsory traffic per stage: the bases and one probe sector per window,
// bucket entries read (8 B) and hit records written (12 B); a read and a
// write of every 12-byte record the KmerMatch sort moves (all hits on the
// emit + sort path, the flagged queries' hits on the sorted emission); the
// group stage reads the records of the groups it prefilters (12 B each, and
// on the emit + sort path another 8 B for the group bounds and ext
// positions); the DP reads (cur, ext) and writes (score, backtrack); the
// backtrack reads its table once.
void set_stage_bytes(cuflye_ctx* c, uint64_t bases, uint64_t windows, uint64_t hits) {
  c->stage_bytes[0] = bases / 4 + windows * 32 + hits * 20;
  c->stage_bytes[1] = (c->hits_emit_sort + c->hits_flagged) * 24;
  c->stage_bytes[2] = c->hits_emit_sort * 20 + c->hits_prefiltered * 12;
  c->stage_bytes[3] = hits * 16;
  c->stage_bytes[4] = hits * 4;
}

size_t pass_size(cuflye_ctx* c, size_t n) {
  if (c->queries_per_pass) return std::min(n, c->queries_per_pass);
  return n;
}

// Buffers a pass body does not own: the index, the graph, the logf table, the
// status word, and the per-hit and per-window buffers that passes reuse.
bool kept_buffer(const std::string& name) {
  static const char* const kPrefixes[] = {"ix_", "gr_", "logf_", "q_"};
  for (const char* p : kPrefixes)
    if (name.compare(0, std::strlen(p), p) == 0) return true;
  if (name == "status") return true;
  for (const char* nm : kPerHitBuffers)
    if (name == nm) return true;
  for (const char* nm : kPerWindowBuffers)
    if (name == nm) return true;
  return false;
}

// Frees every buffer of the pass body (its tables, lists and rows).
void release_pass_buffers(cuflye_ctx* c) {
  std::vector<std::string> names;
  for (const auto& kv : c->bufs)
    if (!kept_buffer(kv.first)) names.push_back(kv.first);
  for (const std::string& n : names) release(c, n);
}

// Runs passes over [0, n): `body(q0, q1, ps)` consumes each pass.  A body
// whose later buffers (per-group tables, the row pool) do not fit the budget
// runs again on the first half of the pass's queries; bodies make their
// results visible only after their last allocation, so the retry repeats no
// output.
template <typename Body>
void for_each_pass(cuflye_ctx* c, const Queries& Q, bool kmers, uint64_t bytes_per_hit,
                   Body body) {
  size_t q0 = 0;
  const size_t full = std::max<size_t>(pass_size(c, Q.n), 1);
  size_t step = full;
  double hpw = 0;  // hits per window of the previous pass
  while (q0 < Q.n) {
    size_t q1 = run_end(c, Q, q0, std::min(Q.n, q0 + step), bytes_per_hit, hpw);
    PassState ps;
    c->pass_need.clear();
    CUFLYE_CHECK(cudaEventRecord(c->ev[0], c->stream));
    run_hits(c, Q, q0, q1, kmers, bytes_per_hit, ps);
    q1 = q0 + ps.nq;
    CUFLYE_CHECK(cudaEventRecord(c->ev[1], c->stream));
    try {
      body(q0, q1, ps);
    } catch (const Error& e) {
      if (e.code != CUFLYE_ERR_BUDGET || ps.nq <= 1) throw;
      // the failed body's buffers go, so that half the queries find room
      sync(c);
      release_pass_buffers(c);
      ++c->pass_retries;
      // later passes of the call stay at the size that is tried next
      c->pass_hit_cap = std::max<uint64_t>(1, ps.nhits / 2);
      step = std::max<size_t>(ps.nq / 2, 1);
      continue;
    }
    // Learn the body's other buffers per hit from the ones this pass used
    // (at the size they are held), and only from passes of at least a 64th
    // of what the memory left could hold: a small pass's tables (held at the
    // size an earlier, larger pass grew them to), divided by its few hits,
    // would make every later pass of the context tiny.
    if (c->budget && ps.nhits && ps.nhits * 64 >= ps.fit_hits) {
      uint64_t other = 0;
      for (const auto& kv : c->pass_need) {
        if (kept_buffer(kv.first)) continue;
        auto it = c->bufs.find(kv.first);
        if (it != c->bufs.end()) other += it->second.cap;
      }
      c->other_per_hit =
          std::max(c->other_per_hit, static_cast<double>(other) / static_cast<double>(ps.nhits));
    }
    ++c->passes;
    q0 = q1;
    step = std::min(full, step * 2);  // a halved step grows back after a pass that fits
    if (ps.nwin) hpw = static_cast<double>(ps.nhits) / static_cast<double>(ps.nwin);
  }
}

// Device bytes per hit of one pass: keys, values, the two rank maps, the
// radix sort's second key / value buffer, score and backtrack, plus about 2
// bytes for the per-group tables, tiles, bitmaps and the sort's task list.
constexpr uint64_t kChainBytesPerHit = 8 + 4 + 4 + 4 + 8 + 4 + 4 + 4 + 2;

void require_index(cuflye_ctx* c) {
  if (!c->has_index) throw Error(CUFLYE_ERR_NO_INDEX, "no k-mer index: call cuflye_index_build");
}

void check_params(cuflye_ctx* c, const cuflye_overlap_params* p) {
  if (!p) throw Error(CUFLYE_ERR_INVALID, "params must not be null");
  if (p->kmer_size != c->idx.k)
    throw Error(CUFLYE_ERR_INVALID, "params.kmer_size differs from the index k");
  if (p->max_jump <= 0 || p->min_overlap < 0)
    throw Error(CUFLYE_ERR_INVALID, "max_jump must be > 0 and min_overlap >= 0");
}

// Device buffers for graph tables.
struct GraphDev {
  int64_t* edge_of_slot;
  int32_t* left;
  int32_t* right;
};

}  // namespace

// ================================================================ C ABI

namespace {

// The reference stub's fail-fast text names the adapter, the device and the
// budget (patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-46); an
// unsupported shape or an exhausted budget keeps those fields in front of
// the reason, so Flye's runtime_error reads the same way.
std::string stub_fields(int device, uint64_t budget) {
  return "cuFlye CUDA candidate backend selected; adapter=cuflye_gb300; CUFLYE_CUDA_DEVICE=" +
         std::to_string(device) + "; CUFLYE_CUDA_MEMORY_BUDGET_BYTES=" +
         (budget ? std::to_string(budget) : std::string("unbounded")) + "; ";
}

std::string fail_text(const cuflye_ctx* c, const Error& e) {
  if (e.code == CUFLYE_ERR_UNSUPPORTED || e.code == CUFLYE_ERR_BUDGET)
    return stub_fields(c->device, c->budget) + e.what();
  return e.what();
}

// Why the calling thread's last cuflye_open / cuflye_open_from_env failed
// (there is no context to hold it); cuflye_last_error(NULL) returns it.
thread_local std::string t_open_error;

}  // namespace

#define CUFLYE_API_BEGIN(ctx)                   \
  if (!(ctx)) return CUFLYE_ERR_INVALID;        \
  std::lock_guard<std::mutex> lock_((ctx)->mu); \
  try {
#define CUFLYE_API_END(ctx)           \
  }                                   \
  catch (const Error& e) {            \
    (ctx)->err = fail_text(ctx, e);   \
    return e.code;                    \
  }                                   \
  catch (const std::exception& e) {   \
    (ctx)->err = e.what();            \
    return CUFLYE_ERR_CUDA;           \
  }                                   \
  (ctx)->err.clear();                 \
  return CUFLYE_OK;

extern "C" {

int cuflye_candidate_backend(char* msg, size_t msg_cap) {
  const char* v = std::getenv("CUFLYE_CANDIDATE_BACKEND");
  if (!v || !v[0] || std::strcmp(v, "cpu") == 0) return 0;
  if (std::strcmp(v, "cuda") == 0) return 1;
  if (msg && msg_cap) std::snprintf(msg, msg_cap, "Unsupported CUFLYE_CANDIDATE_BACKEND: %s", v);
  return -1;
}

cuflye_status cuflye_open(int device, uint64_t memory_budget_bytes, cuflye_ctx** out) {
  if (!out) {
    t_open_error = "cuflye_open: null output pointer";
    return CUFLYE_ERR_INVALID;
  }
  *out = nullptr;
  cuflye_ctx* c = new cuflye_ctx();
  try {
    int ndev = 0;
    CUFLYE_CHECK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev)
      throw Error(CUFLYE_ERR_INVALID, "CUFLYE_CUDA_DEVICE=" + std::to_string(device) +
                                          " is not a visible device (" + std::to_string(ndev) +
                                          " visible)");
    c->device = device;
    c->budget = memory_budget_bytes;
    CUFLYE_CHECK(cudaSetDevice(device));
    CUFLYE_CHECK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CUFLYE_CHECK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    for (auto& e : c->ev) CUFLYE_CHECK(cudaEventCreate(&e));
    CUFLYE_CHECK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CUFLYE_CHECK(cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking));
    for (auto& e : c->side_ev) CUFLYE_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->status = buf<DeviceStatus>(c, "status", 1);
    CUFLYE_CHECK(cudaMemset(c->status, 0, sizeof(DeviceStatus)));
    load_logf_table(c);
  } catch (const Error& e) {
    t_open_error = stub_fields(device, memory_budget_bytes) + e.what();
    cuflye_close(c);
    return e.code;
  }
  t_open_error.clear();
  *out = c;
  return CUFLYE_OK;
}

cuflye_status cuflye_open_from_env(cuflye_ctx** out) {
  const char* dev = std::getenv("CUFLYE_CUDA_DEVICE");
  const char* bud = std::getenv("CUFLYE_CUDA_MEMORY_BUDGET_BYTES");
  int d = 0;
  uint64_t b = 0;
  auto bad = [&](const char* what) {
    t_open_error = std::string("cuFlye CUDA candidate backend selected; adapter=cuflye_gb300; "
                               "CUFLYE_CUDA_DEVICE=") +
                   (dev && dev[0] ? dev : "0") + "; CUFLYE_CUDA_MEMORY_BUDGET_BYTES=" +
                   (bud && bud[0] ? bud : "unbounded") + "; " + what;
    if (out) *out = nullptr;
    return CUFLYE_ERR_INVALID;
  };
  if (dev && dev[0]) {
    char* end = nullptr;
    errno = 0;
    long v = std::strtol(dev, &end, 10);
    if (!end || *end || errno || v < 0 || v > INT_MAX)
      return bad("CUFLYE_CUDA_DEVICE is not a device ordinal");
    d = static_cast<int>(v);
  }
  if (bud && bud[0] && std::strcmp(bud, "unbounded") != 0) {
    char* end = nullptr;
    errno = 0;
    unsigned long long v = std::strtoull(bud, &end, 10);
    if (!end || *end || errno || bud[0] == '-')
      return bad("CUFLYE_CUDA_MEMORY_BUDGET_BYTES is neither a byte count nor \"unbounded\"");
    b = v;
  }
  return cuflye_open(d, b, out);
}

cuflye_status cuflye_open_shared(cuflye_ctx* owner, uint64_t memory_budget_bytes,
                                 cuflye_ctx** out) {
  if (!out) return CUFLYE_ERR_INVALID;
  *out = nullptr;
  if (!owner) return CUFLYE_ERR_INVALID;
  int device = 0;
  {
    std::lock_guard<std::mutex> lock(owner->mu);
    if (!owner->has_index) {
      owner->err = "cuflye_open_shared: the owner has no index";
      return CUFLYE_ERR_NO_INDEX;
    }
    if (owner->lender) {
      owner->err = "cuflye_open_shared: the owner borrows its index itself";
      return CUFLYE_ERR_INVALID;
    }
    device = owner->device;
  }
  cuflye_ctx* c = nullptr;
  const cuflye_status st = cuflye_open(device, memory_budget_bytes, &c);
  if (st != CUFLYE_OK) return st;
  std::lock_guard<std::mutex> lock(owner->mu);
  // the owner's resident index, read only (its device buffers stay the owner's)
  c->idx = owner->idx;
  c->slot_of = owner->slot_of;
  c->slot_signed_h = owner->slot_signed_h;
  c->has_index = true;
  c->lender = owner;
  ++owner->servers;
  *out = c;
  return CUFLYE_OK;
}

void cuflye_close(cuflye_ctx* c) {
  if (!c) return;
  if (c->lender) {
    std::lock_guard<std::mutex> lock(c->lender->mu);
    --c->lender->servers;
  }
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& kv : c->bufs)
    if (kv.second.p) cudaFree(kv.second.p);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->side2) cudaStreamSynchronize(c->side2);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->side_ev)
    if (e) cudaEventDestroy(e);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->side2) cudaStreamDestroy(c->side2);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* cuflye_last_error(const cuflye_ctx* c) {
  return c ? c->err.c_str() : t_open_error.c_str();
}

cuflye_status cuflye_memory_stats(const cuflye_ctx* c, uint64_t* in_use, uint64_t* peak) {
  if (!c) return CUFLYE_ERR_INVALID;
  if (in_use) *in_use = c->in_use;
  if (peak) *peak = c->peak;
  return CUFLYE_OK;
}

cuflye_status cuflye_index_build(cuflye_ctx* c, int k, size_t n, const int64_t* ids,
                                 const int64_t* offsets, const char* bases, uint32_t min_freq,
                                 uint32_t max_freq) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  if (!ids || !offsets || (!bases && n)) throw Error(CUFLYE_ERR_INVALID, "null input");
  if (c->servers)
    throw Error(CUFLYE_ERR_INVALID, "a serving loop or shared context borrows this context's "
                                    "index; close it first");
  if (c->lender)
    throw Error(CUFLYE_ERR_INVALID, "this context shares another context's index");
  build_index(c, k, n, ids, offsets, bases, min_freq, max_freq);
  CUFLYE_API_END(c)
}

cuflye_status cuflye_index_from_entries(cuflye_ctx* c, int k, size_t n, const int64_t* tids,
                                        const int64_t* positions, const uint64_t* keys,
                                        size_t n_rep, const uint64_t* rep_keys) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  if (c->servers)
    throw Error(CUFLYE_ERR_INVALID, "a serving loop or shared context borrows this context's "
                                    "index; close it first");
  if (c->lender)
    throw Error(CUFLYE_ERR_INVALID, "this context shares another context's index");
  build_index_entries(c, k, n, tids, positions, keys, n_rep, rep_keys);
  CUFLYE_API_END(c)
}

cuflye_status cuflye_index_stats(const cuflye_ctx* c, uint64_t* keys, uint64_t* positions,
                                 uint64_t* repetitive) {
  if (!c) return CUFLYE_ERR_INVALID;
  if (!c->has_index) return CUFLYE_ERR_NO_INDEX;
  if (keys) *keys = c->idx.nkeys;
  if (positions) *positions = c->idx.npos;
  if (repetitive) *repetitive = c->idx.nrep;
  return CUFLYE_OK;
}

cuflye_status cuflye_set_batch_queries(cuflye_ctx* c, size_t q) {
  if (!c) return CUFLYE_ERR_INVALID;
  c->queries_per_pass = q;
  return CUFLYE_OK;
}

cuflye_status cuflye_set_sorted_emission(cuflye_ctx* c, int enable) {
  if (!c || enable < 0 || enable > 2) return CUFLYE_ERR_INVALID;
  std::lock_guard<std::mutex> lock(c->mu);
  c->sorted_emission = enable;
  return CUFLYE_OK;
}

cuflye_status cuflye_set_launch_shape(cuflye_ctx* c, const cuflye_launch_shape* s) {
  if (!c || !s) return CUFLYE_ERR_INVALID;
  if (s->dp_blocks_per_sm < 0 || s->dp_blocks_per_sm > 8 || s->backtrack_blocks_per_sm < 0 ||
      s->backtrack_blocks_per_sm > 4 || s->scatter_blocks_per_sm < 0 ||
      s->scatter_blocks_per_sm > 2 || s->round_blocks_per_sm < 0 || s->round_blocks_per_sm > 2) {
    std::lock_guard<std::mutex> g(c->mu);
    c->err = "launch shape out of range (DP 0-8, backtrack 0-4, scatter 0-2, rounds 0-2)";
    return CUFLYE_ERR_INVALID;
  }
  c->shape = *s;
  return CUFLYE_OK;
}

cuflye_status cuflye_get_launch_shape(const cuflye_ctx* c, cuflye_launch_shape* s) {
  if (!c || !s) return CUFLYE_ERR_INVALID;
  *s = c->shape;
  return CUFLYE_OK;
}

namespace {
// Device time (stages 0-4) of one overlap call on Q; the rows stay on the
// device.
double overlaps_device_ms(cuflye_ctx* c, const Queries& Q, const ChainParams& cp) {
  reset_timing(c);
  for_each_pass(c, Q, false, kChainBytesPerHit, [&](size_t, size_t, PassState& ps) {
    run_chain(c, ps, cp);
    CUFLYE_CHECK(cudaEventRecord(c->ev[4], c->stream));
    accumulate_timing(c, true);
  });
  double ms = 0;
  for (int i = 0; i < 5; ++i) ms += c->stage_ms[i];
  return ms;
}
}  // namespace

cuflye_status cuflye_autotune(cuflye_ctx* c, size_t n, const int64_t* ids, const int64_t* offsets,
                              const char* bases, const cuflye_overlap_params* params,
                              cuflye_launch_shape* chosen, double* ms_start, double* ms_chosen) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  require_index(c);
  check_params(c, params);
  if (!ids || !offsets || (!bases && n)) throw Error(CUFLYE_ERR_INVALID, "null input");
  const ChainParams cp = to_chain_params(params);
  const Queries Q{n, ids, offsets, bases};
  const cuflye_launch_shape start_shape = c->shape;
  try {
    auto best_of_two = [&]() {
      const double a = overlaps_device_ms(c, Q, cp);
      return std::min(a, overlaps_device_ms(c, Q, cp));
    };
    overlaps_device_ms(c, Q, cp);  // buffers at their sizes
    const double start = best_of_two();
    double best = start;
    struct Knob {
      int32_t cuflye_launch_shape::*field;
      int32_t dflt;
      std::vector<int32_t> values;
    };
    const Knob knobs[] = {{&cuflye_launch_shape::dp_blocks_per_sm, 8, {2, 4, 6, 8}},
                          {&cuflye_launch_shape::backtrack_blocks_per_sm, 4, {1, 2, 3, 4}},
                          {&cuflye_launch_shape::scatter_blocks_per_sm, 2, {1, 2}},
                          {&cuflye_launch_shape::round_blocks_per_sm, 2, {1, 2}}};
    for (const Knob& k : knobs) {
      const int32_t cur = c->shape.*k.field ? c->shape.*k.field : k.dflt;
      int32_t pick = cur;
      for (int32_t v : k.values) {
        if (v == cur) continue;
        c->shape.*k.field = v;
        const double t = best_of_two();
        if (t < best * 0.99) {
          best = t;
          pick = v;
        }
      }
      c->shape.*k.field = pick;
    }
    if (chosen) *chosen = c->shape;
    if (ms_start) *ms_start = start;
    if (ms_chosen) *ms_chosen = best;
  } catch (...) {
    c->shape = start_shape;
    throw;
  }
  CUFLYE_API_END(c)
}

cuflye_status cuflye_candidates(cuflye_ctx* c, size_t n, const int64_t* ids,
                                const int64_t* offsets, const char* bases, cuflye_candidate* out,
                                size_t out_cap, size_t* n_out, cuflye_filtered_pos* filtered,
                                size_t filtered_cap, size_t* n_filtered) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  require_index(c);
  if (!ids || !offsets || (!bases && n)) throw Error(CUFLYE_ERR_INVALID, "null input");
  reset_timing(c);
  Queries Q{n, ids, offsets, bases};
  size_t total = 0, ftotal = 0;
  bool overflow = false;
  for_each_pass(c, Q, true, 8 + 4 + 8 + 32, [&](size_t, size_t, PassState& ps) {
    if (!overflow && total + ps.nhits <= out_cap && ftotal + ps.nfilt <= filtered_cap) {
      cuflye_candidate* d_out = buf<cuflye_candidate>(c, "a_cand", ps.nhits);
      cuflye_filtered_pos* d_f = buf<cuflye_filtered_pos>(c, "a_filt", ps.nfilt);
      CUFLYE_CHECK(hits_to_abi(ps.keys, ps.vals, ps.kmers, ps.nhits, ps.q_off, ps.nq, ps.qinfo,
                               c->idx.slot_signed, d_out, c->stream));
      CUFLYE_CHECK(filtered_to_abi(ps.fpos, ps.nfilt, ps.f_off, ps.nq, ps.qinfo, d_f, c->stream));
      if (ps.nhits)
        CUFLYE_CHECK(cudaMemcpyAsync(out + total, d_out, ps.nhits * sizeof(cuflye_candidate),
                                     cudaMemcpyDeviceToHost, c->stream));
      if (ps.nfilt)
        CUFLYE_CHECK(cudaMemcpyAsync(filtered + ftotal, d_f,
                                     ps.nfilt * sizeof(cuflye_filtered_pos),
                                     cudaMemcpyDeviceToHost, c->stream));
      sync(c);
    } else {
      overflow = true;
    }
    total += ps.nhits;
    ftotal += ps.nfilt;
    accumulate_timing(c, false);
  });
  if (n_out) *n_out = total;
  if (n_filtered) *n_filtered = ftotal;
  if (overflow)
    throw Error(CUFLYE_ERR_CAPACITY, "output capacity too small: need " + std::to_string(total) +
                                         " candidates and " + std::to_string(ftotal) +
                                         " filtered positions");
  CUFLYE_API_END(c)
}

cuflye_status cuflye_overlaps(cuflye_ctx* c, size_t n, const int64_t* ids, const int64_t* offsets,
                              const char* bases, const cuflye_overlap_params* params,
                              cuflye_overlap_range* out, size_t out_cap, size_t* n_out) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  require_index(c);
  check_params(c, params);
  if (!ids || !offsets || (!bases && n)) throw Error(CUFLYE_ERR_INVALID, "null input");
  reset_timing(c);
  const ChainParams cp = to_chain_params(params);
  Queries Q{n, ids, offsets, bases};
  size_t total = 0;
  bool overflow = false;
  uint64_t hits_total = 0, windows_total = 0, bases_total = 0;
  for_each_pass(c, Q, false, kChainBytesPerHit, [&](size_t q0, size_t q1, PassState& ps) {
    const uint64_t R = run_chain(c, ps, cp);
    if (!overflow && total + R <= out_cap) {
      cuflye_overlap_range* d_out = buf<cuflye_overlap_range>(c, "a_ovl", R);
      CUFLYE_CHECK(rows_to_abi(buf<OverlapRow>(c, "o_rows", R), R, ps.qinfo,
                               c->idx.slot_signed, d_out, c->stream));
      if (R)
        CUFLYE_CHECK(cudaMemcpyAsync(out + total, d_out, R * sizeof(cuflye_overlap_range),
                                     cudaMemcpyDeviceToHost, c->stream));
    } else {
      overflow = true;
    }
    hits_total += ps.nhits;
    windows_total += ps.nwin;
    bases_total += static_cast<uint64_t>(offsets[q1] - offsets[q0]);
    CUFLYE_CHECK(cudaEventRecord(c->ev[4], c->stream));
    total += R;
    accumulate_timing(c, true);
  });
  set_stage_bytes(c, bases_total, windows_total, hits_total);
  if (n_out) *n_out = total;
  if (overflow)
    throw Error(CUFLYE_ERR_CAPACITY,
                "output capacity too small: need " + std::to_string(total) + " overlap rows");
  CUFLYE_API_END(c)
}

cuflye_status cuflye_graph_set(cuflye_ctx* c, size_t ne, const int64_t* edge_ids,
                               const int64_t* seq_ids, const int32_t* left,
                               const int32_t* right) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  require_index(c);
  if (!c->idx.transform)
    throw Error(CUFLYE_ERR_UNSUPPORTED, "read-to-graph needs an index built from edge sequences");
  const uint32_t ns = c->idx.nslots;
  std::vector<int64_t> eos(ns, 0);
  std::vector<int32_t> l(ns, -1), r(ns, -1);
  for (size_t e = 0; e < ne; ++e) {
    if (edge_ids[e] <= 0 || seq_ids[e] <= 0)
      throw Error(CUFLYE_ERR_INVALID, "edge ids and sequence ids must be > 0");
    auto it = c->slot_of.find(seq_ids[e]);
    if (it == c->slot_of.end())
      throw Error(CUFLYE_ERR_INVALID,
                  "edge sequence " + std::to_string(seq_ids[e]) + " is not in the index");
    eos[it->second] = edge_ids[e];
    l[it->second] = left[e];
    r[it->second] = right[e];
  }
  for (uint32_t s = 0; s < ns; ++s)
    if (eos[s] == 0)
      throw Error(CUFLYE_ERR_INVALID, "indexed sequence " + std::to_string(c->slot_signed_h[s]) +
                                          " has no graph edge");
  int64_t* de = buf<int64_t>(c, "gr_edge", ns);
  int32_t* dl = buf<int32_t>(c, "gr_left", ns);
  int32_t* dr = buf<int32_t>(c, "gr_right", ns);
  CUFLYE_CHECK(cudaMemcpy(de, eos.data(), ns * 8ull, cudaMemcpyHostToDevice));
  CUFLYE_CHECK(cudaMemcpy(dl, l.data(), ns * 4ull, cudaMemcpyHostToDevice));
  CUFLYE_CHECK(cudaMemcpy(dr, r.data(), ns * 4ull, cudaMemcpyHostToDevice));
  c->has_graph = true;
  CUFLYE_API_END(c)
}

}  // extern "C"

namespace {

// Device state of one pass's read-to-graph chain stage.
struct R2GPass {
  uint32_t nq = 0;
  uint64_t A = 0;                // chain-input rows
  OverlapRow* rows = nullptr;    // chain input, per read in curBegin order
  R2GRowMeta* meta = nullptr;
  uint64_t* a_off = nullptr;     // nq + 1
  void* recs = nullptr;
  int32_t* cand = nullptr;
  uint32_t* n_cand = nullptr;
  int64_t* read_ids = nullptr;   // nq
};

R2GParams to_r2g_params(const cuflye_r2g_params* r2g) {
  return R2GParams{r2g->max_jump,       r2g->max_read_overlap, r2g->min_overlap,
                   r2g->max_separation, r2g->long_edge,        r2g->big_aln,
                   r2g->max_chain_divergence};
}

void check_r2g(cuflye_ctx* c, const cuflye_r2g_params* r2g) {
  if (!c->has_graph) throw Error(CUFLYE_ERR_INVALID, "no graph: call cuflye_graph_set");
  if (!r2g) throw Error(CUFLYE_ERR_INVALID, "r2g params must not be null");
}

// Buffers of the chain stage for A rows of nq reads.
void r2g_alloc(cuflye_ctx* c, R2GPass& rp2, uint64_t A, uint32_t nq) {
  rp2.nq = nq;
  rp2.A = A;
  rp2.meta = buf<R2GRowMeta>(c, "r_meta", A);
  rp2.recs = buf<uint8_t>(c, "r_recs", A * r2g_rec_bytes());
  rp2.cand = buf<int32_t>(c, "r_cand", A);
  rp2.n_cand = buf<uint32_t>(c, "r_ncand", nq);
  rp2.read_ids = buf<int64_t>(c, "r_ids", nq);
}

// quickSeqOverlaps rows of the pass -> the LONG_EDGE / BIG_ALN filter -> the
// curBegin sort -> candidate chains.
R2GPass r2g_candidates(cuflye_ctx* c, PassState& ps, const ChainParams& cp, const R2GParams& rp,
                       const int64_t* ids) {
  cudaStream_t st = c->stream;
  const uint64_t R = run_chain(c, ps, cp);
  const uint32_t nq = ps.nq;
  const uint32_t ns = c->idx.nslots;
  R2GGraph g{buf<int64_t>(c, "gr_edge", ns), buf<int32_t>(c, "gr_left", ns),
             buf<int32_t>(c, "gr_right", ns), c->idx.slot_signed};
  OverlapRow* rows = buf<OverlapRow>(c, "o_rows", R);
  const uint64_t* row_off = buf<uint64_t>(c, "o_qrowoff", nq + 1);
  uint32_t* keep = buf<uint32_t>(c, "r_keep", R);
  uint64_t* kpos = buf<uint64_t>(c, "r_kpos", R + 1);
  CUFLYE_CHECK(r2g_filter(rows, R, rp, keep, st));
  const uint64_t A = scan_u32(c, keep, kpos, R, "r_scan");
  OverlapRow* aln = buf<OverlapRow>(c, "r_aln", A);
  uint64_t* src = buf<uint64_t>(c, "r_src", A);
  CUFLYE_CHECK(r2g_compact(rows, R, keep, kpos, aln, src, st));
  R2GPass out;
  r2g_alloc(c, out, A, nq);
  // each read's first kept row: the kept-row scan at the read's first row
  out.a_off = buf<uint64_t>(c, "r_aoff", nq + 1);
  CUFLYE_CHECK(gather_query_offsets(row_off, kpos, nq, out.a_off, st));
  uint64_t* skeys = buf<uint64_t>(c, "r_skeys", A);
  uint32_t* svals = buf<uint32_t>(c, "r_svals", A);
  CUFLYE_CHECK(r2g_sort_keys(aln, out.a_off, nq, skeys, svals, st));
  uint32_t* sl = buf<uint32_t>(c, "r_sl", A + 1);
  uint32_t* sr = buf<uint32_t>(c, "r_sr", A + 1);
  uint32_t* slists = buf<uint32_t>(c, "r_slists", 4ull * nq);
  uint32_t* scounts = buf<uint32_t>(c, "r_scounts", 16);
  CUFLYE_CHECK(segmented_std_sort(skeys, svals, sl, sr, out.a_off, out.a_off + 1, nq, nullptr,
                                  slists, scounts, c->num_sms, st, sort_tasks(c, "r", A, nq)));
  out.rows = buf<OverlapRow>(c, "r_sorted", A);
  CUFLYE_CHECK(r2g_permute(aln, out.a_off, nq, svals, src, row_off, g, out.rows, out.meta, st));
  CUFLYE_CHECK(cudaMemcpyAsync(out.read_ids, ids, nq * sizeof(int64_t), cudaMemcpyHostToDevice,
                               st));
  CUFLYE_CHECK(r2g_chain(out.rows, out.a_off, nq, out.meta, rp, out.recs,
                         buf<int32_t>(c, "r_act", A), buf<int32_t>(c, "r_frz", A), out.cand,
                         out.n_cand, st));
  return out;
}

// Exclusive scan of n 32-bit counts on the device; the offsets are also
// returned on the host (n + 1 entries, starting at base).
std::vector<uint64_t> host_offsets(cuflye_ctx* c, const uint32_t* counts, uint32_t n,
                                   uint64_t base = 0) {
  std::vector<uint32_t> h(n);
  if (n) CUFLYE_CHECK(cudaMemcpyAsync(h.data(), counts, n * 4ull, cudaMemcpyDeviceToHost,
                                      c->stream));
  sync(c);
  std::vector<uint64_t> off(n + 1);
  off[0] = base;
  for (uint32_t i = 0; i < n; ++i) off[i + 1] = off[i] + h[i];
  return off;
}

uint64_t* upload(cuflye_ctx* c, const char* name, const std::vector<uint64_t>& v) {
  uint64_t* d = buf<uint64_t>(c, name, v.size());
  CUFLYE_CHECK(cudaMemcpyAsync(d, v.data(), v.size() * 8ull, cudaMemcpyHostToDevice, c->stream));
  return d;
}

// Divergence + accept of the pass's candidate chains, then the kept chains
// and their complements as rows (chain ids from chain_base).  Returns the
// rows; they stay in "r_out".
uint64_t r2g_good_rows(cuflye_ctx* c, R2GPass& r, const R2GParams& rp, const float* div_in,
                       const uint64_t* div_off, float* div_out, uint8_t* acc_out,
                       uint64_t& chain_base) {
  cudaStream_t st = c->stream;
  const uint32_t nq = r.nq;
  int32_t* good = buf<int32_t>(c, "r_good", r.A);
  uint32_t* n_good = buf<uint32_t>(c, "r_ngood", nq);
  uint32_t* n_rows = buf<uint32_t>(c, "r_nrows", nq);
  CUFLYE_CHECK(r2g_divergence(r.rows, r.a_off, nq, r.recs, r.cand, r.n_cand, div_in, div_off, rp,
                              div_out, acc_out, good, n_good, n_rows, nullptr, st));
  uint64_t* row_off = buf<uint64_t>(c, "r_rowoff", nq + 1);
  const uint64_t nrows = scan_u32(c, n_rows, row_off, nq, "r_scan");
  // chain ids: two per good chain (the chain and its complement)
  std::vector<uint64_t> coff = host_offsets(c, n_good, nq, 0);
  for (auto& v : coff) v = chain_base + 2 * v;
  uint64_t* d_coff = upload(c, "r_coff", coff);
  cuflye_read_alignment* d_out = buf<cuflye_read_alignment>(c, "r_out", nrows);
  int32_t* tmp = buf<int32_t>(c, "r_tmp", r.A);
  CUFLYE_CHECK(r2g_emit(r.rows, r.a_off, nq, r.meta, r.read_ids, r.recs, good, n_good, d_coff,
                        row_off, tmp, d_out, st));
  chain_base = coff[nq];
  return nrows;
}

// The pass's candidate chains as chain records (in "r_records"); returns their
// number.  query_ids (device, nq) name the fixtures.
uint64_t r2g_chain_records(cuflye_ctx* c, R2GPass& r, const R2GParams& rp,
                           const int64_t* query_ids) {
  cudaStream_t st = c->stream;
  const uint32_t nq = r.nq;
  uint32_t* n_good = buf<uint32_t>(c, "r_ngood", nq);
  uint32_t* n_rows = buf<uint32_t>(c, "r_nrows", nq);
  uint32_t* n_segs = buf<uint32_t>(c, "r_nsegs", nq);
  CUFLYE_CHECK(r2g_divergence(r.rows, r.a_off, nq, r.recs, r.cand, r.n_cand, nullptr, nullptr, rp,
                              nullptr, nullptr, buf<int32_t>(c, "r_good", r.A), n_good, n_rows,
                              n_segs, st));
  uint64_t* rec_off = buf<uint64_t>(c, "r_recoff", nq + 1);
  const uint64_t nrec = scan_u32(c, n_segs, rec_off, nq, "r_scan");
  cuflye_chain_record* d = buf<cuflye_chain_record>(c, "r_records", nrec);
  CUFLYE_CHECK(r2g_records(r.rows, r.a_off, nq, r.meta, query_ids, r.read_ids, r.recs, r.cand,
                           r.n_cand, rec_off, d, st));
  return nrec;
}

}  // namespace

extern "C" {

cuflye_status cuflye_read_to_graph(cuflye_ctx* c, size_t n, const int64_t* ids,
                                   const int64_t* offsets, const char* bases,
                                   const cuflye_overlap_params* params,
                                   const cuflye_r2g_params* r2g, cuflye_read_alignment* out,
                                   size_t out_cap, size_t* n_out) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  require_index(c);
  check_params(c, params);
  check_r2g(c, r2g);
  if (!ids || !offsets || (!bases && n)) throw Error(CUFLYE_ERR_INVALID, "null input");
  reset_timing(c);
  const ChainParams cp = to_chain_params(params);
  const R2GParams rp = to_r2g_params(r2g);
  Queries Q{n, ids, offsets, bases};
  size_t total = 0;
  uint64_t chain_base = 0;
  bool overflow = false;
  for_each_pass(c, Q, false, kChainBytesPerHit, [&](size_t q0, size_t, PassState& ps) {
    R2GPass r = r2g_candidates(c, ps, cp, rp, ids + q0);
    const uint64_t nrows =
        r2g_good_rows(c, r, rp, nullptr, nullptr, nullptr, nullptr, chain_base);
    if (!overflow && total + nrows <= out_cap) {
      if (nrows)
        CUFLYE_CHECK(cudaMemcpyAsync(out + total, buf<cuflye_read_alignment>(c, "r_out", nrows),
                                     nrows * sizeof(cuflye_read_alignment),
                                     cudaMemcpyDeviceToHost, c->stream));
    } else {
      overflow = true;
    }
    CUFLYE_CHECK(cudaEventRecord(c->ev[4], c->stream));
    total += nrows;
    accumulate_timing(c, true);
  });
  if (n_out) *n_out = total;
  if (overflow)
    throw Error(CUFLYE_ERR_CAPACITY,
                "output capacity too small: need " + std::to_string(total) + " alignment rows");
  CUFLYE_API_END(c)
}

cuflye_status cuflye_read_to_graph_chains(cuflye_ctx* c, size_t n, const int64_t* ids,
                                          const int64_t* offsets, const char* bases,
                                          const cuflye_overlap_params* params,
                                          const cuflye_r2g_params* r2g,
                                          cuflye_chain_record* out, size_t out_cap,
                                          size_t* n_out, uint64_t* inputs_per_read) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  require_index(c);
  check_params(c, params);
  check_r2g(c, r2g);
  if (!ids || !offsets || (!bases && n)) throw Error(CUFLYE_ERR_INVALID, "null input");
  reset_timing(c);
  const ChainParams cp = to_chain_params(params);
  const R2GParams rp = to_r2g_params(r2g);
  Queries Q{n, ids, offsets, bases};
  size_t total = 0;
  bool overflow = false;
  for_each_pass(c, Q, false, kChainBytesPerHit, [&](size_t q0, size_t, PassState& ps) {
    R2GPass r = r2g_candidates(c, ps, cp, rp, ids + q0);
    const uint64_t nrec = r2g_chain_records(c, r, rp, r.read_ids);
    if (!overflow && total + nrec <= out_cap) {
      if (nrec)
        CUFLYE_CHECK(cudaMemcpyAsync(out + total, buf<cuflye_chain_record>(c, "r_records", nrec),
                                     nrec * sizeof(cuflye_chain_record), cudaMemcpyDeviceToHost,
                                     c->stream));
    } else {
      overflow = true;
    }
    if (inputs_per_read) {
      std::vector<uint64_t> a(r.nq + 1);
      CUFLYE_CHECK(cudaMemcpyAsync(a.data(), r.a_off, (r.nq + 1) * 8ull, cudaMemcpyDeviceToHost,
                                   c->stream));
      sync(c);
      for (uint32_t q = 0; q < r.nq; ++q) inputs_per_read[q0 + q] = a[q + 1] - a[q];
    }
    CUFLYE_CHECK(cudaEventRecord(c->ev[4], c->stream));
    total += nrec;
    accumulate_timing(c, true);
  });
  if (n_out) *n_out = total;
  if (overflow)
    throw Error(CUFLYE_ERR_CAPACITY,
                "output capacity too small: need " + std::to_string(total) + " chain records");
  CUFLYE_API_END(c)
}

cuflye_status cuflye_chain_read_alignments(
    cuflye_ctx* c, size_t n_fixtures, const uint64_t* fixture_offsets, const int64_t* query_ids,
    const cuflye_edge_overlap* overlaps, const cuflye_r2g_params* r2g, const float* chain_div_in,
    size_t n_chain_div_in, cuflye_chain_record* out, size_t out_cap, size_t* n_out,
    float* chain_div, uint8_t* chain_kept, size_t chain_cap, size_t* n_chains,
    cuflye_read_alignment* kept_rows, size_t rows_cap, size_t* n_rows) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  if (!r2g) throw Error(CUFLYE_ERR_INVALID, "r2g params must not be null");
  if (n_fixtures && (!fixture_offsets || !query_ids))
    throw Error(CUFLYE_ERR_INVALID, "null input");
  if (n_fixtures >= (1ull << 31)) throw Error(CUFLYE_ERR_UNSUPPORTED, "too many fixtures");
  const uint64_t total_rows = n_fixtures ? fixture_offsets[n_fixtures] : 0;
  if (total_rows && !overlaps) throw Error(CUFLYE_ERR_INVALID, "null overlaps");
  for (size_t f = 0; f < n_fixtures; ++f) {
    if (fixture_offsets[f + 1] < fixture_offsets[f])
      throw Error(CUFLYE_ERR_INVALID, "fixture offsets must not decrease");
    if (fixture_offsets[f + 1] - fixture_offsets[f] >= (1ull << 31))
      throw Error(CUFLYE_ERR_UNSUPPORTED, "fixture longer than 2^31 overlaps");
  }
  if (fixture_offsets && n_fixtures && fixture_offsets[0] != 0)
    throw Error(CUFLYE_ERR_INVALID, "fixture offsets must start at 0");
  reset_timing(c);
  const R2GParams rp = to_r2g_params(r2g);
  cudaStream_t st = c->stream;
  const uint32_t nq = static_cast<uint32_t>(n_fixtures);
  R2GPass r;
  r2g_alloc(c, r, total_rows, nq);
  r.rows = buf<OverlapRow>(c, "r_sorted", total_rows);
  cuflye_edge_overlap* d_in = buf<cuflye_edge_overlap>(c, "r_replay_in", total_rows);
  if (total_rows)
    CUFLYE_CHECK(cudaMemcpyAsync(d_in, overlaps, total_rows * sizeof(cuflye_edge_overlap),
                                 cudaMemcpyHostToDevice, st));
  r.a_off = upload(c, "r_aoff", std::vector<uint64_t>(fixture_offsets, fixture_offsets + nq + 1));
  // a fixture's read id: its first overlap's (the query id when it has none)
  std::vector<int64_t> rids(nq);
  for (uint32_t f = 0; f < nq; ++f)
    rids[f] = fixture_offsets[f + 1] > fixture_offsets[f] ? overlaps[fixture_offsets[f]].read_id
                                                          : query_ids[f];
  if (nq)
    CUFLYE_CHECK(cudaMemcpyAsync(r.read_ids, rids.data(), nq * 8ull, cudaMemcpyHostToDevice, st));
  int64_t* d_qids = buf<int64_t>(c, "r_qids", nq);
  if (nq)
    CUFLYE_CHECK(cudaMemcpyAsync(d_qids, query_ids, nq * 8ull, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(r2g_replay_rows(d_in, total_rows, r.rows, r.meta, st));
  CUFLYE_CHECK(r2g_chain(r.rows, r.a_off, nq, r.meta, rp, r.recs,
                         buf<int32_t>(c, "r_act", total_rows), buf<int32_t>(c, "r_frz", total_rows),
                         r.cand, r.n_cand, st));
  // candidate chains per fixture
  const std::vector<uint64_t> coff = host_offsets(c, r.n_cand, nq);
  const uint64_t nchains = coff[nq];
  if (n_chains) *n_chains = nchains;
  if (chain_div_in && n_chain_div_in != nchains)
    throw Error(CUFLYE_ERR_INVALID, "chain divergences: " + std::to_string(n_chain_div_in) +
                                        " given for " + std::to_string(nchains) +
                                        " candidate chains");
  uint64_t* d_coff = upload(c, "r_divoff", coff);
  float* d_divin = nullptr;
  if (chain_div_in) {
    d_divin = buf<float>(c, "r_divin", nchains);
    if (nchains)
      CUFLYE_CHECK(cudaMemcpyAsync(d_divin, chain_div_in, nchains * 4ull, cudaMemcpyHostToDevice,
                                   st));
  }
  float* d_div = buf<float>(c, "r_div", total_rows);
  uint8_t* d_acc = buf<uint8_t>(c, "r_acc", total_rows);
  uint64_t chain_base = 0;
  const uint64_t nrows = r2g_good_rows(c, r, rp, d_divin, d_coff, d_div, d_acc, chain_base);
  const uint64_t nrec = r2g_chain_records(c, r, rp, d_qids);
  // the per-chain values, compacted from per-fixture slots into chain order
  std::vector<float> hdiv(total_rows);
  std::vector<uint8_t> hacc(total_rows);
  if (total_rows) {
    CUFLYE_CHECK(cudaMemcpyAsync(hdiv.data(), d_div, total_rows * 4ull, cudaMemcpyDeviceToHost,
                                 st));
    CUFLYE_CHECK(cudaMemcpyAsync(hacc.data(), d_acc, total_rows, cudaMemcpyDeviceToHost, st));
  }
  bool short_buf = false;
  if (nrec <= out_cap) {
    if (nrec && out)
      CUFLYE_CHECK(cudaMemcpyAsync(out, buf<cuflye_chain_record>(c, "r_records", nrec),
                                   nrec * sizeof(cuflye_chain_record), cudaMemcpyDeviceToHost,
                                   st));
  } else {
    short_buf = true;
  }
  if (kept_rows && nrows <= rows_cap) {
    if (nrows)
      CUFLYE_CHECK(cudaMemcpyAsync(kept_rows, buf<cuflye_read_alignment>(c, "r_out", nrows),
                                   nrows * sizeof(cuflye_read_alignment), cudaMemcpyDeviceToHost,
                                   st));
  } else if (kept_rows) {
    short_buf = true;
  }
  sync(c);
  if (nchains > chain_cap && (chain_div || chain_kept)) short_buf = true;
  if (!short_buf) {
    for (uint32_t f = 0; f < nq; ++f) {
      for (uint64_t t = 0; t < coff[f + 1] - coff[f]; ++t) {
        const uint64_t from = fixture_offsets[f] + t;
        if (chain_div) chain_div[coff[f] + t] = hdiv[from];
        if (chain_kept) chain_kept[coff[f] + t] = hacc[from];
      }
    }
  }
  if (n_out) *n_out = nrec;
  if (n_rows) *n_rows = nrows;
  if (short_buf)
    throw Error(CUFLYE_ERR_CAPACITY, "output capacity too small: need " + std::to_string(nrec) +
                                         " chain records, " + std::to_string(nchains) +
                                         " chains, " + std::to_string(nrows) + " rows");
  CUFLYE_API_END(c)
}

cuflye_status cuflye_compact_binary(const cuflye_chain_record* records, size_t n_records,
                                    size_t fixtures, const uint64_t* inputs_per_fixture,
                                    unsigned char* out, size_t out_cap, size_t* n_out) {
  if ((!records && n_records) || (!inputs_per_fixture && fixtures) || !n_out)
    return CUFLYE_ERR_INVALID;
  const uint64_t bytes = CUFLYE_COMPACT_HEADER_BYTES +
                         static_cast<uint64_t>(n_records) * CUFLYE_COMPACT_RECORD_BYTES;
  *n_out = static_cast<size_t>(bytes);
  if (!out || out_cap < bytes) return CUFLYE_ERR_CAPACITY;
  uint64_t total = 0, mn = 0, mx = 0;
  for (size_t f = 0; f < fixtures; ++f) {
    const uint64_t v = inputs_per_fixture[f];
    total += v;
    mn = f == 0 ? v : std::min(mn, v);
    mx = std::max(mx, v);
  }
  if (mx > 0xffffffffull) return CUFLYE_ERR_UNSUPPORTED;
  compact_write_header(out, fixtures, n_records, total, static_cast<uint32_t>(mn),
                       static_cast<uint32_t>(mx));
  for (size_t i = 0; i < n_records; ++i)
    compact_write_record(out + CUFLYE_COMPACT_HEADER_BYTES + i * CUFLYE_COMPACT_RECORD_BYTES,
                         records[i]);
  return CUFLYE_OK;
}

cuflye_status cuflye_std_sort_segments(cuflye_ctx* c, uint64_t* keys, uint32_t* values,
                                       const uint64_t* seg_offsets, size_t n_segments) {
  CUFLYE_API_BEGIN(c)
  CUFLYE_CHECK(cudaSetDevice(c->device));
  if (!seg_offsets) throw Error(CUFLYE_ERR_INVALID, "null segment offsets");
  if (n_segments >= (1ull << 32)) throw Error(CUFLYE_ERR_UNSUPPORTED, "too many segments");
  const uint64_t n = seg_offsets[n_segments];
  for (size_t s = 0; s < n_segments; ++s) {
    if (seg_offsets[s + 1] < seg_offsets[s]) throw Error(CUFLYE_ERR_INVALID, "offsets decrease");
    if (seg_offsets[s + 1] - seg_offsets[s] >= (1ull << 32))
      throw Error(CUFLYE_ERR_UNSUPPORTED, "segment longer than 2^32 - 1");
  }
  if (n && (!keys || !values)) throw Error(CUFLYE_ERR_INVALID, "null keys or values");
  if (n_segments == 0 || n == seg_offsets[0]) {
    c->err.clear();
    return CUFLYE_OK;
  }
  cudaStream_t st = c->stream;
  const uint64_t base = seg_offsets[0];
  const uint64_t m = n - base;
  uint64_t* dk = buf<uint64_t>(c, "t_keys", m);
  uint32_t* dv = buf<uint32_t>(c, "t_vals", m);
  uint32_t* dl = buf<uint32_t>(c, "t_l", m + 1);
  uint32_t* dr = buf<uint32_t>(c, "t_r", m + 1);
  uint64_t* off = buf<uint64_t>(c, "t_off", n_segments + 1);
  uint32_t* lists = buf<uint32_t>(c, "t_lists", 4 * n_segments);
  uint32_t* counts = buf<uint32_t>(c, "t_counts", 16);
  std::vector<uint64_t> rel(n_segments + 1);
  for (size_t s = 0; s <= n_segments; ++s) rel[s] = seg_offsets[s] - base;
  CUFLYE_CHECK(cudaMemcpyAsync(dk, keys + base, m * 8, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(dv, values + base, m * 4, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(cudaMemcpyAsync(off, rel.data(), rel.size() * 8, cudaMemcpyHostToDevice, st));
  CUFLYE_CHECK(segmented_std_sort(dk, dv, dl, dr, off, off + 1,
                                  static_cast<uint32_t>(n_segments), nullptr, lists, counts,
                                  c->num_sms, st,
                                  sort_tasks(c, "t", m, static_cast<uint32_t>(n_segments))));
  CUFLYE_CHECK(cudaMemcpyAsync(keys + base, dk, m * 8, cudaMemcpyDeviceToHost, st));
  CUFLYE_CHECK(cudaMemcpyAsync(values + base, dv, m * 4, cudaMemcpyDeviceToHost, st));
  sync(c);
  CUFLYE_API_END(c)
}

cuflye_status cuflye_last_timing(const cuflye_ctx* c, double* stage_ms, uint64_t* stage_bytes,
                                 size_t n_stages) {
  if (!c) return CUFLYE_ERR_INVALID;
  for (size_t i = 0; i < n_stages && i < static_cast<size_t>(kStages); ++i) {
    if (stage_ms) stage_ms[i] = c->stage_ms[i];
    if (stage_bytes) stage_bytes[i] = c->stage_bytes[i];
  }
  return CUFLYE_OK;
}

cuflye_status cuflye_last_sort_stats(const cuflye_ctx* c, uint64_t* counts, size_t n) {
  if (!c || (!counts && n)) return CUFLYE_ERR_INVALID;
  for (size_t i = 0; i < n && i < 8; ++i) counts[i] = c->sort_stats[i];
  return CUFLYE_OK;
}

cuflye_status cuflye_last_passes(const cuflye_ctx* c, uint64_t* passes) {
  if (!c || !passes) return CUFLYE_ERR_INVALID;
  *passes = c->passes;
  return CUFLYE_OK;
}

cuflye_status cuflye_trim(cuflye_ctx* c) {
  CUFLYE_API_BEGIN(c)
  sync(c);
  std::vector<std::string> names;
  for (const auto& kv : c->bufs) {
    const std::string& n = kv.first;
    const bool keep = n.compare(0, 3, "ix_") == 0 || n.compare(0, 3, "gr_") == 0 ||
                      n.compare(0, 5, "logf_") == 0 || n == "status";
    if (!keep) names.push_back(n);
  }
  for (const std::string& n : names) release(c, n);
  CUFLYE_API_END(c)
}

cuflye_status cuflye_last_pass_stats(const cuflye_ctx* c, uint64_t* passes, uint64_t* retries,
                                     double* alloc_ms) {
  if (!c) return CUFLYE_ERR_INVALID;
  if (passes) *passes = c->passes;
  if (retries) *retries = c->pass_retries;
  if (alloc_ms) *alloc_ms = c->alloc_ms;
  return CUFLYE_OK;
}

cuflye_status cuflye_set_index_build_windows(cuflye_ctx* c, uint64_t max_windows) {
  if (!c) return CUFLYE_ERR_INVALID;
  c->build_window_cap = max_windows;
  return CUFLYE_OK;
}

cuflye_status cuflye_last_index_ranges(const cuflye_ctx* c, uint64_t* ranges) {
  if (!c || !ranges) return CUFLYE_ERR_INVALID;
  *ranges = c->build_ranges;
  return CUFLYE_OK;
}

cuflye_status cuflye_kernel_launches(uint64_t* total) {
  if (!total) return CUFLYE_ERR_INVALID;
  *total = launches_total();
  return CUFLYE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- serving
//
// Continuous batching on one device.  A server borrows the owner context's
// resident index and runs `workers` worker contexts, each with its own
// stream and device arena, on one host thread each.  A worker that falls
// idle takes every request that has arrived (up to max_batch_bases of
// query bases) and runs them as one batch through the overlap stage, so
// requests that arrive while a batch is on the GPU are admitted into the
// next free worker's batch and their work overlaps on the device.  Each
// batch is split back into its requests by the per-query row counts; a
// request's rows are exactly what cuflye_overlaps returns for its queries
// alone.

namespace {

struct ServeRequest {
  uint64_t ticket = 0;
  std::vector<int64_t> ids, offsets;
  std::vector<char> bases;
};

struct ServeResult {
  bool done = false;
  cuflye_status status = CUFLYE_OK;
  std::string err;
  std::vector<cuflye_overlap_range> rows;
};

// Overlap rows of Q (every pass) with the rows of each query.
void overlaps_collect(cuflye_ctx* c, const Queries& Q, const ChainParams& cp,
                      std::vector<cuflye_overlap_range>& rows, std::vector<uint64_t>& per_query) {
  rows.clear();
  per_query.assign(Q.n, 0);
  reset_timing(c);
  for_each_pass(c, Q, false, kChainBytesPerHit, [&](size_t q0, size_t, PassState& ps) {
    const uint64_t R = run_chain(c, ps, cp, per_query.data() + q0);
    cuflye_overlap_range* d_out = buf<cuflye_overlap_range>(c, "a_ovl", R);
    const size_t base = rows.size();
    rows.resize(base + R);
    CUFLYE_CHECK(rows_to_abi(buf<OverlapRow>(c, "o_rows", R), R, ps.qinfo, c->idx.slot_signed, d_out,
                             c->stream));
    if (R)
      CUFLYE_CHECK(cudaMemcpyAsync(rows.data() + base, d_out, R * sizeof(cuflye_overlap_range),
                                   cudaMemcpyDeviceToHost, c->stream));
    CUFLYE_CHECK(cudaEventRecord(c->ev[4], c->stream));
    accumulate_timing(c, true);  // synchronises the pass
  });
}

}  // namespace

struct cuflye_server {
  cuflye_ctx* owner = nullptr;
  cuflye_overlap_params params{};
  uint64_t max_batch_bases = 0;
  std::vector<cuflye_ctx*> workers;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ServeRequest> pending;
  std::unordered_map<uint64_t, ServeResult> results;
  std::deque<uint64_t> finished;  // tickets in completion order, for cuflye_poll_any
  uint64_t next_ticket = 1;
  bool stop = false;
  uint64_t batches = 0, batched_requests = 0;
  std::string err;
};

namespace {

void serve_worker(cuflye_server* s, cuflye_ctx* c) {
  cudaSetDevice(c->device);
  const ChainParams cp = to_chain_params(&s->params);
  for (;;) {
    std::vector<ServeRequest> batch;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
      if (s->pending.empty()) return;
      uint64_t taken = 0;
      while (!s->pending.empty()) {
        const uint64_t b = s->pending.front().bases.size();
        if (!batch.empty() && s->max_batch_bases && taken + b > s->max_batch_bases) break;
        taken += b;
        batch.push_back(std::move(s->pending.front()));
        s->pending.pop_front();
      }
    }
    std::vector<int64_t> ids, offs{0};
    std::vector<char> bases;
    for (const ServeRequest& r : batch) {
      ids.insert(ids.end(), r.ids.begin(), r.ids.end());
      for (size_t i = 0; i + 1 < r.offsets.size(); ++i)
        offs.push_back(offs.back() + (r.offsets[i + 1] - r.offsets[i]));
      bases.insert(bases.end(), r.bases.begin(), r.bases.end());
    }
    std::vector<cuflye_overlap_range> rows;
    std::vector<uint64_t> per_query;
    cuflye_status st = CUFLYE_OK;
    std::string msg;
    try {
      std::lock_guard<std::mutex> g(c->mu);
      const Queries Q{ids.size(), ids.data(), offs.data(), bases.data()};
      overlaps_collect(c, Q, cp, rows, per_query);
    } catch (const Error& e) {
      st = e.code;
      msg = e.what();
    } catch (const std::exception& e) {
      st = CUFLYE_ERR_CUDA;
      msg = e.what();
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      size_t q = 0, r = 0;
      for (const ServeRequest& req : batch) {
        ServeResult& res = s->results[req.ticket];
        res.done = true;
        s->finished.push_back(req.ticket);
        res.status = st;
        res.err = msg;
        if (st == CUFLYE_OK) {
          size_t nr = 0;
          for (size_t i = 0; i < req.ids.size(); ++i) nr += per_query[q + i];
          res.rows.assign(rows.begin() + r, rows.begin() + r + nr);
          r += nr;
        }
        q += req.ids.size();
      }
      ++s->batches;
      s->batched_requests += batch.size();
    }
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

cuflye_status cuflye_server_open(cuflye_ctx* owner, int workers,
                                 const cuflye_overlap_params* params, uint64_t max_batch_bases,
                                 cuflye_server** out) {
  if (!out) return CUFLYE_ERR_INVALID;
  *out = nullptr;
  cuflye_server* s = nullptr;
  CUFLYE_API_BEGIN(owner)
  require_index(owner);
  check_params(owner, params);
  if (workers < 1 || workers > 8) throw Error(CUFLYE_ERR_INVALID, "workers must be in [1, 8]");
  CUFLYE_CHECK(cudaSetDevice(owner->device));
  // the workers share what is left of the budget (or of the free memory)
  uint64_t avail = 0;
  if (owner->budget) {
    avail = owner->budget > owner->in_use ? owner->budget - owner->in_use : 0;
  } else {
    size_t free_b = 0, total_b = 0;
    CUFLYE_CHECK(cudaMemGetInfo(&free_b, &total_b));
    const uint64_t margin = 8ull << 30;
    avail = free_b > margin ? free_b - margin : free_b / 2;
  }
  const uint64_t per = avail / static_cast<uint64_t>(workers);
  if (per < (64ull << 20))
    throw Error(CUFLYE_ERR_BUDGET, "memory budget leaves under 64 MiB per serving worker");
  s = new cuflye_server();
  s->owner = owner;
  s->params = *params;
  s->max_batch_bases = max_batch_bases;
  for (int w = 0; w < workers; ++w) {
    cuflye_ctx* c = nullptr;
    const cuflye_status st = cuflye_open(owner->device, per, &c);
    if (st != CUFLYE_OK) {
      for (cuflye_ctx* x : s->workers) cuflye_close(x);
      delete s;
      s = nullptr;
      throw Error(st, "cannot open a serving worker context");
    }
    // borrow the owner's resident index (device buffers stay the owner's)
    c->idx = owner->idx;
    c->slot_of = owner->slot_of;
    c->slot_signed_h = owner->slot_signed_h;
    c->has_index = true;
    s->workers.push_back(c);
  }
  for (cuflye_ctx* c : s->workers) s->threads.emplace_back(serve_worker, s, c);
  ++owner->servers;
  *out = s;
  CUFLYE_API_END(owner)
}

cuflye_status cuflye_submit(cuflye_server* s, size_t n, const int64_t* ids, const int64_t* offsets,
                            const char* bases, uint64_t* ticket) {
  if (!s || !ticket || (n && (!ids || !offsets || !bases))) return CUFLYE_ERR_INVALID;
  ServeRequest r;
  r.ids.assign(ids, ids + n);
  r.offsets.assign(offsets, offsets + n + 1);
  for (size_t i = 0; i < n; ++i)
    if (ids[i] == 0 || offsets[i + 1] < offsets[i]) {
      std::lock_guard<std::mutex> lk(s->mu);
      s->err = "query ids must not be zero and offsets must not decrease";
      return CUFLYE_ERR_INVALID;
    }
  const int64_t b0 = n ? offsets[0] : 0, b1 = n ? offsets[n] : 0;
  r.bases.assign(bases + b0, bases + b1);
  for (int64_t& o : r.offsets) o -= b0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r.ticket = s->next_ticket++;
    *ticket = r.ticket;
    s->results[r.ticket];
    s->pending.push_back(std::move(r));
  }
  s->cv_work.notify_one();
  return CUFLYE_OK;
}

cuflye_status cuflye_poll(cuflye_server* s, uint64_t ticket, int wait_ms, cuflye_overlap_range* out,
                          size_t out_cap, size_t* n_out) {
  if (!s) return CUFLYE_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->results.find(ticket);
  if (it == s->results.end()) {
    s->err = "unknown ticket " + std::to_string(ticket);
    return CUFLYE_ERR_INVALID;
  }
  if (!it->second.done && wait_ms != 0) {
    auto ready = [&] {
      auto f = s->results.find(ticket);
      return f == s->results.end() || f->second.done;
    };
    if (wait_ms < 0)
      s->cv_done.wait(lk, ready);
    else
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready);
    it = s->results.find(ticket);
    if (it == s->results.end()) {
      s->err = "ticket " + std::to_string(ticket) + " was consumed by another poll";
      return CUFLYE_ERR_INVALID;
    }
  }
  ServeResult& res = it->second;
  if (!res.done) return CUFLYE_PENDING;
  if (res.status != CUFLYE_OK) {
    const cuflye_status st = res.status;
    s->err = res.err;
    s->results.erase(it);
    return st;
  }
  if (n_out) *n_out = res.rows.size();
  if (res.rows.size() > out_cap) {
    s->err = "output capacity too small: need " + std::to_string(res.rows.size()) +
             " overlap rows";
    return CUFLYE_ERR_CAPACITY;
  }
  if (!res.rows.empty()) std::memcpy(out, res.rows.data(), res.rows.size() * sizeof(res.rows[0]));
  s->results.erase(it);
  return CUFLYE_OK;
}

cuflye_status cuflye_poll_any(cuflye_server* s, int wait_ms, uint64_t* ticket,
                              cuflye_overlap_range* out, size_t out_cap, size_t* n_out) {
  if (!s || !ticket) return CUFLYE_ERR_INVALID;
  *ticket = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  // drop tickets that cuflye_poll consumed already
  auto settle = [&] {
    while (!s->finished.empty() && !s->results.count(s->finished.front())) s->finished.pop_front();
    return !s->finished.empty();
  };
  if (!settle() && wait_ms != 0) {
    if (wait_ms < 0)
      s->cv_done.wait(lk, settle);
    else
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), settle);
  }
  if (!settle()) return CUFLYE_PENDING;
  const uint64_t tk = s->finished.front();
  s->finished.pop_front();
  *ticket = tk;
  auto it = s->results.find(tk);
  ServeResult& res = it->second;
  if (res.status != CUFLYE_OK) {
    const cuflye_status st = res.status;
    s->err = res.err;
    s->results.erase(it);
    return st;
  }
  if (n_out) *n_out = res.rows.size();
  if (res.rows.size() > out_cap) {
    s->err = "output capacity too small: need " + std::to_string(res.rows.size()) +
             " overlap rows (ticket " + std::to_string(tk) + ", kept for cuflye_poll)";
    return CUFLYE_ERR_CAPACITY;
  }
  if (!res.rows.empty()) std::memcpy(out, res.rows.data(), res.rows.size() * sizeof(res.rows[0]));
  s->results.erase(it);
  return CUFLYE_OK;
}

cuflye_status cuflye_server_stats(cuflye_server* s, uint64_t* batches, uint64_t* requests,
                                  uint64_t* pending) {
  if (!s) return CUFLYE_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (batches) *batches = s->batches;
  if (requests) *requests = s->batched_requests;
  if (pending) *pending = s->pending.size();
  return CUFLYE_OK;
}

const char* cuflye_server_last_error(cuflye_server* s) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lk(s->mu);
  return s->err.c_str();
}

void cuflye_server_close(cuflye_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (std::thread& t : s->threads) t.join();
  for (cuflye_ctx* c : s->workers) cuflye_close(c);
  {
    std::lock_guard<std::mutex> g(s->owner->mu);
    --s->owner->servers;
  }
  delete s;
}

}  // extern "C"
