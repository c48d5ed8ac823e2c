// kernels.h — host-side launchers of the device stages (one stream each).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace cuflye {

// Every kernel launch of the library is counted (cuflye_kernel_launches).
void count_launch();
unsigned long long launches_total();

// ---------------------------------------------------------------- scan
// Exclusive prefix sums (out may alias in).  temp needs scan_temp_words(n) words.
size_t scan_temp_words(uint64_t n);
cudaError_t exclusive_scan_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n,
                                      uint64_t* temp, cudaStream_t s);
cudaError_t exclusive_scan_u64(const uint64_t* in, uint64_t* out, uint64_t n, uint64_t* temp,
                               cudaStream_t s);

// ---------------------------------------------------------------- sort
size_t segsort_smem_bytes();
// Task list handed from the global phase of large segments to the
// shared-memory phase: segsort_task_words(n, nseg) entries each.
// Longest heap range one block sorts in its own shared memory; longer ones
// take a block pair.
constexpr uint32_t kHeapPackCap = 57344;
// Rounds of the global phase (partitions of ranges beyond shared memory).
constexpr int kSortRounds = 64;
constexpr size_t kRoundItemBytes = 40;  // one range of a global-phase round
struct SortTasks {
  uint64_t* f;
  uint32_t* n;
  int* d;
  uint32_t cap;           // entries of f, n and d (segsort_task_words)
  uint32_t pair_reserve;  // top entries kept for heap ranges beyond kHeapPackCap
  uint64_t nelems;        // elements of the call at most (no global phase up to 4,096)
  void* round[2];         // two round lists of segsort_round_bytes(nelems) each
  uint32_t* round_counts;  // 2 * (kSortRounds + 1) words
  int round_per_sm = 0;    // blocks per SM of the global phase (1-2; 0: 2)
  // Pruning (optional): segment s's keys that may repeat, sorted, are
  // prune_keys[prune_off[s] .. prune_off[s + 1]).  A global-phase range whose
  // key interval holds none of them has distinct keys, so any sort gives its
  // final order: it is dropped (left as it is) and not listed as a task.
  const uint64_t* prune_keys = nullptr;
  const uint32_t* prune_off = nullptr;
  // Side streams (optional): the whole-segment sorts (tiny, warp and CTA
  // segments) run on `side` beside the global phase, and the heap ranges on
  // `side2` beside the final tasks once the global phase is done.  They all
  // sort disjoint element ranges, and each ends with the serial chain of its
  // slowest range, so their tails overlap instead of adding up.  fork and
  // rounds_done order the side streams after the call's stream; the call
  // returns with its stream waiting for both (join, join2).  Null:
  // everything on the call's stream.
  cudaStream_t side = nullptr, side2 = nullptr;
  cudaEvent_t fork = nullptr, rounds_done = nullptr, join = nullptr, join2 = nullptr;
};
uint32_t segsort_pair_reserve(uint64_t nelems);
size_t segsort_round_bytes(uint64_t nelems);
size_t segsort_task_words(uint64_t nelems, uint32_t nseg);
// lists: 4 * nseg words; counts: 16 words.  l/r scratch: one word per element.
// nseg_dev (optional) holds the live segment count on the device (<= nseg).
cudaError_t segmented_std_sort(uint64_t* keys, uint32_t* vals, uint32_t* lscratch,
                               uint32_t* rscratch, const uint64_t* begin, const uint64_t* end,
                               uint32_t nseg, const uint32_t* nseg_dev, uint32_t* lists,
                               uint32_t* counts, int num_sms, cudaStream_t stream,
                               SortTasks tasks);
// Copies the ranges of (keys, vals) starting at begin[s] to (ck, cv) at
// cbeg[s], where cbeg ascends and the ranges fill [0, total) end to end
// (the flagged queries' generation order, gathered for a pruned sort).
cudaError_t gather_ranges(const uint64_t* keys, const uint32_t* vals, const uint64_t* begin,
                          const uint64_t* cbeg, uint32_t nseg, uint64_t total, uint64_t* ck,
                          uint32_t* cv, int num_sms, cudaStream_t s);
// After a pruned segmented_std_sort of (ck, cv) over the segments
// [cbeg[s], cend[s]) with `counts` and `tasks`: copies every range it sorted
// (segments of up to 4,096 elements whole, its tasks and its heap ranges) to
// (keys, vals) at begin[s] + (offset within the segment); cbeg ascending.
cudaError_t copy_sorted_ranges(const uint64_t* ck, const uint32_t* cv, const uint64_t* cbeg,
                               const uint64_t* cend, const uint64_t* begin, uint32_t nseg,
                               const uint32_t* counts, const SortTasks& tasks, uint64_t* keys,
                               uint32_t* vals, int num_sms, cudaStream_t s);
size_t radix_hist_words(uint64_t n);
cudaError_t radix_sort_pairs(uint64_t* keys, uint64_t* vals, uint64_t* keys_alt,
                             uint64_t* vals_alt, uint64_t n, const int* digits, int ndigits,
                             uint32_t* hist, int* result_in_alt, cudaStream_t stream);

// ---------------------------------------------------------------- sequences
// ASCII bases -> MSB-first 2-bit words (32 bases per word, one padding word).
cudaError_t pack_bases(const uint8_t* ascii, uint64_t nbases, uint64_t* words, cudaStream_t s);

// ---------------------------------------------------------------- index
struct DeviceIndex {
  int k = 0;
  bool transform = true;
  TableEntry* table = nullptr;
  uint64_t cap = 0;              // table slots (load <= 1/2)
  uint64_t* pos = nullptr;       // (dense id << 32) | stored position, bucket order
  uint64_t npos = 0;
  int32_t* slot_len = nullptr;   // target length per dense slot
  int64_t* slot_signed = nullptr;  // signed id per dense slot
  uint32_t nslots = 0;
  uint64_t nkeys = 0, nrep = 0;
  // optional (one-range builds): per window of the indexed targets (slot
  // order, win_off per slot), the index of its own entry in its k-mer's
  // bucket when that k-mer is solid (other windows: any value)
  uint32_t* self_at = nullptr;
  uint64_t* win_off = nullptr;
};

// Window enumeration over packed targets: keys = standard forms, vals =
// (stored dense id << 32) | stored position.
cudaError_t index_enumerate(const uint64_t* words, const uint64_t* base_off,
                            const uint64_t* win_off, const int32_t* slot_len, uint32_t nslots,
                            uint64_t nwin, int k, uint64_t* keys, uint64_t* vals,
                            cudaStream_t s);
// Run detection over sorted keys: flags[i] = key starts a run.
cudaError_t index_mark_runs(const uint64_t* keys, uint64_t n, uint32_t* flags, cudaStream_t s);
// Given run ids (exclusive scan of flags), write run starts (nruns + 1 entries).
cudaError_t index_run_starts(const uint32_t* flags, const uint64_t* run_id, uint64_t n,
                             uint64_t nruns, uint64_t* run_start, cudaStream_t s);
// Windows per key prefix: hist[key >> shift] over nbins (<= 16384) bins.
cudaError_t index_prefix_hist(const uint64_t* words, const uint64_t* base_off,
                              const uint64_t* win_off, const int32_t* slot_len, uint32_t nslots,
                              uint64_t nwin, int k, int shift, int nbins,
                              unsigned long long* hist, int num_sms, cudaStream_t s);
// The windows whose key lies in [lo, hi), appended in no particular order;
// *count receives how many (at most cap are written).
cudaError_t index_enumerate_range(const uint64_t* words, const uint64_t* base_off,
                                  const uint64_t* win_off, const int32_t* slot_len,
                                  uint32_t nslots, uint64_t nwin, int k, uint64_t lo,
                                  uint64_t hi, uint64_t* keys, uint64_t* vals,
                                  unsigned long long* count, uint64_t cap, cudaStream_t s);
// Per run: kept count (solid ? freq : 0) and class (0 none, 1 solid, 2
// repetitive); tally (optional, 2 words) counts solid and repetitive runs.
cudaError_t index_classify_runs(const uint64_t* run_start, uint64_t nruns, uint32_t min_freq,
                                uint32_t max_freq, uint32_t* kept, uint8_t* cls,
                                unsigned long long* tally, cudaStream_t s);
cudaError_t index_copy_positions(const uint64_t* vals, const uint64_t* run_id,
                                 const uint64_t* run_start, const uint8_t* cls,
                                 const uint64_t* kept_off, uint64_t n, uint64_t* pos,
                                 cudaStream_t s, uint32_t* self_at = nullptr,
                                 const uint64_t* win_off = nullptr,
                                 const int32_t* slot_len = nullptr, int k = 0);
// Table insert of every solid and repetitive run, a solid run's positions
// at pos_base + kept_off of the position array.  Solid buckets that list
// one stored id twice get kDupIdsBit (sorted_ids: runs are in (id, position)
// order; otherwise every run of two or more entries is marked).
cudaError_t index_insert(const uint64_t* keys, const uint64_t* vals, const uint64_t* run_start,
                         const uint8_t* cls, const uint64_t* kept_off, uint64_t nruns,
                         uint64_t pos_base, bool sorted_ids, TableEntry* table, uint64_t cap,
                         DeviceStatus* st, cudaStream_t s);
// Per key prefix (key >> shift) of sorted runs: solid positions into
// npos_bin, solid and repetitive runs into nent_bin (both accumulate).
cudaError_t index_bin_totals(const uint64_t* keys, const uint64_t* run_start, const uint8_t* cls,
                             uint64_t nruns, int shift, unsigned long long* npos_bin,
                             unsigned long long* nent_bin, cudaStream_t s);
cudaError_t index_insert_repetitive(const uint64_t* rep_keys, uint64_t n, TableEntry* table,
                                    uint64_t cap, DeviceStatus* st, cudaStream_t s);

// ---------------------------------------------------------------- hits
struct QueryBatch {
  const uint64_t* words = nullptr;    // packed bases
  const uint64_t* base_off = nullptr; // nq + 1
  const uint64_t* win_off = nullptr;  // nq + 1
  const int32_t* qdi = nullptr;       // dense internal id of the query in the index, or -1
  uint32_t nq = 0;
  uint64_t nwin = 0;
};

// q_tie[i] (zeroed by the caller) becomes nonzero when query i looks up a
// bucket with kDupIdsBit, i.e. when its KmerMatch keys may repeat.  wself
// (optional) receives, for windows flagged kWinTrivial, the bucket index of
// the query's own position (built indexes only: one such entry at most).
cudaError_t hits_count(const DeviceIndex& idx, const QueryBatch& q, uint32_t* cnt,
                       uint32_t* filt, uint64_t* wmeta, uint8_t* wflags, uint32_t* q_tie,
                       uint32_t* wself, cudaStream_t s);
// keys[j] = (ext dense id << 32) | cur pos, vals[j] = ext pos, kmers
// (optional), in generation order; filtered positions into fpos.
cudaError_t hits_emit(const DeviceIndex& idx, const QueryBatch& q, const uint64_t* hit_off,
                      const uint64_t* filt_off, const uint64_t* wmeta, const uint8_t* wflags,
                      uint64_t* keys, uint32_t* vals, uint64_t* kmers, int32_t* fpos,
                      cudaStream_t s);
// Gather per-query segment bounds from window-level offsets.
cudaError_t gather_query_offsets(const uint64_t* win_off, const uint64_t* wl_off, uint32_t nq,
                                 uint64_t* q_off, cudaStream_t s);

// ---------------------------------------------------------------- chaining
struct ChainParams {
  int32_t k, min_overlap, max_jump, max_gap, gap_jump_threshold, max_overhang;
  int32_t check_overhang, force_local, only_max_ext, max_overlaps;
  float large_gap_penalty, small_gap_penalty, min_kmer_survival_rate, max_divergence,
      sample_rate;
};

struct GroupInfo {
  uint64_t start;
  uint32_t n;
  uint32_t query;  // batch-local query index
  uint32_t ext_di;
  int32_t ext_len;
  int32_t survive;
  int32_t ext_sorted;  // 0: cur-pos order; 1: re-sorted by ext pos; 2: ext order already
};

// Device-side overlap row before the final ABI conversion.
struct OverlapRow {
  uint32_t query;
  uint32_t ext_di;
  int32_t cur_begin, cur_end, cur_len;
  int32_t ext_begin, ext_end, ext_len;
  int32_t score;
  int32_t chain_len;
  float div;
  uint32_t group;
  uint32_t rank;
};

struct QueryInfo {
  int64_t signed_id;
  int32_t len;
  int32_t pad;
};

// ---------------------------------------------------------------- exact fast sorts
// Sort points whose segments hold no equal keys need no libstdc++-order
// emulation (fastsort.cu); segments that may hold equal keys are listed in
// (emu_begin, emu_end, *emu_count) for segmented_std_sort.
constexpr uint32_t kMatchTile = 4096;  // hits per radix tile (never across queries)
constexpr uint32_t kGroupCap = 16384;      // largest group re-sorted in shared memory
constexpr uint32_t kBacktrackCap = 8192;  // largest group backtracked over shared-memory maps

struct MatchTile {
  uint64_t begin;
  uint32_t n;
  uint32_t query;
};

// Per query with two or more hits: flagged queries (q_tie, keys may repeat)
// are listed for the emulated sort; the others get ntiles[q] radix tiles.
// tile_flagged: the flagged queries get the tiles (their sorted order up to
// the order among equal keys) and nothing is listed.
cudaError_t match_plan(const uint64_t* q_off, const uint32_t* q_tie, uint32_t nq, uint32_t* ntiles,
                       uint64_t* emu_begin, uint64_t* emu_end, uint32_t* emu_count,
                       cudaStream_t s, bool tile_flagged = false);
// tile_off: exclusive scan of ntiles.
cudaError_t match_tiles(const uint64_t* q_off, const uint32_t* ntiles, const uint64_t* tile_off,
                        uint32_t nq, MatchTile* tiles, cudaStream_t s);
// Stable radix sort by the ext id (key bits 32 .. 32 + id_bits) of every
// tiled query, in place in (keys, vals); (alt_keys, alt_vals) is a second
// buffer of the same shape and counts holds 256 words per tile.
cudaError_t match_radix(uint64_t* keys, uint32_t* vals, uint64_t* alt_keys, uint32_t* alt_vals,
                        const MatchTile* tiles, uint32_t ntile,
                        const uint64_t* q_off, const uint32_t* ntiles, const uint64_t* tile_off,
                        uint32_t nq, int id_bits, uint32_t* counts, int num_sms,
                        int scatter_per_sm, cudaStream_t s);
// stats[i_emul] += *emul; stats[i_plain] += total - *emul (total from
// total_dev when given, else total_host; i_plain < 0 skips it).
cudaError_t sort_stats_add(uint64_t* stats, int i_plain, int i_emul, const uint32_t* total_dev,
                           uint32_t total_host, const uint32_t* emul, cudaStream_t s);
// Ext-pos re-sort of the groups list[0 .. *list_count) (out: key = ext pos,
// val = cur pos); groups with equal ext positions or over kGroupCap elements
// are listed for segmented_std_sort instead.
// scratch_a and scratch_b hold nhits words each, scratch_c 2 * nhits (groups
// beyond shared memory sort there).
cudaError_t group_ext_sort(uint64_t* keys, uint32_t* vals, const GroupInfo* groups,
                           const uint32_t* list, const uint32_t* list_count, uint32_t max_groups,
                           uint64_t* emu_begin, uint64_t* emu_end, uint32_t* emu_count,
                           uint32_t* scratch_a, uint32_t* scratch_b, uint32_t* scratch_c,
                           uint64_t nhits, uint32_t* work, int num_sms, cudaStream_t s);

// Groups (runs of one ext id within a query's sorted hits) in two passes
// over tiles of kGroupTile hits: counts per tile, then (after an exclusive
// scan of the counts into tile_off) each group's start, query and ext id.
constexpr uint32_t kGroupTile = 4096;
cudaError_t groups_count(const uint64_t* keys, const uint64_t* q_off, uint32_t nq, uint64_t nhits,
                         uint32_t* tile_counts, cudaStream_t s);
cudaError_t groups_write(const uint64_t* keys, const uint64_t* q_off, uint32_t nq, uint64_t nhits,
                         const uint64_t* tile_off, GroupInfo* groups, cudaStream_t s);
cudaError_t groups_prefilter_n(const uint64_t* keys, const uint32_t* vals, GroupInfo* groups,
                               uint64_t ngroups, uint64_t nhits, const QueryInfo* qinfo,
                               const int32_t* slot_len, const ChainParams& p,
                               uint32_t* ext_list, uint32_t* dp_list, uint32_t* counts,
                               cudaStream_t s);
// Rewrite ext-sorted groups as (key = ext, val = cur) for their re-sort.
cudaError_t groups_prepare_ext_sort(uint64_t* keys, uint32_t* vals, const GroupInfo* groups,
                                    const uint32_t* ext_list, const uint32_t* counts,
                                    uint64_t* seg_begin, uint64_t* seg_end, cudaStream_t s);
// Ext-sorted groups already in strict ext-pos order get ext_sorted = 2 (read
// in place); the others are appended to out / *out_count (zeroed here).
cudaError_t groups_ext_presorted(const uint32_t* vals, GroupInfo* groups, const uint32_t* ext_list,
                                 const uint32_t* counts, uint32_t* out, uint32_t* out_count,
                                 cudaStream_t s);
// The group prefilter of tools/replay_overlap_chains.py:245-270: survival
// (unique query positions against min_kmer_survival_rate * min_overlap), the
// cur and ext spans against min_overlap, and the overhangs when
// check_overhang && !force_local.  mn / mx: the group's least and greatest
// ext pos; min_cur / max_cur its first and last cur pos.
__device__ __forceinline__ bool prefilter_keeps(uint32_t uniq, int32_t min_cur, int32_t max_cur,
                                                int32_t mn, int32_t mx, int32_t cur_len,
                                                int32_t ext_len, const ChainParams& p) {
  bool ok = !(static_cast<float>(uniq) <
              __fmul_rn(p.min_kmer_survival_rate, static_cast<float>(p.min_overlap)));
  if (ok && (max_cur - min_cur < p.min_overlap || mx - mn < p.min_overlap)) ok = false;
  if (ok && p.check_overhang && !p.force_local) {
    if (min(min_cur, mn) > p.max_overhang) ok = false;
    if (min(cur_len - max_cur, ext_len - mx) > p.max_overhang) ok = false;
  }
  return ok;
}

// ---------------------------------------------------------------- sorted emission
// Hits written straight into KmerMatch order (match_emit.cu).  A query whose
// distinct ext ids exceed kMatchDictCap makes the pass take the emit + sort
// path instead.
constexpr uint32_t kMatchDictCap = 2048;

struct MatchEmitArgs {
  DeviceIndex idx;
  const uint64_t* win_off = nullptr;   // nq + 1: each query's first window in the pass
  const uint64_t* q_off = nullptr;     // nq + 1: each query's first hit in the pass
  const uint64_t* hit_off = nullptr;   // per window: its first hit (generation order)
  const uint64_t* wmeta = nullptr;     // per window: table meta of its k-mer
  const uint8_t* wflags = nullptr;     // per window: kWin* flags
  const uint32_t* wself = nullptr;     // per kWinTrivial window: bucket index of the self hit
  const uint64_t* filt_off = nullptr;  // per window: its filtered-position slot
  int32_t* fpos = nullptr;             // filtered positions (written by match_emit)
  DeviceStatus* status = nullptr;
  uint32_t nq = 0;
};

struct MatchEmitLists {
  uint32_t* dp_list;    // surviving groups decided by match_emit
  uint32_t* ext_list;   // those of them that are ext-sorted
  uint32_t* pf_list;    // groups left to the prefilter kernel (flagged queries')
  uint32_t* counts;     // [0] ext_list, [1] dp_list, [2] pf_list entries (zeroed by the caller)
  uint64_t* emu_begin;  // flagged queries' hit ranges for the libstdc++-order sort
  uint64_t* emu_end;
  uint32_t* emu_count;  // zeroed by the caller
  unsigned long long* tally;  // [0]: flagged queries' hits, [1]: hits of pf_list groups
  // flagged queries' keys that may repeat (optional): (the query's first hit,
  // key) of every hit whose window's bucket lists its target just before it;
  // tie_count (zeroed by the caller) counts them all, tie_cap are stored
  uint64_t* tie_h0 = nullptr;
  uint64_t* tie_key = nullptr;
  uint32_t* tie_count = nullptr;
  uint32_t tie_cap = 0;
};

size_t match_dict_smem_bytes();
size_t match_emit_smem_bytes();
// Per query: its distinct ext ids (sorted) with their hit counts, as words
// (ext id << 32) | count at dict[q_dbase[q] ..] (dict needs one word per hit
// at most; *dict_cursor zeroed by the caller), and their number q_ng[q].  A
// query with more than kMatchDictCap ext ids gets q_ng = 0 and counts in
// *overflow (zeroed by the caller).  counter: one word of scratch.
cudaError_t match_dict(const MatchEmitArgs& a, uint64_t* dict, unsigned long long* dict_cursor,
                       uint32_t* q_ng, uint64_t* q_dbase, uint32_t* overflow, uint32_t* counter,
                       int num_sms, cudaStream_t s);
// The hits of every query in KmerMatch order (flagged queries: generation
// order, listed in emu_*), the filtered positions, one GroupInfo per
// (query, ext id) at q_goff[q] + rank, and the prefilter of every group of
// an unflagged query (a flagged query's groups go to pf_list).
cudaError_t match_emit(const MatchEmitArgs& a, const uint64_t* dict, const uint32_t* q_ng,
                       const uint64_t* q_dbase, const uint64_t* q_goff, const uint32_t* q_tie,
                       const QueryInfo* qinfo, const ChainParams& p, uint64_t* keys,
                       uint32_t* vals, GroupInfo* groups, const MatchEmitLists& lists,
                       uint32_t* counter, int num_sms, cudaStream_t s);
// The prefilter of the groups list[0 .. counts[2]) (GroupInfo.n already set):
// survivors go to dp_list (counts[1]) and, when ext-sorted, to ext_list
// (counts[0]).  Does not clear the counts.
cudaError_t groups_prefilter_list(const uint64_t* keys, const uint32_t* vals, GroupInfo* groups,
                                  const uint32_t* list, const QueryInfo* qinfo,
                                  const int32_t* slot_len, const ChainParams& p,
                                  uint32_t* ext_list, uint32_t* dp_list, uint32_t* counts,
                                  uint32_t max_groups, cudaStream_t s);

// Highest score of a group, its first element and how many elements have it.
struct GroupTop {
  int32_t score;
  uint32_t first;
  uint32_t count;
  uint32_t pad;
};

// keys / vals: the sorted matches (key = (ext id << 32) | cur pos, val = ext
// pos; groups with ext_sorted == 1 hold key = ext pos, val = cur pos).
// work: one word of device scratch (the group counter of the launch); top
// (indexed by group) receives each group's GroupTop; pmc: chain_dp_pmc_words
// words of scratch (running score maxima per 32 elements).
// The list reordered by length bucket, longest first (order within a bucket
// unspecified).  scratch: 10 words.
cudaError_t groups_length_order(const GroupInfo* groups, const uint32_t* list,
                                const uint32_t* list_count, uint32_t max_groups,
                                uint32_t* scratch, uint32_t* out, cudaStream_t s);
cudaError_t chain_dp(const uint64_t* keys, const uint32_t* vals, int32_t* score, int32_t* bt,
                     const GroupInfo* groups, const uint32_t* dp_list, const uint32_t* counts,
                     const ChainParams& p, GroupTop* top, int32_t* pmc, uint32_t* work,
                     int num_sms, int per_sm, cudaStream_t s);
inline uint64_t chain_dp_pmc_words(uint64_t nhits, uint64_t ngroups) {
  return (nhits >> 5) + ngroups + 2;
}
// Score-order sort inputs of the groups list[0 .. *list_count): key =
// INT32_MAX - score, val = local index, and their segment bounds.
cudaError_t chain_prepare_order(const int32_t* score, uint64_t* keys, uint32_t* vals,
                                const GroupInfo* groups, const uint32_t* list,
                                const uint32_t* list_count, uint64_t* seg_begin,
                                uint64_t* seg_end, cudaStream_t s);
// Backtrack of the groups list[0 .. *list_count).  With `top` (the DP's
// GroupTop per group) every group picks its starts in score order itself,
// and a group whose result could depend on the order among equal scores is
// not finished but appended to redo_list, to be run again with Flye's order;
// with top null every group follows the score order in `order` (local
// indices, libstdc++ order).  gmaps: 3 * gmap_words words of device scratch
// (the walk bitmaps of groups over 16,384 elements), gmap_words =
// chain_dp_pmc_words(nhits, ngroups).
cudaError_t chain_backtrack(const uint64_t* keys, const uint32_t* vals, const int32_t* score,
                            int32_t* bt, const uint32_t* order, const GroupInfo* groups,
                            const uint32_t* list, const uint32_t* list_count,
                            const GroupTop* top, uint32_t* redo_list, uint32_t* redo_count,
                            const QueryInfo* qinfo, const uint64_t* f_off, const int32_t* fpos,
                            const int64_t* slot_signed, const LogfTable& logt,
                            const ChainParams& p, OverlapRow* pool, uint64_t pool_cap,
                            uint32_t* pool_count, uint32_t* group_rows, DeviceStatus* st,
                            uint32_t max_groups, uint32_t* gmaps, uint64_t gmap_words,
                            uint32_t* work, int per_sm, cudaStream_t s);
// max_overlaps cutoff and group-order compaction of the pooled rows.
cudaError_t rows_limit(const uint32_t* group_rows, const uint64_t* q_group_off, uint32_t nq,
                       int32_t max_overlaps, uint32_t* kept_rows, cudaStream_t s);
cudaError_t rows_scatter(const OverlapRow* pool, uint32_t npool, const uint32_t* kept_rows,
                         const uint64_t* kept_off, OverlapRow* rows, cudaStream_t s);
cudaError_t query_group_offsets(const GroupInfo* groups, uint64_t ngroups, uint32_t nq,
                                uint64_t* q_group_off, cudaStream_t s);
// Rows of each query after compaction: out[q] = kept_off[qg[q + 1]] - kept_off[qg[q]].
cudaError_t query_row_counts(const uint64_t* q_group_off, const uint64_t* kept_off, uint32_t nq,
                             uint64_t* out, cudaStream_t s);

}  // namespace cuflye
