/*
 * cuflye.h — C ABI of the GB300 overlap hot-path library (libcuflye_gb300.so).
 *
 * Plain pointers and sizes only.  Every entry point returns a cuflye_status;
 * on failure cuflye_last_error(ctx) holds a one-line message.  No call falls
 * back to a CPU path: an unsupported case fails with CUFLYE_ERR_UNSUPPORTED,
 * as the reference's CUDA stub does
 * (patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-46).
 *
 * Sequences are passed the way Flye's FastaRecord carries them: a signed id
 * (FastaRecord::Id::signedId(), +n forward / -n reverse complement) and ASCII
 * bases (A/C/G/T, any case; any other byte encodes as A, as
 * cuda/cuflye_cuda_read_window_smoke.cu:172-193 does).  Batches are
 * concatenated bases plus n+1 offsets.
 *
 * Output buffers are caller-owned host memory with a capacity.  When a
 * capacity is too small the call returns CUFLYE_ERR_CAPACITY and writes the
 * required counts; repeat the call with larger buffers.  Device memory is
 * owned by the context and is reused across calls (arena).
 *
 * Threading: a context serialises its own calls with an internal mutex.  Use
 * one context per host thread for concurrency; contexts may share a device.
 */
#ifndef CUFLYE_H
#define CUFLYE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cuflye_status {
  CUFLYE_OK = 0,
  CUFLYE_ERR_INVALID = 1,     /* bad argument or malformed input            */
  CUFLYE_ERR_UNSUPPORTED = 2, /* shape this backend does not handle: fail fast */
  CUFLYE_ERR_BUDGET = 3,      /* device memory budget exceeded (never truncates) */
  CUFLYE_ERR_CUDA = 4,        /* CUDA runtime error                          */
  CUFLYE_ERR_CAPACITY = 5,    /* caller buffer too small; counts written     */
  CUFLYE_ERR_TIMEOUT = 6,     /* a bounded device wait expired               */
  CUFLYE_ERR_NO_INDEX = 7,    /* call needs an index; none built             */
  CUFLYE_PENDING = 8          /* serving: the request is not finished yet    */
} cuflye_status;

typedef struct cuflye_ctx cuflye_ctx;

/* --------------------------------------------------------------------------
 * Backend seam.  Replaces candidateBackend() / cudaEnvOrDefault() in
 * patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:29-43 and
 * patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-46.
 * Returns 0 for "cpu" (unset, empty or "cpu"), 1 for "cuda"; any other value
 * of CUFLYE_CANDIDATE_BACKEND returns -1 and writes
 * "Unsupported CUFLYE_CANDIDATE_BACKEND: <value>" into msg.
 * ------------------------------------------------------------------------ */
int cuflye_candidate_backend(char* msg, size_t msg_cap);

/* Opens a context on `device` with a device-memory budget in bytes
 * (0 = unbounded).  Replaces the CUFLYE_CUDA_DEVICE /
 * CUFLYE_CUDA_MEMORY_BUDGET_BYTES handling of
 * patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-44. */
cuflye_status cuflye_open(int device, uint64_t memory_budget_bytes, cuflye_ctx** out);

/* Same, reading CUFLYE_CUDA_DEVICE (default "0") and
 * CUFLYE_CUDA_MEMORY_BUDGET_BYTES (default "unbounded") from the
 * environment. */
cuflye_status cuflye_open_from_env(cuflye_ctx** out);

/* A context of its own (stream, device arena, budget) that uses `owner`'s
 * resident index, read only, so that host threads can each run queries on
 * one index (no counterpart in the reference, whose adapter serialises every
 * call behind one mutex: patches/flye/2.9.6/0004-cuflye-cuda-adapter-shell.patch:105-109,
 * 390-392).  The owner must have an index, keep it (rebuilding it fails with
 * CUFLYE_ERR_INVALID while shared contexts are open) and stay open until
 * they are closed.  A shared context cannot build an index of its own; it
 * starts without a graph (cuflye_graph_set gives it one). */
cuflye_status cuflye_open_shared(cuflye_ctx* owner, uint64_t memory_budget_bytes,
                                 cuflye_ctx** out);

void cuflye_close(cuflye_ctx* ctx);

/* The last failure's one-line message.  With ctx == NULL: why the calling
 * thread's last cuflye_open / cuflye_open_from_env failed (empty after a
 * success).  Unsupported shapes, budget failures and failed opens carry the
 * reference stub's fields first ("cuFlye CUDA candidate backend selected;
 * adapter=cuflye_gb300; CUFLYE_CUDA_DEVICE=<d>;
 * CUFLYE_CUDA_MEMORY_BUDGET_BYTES=<b>; <reason>"), as
 * patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-46 throws them. */
const char* cuflye_last_error(const cuflye_ctx* ctx);

/* Device memory the context holds now and at its peak, in bytes. */
cuflye_status cuflye_memory_stats(const cuflye_ctx* ctx, uint64_t* in_use, uint64_t* peak);

/* --------------------------------------------------------------------------
 * Index (Flye VertexIndex equivalent, device resident).
 * Builds an open-addressing table of standard-form k-mers over the forward
 * strands of `n` target sequences (signed ids must be > 0 and distinct).
 * freq(key) counts windows over all targets; keys with freq > max_freq are
 * repetitive (query windows hitting them become filtered positions), keys
 * with min_freq <= freq <= max_freq are solid and keep their positions.
 * Serves isRepetitive / kmerFreq / iterKmerPos as called in
 * patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:55-80.
 * k in [1, 31].  Replaces any previous index in the context.
 * ------------------------------------------------------------------------ */
cuflye_status cuflye_index_build(cuflye_ctx* ctx, int k, size_t n, const int64_t* target_ids,
                                 const int64_t* offsets, const char* bases, uint32_t min_freq,
                                 uint32_t max_freq);

/* Index from explicit, already strand-resolved entries (the flattened
 * index.tsv of cuda/cuflye_cuda_read_window_smoke.cu and
 * docs/abi/cuda-real-data-pack-dump-v0.md): entry i lists target signed id
 * target_ids[i] at positions[i] under standard-form key keys[i]; buckets keep
 * input order and lookups apply no strand transform.  rep_keys are the
 * repetitive standard-form keys. */
cuflye_status cuflye_index_from_entries(cuflye_ctx* ctx, int k, size_t n,
                                        const int64_t* target_ids, const int64_t* positions,
                                        const uint64_t* keys, size_t n_rep,
                                        const uint64_t* rep_keys);

/* Counts of the built index: distinct keys, stored positions, repetitive keys. */
cuflye_status cuflye_index_stats(const cuflye_ctx* ctx, uint64_t* keys, uint64_t* positions,
                                 uint64_t* repetitive);

/* Index construction in key ranges (no counterpart in the reference, whose
 * VertexIndex is built in host memory).  cuflye_index_build sorts all
 * windows at once when they fit the memory budget; otherwise it builds one
 * contiguous range of standard-form keys at a time, each range sized to what
 * the budget leaves, and fills the table from every range's entries at the
 * end.  The index is the same either way.  max_windows > 0 also caps the
 * windows of one range (0, the default: the budget alone decides).
 * cuflye_last_index_ranges gives the ranges of the last cuflye_index_build. */
cuflye_status cuflye_set_index_build_windows(cuflye_ctx* ctx, uint64_t max_windows);
cuflye_status cuflye_last_index_ranges(const cuflye_ctx* ctx, uint64_t* ranges);

/* --------------------------------------------------------------------------
 * Candidate records (candidate-record-v1, docs/abi/candidate-record-v1.md:31-51).
 * Replaces collectCandidateMatchesCpu
 * (patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:53-95) and the
 * callee signature of patches/flye/2.9.6/0005-cuflye-real-data-pack-dump.patch:246-250:
 * per query, the records are in Flye's generation order (window order, then
 * bucket order); `filtered` receives the repetitive window positions
 * (curFilteredPos).
 * ------------------------------------------------------------------------ */
typedef struct cuflye_candidate {
  int64_t query_id;
  int64_t target_id; /* signed; strand '+' iff > 0 */
  uint64_t kmer;     /* forward query k-mer, Kmer::numRepr() */
  int32_t query_pos;
  int32_t target_pos;
} cuflye_candidate;

typedef struct cuflye_filtered_pos {
  int64_t query_id;
  int32_t pos;
  int32_t reserved;
} cuflye_filtered_pos;

cuflye_status cuflye_candidates(cuflye_ctx* ctx, size_t n, const int64_t* query_ids,
                                const int64_t* offsets, const char* bases,
                                cuflye_candidate* out, size_t out_cap, size_t* n_out,
                                cuflye_filtered_pos* filtered, size_t filtered_cap,
                                size_t* n_filtered);

/* --------------------------------------------------------------------------
 * Overlaps (overlap-range-v1, docs/abi/overlap-range-v1.md:21-41).
 * Replaces OverlapDetector::getSeqOverlaps after candidate collection:
 * Flye's KmerMatch sort, group prefilter, ext re-sort, chaining DP,
 * score-ordered backtrack, overlapTest, k-mer divergence, primary selection
 * and max_overlaps (tools/replay_overlap_chains.py:196-422).  Rows come per
 * query in Flye's emission order.
 * ------------------------------------------------------------------------ */
typedef struct cuflye_overlap_params {
  int32_t kmer_size;          /* must equal the index k                      */
  int32_t min_overlap;
  int32_t max_jump;
  int32_t max_gap;            /* max_jump_gap                                */
  int32_t gap_jump_threshold;
  int32_t max_overhang;
  int32_t check_overhang;
  int32_t force_local;
  int32_t only_max_ext;
  int32_t max_overlaps;       /* 0 = unlimited                               */
  float large_gap_penalty;
  float small_gap_penalty;
  float min_kmer_survival_rate;
  float max_divergence;
  float sample_rate;
} cuflye_overlap_params;

typedef struct cuflye_overlap_range {
  int64_t cur_id;
  int64_t ext_id;
  int32_t cur_begin, cur_end, cur_len;
  int32_t ext_begin, ext_end, ext_len;
  int32_t score;
  float seq_divergence;
} cuflye_overlap_range;

cuflye_status cuflye_overlaps(cuflye_ctx* ctx, size_t n, const int64_t* query_ids,
                              const int64_t* offsets, const char* bases,
                              const cuflye_overlap_params* params, cuflye_overlap_range* out,
                              size_t out_cap, size_t* n_out);

/* Batch sizing: queries per device pass (0 = as many as the budget allows).
 * 1 gives the plain one-read-per-launch path. */
cuflye_status cuflye_set_batch_queries(cuflye_ctx* ctx, size_t queries_per_pass);

/* Sorted emission (no counterpart in the reference; on by default): overlap
 * and read-to-graph calls on a built index write each query's candidate hits
 * straight into the order of Flye's KmerMatch sort, one block per query, and
 * decide most target groups' prefilter on the way, instead of writing them
 * in generation order and sorting.  The rows are the same either way.  1
 * (the default) takes it for passes whose windows average at least 6 hits
 * and that hold at least two queries per SM, where it pays off; sparser
 * passes (reads against a genome or a graph) and small ones (the one-read
 * path) emit and sort.  2 takes it for every pass, 0 for none (for comparison).  A pass
 * holding a query that hits more than 2,048 distinct targets takes the emit
 * + sort path by itself (counted in cuflye_last_sort_stats, entry 7). */
cuflye_status cuflye_set_sorted_emission(cuflye_ctx* ctx, int enable);

/* --------------------------------------------------------------------------
 * Launch shapes and the autotuner (no counterpart in the reference).
 * Blocks per SM of the four kernels that take their work from a counter or
 * grid-stride, so that their grid changes no result: the chaining DP (1-8),
 * the backtrack (1-4), the KmerMatch radix scatter (1-2) and the rounds of
 * the libstdc++-order sort (1-2).  0 keeps a kernel's default (8, 4, 2, 2).
 * ------------------------------------------------------------------------ */
typedef struct cuflye_launch_shape {
  int32_t dp_blocks_per_sm;
  int32_t backtrack_blocks_per_sm;
  int32_t scatter_blocks_per_sm;
  int32_t round_blocks_per_sm;
} cuflye_launch_shape;

cuflye_status cuflye_set_launch_shape(cuflye_ctx* ctx, const cuflye_launch_shape* shape);
cuflye_status cuflye_get_launch_shape(const cuflye_ctx* ctx, cuflye_launch_shape* shape);

/* Runs the overlap path on the given queries (a sample of the workload; the
 * rows are discarded) under candidate shapes, one kernel at a time, and
 * keeps for each kernel the blocks per SM with the least device time of
 * stages 0-4 (the better of two calls; a change must gain 1 %).  The
 * context's shape becomes the chosen one.  chosen (optional) receives it;
 * ms_start / ms_chosen (optional) the device time of one call under the
 * starting and the chosen shape. */
cuflye_status cuflye_autotune(cuflye_ctx* ctx, size_t n, const int64_t* query_ids,
                              const int64_t* offsets, const char* bases,
                              const cuflye_overlap_params* params, cuflye_launch_shape* chosen,
                              double* ms_start, double* ms_chosen);

/* --------------------------------------------------------------------------
 * Read-to-graph chains (read-alignment-v1, docs/abi/read-alignment-v1.md:25-48).
 * Replaces the per-read body of ReadAligner::alignReads
 * (patches/flye/2.9.6/0039-cuflye-read-to-graph-input-boundary-oracle.patch:226-251,
 * patches/flye/2.9.6/0026-cuflye-read-alignment-replay-fixture-dump.patch:215-235):
 * quickSeqOverlaps against the edge index, the LONG_EDGE/BIG_ALN input
 * filter, the curBegin sort, chainReadAlignments, the chain divergence
 * filter, then good chains followed by their complements.  The index must be
 * built from the edge sequences (ids = edge-sequence ids).  Edge e (> 0) owns
 * edge sequence seq_ids[e] and runs left[e] -> right[e]; its complement -e
 * runs right^1 -> left^1.
 * ------------------------------------------------------------------------ */
typedef struct cuflye_r2g_params {
  int32_t max_jump;
  int32_t max_read_overlap;
  int32_t min_overlap;
  int32_t max_separation;
  int32_t long_edge;
  int32_t big_aln;
  float max_chain_divergence; /* read_align_ovlp_divergence */
} cuflye_r2g_params;

typedef struct cuflye_read_alignment {
  int64_t chain_id;
  int64_t segment_id;
  int64_t read_id;
  int64_t edge_id;
  int64_t edge_seq_id;
  int32_t read_begin, read_end, read_len;
  int32_t edge_begin, edge_end, edge_len;
  int32_t score;
  float seq_divergence;
} cuflye_read_alignment;

cuflye_status cuflye_graph_set(cuflye_ctx* ctx, size_t n_edges, const int64_t* edge_ids,
                               const int64_t* seq_ids, const int32_t* left,
                               const int32_t* right);

cuflye_status cuflye_read_to_graph(cuflye_ctx* ctx, size_t n, const int64_t* read_ids,
                                   const int64_t* offsets, const char* bases,
                                   const cuflye_overlap_params* params,
                                   const cuflye_r2g_params* r2g, cuflye_read_alignment* out,
                                   size_t out_cap, size_t* n_out);

/* --------------------------------------------------------------------------
 * Candidate chains before the divergence filter (Flye's readChains,
 * patches/flye/2.9.6/0026-cuflye-read-alignment-replay-fixture-dump.patch:215-226)
 * as the records of the compact binary payload
 * (docs/abi/read-alignment-compact-binary-v0.md:37-58; the reference writes
 * them in cuda/cuflye_cuda_read_alignment_chain_replay.cu:2575-2660).  Per
 * read (fixture): chains in acceptance order, segments in chain order.
 * overlap_index is the segment's position in the read's chain input (its
 * edge overlaps after the LONG_EDGE / BIG_ALN filter and the curBegin sort);
 * candidate_id is the replay fixture's candidate id, or for in-process reads
 * the overlap's index among the read's quickSeqOverlaps rows before the
 * filter.  query_id is the fixture's query id (in-process: the read id).
 * ------------------------------------------------------------------------ */
typedef struct cuflye_chain_record {
  int64_t query_id;
  int32_t chain_id;
  int32_t segment_id;
  int32_t overlap_index;
  int32_t reserved;
  int64_t candidate_id;
  int64_t read_id;
  int64_t edge_id;
  int64_t edge_seq_id;
  int32_t read_begin, read_end, read_len;
  int32_t edge_left, edge_right;
  int32_t edge_begin, edge_end, edge_len;
  int32_t score;
  float seq_divergence;
} cuflye_chain_record;

/* Read-to-graph up to the candidate chains: quickSeqOverlaps against the edge
 * index, the LONG_EDGE / BIG_ALN filter, the curBegin sort and
 * chainReadAlignments, for each read; the candidate chains as chain records.
 * inputs_per_read (optional, n entries) receives each read's chain-input
 * overlaps (the payload header's input record counts). */
cuflye_status cuflye_read_to_graph_chains(cuflye_ctx* ctx, size_t n, const int64_t* read_ids,
                                          const int64_t* offsets, const char* bases,
                                          const cuflye_overlap_params* params,
                                          const cuflye_r2g_params* r2g,
                                          cuflye_chain_record* out, size_t out_cap,
                                          size_t* n_out, uint64_t* inputs_per_read);

/* Read-alignment replay fixtures (docs/abi/read-alignment-replay-fixture-v0.md):
 * the GPU path of cuda/cuflye_cuda_read_alignment_chain_replay.cu:1044-1253.
 * Fixture f is one read's chain input, overlaps[fixture_offsets[f] ..
 * fixture_offsets[f + 1]) in edge-overlaps.tsv order, with query id
 * query_ids[f].  The call chains every fixture on the device and returns its
 * candidate chains as chain records, and per candidate chain (fixture by
 * fixture, chains in acceptance order) its divergence and whether it is kept
 * (divergence < r2g->max_chain_divergence, Flye's read_align_ovlp_divergence
 * test).  With chain_div_in == NULL the divergence is this library's k-mer
 * form (the curRange-weighted mean of the segments' divergences, summed in
 * chain order in float); otherwise chain_div_in holds one value per candidate
 * chain (chain-divergence.tsv, fixture by fixture) and n_chain_div_in must
 * equal the number of candidate chains, else CUFLYE_ERR_INVALID with that
 * number in *n_chains.  kept_rows (optional) receives the read-alignment
 * rows of the kept chains and their complements (read-alignment-v1, chain
 * ids numbered across fixtures), as cuflye_read_to_graph emits them. */
typedef struct cuflye_edge_overlap {
  int64_t candidate_id;
  int64_t read_id;
  int32_t read_begin, read_end, read_len;
  int32_t edge_left, edge_right;
  int32_t edge_begin, edge_end, edge_len;
  int64_t edge_id;
  int64_t edge_seq_id;
  int32_t score;
  float seq_divergence;
} cuflye_edge_overlap;

cuflye_status cuflye_chain_read_alignments(
    cuflye_ctx* ctx, size_t n_fixtures, const uint64_t* fixture_offsets,
    const int64_t* query_ids, const cuflye_edge_overlap* overlaps,
    const cuflye_r2g_params* r2g, const float* chain_div_in, size_t n_chain_div_in,
    cuflye_chain_record* out, size_t out_cap, size_t* n_out, float* chain_div,
    uint8_t* chain_kept, size_t chain_cap, size_t* n_chains, cuflye_read_alignment* kept_rows,
    size_t rows_cap, size_t* n_rows);

/* The compact binary payload (docs/abi/read-alignment-compact-binary-v0.md):
 * a 64-byte header (magic CUFRALB0, sizes, version 0.0, fixture count,
 * record count, input record totals, output mode 1 = pre-divergence chains)
 * and one 92-byte little-endian record per chain record, written into the
 * caller's buffer (host code only, no device).  fixtures: the reads or
 * fixtures the records come from; inputs_per_fixture: each one's chain-input
 * overlaps (for the header's total, minimum and maximum).  out_cap too small:
 * CUFLYE_ERR_CAPACITY with the payload size in *n_out. */
#define CUFLYE_COMPACT_HEADER_BYTES 64u
#define CUFLYE_COMPACT_RECORD_BYTES 92u
cuflye_status cuflye_compact_binary(const cuflye_chain_record* records, size_t n_records,
                                    size_t fixtures, const uint64_t* inputs_per_fixture,
                                    unsigned char* out, size_t out_cap, size_t* n_out);

/* --------------------------------------------------------------------------
 * The device sort every Flye sort point above runs on: sorts each segment
 * [seg_offsets[s], seg_offsets[s+1]) of (key, value) pairs in place, leaving
 * equal keys in exactly the order libstdc++'s std::sort(first, last,
 * [](a, b) { return a.key < b.key; }) leaves them (introsort; see
 * tools/replay_read_to_graph_source_pack.py:95-181 for the reference's
 * restatement of that order).  Host arrays in, host arrays out.
 * ------------------------------------------------------------------------ */
cuflye_status cuflye_std_sort_segments(cuflye_ctx* ctx, uint64_t* keys, uint32_t* values,
                                       const uint64_t* seg_offsets, size_t n_segments);

/* --------------------------------------------------------------------------
 * Allocation-free variant of cuflye_std_sort_segments, for callers that may
 * not allocate device memory (for example a host process whose GPU memory
 * is entirely owned by another allocator, or a worker held to a fixed,
 * pre-declared footprint).  No counterpart in the reference.
 *
 * keys / values: the caller's DEVICE arrays, sorted in place.
 * seg_offsets:   HOST array of n_segments + 1 offsets into them, all within
 *                [0, n_elements]; elements past seg_offsets[n_segments]
 *                are left untouched.
 * stream:        a cudaStream_t (NULL = default stream).  With n_elements
 *                <= 4,096 the call returns once the work is queued.  With
 *                more, the sort reads its round counts back to the host
 *                between rounds of its large-segment phase, so the call
 *                waits on `stream` and returns after the work is done.
 * Needs no context and makes no cudaMalloc / cudaFree or other allocating
 * call: its scratch is one fixed device array of about 13.6 MiB that every
 * GPU loading the library holds until exit.  Limits: n_elements <=
 * CUFLYE_NOALLOC_MAX_ELEMENTS, n_segments <= CUFLYE_NOALLOC_MAX_SEGMENTS
 * (larger requests return CUFLYE_ERR_UNSUPPORTED before anything is
 * queued).  The first call on each device looks up that array's device
 * address (with that device current) and caches it for the life of the
 * process (not valid across a cudaDeviceReset); make that first call before
 * any stream capture.  Calls share the array: calls whose work overlaps on
 * the GPU race and must not be issued.
 * ------------------------------------------------------------------------ */
#define CUFLYE_NOALLOC_MAX_ELEMENTS 1048576u
#define CUFLYE_NOALLOC_MAX_SEGMENTS 65536u
cuflye_status cuflye_std_sort_segments_noalloc(uint64_t* keys, uint32_t* values,
                                               const uint64_t* seg_offsets, size_t n_segments,
                                               size_t n_elements, void* stream);

/* --------------------------------------------------------------------------
 * Serving: continuous batching of overlap requests on the owner's device.
 * The cuflye_submit / cuflye_poll pair of the C-ABI the reference's worker
 * protocol stands in for (docs/abi/cuda-overlap-worker-protocol-v0.md:30-142,
 * file-backed requests and responses); no in-process counterpart exists in
 * the reference.
 *
 * cuflye_server_open borrows `owner`'s resident index (the owner must keep it
 * and stay open until cuflye_server_close; rebuilding the owner's index while
 * a server is open fails with CUFLYE_ERR_INVALID) and starts `workers` (1-8)
 * worker contexts, each with its own stream and device arena; the owner's budget
 * left over (or the free device memory less 8 GiB when unbounded) is split
 * between them.  A worker that falls idle takes every request that has
 * arrived, up to max_batch_bases query bases (0 = no limit), and runs them
 * as one batch with `params`; requests arriving meanwhile go to the next
 * idle worker, so batches overlap on the device.  A request's rows are the
 * rows cuflye_overlaps gives for its queries alone, in the same order.
 *
 * cuflye_submit copies the request (queries as for cuflye_overlaps) and
 * returns a ticket.  cuflye_poll waits up to wait_ms (negative: until done,
 * 0: no wait) and returns CUFLYE_PENDING, the request's error, or its rows;
 * with too small a capacity it returns CUFLYE_ERR_CAPACITY and the row count,
 * and keeps the result for a retry.  A finished ticket is consumed by the
 * poll that returns its rows or its error.
 * ------------------------------------------------------------------------ */
typedef struct cuflye_server cuflye_server;

cuflye_status cuflye_server_open(cuflye_ctx* owner, int workers,
                                 const cuflye_overlap_params* params, uint64_t max_batch_bases,
                                 cuflye_server** out);
cuflye_status cuflye_submit(cuflye_server* server, size_t n, const int64_t* query_ids,
                            const int64_t* offsets, const char* bases, uint64_t* ticket);
cuflye_status cuflye_poll(cuflye_server* server, uint64_t ticket, int wait_ms,
                          cuflye_overlap_range* out, size_t out_cap, size_t* n_out);
/* The next finished request in completion order, for a caller with many in
 * flight: waits up to wait_ms (negative: until one finishes, 0: no wait) and
 * returns CUFLYE_PENDING with *ticket = 0, or the ticket with the request's
 * error or rows (consumed as by cuflye_poll).  With too small a capacity it
 * returns CUFLYE_ERR_CAPACITY with the ticket and the row count; the result
 * is then kept for cuflye_poll on that ticket and not returned here again.
 * Tickets that cuflye_poll consumed first are skipped. */
cuflye_status cuflye_poll_any(cuflye_server* server, int wait_ms, uint64_t* ticket,
                              cuflye_overlap_range* out, size_t out_cap, size_t* n_out);
/* Batches run so far, requests they carried, requests waiting. */
cuflye_status cuflye_server_stats(cuflye_server* server, uint64_t* batches, uint64_t* requests,
                                  uint64_t* pending);
const char* cuflye_server_last_error(cuflye_server* server);
void cuflye_server_close(cuflye_server* server);

/* --------------------------------------------------------------------------
 * Timing of the last call's device work (CUDA events on the context's
 * stream; the work its sorts run on the context's two side streams is joined
 * into that stream before each sort returns), in milliseconds, by stage: 0 hit generation, 1 KmerMatch sort,
 * 2 group prefilter + ext re-sort, 3 chaining DP, 4 score sort + backtrack +
 * row compaction, 5 output conversion + device-to-host copy, 6 host-to-device
 * copy of the queries.  Stages 0-4 run on inputs already in device memory.
 * stage_bytes gives the algorithmic bytes of stages 0-4 (overlaps only).
 * ------------------------------------------------------------------------ */
cuflye_status cuflye_last_timing(const cuflye_ctx* ctx, double* stage_ms, uint64_t* stage_bytes,
                                 size_t n_stages);

/* Diagnostics of the last overlaps / read-to-graph call (no counterpart in
 * the reference): how its sort points ran.  Segments whose keys are all
 * distinct have one sorted order and need no emulation of libstdc++'s
 * std::sort; the others take the libstdc++-order sort.  counts[0] / [1]:
 * queries whose KmerMatch sort ran plain / libstdc++-order; [2] / [3]:
 * ext-sorted groups put in ext-pos order plain (most already are) /
 * libstdc++-order; [4]: groups whose backtrack picked its starts by score
 * itself; [5]: 0 (no score order is sorted ahead of the backtrack); [6]:
 * groups whose backtrack ran again in the libstdc++ order because equal
 * scores could change their result; [7]: passes that left the sorted
 * emission for the emit + sort path (a query with more distinct targets than
 * its dictionary holds). */
cuflye_status cuflye_last_sort_stats(const cuflye_ctx* ctx, uint64_t* counts, size_t n);

/* Passes of the last candidates / overlaps / read-to-graph call: runs of
 * queries that fitted the memory budget (or cuflye_set_batch_queries) and
 * went through the device one after another (no counterpart in the
 * reference). */
cuflye_status cuflye_last_passes(const cuflye_ctx* ctx, uint64_t* passes);

/* Host-side statistics of the last call (no counterpart in the reference):
 * its passes, the passes that ran again on half their queries because their
 * later buffers exceeded the memory budget, and the host milliseconds spent
 * in device allocation and release. */
cuflye_status cuflye_last_pass_stats(const cuflye_ctx* ctx, uint64_t* passes, uint64_t* retries,
                                     double* alloc_ms);

/* Returns the context's cached working buffers to the device: everything a
 * call allocates and keeps for the next one (hit arrays, sort scratch,
 * per-group tables, rows), leaving the index, the graph and the logf table.
 * The next call allocates what it needs again.  For a long-lived process
 * that holds a context between large calls. */
cuflye_status cuflye_trim(cuflye_ctx* ctx);

/* Kernel launches issued by the library in this process so far. */
cuflye_status cuflye_kernel_launches(uint64_t* total);

#ifdef __cplusplus
}
#endif

#endif /* CUFLYE_H */
