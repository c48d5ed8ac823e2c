// r2g.h — launchers of the read-to-graph chain stage.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/cuflye.h"
#include "kernels.h"

namespace cuflye {

struct R2GParams {
  int32_t max_jump, max_read_overlap, min_overlap, max_separation, long_edge, big_aln;
  float max_chain_divergence;
};

// Graph tables indexed by the dense slot of each edge sequence.
struct R2GGraph {
  const int64_t* edge_of_slot;  // signed id (> 0) of the forward edge owning the sequence
  const int32_t* left_of_slot;
  const int32_t* right_of_slot;
  const int64_t* slot_signed;   // edge-sequence signed id (> 0) of the slot
};

// Per chain-input row: the graph nodes and ids of the edge it aligns to, and
// its candidate id (replay: the fixture's; in-process: its index among the
// read's quickSeqOverlaps rows before the filter).
struct R2GRowMeta {
  int64_t candidate_id;
  int64_t edge_id;      // signed
  int64_t edge_seq_id;  // signed
  int32_t left, right;  // graph nodes of the (signed) edge
};

cudaError_t r2g_filter(const OverlapRow* rows, uint64_t n, const R2GParams& rp, uint32_t* keep,
                       cudaStream_t s);
// kept rows in order; src[j] = the j-th kept row's index among all rows
cudaError_t r2g_compact(const OverlapRow* rows, uint64_t n, const uint32_t* keep,
                        const uint64_t* pos, OverlapRow* out, uint64_t* src, cudaStream_t s);
cudaError_t r2g_sort_keys(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                          uint64_t* keys, uint32_t* vals, cudaStream_t s);
// the sorted chain input and its metadata; row_off: each read's first row
// before the filter
cudaError_t r2g_permute(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                        const uint32_t* vals, const uint64_t* src, const uint64_t* row_off,
                        const R2GGraph& g, OverlapRow* out, R2GRowMeta* meta, cudaStream_t s);
// replay fixtures' edge overlaps as chain input
cudaError_t r2g_replay_rows(const cuflye_edge_overlap* in, uint64_t n, OverlapRow* out,
                            R2GRowMeta* meta, cudaStream_t s);
size_t r2g_rec_bytes();
// candidate chains (before the divergence filter): cand[a_off[q] + t], n_cand[q]
cudaError_t r2g_chain(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                      const R2GRowMeta* meta, const R2GParams& rp, void* recs, int32_t* active,
                      int32_t* frozen, int32_t* cand, uint32_t* n_cand, cudaStream_t s);
// per candidate chain: divergence (div_in at div_off[q] + t when given, else
// the k-mer form) into div_out and the accept flag into acc_out (both at
// a_off[q] + t, optional); good chains, their count and rows per read, and
// all candidate chains' segments per read (n_segs, optional)
cudaError_t r2g_divergence(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                           const void* recs, const int32_t* cand, const uint32_t* n_cand,
                           const float* div_in, const uint64_t* div_off, const R2GParams& rp,
                           float* div_out, uint8_t* acc_out, int32_t* good, uint32_t* n_good,
                           uint32_t* n_rows, uint32_t* n_segs, cudaStream_t s);
cudaError_t r2g_emit(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                     const R2GRowMeta* meta, const int64_t* read_ids, const void* recs,
                     const int32_t* good, const uint32_t* n_good, const uint64_t* chain_off,
                     const uint64_t* row_off, int32_t* tmp, cuflye_read_alignment* out,
                     cudaStream_t s);
// the candidate chains as chain records at rec_off[q]
cudaError_t r2g_records(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                        const R2GRowMeta* meta, const int64_t* query_ids, const int64_t* read_ids,
                        const void* recs, const int32_t* cand, const uint32_t* n_cand,
                        const uint64_t* rec_off, cuflye_chain_record* out, cudaStream_t s);

// Overlap rows -> ABI records (candidate output of the overlaps entry point).
cudaError_t rows_to_abi(const OverlapRow* rows, uint64_t n, const QueryInfo* qinfo,
                        const int64_t* slot_signed, cuflye_overlap_range* out, cudaStream_t s);
// Hits -> candidate-record ABI.
cudaError_t hits_to_abi(const uint64_t* keys, const uint32_t* vals, const uint64_t* kmers,
                        uint64_t n, const uint64_t* q_off, uint32_t nq, const QueryInfo* qinfo,
                        const int64_t* slot_signed, cuflye_candidate* out, cudaStream_t s);
cudaError_t filtered_to_abi(const int32_t* fpos, uint64_t n, const uint64_t* f_off, uint32_t nq,
                            const QueryInfo* qinfo, cuflye_filtered_pos* out, cudaStream_t s);

// The compact binary payload's 64-byte header and one 92-byte record, little
// endian field by field (host code).
void compact_write_header(unsigned char* out, uint64_t fixtures, uint64_t records,
                          uint64_t total_inputs, uint32_t min_inputs, uint32_t max_inputs);
void compact_write_record(unsigned char* out, const cuflye_chain_record& r);

}  // namespace cuflye
