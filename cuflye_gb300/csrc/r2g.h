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

cudaError_t r2g_filter(const OverlapRow* rows, uint64_t n, const R2GParams& rp, uint32_t* keep,
                       cudaStream_t s);
cudaError_t r2g_compact(const OverlapRow* rows, uint64_t n, const uint32_t* keep,
                        const uint64_t* pos, OverlapRow* out, cudaStream_t s);
cudaError_t r2g_sort_keys(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                          uint64_t* keys, uint32_t* vals, cudaStream_t s);
cudaError_t r2g_permute(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                        const uint32_t* vals, OverlapRow* out, cudaStream_t s);
size_t r2g_rec_bytes();
cudaError_t r2g_chain(const OverlapRow* a, const uint64_t* a_off, uint32_t nq,
                      const R2GGraph& g, const R2GParams& rp, void* recs, int32_t* active,
                      int32_t* frozen, int32_t* good, uint32_t* n_good, uint32_t* n_rows,
                      cudaStream_t s);
cudaError_t r2g_emit(const OverlapRow* a, const uint64_t* a_off, uint32_t nq, const R2GGraph& g,
                     const QueryInfo* qinfo, const void* recs, const int32_t* good,
                     const uint32_t* n_good, const uint64_t* chain_off, const uint64_t* row_off,
                     int32_t* tmp, cuflye_read_alignment* out, cudaStream_t s);

// Overlap rows -> ABI records (candidate output of the overlaps entry point).
cudaError_t rows_to_abi(const OverlapRow* rows, uint64_t n, const QueryInfo* qinfo,
                        const int64_t* slot_signed, cuflye_overlap_range* out, cudaStream_t s);
// Hits -> candidate-record ABI.
cudaError_t hits_to_abi(const uint64_t* keys, const uint32_t* vals, const uint64_t* kmers,
                        uint64_t n, const uint64_t* q_off, uint32_t nq, const QueryInfo* qinfo,
                        const int64_t* slot_signed, cuflye_candidate* out, cudaStream_t s);
cudaError_t filtered_to_abi(const int32_t* fpos, uint64_t n, const uint64_t* f_off, uint32_t nq,
                            const QueryInfo* qinfo, cuflye_filtered_pos* out, cudaStream_t s);

}  // namespace cuflye
