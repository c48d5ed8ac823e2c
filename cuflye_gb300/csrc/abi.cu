// abi.cu — device-side conversion of internal records to the C-ABI structs
// (candidate-record-v1 / overlap-range-v1 fields), so results leave the GPU
// in their final layout with one D2H copy.
#include <cstdint>
#include <cstring>

#include "../../include/cuflye.h"
#include "kernels.h"
#include "r2g.h"

namespace cuflye {
namespace {

__device__ __forceinline__ int64_t signed_of(const int64_t* slot_signed, uint32_t di) {
  const int64_t s = slot_signed[di >> 1];
  return (di & 1u) ? -s : s;
}

__device__ __forceinline__ uint32_t seg_of(const uint64_t* __restrict__ off, uint32_t n,
                                           uint64_t i) {
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void rows_abi_kernel(const OverlapRow* __restrict__ rows, uint64_t n,
                                const QueryInfo* __restrict__ qinfo,
                                const int64_t* __restrict__ slot_signed,
                                cuflye_overlap_range* __restrict__ out) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const OverlapRow r = rows[i];
  cuflye_overlap_range o;
  o.cur_id = qinfo[r.query].signed_id;
  o.ext_id = signed_of(slot_signed, r.ext_di);
  o.cur_begin = r.cur_begin;
  o.cur_end = r.cur_end;
  o.cur_len = r.cur_len;
  o.ext_begin = r.ext_begin;
  o.ext_end = r.ext_end;
  o.ext_len = r.ext_len;
  o.score = r.score;
  o.seq_divergence = r.div;
  out[i] = o;
}

__global__ void hits_abi_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                const uint64_t* __restrict__ kmers, uint64_t n,
                                const uint64_t* __restrict__ q_off, uint32_t nq,
                                const QueryInfo* __restrict__ qinfo,
                                const int64_t* __restrict__ slot_signed,
                                cuflye_candidate* __restrict__ out) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = keys[i];
  cuflye_candidate c;
  c.query_id = qinfo[seg_of(q_off, nq, i)].signed_id;
  c.target_id = signed_of(slot_signed, static_cast<uint32_t>(k >> 32));
  c.kmer = kmers[i];
  c.query_pos = static_cast<int32_t>(k & 0xffffffffu);
  c.target_pos = static_cast<int32_t>(vals[i]);
  out[i] = c;
}

__global__ void filtered_abi_kernel(const int32_t* __restrict__ fpos, uint64_t n,
                                    const uint64_t* __restrict__ f_off, uint32_t nq,
                                    const QueryInfo* __restrict__ qinfo,
                                    cuflye_filtered_pos* __restrict__ out) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cuflye_filtered_pos f;
  f.query_id = qinfo[seg_of(f_off, nq, i)].signed_id;
  f.pos = fpos[i];
  f.reserved = 0;
  out[i] = f;
}

inline unsigned grid(uint64_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

cudaError_t rows_to_abi(const OverlapRow* rows, uint64_t n, const QueryInfo* qinfo,
                        const int64_t* slot_signed, cuflye_overlap_range* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  rows_abi_kernel<<<grid(n, 256), 256, 0, s>>>(rows, n, qinfo, slot_signed, out);
  return cudaGetLastError();
}

cudaError_t hits_to_abi(const uint64_t* keys, const uint32_t* vals, const uint64_t* kmers,
                        uint64_t n, const uint64_t* q_off, uint32_t nq, const QueryInfo* qinfo,
                        const int64_t* slot_signed, cuflye_candidate* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  hits_abi_kernel<<<grid(n, 256), 256, 0, s>>>(keys, vals, kmers, n, q_off, nq, qinfo,
                                               slot_signed, out);
  return cudaGetLastError();
}

cudaError_t filtered_to_abi(const int32_t* fpos, uint64_t n, const uint64_t* f_off, uint32_t nq,
                            const QueryInfo* qinfo, cuflye_filtered_pos* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  count_launch();
  filtered_abi_kernel<<<grid(n, 256), 256, 0, s>>>(fpos, n, f_off, nq, qinfo, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- compact payload
// Fields are stored byte by byte, least significant first, so the payload is
// the same on any host (docs/abi/read-alignment-compact-binary-v0.md: "not a
// raw C++ struct dump").
namespace {
unsigned char* put_u32(unsigned char* p, uint32_t v) {
  for (int i = 0; i < 4; ++i) *p++ = static_cast<unsigned char>((v >> (8 * i)) & 0xffu);
  return p;
}
unsigned char* put_u64(unsigned char* p, uint64_t v) {
  for (int i = 0; i < 8; ++i) *p++ = static_cast<unsigned char>((v >> (8 * i)) & 0xffu);
  return p;
}
unsigned char* put_i32(unsigned char* p, int32_t v) { return put_u32(p, static_cast<uint32_t>(v)); }
unsigned char* put_i64(unsigned char* p, int64_t v) { return put_u64(p, static_cast<uint64_t>(v)); }
unsigned char* put_f32(unsigned char* p, float v) {
  uint32_t bits;
  std::memcpy(&bits, &v, sizeof(bits));
  return put_u32(p, bits);
}
}  // namespace

void compact_write_header(unsigned char* out, uint64_t fixtures, uint64_t records,
                          uint64_t total_inputs, uint32_t min_inputs, uint32_t max_inputs) {
  static const char kMagic[8] = {'C', 'U', 'F', 'R', 'A', 'L', 'B', '0'};
  std::memcpy(out, kMagic, 8);
  unsigned char* p = out + 8;
  p = put_u32(p, CUFLYE_COMPACT_HEADER_BYTES);
  p = put_u32(p, CUFLYE_COMPACT_RECORD_BYTES);
  p = put_u32(p, 0);  // version major
  p = put_u32(p, 0);  // version minor
  p = put_u64(p, fixtures);
  p = put_u64(p, records);
  p = put_u64(p, total_inputs);
  p = put_u32(p, min_inputs);
  p = put_u32(p, max_inputs);
  p = put_u32(p, 1);  // output mode: pre-divergence chains
  put_u32(p, 0);      // reserved
}

void compact_write_record(unsigned char* out, const cuflye_chain_record& r) {
  unsigned char* p = out;
  p = put_i64(p, r.query_id);
  p = put_i32(p, r.chain_id);
  p = put_i32(p, r.segment_id);
  p = put_i32(p, r.overlap_index);
  p = put_i64(p, r.candidate_id);
  p = put_i64(p, r.read_id);
  p = put_i32(p, r.read_begin);
  p = put_i32(p, r.read_end);
  p = put_i32(p, r.read_len);
  p = put_i64(p, r.edge_id);
  p = put_i32(p, r.edge_left);
  p = put_i32(p, r.edge_right);
  p = put_i64(p, r.edge_seq_id);
  p = put_i32(p, r.edge_begin);
  p = put_i32(p, r.edge_end);
  p = put_i32(p, r.edge_len);
  p = put_i32(p, r.score);
  put_f32(p, r.seq_divergence);
}

}  // namespace cuflye
