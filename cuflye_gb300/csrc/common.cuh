// common.cuh — device helpers shared by every kernel of the overlap hot path.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cuflye {

// ---------------------------------------------------------------- ids
// Flye internal ids: +n -> 2(n-1), -n -> 2n-1; the reverse strand is id ^ 1
// (patches/flye/2.9.6/0004-cuflye-cuda-adapter-shell.patch:74-86).  On the
// device a target is addressed by its dense slot t (rank of its signed id);
// its dense internal id 2t + strand orders exactly like Flye's internal id.

// ---------------------------------------------------------------- 2-bit k-mers
// Bases are packed MSB-first, 32 per 64-bit word, so the numeric value of a
// window equals Flye's Kmer::numRepr() (A=0 C=1 G=2 T=3, first base most
// significant: cuda/cuflye_cuda_read_window_smoke.cu:172-206).
__host__ __device__ __forceinline__ uint32_t base_code(uint8_t c) {
  switch (c) {
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 0;
  }
}

// Window of k bases starting at global base index g (k <= 32).  `words`
// must hold one padding word past the last base.
__device__ __forceinline__ uint64_t kmer_at(const uint64_t* __restrict__ words, uint64_t g,
                                            int k) {
  const uint64_t w = g >> 5;
  const uint32_t s = static_cast<uint32_t>(g & 31u);
  const uint64_t hi = __ldg(words + w);
  uint64_t win = hi;
  if (s) win = (hi << (2 * s)) | (__ldg(words + w + 1) >> (64 - 2 * s));
  return win >> (64 - 2 * k);
}

// Reverse complement of a k-mer held in the low 2k bits: reverse the 2-bit
// groups of the whole word, complement, drop the 64-2k high groups.
__device__ __forceinline__ uint64_t revcomp(uint64_t x, int k) {
  uint64_t r = __brevll(x);
  r = ((r >> 1) & 0x5555555555555555ULL) | ((r & 0x5555555555555555ULL) << 1);
  return (~r) >> (64 - 2 * k);
}

// ---------------------------------------------------------------- hashing
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

// Open-addressing table entry: 16 bytes, one sector-aligned 128-bit load.
// meta: bits 0-39 bucket offset, 40-61 bucket count, 62 repeated stored id,
// 63 repetitive.
struct alignas(16) TableEntry {
  uint64_t key;
  uint64_t meta;
};
constexpr uint64_t kEmptyKey = ~0ULL;  // never a standard form (see index.cu)
constexpr uint64_t kOffsetMask = (1ULL << 40) - 1;
constexpr uint32_t kCountBits = 22;
constexpr uint64_t kRepetitiveBit = 1ULL << 63;
// A solid bucket listing one stored target id more than once: a query window
// that looks it up yields two hits on one target, i.e. two equal
// (ext id, cur pos) KmerMatch keys.
constexpr uint64_t kDupIdsBit = 1ULL << 62;

// Per-window flags of hit counting.
constexpr uint8_t kWinRev = 1;       // the window k-mer is not in standard form
constexpr uint8_t kWinFiltered = 2;  // repetitive: a filtered position
constexpr uint8_t kWinTrivial = 4;   // the bucket held the window's own position

// A key's first slot in a table of cap slots (any cap >= 1): the high half
// of mix64(key) * cap, which maps the hash onto [0, cap) evenly.  Probing
// continues at slot + 1, wrapping at cap.
__device__ __forceinline__ uint64_t table_slot(uint64_t key, uint64_t cap) {
  return __umul64hi(mix64(key), cap);
}
__device__ __forceinline__ uint64_t table_next(uint64_t slot, uint64_t cap) {
  return slot + 1 == cap ? 0 : slot + 1;
}

// The table keeps its load at 1/2 or below, so a probe always meets an
// empty slot.
__device__ __forceinline__ uint64_t table_probe(const TableEntry* __restrict__ table,
                                                uint64_t cap, uint64_t key, bool* found) {
  uint64_t slot = table_slot(key, cap);
  for (;;) {
    const ulonglong2 e = __ldg(reinterpret_cast<const ulonglong2*>(table + slot));
    if (e.x == key) {
      *found = true;
      return e.y;
    }
    if (e.x == kEmptyKey) {
      *found = false;
      return 0;
    }
    slot = table_next(slot, cap);
  }
}

// ---------------------------------------------------------------- float rules
// Every float expression of the chaining path is spelled with explicit
// round-to-nearest intrinsics so the compiler cannot contract it into FMAs;
// the host side is compiled with -ffp-contract=off and gives the same bits.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }

// ---------------------------------------------------------------- logf
// Natural log of a float x >= 1 as Flye computes it with the C library's
// logf.  The C library's logf is not correctly rounded, so the device
// computes its own double-precision log (log_wide, below), rounds it to float,
// and then applies an exception table built on the same machine by comparing
// the C library's logf with that very function over every float in
// [1, 2^24).  The table (sorted x bits -> result bits) lives in device memory.
struct LogfTable {
  const uint32_t* x_bits;
  const uint32_t* y_bits;
  uint32_t n;
};

#ifdef __CUDA_ARCH__
#define CUFLYE_DADD(a, b) __dadd_rn((a), (b))
#define CUFLYE_DSUB(a, b) __dsub_rn((a), (b))
#define CUFLYE_DMUL(a, b) __dmul_rn((a), (b))
#define CUFLYE_DDIV(a, b) __ddiv_rn((a), (b))
#else
#define CUFLYE_DADD(a, b) ((a) + (b))
#define CUFLYE_DSUB(a, b) ((a) - (b))
#define CUFLYE_DMUL(a, b) ((a) * (b))
#define CUFLYE_DDIV(a, b) ((a) / (b))
#endif

// log(x) for finite x > 0 in double: x = 2^e * m with m in [sqrt(1/2), sqrt(2)),
// log(m) = 2 atanh(s) with s = (m - 1) / (m + 1), summed as the odd power
// series of atanh (|s| < 0.1716, twelve terms), plus e * ln 2 in two parts.
// Every operation is an explicit IEEE double op, so host and device agree.
__host__ __device__ inline double log_wide(float xf) {
  union {
    double d;
    uint64_t u;
  } v;
  v.d = static_cast<double>(xf);
  int e = static_cast<int>((v.u >> 52) & 0x7ff) - 1023;
  v.u = (v.u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;  // m in [1, 2)
  double m = v.d;
  if (m > 1.4142135623730951) {
    m = CUFLYE_DMUL(m, 0.5);
    e += 1;
  }
  const double s = CUFLYE_DDIV(CUFLYE_DSUB(m, 1.0), CUFLYE_DADD(m, 1.0));
  const double s2 = CUFLYE_DMUL(s, s);
  // 1 + s2/3 + s2^2/5 + ... + s2^11/23, Horner from the top
  double t = 1.0 / 23.0;
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 21.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 19.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 17.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 15.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 13.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 11.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 9.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 7.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 5.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0 / 3.0);
  t = CUFLYE_DADD(CUFLYE_DMUL(t, s2), 1.0);
  const double logm = CUFLYE_DMUL(CUFLYE_DMUL(2.0, s), t);
  // ln 2 = LN2_HI + LN2_LO with LN2_HI = 726816 / 2^20 (20 fractional bits),
  // so e * LN2_HI is exact for every exponent a float can have.
  const double LN2_HI = 0.693145751953125;
  const double LN2_LO = 0.000001428606820309417232;
  const double de = static_cast<double>(e);
  return CUFLYE_DADD(CUFLYE_DMUL(de, LN2_HI), CUFLYE_DADD(CUFLYE_DMUL(de, LN2_LO), logm));
}

__host__ __device__ inline float logf_wide(float x) { return static_cast<float>(log_wide(x)); }

#ifdef __CUDACC__
__device__ __forceinline__ float flye_logf(float x, const LogfTable& t) {
  uint32_t xb = __float_as_uint(x);
  uint32_t lo = 0, hi = t.n;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    uint32_t v = __ldg(t.x_bits + mid);
    if (v < xb)
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo < t.n && __ldg(t.x_bits + lo) == xb) return __uint_as_float(__ldg(t.y_bits + lo));
  return __double2float_rn(log_wide(x));
}
#endif

// ---------------------------------------------------------------- status
// Device-side error word: the first failing kernel records a code and a
// detail value; the host reads it after the stage and fails the call.
struct DeviceStatus {
  int32_t code;
  int32_t where;
  int64_t detail;
};
enum : int32_t {
  kDevOk = 0,
  kDevProposalOverflow = 1,
  kDevLogDomain = 2,
  kDevChainOverflow = 3,
  kDevTableFull = 4,
  kDevMatchDict = 5,  // a hit's ext id missing from its query's dictionary
};

#ifdef __CUDACC__
__device__ __forceinline__ void raise_status(DeviceStatus* st, int32_t code, int32_t where,
                                             int64_t detail) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->where = where;
    st->detail = detail;
  }
}
#endif

}  // namespace cuflye
