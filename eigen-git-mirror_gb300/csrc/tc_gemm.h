// Tensor-core (tcgen05) trailing-update interface.
#pragma once
#include "internal.h"

namespace gbllt {

// A K-major operand: `rows` rows of `k` elements, `ld` elements apart (ld * element size a multiple
// of 16 bytes, base 16-byte aligned).  parts[0..2] are the successive roundings of a split operand
// (hi, mid, lo; unused parts may be null).  Row `row0` of the operand lines up with row/column 0
// of C.
struct TcOperand {
  const void* parts[3];
  int64_t rows;
  int64_t k;
  int64_t ld;
  int64_t row0;
};

// Element kinds of the operands.
constexpr int kTcBF16 = 0;
constexpr int kTcTF32 = 1;

// C (m x n fp32, column-major, ldc) -= sum over nseg segments of A_s B_s^T; segment s reads part
// (code & 3) of A and part (code >> 2) of B, code = (seg_code >> 4s) & 15.  lower: 0 = the whole
// rectangle; 1 = the lower triangle of a square C (SYRK); 2 = the rectangle, writing only entries
// with row >= column.  d_err receives 1 if a bounded wait ran out.
// reserve_sms > 0: the persistent grid leaves that many SMs out and each CTA claims the whole
// shared memory of its SM, so kernels launched meanwhile on other streams (the panel factorisation
// of the look-ahead schedule) run on the reserved SMs instead of sharing the update's SMs.
// max_ctas > 0 caps the persistent grid (an update that must fit on the reserved SMs).
// diag (kTcLowerRect only): C's origin sits diag rows below the diagonal of the full matrix, so the
// entries written are those with row + diag >= column.
constexpr int kTcFull = 0, kTcLowerTri = 1, kTcLowerRect = 2;
int tc_update(const TcOperand& a, const TcOperand& b, int kind, int nseg, uint32_t seg_code, float* c, int64_t ldc,
              int64_t m, int64_t n, int lower, int* d_err, cudaStream_t s, int reserve_sms = 0, int max_ctas = 0,
              int diag = 0);

// Segment tables (parts: 0 = hi, 1 = mid/lo of a two-way split, 2 = lo of a three-way split),
// ordered smallest terms first.
constexpr uint32_t tc_code(uint32_t pa, uint32_t pb) { return pa | (pb << 2); }
constexpr uint32_t kSegX1 = tc_code(0, 0);
// two-way split: hi*lo, lo*hi, hi*hi
constexpr uint32_t kSegX3 = tc_code(0, 1) | (tc_code(1, 0) << 4) | (tc_code(0, 0) << 8);
// three-way split: hi*lo, lo*hi, mid*mid, hi*mid, mid*hi, hi*hi (drops mid*lo, lo*mid, lo*lo)
constexpr uint32_t kSegX6 = tc_code(0, 2) | (tc_code(2, 0) << 4) | (tc_code(1, 1) << 8) | (tc_code(0, 1) << 12) |
                            (tc_code(1, 0) << 16) | (tc_code(0, 0) << 20);

}  // namespace gbllt
