// Tensor-core (tcgen05) trailing-update interface.
#pragma once
#include "internal.h"

namespace gbllt {

// A K-major operand: `rows` rows of `k` elements, `ld` elements apart (ld * element size a multiple
// of 16 bytes, base 16-byte aligned).  `lo` is the second half of a split operand (may be null when
// no segment reads it).  Row `row0` of the operand lines up with row/column 0 of C.
struct TcOperand {
  const void* hi;
  const void* lo;
  int64_t rows;
  int64_t k;
  int64_t ld;
  int64_t row0;
};

// Element kinds of the operands.
constexpr int kTcBF16 = 0;
constexpr int kTcTF32 = 1;

// C (m x n fp32, column-major, ldc) -= sum over nseg segments of A_s B_s^T (lower tiles and
// entries only when `lower`); segment s reads A "lo" when bit 2s of seg_mask is set and B "lo"
// when bit 2s+1 is set.  d_err receives 1 if a bounded wait ran out.
int tc_update(const TcOperand& a, const TcOperand& b, int kind, int nseg, uint32_t seg_mask, float* c, int64_t ldc,
              int64_t m, int64_t n, bool lower, int* d_err, cudaStream_t s);

}  // namespace gbllt
