// FP32-accurate products on the warp-level tensor-core path (mma.sync, BF16 operands, FP32
// accumulation): each FP32 operand is split into three BF16 parts, x = x0 + x1 + x2 with 8
// significant bits each (24 bits: exact for normal FP32 values), and the six part products with
// p + q <= 2 are accumulated, the small ones first.  The dropped three are below 2^-24 of the
// product.
//
// The tensor cores' FP32 accumulation truncates.  Every user of these helpers starts a fresh
// accumulator for each 64-deep product and adds it to a running sum, if any, with an ordinary FP32
// add: accumulating hundreds of products into one long running sum on the tensor cores biases it.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace gbllt {

// x0, x1 (a pair of FP32 values, x0 in the low half) as three packed BF16x2 parts, rounded to
// nearest one after the other: part[0] = rn(x), part[1] = rn(x - part[0]), ...
__device__ __forceinline__ void split3_bf16x2(float x0, float x1, uint32_t* part) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(x0, x1);
    part[i] = *reinterpret_cast<const uint32_t*>(&v);
    x0 -= __low2float(v);
    x1 -= __high2float(v);
  }
}

// c (m16n8 FP32 fragment) += A (m16k16 BF16 fragment a0..a3) B (k16n8 BF16 fragment b0, b1).
// Fragment layouts (g = lane / 4, t = lane % 4): a0 = (row g, k 2t..2t+1), a1 = (row g + 8, k
// 2t..), a2 = (row g, k 2t+8..), a3 = (row g + 8, k 2t+8..); b0 = (k 2t..2t+1, col g), b1 = (k
// 2t+8.., col g); c[i] = (row g + 8 (i / 2), col 2t + i % 2).
__device__ __forceinline__ void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// The six split products of one k16 step: ap[i][p] is part p of A fragment register i, b0p / b1p
// the parts of the two B registers.
__device__ __forceinline__ void mma_split6(float* c, const uint32_t (*ap)[3], const uint32_t* b0p,
                                           const uint32_t* b1p) {
  mma_bf16(c, ap[0][2], ap[1][2], ap[2][2], ap[3][2], b0p[0], b1p[0]);
  mma_bf16(c, ap[0][1], ap[1][1], ap[2][1], ap[3][1], b0p[1], b1p[1]);
  mma_bf16(c, ap[0][0], ap[1][0], ap[2][0], ap[3][0], b0p[2], b1p[2]);
  mma_bf16(c, ap[0][1], ap[1][1], ap[2][1], ap[3][1], b0p[0], b1p[0]);
  mma_bf16(c, ap[0][0], ap[1][0], ap[2][0], ap[3][0], b0p[1], b1p[1]);
  mma_bf16(c, ap[0][0], ap[1][0], ap[2][0], ap[3][0], b0p[0], b1p[0]);
}

}  // namespace gbllt
