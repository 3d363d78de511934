// FP64 residual R = B - A X on the BF16 tensor cores, exact to FP64 level, for the refinement of
// the mixed-precision solve (A symmetric, stored in one triangle; X, B column-major n x nrhs).
//
// The FP64 pipe of GB300 delivers about 1.1 TFLOP/s, so the FP64 residual of a 16384 x 16384
// system with 64 right-hand sides (34 GFLOP) takes about 31 ms, more than the whole tensor-core
// factorisation.  This file computes the same product with error-free splitting (the Ozaki scheme:
// Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms 59, 2012):
//
//   - every row i of A is scaled by a power of two 2^-e_i so that |a| < 1, and every column j of X
//     by 2^-f_j; the scaled values are split into S = 8 slices of BETA = 7 bits,
//         a / 2^e_i = sum_p s_p 2^(-7p),  s_1 in [-128, 128], s_p in [-64, 64] (p > 1),
//     each slice an integer, so each is exact in BF16 (8 significant bits);
//   - the product is sum over slice pairs (p, q) with p + q <= S + 1 (36 pairs; the dropped terms
//     are below 2^-63 relative to 2^(e_i + f_j)) of 2^(-7(p+q)) (S_p X_q); pairs with the same
//     weight w = p + q accumulate in one TMEM accumulator (8 of them, 64 columns each);
//   - the products of integer slices are integers, and a chunk of KC = 256 K-elements keeps every
//     partial sum of every weight below 2^24 (the largest weight sums 2^14 + 6 * 2^12 per K term),
//     so the FP32 tensor-core accumulation of a chunk is exact; after each chunk the epilogue warps
//     convert the accumulators to integers and add them into two int64 sums per output (weights
//     2-5 and 6-9, each a fixed-point number), which stay exact for n up to about 2^20;
//   - at the end, R = B - 2^(e_i + f_j) (hi 2^-35 + lo 2^-63), rounded once to FP64 (in integer
//     arithmetic: the FP64 pipe is kept for the final subtraction).
//
// oz_kernel: persistent CTAs walking a list of 128-row x 64-column output tiles, 576 threads: a TMA
// producer warp (A slice tiles through a 4-stage ring, the 8 X slice tiles of a 64-wide K block
// double-buffered, running ahead across tiles), an MMA warp (tcgen05.mma M = 128, K = 16, N = 64 to
// 256: the pairs of one A slice with up to four X slices in one instruction, 48 per K block) and 16
// epilogue warps (four per TMEM lane quadrant, 16 columns each).  The same
// kernel forms the residual (K = n, chunks of 256) and the trailing update of the FP64 factorisation
// (K = one 64-wide panel, one chunk, C -= product on the lower tiles).  Every mbarrier wait is bounded.
// A non-finite value in A or X makes the whole residual NaN, which the refinement reports as
// non-convergence, as it would with an FP64 residual.
#include <cuda_bf16.h>

#include <cstring>
#include <mutex>

#include "internal.h"
#include "tc_ptx.cuh"

namespace gbllt {

namespace {

using namespace tcptx;

constexpr int S = 8;          // slices per operand
constexpr int BETA = 7;       // bits per slice
constexpr int KB = 64;        // K elements per 128-byte row (BF16)
constexpr int KC_BLOCKS = 4;  // K blocks per exact chunk (KC = 256)
constexpr int kMaxKParts = 8;  // K ranges of the residual's K-split (at most)
constexpr int BM = 128;
constexpr int BN = 64;
constexpr int A_STAGES = 4;
constexpr int A_BYTES = BM * 128;  // 16 KB: one A slice tile
constexpr int X_BYTES = BN * 128;  // 8 KB: one X slice tile
constexpr int X_SET = S * X_BYTES;  // 64 KB: the 8 X slices of one K block
constexpr int SMEM_BYTES = A_STAGES * A_BYTES + 2 * X_SET + 1024;
constexpr int EPI_WARPS = 16;  // four per TMEM lane quadrant, 16 columns each
constexpr int THREADS = (2 + EPI_WARPS) * 32;  // 576
constexpr int TMEM_COLS = S * BN;  // 512: one 64-column accumulator per weight w = 2 .. 9

// ---- slicing ------------------------------------------------------------------------------------

// |A| maxima per row of the full symmetric matrix (bit patterns of non-negative doubles compare
// like unsigned integers), one CTA per stored 64 x 64 tile: entry (i, j) counts for rows i and j.
// flag: set when A holds a non-finite value.
template <bool UP>
__global__ void __launch_bounds__(256) oz_rowmax_kernel(const double* __restrict__ a, long long lda, long long n,
                                                        unsigned long long* __restrict__ rmax, int* __restrict__ flag) {
  __shared__ unsigned long long rm[64], cm[64];
  int ti, tj;
  lower_tile_coords(blockIdx.x, ti, tj);
  // lower storage: tile rows ti, columns tj (ti >= tj); upper: rows tj, columns ti
  const long long i0 = (long long)(UP ? tj : ti) * 64, j0 = (long long)(UP ? ti : tj) * 64;
  if (threadIdx.x < 64) {
    rm[threadIdx.x] = 0;
    cm[threadIdx.x] = 0;
  }
  __syncthreads();
  int bad = 0;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int r = idx & 63, c = idx >> 6;
    const long long i = i0 + r, j = j0 + c;
    if (i < n && j < n && (UP ? i <= j : i >= j)) {
      const double v = fabs(a[j * lda + i]);
      if (!(v <= 1.7976931348623157e308)) bad = 1;  // inf or NaN
      const unsigned long long bits = __double_as_longlong(v);
      atomicMax(&rm[r], bits);
      atomicMax(&cm[c], bits);
    }
  }
  __syncthreads();
  if (threadIdx.x < 64) {
    if (i0 + threadIdx.x < n) atomicMax(&rmax[i0 + threadIdx.x], rm[threadIdx.x]);
    if (j0 + threadIdx.x < n) atomicMax(&rmax[j0 + threadIdx.x], cm[threadIdx.x]);
  }
  if (bad) atomicOr(flag, 1);
}

// The scale exponent of a maximum m: |v| <= m < 2^e (e = 0 for m = 0).
__device__ __forceinline__ int scale_exp(double m) {
  int e = 0;
  if (m > 0.0) frexp(m, &e);
  return e;
}

// The 8 slices of v / 2^e (|v| < 2^e) in integer arithmetic on v's bit pattern (the FP64 pipe of
// GB300 is too slow to spend on this): N = round(v 2^(56 - e)), |N| < 2^56, as a 64-bit integer, then
// balanced base-128 digits taken from the bottom in 32-bit arithmetic on its two 28-bit halves,
// d = ((x + 64) mod 128) - 64 and x = (x - d) / 128, with the carry of the low half passed to the
// high half.  The seven low digits lie in [-64, 63] and the top one in [-128, 128]; sum_p d_p
// 2^(7(8-p)) = N exactly.  What falls below 2^-56 is rounded away.
__device__ __forceinline__ void split8(double v, int e, float* sl) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int E = (int)((bits >> 52) & 0x7FF);
  unsigned long long M = bits & 0xFFFFFFFFFFFFFull;
  int ex;
  if (E == 0) {
    ex = -1074;  // subnormal
  } else {
    M |= 1ull << 52;
    ex = E - 1075;
  }
  const int sh = ex + 56 - e;  // |v| = M 2^ex, N = M 2^sh
  unsigned long long U;
  if (E == 0x7FF) U = 0;  // non-finite: reported through the flag, not the slices
  else if (sh >= 0) U = M << (sh > 3 ? 3 : sh);
  else if (sh > -64) U = (M + (1ull << (-sh - 1))) >> (-sh);
  else U = 0;
  const bool neg = (bits >> 63) != 0;
  // two's-complement halves of +-U: N = hi 2^28 + lo, lo in [0, 2^28)
  const long long N = neg ? -(long long)U : (long long)U;
  int lo = (int)(N & 0xFFFFFFF);
  int hi = (int)(N >> 28);
#pragma unroll
  for (int p = S - 1; p >= 4; --p) {  // low half: digits 8, 7, 6, 5
    const int d = ((lo + 64) & 127) - 64;
    sl[p] = (float)d;
    lo = (lo - d) >> 7;
  }
  hi += lo;  // the carry out of the low half (0 or 1)
#pragma unroll
  for (int p = 3; p >= 1; --p) {
    const int d = ((hi + 64) & 127) - 64;
    sl[p] = (float)d;
    hi = (hi - d) >> 7;
  }
  sl[0] = (float)hi;
}

// Scale exponent of every row from its maximum (one thread per row).
__global__ void oz_rowexp_kernel(const unsigned long long* __restrict__ rmax, long long n, int* __restrict__ rexp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rexp[i] = scale_exp(__longlong_as_double(rmax[i]));
}

// Slices of the full symmetric A, row-major (row i holds its n entries contiguously: the K-major
// layout of the MMA's A operand), slice p at slices + p * sstride, leading dimension lds.  One CTA
// per 64 x 64 tile of the full matrix; the tile is read from the stored triangle (mirrored where
// needed) through shared memory so that reads and writes are both coalesced.
template <bool UP>
__global__ void __launch_bounds__(256) oz_slice_a_kernel(const double* __restrict__ a, long long lda, long long n,
                                                         const int* __restrict__ rexp,
                                                         __nv_bfloat16* __restrict__ slices, long long lds,
                                                         long long sstride) {
  __shared__ double tile[64][65];  // tile[r][c] = A(i0 + r, j0 + c)
  const long long i0 = (long long)blockIdx.y * 64, j0 = (long long)blockIdx.x * 64;
  // stored orientation of this tile: (i, j) with i >= j (lower) or i <= j (upper) is read directly
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    // direct entries: consecutive threads walk r (contiguous in a column of the storage)
    const int r = idx & 63, c = idx >> 6;
    const long long i = i0 + r, j = j0 + c;
    if (i < n && j < n && (UP ? i <= j : i >= j)) tile[r][c] = a[j * lda + i];
  }
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    // mirrored entries: A(i, j) = A(j, i), stored at a[i * lda + j]; consecutive threads walk c
    const int c = idx & 63, r = idx >> 6;
    const long long i = i0 + r, j = j0 + c;
    if (i < n && j < n && !(UP ? i <= j : i >= j)) tile[r][c] = a[i * lda + j];
  }
  __syncthreads();
  // each thread: 8 consecutive columns of one row, written as one 16-byte vector per slice
  for (int idx = threadIdx.x; idx < 64 * 8; idx += 256) {
    const int c8 = (idx & 7) * 8, r = idx >> 3;
    const long long i = i0 + r, j = j0 + c8;
    if (i >= n || j >= n) continue;
    const int e = rexp[i];
    if (j + 8 <= n) {
      uint32_t packed[S][4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        float lo[S], hi[S];
        split8(tile[r][c8 + 2 * h], e, lo);
        split8(tile[r][c8 + 2 * h + 1], e, hi);
#pragma unroll
        for (int p = 0; p < S; ++p) {
          const __nv_bfloat162 v2 = __floats2bfloat162_rn(lo[p], hi[p]);
          packed[p][h] = *reinterpret_cast<const uint32_t*>(&v2);
        }
      }
#pragma unroll
      for (int p = 0; p < S; ++p)
        *reinterpret_cast<uint4*>(slices + p * sstride + i * lds + j) =
            make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
    } else {
      for (int cc = 0; cc < 8 && j + cc < n; ++cc) {
        float sl[S];
        split8(tile[r][c8 + cc], e, sl);
#pragma unroll
        for (int p = 0; p < S; ++p) slices[p * sstride + i * lds + j + cc] = __float2bfloat16_rn(sl[p]);
      }
    }
  }
}

// Slices of X: one CTA per right-hand side j (column j of X, contiguous): its maximum, the scale
// exponent f_j (stored in xexp[j]), then slice q of column j at xs + q * xstride + j * ldxs.
__global__ void __launch_bounds__(256) oz_slice_x_kernel(const double* __restrict__ x, long long ldx, long long n,
                                                         __nv_bfloat16* __restrict__ xs, long long ldxs,
                                                         long long xstride, int* __restrict__ xexp,
                                                         int* __restrict__ flag) {
  __shared__ double red[256];
  const long long j = blockIdx.x;
  const double* col = x + j * ldx;
  double m = 0.0;
  int bad = 0;
  for (long long l = threadIdx.x; l < n; l += 256) {
    const double v = fabs(col[l]);
    if (!(v <= 1.7976931348623157e308)) bad = 1;
    m = fmax(m, v);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const int f = scale_exp(red[0]);
  if (threadIdx.x == 0) xexp[j] = f;
  if (bad) atomicOr(flag, 1);
  for (long long l = threadIdx.x; l < n; l += 256) {
    float sl[S];
    split8(col[l], f, sl);
#pragma unroll
    for (int q = 0; q < S; ++q) xs[q * xstride + j * ldxs + l] = __float2bfloat16_rn(sl[q]);
  }
}

}  // namespace

namespace {

// ---- the product --------------------------------------------------------------------------------

struct OzMaps {
  CUtensorMap a[S];  // slices of the M operand (rows of A, or of the panel), box 64 x 128 rows
  CUtensorMap x[S];  // slices of the N operand (columns of X, or rows of the panel), box 64 x 64 rows
};

struct OzParams {
  long long kdim;                  // K: n for the residual, the panel width for the trailing update
  long long tiles;                 // entries of the tile list
  int nrt, nct;                    // row tiles (128) and column tiles (64)
  int* err;                        // set to 1 when a bounded wait ran out
  // residual R = B - A X
  long long n, nrhs;
  const int* rexp;                 // per-row scale exponents of A
  const int* xexp;                 // per-column scale exponents of X
  const int* flag;                 // [0]: A holds a non-finite value, [1]: X does
  const double* b;
  long long ldb;
  double* r;
  long long ldr;
  // update C -= 2^scale P Q^T (lower part only in the lower mode: P = Q = L21 for a Cholesky update,
  // Q = L21 D for LDL^T; every entry of the rs x ncols rectangle in the rectangle mode)
  double* c;
  long long ldc;
  long long rs;                    // rows of the updated block
  long long ncols;                 // its columns (ncols = rs: the whole trailing lower triangle)
  const int* pexp;                 // per-row scale exponents of P (the M operand)
  const int* pexp_b;               // per-row scale exponents of Q (the N operand)
  int scale;                       // power of two applied to the product (rectangle mode)
  int nsl;                         // slices used per operand (S: FP64-exact; fewer: 7 nsl bits)
  const DevStatus* st;             // lower mode: skip the update after a failed pivot
  // residual mode with kparts > 1: K is cut into kparts ranges of whole chunks, the tile list holds
  // every (tile, range) pair, and each writes its two int64 sums per output to part
  // ([range][0 / 1][column][row]); oz_residual_sum_kernel adds them and forms R
  int kparts;
  long long* part;
};

// Kernel modes: the refinement residual R = B - A X, the trailing update C -= P Q^T on the lower
// part of a block, and the general update C -= 2^scale P Q^T of a rectangle.
constexpr int OZ_RESIDUAL = 0, OZ_LOWER = 1, OZ_RECT = 2;

// round((hi 2^28 + lo) 2^(e - 63)) to FP64, to nearest even, in integer arithmetic (the FP64 pipe
// of GB300 retires two operations per SM clock, too few for a per-element conversion); the value is
// rounded once, as ldexp(hi, -35) + ldexp(lo, -63) would round it.  Subnormal and overflowing results
// (far outside any residual or update) take the library's ldexp.
__device__ __forceinline__ double fixed_to_double(long long hi, long long lo, int e) {
  const __int128 v = ((__int128)hi << 28) + (__int128)lo;
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
  const int bl = mh ? 128 - __clzll((long long)mh) : 64 - __clzll((long long)ml);  // bit length
  int sh = bl - 53;
  unsigned long long mant;
  if (sh <= 0) {
    mant = (unsigned long long)(m << (-sh));
  } else {
    unsigned __int128 q = m >> sh;
    const unsigned __int128 rem = m - (q << sh), half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) q += 1;
    if (q >> 53) {
      q >>= 1;
      sh += 1;
    }
    mant = (unsigned long long)q;
  }
  const int biased = sh + e - 63 + 52 + 1023;  // exponent field of mant * 2^(sh + e - 63)
  if (biased <= 0 || biased >= 2047) {
    const double d = ldexp((double)(long long)mant, sh + e - 63);
    return neg ? -d : d;
  }
  const unsigned long long bits = ((unsigned long long)neg << 63) | ((unsigned long long)biased << 52) |
                                  (mant & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

// Tile t of the list: the residual walks row tiles fastest; the trailing update walks the same
// 128 x 64 grid over its rs x ncols block and skips the tiles strictly above the diagonal.
template <int MODE>
__device__ __forceinline__ bool oz_tile(const OzParams& p, long long t, long long& row0, long long& col0) {
  if (MODE == OZ_RESIDUAL && p.kparts > 1) t %= (long long)p.nrt * p.nct;
  row0 = (t % p.nrt) * BM;
  col0 = (t / p.nrt) * BN;
  if (MODE != OZ_LOWER) return true;
  return col0 < p.ncols && col0 <= row0 + BM - 1;
}

// The K blocks [kb0, kb1) of list entry t and its K range index: all of K, or in the residual's
// K-split the range t / (tiles per range), whole 256-deep chunks each.
template <int MODE>
__device__ __forceinline__ int oz_krange(const OzParams& p, long long t, int nkb, int& kb0, int& kb1) {
  kb0 = 0;
  kb1 = nkb;
  if (MODE != OZ_RESIDUAL || p.kparts <= 1) return 0;
  const int kp = (int)(t / ((long long)p.nrt * p.nct));
  const int nch = (nkb + KC_BLOCKS - 1) / KC_BLOCKS;
  const int c0 = (int)((long long)kp * nch / p.kparts), c1 = (int)((long long)(kp + 1) * nch / p.kparts);
  kb0 = c0 * KC_BLOCKS;
  kb1 = c1 * KC_BLOCKS < nkb ? c1 * KC_BLOCKS : nkb;
  return kp;
}

// Persistent: each CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...  The producer runs up to
// two K blocks (of any tile) ahead of the MMA warp, so the next tile's loads overlap this tile's
// products and epilogue; the TMEM accumulators (all 512 columns) are released chunk by chunk.
template <int MODE>
__global__ void __launch_bounds__(THREADS, 1) oz_kernel(const __grid_constant__ OzMaps maps, const OzParams p) {
  extern __shared__ uint8_t oz_smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)oz_smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* a_ring = smem;                           // A_STAGES x 16 KB
  uint8_t* x_buf = smem + A_STAGES * A_BYTES;       // 2 x (8 x 8 KB)
  __shared__ __align__(8) uint64_t afull[A_STAGES], aempty[A_STAGES];
  __shared__ __align__(8) uint64_t xfull[2], xempty[2];
  __shared__ __align__(8) uint64_t tfull, tempty;
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;

  if (MODE == OZ_LOWER && p.st->fail_col >= 0) return;  // an earlier pivot failed: nothing to update
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = (int)((p.kdim + KB - 1) / KB);

  if (threadIdx.x == 0) {
    abort_s = 0;
    for (int s = 0; s < A_STAGES; ++s) {
      mbar_init(&afull[s], 1);
      mbar_init(&aempty[s], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&xfull[i], 1);
      mbar_init(&xempty[i], 1);
    }
    mbar_init(&tfull, 1);
    mbar_init(&tempty, EPI_WARPS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer
    long long kbg = 0, it = 0, issued_a = 0, issued_x = 0;
    bool ok = true;
    for (long long t = blockIdx.x; t < p.tiles && ok && !abort_s; t += gridDim.x) {
      long long row0, col0;
      if (!oz_tile<MODE>(p, t, row0, col0)) continue;
      int kb0, kb1;
      oz_krange<MODE>(p, t, nkb, kb0, kb1);
      for (int kb = kb0; kb < kb1 && ok; ++kb, ++kbg) {
        const int xb = (int)(kbg & 1);
        if (!mbar_wait(&xempty[xb], ((uint32_t)(kbg >> 1) & 1u) ^ 1u, &abort_s)) { ok = false; break; }
        mbar_expect_tx(&xfull[xb], p.nsl * X_BYTES);
        for (int q = 0; q < p.nsl; ++q)
          tma_load_2d(x_buf + xb * X_SET + q * X_BYTES, &maps.x[q], &xfull[xb], kb * KB, (int)col0);
        issued_x = kbg + 1;
        for (int sp = 0; sp < p.nsl; ++sp, ++it) {
          const int st = (int)(it % A_STAGES);
          if (!mbar_wait(&aempty[st], ((uint32_t)(it / A_STAGES) & 1u) ^ 1u, &abort_s)) { ok = false; break; }
          mbar_expect_tx(&afull[st], A_BYTES);
          tma_load_2d(a_ring + st * A_BYTES, &maps.a[sp], &afull[st], kb * KB, (int)row0);
          issued_a = it + 1;
        }
      }
    }
    if (abort_s) {
      // let the copies this thread started land before the CTA exits (bounded)
      volatile int dummy = 0;
      for (long long i = issued_a - A_STAGES < 0 ? 0 : issued_a - A_STAGES; i < issued_a; ++i)
        mbar_wait(&afull[i % A_STAGES], (uint32_t)(i / A_STAGES) & 1u, &dummy);
      for (long long k = issued_x - 2 < 0 ? 0 : issued_x - 2; k < issued_x; ++k)
        mbar_wait(&xfull[k & 1], (uint32_t)(k >> 1) & 1u, &dummy);
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer: pairs (p, q) with p + q <= S - 1 (0-based) into accumulator w = p + q.  The X
    // slices of a K block sit back to back in shared memory (64 rows each, whole 1024-byte swizzle
    // atoms) and the accumulators of q = 0, 1, ... in consecutive TMEM columns, so one MMA with
    // N = 64 * (number of slices) covers up to four pairs of the same A slice: the A tile is read
    // once per 256 columns instead of once per 64.
    long long kbg = 0, it = 0, chunkg = 0;
    bool ok = true;
    for (long long t = blockIdx.x; t < p.tiles && ok; t += gridDim.x) {
      long long row0, col0;
      if (!oz_tile<MODE>(p, t, row0, col0)) continue;
      int kb0, kb1;
      oz_krange<MODE>(p, t, nkb, kb0, kb1);
      for (int kb = kb0; kb < kb1 && ok; ++kb, ++kbg) {
        const bool first = ((kb - kb0) % KC_BLOCKS) == 0;
        if (first && chunkg > 0) {  // the epilogue has taken the previous chunk's sums out of TMEM
          if (!mbar_wait(&tempty, (uint32_t)(chunkg - 1) & 1u, &abort_s)) { ok = false; break; }
          tc_fence_after();
        }
        const int xb = (int)(kbg & 1);
        if (!mbar_wait(&xfull[xb], (uint32_t)(kbg >> 1) & 1u, &abort_s)) { ok = false; break; }
        tc_fence_after();
        const uint32_t xs0 = smem_u32(x_buf + xb * X_SET);
        for (int sp = 0; sp < p.nsl; ++sp, ++it) {
          const int st = (int)(it % A_STAGES);
          if (!mbar_wait(&afull[st], (uint32_t)(it / A_STAGES) & 1u, &abort_s)) { ok = false; break; }
          tc_fence_after();
          const uint64_t ad = sw128_desc(smem_u32(a_ring + st * A_BYTES));
          for (int q0 = 0; q0 + sp < p.nsl; q0 += 4) {
            const int nq = p.nsl - sp - q0 < 4 ? p.nsl - sp - q0 : 4;
            const uint32_t idesc = instr_desc_mn(1u, BM, nq * BN);
            const uint64_t bd = sw128_desc(xs0 + q0 * X_BYTES);
            const uint32_t d = tmem + (uint32_t)((sp + q0) * BN);
#pragma unroll
            for (int j = 0; j < KB / 16; ++j)  // 32 bytes along K per MMA: +2 in the (addr >> 4) field
              mma<0>(d, ad + 2 * j, bd + 2 * j, idesc, (first && sp == 0 && j == 0) ? 0u : 1u);
          }
          mma_commit(&aempty[st]);
        }
        if (!ok) break;
        mma_commit(&xempty[xb]);
        if (((kb - kb0) % KC_BLOCKS) == KC_BLOCKS - 1 || kb == kb1 - 1) {
          mma_commit(&tfull);
          ++chunkg;
        }
      }
    }
  } else if (warp >= 2) {
    // ---- epilogue: per chunk, the 8 weight accumulators of this thread's row and 16 columns into
    // two int64 fixed-point sums; per tile, the FP64 result 2^(e_i + f_j) (hi 2^-35 + lo 2^-63)
    const int quad = warp & 3;                  // TMEM lane quadrant this warp may access
    const int part = (warp - 2) >> 2;           // which 16 of the 64 columns
    const int r = quad * 32 + lane;             // tile row
    long long chunkg = 0;
    bool ok = true;
    for (long long t = blockIdx.x; t < p.tiles && ok; t += gridDim.x) {
      long long row0, col0;
      if (!oz_tile<MODE>(p, t, row0, col0)) continue;
      int kb0, kb1;
      const int kp = oz_krange<MODE>(p, t, nkb, kb0, kb1);
      const int nchunks = (kb1 - kb0 + KC_BLOCKS - 1) / KC_BLOCKS;
      long long hi[16], lo[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        hi[c] = 0;
        lo[c] = 0;
      }
      for (int ch = 0; ch < nchunks; ++ch, ++chunkg) {
        if (!mbar_wait(&tfull, (uint32_t)chunkg & 1u, &abort_s)) { ok = false; break; }
        tc_fence_after();
        const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(part * 16);
#pragma unroll
        for (int w = 0; w < S; ++w) {
          if (w >= p.nsl) break;  // weights past the slices used hold nothing
          float v[16];
          tmem_ld16(base + (uint32_t)(w * BN), v);
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const long long P = (long long)__float2int_rn(v[c]);  // an exact integer below 2^24
            if (w < 4) hi[c] += P * (1ll << (BETA * (3 - w)));
            else lo[c] += P * (1ll << (BETA * (7 - w)));
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty);
      }
      if (!ok) break;
      const long long i = row0 + r;
      if (MODE == OZ_LOWER) {
        if (i < p.rs) {
          const int ei = p.pexp[i];
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const long long j = col0 + part * 16 + c;
            if (j <= i) {
              p.c[j * p.ldc + i] -= fixed_to_double(hi[c], lo[c], ei + p.pexp_b[j]);
            }
          }
        }
      } else if (MODE == OZ_RECT) {
        if (i < p.rs) {
          const int ei = p.pexp[i] + p.scale;
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const long long j = col0 + part * 16 + c;
            if (j < p.ncols) p.c[j * p.ldc + i] -= fixed_to_double(hi[c], lo[c], ei + p.pexp_b[j]);
          }
        }
      } else if (p.kparts > 1) {  // residual, one K range: its sums for oz_residual_sum_kernel
        if (i < p.n) {
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const long long j = col0 + part * 16 + c;
            if (j < p.nrhs) {
              p.part[((long long)(kp * 2) * p.nrhs + j) * p.n + i] = hi[c];
              p.part[((long long)(kp * 2 + 1) * p.nrhs + j) * p.n + i] = lo[c];
            }
          }
        }
      } else if (i < p.n) {
        const int e = p.rexp[i];
        const bool bad = (p.flag[0] | p.flag[1]) != 0;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const long long j = col0 + part * 16 + c;
          if (j < p.nrhs) {
            const double ax = fixed_to_double(hi[c], lo[c], e + p.xexp[j]);
            p.r[j * p.ldr + i] = bad ? __longlong_as_double(0x7ff8000000000000ll) : p.b[j * p.ldb + i] - ax;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && abort_s) atomicExch(p.err, 1);
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// The residual from a K-split product: the kparts ranges' int64 sums added (exactly), rounded once to
// FP64, R = B - A X (NaN everywhere when A or X held a non-finite value).
__global__ void __launch_bounds__(256) oz_residual_sum_kernel(const long long* __restrict__ part, int kparts,
                                                              long long n, long long nrhs,
                                                              const int* __restrict__ rexp,
                                                              const int* __restrict__ xexp,
                                                              const int* __restrict__ flag,
                                                              const double* __restrict__ b, long long ldb,
                                                              double* __restrict__ r, long long ldr) {
  const bool bad = (flag[0] | flag[1]) != 0;
  for (long long idx = (long long)blockIdx.x * 256 + threadIdx.x; idx < n * nrhs; idx += (long long)gridDim.x * 256) {
    const long long j = idx / n, i = idx - j * n;
    long long hi = 0, lo = 0;
    for (int kp = 0; kp < kparts; ++kp) {
      hi += part[((long long)(kp * 2) * nrhs + j) * n + i];
      lo += part[((long long)(kp * 2 + 1) * nrhs + j) * n + i];
    }
    const double ax = fixed_to_double(hi, lo, rexp[i] + xexp[j]);
    r[j * ldr + i] = bad ? __longlong_as_double(0x7ff8000000000000ll) : b[j * ldb + i] - ax;
  }
}

}  // namespace

// ---- host driver --------------------------------------------------------------------------------

namespace {

// Per-device setup, once, under a lock: the product kernels' shared-memory size and the SM count
// (the persistent grid).
int oz_prepare_device(int* sms) {
  static std::mutex mu;
  static int nsm[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return GBLLT_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!nsm[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(oz_kernel<OZ_RESIDUAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    GB_CUDA_TRY(cudaFuncSetAttribute(oz_kernel<OZ_LOWER>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    GB_CUDA_TRY(cudaFuncSetAttribute(oz_kernel<OZ_RECT>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    int v = 0;
    GB_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    nsm[dev] = v > 0 ? v : 1;
  }
  *sms = nsm[dev];
  return GBLLT_SUCCESS;
}

inline size_t oz_up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

OzakiResidual::~OzakiResidual() {
  if (buf) cudaFreeAsync(buf, stream);
}

size_t OzakiResidual::bytes(int64_t n, int64_t nrhs) {
  const int64_t lds = (n + 7) / 8 * 8;  // 16-byte row pitch for TMA
  return oz_up256((size_t)S * n * lds * 2) + oz_up256((size_t)S * nrhs * lds * 2) + oz_up256((size_t)n * 8) +
         oz_up256((size_t)n * 4) + oz_up256((size_t)nrhs * 4) + 256 + oz_up256((size_t)kMaxKParts * 2 * nrhs * n * 8) +
         256;
}

int OzakiResidual::reserve(int64_t n_, int64_t nrhs_, cudaStream_t s) {
  if (buf) return GBLLT_SUCCESS;
  n = n_;
  nrhs = nrhs_;
  stream = s;
  lds = (n + 7) / 8 * 8;
  if (dev_malloc_async(&buf, bytes(n, nrhs), s) != cudaSuccess) {
    cudaGetLastError();
    buf = nullptr;
    set_error_message("cudaMallocAsync failed (tensor-core residual slices)");
    return GBLLT_ERR_ALLOC;
  }
  return GBLLT_SUCCESS;
}

int OzakiResidual::setup(bool upper, int64_t n_, int64_t nrhs_, const double* a, int64_t lda, cudaStream_t s) {
  int sms = 0;
  int rc = oz_prepare_device(&sms);
  if (rc) return rc;
  if (!buf) {
    if ((rc = reserve(n_, nrhs_, s))) return rc;
  } else if (n_ != n || nrhs_ != nrhs) {
    return GBLLT_ERR_INTERNAL;
  }
  char* q = (char*)buf;
  aslices = q;
  q += oz_up256((size_t)S * n * lds * 2);
  xslices = q;
  q += oz_up256((size_t)S * nrhs * lds * 2);
  rmax = (unsigned long long*)q;
  q += oz_up256((size_t)n * 8);
  rexp = (int*)q;
  q += oz_up256((size_t)n * 4);
  xexp = (int*)q;
  q += oz_up256((size_t)nrhs * 4);
  flags = (int*)q;  // [0] A non-finite, [1] X non-finite, [2] timeout
  q += 256;
  part = (long long*)q;  // the K-split's sums: kMaxKParts x 2 x nrhs x n
  GB_CUDA_TRY(cudaMemsetAsync(rmax, 0, (size_t)n * 8, s));
  GB_CUDA_TRY(cudaMemsetAsync(flags, 0, 16, s));
  const int64_t t = ceil_div(n, 64);
  static const std::string ks = "residual_slices_a";
  {
    ProfScope ps(ks.c_str(), s, 0.0, (double)n * n * 8.0 + (double)S * n * n * 2.0);
    if (upper) oz_rowmax_kernel<true><<<(unsigned)(t * (t + 1) / 2), 256, 0, s>>>(a, lda, n, rmax, flags);
    else oz_rowmax_kernel<false><<<(unsigned)(t * (t + 1) / 2), 256, 0, s>>>(a, lda, n, rmax, flags);
    oz_rowexp_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(rmax, n, rexp);
    const dim3 g((unsigned)t, (unsigned)t);
    __nv_bfloat16* as = (__nv_bfloat16*)aslices;
    if (upper) oz_slice_a_kernel<true><<<g, 256, 0, s>>>(a, lda, n, rexp, as, lds, (long long)n * lds);
    else oz_slice_a_kernel<false><<<g, 256, 0, s>>>(a, lda, n, rexp, as, lds, (long long)n * lds);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

int OzakiResidual::residual(const double* x, int64_t ldx, const double* b, int64_t ldb, double* r, int64_t ldr,
                            cudaStream_t s) {
  if (!buf) return GBLLT_ERR_INTERNAL;
  OzMaps maps;
  const __nv_bfloat16* as = (const __nv_bfloat16*)aslices;
  __nv_bfloat16* xs = (__nv_bfloat16*)xslices;
  for (int i = 0; i < S; ++i) {
    if (!make_map_2d(&maps.a[i], as + (size_t)i * n * lds, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, n, n, lds, KB, BM) ||
        !make_map_2d(&maps.x[i], xs + (size_t)i * nrhs * lds, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nrhs, n, lds, KB,
                     BN)) {
      set_error_message("cuTensorMapEncodeTiled failed (tensor-core residual)");
      return GBLLT_ERR_INTERNAL;
    }
  }
  GB_CUDA_TRY(cudaMemsetAsync(flags + 1, 0, 8, s));
  static const std::string kx = "residual_slices_x";
  static const std::string kg = "residual_tc";
  {
    ProfScope ps(kx.c_str(), s, 0.0, (double)n * nrhs * (8.0 + S * 2.0));
    oz_slice_x_kernel<<<(unsigned)nrhs, 256, 0, s>>>(x, ldx, n, xs, lds, (long long)nrhs * lds, xexp, flags);
  }
  int sms = 0;
  int rc = oz_prepare_device(&sms);
  if (rc) return rc;
  OzParams p;
  memset(&p, 0, sizeof p);
  p.nsl = S;
  p.kdim = n;
  p.nrt = (int)ceil_div(n, BM);
  p.nct = (int)ceil_div(nrhs, BN);
  p.tiles = (long long)p.nrt * p.nct;
  p.n = n;
  p.nrhs = nrhs;
  p.rexp = rexp;
  p.xexp = xexp;
  p.flag = flags;
  p.b = b;
  p.ldb = ldb;
  p.r = r;
  p.ldr = ldr;
  p.err = flags + 2;
  // With fewer tiles than a few per SM the last wave of the tile list runs part-empty (n = 32768,
  // 64 RHS: 256 tiles on 152 SMs fill 84 % of two waves).  K is then cut into kparts ranges of whole
  // chunks, at least 4 chunks each, so that the (tile, range) list fills its waves to >= 95 %; the
  // ranges' exact int64 sums are added by a second kernel.
  const long long base_tiles = p.tiles;
  const int nch = (int)ceil_div(ceil_div(n, KB), KC_BLOCKS);
  int kparts = 1;
  {
    auto fill = [&](int kp) {
      const long long u = base_tiles * kp, waves = (u + sms - 1) / sms;
      return (double)u / (double)(waves * sms);
    };
    double best = fill(1);
    for (int kp = 2; kp <= kMaxKParts && nch / kp >= 4 && best < 0.95; ++kp)
      if (fill(kp) > best + 0.02) {
        best = fill(kp);
        kparts = kp;
      }
  }
  p.kparts = kparts;
  p.part = part;
  p.tiles = base_tiles * kparts;
  const unsigned grid = (unsigned)(p.tiles < sms ? p.tiles : sms);
  {
    // algorithmic work: the FP64 product 2 n^2 nrhs; bytes: the 8 A slices read once per column tile,
    // X slices, B read and R written
    ProfScope ps(kg.c_str(), s, 2.0 * n * n * nrhs,
                 (double)S * n * n * 2.0 * p.nct + (double)S * n * nrhs * 2.0 + 2.0 * n * nrhs * 8.0);
    oz_kernel<OZ_RESIDUAL><<<grid, THREADS, SMEM_BYTES, s>>>(maps, p);
  }
  GB_CUDA_TRY(cudaGetLastError());
  if (kparts > 1) {
    static const std::string kr = "residual_sum";
    ProfScope ps(kr.c_str(), s, 0.0, (double)kparts * 2 * n * nrhs * 8.0 + 2.0 * n * nrhs * 8.0);
    const long long tot = n * nrhs;
    const unsigned g = (unsigned)std::min<long long>((tot + 255) / 256, 8LL * sms);
    oz_residual_sum_kernel<<<g, 256, 0, s>>>(part, kparts, n, nrhs, rexp, xexp, flags, b, ldb, r, ldr);
    GB_CUDA_TRY(cudaGetLastError());
  }
  return GBLLT_SUCCESS;
}

int OzakiResidual::timeout_flag_into(int* host_flag, cudaStream_t s) const {
  GB_CUDA_TRY(cudaMemcpyAsync(host_flag, flags + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
  return GBLLT_SUCCESS;
}

}  // namespace gbllt

// ---- the trailing update of the FP64 factorisation on the tensor cores ------------------------
//
// A22 -= L21 L21^T (lower tiles), L21 the rs x 64 panel below the diagonal block: the same
// error-free slicing, with one exponent per row of L21 (its maximum), so the product of rows i and j
// carries 2^(e_i + e_j).  The depth is one panel (64), so a single exact FP32 chunk holds every
// weight (at most 64 * 2.5 * 2^14 < 2^22) and the epilogue rounds once into FP64.

namespace gbllt {

namespace {

constexpr int PK = 64;  // sub-panel width (the diagonal-block size)

// Slices of the panel L21 (rs x bs, column-major at l21 with leading dimension lda) as K-major rows of
// w >= bs elements (zero past bs): row i of slice q at slices + q * sstride + i * w; pexp[i] = the
// scale exponent of row i (its maximum over the panel).
__global__ void __launch_bounds__(128) oz_panel_slice_kernel(const double* __restrict__ l21, long long lda,
                                                             long long rs, int bs, int w,
                                                             __nv_bfloat16* __restrict__ slices, long long sstride,
                                                             int* __restrict__ pexp) {
  const long long i = (long long)blockIdx.x * 128 + threadIdx.x;
  if (i >= rs) return;
  // the maximum of |v| on bit patterns (integer pipe): non-negative doubles order like integers
  unsigned long long mb = 0;
#pragma unroll 8
  for (int p = 0; p < bs; ++p) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(l21[(long long)p * lda + i]) & ~(1ull << 63);
    mb = b > mb ? b : mb;
  }
  const int e = scale_exp(__longlong_as_double((long long)mb));
  pexp[i] = e;
#pragma unroll 1
  for (int p0 = 0; p0 < w; p0 += 8) {
    uint32_t packed[S][4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int pa = p0 + 2 * h, pb = pa + 1;
      float lo[S], hi[S];
      split8(pa < bs ? l21[(long long)pa * lda + i] : 0.0, e, lo);
      split8(pb < bs ? l21[(long long)pb * lda + i] : 0.0, e, hi);
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const __nv_bfloat162 v2 = __floats2bfloat162_rn(lo[q], hi[q]);
        packed[q][h] = *reinterpret_cast<const uint32_t*>(&v2);
      }
    }
#pragma unroll
    for (int q = 0; q < S; ++q)
      *reinterpret_cast<uint4*>(slices + q * sstride + i * w + p0) =
          make_uint4(packed[q][0], packed[q][1], packed[q][2], packed[q][3]);
  }
}

}  // namespace

OzakiSyrk::~OzakiSyrk() {
  release_maps();
  if (buf) cudaFreeAsync(buf, stream);
}

int OzakiSyrk::init(int64_t nmax_, cudaStream_t s, bool two_sided) {
  int rc = oz_prepare_device(&sms);
  if (rc) return rc;
  nmax = nmax_;
  stream = s;
  // [slices of a 64-wide sub-panel | their exponents | slices of a 256-wide panel | their exponents
  //  | (two_sided) slices of a second 64-wide operand | their exponents]
  const size_t s64 = oz_up256((size_t)S * nmax * PK * 2), s256 = oz_up256((size_t)S * nmax * kWide * 2),
               e = oz_up256((size_t)nmax * 4);
  if (dev_malloc_async(&buf, s64 + e + s256 + e + (two_sided ? s64 + e : 0), s) != cudaSuccess) {
    cudaGetLastError();
    buf = nullptr;
    return GBLLT_ERR_ALLOC;
  }
  slices = buf;
  pexp = (int*)((char*)buf + s64);
  slices_w = (char*)buf + s64 + e;
  pexp_w = (int*)((char*)buf + s64 + e + s256);
  if (two_sided) {
    slices_b = (char*)buf + s64 + e + s256 + e;
    pexp_b = (int*)((char*)buf + s64 + e + s256 + e + s64);
  }
  maps = new OzMaps[3];
  OzMaps* m = (OzMaps*)maps;
  const __nv_bfloat16* sl = (const __nv_bfloat16*)slices;
  const __nv_bfloat16* sw = (const __nv_bfloat16*)slices_w;
  const __nv_bfloat16* sb = (const __nv_bfloat16*)slices_b;
  for (int q = 0; q < S; ++q) {
    const __nv_bfloat16* b64 = sl + (size_t)q * nmax * PK;
    const __nv_bfloat16* b256 = sw + (size_t)q * nmax * kWide;
    if (!make_map_2d(&m[0].a[q], b64, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nmax, PK, PK, KB, BM) ||
        !make_map_2d(&m[0].x[q], b64, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nmax, PK, PK, KB, BN) ||
        !make_map_2d(&m[1].a[q], b256, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nmax, kWide, kWide, KB, BM) ||
        !make_map_2d(&m[1].x[q], b256, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nmax, kWide, kWide, KB, BN) ||
        (two_sided && (!make_map_2d(&m[2].a[q], b64, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, nmax, PK, PK, KB, BM) ||
                       !make_map_2d(&m[2].x[q], sb + (size_t)q * nmax * PK, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                    nmax, PK, PK, KB, BN)))) {
      set_error_message("cuTensorMapEncodeTiled failed (tensor-core trailing update)");
      return GBLLT_ERR_INTERNAL;
    }
  }
  return GBLLT_SUCCESS;
}

void OzakiSyrk::release_maps() {
  delete[](OzMaps*) maps;
  maps = nullptr;
}

// C -= L21 L21^T on the rs x ncols block at (k0 + pw, k0 + pw), L21 = the rs x pw panel below the
// panel's diagonal block at (k0, k0); pw <= 64 uses the 64-wide slices, pw <= 256 the wide ones.
int OzakiSyrk::update(double* a, int64_t lda, int64_t k0, int pw, int64_t rs, int64_t ncols, DevStatus* st,
                      cudaStream_t s) {
  if (rs <= 0 || ncols <= 0) return GBLLT_SUCCESS;
  if (!buf || !maps || rs > nmax || pw > kWide) return GBLLT_ERR_INTERNAL;
  const bool wide = pw > PK;
  const int w = wide ? kWide : PK;
  static const std::string kp = "panel_slices_f64";
  static const std::string ks = "syrk_tc_f64";
  const double* l21 = a + k0 * lda + k0 + pw;
  __nv_bfloat16* sl = (__nv_bfloat16*)(wide ? slices_w : slices);
  int* ex = wide ? pexp_w : pexp;
  {
    ProfScope ps(kp.c_str(), s, 0.0, (double)rs * pw * 8.0 + (double)S * rs * w * 2.0);
    oz_panel_slice_kernel<<<(unsigned)ceil_div(rs, 128), 128, 0, s>>>(l21, lda, rs, pw, w, sl, (long long)nmax * w,
                                                                     ex);
  }
  OzParams p;
  memset(&p, 0, sizeof p);
  p.nsl = S;
  p.kdim = w;
  p.nrt = (int)ceil_div(rs, BM);
  p.nct = (int)ceil_div(ncols, BN);
  p.tiles = (long long)p.nrt * p.nct;
  p.c = a + (k0 + pw) * lda + k0 + pw;
  p.ldc = lda;
  p.rs = rs;
  p.ncols = ncols;
  p.pexp = ex;
  p.pexp_b = ex;
  p.st = st;
  p.err = &st->timeout;
  const unsigned grid = (unsigned)(p.tiles < sms ? p.tiles : sms);
  {
    // algorithmic work: the FP64 update of the block's lower part, 2 pw flops per entry
    const double c = (double)(ncols < rs ? ncols : rs);
    const double entries = c * (double)rs - c * (c - 1) / 2.0;
    ProfScope ps(ks.c_str(), s, 2.0 * entries * pw, 2.0 * entries * 8.0 + (double)S * rs * w * 2.0);
    oz_kernel<OZ_LOWER><<<grid, THREADS, SMEM_BYTES, s>>>(((const OzMaps*)maps)[wide ? 1 : 0], p);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

// C -= P Q^T on the lower part of the rs x rs block at (k0 + pw, k0 + pw): P = the rs x pw panel below
// the diagonal block at (k0, k0) of a, Q = the rs x pw array at q (leading dimension ldq); pw <= 64.
// The LDL^T update, Q = L21 D: both operands are sliced, each with its own row exponents.
int OzakiSyrk::update_pq(double* a, int64_t lda, int64_t k0, int pw, int64_t rs, const double* q, int64_t ldq,
                         DevStatus* st, cudaStream_t s) {
  if (rs <= 0) return GBLLT_SUCCESS;
  if (!buf || !maps || !slices_b || rs > nmax || pw > PK) return GBLLT_ERR_INTERNAL;
  static const std::string kp = "panel_slices_f64";
  static const std::string ks = "syrk_tc_f64";
  const double* l21 = a + k0 * lda + k0 + pw;
  {
    ProfScope ps(kp.c_str(), s, 0.0, 2.0 * ((double)rs * pw * 8.0 + (double)S * rs * PK * 2.0));
    oz_panel_slice_kernel<<<(unsigned)ceil_div(rs, 128), 128, 0, s>>>(l21, lda, rs, pw, PK, (__nv_bfloat16*)slices,
                                                                     (long long)nmax * PK, pexp);
    oz_panel_slice_kernel<<<(unsigned)ceil_div(rs, 128), 128, 0, s>>>(q, ldq, rs, pw, PK, (__nv_bfloat16*)slices_b,
                                                                     (long long)nmax * PK, pexp_b);
  }
  OzParams p;
  memset(&p, 0, sizeof p);
  p.nsl = S;
  p.kdim = PK;
  p.nrt = (int)ceil_div(rs, BM);
  p.nct = (int)ceil_div(rs, BN);
  p.tiles = (long long)p.nrt * p.nct;
  p.c = a + (k0 + pw) * lda + k0 + pw;
  p.ldc = lda;
  p.rs = rs;
  p.ncols = rs;
  p.pexp = pexp;
  p.pexp_b = pexp_b;
  p.st = st;
  p.err = &st->timeout;
  const unsigned grid = (unsigned)(p.tiles < sms ? p.tiles : sms);
  {
    const double entries = (double)rs * (rs + 1) / 2.0;
    ProfScope ps(ks.c_str(), s, 2.0 * entries * pw, 2.0 * entries * 8.0 + 2.0 * S * rs * PK * 2.0);
    oz_kernel<OZ_LOWER><<<grid, THREADS, SMEM_BYTES, s>>>(((const OzMaps*)maps)[2], p);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace gbllt

// ---- the general FP64-exact product C -= 2^scale P Q^T of a rectangle ----------------------------
//
// The blocked triangular solves and the blocked adjoint are made of products of panels with
// rectangles.  Both operands are sliced like the residual's (one exponent per row, its maximum over
// k), each from any strided layout, and the product runs in the kernel's rectangle mode: exact
// 256-deep FP32 chunks, int64 combination across chunks, one rounding into FP64.

namespace gbllt {

namespace {

// Slices of a rows x k operand whose element (i, kk) lies at src[i * rstride + kk * kstride], as
// K-major rows of w >= k elements (zero past k): row i of slice q at slices + q * sstride + i * w;
// pexp[i] = the scale exponent of row i.  One thread per row; with kstride = 1 each thread reads its
// row contiguously, with rstride = 1 a warp reads 32 consecutive rows of each column.
__global__ void __launch_bounds__(128) oz_rows_slice_kernel(const double* __restrict__ src, long long rstride,
                                                            long long kstride, long long rows, long long k, long long w,
                                                            __nv_bfloat16* __restrict__ slices, long long sstride,
                                                            int* __restrict__ pexp) {
  const long long i = (long long)blockIdx.x * 128 + threadIdx.x;
  if (i >= rows) return;
  const double* row = src + i * rstride;
  unsigned long long mb = 0;
  for (long long kk = 0; kk < k; ++kk) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(row[kk * kstride]) & ~(1ull << 63);
    mb = b > mb ? b : mb;
  }
  const int e = scale_exp(__longlong_as_double((long long)mb));
  pexp[i] = e;
#pragma unroll 1
  for (long long p0 = 0; p0 < w; p0 += 8) {
    uint32_t packed[S][4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const long long pa = p0 + 2 * h, pb = pa + 1;
      float lo[S], hi[S];
      split8(pa < k ? row[pa * kstride] : 0.0, e, lo);
      split8(pb < k ? row[pb * kstride] : 0.0, e, hi);
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const __nv_bfloat162 v2 = __floats2bfloat162_rn(lo[q], hi[q]);
        packed[q][h] = *reinterpret_cast<const uint32_t*>(&v2);
      }
    }
#pragma unroll
    for (int q = 0; q < S; ++q)
      *reinterpret_cast<uint4*>(slices + q * sstride + i * w + p0) =
          make_uint4(packed[q][0], packed[q][1], packed[q][2], packed[q][3]);
  }
}

// The same slices for an operand whose rows are contiguous (kstride 1): one warp per row, lanes
// along k, so that the reads (8 consecutive values per lane) and the 16-byte slice stores are
// coalesced.  Four rows per warp, eight warps per CTA.
__global__ void __launch_bounds__(256) oz_rows_slice_contig_kernel(const double* __restrict__ src, long long rstride,
                                                                   long long rows, long long k, long long w,
                                                                   __nv_bfloat16* __restrict__ slices,
                                                                   long long sstride, int* __restrict__ pexp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int rr = 0; rr < 4; ++rr) {
    const long long i = (long long)blockIdx.x * 32 + warp * 4 + rr;
    if (i >= rows) return;
    const double* row = src + i * rstride;
    unsigned long long mb = 0;
    for (long long kk = lane; kk < k; kk += 32) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(row[kk]) & ~(1ull << 63);
      mb = b > mb ? b : mb;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xffffffffu, mb, o);
      mb = other > mb ? other : mb;
    }
    const int e = scale_exp(__longlong_as_double((long long)mb));
    if (lane == 0) pexp[i] = e;
    for (long long p0 = (long long)lane * 8; p0 < w; p0 += 256) {
      uint32_t packed[S][4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const long long pa = p0 + 2 * h, pb = pa + 1;
        float lo[S], hi[S];
        split8(pa < k ? row[pa] : 0.0, e, lo);
        split8(pb < k ? row[pb] : 0.0, e, hi);
#pragma unroll
        for (int q = 0; q < S; ++q) {
          const __nv_bfloat162 v2 = __floats2bfloat162_rn(lo[q], hi[q]);
          packed[q][h] = *reinterpret_cast<const uint32_t*>(&v2);
        }
      }
#pragma unroll
      for (int q = 0; q < S; ++q)
        *reinterpret_cast<uint4*>(slices + q * sstride + i * w + p0) =
            make_uint4(packed[q][0], packed[q][1], packed[q][2], packed[q][3]);
    }
  }
}

// A column-major operand (rstride 1) in two passes spread over both dimensions: the row maxima by
// 256-column chunks (atomicMax on the bit patterns of |v|, which order like the values), then the
// slices of 64-column blocks, one thread per row and block.
__global__ void __launch_bounds__(256) oz_colmajor_max_kernel(const double* __restrict__ src, long long kstride,
                                                              long long rows, long long k,
                                                              unsigned long long* __restrict__ rmax) {
  const long long i = (long long)blockIdx.x * 256 + threadIdx.x;
  if (i >= rows) return;
  const long long k0 = (long long)blockIdx.y * 256, k1 = k0 + 256 < k ? k0 + 256 : k;
  unsigned long long mb = 0;
  for (long long kk = k0; kk < k1; ++kk) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(src[i + kk * kstride]) & ~(1ull << 63);
    mb = b > mb ? b : mb;
  }
  atomicMax(rmax + i, mb);
}

__global__ void __launch_bounds__(128) oz_colmajor_slice_kernel(const double* __restrict__ src, long long kstride,
                                                                long long rows, long long k, long long w,
                                                                const unsigned long long* __restrict__ rmax,
                                                                __nv_bfloat16* __restrict__ slices, long long sstride,
                                                                int* __restrict__ pexp) {
  const long long i = (long long)blockIdx.x * 128 + threadIdx.x;
  if (i >= rows) return;
  const int e = scale_exp(__longlong_as_double((long long)rmax[i]));
  if (blockIdx.y == 0) pexp[i] = e;
  const long long pbeg = (long long)blockIdx.y * 64;
#pragma unroll 1
  for (long long p0 = pbeg; p0 < pbeg + 64 && p0 < w; p0 += 8) {
    uint32_t packed[S][4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const long long pa = p0 + 2 * h, pb = pa + 1;
      float lo[S], hi[S];
      split8(pa < k ? src[i + pa * kstride] : 0.0, e, lo);
      split8(pb < k ? src[i + pb * kstride] : 0.0, e, hi);
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const __nv_bfloat162 v2 = __floats2bfloat162_rn(lo[q], hi[q]);
        packed[q][h] = *reinterpret_cast<const uint32_t*>(&v2);
      }
    }
#pragma unroll
    for (int q = 0; q < S; ++q)
      *reinterpret_cast<uint4*>(slices + q * sstride + i * w + p0) =
          make_uint4(packed[q][0], packed[q][1], packed[q][2], packed[q][3]);
  }
}

// Slices of one operand: the row-contiguous kernel when kstride is 1, the two-pass column-major one
// when rstride is 1 (rmax: rows words of scratch), else one thread per row.
int oz_slice_rows(const double* src, long long rstride, long long kstride, long long rows, long long k, long long w,
                  __nv_bfloat16* slices, long long sstride, int* pexp, unsigned long long* rmax, cudaStream_t s) {
  if (kstride == 1) {
    oz_rows_slice_contig_kernel<<<(unsigned)ceil_div(rows, 32), 256, 0, s>>>(src, rstride, rows, k, w, slices, sstride,
                                                                           pexp);
  } else if (rstride == 1 && rmax) {
    GB_CUDA_TRY(cudaMemsetAsync(rmax, 0, (size_t)rows * 8, s));
    oz_colmajor_max_kernel<<<dim3((unsigned)ceil_div(rows, 256), (unsigned)ceil_div(k, 256)), 256, 0, s>>>(
        src, kstride, rows, k, rmax);
    oz_colmajor_slice_kernel<<<dim3((unsigned)ceil_div(rows, 128), (unsigned)(w / 64)), 128, 0, s>>>(
        src, kstride, rows, k, w, rmax, slices, sstride, pexp);
  } else {
    oz_rows_slice_kernel<<<(unsigned)ceil_div(rows, 128), 128, 0, s>>>(src, rstride, kstride, rows, k, w, slices,
                                                                      sstride, pexp);
  }
  return GBLLT_SUCCESS;
}

inline int64_t oz_kpad(int64_t k) { return (k + KB - 1) / KB * KB; }

}  // namespace

size_t OzakiGemm::bytes(int64_t mmax, int64_t nmax, int64_t kmax) {
  const size_t w = (size_t)oz_kpad(kmax);
  return oz_up256((size_t)S * mmax * w * 2) + oz_up256((size_t)S * nmax * w * 2) + oz_up256((size_t)mmax * 4) +
         oz_up256((size_t)nmax * 4) + oz_up256((size_t)(mmax > nmax ? mmax : nmax) * 8);
}

int OzakiGemm::attach(void* ws, int64_t mmax_, int64_t nmax_, int64_t kmax_) {
  int rc = oz_prepare_device(&sms);
  if (rc) return rc;
  mmax = mmax_;
  nmax = nmax_;
  kmax = kmax_;
  const size_t w = (size_t)oz_kpad(kmax);
  char* q = (char*)ws;
  pslices = q;
  q += oz_up256((size_t)S * mmax * w * 2);
  qslices = q;
  q += oz_up256((size_t)S * nmax * w * 2);
  pexp = (int*)q;
  q += oz_up256((size_t)mmax * 4);
  qexp = (int*)q;
  q += oz_up256((size_t)nmax * 4);
  rmax = (unsigned long long*)q;
  return GBLLT_SUCCESS;
}

int OzakiGemm::run(double* c, int64_t ldc, int64_t m, int64_t n, int64_t k, const double* pa, int64_t p_rs,
                   int64_t p_ks, const double* qa, int64_t q_rs, int64_t q_ks, int scale, int* err, cudaStream_t s,
                   int nsl) {
  if (m <= 0 || n <= 0 || k <= 0) return GBLLT_SUCCESS;
  if (!pslices || m > mmax || n > nmax || k > kmax || nsl < 1 || nsl > S) return GBLLT_ERR_INTERNAL;
  static const std::string kp = "gemm_slices_f64";
  static const std::string kg = "gemm_tc_f64";
  static const std::string kg28 = "gemm_tc_28bit";
  const int64_t w = oz_kpad(k);
  __nv_bfloat16* ps = (__nv_bfloat16*)pslices;
  __nv_bfloat16* qs = (__nv_bfloat16*)qslices;
  {
    ProfScope pr(kp.c_str(), s, 0.0, (double)(m + n) * k * 8.0 + (double)S * (m + n) * w * 2.0);
    int rc = oz_slice_rows(pa, p_rs, p_ks, m, k, w, ps, (long long)m * w, pexp, rmax, s);
    if (!rc) rc = oz_slice_rows(qa, q_rs, q_ks, n, k, w, qs, (long long)n * w, qexp, rmax, s);
    if (rc) return rc;
  }
  OzMaps maps;
  for (int q = 0; q < S; ++q) {
    if (!make_map_2d(&maps.a[q], ps + (size_t)q * m * w, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, m, w, w, KB, BM) ||
        !make_map_2d(&maps.x[q], qs + (size_t)q * n * w, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, n, w, w, KB, BN)) {
      set_error_message("cuTensorMapEncodeTiled failed (tensor-core FP64 product)");
      return GBLLT_ERR_INTERNAL;
    }
  }
  OzParams p;
  memset(&p, 0, sizeof p);
  p.nsl = S;
  p.kdim = k;
  p.nrt = (int)ceil_div(m, BM);
  p.nct = (int)ceil_div(n, BN);
  p.tiles = (long long)p.nrt * p.nct;
  p.c = c;
  p.ldc = ldc;
  p.rs = m;
  p.ncols = n;
  p.pexp = pexp;
  p.pexp_b = qexp;
  p.scale = scale;
  p.nsl = nsl;
  p.err = err;
  const unsigned grid = (unsigned)(p.tiles < sms ? p.tiles : sms);
  {
    ProfScope pr(nsl == S ? kg.c_str() : kg28.c_str(), s, 2.0 * m * n * k,
                 2.0 * m * n * 8.0 + (double)nsl * (m + n) * w * 2.0);
    oz_kernel<OZ_RECT><<<grid, THREADS, SMEM_BYTES, s>>>(maps, p);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace gbllt
