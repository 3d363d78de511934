// Single-pass blocked triangular sweeps for the solve L L^T X = B (LLT::_solve_impl_transposed,
// Eigen/src/Cholesky/LLT.h:490-498; TriangularSolverMatrix.h:38-184 / TriangularSolverVector.h:30-142).
//
// One kernel per sweep.  Row blocks of 64 are taken in ticket order from an atomic counter, so a
// CTA only ever waits on blocks whose CTAs started before it (no deadlock whatever the residency).
// CTA I (forward: Y_I = L_II^{-1} (B_I - sum_{J<I} L_IJ Y_J)):
//   - loads each off-diagonal 64 x 64 tile of L into shared memory with coalesced loads (the
//     loads do not depend on other blocks, so most CTAs stream L at HBM speed);
//   - waits for block J's flag (bounded: 2 s, then an error word is set and the CTA stops), reads
//     Y_J through L2 (ld.global.cg) and accumulates the tile product;
//   - applies the pre-inverted diagonal triangle (a 64 x 64 product instead of a 64-step
//     substitution on the critical path), stores Y_I, fences, and raises its flag.
// The backward sweep runs the same scheme on L^T from the last block up.  Right-hand sides are
// split into chunks of 16 that run as independent chains in the same launch (grid.y), so the FP64
// work of the last row blocks is spread over several SMs.  That is the FP64 sweep (sweep_kernel);
// the FP32 sweep (sweep_ll_kernel, below) shortens each link of the chain further.
//
// The diagonal inverses come from trinv_kernel (one CTA per block, column-wise substitution).
//
// The same sweeps solve with the factor of LDL^T (LDLT::_solve_impl_transposed, LDLT.h:573-613):
// L has a unit diagonal (trinv_kernel<UNIT>) and the diagonal of the stored factor holds D; the
// backward sweep applies D's pseudo-inverse to each block's right-hand sides as it loads them
// (DSCALE: divide where |d| > the smallest normal number, else 0, LDLT.h:587-600).
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "internal.h"
#include "mma_split.cuh"

namespace gbllt {

namespace {

constexpr int RB = 64;
constexpr int RC = 512;  // right-hand sides per launch (at most 32 chains of 16)
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <typename T, bool UP>
__device__ __forceinline__ T lget(const T* __restrict__ a, long long lda, long long i, long long j) {
  return UP ? a[i * lda + j] : a[j * lda + i];  // L(i, j)
}

// inv[blk] (64 x 64, column-major, lower) = L_blk^{-1}; identity padding beyond n.  UNIT: the
// diagonal of L is 1 and the stored diagonal (D of an LDL^T factor) is not read.
template <typename T, bool UP, bool UNIT>
__global__ void __launch_bounds__(128) trinv_kernel(const T* __restrict__ a, long long lda, long long n,
                                                    T* __restrict__ inv) {
  __shared__ T L[RB][RB + 1];  // L[i][p]
  const long long b0 = (long long)blockIdx.x * RB;
  const int bs = (int)(n - b0 < RB ? n - b0 : RB);
  for (int idx = threadIdx.x; idx < RB * RB; idx += 128) {
    int i, p;
    if (UP) { p = idx % RB; i = idx / RB; }
    else    { i = idx % RB; p = idx / RB; }
    T v = (i == p) ? T(1) : T(0);
    if (i < bs && p < bs && (UNIT ? i > p : i >= p)) v = lget<T, UP>(a, lda, b0 + i, b0 + p);
    L[i][p] = v;
  }
  __syncthreads();
  T* out = inv + (long long)blockIdx.x * RB * RB;
  if (threadIdx.x < RB) {
    const int c = threadIdx.x;  // column c of the inverse: L x = e_c
    T x[RB];
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      T v = (i == c) ? T(1) : T(0);
#pragma unroll
      for (int p = 0; p < i; ++p) v = fma(-L[i][p], x[p], v);
      x[i] = i < c ? T(0) : (UNIT ? v : v / L[i][i]);
    }
#pragma unroll
    for (int i = 0; i < RB; ++i) out[(long long)c * RB + i] = x[i];
  }
}

template <typename T, int RCT>
struct SweepSmem {
  T Ls[RB][RB + 1];    // Ls[p][r]: forward L(I0+r, J0+p); backward L(J0+p, I0+r)
  T Ds[RB][RB + 1];    // inverse of the diagonal triangle, Ds[i][p] = Linv(i, p)
  T Ys[RB][RCT + 1];   // the solved block J
  T Bs[RB][RCT + 1];   // this block's right-hand sides
};

// The pseudo-inverse of one entry of D (LDLT.h:594-600).
template <typename T>
__device__ __forceinline__ T dplus(T v, T d) {
  const T tiny = sizeof(T) == 8 ? (T)DBL_MIN : (T)FLT_MIN;
  return fabs(d) > tiny ? v / d : T(0);
}

// RCT right-hand sides per pass; thread (r, cq) owns row r and RCT/4 of them.  DSCALE (backward
// sweep of the LDL^T solve): the block's right-hand sides are multiplied by D^+ as they are loaded.
template <typename T, bool UP, bool BWD, int RCT, bool DSCALE>
__global__ void __launch_bounds__(256) sweep_kernel(const T* __restrict__ a, long long lda, long long n,
                                                    T* __restrict__ b, long long ldb, int nrhs, const T* __restrict__ inv,
                                                    int* __restrict__ flags, int* __restrict__ counter,
                                                    int* __restrict__ err, unsigned long long wait_ns) {
  constexpr int CPT = RCT / 4;
  // right-hand-side chunk: an independent chain with its own tickets and flags
  {
    const int chunk = blockIdx.y;
    b += (long long)chunk * RCT * ldb;
    nrhs -= chunk * RCT;
    flags += (long long)chunk * ((n + RB - 1) / RB);
    counter += chunk;
  }
  extern __shared__ __align__(16) unsigned char sweep_raw[];
  SweepSmem<T, RCT>& sm = *reinterpret_cast<SweepSmem<T, RCT>*>(sweep_raw);
  __shared__ int s_ticket, s_abort;
  const int tid = threadIdx.x, r = tid & 63, cq = tid >> 6;
  const int nb = (int)((n + RB - 1) / RB);
  if (tid == 0) {
    s_ticket = atomicAdd(counter, 1);
    s_abort = 0;
  }
  __syncthreads();
  const int I = BWD ? nb - 1 - s_ticket : s_ticket;
  const long long I0 = (long long)I * RB;
  // inputs that do not depend on other blocks are fetched first, off the critical path
  const T* Dinv = inv + (long long)I * RB * RB;
  for (int idx = tid; idx < RB * RB; idx += 256) {
    const int i = idx & 63, p = idx >> 6;
    sm.Ds[i][p] = Dinv[(long long)p * RB + i];
  }
  for (int idx = tid; idx < RB * RCT; idx += 256) {
    const int p = idx & 63, c = idx >> 6;
    T v = (I0 + p < n && c < nrhs) ? b[(long long)c * ldb + I0 + p] : T(0);
    if (DSCALE && I0 + p < n) v = dplus(v, a[(I0 + p) * (lda + 1)]);
    sm.Bs[p][c] = v;
  }
  T acc[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) acc[q] = T(0);
  // off-diagonal blocks in the order they become ready
  const int jfirst = BWD ? nb - 1 : 0;
  const int jstep = BWD ? -1 : 1;
  for (int J = jfirst; J != I; J += jstep) {
    const long long J0 = (long long)J * RB;
    constexpr bool r_fast = (!BWD && !UP) || (BWD && UP);
    for (int idx = tid; idx < RB * RB; idx += 256) {
      int rr, p;
      if (r_fast) { rr = idx & 63; p = idx >> 6; }
      else        { p = idx & 63; rr = idx >> 6; }
      T v = T(0);
      if (I0 + rr < n && J0 + p < n)
        v = BWD ? lget<T, UP>(a, lda, J0 + p, I0 + rr) : lget<T, UP>(a, lda, I0 + rr, J0 + p);
      sm.Ls[p][rr] = v;
    }
    if (tid == 0) {
      const volatile int* f = flags + J;
      const unsigned long long t0 = gtimer();
      while (*f == 0) {
        if (*(volatile int*)err) {  // another block's wait already ran out: this chain is broken
          s_abort = 1;
          break;
        }
        if (gtimer() - t0 > wait_ns) {
          s_abort = 1;
          atomicExch(err, 1);
          break;
        }
      }
      __threadfence();
    }
    __syncthreads();
    if (s_abort) {
      // the block's solution cannot be formed: its rows become NaN, so a stream-ordered caller
      // that never reads the error word still sees that the result is invalid
      for (int idx = tid; idx < RB * RCT; idx += 256) {
        const int p = idx & 63, c = idx >> 6;
        if (I0 + p < n && c < nrhs) b[(long long)c * ldb + I0 + p] = T(NAN);
      }
      return;
    }
    for (int idx = tid; idx < RB * RCT; idx += 256) {
      const int p = idx & 63, c = idx >> 6;
      sm.Ys[p][c] = (J0 + p < n && c < nrhs) ? __ldcg(b + (long long)c * ldb + J0 + p) : T(0);
    }
    __syncthreads();
#pragma unroll 4
    for (int p = 0; p < RB; ++p) {
      const T l = sm.Ls[p][r];
#pragma unroll
      for (int q = 0; q < CPT; ++q) acc[q] = fma(l, sm.Ys[p][cq * CPT + q], acc[q]);
    }
    __syncthreads();
  }
  // V = B_I - acc, then X_I = Linv V (forward) or Linv^T V (backward).  The barrier orders the Ds/Bs
  // preload (written under another thread mapping) before these reads when the J loop ran no pass.
  __syncthreads();
#pragma unroll
  for (int q = 0; q < CPT; ++q) sm.Ys[r][cq * CPT + q] = sm.Bs[r][cq * CPT + q] - acc[q];
  __syncthreads();
  T x[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) x[q] = T(0);
#pragma unroll 4
  for (int p = 0; p < RB; ++p) {
    const T d = BWD ? sm.Ds[p][r] : sm.Ds[r][p];
#pragma unroll
    for (int q = 0; q < CPT; ++q) x[q] = fma(d, sm.Ys[p][cq * CPT + q], x[q]);
  }
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int c = cq * CPT + q;
    if (I0 + r < n && c < nrhs) b[(long long)c * ldb + I0 + r] = x[q];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) atomicExch(flags + I, 1);
}

// grid_blocks (0: all nb): CTAs launched per chain; the self-test launches fewer, behind a preset
// ticket counter, so that one block's predecessor never publishes.
template <typename T, bool UP, bool BWD, int RCT, bool DSCALE>
void launch_sweep_rc(int nb, const T* a, long long lda, long long n, T* b, long long ldb, int nrhs, const T* inv,
                     int* flags, int* counter, int* err, cudaStream_t s, unsigned long long wait_ns = WAIT_NS,
                     int grid_blocks = 0) {
  // set on every launch: cheap, and correct for every device and host thread
  const int smem = (int)sizeof(SweepSmem<T, RCT>);
  cudaFuncSetAttribute(sweep_kernel<T, UP, BWD, RCT, DSCALE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  dim3 grid((unsigned)(grid_blocks > 0 ? grid_blocks : nb), (unsigned)((nrhs + RCT - 1) / RCT));
  sweep_kernel<T, UP, BWD, RCT, DSCALE>
      <<<grid, 256, smem, s>>>(a, lda, n, b, ldb, nrhs, inv, flags, counter, err, wait_ns);
}

// One launch per sweep: chunks of RCT right-hand sides run as parallel chains (grid.y); 4 columns
// per chunk for a single right-hand side, 16 otherwise (more chains spread the FP64 work of the
// last row blocks over more SMs).
// narrow: chains of 4 whatever nrhs (more CTAs, each with a quarter of the FP64 work per link).
template <typename T, bool UP, bool BWD, bool DSCALE = false>
void launch_sweep(int nb, const T* a, long long lda, long long n, T* b, long long ldb, int nrhs, const T* inv,
                  int* flags, int* counter, int* err, cudaStream_t s, bool narrow = false) {
  if (nrhs <= 4 || narrow)
    launch_sweep_rc<T, UP, BWD, 4, DSCALE>(nb, a, lda, n, b, ldb, nrhs, inv, flags, counter, err, s);
  else launch_sweep_rc<T, UP, BWD, 16, DSCALE>(nb, a, lda, n, b, ldb, nrhs, inv, flags, counter, err, s);
}

// ---------------------------------------------------------------------------------------------
// FP32 sweeps that publish each solved value as its own ready signal.
//
// Each solved value is published once more in a word buffer that is filled with the all-ones
// pattern (a NaN) before every sweep; a word is ready when it differs from that pattern, and a
// solved value with exactly that bit pattern is published as the canonical NaN instead.  A
// consumer polls the values themselves, so a chain link costs one store and one load round trip:
// no fence, no separate flag, no re-read of the block.
//
// Per row block I the CTA forms, off the chain's critical path:
//   M_I = D_I G_{I-1}            (D_I = the inverted diagonal triangle, G_{I-1} = the tile of the
//                                 block the chain delivers last),
//   z_I = D_I (B_I - sum_J G_J Y_J) over the blocks before that one,
// and on the critical path only x_I = z_I - M_I Y_{I-1}: one 64 x 64 x RCT product per link.
// Off-diagonal tiles stream into shared memory with cp.async one tile ahead, and the next block's
// words are requested before the current product, so a CTA that starts behind the chain catches up
// at the rate of its tile loads.  Tickets interleave the right-hand-side chains (ticket t: chain
// t % nch, t / nch-th block of the sweep), so the CTAs resident at any time work on the same part
// of every chain.
// ---------------------------------------------------------------------------------------------

constexpr int LL_RC = 64;     // right-hand sides per launch: one chain of 64, or chains of 16 or 4
constexpr int PF_PITCH = 68;  // row pitch (floats) of a tile stored with p contiguous

constexpr int LL_NT = 4;      // tile slots: the last-delivered tile, then a ring of look-back tiles

template <int RCT>
struct LLSmem {
  float Lb[LL_NT][RB * PF_PITCH];  // off-diagonal tiles: three loads in flight behind the one in use
  float Ds[RB * (RB + 1)];     // Ds[i * 65 + r] = D(r, i)
  float Ms[RB * RB];           // Ms[p * 64 + r] = M(r, p)
  // staged 64 x RCT block, flat index = word index; for 32-column chains, whose look-back products
  // run on the tensor cores, the block's three BF16 parts instead (ys_part_index), 12 KB
  float Ys[RCT == 32 ? 3 * 32 * 32 : RB * RCT];
};

// Word of the packed BF16 pair (Y(2 pi, c), Y(2 pi + 1, c)) of part `part` in the staged parts: column c
// holds its 32 pairs at c * 32, the pair index XOR-swizzled by (c % 8) * 4 so that the eight columns
// and four pairs that a warp's B-fragment load touches fall in 32 different banks.
__device__ __forceinline__ int ys_part_index(int part, int c, int pi) { return part * 1024 + c * 32 + (pi ^ ((c & 7) << 2)); }

__device__ __forceinline__ uint32_t sptr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sptr(dst)), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(sptr(dst)), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Tile G(rr, p) of the sweep for row block I0 and column block J0.  RFAST: element (rr, p) at
// a[(J0 + p) lda + I0 + rr], kept as lb[p * 68 + rr]; otherwise at a[(I0 + rr) lda + J0 + p], kept as
// lb[rr * 68 + p] (the pitch of 68 keeps the tensor-core fragment reads of either layout within two
// banks' conflicts).  Entries beyond n are zero-filled.  VEC: 16-byte copies (a 16-byte aligned,
// lda a multiple of 4).
template <bool RFAST, bool VEC>
__device__ __forceinline__ void load_tile(float* lb, const float* __restrict__ a, long long lda, long long n,
                                          long long I0, long long J0, int tid) {
  if (VEC) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int idx = tid + k * 256;
      const int f = (idx & 15) * 4, s = idx >> 4;  // f: contiguous index (4 per chunk), s: strided
      const long long fg = (RFAST ? I0 : J0) + f, sg = (RFAST ? J0 : I0) + s;
      const int bytes = (fg < n && sg < n) ? (int)(n - fg < 4 ? n - fg : 4) * 4 : 0;
      const float* src = bytes ? a + sg * lda + fg : a;
      cp_async16(lb + s * PF_PITCH + f, src, bytes);
    }
  } else {
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const int idx = tid + k * 256;
      const int f = idx & 63, s = idx >> 6;
      const long long fg = (RFAST ? I0 : J0) + f, sg = (RFAST ? J0 : I0) + s;
      const int bytes = (fg < n && sg < n) ? 4 : 0;
      const float* src = bytes ? a + sg * lda + fg : a;
      cp_async4(lb + s * PF_PITCH + f, src, bytes);
    }
  }
}

constexpr unsigned NOT_READY = 0xFFFFFFFFu;  // the fill pattern of the word buffer
constexpr unsigned CANON_NAN = 0x7FC00000u;

template <int CPT>
__device__ __forceinline__ void ll_load(const unsigned* src, unsigned* w) {
  if (CPT % 4 == 0) {
#pragma unroll
    for (int k = 0; k < CPT; k += 4)
      asm volatile("ld.volatile.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                   : "=r"(w[k]), "=r"(w[k + 1]), "=r"(w[k + 2]), "=r"(w[k + 3])
                   : "l"(src + k)
                   : "memory");
  } else {
    asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(w[0]) : "l"(src) : "memory");
  }
}

template <int CPT>
__device__ __forceinline__ bool ll_valid(const unsigned* w) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < CPT; ++k) ok = ok && w[k] != NOT_READY;
  return ok;
}

template <int CPT>
__device__ __forceinline__ void ll_store(unsigned* dst, const float* x) {
  unsigned w[CPT];
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const unsigned u = __float_as_uint(x[k]);
    w[k] = u == NOT_READY ? CANON_NAN : u;
  }
  if (CPT % 4 == 0) {
#pragma unroll
    for (int k = 0; k < CPT; k += 4)
      asm volatile("st.volatile.global.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(dst + k), "r"(w[k]), "r"(w[k + 1]),
                   "r"(w[k + 2]), "r"(w[k + 3])
                   : "memory");
  } else {
    asm volatile("st.volatile.global.u32 [%0], %1;" ::"l"(dst), "r"(w[0]) : "memory");
  }
}

template <bool RFAST, int CPT>
__device__ __forceinline__ void tile_product(const float* lb, const float* ys, int r, int cq, float* acc) {
  constexpr int RCT = 4 * CPT;
  if (RFAST) {
#pragma unroll 8
    for (int p = 0; p < RB; ++p) {
      const float l = lb[p * PF_PITCH + r];
      if (CPT % 4 == 0) {
#pragma unroll
        for (int k = 0; k < CPT; k += 4) {
          const float4 y = *reinterpret_cast<const float4*>(ys + p * RCT + cq * CPT + k);
          acc[k] = fmaf(l, y.x, acc[k]);
          acc[k + 1] = fmaf(l, y.y, acc[k + 1]);
          acc[k + 2] = fmaf(l, y.z, acc[k + 2]);
          acc[k + 3] = fmaf(l, y.w, acc[k + 3]);
        }
      } else {
        acc[0] = fmaf(l, ys[p * RCT + cq], acc[0]);
      }
    }
  } else {
#pragma unroll 2
    for (int p = 0; p < RB; p += 4) {
      const float4 l4 = *reinterpret_cast<const float4*>(lb + r * PF_PITCH + p);
      const float lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (CPT % 4 == 0) {
#pragma unroll
          for (int k = 0; k < CPT; k += 4) {
            const float4 y = *reinterpret_cast<const float4*>(ys + (p + u) * RCT + cq * CPT + k);
            acc[k] = fmaf(lv[u], y.x, acc[k]);
            acc[k + 1] = fmaf(lv[u], y.y, acc[k + 1]);
            acc[k + 2] = fmaf(lv[u], y.z, acc[k + 2]);
            acc[k + 3] = fmaf(lv[u], y.w, acc[k + 3]);
          }
        } else {
          acc[0] = fmaf(lv[u], ys[(p + u) * RCT + cq], acc[0]);
        }
      }
    }
  }
}

// The look-back product of a 32-column chain on the tensor cores: acc (64 x 32) += G (64 x 64) Y
// (64 x 32) with mma.sync m16n8k16 BF16 and the three-part split of mma_split.cuh: the six part
// products of one tile are accumulated, the small ones first, in registers that start at zero; the
// tile's sum is then added to acc with an FP32 add.  The tensor cores' FP32 accumulation truncates,
// and adding every product straight into acc's long running sum biased it: the solve's error grew
// 40-fold and cost the refinement one to two steps.  Per tile, the error is below the CUDA-core
// product's (2.0e-7 vs 8.1e-7 relative at n = 32768, 64 RHS, against an FP64 triangular solve).
// Y's parts are split once per tile when the block is staged (stage_y_parts); warp w takes rows
// 16 (w % 4) .. + 16 and the K half 32 (w / 4) .. + 32 of the tile for all 32 columns, so each G entry
// is split by one warp.  (Splitting Y in every warp and G in two, the product bounded how fast a CTA
// that starts behind the chain caught up: two sweeps at n = 32768, 64 RHS, took 6.26 ms, 4.01 ms
// with no product at all.)  c[n][i] is the m16n8 accumulator fragment of the warp's n-th 8-column
// tile over its K half: rows g (i < 2) and g + 8, columns 2 t + (i & 1), g = lane / 4, t = lane % 4.
// G: lb (RFAST: lb[p * 68 + rr], else lb[rr * 68 + p]).
template <bool RFAST>
__device__ __forceinline__ void tile_product_tc(const float* lb, const uint32_t* yp, int tid, float (*c)[4]) {
  const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int m0 = 16 * (warp & 3), kh = 32 * (warp >> 2);
  float s[4][4] = {};  // this tile's product, added to c once at the end
#pragma unroll
  for (int k0 = kh; k0 < kh + 32; k0 += 16) {
    // A fragment: rows m0 + g (+8), k columns k0 + 2t, +1 (regs 0, 1) and k0 + 2t + 8, +9 (regs 2, 3)
    float av[8];
#pragma unroll
    for (int h = 0; h < 2; ++h) {      // k half: +0 / +8
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {  // row: g / g + 8
        const int row = m0 + g + 8 * rr, k = k0 + 2 * t + 8 * h;
        if (RFAST) {
          av[4 * h + 2 * rr] = lb[k * PF_PITCH + row];
          av[4 * h + 2 * rr + 1] = lb[(k + 1) * PF_PITCH + row];
        } else {
          const float2 v = *reinterpret_cast<const float2*>(lb + row * PF_PITCH + k);
          av[4 * h + 2 * rr] = v.x;
          av[4 * h + 2 * rr + 1] = v.y;
        }
      }
    }
    uint32_t ap[4][3];  // register i of the fragment (rows g, g+8, g, g+8 for i = 0..3), part
#pragma unroll
    for (int i = 0; i < 4; ++i) split3_bf16x2(av[2 * i], av[2 * i + 1], ap[i]);
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int col = 8 * nt + g, pi = k0 / 2 + t;
      uint32_t bp0[3], bp1[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        bp0[q] = yp[ys_part_index(q, col, pi)];
        bp1[q] = yp[ys_part_index(q, col, pi + 4)];
      }
      mma_split6(s[nt], ap, bp0, bp1);
    }
  }
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) c[nt][i] += s[nt][i];
}

// Stage the awaited block's words (thread tid holds Y(tid / 4, (tid % 4) * 8 + q) in w[q]) as the
// three BF16 parts of row pairs: a thread and the one holding the neighbouring row (tid ^ 4) swap
// one word per column, the even row's thread packs and splits columns 0..3 of its eight, the odd
// row's columns 4..7.
__device__ __forceinline__ void stage_y_parts(const unsigned* w, uint32_t* yp, int tid) {
  const int p = tid >> 2, c0 = (tid & 3) * 8;
  const bool even = (p & 1) == 0;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const unsigned other = __shfl_xor_sync(0xffffffffu, even ? w[u + 4] : w[u], 4);
    const int q = even ? u : u + 4;
    const float lo = __uint_as_float(even ? w[u] : other), hi = __uint_as_float(even ? other : w[u + 4]);
    uint32_t part[3];
    split3_bf16x2(lo, hi, part);
#pragma unroll
    for (int k = 0; k < 3; ++k) yp[ys_part_index(k, c0 + q, p >> 1)] = part[k];
  }
}

// out[q] (+)= sum_p S[p * pitch + r] * ys[p][cq * CPT + q]: the product of a shared 64 x 64 matrix
// stored column by column (consecutive r) with the staged block.
template <int CPT>
__device__ __forceinline__ void colmajor_product(const float* S, int pitch, const float* ys, int r, int cq,
                                                 float* out) {
  constexpr int RCT = 4 * CPT;
#pragma unroll 8
  for (int p = 0; p < RB; ++p) {
    const float s = S[p * pitch + r];
    if (CPT % 4 == 0) {
#pragma unroll
      for (int k = 0; k < CPT; k += 4) {
        const float4 y = *reinterpret_cast<const float4*>(ys + p * RCT + cq * CPT + k);
        out[k] = fmaf(s, y.x, out[k]);
        out[k + 1] = fmaf(s, y.y, out[k + 1]);
        out[k + 2] = fmaf(s, y.z, out[k + 2]);
        out[k + 3] = fmaf(s, y.w, out[k + 3]);
      }
    } else {
      out[0] = fmaf(s, ys[p * RCT + cq], out[0]);
    }
  }
}

// Sleep between polls of a block `dist` links before this CTA's own.  The blocks one and two links
// back are polled without sleeping: the product with the block two back and the diagonal solve
// that follows it must finish before the block one back arrives.
__device__ __forceinline__ unsigned poll_sleep_ns(int dist) { return dist <= 2 ? 0u : (dist > 6 ? 2000u : 400u * (dist - 2)); }

template <int CPT>
__device__ __forceinline__ bool ll_wait_block(const unsigned* src, unsigned* w, int dist, int* err,
                                              unsigned long long wait_ns) {
  if (ll_valid<CPT>(w)) return true;
  const unsigned ns = poll_sleep_ns(dist);
  const unsigned long long t0 = gtimer();
  for (int it = 1;; ++it) {
    if (ns) __nanosleep(ns);
    ll_load<CPT>(src, w);
    if (ll_valid<CPT>(w)) return true;
    if ((it & 63) == 0) {
      if (*(volatile int*)err) return false;
      if (gtimer() - t0 > wait_ns) {
        atomicExch(err, 1);
        return false;
      }
    }
  }
}

// A block whose wait ran out (or whose chain is broken) writes NaN into its rows of the solution,
// so that a stream-ordered caller that never reads the error word still sees an invalid result.
template <int CPT>
__device__ __forceinline__ void ll_fill_nan(float* b, long long ldb, long long n, int nrhs, long long I0, int r,
                                            int cq) {
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int c = cq * CPT + q;
    if (I0 + r < n && c < nrhs) b[(long long)c * ldb + I0 + r] = NAN;
  }
}

// One CTA per (row block, right-hand-side chain); 256 threads, thread (r, cq) owns row r and
// right-hand sides cq * CPT .. cq * CPT + CPT - 1 of its chain (RCT = 4 CPT columns per chain).
template <bool UP, bool BWD, int CPT, bool DSCALE, bool VEC>
__global__ void __launch_bounds__(256, 2) sweep_ll_kernel(const float* __restrict__ a, long long lda, long long n,
                                                       float* __restrict__ b, long long ldb, int nrhs,
                                                       const float* __restrict__ inv, unsigned* __restrict__ ll,
                                                       int nch, int* __restrict__ counter, int* __restrict__ err,
                                                       unsigned long long wait_ns) {
  constexpr int RCT = 4 * CPT;
  constexpr bool RFAST = (!BWD && !UP) || (BWD && UP);
  extern __shared__ __align__(16) unsigned char ll_raw[];
  LLSmem<RCT>& sm = *reinterpret_cast<LLSmem<RCT>*>(ll_raw);
  __shared__ int s_ticket;
  const int tid = threadIdx.x, r = tid & 63, cq = tid >> 6;
  const int nb = (int)((n + RB - 1) / RB);
  if (tid == 0) s_ticket = atomicAdd(counter, 1);
  __syncthreads();
  const int ch = s_ticket % nch, rank = s_ticket / nch;
  const int I = BWD ? nb - 1 - rank : rank;
  const long long I0 = (long long)I * RB;
  b += (long long)ch * RCT * ldb;
  nrhs -= ch * RCT;
  unsigned* llc = ll + (size_t)ch * nb * RB * RCT;  // block J's words at J * 64 * RCT
  const int step = BWD ? -1 : 1;
  const bool has_prev = BWD ? I < nb - 1 : I > 0;
  const int Jlast = I - step;  // the block the chain delivers last to this one
  const int Jfirst = BWD ? nb - 1 : 0;
  const int nloop = has_prev ? (BWD ? nb - 2 - I : I - 1) : 0;  // blocks before Jlast

  // 1. inputs that depend on no other block: the last-delivered tile (group 0, slot 0), the first
  //    LL_NT - 1 loop tiles (groups 1 .. LL_NT - 1, slots 1 .. LL_NT - 1), the diagonal inverse and
  //    this block's right-hand sides.  Loop tile k lives in slot (k + 1) % LL_NT and group k + 1.
  if (has_prev) load_tile<RFAST, VEC>(sm.Lb[0], a, lda, n, I0, (long long)Jlast * RB, tid);
  cp_commit();
#pragma unroll
  for (int k = 0; k < LL_NT - 1; ++k) {
    if (k < nloop) load_tile<RFAST, VEC>(sm.Lb[1 + k], a, lda, n, I0, (long long)(Jfirst + k * step) * RB, tid);
    cp_commit();
  }
  const float* Dinv = inv + (long long)I * RB * RB;  // column-major Linv of block I
  for (int idx = tid; idx < RB * RB; idx += 256) {
    const int lo = idx & 63, hi = idx >> 6;
    if (!BWD) sm.Ds[hi * 65 + lo] = Dinv[idx];  // D(lo, hi) = Linv(lo, hi)
    else sm.Ds[lo * 65 + hi] = Dinv[idx];       // D(hi, lo) = Linv(lo, hi)
  }
  float bv[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int c = cq * CPT + q;
    float v = 0.f;
    if (I0 + r < n && c < nrhs) {
      v = b[(long long)c * ldb + I0 + r];
      if (DSCALE) v = dplus(v, a[(I0 + r) * (lda + 1)]);
    }
    bv[q] = v;
  }
  unsigned w[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) w[q] = NOT_READY;
  if (has_prev) ll_load<CPT>(llc + (size_t)(nloop > 0 ? Jfirst : Jlast) * RB * RCT + tid * CPT, w);

  // 2. M = D G_last, kept column by column (Ms[p * 64 + r] = M(r, p)); thread (r, cq) forms
  //    columns cq * 16 .. cq * 16 + 15
  cp_wait<LL_NT - 1>();  // group 0 has landed
  __syncthreads();
  if (has_prev) {
    float m[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) m[j] = 0.f;
#pragma unroll 4
    for (int i = 0; i < RB; ++i) {
      const float d = sm.Ds[i * 65 + r];
      if (RFAST) {
#pragma unroll
        for (int j = 0; j < 16; ++j) m[j] = fmaf(d, sm.Lb[0][(cq * 16 + j) * PF_PITCH + i], m[j]);
      } else {
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4) {
          const float4 g = *reinterpret_cast<const float4*>(sm.Lb[0] + i * PF_PITCH + cq * 16 + 4 * k4);
          m[4 * k4 + 0] = fmaf(d, g.x, m[4 * k4 + 0]);
          m[4 * k4 + 1] = fmaf(d, g.y, m[4 * k4 + 1]);
          m[4 * k4 + 2] = fmaf(d, g.z, m[4 * k4 + 2]);
          m[4 * k4 + 3] = fmaf(d, g.w, m[4 * k4 + 3]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) sm.Ms[(cq * 16 + j) * 64 + r] = m[j];
  }
  __syncthreads();  // slot 0 is free for the first prefetch

  // 3. the blocks before Jlast, in the order the chain delivers them.  Iteration k loads tile
  //    k + LL_NT - 1 into slot k % LL_NT (freed by tile k - 1, or by G_last for k = 0) and uses tile
  //    k from slot (k + 1) % LL_NT; its group is complete once at most LL_NT - 1 newer ones are pending.
  constexpr bool TC = CPT == 8;  // 32-column chains: the look-back products on the tensor cores
  float acc[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) acc[q] = 0.f;
  float cf[4][4];
#pragma unroll
  for (int i = 0; i < 16; ++i) cf[i >> 2][i & 3] = 0.f;
  uint32_t* const yp = reinterpret_cast<uint32_t*>(sm.Ys);
  for (int k = 0; k < nloop; ++k) {
    const int J = Jfirst + k * step;
    if (k + LL_NT - 1 < nloop)
      load_tile<RFAST, VEC>(sm.Lb[k % LL_NT], a, lda, n, I0, (long long)(J + (LL_NT - 1) * step) * RB, tid);
    cp_commit();
    const bool ok =
        ll_wait_block<CPT>(llc + (size_t)J * RB * RCT + tid * CPT, w, BWD ? J - I : I - J, err, wait_ns);
    if (TC) {  // word tid * 8 + q is Y(tid / 4, (tid % 4) * 8 + q)
      stage_y_parts(w, yp, tid);
    } else {
#pragma unroll
      for (int q = 0; q < CPT; ++q) sm.Ys[tid * CPT + q] = __uint_as_float(w[q]);
    }
    cp_wait<LL_NT - 1>();
    if (__syncthreads_or(!ok)) {
      asm volatile("cp.async.wait_all;" ::: "memory");
      ll_fill_nan<CPT>(b, ldb, n, nrhs, I0, r, cq);
      return;
    }
    // request the next awaited block's words before this product
    ll_load<CPT>(llc + (size_t)(k + 1 < nloop ? J + step : Jlast) * RB * RCT + tid * CPT, w);
    if (TC) tile_product_tc<RFAST>(sm.Lb[(k + 1) % LL_NT], yp, tid, cf);
    else tile_product<RFAST, CPT>(sm.Lb[(k + 1) % LL_NT], sm.Ys, r, cq, acc);
    __syncthreads();
  }
  if (TC) {  // the two K halves' fragments back to thread (r, cq)'s row and columns, through the idle
             // tile slots 1 and 2 (row pitch 36)
    const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const int m0 = 16 * (warp & 3);
    float* const half = sm.Lb[1 + (warp >> 2)];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) half[(m0 + g + (i >> 1) * 8) * 36 + 8 * nt + 2 * t + (i & 1)] = cf[nt][i];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < CPT; ++q) acc[q] = sm.Lb[1][r * 36 + cq * CPT + q] + sm.Lb[2][r * 36 + cq * CPT + q];
    __syncthreads();
  }

  // 4. z = D (B - acc), then x = z - M Y_last
#pragma unroll
  for (int q = 0; q < CPT; ++q) sm.Ys[r * RCT + cq * CPT + q] = bv[q] - acc[q];
  __syncthreads();
  float x[CPT];
#pragma unroll
  for (int q = 0; q < CPT; ++q) x[q] = 0.f;
  colmajor_product<CPT>(sm.Ds, RB + 1, sm.Ys, r, cq, x);
  if (has_prev) {
    float* yl = sm.Lb[0];  // every tile slot is idle now
    const bool ok = ll_wait_block<CPT>(llc + (size_t)Jlast * RB * RCT + tid * CPT, w, 1, err, wait_ns);
#pragma unroll
    for (int q = 0; q < CPT; ++q) yl[tid * CPT + q] = __uint_as_float(w[q]);
    if (__syncthreads_or(!ok)) {
      ll_fill_nan<CPT>(b, ldb, n, nrhs, I0, r, cq);
      return;
    }
    float mv[CPT];
#pragma unroll
    for (int q = 0; q < CPT; ++q) mv[q] = 0.f;
    colmajor_product<CPT>(sm.Ms, RB, yl, r, cq, mv);
#pragma unroll
    for (int q = 0; q < CPT; ++q) x[q] -= mv[q];
  }
  ll_store<CPT>(llc + (size_t)I * RB * RCT + r * RCT + cq * CPT, x);
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int c = cq * CPT + q;
    if (I0 + r < n && c < nrhs) b[(long long)c * ldb + I0 + r] = x[q];
  }
}

// grid_blocks (0: all nb): row blocks launched per chain (the self-test launches fewer).
template <bool UP, bool BWD, int CPT, bool DSCALE>
void launch_sweep_ll_cpt(int nb, int nch, const float* a, long long lda, long long n, float* b, long long ldb,
                         int nrhs, const float* inv, unsigned* ll, int* counter, int* err,
                         cudaStream_t s, unsigned long long wait_ns = WAIT_NS, int grid_blocks = 0) {
  const int smem = (int)sizeof(LLSmem<4 * CPT>);
  const bool vec = ((uintptr_t)a % 16 == 0) && (lda % 4 == 0);
  const unsigned grid = (unsigned)((grid_blocks > 0 ? grid_blocks : nb) * nch);
  if (vec) {
    cudaFuncSetAttribute(sweep_ll_kernel<UP, BWD, CPT, DSCALE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         smem);
    sweep_ll_kernel<UP, BWD, CPT, DSCALE, true>
        <<<grid, 256, smem, s>>>(a, lda, n, b, ldb, nrhs, inv, ll, nch, counter, err, wait_ns);
  } else {
    cudaFuncSetAttribute(sweep_ll_kernel<UP, BWD, CPT, DSCALE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         smem);
    sweep_ll_kernel<UP, BWD, CPT, DSCALE, false>
        <<<grid, 256, smem, s>>>(a, lda, n, b, ldb, nrhs, inv, ll, nch, counter, err, wait_ns);
  }
}

// Chains of 4 right-hand sides for nrhs <= 4, else of 16 (nrhs <= LL_RC per launch).
// Chains of 4 right-hand sides for nrhs <= 4, of 16 up to 16, else of 32.  Every CTA of a chain
// streams all the tiles left of its block, and a CTA that starts once earlier ones have finished
// must catch up with the chain at the rate of its tile products: wider chains mean fewer CTAs and
// fewer re-reads of L, but a longer product on the chain's critical path.  32 columns measured best
// for 64 right-hand sides (64 was slower: its link carries a 64 x 64 x 64 product).
inline int ll_chain_cols(int nrhs) { return nrhs <= 4 ? 4 : (nrhs <= 16 ? 16 : 32); }

template <bool UP, bool BWD, bool DSCALE = false>
void launch_sweep_ll(int nb, const float* a, long long lda, long long n, float* b, long long ldb, int nrhs,
                     const float* inv, unsigned* ll, int* counter, int* err, cudaStream_t s) {
  const int rct = ll_chain_cols(nrhs), nch = (nrhs + rct - 1) / rct;
  if (rct == 4)
    launch_sweep_ll_cpt<UP, BWD, 1, DSCALE>(nb, nch, a, lda, n, b, ldb, nrhs, inv, ll, counter, err, s);
  else if (rct == 16)
    launch_sweep_ll_cpt<UP, BWD, 4, DSCALE>(nb, nch, a, lda, n, b, ldb, nrhs, inv, ll, counter, err, s);
  else
    launch_sweep_ll_cpt<UP, BWD, 8, DSCALE>(nb, nch, a, lda, n, b, ldb, nrhs, inv, ll, counter, err, s);
}

// Workspace layouts.  Both start with the diagonal inverses, then a 256-byte block whose first word
// is the call's error word (cleared once per call, set by any bounded wait that ran out).
// FP64: inverses | error word | flags and tickets (chains of one launch).
// FP32: inverses | error word, tickets | published words (LL_RC per row).
size_t ws_flags_offset(int64_t nb, size_t elem) { return ((size_t)nb * RB * RB * elem + 255) & ~(size_t)255; }
size_t ws_words_offset(int64_t nb) { return ws_flags_offset(nb, sizeof(float)) + 256; }
size_t ws_bytes_f64(int64_t nb) {
  const int64_t nch = RC / 16;  // chains of one launch, at most
  return ws_flags_offset(nb, sizeof(double)) + 256 + (size_t)(2 * nch * nb + 2 * nch + 8) * sizeof(int) + 256;
}
constexpr int kWsFlagsSkip = 64;  // ints of the error block before the FP64 flags
size_t ws_bytes_f32(int64_t nb) { return ws_words_offset(nb) + (size_t)nb * RB * LL_RC * sizeof(unsigned) + 256; }

}  // namespace

int* potrs_ws_error_word(int64_t n, size_t elem, void* ws) {
  return (int*)((char*)ws + ws_flags_offset((n + RB - 1) / RB, elem));
}

// A workspace sized for FP64 also serves the FP32 solve of the same order (the mixed-precision
// driver runs both on one workspace).
size_t potrs_ws_bytes(int64_t n, size_t elem) {
  const int64_t nb = (n + RB - 1) / RB;
  const size_t f32 = ws_bytes_f32(nb);
  if (elem == sizeof(float)) return f32;
  const size_t f64 = ws_bytes_f64(nb);
  return f64 > f32 ? f64 : f32;
}

// Both sweeps; ldl: the factor is the unit L of LDL^T with D on its diagonal.
template <typename T>
int sweeps_ws(bool upper, bool ldl, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, void* ws,
              cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
  static const std::string ki = std::string("trinv_diag_") + tname<T>();
  static const std::string kf = std::string("sweep_") + tname<T>();
  const int nb = (int)ceil_div(n, RB);
  T* inv = (T*)ws;
  int* base = (int*)((char*)ws + ws_flags_offset(nb, sizeof(T)));
  int* err = base;  // the call's error word
  GB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  {
    ProfScope ps(ki.c_str(), s, (double)nb * RB * RB * RB / 3.0, (double)n * RB * sizeof(T) * 1.5);
    if (ldl) {
      if (upper) trinv_kernel<T, true, true><<<nb, 128, 0, s>>>(a, lda, n, inv);
      else trinv_kernel<T, false, true><<<nb, 128, 0, s>>>(a, lda, n, inv);
    } else {
      if (upper) trinv_kernel<T, true, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
      else trinv_kernel<T, false, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    unsigned* words = (unsigned*)((char*)ws + ws_words_offset(nb));
    int* fctr = base + 1;
    int* bctr = base + 2;
    for (int64_t c0 = 0; c0 < nrhs; c0 += LL_RC) {
      const int nc = (int)(nrhs - c0 < LL_RC ? nrhs - c0 : LL_RC);
      const int rct = ll_chain_cols(nc), nch = (nc + rct - 1) / rct;
      const size_t wbytes = (size_t)nch * nb * RB * rct * sizeof(unsigned);
      float* bc = b + c0 * ldb;
      GB_CUDA_TRY(cudaMemsetAsync(fctr, 0, 2 * sizeof(int), s));
      GB_CUDA_TRY(cudaMemsetAsync(words, 0xFF, wbytes, s));
      const double fl = (double)n * (n + 1) * nc, by = (double)n * (n + 1) / 2.0 * sizeof(T) + 2.0 * n * nc * sizeof(T);
      {
        ProfScope ps(kf.c_str(), s, fl, by);
        if (upper) launch_sweep_ll<true, false>(nb, a, lda, n, bc, ldb, nc, inv, words, fctr, err, s);
        else launch_sweep_ll<false, false>(nb, a, lda, n, bc, ldb, nc, inv, words, fctr, err, s);
      }
      GB_CUDA_TRY(cudaMemsetAsync(words, 0xFF, wbytes, s));
      {
        ProfScope ps(kf.c_str(), s, fl, by);
        if (ldl) {
          if (upper) launch_sweep_ll<true, true, true>(nb, a, lda, n, bc, ldb, nc, inv, words, bctr, err, s);
          else launch_sweep_ll<false, true, true>(nb, a, lda, n, bc, ldb, nc, inv, words, bctr, err, s);
        } else {
          if (upper) launch_sweep_ll<true, true>(nb, a, lda, n, bc, ldb, nc, inv, words, bctr, err, s);
          else launch_sweep_ll<false, true>(nb, a, lda, n, bc, ldb, nc, inv, words, bctr, err, s);
        }
      }
    }
  } else {
    for (int64_t c0 = 0; c0 < nrhs; c0 += RC) {
      const int nc = (int)(nrhs - c0 < RC ? nrhs - c0 : RC);
      const int nch = nc <= 4 ? 1 : (nc + 15) / 16;  // chains in this launch
      int* fflags = base + kWsFlagsSkip;  // forward: nch x nb
      int* bflags = fflags + nch * nb;    // backward: nch x nb
      int* fctr = fflags + 2 * nch * nb;  // nch forward tickets, nch backward tickets
      int* bctr = fctr + nch;
      T* bc = b + c0 * ldb;
      GB_CUDA_TRY(cudaMemsetAsync(fflags, 0, (size_t)(2 * nch * nb + 2 * nch) * sizeof(int), s));
      // algorithmic work per sweep: the lower triangle of L read once, 2 flops per entry and RHS
      const double fl = (double)n * (n + 1) * nc, by = (double)n * (n + 1) / 2.0 * sizeof(T) + 2.0 * n * nc * sizeof(T);
      {
        ProfScope ps(kf.c_str(), s, fl, by);
        if (upper) launch_sweep<T, true, false>(nb, a, lda, n, bc, ldb, nc, inv, fflags, fctr, err, s);
        else launch_sweep<T, false, false>(nb, a, lda, n, bc, ldb, nc, inv, fflags, fctr, err, s);
      }
      {
        ProfScope ps(kf.c_str(), s, fl, by);
        if (ldl) {
          if (upper) launch_sweep<T, true, true, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
          else launch_sweep<T, false, true, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
        } else {
          if (upper) launch_sweep<T, true, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
          else launch_sweep<T, false, true>(nb, a, lda, n, bc, ldb, nc, inv, bflags, bctr, err, s);
        }
      }
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int potrs_ws(bool upper, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, void* ws,
             cudaStream_t s) {
  return sweeps_ws<T>(upper, false, n, nrhs, a, lda, b, ldb, ws, s);
}

template <typename T>
int trinv_all(bool upper, int64_t n, const T* a, int64_t lda, T* inv, cudaStream_t s) {
  if (n <= 0) return GBLLT_SUCCESS;
  static const std::string ki = std::string("trinv_diag_") + tname<T>();
  const int nb = (int)ceil_div(n, RB);
  ProfScope ps(ki.c_str(), s, (double)nb * RB * RB * RB / 3.0, (double)n * RB * sizeof(T) * 1.5);
  if (upper) trinv_kernel<T, true, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
  else trinv_kernel<T, false, false><<<nb, 128, 0, s>>>(a, lda, n, inv);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}
template int trinv_all<double>(bool, int64_t, const double*, int64_t, double*, cudaStream_t);

template <typename T>
int trsm_sweep_ws(bool upper, bool bwd, bool unit, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b,
                  int64_t ldb, void* ws, cudaStream_t s, int* ext_err, const T* pre_inv) {
  if (n <= 0 || nrhs <= 0) return GBLLT_SUCCESS;
  static const std::string ki = std::string("trinv_diag_") + tname<T>();
  static const std::string kf = std::string("sweep_") + tname<T>();
  const int nb = (int)ceil_div(n, RB);
  // the inverses: the caller's, or formed here in the workspace
  const T* inv = pre_inv ? pre_inv : (const T*)ws;
  int* base = (int*)((char*)ws + ws_flags_offset(nb, sizeof(T)));
  int* err = ext_err ? ext_err : base;  // the call's error word, or the caller's (not cleared here)
  if (!ext_err) GB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (!pre_inv) {
    T* winv = (T*)ws;
    ProfScope ps(ki.c_str(), s, (double)nb * RB * RB * RB / 3.0, (double)n * RB * sizeof(T) * 1.5);
    if (unit) {
      if (upper) trinv_kernel<T, true, true><<<nb, 128, 0, s>>>(a, lda, n, winv);
      else trinv_kernel<T, false, true><<<nb, 128, 0, s>>>(a, lda, n, winv);
    } else {
      if (upper) trinv_kernel<T, true, false><<<nb, 128, 0, s>>>(a, lda, n, winv);
      else trinv_kernel<T, false, false><<<nb, 128, 0, s>>>(a, lda, n, winv);
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    unsigned* words = (unsigned*)((char*)ws + ws_words_offset(nb));
    int* ctr = base + 1;
    for (int64_t c0 = 0; c0 < nrhs; c0 += LL_RC) {
      const int nc = (int)(nrhs - c0 < LL_RC ? nrhs - c0 : LL_RC);
      const int rct = ll_chain_cols(nc), nch = (nc + rct - 1) / rct;
      float* bc = b + c0 * ldb;
      GB_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(int), s));
      GB_CUDA_TRY(cudaMemsetAsync(words, 0xFF, (size_t)nch * nb * RB * rct * sizeof(unsigned), s));
      const double fl = (double)n * (n + 1) * nc, by = (double)n * (n + 1) / 2.0 * sizeof(T) + 2.0 * n * nc * sizeof(T);
      ProfScope ps(kf.c_str(), s, fl, by);
      if (bwd) {
        if (upper) launch_sweep_ll<true, true>(nb, a, lda, n, bc, ldb, nc, inv, words, ctr, err, s);
        else launch_sweep_ll<false, true>(nb, a, lda, n, bc, ldb, nc, inv, words, ctr, err, s);
      } else {
        if (upper) launch_sweep_ll<true, false>(nb, a, lda, n, bc, ldb, nc, inv, words, ctr, err, s);
        else launch_sweep_ll<false, false>(nb, a, lda, n, bc, ldb, nc, inv, words, ctr, err, s);
      }
    }
  } else {
    // chains per launch stay within the RC / 16 the workspace holds flags for: 16-wide chains up to
    // RC right-hand sides, or (panel sub-solves) 4-wide chains up to 64
    const int step = pre_inv ? 64 : RC;
    for (int64_t c0 = 0; c0 < nrhs; c0 += step) {
      const int nc = (int)(nrhs - c0 < step ? nrhs - c0 : step);
      const int nch = (nc <= 4 || pre_inv) ? (nc + 3) / 4 : (nc + 15) / 16;
      int* flags = base + kWsFlagsSkip;
      int* ctr = flags + nch * nb;
      T* bc = b + c0 * ldb;
      GB_CUDA_TRY(cudaMemsetAsync(flags, 0, (size_t)(nch * nb + nch) * sizeof(int), s));
      const double fl = (double)n * (n + 1) * nc, by = (double)n * (n + 1) / 2.0 * sizeof(T) + 2.0 * n * nc * sizeof(T);
      ProfScope ps(kf.c_str(), s, fl, by);
      // a caller that supplies the inverses solves one panel of a blocked solve: chains of 4 spread
      // its few row blocks' FP64 work over more SMs
      const bool narrow = pre_inv != nullptr;
      if (bwd) {
        if (upper) launch_sweep<T, true, true>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s, narrow);
        else launch_sweep<T, false, true>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s, narrow);
      } else {
        if (upper) launch_sweep<T, true, false>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s, narrow);
        else launch_sweep<T, false, false>(nb, a, lda, n, bc, ldb, nc, inv, flags, ctr, err, s, narrow);
      }
    }
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

template <typename T>
int ldlt_sweeps_ws(bool upper, int64_t n, int64_t nrhs, const T* a, int64_t lda, T* b, int64_t ldb, void* ws,
                   cudaStream_t s) {
  return sweeps_ws<T>(upper, true, n, nrhs, a, lda, b, ldb, ws, s);
}

// Failure-detection self-test: one forward FP64 sweep and one forward FP32 sweep of order 256
// whose ticket counters start at 1 and whose grids leave block 0 out, so that no CTA ever solves
// block 0 and every other block waits for a value that is never published.  The first wait gives
// up after wait_ns and sets the error word; the others see the word (or time out themselves) and
// give up too, and every block that gave up writes NaN into its rows.  Checked: both error words
// set, rows 64..255 NaN, rows 0..63 untouched.  Every access stays inside the buffers: the tickets
// taken are 1..3 of the 4 row blocks, and no kernel goes past its first wait.
int sweep_wait_selftest(unsigned long long wait_ns, cudaStream_t s, int* observed) {
  constexpr int64_t n = 256;
  const int nb = (int)(n / RB);
  const size_t a_bytes = n * n * 8, af_bytes = n * n * 4, b_bytes = 256 * 8;
  const size_t ws64 = (potrs_ws_bytes(n, 8) + 255) & ~(size_t)255, ws32 = (potrs_ws_bytes(n, 4) + 255) & ~(size_t)255;
  char* buf = nullptr;
  if (dev_malloc_async((void**)&buf, a_bytes + af_bytes + 2 * b_bytes + ws64 + ws32, s) != cudaSuccess) {
    cudaGetLastError();
    return GBLLT_ERR_ALLOC;
  }
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{buf, s};
  double* a = (double*)buf;
  float* af = (float*)(buf + a_bytes);
  double* b = (double*)(buf + a_bytes + af_bytes);
  float* bf = (float*)(buf + a_bytes + af_bytes + b_bytes);
  char* w64 = buf + a_bytes + af_bytes + 2 * b_bytes;
  char* w32 = w64 + ws64;
  GB_CUDA_TRY(cudaMemsetAsync(buf, 0, a_bytes + af_bytes + 2 * b_bytes + ws64 + ws32, s));
  std::vector<double> hb(n, 1.0);
  std::vector<float> hbf(n, 1.0f);
  GB_CUDA_TRY(cudaMemcpyAsync(b, hb.data(), n * 8, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(bf, hbf.data(), n * 4, cudaMemcpyHostToDevice, s));
  // FP64: error word | flags (nb) | ticket counter, preset to 1
  int* err64 = potrs_ws_error_word(n, 8, w64);
  int* flags64 = err64 + kWsFlagsSkip;
  int* ctr64 = flags64 + nb;
  const int one = 1;
  GB_CUDA_TRY(cudaMemcpyAsync(ctr64, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  launch_sweep_rc<double, false, false, 4, false>(nb, a, n, n, b, n, 1, (const double*)w64, flags64, ctr64, err64, s,
                                                  wait_ns, nb - 1);
  // FP32: error word, ticket counter (preset to 1) | published words, all not ready
  int* err32 = potrs_ws_error_word(n, 4, w32);
  int* ctr32 = err32 + 1;
  unsigned* words = (unsigned*)(w32 + ws_words_offset(nb));
  GB_CUDA_TRY(cudaMemsetAsync(words, 0xFF, (size_t)nb * RB * 4 * sizeof(unsigned), s));
  GB_CUDA_TRY(cudaMemcpyAsync(ctr32, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  launch_sweep_ll_cpt<false, false, 1, false>(nb, 1, af, n, n, bf, n, 1, (const float*)w32, words, ctr32, err32, s,
                                              wait_ns, nb - 1);
  GB_CUDA_TRY(cudaGetLastError());
  int e64 = 0, e32 = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&e64, err64, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&e32, err32, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(hb.data(), b, n * 8, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(hbf.data(), bf, n * 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  bool rows_ok = true;
  for (int64_t i = 0; i < n; ++i) {
    if (i < RB) rows_ok = rows_ok && hb[i] == 1.0 && hbf[i] == 1.0f;
    else rows_ok = rows_ok && std::isnan(hb[i]) && std::isnan(hbf[i]);
  }
  *observed = (e64 && e32) ? GBLLT_ERR_TIMEOUT : GBLLT_SUCCESS;
  if (!(e64 && e32 && rows_ok)) {
    char msg[160];
    snprintf(msg, sizeof msg, "wait self-test: error words %d/%d, rows %s", e64, e32,
             rows_ok ? "as expected" : "not as expected");
    set_error_message(msg);
    return GBLLT_ERR_INTERNAL;
  }
  return GBLLT_SUCCESS;
}

template int potrs_ws<double>(bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, void*, cudaStream_t);
template int potrs_ws<float>(bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, void*, cudaStream_t);
template int ldlt_sweeps_ws<double>(bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, void*,
                                    cudaStream_t);
template int ldlt_sweeps_ws<float>(bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, void*, cudaStream_t);
template int trsm_sweep_ws<double>(bool, bool, bool, int64_t, int64_t, const double*, int64_t, double*, int64_t, void*,
                                   cudaStream_t, int*, const double*);
template int trsm_sweep_ws<float>(bool, bool, bool, int64_t, int64_t, const float*, int64_t, float*, int64_t, void*,
                                  cudaStream_t, int*, const float*);

}  // namespace gbllt
