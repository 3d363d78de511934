// Tensor-core trailing update for the mixed-precision factorisation:
//
//     C (fp32, column-major) -= sum_s  A_s * B_s^T          (lower tiles only for a SYRK)
//
// This replaces the rank update A22 -= A21 A21^T of llt_inplace::blocked (LLT.h:365 ->
// GeneralMatrixMatrixTriangular.h:57-194, gebp_kernel GeneralBlockPanelKernel.h:1548+) by
// Blackwell 5th-generation tensor-core tiles:
//   - operands are K-major (row r holds its K values contiguously) BF16 or TF32 copies of the
//     panel in NP parts (successive roundings of the same values: hi = round(x), mid =
//     round(x - hi), lo = round(x - hi - mid)).  Every part of A and of B for one 64-byte K-block
//     is streamed once by TMA (cp.async.bulk.tensor, 64-byte swizzle) into one stage of a shared
//     memory ring guarded by mbarriers, and all the split products of that K-block are issued from
//     it: a 3-part split runs 6 products on each byte it loads;
//   - one elected thread issues tcgen05.mma (M = 128, N = BN = 128 or 256, K = 16 for bf16 / 8 for
//     tf32), accumulating in TMEM; the grid is persistent (one CTA per SM walks many tiles) and the
//     accumulator is double-buffered (2 x BN fp32 TMEM columns), so one tile's epilogue overlaps
//     the next tile's loads and MMAs;
//   - eight epilogue warps (two per TMEM lane quadrant, each half of the columns) read the
//     accumulator with tcgen05.ld, 32 columns at a time, and apply C -= acc with coalesced
//     column-major loads and stores.
// Split precision (Markidis et al. 2018, Ootomo & Yokota 2022): up to eight segments, each pairing
// one part of A with one part of B, accumulated in one TMEM tile.  The tensor cores' FP32
// accumulation aligns each step's products to the running sum, so small terms added to a large
// sum lose low bits.  A tile therefore runs two passes over K when the last segment is hi*hi: the
// cross terms of every K-block first (the sum stays small), then hi*hi with only the hi parts
// loaded, NP K-blocks to a stage (one K-block's hi parts would feed too few MMAs to cover the
// copies' latency with the ring's few stages).  A 128 x 256 tile of a 3-part split then performs
// 128 flops per byte it loads (170 in one pass), against 64 for a 128 x 128 tile that loads one
// part pair per product.
//
// Every mbarrier wait is bounded; on timeout the kernel raises an error flag, waits (bounded)
// for its own TMA copies, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "internal.h"
#include <mutex>

#include "tc_gemm.h"
#include "tc_ptx.cuh"

namespace gbllt {

namespace {

using namespace tcptx;

constexpr int BM = 128;
constexpr int ROW_BYTES = 64;                    // one 64-byte swizzle row: 32 bf16 or 16 tf32
constexpr int SMEM_RING = 216 * 1024;           // operand ring (stages of all parts of one K-block)
constexpr int THREADS = 320;                     // TMA warp, MMA warp, eight epilogue warps

template <int BN, int NP>
struct TcShape {
  static constexpr int A_PART = BM * ROW_BYTES;                  // 8 KB
  static constexpr int B_PART = BN * ROW_BYTES;                  // 8 or 16 KB
  static constexpr int STAGE = NP * (A_PART + B_PART);
  static constexpr int STAGES = SMEM_RING / STAGE > 8 ? 8 : SMEM_RING / STAGE;
  static constexpr int SMEM = STAGES * STAGE + 1024;             // + alignment slack
  static_assert(STAGES >= 2, "ring too small");
};

struct TcParams {
  float* c;
  long long ldc;
  int m, n;            // C is m x n; A rows [a_row0, a_row0 + m), B rows [b_row0, b_row0 + n)
  int a_row0, b_row0;
  int k;               // depth of one segment (elements)
  int nseg;            // 1..8
  uint32_t seg_code;   // 4 bits per segment s: bits [4s, 4s+2) = part of A, [4s+2, 4s+4) = part of B
  int lower;           // 0: every tile of the m x n rectangle; 1: lower-triangle tiles of a square (SYRK);
                       // 2: every tile of the rectangle; with 1 and 2 only entries with
                       // row + diag >= column are written
  int diag;            // 0 except for an offset lower rectangle (lower == 2)
  int two_pass;        // segments 0 .. nseg-2 over all of K, then the last (hi*hi) over all of K
  int mt;              // tiles along m
  long long tiles;     // tiles in the launch
  int* err;            // device error word (set to 1 on a timeout)
};

struct TcMaps {
  CUtensorMap a[3];    // parts of A (hi, mid, lo); box 64 bytes x BM rows
  CUtensorMap b[3];    // parts of B; box 64 bytes x BN rows
};

// Tile t of the launch -> (row0, col0).  lower == 1: the tiles of a square's lower triangle, column
// by column (tile column tj starts at tile row tj * BN / BM); otherwise column-major over mt rows.
template <int BN>
__device__ __forceinline__ void tile_coords(const TcParams& p, long long t, int& row0, int& col0) {
  int ti, tj;
  if (p.lower == 1) {
    constexpr int R = BN / BM;  // tile rows per tile column width
    tj = 0;
    long long cnt = p.mt;      // tiles in column 0
    while (t >= cnt) {
      t -= cnt;
      ++tj;
      cnt = p.mt - (long long)tj * R;
    }
    ti = tj * R + (int)t;
  } else {
    ti = (int)(t % p.mt);
    tj = (int)(t / p.mt);
  }
  row0 = ti * BM;
  col0 = tj * BN;
}

// Persistent: each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...
template <int KIND, int BN, int NP>
__global__ void __launch_bounds__(THREADS, 1) tc_update_kernel(const __grid_constant__ TcMaps maps, const TcParams p) {
  using S = TcShape<BN, NP>;
  constexpr int STAGES = S::STAGES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t tfull[2];   // accumulator ready for the epilogue
  __shared__ __align__(8) uint64_t tempty[2];  // accumulator drained by the epilogue (8 warps arrive)
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int KE = ROW_BYTES / (KIND == 0 ? 2 : 4);  // elements per K-block
  constexpr int KI = KIND == 0 ? 16 : 8;               // K of one MMA instruction
  constexpr int MMAS = KE / KI;                        // MMAs per K-block and segment (2)
  const int nk = (p.k + KE - 1) / KE;                  // K-blocks
  // stages per tile: one per K-block; in a second (hi*hi) pass each stage carries the hi parts of
  // NP K-blocks in its NP part slots, so that pass keeps as many MMAs in flight per stage
  const int nk2 = p.two_pass ? (nk + NP - 1) / NP : 0;
  const int nkt = nk + nk2;

  if (threadIdx.x == 0) {
    abort_s = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 8);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(2 * BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer: all NP parts of A and B for one K-block per stage
    long long it = 0, issued = 0;
    for (long long t = blockIdx.x; t < p.tiles && !abort_s; t += gridDim.x) {
      int row0, col0;
      tile_coords<BN>(p, t, row0, col0);
      for (int kt = 0; kt < nkt; ++kt, ++it) {
        const int s = (int)(it % STAGES);
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_s)) break;
        uint8_t* st = smem + s * S::STAGE;
        if (kt < nk) {  // all NP parts of K-block kt, part q in slot q
          mbar_expect_tx(&full_bar[s], NP * (S::A_PART + S::B_PART));
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            tma_load_2d(st + q * S::A_PART, &maps.a[q], &full_bar[s], kt * KE, p.a_row0 + row0);
            tma_load_2d(st + NP * S::A_PART + q * S::B_PART, &maps.b[q], &full_bar[s], kt * KE, p.b_row0 + col0);
          }
        } else {  // second pass: the hi parts of K-blocks kb0 .. kb0 + nq - 1, K-block kb0 + q in slot q
          const int kb0 = (kt - nk) * NP;
          const int nq = nk - kb0 < NP ? nk - kb0 : NP;
          mbar_expect_tx(&full_bar[s], nq * (S::A_PART + S::B_PART));
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            if (q < nq) {
              tma_load_2d(st + q * S::A_PART, &maps.a[0], &full_bar[s], (kb0 + q) * KE, p.a_row0 + row0);
              tma_load_2d(st + NP * S::A_PART + q * S::B_PART, &maps.b[0], &full_bar[s], (kb0 + q) * KE,
                          p.b_row0 + col0);
            }
          }
        }
        issued = it + 1;
      }
    }
    if (abort_s) {
      // let the copies this thread started land before the CTA exits (bounded)
      for (long long i = issued - STAGES < 0 ? 0 : issued - STAGES; i < issued; ++i) {
        volatile int dummy = 0;
        mbar_wait(&full_bar[i % STAGES], (uint32_t)(i / STAGES) & 1u, &dummy);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer: every segment of each K-block from the one stage that holds its parts
    constexpr uint32_t idesc = instr_desc_mn(KIND == 0 ? 1u : 2u, BM, BN);
    long long it = 0;
    int local = 0;
    for (long long t = blockIdx.x; t < p.tiles && !abort_s; t += gridDim.x, ++local) {
      const int acc = local & 1;
      const uint32_t use = (uint32_t)(local >> 1);
      if (!mbar_wait(&tempty[acc], (use & 1u) ^ 1u, &abort_s)) break;
      tc_fence_after();
      const uint32_t d_tmem = tmem + (uint32_t)(acc * BN);
      bool ok = true;
      for (int kt = 0; kt < nkt; ++kt, ++it) {
        const int s = (int)(it % STAGES);
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_s)) { ok = false; break; }
        tc_fence_after();
        const uint32_t st = smem_u32(smem + s * S::STAGE);
        if (kt < nk) {
          // one pass: every segment; two passes: segments 0 .. nseg-2 here, the last one (hi*hi) below
          const int seg1 = p.two_pass ? p.nseg - 1 : p.nseg;
          for (int seg = 0; seg < seg1; ++seg) {
            const uint32_t code = (p.seg_code >> (4 * seg)) & 0xFu;
            const uint64_t ad = sw64_desc(st + (code & 3u) * S::A_PART);
            const uint64_t bd = sw64_desc(st + NP * S::A_PART + (code >> 2) * S::B_PART);
#pragma unroll
            for (int j = 0; j < MMAS; ++j) {
              // advance 32 bytes along K inside the 64-byte swizzle row: +2 in the (addr >> 4) field
              mma<KIND>(d_tmem, ad + 2 * j, bd + 2 * j, idesc, (kt > 0 || seg > 0 || j > 0) ? 1u : 0u);
            }
          }
        } else {  // second pass: hi*hi of the K-blocks held in the stage's slots
          const int kb0 = (kt - nk) * NP;
          const int nq = nk - kb0 < NP ? nk - kb0 : NP;
          for (int q = 0; q < nq; ++q) {
            const uint64_t ad = sw64_desc(st + q * S::A_PART);
            const uint64_t bd = sw64_desc(st + NP * S::A_PART + q * S::B_PART);
#pragma unroll
            for (int j = 0; j < MMAS; ++j) mma<KIND>(d_tmem, ad + 2 * j, bd + 2 * j, idesc, 1u);
          }
        }
        mma_commit(&empty_bar[s]);
      }
      if (!ok) break;
      mma_commit(&tfull[acc]);
    }
  } else if (warp >= 2) {
    // ---- epilogue: C -= acc, one row of the tile per thread, half of the columns per warp
    const int q = warp & 3;                 // TMEM lane quadrant this warp may access
    const int half = (warp - 2) >> 2;       // warps 2-5: columns [0, BN/2), warps 6-9: [BN/2, BN)
    const int r = q * 32 + lane;            // tile row
    int local = 0;
    for (long long t = blockIdx.x; t < p.tiles && !abort_s; t += gridDim.x, ++local) {
      int row0, col0;
      tile_coords<BN>(p, t, row0, col0);
      const long long gi = (long long)row0 + r;
      const int acc = local & 1;
      const uint32_t use = (uint32_t)(local >> 1);
      const bool row_ok = gi < p.m;
      float* crow = p.c + (long long)col0 * p.ldc + gi;  // C(gi, col0)
      if (!mbar_wait(&tfull[acc], use & 1u, &abort_s)) break;
      tc_fence_after();
#pragma unroll 1
      for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
        // 32 independent loads of this thread's row segment (coalesced across the warp), then the
        // matching 32 accumulator columns; this epilogue overlaps the next tile's main loop
        float cv[32];
        const int jmax = (int)min((long long)32, (long long)p.n - (col0 + c0));
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const long long gj = (long long)col0 + c0 + j;
          cv[j] = (row_ok && j < jmax && (!p.lower || gi + p.diag >= gj)) ? crow[(long long)(c0 + j) * p.ldc] : 0.f;
        }
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * BN + c0), v);
        if (row_ok) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const long long gj = (long long)col0 + c0 + j;
            if (j < jmax && (!p.lower || gi + p.diag >= gj)) crow[(long long)(c0 + j) * p.ldc] = cv[j] - v[j];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && abort_s) atomicExch(p.err, 1);
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
  }
}

// The kernel instantiations: KIND (bf16, tf32) x BN (128, 256) x NP (1..3 parts).
using KernelFn = void (*)(const TcMaps, const TcParams);
template <int KIND, int BN, int NP>
constexpr KernelFn kfn() {
  return tc_update_kernel<KIND, BN, NP>;
}
template <int BN, int NP>
constexpr int kernel_smem() {
  return TcShape<BN, NP>::SMEM;
}
constexpr int kVariants = 12;
inline int variant_index(int kind, int bn, int np) { return kind * 6 + (bn == 256 ? 3 : 0) + (np - 1); }
const KernelFn kKernels[kVariants] = {
    kfn<0, 128, 1>(), kfn<0, 128, 2>(), kfn<0, 128, 3>(), kfn<0, 256, 1>(), kfn<0, 256, 2>(), kfn<0, 256, 3>(),
    kfn<1, 128, 1>(), kfn<1, 128, 2>(), kfn<1, 128, 3>(), kfn<1, 256, 1>(), kfn<1, 256, 2>(), kfn<1, 256, 3>()};
const int kSmem[kVariants] = {kernel_smem<128, 1>(), kernel_smem<128, 2>(), kernel_smem<128, 3>(),
                              kernel_smem<256, 1>(), kernel_smem<256, 2>(), kernel_smem<256, 3>(),
                              kernel_smem<128, 1>(), kernel_smem<128, 2>(), kernel_smem<128, 3>(),
                              kernel_smem<256, 1>(), kernel_smem<256, 2>(), kernel_smem<256, 3>()};

// Per-device launch configuration of the update kernels, set up once per device under a lock
// (calls may come from several host threads): SM count, the largest dynamic shared-memory request
// (the per-block limit less the kernels' static shared memory), and the kernels' attribute raised
// to it.
struct TcDevCfg {
  int sms = 0;
  int smem_optin = 0;
  int rc = 0;
};

const TcDevCfg& tc_cfg() {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static TcDevCfg cfg[kMaxDev];
  static bool done[kMaxDev] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
    cudaGetLastError();
    dev = 0;
  }
  std::lock_guard<std::mutex> lk(mu);
  TcDevCfg& c = cfg[dev];
  if (!done[dev]) {
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
    if (c.sms <= 0) c.sms = 1;
    size_t stat = 0;
    cudaFuncAttributes fa;
    for (int v = 0; v < kVariants; ++v)
      if (cudaFuncGetAttributes(&fa, kKernels[v]) == cudaSuccess && fa.sharedSizeBytes > stat) stat = fa.sharedSizeBytes;
    cudaGetLastError();
    c.smem_optin = optin - (int)stat - 64;
    for (int v = 0; v < kVariants && !c.rc; ++v) {
      if (kSmem[v] > c.smem_optin) {
        set_error_message("tc_update: the device's shared memory per block is too small for the update kernel");
        c.rc = GBLLT_ERR_INTERNAL;
      } else if (cudaFuncSetAttribute(kKernels[v], cudaFuncAttributeMaxDynamicSharedMemorySize, c.smem_optin) !=
                 cudaSuccess) {
        set_last_error(cudaGetLastError(), "cudaFuncSetAttribute(tc_update_kernel)", __FILE__, __LINE__);
        c.rc = GBLLT_ERR_CUDA;
      }
    }
    done[dev] = true;
  }
  return c;
}

// 2-D map over a K-major operand: `rows` rows of `k` elements, `ld` elements apart; box = one
// 64-byte row segment x box_rows rows, 64-byte swizzle.
int make_map(CUtensorMap* m, const void* base, int kind, int64_t rows, int64_t k, int64_t ld, int box_rows) {
  const int es = kind == 0 ? 2 : 4;
  return make_map_2d(m, base, kind == 0 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, es,
                     rows, k, ld, ROW_BYTES / es, box_rows, CU_TENSOR_MAP_SWIZZLE_64B)
             ? GBLLT_SUCCESS
             : GBLLT_ERR_INTERNAL;
}

}  // namespace

int tc_update(const TcOperand& a, const TcOperand& b, int kind, int nseg, uint32_t seg_code, float* c, int64_t ldc,
              int64_t m, int64_t n, int lower, int* d_err, cudaStream_t s, int reserve_sms, int max_ctas,
              int diag) {
  if (m <= 0 || n <= 0 || a.k <= 0) return GBLLT_SUCCESS;
  if (nseg < 1 || nseg > 8) return GBLLT_ERR_INTERNAL;
  const int es = kind == 0 ? 2 : 4;
  if ((a.ld * es) % 16 != 0 || (b.ld * es) % 16 != 0) return GBLLT_ERR_INTERNAL;
  // parts the segments use: NP = 1 + the largest part index of A or B
  int np = 1;
  for (int sg = 0; sg < nseg; ++sg) {
    const uint32_t code = (seg_code >> (4 * sg)) & 0xFu;
    const int pa = (int)(code & 3u), pb = (int)(code >> 2);
    if (pa > 2 || pb > 2) return GBLLT_ERR_INTERNAL;
    np = pa + 1 > np ? pa + 1 : np;
    np = pb + 1 > np ? pb + 1 : np;
  }
  // 256-wide tiles, except for a C of at most 128 columns
  const int bn = n <= 128 ? 128 : 256;
  TcMaps maps;
  int rc;
  for (int i = 0; i < 3; ++i) {
    const void* pa = a.parts[i] ? a.parts[i] : a.parts[0];
    const void* pb = b.parts[i] ? b.parts[i] : b.parts[0];
    if (((uintptr_t)pa & 15) || ((uintptr_t)pb & 15)) return GBLLT_ERR_INTERNAL;
    if ((rc = make_map(&maps.a[i], pa, kind, a.rows, a.k, a.ld, BM))) return rc;
    if ((rc = make_map(&maps.b[i], pb, kind, b.rows, b.k, b.ld, bn))) return rc;
  }
  TcParams p;
  p.c = c;
  p.ldc = ldc;
  p.m = (int)m;
  p.n = (int)n;
  p.a_row0 = (int)a.row0;
  p.b_row0 = (int)b.row0;
  p.k = (int)a.k;
  p.nseg = nseg;
  p.seg_code = seg_code;
  p.lower = lower;
  p.diag = lower == 1 ? 0 : diag;
  // two passes when the last segment is hi*hi (the split tables put it last)
  p.two_pass = (nseg > 1 && ((seg_code >> (4 * (nseg - 1))) & 0xFu) == 0u) ? 1 : 0;
  p.mt = (int)ceil_div(m, BM);
  p.err = d_err;
  const int64_t nt = ceil_div(n, bn);
  if (lower == 1) {  // tile column tj holds the tile rows from tj * bn / BM on
    const int64_t r = bn / BM;
    int64_t tiles = 0;
    for (int64_t tj = 0; tj < nt && tj * r < p.mt; ++tj) tiles += p.mt - tj * r;
    p.tiles = tiles;
  } else {
    p.tiles = (int64_t)p.mt * nt;
  }
  const TcDevCfg& cfg = tc_cfg();
  if (cfg.rc) return cfg.rc;
  const int sms = cfg.sms;
  int usable = sms;
  const int v = variant_index(kind, bn, np);
  size_t smem = (size_t)kSmem[v];
  if (reserve_sms > 0 && reserve_sms < sms) {
    usable = sms - reserve_sms;
    smem = (size_t)cfg.smem_optin;  // one CTA fills its SM's shared memory: nothing else is placed beside it
  }
  if (max_ctas > 0 && max_ctas < usable) usable = max_ctas;
  const unsigned grid = (unsigned)(p.tiles < usable ? p.tiles : usable);
  static const std::string kname[2] = {"tc_update_bf16", "tc_update_tf32"};
  // algorithmic work: 2 k flops per updated entry and segment; operands read once, C read+written
  const double nt_tri = (double)(n - diag > 0 ? n - diag : 0);  // columns that meet the masked corner
  const double entries = lower == 1   ? (double)m * (m + 1) / 2.0
                         : lower == 2 ? (double)m * n - nt_tri * (nt_tri - 1) / 2.0
                                      : (double)m * n;
  ProfScope ps(kname[kind].c_str(), s, 2.0 * entries * a.k * nseg,
               ((double)(m + (lower == 1 ? 0 : n)) * a.k * (np + p.two_pass) * es) + entries * 8.0);
  kKernels[v]<<<grid, THREADS, smem, s>>>(maps, p);
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace gbllt
