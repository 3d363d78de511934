// Tensor-core trailing update for the mixed-precision factorisation:
//
//     C (fp32, column-major) -= sum_s  A_s * B_s^T          (lower tiles only for a SYRK)
//
// This replaces the rank update A22 -= A21 A21^T of llt_inplace::blocked (LLT.h:365 ->
// GeneralMatrixMatrixTriangular.h:57-194, gebp_kernel GeneralBlockPanelKernel.h:1548+) by
// Blackwell 5th-generation tensor-core tiles:
//   - operands are K-major (row r holds its K values contiguously) BF16 or TF32 copies of the
//     panel, streamed by TMA (cp.async.bulk.tensor, 128-byte swizzle) into a 4-stage shared
//     memory ring guarded by mbarriers;
//   - one elected thread issues tcgen05.mma (M = 128, N = 128, K = 16 for bf16 / 8 for tf32),
//     accumulating in TMEM; the grid is persistent (one CTA per SM walks many tiles) and the
//     accumulator is double-buffered (2 x 128 fp32 TMEM columns), so one tile's epilogue overlaps
//     the next tile's loads and MMAs;
//   - four epilogue warps read the accumulator with tcgen05.ld, 32 columns at a time, and apply
//     C -= acc with coalesced column-major loads and stores.
// Split precision: the K loop runs over up to eight segments, each pairing one part of A with one
// part of B, where the parts are successive roundings of the same values (hi = round(x),
// mid = round(x - hi), lo = round(x - hi - mid)); e.g. hi*hi^T + hi*lo^T + lo*hi^T for a two-way
// split, accumulated in one TMEM tile (Markidis et al. 2018, Ootomo & Yokota 2022: split-precision
// products), smallest terms first.
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
constexpr int BN = 128;
constexpr int STAGES = 4;
constexpr int ROW_BYTES = 128;                 // one swizzle atom row: 64 bf16 or 32 tf32
constexpr int A_STAGE = BM * ROW_BYTES;        // 16 KB
constexpr int B_STAGE = BN * ROW_BYTES;        // 16 KB
constexpr int SMEM_BYTES = STAGES * (A_STAGE + B_STAGE) + 1024;
// Instruction descriptor of this kernel's M = BM, N = BN tile.
__host__ __device__ constexpr uint32_t instr_desc(uint32_t fmt) { return instr_desc_mn(fmt, BM, BN); }

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
  int mt;              // tiles along m
  long long tiles;     // tiles in the launch
  int* err;            // device error word (set to 1 on a timeout)
};

struct TcMaps {
  CUtensorMap a[3];    // parts of A (hi, mid, lo)
  CUtensorMap b[3];    // parts of B
};

// Persistent: each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...  The accumulator is
// double-buffered in TMEM (2 x BN columns), so the epilogue of one tile overlaps the TMA loads and
// MMAs of the next.
template <int KIND>
__global__ void __launch_bounds__(192, 1) tc_update_kernel(const __grid_constant__ TcMaps maps, const TcParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t tfull[2];   // accumulator ready for the epilogue
  __shared__ __align__(8) uint64_t tempty[2];  // accumulator drained by the epilogue (4 warps arrive)
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int abort_s;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int KE = KIND == 0 ? 64 : 32;   // elements per 128-byte row
  constexpr int KI = KIND == 0 ? 16 : 8;    // K of one MMA instruction
  constexpr int MMAS = ROW_BYTES / (KI * (KIND == 0 ? 2 : 4));
  const int kpb = (p.k + KE - 1) / KE;      // k-blocks per segment
  const int nk = kpb * p.nseg;

  auto coords = [&](long long t, int& row0, int& col0) {
    int ti, tj;
    if (p.lower == 1) lower_tile_coords(t, ti, tj);
    else { ti = (int)(t % p.mt); tj = (int)(t / p.mt); }
    row0 = ti * BM;
    col0 = tj * BN;
  };

  if (threadIdx.x == 0) {
    abort_s = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 4);
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
    // ---- TMA producer
    long long it = 0, issued = 0;
    for (long long t = blockIdx.x; t < p.tiles && !abort_s; t += gridDim.x) {
      int row0, col0;
      coords(t, row0, col0);
      for (int kk = 0; kk < nk; ++kk, ++it) {
        const int s = (int)(it % STAGES);
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_s)) break;
        const int seg = kk / kpb;
        const int kx = (kk % kpb) * KE;
        const uint32_t code = (p.seg_code >> (4 * seg)) & 0xFu;
        uint8_t* sa = smem + s * (A_STAGE + B_STAGE);
        uint8_t* sb = sa + A_STAGE;
        mbar_expect_tx(&full_bar[s], A_STAGE + B_STAGE);
        tma_load_2d(sa, &maps.a[code & 3u], &full_bar[s], kx, p.a_row0 + row0);
        tma_load_2d(sb, &maps.b[code >> 2], &full_bar[s], kx, p.b_row0 + col0);
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
    // ---- MMA issuer
    constexpr uint32_t idesc = instr_desc(KIND == 0 ? 1u : 2u);
    long long it = 0;
    int local = 0;
    for (long long t = blockIdx.x; t < p.tiles && !abort_s; t += gridDim.x, ++local) {
      const int acc = local & 1;
      const uint32_t use = (uint32_t)(local >> 1);
      if (!mbar_wait(&tempty[acc], (use & 1u) ^ 1u, &abort_s)) break;
      tc_fence_after();
      const uint32_t d_tmem = tmem + (uint32_t)(acc * BN);
      bool ok = true;
      for (int kk = 0; kk < nk; ++kk, ++it) {
        const int s = (int)(it % STAGES);
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, &abort_s)) { ok = false; break; }
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + s * (A_STAGE + B_STAGE));
        const uint64_t ad = sw128_desc(sa), bd = sw128_desc(sa + A_STAGE);
#pragma unroll
        for (int j = 0; j < MMAS; ++j) {
          // advance 32 bytes along K inside the swizzle atom: +2 in the (addr >> 4) field
          mma<KIND>(d_tmem, ad + 2 * j, bd + 2 * j, idesc, (kk > 0 || j > 0) ? 1u : 0u);
        }
        mma_commit(&empty_bar[s]);
      }
      if (!ok) break;
      mma_commit(&tfull[acc]);
    }
  } else if (warp >= 2) {
    // ---- epilogue: C -= acc, one row of the tile per thread
    const int q = warp & 3;                 // TMEM lane quadrant this warp may access
    const int r = q * 32 + lane;            // tile row
    int local = 0;
    for (long long t = blockIdx.x; t < p.tiles && !abort_s; t += gridDim.x, ++local) {
      int row0, col0;
      coords(t, row0, col0);
      const long long gi = (long long)row0 + r;
      const int acc = local & 1;
      const uint32_t use = (uint32_t)(local >> 1);
      const bool row_ok = gi < p.m;
      float* crow = p.c + (long long)col0 * p.ldc + gi;  // C(gi, col0)
      if (!mbar_wait(&tfull[acc], use & 1u, &abort_s)) break;
      tc_fence_after();
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
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
    if (cudaFuncGetAttributes(&fa, tc_update_kernel<0>) == cudaSuccess) stat = fa.sharedSizeBytes;
    if (cudaFuncGetAttributes(&fa, tc_update_kernel<1>) == cudaSuccess && fa.sharedSizeBytes > stat)
      stat = fa.sharedSizeBytes;
    cudaGetLastError();
    c.smem_optin = optin - (int)stat - 64;
    if (c.smem_optin < SMEM_BYTES) c.smem_optin = SMEM_BYTES;
    if (cudaFuncSetAttribute(tc_update_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, c.smem_optin) !=
            cudaSuccess ||
        cudaFuncSetAttribute(tc_update_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, c.smem_optin) !=
            cudaSuccess) {
      set_last_error(cudaGetLastError(), "cudaFuncSetAttribute(tc_update_kernel)", __FILE__, __LINE__);
      c.rc = GBLLT_ERR_CUDA;
    }
    done[dev] = true;
  }
  return c;
}

// 2-D map over a K-major operand: `rows` rows of `k` elements, `ld` elements apart.
int make_map(CUtensorMap* m, const void* base, int kind, int64_t rows, int64_t k, int64_t ld) {
  const int es = kind == 0 ? 2 : 4;
  return make_map_2d(m, base, kind == 0 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, es,
                     rows, k, ld, ROW_BYTES / es, BM)
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
  TcMaps maps;
  int rc;
  for (int i = 0; i < 3; ++i) {
    const void* pa = a.parts[i] ? a.parts[i] : a.parts[0];
    const void* pb = b.parts[i] ? b.parts[i] : b.parts[0];
    if (((uintptr_t)pa & 15) || ((uintptr_t)pb & 15)) return GBLLT_ERR_INTERNAL;
    if ((rc = make_map(&maps.a[i], pa, kind, a.rows, a.k, a.ld))) return rc;
    if ((rc = make_map(&maps.b[i], pb, kind, b.rows, b.k, b.ld))) return rc;
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
  p.mt = (int)ceil_div(m, BM);
  p.err = d_err;
  const int64_t nt = ceil_div(n, BN);
  p.tiles = lower == 1 ? (int64_t)p.mt * (p.mt + 1) / 2 : (int64_t)p.mt * nt;
  const TcDevCfg& cfg = tc_cfg();
  if (cfg.rc) return cfg.rc;
  const int sms = cfg.sms;
  int usable = sms;
  size_t smem = SMEM_BYTES;
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
               ((double)(m + (lower == 1 ? 0 : n)) * a.k * nseg * es) + entries * 8.0);
  if (kind == 0) {
    tc_update_kernel<0><<<grid, 192, smem, s>>>(maps, p);
  } else {
    tc_update_kernel<1><<<grid, 192, smem, s>>>(maps, p);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GBLLT_SUCCESS;
}

}  // namespace gbllt
