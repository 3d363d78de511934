// Mixed-precision solve that allocates nothing.
//
// gbllt_dposv_mixed_dev needs scratch memory next to its inputs and outputs: the rounded FP32
// working matrix, the BF16/TF32 panel operands, residuals, partial sums and a status word.  It
// takes that memory from the stream-ordered pool with cudaMallocAsync.  Some callers cannot let a
// library allocate: an application whose device memory is owned by its own caching allocator or a
// fixed budget (a second allocator in the same process fragments it and escapes its accounting), or
// a plug-in that is handed only the buffers it works on.  For them this entry point runs the same
// solve on a fixed scratch area that is part of the library image: a file-scope __device__ array of
// kScratchBytes, which every GPU that loads the library keeps until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it names a host-side
// stand-in), so the device address is looked up once per device with cudaGetSymbolAddress, with
// that device current, on the first call made on that device.  Make that first call before any
// stream capture begins.
//
// All calls share the one array and it keeps whatever the last call left in it; the solve
// initialises everything it reads before reading it.  Calls whose GPU work overlaps (several
// streams, several host threads, or a second call issued before the first one's work finished)
// race on the array: serialise them.
#include <cstring>
#include <mutex>

#include "internal.h"

namespace gbllt {
namespace {

// 64 MiB: n <= 2048 with 64 right-hand sides and the FP64 fallback, at the default panel width of 256
// (a wider panel widens the panel operands and can push a problem of that size over the limit)
constexpr size_t kScratchBytes = 64ull << 20;
__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_dev[64] = {};

// Device address of g_scratch on the current device (set-up on the first call per device).
int scratch_address(void** out) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return GBLLT_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    GB_CUDA_TRY(cudaGetSymbolAddress(&p, g_scratch));
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
  return GBLLT_SUCCESS;
}

}  // namespace
}  // namespace gbllt

using namespace gbllt;

extern "C" int gbllt_dposv_mixed_dev_noalloc(char uplo, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                                             const double* d_b, int64_t ldb, double* d_x, int64_t ldx,
                                             const gbllt_mixed_opts* opts, gbllt_mixed_report* report,
                                             void* stream) {
  if (check_uplo(uplo)) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (n > 0 && !d_a) return -4;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (n > 0 && nrhs > 0 && !d_b) return -6;
  if (ldb < (n > 1 ? n : 1)) return -7;
  if (n > 0 && nrhs > 0 && !d_x) return -8;
  if (ldx < (n > 1 ? n : 1)) return -9;
  gbllt_mixed_opts o;
  if (resolve_mixed_opts(opts, &o, n)) return -10;
  if (report) memset(report, 0, sizeof *report);
  if (n == 0 || nrhs == 0) return GBLLT_SUCCESS;
  const MixedLayout ly = mixed_layout(n, nrhs, o, false);
  const size_t need = ly.bytes + (o.fallback_fp64 ? ly.fallback_bytes + 256 : 0);
  if (need > kScratchBytes) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "gbllt_dposv_mixed_dev_noalloc: n=%lld, nrhs=%lld needs %zu bytes of scratch%s; the fixed scratch "
             "area holds %zu bytes",
             (long long)n, (long long)nrhs, need, o.fallback_fp64 ? " (with the FP64 fallback)" : "",
             kScratchBytes);
    set_error_message(buf);
    return GBLLT_ERR_SCRATCH_LIMIT;
  }
  int rc = ensure_device();
  if (rc) return rc;
  void* ws = nullptr;
  if ((rc = scratch_address(&ws))) return rc;
  const bool upper = uplo == 'U' || uplo == 'u';
  return posv_mixed_core(upper, n, nrhs, d_a, lda, d_b, ldb, d_x, ldx, o, report, ws, kScratchBytes, false,
                         (cudaStream_t)stream);
}
