// Mixed-model fit for callers that cannot allocate device memory.
//
// pcgb_multi_run needs one 32-bit word of device scratch: the work counter
// from which the persistent kernel's warps claim chunks of voxels. Most
// callers pass a word they allocated. Some cannot: hosts whose device memory
// is owned by another framework's pool allocator that hands out only the
// buffers it manages, and embedded or long-running services that reserve
// their memory at start-up and must not grow it afterwards. For them, this
// file keeps the counter in a statically allocated device array that the
// library owns, so a fit needs no allocation at all; the caller still passes
// every input and output.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "pcgb.h"

namespace {

// The scratch of every no-allocation fit: word 0 is the work counter. Sized
// to one 256-byte block (64 words); every GPU that loads the library holds
// these 256 bytes until the process exits.
constexpr int kScratchWords = 64;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// The counter claims chunk indices up to (chunks + warps in the grid); keeping
// the chunk count at or below 2^31 leaves the upper half of its 32-bit range
// for those final claims, so the counter cannot wrap. pcgb_multi_run enforces
// the same limit.
constexpr int64_t kMaxChunks = int64_t(1) << 31;
constexpr int kMaxDevices = 64;

// The array's device address belongs to one CUDA context. It is cached per
// device together with that context's process-unique id (cuCtxGetId), so a
// call made after cudaDeviceReset, or under another context made current
// through the driver API, looks the address up again instead of using a
// stale one.
struct ScratchSlot {
  uint32_t* ptr = nullptr;
  unsigned long long ctx_id = 0;
};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

std::mutex g_mu;
ScratchSlot g_slot[kMaxDevices];
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
thread_local std::string g_err;

int fail(int code, const char* msg) {
  g_err = msg;
  return code;
}

// Driver entry points through the runtime (the library links no libcuda).
int driver_fns() {
  if (g_ctx_get_current && g_ctx_get_id) return PCGB_OK;
  void* f1 = nullptr;
  void* f2 = nullptr;
  cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
  if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
  if (e != cudaSuccess) return fail(PCGB_ECUDA, cudaGetErrorString(e));
  if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
    return fail(PCGB_ECUDA, "the CUDA driver provides no cuCtxGetCurrent / cuCtxGetId");
  g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
  g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  return PCGB_OK;
}

// Device address of the scratch array in the current device's current
// context: looked up (with that device current) the first time and whenever
// the context differs from the one of the cached address.
int scratch_for_current_device(uint32_t** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PCGB_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PCGB_ERANGE, "device index beyond the supported 64 devices");
  // makes the device's primary context current when no context is (the
  // runtime does this lazily; a no-op otherwise)
  e = cudaFree(nullptr);
  if (e != cudaSuccess) return fail(PCGB_ECUDA, cudaGetErrorString(e));
  std::lock_guard<std::mutex> lock(g_mu);
  if (int rc = driver_fns()) return rc;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_get_id(ctx, &id) != CUDA_SUCCESS)
    return fail(PCGB_ECUDA, "no current CUDA context");
  ScratchSlot& s = g_slot[dev];
  if (!s.ptr || s.ctx_id != id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return fail(PCGB_ECUDA, e != cudaSuccess ? cudaGetErrorString(e) : "null symbol address");
    s.ptr = static_cast<uint32_t*>(p);
    s.ctx_id = id;
  }
  *out = s.ptr;
  return PCGB_OK;
}

}  // namespace

extern "C" {

const char* pcgb_noalloc_last_error(void) { return g_err.c_str(); }

int pcgb_multi_run_noalloc(pcgb_multi* program, const pcgb_multi_job* jobs, int n_jobs, const int* order, int iters,
                           double tol, double mu, double eta, double acc, double dec, int chunk, int grid,
                           void* stream) {
  g_err.clear();
  if (!jobs || n_jobs < 1 || n_jobs > 8) return fail(PCGB_EINVAL, "need 1..8 jobs");
  if (chunk < 32 || chunk % 32 || chunk > 4096) return fail(PCGB_EINVAL, "chunk must be a multiple of 32 up to 4096");
  int64_t chunks = 0;
  for (int k = 0; k < n_jobs; ++k) {
    const int64_t n = jobs[k].nprobs;
    if (n < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
    chunks += n / chunk + (n % chunk != 0);  // no overflow: each term <= 2^58, the sum is checked per job
    if (chunks > kMaxChunks)
      return fail(PCGB_ERANGE,
                  "too many voxels for the library-owned work counter: at most 2^31 chunks per call "
                  "(use a larger chunk, split the call, or pcgb_multi_run with your own counter)");
  }
  uint32_t* scratch = nullptr;
  if (int rc = scratch_for_current_device(&scratch)) return rc;
  // pcgb_multi_run clears the counter (cudaMemsetAsync on this stream) before its launch
  const int rc = pcgb_multi_run(program, jobs, n_jobs, order, iters, tol, mu, eta, acc, dec, chunk, grid, scratch,
                                stream);
  if (rc) g_err = pcgb_last_error();
  return rc;
}

}  // extern "C"
