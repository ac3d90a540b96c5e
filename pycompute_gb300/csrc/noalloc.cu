// Mixed-model fit for callers that cannot allocate device memory.
//
// pcgb_multi_run needs one 32-bit word of device scratch: the work counter
// from which the persistent kernel's warps claim chunks of voxels. Most
// callers pass a word they allocated. Some cannot: code that runs while a
// CUDA graph is being captured (a cudaMalloc there breaks the capture), hosts
// whose device memory is owned by another framework's pool allocator that
// hands out only the buffers it manages, and embedded callers that must not
// grow their memory after start-up. For them, this file keeps the counter in
// a statically allocated device array that the library owns, so a fit needs
// no allocation at all; the caller still passes every input and output.
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
// for those final claims, so the counter cannot wrap.
constexpr int64_t kMaxChunks = int64_t(1) << 31;
constexpr int kMaxDevices = 64;

std::mutex g_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {};
thread_local std::string g_err;

int fail(int code, const char* msg) {
  g_err = msg;
  return code;
}

// Device address of the scratch array on the current device, looked up once
// per device (with that device current) and cached.
int scratch_for_current_device(uint32_t** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PCGB_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PCGB_ERANGE, "device index beyond the supported 64 devices");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return fail(PCGB_ECUDA, e != cudaSuccess ? cudaGetErrorString(e) : "null symbol address");
    g_scratch_ptr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_scratch_ptr[dev];
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
    if (jobs[k].nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
    chunks += (jobs[k].nprobs + chunk - 1) / chunk;
  }
  if (chunks > kMaxChunks)
    return fail(PCGB_ERANGE,
                "too many voxels for the library-owned work counter: at most 2^31 chunks per call "
                "(use a larger chunk, split the call, or pcgb_multi_run with your own counter)");
  uint32_t* scratch = nullptr;
  if (int rc = scratch_for_current_device(&scratch)) return rc;
  // pcgb_multi_run clears the counter (cudaMemsetAsync on this stream) before its launch
  const int rc = pcgb_multi_run(program, jobs, n_jobs, order, iters, tol, mu, eta, acc, dec, chunk, grid, scratch,
                                stream);
  if (rc) g_err = pcgb_last_error();
  return rc;
}

}  // extern "C"
