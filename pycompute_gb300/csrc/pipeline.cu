// Fit-pipeline kernels around the LM fitter: constant initialisation, and the
// fallback pass of the warm-started fit (flag voxels whose warm fit is not
// trustworthy, compact their indices, refit them from the constant
// initialisation, keep whichever fit has the lower cost).
//
// All arrays are structure-of-arrays with the voxel index fastest, fp32.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "lm_params.h"
#include "pcgb.h"

namespace pcgb_pipe {

thread_local std::string g_err;
int fail(int code, const char* m) {
  g_err = m;
  return code;
}
int cuda_rc() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PCGB_OK : fail(PCGB_ECUDA, cudaGetErrorString(e));
}

struct InitArgs {
  const float* data;
  long long n;
  int m, nparam;
  float values[PCGB_MAX_PARAMS];
  int from_max[PCGB_MAX_PARAMS];
  float* pars;
};

// pars[k][v] = values[k], or max_i data[i][v] where from_max[k]
// (the reference notebooks start S0 from the largest sample).
__global__ void init_constant_kernel(const InitArgs a) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.n) return;
  float mx = -INFINITY;
  for (int i = 0; i < a.m; ++i) mx = fmaxf(mx, a.data[(long long)i * a.n + v]);
  for (int k = 0; k < a.nparam; ++k) a.pars[(long long)k * a.n + v] = a.from_max[k] ? mx : a.values[k];
}

struct FlagArgs {
  const float* pars;
  const float* cost;
  const float* cost_ref;
  long long n;
  int nparam;
  float lb[PCGB_MAX_PARAMS], ub[PCGB_MAX_PARAMS];
  signed char* flags;
  int* idx;
  int* count;
};

// flag = non-finite cost, cost not below cost_ref, or a parameter on a bound
// (the fitter clamps to [lb, ub], so "on a bound" is exact equality).
// Flagged voxel indices are appended to idx with one atomic per warp.
__global__ void flag_compact_kernel(const FlagArgs a) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool flag = false;
  if (v < a.n) {
    const float c = a.cost[v];
    flag = !isfinite(c) || !(c < a.cost_ref[v]);
    for (int k = 0; k < a.nparam; ++k) {
      const float p = a.pars[(long long)k * a.n + v];
      flag = flag || !(p > a.lb[k]) || !(p < a.ub[k]);
    }
    if (a.flags) a.flags[v] = flag ? 1 : 0;
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned ballot = __ballot_sync(0xffffffffu, flag);
  if (!ballot) return;
  int base = 0;
  if (lane == 0) base = atomicAdd(a.count, __popc(ballot));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (flag) a.idx[base + __popc(ballot & ((1u << lane) - 1u))] = int(v);
}

struct PrepArgs {
  const int* idx;
  long long n_items, n;
  int nparam, m;
  float values[PCGB_MAX_PARAMS];
  int from_max[PCGB_MAX_PARAMS];
  float* pars;              // (P, n): warm result in, constant init out for listed voxels
  float* backup;            // (P, n_items) warm result out
  const float* cost;        // (n) warm cost
  float* cost_backup;       // (n_items)
  const float* data;        // (M, n)
  float* lam;               // (n) reset to lam0
  float lam0;
  signed char* step_type;   // (n) reset to 1
  float* f;                 // (n) zeroed (fresh cost accumulator)
};

__global__ void fallback_prepare_kernel(const PrepArgs a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n_items) return;
  const long long v = a.idx[i];
  float mx = -INFINITY;
  for (int s = 0; s < a.m; ++s) mx = fmaxf(mx, a.data[(long long)s * a.n + v]);
  for (int k = 0; k < a.nparam; ++k) {
    a.backup[(long long)k * a.n_items + i] = a.pars[(long long)k * a.n + v];
    a.pars[(long long)k * a.n + v] = a.from_max[k] ? mx : a.values[k];
  }
  a.cost_backup[i] = a.cost[v];
  a.lam[v] = a.lam0;
  a.step_type[v] = 1;
  a.f[v] = 0.f;
}

// keep the refit only where its cost is lower; which[v] = 1 refit kept, 0 warm kept
__global__ void fallback_select_kernel(const int* idx, long long n_items, long long n, int nparam, float* pars,
                                       const float* backup, float* cost, const float* cost_backup,
                                       signed char* which) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_items) return;
  const long long v = idx[i];
  const bool refit = cost[v] < cost_backup[i];
  if (!refit) {
    for (int k = 0; k < nparam; ++k) pars[(long long)k * n + v] = backup[(long long)k * n_items + i];
    cost[v] = cost_backup[i];
  }
  if (which) which[v] = refit ? 1 : 0;
}

unsigned blocks(long long n) { return unsigned((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }

}  // namespace pcgb_pipe

using namespace pcgb_pipe;

extern "C" {

const char* pcgb_pipeline_last_error(void) { return g_err.c_str(); }

int pcgb_init_constant(const float* data, int64_t n, int m, int nparam, const double* values, float* pars,
                       void* stream) {
  if (n < 0 || m < 1 || nparam < 1 || nparam > PCGB_MAX_PARAMS || !values)
    return fail(PCGB_EINVAL, "bad init_constant arguments");
  if (n == 0) return PCGB_OK;
  InitArgs a{};
  a.data = data;
  a.n = n;
  a.m = m;
  a.nparam = nparam;
  for (int k = 0; k < nparam; ++k) {
    a.from_max[k] = std::isnan(values[k]) ? 1 : 0;
    a.values[k] = a.from_max[k] ? 0.f : float(values[k]);
  }
  a.pars = pars;
  init_constant_kernel<<<blocks(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cuda_rc();
}

int pcgb_fallback_flags(const float* pars, const float* cost, const float* cost_ref, int64_t n, int nparam,
                        const double* lb, const double* ub, int8_t* flags, int32_t* idx, int32_t* count,
                        void* stream) {
  if (n < 0 || nparam < 1 || nparam > PCGB_MAX_PARAMS || !lb || !ub || !idx || !count)
    return fail(PCGB_EINVAL, "bad fallback_flags arguments");
  if (n == 0) return PCGB_OK;
  FlagArgs a{};
  a.pars = pars;
  a.cost = cost;
  a.cost_ref = cost_ref;
  a.n = n;
  a.nparam = nparam;
  for (int k = 0; k < nparam; ++k) {
    a.lb[k] = float(lb[k]);
    a.ub[k] = float(ub[k]);
  }
  a.flags = reinterpret_cast<signed char*>(flags);
  a.idx = idx;
  a.count = count;
  flag_compact_kernel<<<blocks(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cuda_rc();
}

int pcgb_fallback_prepare(const int32_t* idx, int64_t n_items, int64_t n, int nparam, int m, const double* values,
                          float* pars, float* backup, const float* cost, float* cost_backup, const float* data,
                          float* lam, float lam0, int8_t* step_type, float* f, void* stream) {
  if (n_items < 0 || n < 0 || nparam < 1 || nparam > PCGB_MAX_PARAMS || m < 1 || !values)
    return fail(PCGB_EINVAL, "bad fallback_prepare arguments");
  if (n_items == 0) return PCGB_OK;
  PrepArgs a{};
  a.idx = idx;
  a.n_items = n_items;
  a.n = n;
  a.nparam = nparam;
  a.m = m;
  for (int k = 0; k < nparam; ++k) {
    a.from_max[k] = std::isnan(values[k]) ? 1 : 0;
    a.values[k] = a.from_max[k] ? 0.f : float(values[k]);
  }
  a.pars = pars;
  a.backup = backup;
  a.cost = cost;
  a.cost_backup = cost_backup;
  a.data = data;
  a.lam = lam;
  a.lam0 = lam0;
  a.step_type = reinterpret_cast<signed char*>(step_type);
  a.f = f;
  fallback_prepare_kernel<<<blocks(n_items), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cuda_rc();
}

int pcgb_fallback_select(const int32_t* idx, int64_t n_items, int64_t n, int nparam, float* pars,
                         const float* backup, float* cost, const float* cost_backup, int8_t* which, void* stream) {
  if (n_items < 0 || n < 0 || nparam < 1 || nparam > PCGB_MAX_PARAMS)
    return fail(PCGB_EINVAL, "bad fallback_select arguments");
  if (n_items == 0) return PCGB_OK;
  fallback_select_kernel<<<blocks(n_items), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      idx, n_items, n, nparam, pars, backup, cost, cost_backup, reinterpret_cast<signed char*>(which));
  return cuda_rc();
}

}  // extern "C"
