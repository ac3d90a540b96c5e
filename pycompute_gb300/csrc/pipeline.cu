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
#include "lm_kernel.cuh"
#include "pcgb.h"

namespace pcgb_pipe {

// The integer-pipe helpers of the FP64 GMW81 solve, applied elementwise so
// they can be checked against correctly rounded results: rcp64(x) against 1/x,
// narrow(x) against the double -> float conversion.
__global__ void fp64_helpers_kernel(const double* x, double* rcp, float* nar, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (rcp) rcp[i] = pcgb::rcp64(x[i]);
  if (nar) nar[i] = pcgb::narrow(x[i]);
}

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

// ---- segmented log-linear initialisation --------------------------------------

constexpr int kMaxFitRows = 64;
constexpr int kMaxDeg = 3;

struct PolyArgs {
  const float* x;        // (rows, n) per voxel, or null: shared xs[]
  long long xstride;     // n, or 0 with shared x
  float xs[kMaxFitRows];
  const float* y;        // (M, n); rows [r0, r0 + rows) are fitted
  long long n;
  int r0, rows, deg, log_y;
  float* out;            // (deg + 1, n): coefficients of x^0 .. x^deg
};

// Per-voxel least squares of y (or log y) on 1, x, ..., x^deg: the batched
// pinv(A) @ y of the reference's bpolyfit (pycompute/cuda/lsq.py:18-26). For
// a full-rank design this is the least-squares solution, computed here by
// Householder QR in FP64 (rows <= 64, deg <= 3); a rank-deficient column gets
// coefficient 0.
__global__ void bpolyfit_kernel(const PolyArgs a) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.n) return;
  const int m = a.rows, q = a.deg + 1;
  double A[kMaxFitRows][kMaxDeg + 1];
  double b[kMaxFitRows];
  for (int i = 0; i < m; ++i) {
    const double xi = a.x ? double(a.x[(long long)i * a.xstride + v]) : double(a.xs[i]);
    double pw = 1.0;
    for (int j = 0; j < q; ++j) {
      A[i][j] = pw;
      pw *= xi;
    }
    const double yi = double(a.y[(long long)(a.r0 + i) * a.n + v]);
    b[i] = a.log_y ? log(yi) : yi;
  }
  double R[kMaxDeg + 1];
  for (int j = 0; j < q; ++j) {
    double nrm = 0.0;
    for (int i = j; i < m; ++i) nrm += A[i][j] * A[i][j];
    nrm = sqrt(nrm);
    if (!(nrm > 0.0)) {
      R[j] = 0.0;
      continue;
    }
    const double alpha = A[j][j] > 0 ? -nrm : nrm;
    A[j][j] -= alpha;  // v = x - alpha e1, stored in column j
    double vv = 0.0;
    for (int i = j; i < m; ++i) vv += A[i][j] * A[i][j];
    for (int k = j + 1; k < q; ++k) {
      double s = 0.0;
      for (int i = j; i < m; ++i) s += A[i][j] * A[i][k];
      s = 2.0 * s / vv;
      for (int i = j; i < m; ++i) A[i][k] -= s * A[i][j];
    }
    double s = 0.0;
    for (int i = j; i < m; ++i) s += A[i][j] * b[i];
    s = 2.0 * s / vv;
    for (int i = j; i < m; ++i) b[i] -= s * A[i][j];
    R[j] = alpha;
  }
  double c[kMaxDeg + 1];
  for (int j = q - 1; j >= 0; --j) {
    double t = b[j];
    for (int k = j + 1; k < q; ++k) t -= A[j][k] * c[k];
    c[j] = fabs(R[j]) > 1e-300 ? t / R[j] : 0.0;
  }
  for (int j = 0; j < q; ++j) a.out[(long long)j * a.n + v] = float(c[j]);
}

struct IvimInitArgs {
  const float* low;    // (2, n): log-intercept and slope of the low-b fit
  const float* high;   // (2, n): the same for the high-b fit
  long long n;
  float lb0[4], ub0[4];
  float* pars;         // (4, n) out
  float* lb;           // (4, n) out, data-driven bounds
  float* ub;           // (4, n) out
};

__device__ __forceinline__ float finite_or_zero(float x) { return isfinite(x) ? x : 0.f; }

// The IVIM notebook's segmented initialisation (test_ivim.ipynb cells 6 and
// 10): S0 = exp(low intercept), f = 1 - exp(high intercept) / S0,
// D* = low slope, D = high slope (non-finite -> 0, then clipped to the fixed
// bounds), and per-voxel bounds S0/2..2 S0 (within 500..20000), f +- 0.4
// (within 0.001..0.999), D*/200..200 D* (within 1e-6..0.1), D/200..200 D
// (within 1e-8..0.02).
__global__ void ivim_segmented_init_kernel(const IvimInitArgs a) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.n) return;
  const float s0 = expf(a.low[v]);
  const float s1 = expf(a.high[v]);
  float p[4] = {finite_or_zero(s0), finite_or_zero(1.f - s1 / s0), finite_or_zero(a.low[a.n + v]),
                finite_or_zero(a.high[a.n + v])};
  for (int k = 0; k < 4; ++k) p[k] = fminf(fmaxf(p[k], a.lb0[k]), a.ub0[k]);
  const float lo[4] = {fmaxf(p[0] / 2.f, 500.f), fmaxf(p[1] - 0.4f, 0.001f), fmaxf(p[2] / 200.f, 1e-6f),
                       fmaxf(p[3] / 200.f, 1e-8f)};
  const float hi[4] = {fminf(p[0] * 2.f, 20000.f), fminf(p[1] + 0.4f, 0.999f), fminf(p[2] * 200.f, 0.1f),
                       fminf(p[3] * 200.f, 0.02f)};
  for (int k = 0; k < 4; ++k) {
    a.pars[(long long)k * a.n + v] = p[k];
    if (a.lb) a.lb[(long long)k * a.n + v] = lo[k];
    if (a.ub) a.ub[(long long)k * a.n + v] = hi[k];
  }
}

unsigned blocks(long long n) { return unsigned((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }

}  // namespace pcgb_pipe

using namespace pcgb_pipe;

extern "C" {

const char* pcgb_pipeline_last_error(void) { return g_err.c_str(); }

int pcgb_copy_rows_async(void* dst, int64_t dst_pitch, const void* src, int64_t src_pitch, int64_t row_bytes,
                         int64_t rows, int direction, void* stream) {
  if (rows < 0 || row_bytes < 0 || dst_pitch < row_bytes || src_pitch < row_bytes)
    return fail(PCGB_EINVAL, "copy_rows: pitches must cover row_bytes, sizes >= 0");
  if (rows == 0 || row_bytes == 0) return PCGB_OK;
  if (!dst || !src) return fail(PCGB_EINVAL, "copy_rows: null pointer");
  cudaMemcpyKind kind;
  switch (direction) {
    case 0: kind = cudaMemcpyHostToDevice; break;
    case 1: kind = cudaMemcpyDeviceToHost; break;
    case 2: kind = cudaMemcpyDeviceToDevice; break;
    default: return fail(PCGB_EINVAL, "copy_rows: direction must be 0 (H2D), 1 (D2H) or 2 (D2D)");
  }
  const cudaError_t e = cudaMemcpy2DAsync(dst, size_t(dst_pitch), src, size_t(src_pitch), size_t(row_bytes),
                                          size_t(rows), kind, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? PCGB_OK : fail(PCGB_ECUDA, cudaGetErrorString(e));
}

int pcgb_fp64_helpers(const double* x, double* rcp, float* narrowed, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && !x)) return fail(PCGB_EINVAL, "bad fp64_helpers arguments");
  if (n == 0) return PCGB_OK;
  const long long blocks = (n + 255) / 256;
  if (blocks > 0x7fffffffLL) return fail(PCGB_ERANGE, "fp64_helpers: n too large");
  fp64_helpers_kernel<<<unsigned(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, rcp, narrowed, n);
  return cuda_rc();
}

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

int pcgb_bpolyfit(const float* x, int64_t x_stride, const double* x_shared, const float* y, int64_t n, int row0,
                  int rows, int deg, int log_y, float* out, void* stream) {
  if (n < 0 || rows < 1 || rows > kMaxFitRows || deg < 0 || deg > kMaxDeg || row0 < 0 || !y || !out)
    return fail(PCGB_EINVAL, "bpolyfit: rows 1..64, deg 0..3, y and out required");
  if (!x && !x_shared) return fail(PCGB_EINVAL, "bpolyfit: x or x_shared required");
  if (n == 0) return PCGB_OK;
  PolyArgs a{};
  a.x = x;
  a.xstride = x ? x_stride : 0;
  if (!x)
    for (int i = 0; i < rows; ++i) a.xs[i] = float(x_shared[i]);
  a.y = y;
  a.n = n;
  a.r0 = row0;
  a.rows = rows;
  a.deg = deg;
  a.log_y = log_y;
  a.out = out;
  bpolyfit_kernel<<<unsigned((n + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cuda_rc();
}

int pcgb_ivim_segmented_init(const float* low, const float* high, int64_t n, const double* lb, const double* ub,
                             float* pars, float* lb_out, float* ub_out, void* stream) {
  if (n < 0 || !low || !high || !lb || !ub || !pars) return fail(PCGB_EINVAL, "ivim_segmented_init: bad arguments");
  if (n == 0) return PCGB_OK;
  IvimInitArgs a{};
  a.low = low;
  a.high = high;
  a.n = n;
  for (int k = 0; k < 4; ++k) {
    a.lb0[k] = float(lb[k]);
    a.ub0[k] = float(ub[k]);
  }
  a.pars = pars;
  a.lb = lb_out;
  a.ub = ub_out;
  ivim_segmented_init_kernel<<<blocks(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
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
