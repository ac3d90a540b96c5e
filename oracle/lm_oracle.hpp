// CPU oracle of the reference's second-order Levenberg-Marquardt fitter.
//
// TEST INFRASTRUCTURE ONLY: tests/, the smoke check and the CPU-baseline leg of
// bench.py use this to check and time the GPU fitter. The product never calls it.
//
// It restates, per voxel and in the same order of operations, the CUDA C that
// pycompute renders from its Jinja templates:
//   fghhl  (f, g = J^T r, h, damped hl)   pycompute/cuda/lsqnonlin.py:206-258
//   f      (trial cost)                   pycompute/cuda/lsqnonlin.py:46-67
//   gmw81_solver = diag_pivot -> permute -> Jacobi scale -> gmw81 -> ldl_solve
//                  -> unscale -> inv_permute
//                                         pycompute/cuda/solver.py:431-463
//     max_diag_abs (never updates max_abs) pycompute/cuda/permute.py:47-58
//     diag_pivot                          pycompute/cuda/permute.py:179-193
//     row/col interchange                 pycompute/cuda/permute.py:85-154
//     permute_vec / inv_permute_vec       pycompute/cuda/permute.py:230-236,268-274
//     gmw81 (modified LDL^T)              pycompute/cuda/solver.py:23-95
//     forward_subs_unit_diaged            pycompute/cuda/solver.py:298-308
//     backward_subs_unit_t                pycompute/cuda/solver.py:341-350
//   gain_ratio_step                       pycompute/cuda/lsqnonlin.py:435-493
//   clamp_pars                            pycompute/cuda/lsqnonlin.py:587-602
//   gradient_convergence                  pycompute/cuda/lsqnonlin.py:694-724
//   orchestration of one iteration        pycompute/cuda/lsqnonlin.py:823-924
//   host loop, first_f / last_f           pycompute/cuda/lsqnonlin.py:1058-1073
//
// Precision is a pair of types: TA for the per-sample accumulation, state and
// convergence test, TS for the GMW81 solve and the gain-ratio test.
//   <float, float>   = the reference's fp32 kernel,
//   <float, double>  = FP32 bulk with an FP64 solve and gain ratio,
//   <double, double> = all FP64. Here the reference's fp64 leaks (the partial
//                      sum `entry` hard-typed float, lsqnonlin.py:447, and the
//                      `float tol` of gradient_convergence, lsqnonlin.py:695)
//                      are NOT reproduced: everything is double.
// Constants use the corrected layout consts[(k*M + i)*stride + v]; for one
// constant per sample (every model here) this is the reference's layout.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#ifndef PCGB_HD
#define PCGB_HD inline
#endif

inline float pcgb_exp(float x) { return std::exp(x); }
inline double pcgb_exp(double x) { return std::exp(x); }
inline float pcgb_log(float x) { return std::log(x); }
inline double pcgb_log(double x) { return std::log(x); }
inline float pcgb_sin(float x) { return std::sin(x); }
inline double pcgb_sin(double x) { return std::sin(x); }
inline float pcgb_cos(float x) { return std::cos(x); }
inline double pcgb_cos(double x) { return std::cos(x); }
inline float pcgb_tan(float x) { return std::tan(x); }
inline double pcgb_tan(double x) { return std::tan(x); }
inline float pcgb_asin(float x) { return std::asin(x); }
inline double pcgb_asin(double x) { return std::asin(x); }
inline float pcgb_acos(float x) { return std::acos(x); }
inline double pcgb_acos(double x) { return std::acos(x); }
inline float pcgb_atan(float x) { return std::atan(x); }
inline double pcgb_atan(double x) { return std::atan(x); }
inline float pcgb_sinh(float x) { return std::sinh(x); }
inline double pcgb_sinh(double x) { return std::sinh(x); }
inline float pcgb_cosh(float x) { return std::cosh(x); }
inline double pcgb_cosh(double x) { return std::cosh(x); }
inline float pcgb_tanh(float x) { return std::tanh(x); }
inline double pcgb_tanh(double x) { return std::tanh(x); }
inline float pcgb_abs(float x) { return std::fabs(x); }
inline double pcgb_abs(double x) { return std::fabs(x); }
inline float pcgb_erf(float x) { return std::erf(x); }
inline double pcgb_erf(double x) { return std::erf(x); }
inline float pcgb_sqrt(float x) { return std::sqrt(x); }
inline double pcgb_sqrt(double x) { return std::sqrt(x); }
inline float pcgb_pow(float x, float y) { return std::pow(x, y); }
inline double pcgb_pow(double x, double y) { return std::pow(x, y); }

namespace oracle {

template <typename T> inline T machine_eps();
template <> inline float machine_eps<float>() { return 2e-7f; }     // solver.py:105
template <> inline double machine_eps<double>() { return 4e-16; }   // solver.py:109

template <typename T> inline T min_scaling();
template <> inline float min_scaling<float>() { return 1e-4f; }     // lsqnonlin.py:275
template <> inline double min_scaling<double>() { return 1e-4; }    // lsqnonlin.py:278

// ---- permute.py -----------------------------------------------------------

// permute.py:47-58. max_abs is never updated, so the result is the last
// index >= offset whose |diagonal| compares greater than -1 (every non-NaN
// entry), or 0 when all of them are NaN.
template <typename T>
int max_diag_abs(const T* mat, int n, int offset) {
  T max_abs = T(-1);
  int max_index = 0;
  for (int i = offset; i < n; ++i)
    if (std::fabs(mat[i * n + i]) > max_abs) max_index = i;
  return max_index;
}

template <typename T>
void row_interchange(T* mat, int n, int ii, int jj) {
  for (int k = 0; k < n; ++k) {
    T t = mat[ii * n + k];
    mat[ii * n + k] = mat[jj * n + k];
    mat[jj * n + k] = t;
  }
}

template <typename T>
void col_interchange(T* mat, int n, int ii, int jj) {
  for (int k = 0; k < n; ++k) {
    T t = mat[k * n + ii];
    mat[k * n + ii] = mat[k * n + jj];
    mat[k * n + jj] = t;
  }
}

template <typename T>
void diag_pivot(T* mat, int n, int* perm) {
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int i = 0; i < n; ++i) {
    int mx = max_diag_abs(mat, n, i);
    row_interchange(mat, n, i, mx);
    col_interchange(mat, n, i, mx);
    int t = perm[i];
    perm[i] = perm[mx];
    perm[mx] = t;
  }
}

// ---- solver.py ------------------------------------------------------------

// solver.py:23-95: in-place modified LDL^T of the lower triangle.
template <typename T>
void gmw81(T* mat, int n) {
  T t0;
  T t1 = T(0);  // gamma
  T t2 = T(0);  // nu
  T beta2 = machine_eps<T>();
  T delta = machine_eps<T>();
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      t0 = std::fabs(mat[i * n + j]);
      if (i == j) {
        if (t0 > t1) t1 = t0;
      } else {
        if (t0 > t2) t2 = t0;
      }
    }
  if (n > 1) t2 /= std::sqrt(T(n * n - 1));
  if (beta2 < t1) beta2 = t1;
  if (beta2 < t2) beta2 = t2;
  t0 = t1 + t2;
  if (t0 > T(1)) delta *= t0;

  for (int j = 0; j < n; ++j) {
    for (int s = 0; s < j; ++s) mat[j * n + s] /= mat[s * n + s];
    for (int i = j + 1; i < n; ++i) {
      t0 = mat[i * n + j];
      for (int s = 0; s < j; ++s) t0 -= mat[j * n + s] * mat[i * n + s];
      mat[i * n + j] = t0;
    }
    t1 = T(0);
    for (int i = j + 1; i < n; ++i) {
      t0 = std::fabs(mat[i * n + j]);
      if (t1 < t0) t1 = t0;
    }
    t1 *= t1;
    t2 = std::fabs(mat[j * n + j]);
    if (t2 < delta) t2 = delta;
    t0 = t1 / beta2;
    if (t2 < t0) t2 = t0;
    mat[j * n + j] = t2;
    for (int i = j + 1; i < n; ++i) {
      t0 = mat[i * n + j];
      mat[i * n + i] -= t0 * t0 / t2;
    }
  }
}

// solver.py:298-308 then solver.py:341-350 (ldl_solve, solver.py:386-391).
template <typename T>
void ldl_solve(const T* mat, int n, const T* rhs, T* sol) {
  T arr[8];
  for (int i = 0; i < n; ++i) {
    arr[i] = rhs[i];
    for (int j = 0; j < i; ++j) arr[i] -= mat[i * n + j] * mat[j * n + j] * arr[j];
    arr[i] /= mat[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    sol[i] = arr[i];
    for (int j = i + 1; j < n; ++j) sol[i] -= mat[j * n + i] * sol[j];
  }
}

// solver.py:431-463. mat is a full symmetric n x n matrix; it is overwritten.
template <typename T>
void gmw81_solver(T* mat, int n, const T* rhs, T* sol) {
  int perm[8];
  T arr1[8], arr2[8], scale[8];
  diag_pivot(mat, n, perm);
  for (int i = 0; i < n; ++i) arr1[i] = rhs[perm[i]];
  for (int i = 0; i < n; ++i) {
    scale[i] = std::sqrt(std::fabs(mat[i * n + i]));
    arr1[i] /= scale[i];
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) mat[i * n + j] /= (scale[i] * scale[j]);
  gmw81(mat, n);
  ldl_solve(mat, n, arr1, arr2);
  for (int i = 0; i < n; ++i) arr2[i] /= scale[i];
  for (int i = 0; i < n; ++i) sol[perm[i]] = arr2[i];
}

// ---- the LM voxel fit ------------------------------------------------------

struct Strides {
  long N;            // voxels
  long cstride;      // consts: N (per voxel) or 0 (one protocol shared by all voxels)
  long bstride;      // bounds: N (per voxel) or 0 (shared)
};

template <class Model, typename TA>
inline void gather_consts(const TA* consts, const Strides& s, int M, long v, int i, TA* c) {
  for (int k = 0; k < Model::C; ++k) c[k] = s.cstride ? consts[(long(k) * M + i) * s.cstride + v] : consts[long(k) * M + i];
}

// Accumulating objective, lsqnonlin.py:46-67: f += sum_i (m - d_i)^2.
template <class Model, typename TA>
TA cost(const TA* p, const TA* consts, const TA* data, const Strides& s, int M, long v) {
  TA f = TA(0);
  TA c[Model::C > 0 ? Model::C : 1];
  for (int i = 0; i < M; ++i) {
    gather_consts<Model>(consts, s, M, v, i, c);
    TA res = Model::template value<TA>(p, c) - data[long(i) * s.N + v];
    f += res * res;
  }
  return f;
}

struct RunParams {
  int iters;
  double tol, mu, eta, acc, dec;
};

// One voxel, all iterations of one run() call. Mirrors the host loop of
// lsqnonlin.py:1065-1073 (iters launches; converged voxels return at the top
// of the kernel, lsqnonlin.py:1000-1002) and one launch body per iteration.
template <class Model, typename TA, typename TS>
void lm_voxel(long v, int M, const Strides& s, const RunParams& rp,
              const TA* consts, const TA* data, const TA* lb, const TA* ub,
              TA* pars, TA* lam_a, int8_t* st_a, TA* f_a, TA* first_f, TA* last_f,
              TA* step_a, int32_t* iters_a) {
  constexpr int P = Model::P, H = Model::H, C = Model::C;
  const long N = s.N;
  TA p[P], l[P], u[P];
  for (int k = 0; k < P; ++k) {
    p[k] = pars[k * N + v];
    l[k] = s.bstride ? lb[k * s.bstride + v] : lb[k];
    u[k] = s.bstride ? ub[k * s.bstride + v] : ub[k];
  }
  TA lam = lam_a[v];
  int8_t st = st_a[v];
  TA f = f_a[v];
  TA step[P];
  for (int k = 0; k < P; ++k) step[k] = step_a ? step_a[k * N + v] : TA(0);
  const TA tol = TA(rp.tol), mu = TA(rp.mu), eta = TA(rp.eta), acc = TA(rp.acc), dec = TA(rp.dec);
  int done = 0;
  TA c[C > 0 ? C : 1];

  for (int it = 0; it < rp.iters; ++it) {
    if (st == 0) {
      if (it == 0) first_f[v] = f;
      continue;
    }
    ++done;
    // zero accumulators, lsqnonlin.py:830-840
    f = TA(0);
    TA ftp = TA(0);
    TA g[P], h[H], hl[H];
    for (int k = 0; k < P; ++k) g[k] = TA(0);
    for (int k = 0; k < H; ++k) h[k] = hl[k] = TA(0);

    // fghhl, lsqnonlin.py:225-256
    for (int i = 0; i < M; ++i) {
      gather_consts<Model>(consts, s, M, v, i, c);
      TA m, J[P], Hm[H], hes[H];
      Model::template all<TA>(p, c, m, J, Hm);
      TA res = m - data[long(i) * N + v];
      for (int k = 0; k < H; ++k) hes[k] = Hm[k] * res;
      f += res * res;
      int q = 0;
      for (int j = 0; j < P; ++j) {
        for (int k = 0; k <= j; ++k) {
          TA jtemp = J[j] * J[k];
          TA hjtemp = hes[q] + jtemp;
          h[q] += hjtemp;
          if (j != k)
            hl[q] += hjtemp;
          else
            hl[q] += hjtemp + std::fmax(lam * jtemp, min_scaling<TA>());
          ++q;
        }
        g[j] += J[j] * res;
      }
    }
    if (it == 0) first_f[v] = f;

    // solve step, lsqnonlin.py:848-878
    {
      TS mat[P * P], rhs[P], sol[P];
      for (int k = 0; k < P; ++k) rhs[k] = TS(g[k]);
      int q = 0;
      for (int i = 0; i < P; ++i)
        for (int j = 0; j <= i; ++j) {
          mat[i * P + j] = TS(hl[q]);
          if (i != j) mat[j * P + i] = TS(hl[q]);
          ++q;
        }
      gmw81_solver(mat, P, rhs, sol);
      for (int k = 0; k < P; ++k) step[k] = TA(sol[k]);
    }
    // remove NaN and Inf, lsqnonlin.py:881-891
    for (int k = 0; k < P; ++k)
      if (std::isnan(step[k]) || std::isinf(step[k])) step[k] = TA(0);

    // gradient convergence, lsqnonlin.py:697-723
    {
      bool clamped = false;
      TA norm = TA(0);
      for (int k = 0; k < P; ++k) {
        TA t1 = p[k];
        TA t2 = t1 - g[k];
        if (t2 > u[k]) {
          clamped = true;
          t2 = u[k];
        } else if (t2 < l[k]) {
          clamped = true;
          t2 = l[k];
        }
        t2 = t1 - t2;
        norm += t2 * t2;
      }
      if (norm < tol * (TA(1) + f))
        if ((st & 1) || clamped) st = 0;
      if (st == 0) continue;
    }

    // trial point and trial cost, lsqnonlin.py:902-912
    TA ptp[P];
    for (int k = 0; k < P; ++k) ptp[k] = p[k] - step[k];
    ftp = cost<Model, TA>(ptp, consts, data, s, M, v);

    // gain ratio, lsqnonlin.py:441-491
    {
      TS actual = TS(0.5) * (TS(f) - TS(ftp));
      TS predicted = TS(0);
      int q = 0;
      for (int i = 0; i < P; ++i)
        for (int j = 0; j <= i; ++j) {
          TS entry = TS(h[q]) * TS(step[i]) * TS(step[j]);
          if (i == j)
            predicted -= entry;
          else
            predicted -= TS(2) * entry;
          ++q;
        }
      predicted *= TS(0.5);
      for (int i = 0; i < P; ++i) predicted += TS(step[i]) * TS(g[i]);
      TS rho = actual / predicted;
      if ((rho > TS(mu)) && (actual > TS(0))) {
        for (int k = 0; k < P; ++k) p[k] = ptp[k];
        if (rho > TS(eta)) {
          lam *= acc;
          st = 1;
        } else {
          st = 2;
        }
      } else {
        lam *= dec;
        st = 4;
      }
      if (predicted < TS(0)) {
        lam *= dec;
        st |= 8;
      }
    }
    // clamp, lsqnonlin.py:590-601
    for (int k = 0; k < P; ++k) {
      if (p[k] > u[k])
        p[k] = u[k];
      else if (p[k] < l[k])
        p[k] = l[k];
    }
  }
  if (rp.iters > 0) last_f[v] = f;
  for (int k = 0; k < P; ++k) pars[k * N + v] = p[k];
  if (step_a)
    for (int k = 0; k < P; ++k) step_a[k * N + v] = step[k];
  lam_a[v] = lam;
  st_a[v] = st;
  f_a[v] = f;
  if (iters_a) iters_a[v] += done;
}

// ---- searches ----------------------------------------------------------------

// SearchStep (lsqnonlin.py:1083-1105): f += cost(p); keep p if f < best_f.
template <class Model, typename TA>
void search_step_voxel(long v, int M, const Strides& s, const TA* consts, const TA* data, const TA* p_a, TA* f_a,
                       TA* best_p, TA* best_f) {
  constexpr int P = Model::P;
  TA p[P];
  for (int k = 0; k < P; ++k) p[k] = p_a[k * s.N + v];
  f_a[v] += cost<Model, TA>(p, consts, data, s, M, v);
  if (f_a[v] < best_f[v]) {
    for (int k = 0; k < P; ++k) best_p[k * s.N + v] = p[k];
    best_f[v] = f_a[v];
  }
}

// The draws of the GPU random search: splitmix64's output function (Steele,
// Lea & Flood 2014) keyed by (seed, voxel, draw, component), 24-bit uniforms.
inline unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
inline float uniform01(unsigned long long seed, long v, int d, int k) {
  unsigned long long z = mix64(seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(v + 1));
  z = mix64(z ^ (((unsigned long long)(unsigned)d << 8) | (unsigned)k));
  return float(z >> 40) * (1.0f / 16777216.0f);
}

// RandomSearch.run / SecondOrderRandomSearch.run (lsqnonlin.py:1232-1242,
// 1277-1291) for one voxel: each draw is rand * (ub - lb) + lb, optionally
// refined by lm_iters LM iterations from lambda = 5, step_type = 1 (a fresh
// setup, lsqnonlin.py:1288-1289), and compared by its own cost.
template <class Model, typename TA, typename TS>
void random_search_voxel(long v, int M, const Strides& s, const RunParams& rp, int draws, unsigned long long seed,
                         const TA* consts, const TA* data, const TA* lb, const TA* ub, TA* best_p, TA* best_f) {
  constexpr int P = Model::P, C = Model::C;
  TA d[256], c[256], lo[P], hi[P];
  for (int i = 0; i < M; ++i) d[i] = data[long(i) * s.N + v];
  for (int k = 0; k < C; ++k)
    for (int i = 0; i < M; ++i) c[k * M + i] = s.cstride ? consts[(long(k) * M + i) * s.cstride + v] : consts[k * M + i];
  for (int k = 0; k < P; ++k) {
    lo[k] = s.bstride ? lb[k * s.bstride + v] : lb[k];
    hi[k] = s.bstride ? ub[k * s.bstride + v] : ub[k];
  }
  Strides one{1, 0, 0};
  TA bf = best_f[v];
  TA bp[P];
  for (int k = 0; k < P; ++k) bp[k] = best_p[k * s.N + v];
  for (int dr = 0; dr < draws; ++dr) {
    TA p[P];
    for (int k = 0; k < P; ++k) p[k] = std::fma(TA(uniform01(seed, v, dr, k)), hi[k] - lo[k], lo[k]);
    if (rp.iters > 0) {
      TA lam = TA(5), f = TA(0), ff = TA(0), lf = TA(0);
      int8_t st = 1;
      lm_voxel<Model, TA, TS>(0, M, one, rp, c, d, lo, hi, p, &lam, &st, &f, &ff, &lf, nullptr, nullptr);
    }
    const TA fc = cost<Model, TA>(p, c, d, one, M, 0);
    if (fc < bf) {
      bf = fc;
      for (int k = 0; k < P; ++k) bp[k] = p[k];
    }
  }
  for (int k = 0; k < P; ++k) best_p[k * s.N + v] = bp[k];
  best_f[v] = bf;
}

}  // namespace oracle
