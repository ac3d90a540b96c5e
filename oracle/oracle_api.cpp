// C entry points of the CPU oracle for one generated model.
//
// TEST INFRASTRUCTURE ONLY (tests/, the smoke check, bench.py's CPU-baseline
// leg). Compiled per model by oracle/build.py with
//   -DPCGB_MODEL_FILE="<generated model header>" -DPCGB_MODEL_STRUCT=<struct>
// The algorithm lives in lm_oracle.hpp; this file only dispatches precision
// modes and runs voxels on OpenMP threads.
#include <cstdint>
#include <cstdlib>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lm_oracle.hpp"
#include PCGB_MODEL_FILE

using Model = PCGB_MODEL_STRUCT;

namespace {

template <typename TA, typename TS>
void run_all(int M, long N, long cstride, long bstride, void* pars, const void* consts, const void* data,
             const void* lb, const void* ub, void* lam, int8_t* st, void* f, void* first_f, void* last_f,
             void* step, int32_t* iters_done, const oracle::RunParams& rp) {
  oracle::Strides s{N, cstride, bstride};
#pragma omp parallel for schedule(dynamic, 64)
  for (long v = 0; v < N; ++v) {
    oracle::lm_voxel<Model, TA, TS>(v, M, s, rp, (const TA*)consts, (const TA*)data, (const TA*)lb, (const TA*)ub,
                                   (TA*)pars, (TA*)lam, st, (TA*)f, (TA*)first_f, (TA*)last_f, (TA*)step,
                                   iters_done);
  }
}

template <typename T>
void cost_all(int M, long N, long cstride, const void* pars, const void* consts, const void* data, void* f) {
  oracle::Strides s{N, cstride, 0};
#pragma omp parallel for schedule(static)
  for (long v = 0; v < N; ++v) {
    T p[Model::P];
    for (int k = 0; k < Model::P; ++k) p[k] = ((const T*)pars)[k * N + v];
    ((T*)f)[v] += oracle::cost<Model, T>(p, (const T*)consts, (const T*)data, s, M, v);
  }
}

}  // namespace

extern "C" {

int oracle_model_P() { return Model::P; }
int oracle_model_C() { return Model::C; }

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// mode 0: <float,float> (reference fp32), 1: <float,double>, 2: <double,double>.
int oracle_lm_run(int mode, int M, long N, long cstride, long bstride, void* pars, const void* consts,
                  const void* data, const void* lb, const void* ub, void* lam, int8_t* st, void* f, void* first_f,
                  void* last_f, void* step, int32_t* iters_done, int iters, double tol, double mu, double eta,
                  double acc, double dec) {
  if (M <= 0 || N < 0 || iters < 0) return -22;
  oracle::RunParams rp{iters, tol, mu, eta, acc, dec};
  switch (mode) {
    case 0:
      run_all<float, float>(M, N, cstride, bstride, pars, consts, data, lb, ub, lam, st, f, first_f, last_f, step,
                            iters_done, rp);
      return 0;
    case 1:
      run_all<float, double>(M, N, cstride, bstride, pars, consts, data, lb, ub, lam, st, f, first_f, last_f, step,
                             iters_done, rp);
      return 0;
    case 2:
      run_all<double, double>(M, N, cstride, bstride, pars, consts, data, lb, ub, lam, st, f, first_f, last_f,
                              step, iters_done, rp);
      return 0;
    default:
      return -22;
  }
}

// f[v] += sum_i (m(p_v; c_i) - d_i)^2, accumulating like the reference F.
int oracle_cost(int dbl, int M, long N, long cstride, const void* pars, const void* consts, const void* data,
                void* f) {
  if (M <= 0 || N < 0) return -22;
  if (dbl)
    cost_all<double>(M, N, cstride, pars, consts, data, f);
  else
    cost_all<float>(M, N, cstride, pars, consts, data, f);
  return 0;
}

// One SearchStep over all voxels (f accumulates, best kept).
int oracle_search_step(int dbl, int M, long N, long cstride, const void* consts, const void* data, const void* p,
                       void* f, void* best_p, void* best_f) {
  if (M <= 0 || N < 0) return -22;
  oracle::Strides s{N, cstride, 0};
#pragma omp parallel for schedule(static)
  for (long v = 0; v < N; ++v) {
    if (dbl)
      oracle::search_step_voxel<Model, double>(v, M, s, (const double*)consts, (const double*)data, (const double*)p,
                                               (double*)f, (double*)best_p, (double*)best_f);
    else
      oracle::search_step_voxel<Model, float>(v, M, s, (const float*)consts, (const float*)data, (const float*)p,
                                              (float*)f, (float*)best_p, (float*)best_f);
  }
  return 0;
}

// Random search with optional LM refinement (mode as in oracle_lm_run).
int oracle_random_search(int mode, int M, long N, long cstride, long bstride, const void* consts, const void* data,
                         const void* lb, const void* ub, void* best_p, void* best_f, int draws, int lm_iters,
                         unsigned long long seed, double tol, double mu, double eta, double acc, double dec) {
  if (M <= 0 || M > 256 || N < 0 || draws < 0 || lm_iters < 0) return -22;
  oracle::Strides s{N, cstride, bstride};
  oracle::RunParams rp{lm_iters, tol, mu, eta, acc, dec};
#pragma omp parallel for schedule(dynamic, 16)
  for (long v = 0; v < N; ++v) {
    if (mode == 0)
      oracle::random_search_voxel<Model, float, float>(v, M, s, rp, draws, seed, (const float*)consts,
                                                       (const float*)data, (const float*)lb, (const float*)ub,
                                                       (float*)best_p, (float*)best_f);
    else if (mode == 1)
      oracle::random_search_voxel<Model, float, double>(v, M, s, rp, draws, seed, (const float*)consts,
                                                        (const float*)data, (const float*)lb, (const float*)ub,
                                                        (float*)best_p, (float*)best_f);
    else
      oracle::random_search_voxel<Model, double, double>(v, M, s, rp, draws, seed, (const double*)consts,
                                                         (const double*)data, (const double*)lb, (const double*)ub,
                                                         (double*)best_p, (double*)best_f);
  }
  return 0;
}

// Batched GMW81 solve of packed symmetric (H, N) matrices and (P, N) right-hand
// sides, like the reference GMW81Solver kernel (solver.py:526-563).
int oracle_gmw81_solve(int dbl, int n, long N, const void* mat, const void* rhs, void* sol) {
  if (n <= 0 || n > 8 || N < 0) return -22;
#pragma omp parallel for schedule(static)
  for (long v = 0; v < N; ++v) {
    if (dbl) {
      double a[64], b[8], x[8];
      int q = 0;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j, ++q) a[i * n + j] = a[j * n + i] = ((const double*)mat)[q * N + v];
      for (int i = 0; i < n; ++i) b[i] = ((const double*)rhs)[i * N + v];
      oracle::gmw81_solver(a, n, b, x);
      for (int i = 0; i < n; ++i) ((double*)sol)[i * N + v] = x[i];
    } else {
      float a[64], b[8], x[8];
      int q = 0;
      for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j, ++q) a[i * n + j] = a[j * n + i] = ((const float*)mat)[q * N + v];
      for (int i = 0; i < n; ++i) b[i] = ((const float*)rhs)[i * N + v];
      oracle::gmw81_solver(a, n, b, x);
      for (int i = 0; i < n; ++i) ((float*)sol)[i * N + v] = x[i];
    }
  }
  return 0;
}

}  // extern "C"
