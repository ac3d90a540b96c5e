// Host driver for the reference's generated LM kernel
// test/ivim/second_order_levenberg_marquardt_4_1_21_f_f7def86f0a03.cu
// (IVIM, 4 parameters, 1 constant, fp32), compiled from the reference tree as
// host C++ with ref_shim.h; REF_NDATA is the sample count it was built for
// (21 as generated, 10 for the IVIM-10 protocol).
//
// TEST INFRASTRUCTURE ONLY: pins the CPU oracle and gives golden vectors.
// It repeats what SecondOrderLevenbergMarquardt.setup/run do
// (pycompute/cuda/lsqnonlin.py:1036-1073): scratch arrays, one "launch" per
// iteration over every voxel, first_f / last_f copies after the first and the
// last launch.
#include <cstdint>
#include <cstring>
#include <vector>

#ifndef REF_NDATA
#define REF_NDATA 21
#endif

struct ref_dim3 { unsigned x, y, z; };
thread_local ref_dim3 threadIdx{0, 0, 0}, blockIdx{0, 0, 0}, blockDim{1, 1, 1};

extern "C" void k_second_order_levenberg_marquardt_4_1_21_f_f7def86f0a03(
    const float* consts, const float* data, const float* lower_bound, const float* upper_bound, float tol, float mu,
    float eta, float acc, float dec, float* params, float* params_tp, float* step, float* lam, char* step_type,
    float* f, float* ftp, float* g, float* h, float* hl, int Nprobs);

extern "C" void k_random_search_4_1_21_f_f7def86f0a03(const float* consts, const float* data,
                                                      const float* lower_bound, const float* upper_bound,
                                                      float* best_p, float* p, float* best_f, float* f, int Nprobs);

extern "C" {

int ref_ndata() { return REF_NDATA; }
int ref_nparam() { return 4; }

// pars (4,N) in/out; consts (21,N); data (21,N); lb, ub (4,N); lam, f (1,N)
// in/out; step_type (1,N) in/out; first_f / last_f (1,N) out.
int ref_lm_run(int N, const float* consts, const float* data, const float* lb, const float* ub, float* pars,
               float* lam, int8_t* step_type, float* f, float* first_f, float* last_f, float* step_out, int iters,
               float tol, float mu, float eta, float acc, float dec) {
  std::vector<float> params_tp(size_t(4) * N, 0.f), step(size_t(4) * N, 0.f), ftp(N, 0.f), g(size_t(4) * N),
      h(size_t(10) * N), hl(size_t(10) * N);
  for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int t = 0; t < N; ++t) {
      blockDim.x = 1;
      threadIdx.x = 0;
      blockIdx.x = unsigned(t);
      k_second_order_levenberg_marquardt_4_1_21_f_f7def86f0a03(
          consts, data, lb, ub, tol, mu, eta, acc, dec, pars, params_tp.data(), step.data(), lam,
          reinterpret_cast<char*>(step_type), f, ftp.data(), g.data(), h.data(), hl.data(), N);
    }
    if (it == 0) std::memcpy(first_f, f, sizeof(float) * N);
    if (it == iters - 1) std::memcpy(last_f, f, sizeof(float) * N);
  }
  if (step_out) std::memcpy(step_out, step.data(), sizeof(float) * 4 * N);
  return 0;
}

// One SearchStep launch (lsqnonlin.py:1194-1199): f accumulates the cost at p,
// best_p / best_f keep the better point.
int ref_search_step(int N, const float* consts, const float* data, const float* lb, const float* ub, float* best_p,
                    float* p, float* best_f, float* f) {
#pragma omp parallel for schedule(static)
  for (int t = 0; t < N; ++t) {
    blockDim.x = 1;
    threadIdx.x = 0;
    blockIdx.x = unsigned(t);
    k_random_search_4_1_21_f_f7def86f0a03(consts, data, lb, ub, best_p, p, best_f, f, N);
  }
  return 0;
}

}  // extern "C"
