// Launch parameters of the LM kernels. Shared by the host library (pcgb.cpp)
// and the kernel source that is compiled at run time, so it must stay plain C
// with fixed-size members.
#pragma once

#define PCGB_MAX_PARAMS 8
#define PCGB_MAX_PROTOCOL 256
#define PCGB_MAX_MODELS 8

// PcgbLmParams.flags of an LM run
#define PCGB_LM_FRESH 1      // every voxel starts at lam = lam_start, step_type = 1; lam, f, step are not read
#define PCGB_LM_PARS_ONLY 2  // only pars (and step_type, when given) are written back

struct PcgbLmParams {
  // structure-of-arrays, voxel index fastest; element type is the fitter's
  // state type (float, or double for the all-FP64 build)
  void* pars;              // (P, N) in/out
  const void* consts;      // (C*M, N) per voxel, unused when the protocol is shared
  const void* data;        // (M, N)
  const void* lb;          // (P, N) per voxel, unused when bounds are shared
  const void* ub;          // (P, N)
  void* lam;               // (N) in/out damping
  signed char* step_type;  // (N) in/out, 0 = converged
  void* f;                 // (N) in/out cost at the last evaluated iterate
  void* first_f;           // (N) out, cost after the first iteration of the call
  void* last_f;            // (N) out, cost after the last iteration of the call
  void* step;              // (P, N) out or null
  void* model_out;         // (M, N) model values out (forward-model evaluation)
  void* best_p;            // (P, N) best point of a search, in/out
  void* best_f;            // (N) its cost, in/out
  unsigned long long seed; // random-search draws: counter-based stream per (seed, voxel, draw)
  int lm_iters;            // LM iterations per draw (0: plain random search)
  int* iters_done;         // (N) in/out iteration counter or null
  unsigned int* work;      // voxel work counter of the persistent schedule (zeroed by the host) or null
  const int* vox_idx;      // when set, work item i fits voxel vox_idx[i] (a compacted subset)
  long long n_items;       // number of work items: N, or the length of vox_idx
  long long N;
  long long cstride;       // N: per-voxel constants; 0: protocol_* hold them
  long long bstride;       // N: per-voxel bounds; 0: shared_* hold them
  int iters;
  int flags;               // PCGB_LM_* bits
  double tol, mu, eta, acc, dec;
  float tol_f, mu_f, eta_f, acc_f, dec_f;  // the same constants rounded to float (set with them)
  // fallback check of a warm-started fit (warm_check_grid / warm_select_grid)
  const unsigned int* n_items_dev;  // when set, the work-item count is min(*n_items_dev, n_items)
  void* cost;                       // (N) cost at the fit's final point, out
  void* pars_backup;                // (P, N) warm fits of the flagged voxels, compacted
  void* cost_backup;                // (N) their costs, compacted
  int* fb_idx;                      // (N) flagged voxel indices, compacted
  unsigned int* fb_count;           // [0] flagged voxels, [1] refits kept (zeroed by the host)
  signed char* which;               // (N) 1 where the refit was kept, or null
  double lam0;                      // damping of the refit
  double lam_start;                 // starting damping of every voxel under PCGB_LM_FRESH
  float init_val[PCGB_MAX_PARAMS];  // constant start of the refit; NaN = the voxel's largest sample
  // shared protocol and bounds in both precisions, so the kernel reads its own
  // type straight from the parameter bank (constant k of sample i at k*M + i)
  float shared_lb_f[PCGB_MAX_PARAMS];
  float shared_ub_f[PCGB_MAX_PARAMS];
  double shared_lb_d[PCGB_MAX_PARAMS];
  double shared_ub_d[PCGB_MAX_PARAMS];
  float protocol_f[PCGB_MAX_PROTOCOL];
  double protocol_d[PCGB_MAX_PROTOCOL];
};

// Launch parameters of the mixed-model persistent kernel: one job per model
// (shared protocol and bounds), and the work queue. The queue lists the jobs
// in the order order[0..njobs-1]; chunk c (of `chunk` voxels) belongs to job
// order[t] with chunk_off[t] <= c < chunk_off[t + 1]; warps claim chunks from
// *counter, which the host zeroes before the launch.
struct PcgbMultiParams {
  unsigned int* counter;
  int njobs;
  int chunk;
  int order[PCGB_MAX_MODELS];
  long long chunk_off[PCGB_MAX_MODELS + 1];
  PcgbLmParams jobs[PCGB_MAX_MODELS];
};
