/*
 * pcgb.h - C ABI of the GB300 batched Levenberg-Marquardt fitter.
 *
 * The reference (turbotage/pycompute) has no native library: its Python
 * classes render CUDA C from Jinja templates, compile it with NVRTC through
 * cupy.RawModule and launch the kernels directly. Each entry point below
 * replaces one of those Python-side operations; the comment on each names the
 * reference code it stands for (paths relative to the pycompute tree).
 *
 * Conventions
 *  - All array arguments are device pointers to C-contiguous structure-of-
 *    arrays buffers with the voxel index fastest, exactly the reference's
 *    layouts: params (P, N), data (M, N), consts (C*M, N), bounds (P, N),
 *    lam / f (N), step_type int8 (N).
 *  - "dtype" is 0 for float32 and 1 for float64 buffers.
 *  - Calls are asynchronous on the given cudaStream_t (passed as void*;
 *    NULL = legacy default stream), like the reference's launches on CuPy's
 *    current stream.
 *  - Every function returns 0 on success and a negative errno-style code on
 *    failure; pcgb_last_error() then describes the failure (per host thread).
 *    Nothing aborts, traps or prints.
 *  - A pcgb_fitter is not thread-safe; use one per host thread or lock.
 */
#ifndef PCGB_H
#define PCGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCGB_OK 0
#define PCGB_EINVAL (-22)
#define PCGB_ENOMEM (-12)
#define PCGB_ECOMPILE (-1001)
#define PCGB_ECUDA (-1002)
#define PCGB_ERANGE (-34)

#define PCGB_DTYPE_F32 0
#define PCGB_DTYPE_F64 1

typedef struct pcgb_fitter pcgb_fitter;

/* Library version string and the maximum sizes compiled into it. */
const char* pcgb_version(void);
int pcgb_max_params(void);
int pcgb_max_protocol(void);

/* Description of the last failure on this host thread ("" if none). */
const char* pcgb_last_error(void);

/*
 * Build a fitter program for one model, one protocol length and one precision.
 * Replaces SecondOrderLevenbergMarquardt.__init__/build (lsqnonlin.py:949-975,
 * 1013-1025): code generation of the orchestration kernel and its device
 * functions, cudap.code_gen_walking (cuda_program.py:193-203) and
 * cp.RawModule(code=...) (lsqnonlin.py:1019-1020).
 *   model_source  the generated model struct (m, dm/dp, d2m/dp2)
 *   model_struct  its type name
 *   nparam/nconst/ndata  P, C (constants per sample) and M
 *   dtype         state/accumulation type (PCGB_DTYPE_F32 or _F64)
 *   solve_dtype   type of the GMW81 solve and gain-ratio test
 *   cache_dir     directory for compiled cubins keyed by source hash, or NULL
 * The program is compiled with NVRTC for sm_103a and loaded on the current
 * device.
 */
int pcgb_fitter_create(const char* model_source, const char* model_struct, int nparam, int nconst, int ndata,
                       int dtype, int solve_dtype, const char* cache_dir, pcgb_fitter** out);

/*
 * Compile (and cache) the same program without loading it: no GPU is needed.
 * The compiler log (ptxas register and spill report) is copied into
 * log_buf (truncated to log_len bytes). Used by the build step to check the
 * kernel templates and by tooling; it has no reference counterpart.
 */
int pcgb_fitter_compile(const char* model_source, const char* model_struct, int nparam, int nconst, int ndata,
                        int dtype, int solve_dtype, const char* cache_dir, char* log_buf, size_t log_len);

/* Release the program (cudaLibraryUnload). */
int pcgb_fitter_destroy(pcgb_fitter* fitter);

/* Compiler log of the last build (register use from ptxas -v), "" if cached. */
const char* pcgb_fitter_log(const pcgb_fitter* fitter);

/*
 * Run `iters` LM iterations on N voxels in one launch.
 * Replaces SecondOrderLevenbergMarquardt.run (lsqnonlin.py:1058-1073): the
 * host loop of `iters` launches of k_second_order_levenberg_marquardt_*
 * (kernel arguments lsqnonlin.py:991-994) and the first_f / last_f copies.
 *   consts        (C*M, N) per voxel when consts_stride == N; when
 *                 consts_stride == 0 the protocol is shared by all voxels and
 *                 is taken from protocol_host (C*M host values) instead
 *   lower/upper   (P, N) when bounds_stride == N; shared bounds from
 *                 lb_host / ub_host (P host values) when bounds_stride == 0
 *   params        (P, N) initial values in, fitted values out
 *   step          (P, N) last step out, or NULL
 *   lam           (N) damping in/out (the reference starts it at 5)
 *   step_type     (N) int8 in/out (1 to start; 0 = converged, else 1/2/4 | 8)
 *   f             (N) cost at the last evaluated iterate, in/out
 *   first_f/last_f (N) cost after the first / last iteration of this call
 *   iters_done    (N) int32 counter incremented by the iterations run, or NULL
 *   tol, mu, eta, acc, dec  the reference's run() arguments
 *   block         threads per block (0 = library default)
 */
int pcgb_lm_run(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type, void* f,
                void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host, int block,
                void* stream);

/*
 * pcgb_lm_run restricted to the n_items voxels listed in vox_idx (int32
 * device array of distinct voxel indices < nprobs); all other voxels are left
 * untouched. Used to refit a compacted subset (the warm-start fallback) in
 * one launch without gathering its data. n_items_dev (may be NULL): a device
 * word with the list's length; then the first min(*n_items_dev, n_items)
 * entries are fitted and the launch covers n_items. No reference counterpart.
 */
int pcgb_lm_run_subset(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, const int32_t* vox_idx, int64_t n_items, const uint32_t* n_items_dev,
                       void* stream);

/*
 * pcgb_lm_run with the refill schedule: a persistent grid in which every lane
 * fits one voxel at a time and, when its voxel converges or runs out of
 * iterations, takes the next one (warp ballot + prefix-sum rank; warps claim
 * 256-voxel chunks from work_counter). Per-voxel results equal pcgb_lm_run's;
 * it is faster when voxels converge after very different numbers of
 * iterations. vox_idx / n_items restrict the fit to a list as in
 * pcgb_lm_run_subset (vox_idx may be NULL). n_items_dev (may be NULL; needs
 * vox_idx): a device word holding the list length, of which the first
 * min(*n_items_dev, n_items) entries are fitted, so a compaction's count needs
 * no host round trip. work_counter: one uint32 of device scratch, zeroed by
 * this call; grid <= 0 selects the persistent grid.
 * No reference counterpart (the reference launches one thread per voxel per
 * iteration).
 */
int pcgb_lm_run_refill(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, const int32_t* vox_idx, int64_t n_items, const uint32_t* n_items_dev,
                       uint32_t* work_counter, int grid, void* stream);

/*
 * pcgb_lm_run from a fresh start with only the parameters kept: the first LM
 * stage of the warm-start pipeline (no reference counterpart). Every voxel
 * starts at lam = lam0 (> 0) and step_type = 1 with the given params; no
 * damping, cost or step state is read, and only params (and step_type, when
 * not NULL) are written, so the caller allocates and initialises no other
 * state. The arithmetic of each iteration is pcgb_lm_run's.
 */
int pcgb_lm_run_fresh(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                      const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                      double eta, double acc, double dec, void* params, int8_t* step_type, int64_t nprobs, int iters,
                      const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                      double lam0, int block, void* stream);

/*
 * Fallback check of a warm-started fit, fused per model (no reference
 * counterpart; it implements the rule "refit from the plain fitter's start
 * where the warm fit fails to lower the cost below that start's or lands on a
 * bound"). In one pass over the samples of every voxel: cost[v] = cost at
 * params; the voxel is flagged if that cost is not finite, not below the cost
 * at the constant start (init_values, P host values, NaN = the voxel's largest
 * sample), or a parameter is not strictly inside [lb, ub]. Flagged voxels are
 * appended to fb_idx (order unspecified) with fb_count[0] their number; their
 * warm fit goes to pars_backup (P, nprobs; column i = i-th flagged voxel) and
 * cost_backup, their params are set to the constant start, lam to lam0,
 * step_type to 1 and f to 0, ready for pcgb_lm_run_refill on
 * (fb_idx, n_items_dev = fb_count). fb_count: two uint32 of device memory,
 * zeroed by this call. nprobs < 2^31.
 */
int pcgb_warm_check(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                    const void* lower_bound, const void* upper_bound, int64_t bounds_stride,
                    const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                    const double* init_values, double lam0, void* params, void* lam, int8_t* step_type, void* f,
                    void* cost, void* pars_backup, void* cost_backup, int32_t* fb_idx, uint32_t* fb_count,
                    int64_t nprobs, void* stream);

/*
 * The first LM stage of a warm-started fit and its fallback check in one
 * launch (no reference counterpart): pcgb_lm_run_fresh for `iters`
 * iterations from params at damping lam_start (> 0), then, per voxel and
 * from registers, the rule and outputs of pcgb_warm_check. The warm fit's
 * cost is the one the iterations evaluated at the final parameters (NaN in
 * cost and cost_backup where they did not: the last accepted step was moved
 * by a bound, which flags the voxel; the select evaluates such a cost), so
 * only the cost at the constant start is computed (and, with iters = 0, the
 * cost at params). block: threads per block (0 = default). nprobs < 2^31.
 */
int pcgb_warm_lm_check(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, int iters, double lam_start, const double* protocol_host,
                       int protocol_len, const double* lb_host, const double* ub_host, const double* init_values,
                       double lam0, void* params, void* lam, int8_t* step_type, void* f, void* cost,
                       void* pars_backup, void* cost_backup, int32_t* fb_idx, uint32_t* fb_count, int64_t nprobs,
                       int block, void* stream);

/*
 * pcgb_lm_run with pcgb_warm_check as its epilogue, in one launch: the check
 * runs on the samples and the fit still in registers (no second pass over the
 * signals). Arguments as in pcgb_lm_run followed by those of pcgb_warm_check;
 * results equal pcgb_lm_run then pcgb_warm_check. No reference counterpart.
 */
int pcgb_lm_run_check(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                      const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                      double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                      void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                      const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                      int block, const double* init_values, double lam0, void* cost, void* pars_backup,
                      void* cost_backup, int32_t* fb_idx, uint32_t* fb_count, void* stream);

/*
 * The refit of the fb_count[0] flagged voxels of fb_idx (as pcgb_lm_run_subset
 * with n_items_dev = fb_count) with pcgb_warm_select as its epilogue, in one
 * launch. Results equal the subset run followed by pcgb_warm_select. No
 * reference counterpart.
 */
int pcgb_lm_run_select(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, void* cost, const void* pars_backup, const void* cost_backup,
                       const int32_t* fb_idx, uint32_t* fb_count, int8_t* which, void* stream);

/*
 * After the refit of the flagged voxels: for each of the fb_count[0] voxels of
 * fb_idx, the cost at its refitted params is compared with cost_backup; the
 * lower fit is kept in params and cost, fb_count[1] counts the kept refits,
 * which[v] (may be NULL) = 1 where the refit was kept.
 */
int pcgb_warm_select(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                     const double* protocol_host, int protocol_len, void* params, void* cost, const void* pars_backup,
                     const void* cost_backup, const int32_t* fb_idx, uint32_t* fb_count, int8_t* which,
                     int64_t nprobs, void* stream);

/*
 * Accumulating objective f[v] += sum_i (m(p_v; c_i) - d_i)^2, voxels whose
 * step_type is 0 skipped (step_type may be NULL). Replaces F.run
 * (lsqnonlin.py:137-145; kernel lsqnonlin.py:160-172).
 */
int pcgb_f_run(pcgb_fitter* fitter, const void* params, const void* consts, int64_t consts_stride, const void* data,
               const int8_t* step_type, void* f, int64_t nprobs, const double* protocol_host, int protocol_len,
               void* stream);

/* pcgb_f_run for the voxels listed in vox_idx only (no reference counterpart). */
int pcgb_f_run_subset(pcgb_fitter* fitter, const void* params, const void* consts, int64_t consts_stride,
                      const void* data, const int8_t* step_type, void* f, int64_t nprobs, const double* protocol_host,
                      int protocol_len, const int32_t* vox_idx, int64_t n_items, void* stream);

/*
 * Batched GMW81 modified-Cholesky solve of packed symmetric (H, N) matrices
 * (row i, column j <= i) with (P, N) right-hand sides into (P, N) solutions.
 * Replaces GMW81Solver.run (solver.py:503-510; kernel solver.py:526-563).
 */
int pcgb_gmw81_solve(pcgb_fitter* fitter, const void* mat, const void* rhs, void* sol, int64_t nprobs,
                     void* stream);

/*
 * One search step: f[v] += cost(p_v) (accumulating, like the reference's cost
 * function), then (p_v, f[v]) replaces (best_p_v, best_f[v]) if f[v] is lower.
 * Replaces SearchStep.run (lsqnonlin.py:1194-1199; kernel lsqnonlin.py:1153-1162).
 */
int pcgb_search_step(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data, const void* p,
                     void* f, void* best_p, void* best_f, int64_t nprobs, const double* protocol_host,
                     int protocol_len, void* stream);

/*
 * Random search in one launch: `draws` points per voxel uniform in [lb, ub],
 * each refined by lm_iters LM iterations (from lambda = 5) when lm_iters > 0;
 * best_p / best_f (in/out) keep the point of lowest cost. Draws come from a
 * counter-based generator keyed by (seed, voxel, draw, parameter).
 * Replaces RandomSearch.run (lsqnonlin.py:1232-1242, lm_iters = 0) and
 * SecondOrderRandomSearch.run (lsqnonlin.py:1277-1291), which draw with
 * cp.random on the host and launch once per draw. Each draw is compared by its
 * own cost (the reference's cost buffer accumulates across draws).
 */
int pcgb_random_search(pcgb_fitter* fitter, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, void* best_p,
                       void* best_f, int64_t nprobs, int draws, int lm_iters, double tol, double mu, double eta,
                       double acc, double dec, uint64_t seed, const double* protocol_host, int protocol_len,
                       const double* lb_host, const double* ub_host, void* stream);

/*
 * Forward model out[i][v] = m(p_v; c_i) for all voxels and samples, (M, N).
 * The reference's per-element evaluator (pycompute/cuda/symbolic.py:18-347,
 * Eval) was never compiled at HEAD; this is its working counterpart, used for
 * synthetic signals and fitted curves.
 */
int pcgb_model_eval(pcgb_fitter* fitter, const void* params, const void* consts, int64_t consts_stride, void* out,
                    int64_t nprobs, const double* protocol_host, int protocol_len, void* stream);

/* ---- mixed-model persistent batch (no reference counterpart) ----------------
 *
 * One program holds up to 8 models (each with its own protocol length); one
 * persistent launch fits every voxel of every model: warps claim chunks of
 * `chunk` voxels from a device work counter, so models with fast-converging
 * voxels hand their warps to the others. Protocols and bounds are shared per
 * model (host values in the job). The reference fits one model per program
 * and relaunches per iteration.
 */
typedef struct pcgb_multi pcgb_multi;

typedef struct {
  const void* data;        /* (M, N) signals */
  void* params;            /* (P, N) in/out */
  void* lam;               /* (N) in/out */
  int8_t* step_type;       /* (N) in/out */
  void* f;                 /* (N) in/out */
  void* first_f;           /* (N) out */
  void* last_f;            /* (N) out */
  int32_t* iters_done;     /* (N) in/out or NULL */
  int64_t nprobs;          /* N */
  const double* protocol;  /* host, C*M values */
  const double* lb;        /* host, P values */
  const double* ub;        /* host, P values */
} pcgb_multi_job;

/* Compile one program for n_models models (NVRTC, sm_103a, disk cache).
 * maxrreg: register cap (0 = compiler's choice); block: threads per block;
 * lanes (may be NULL = all 1): per model, the warp lanes that share one
 * voxel (1 or 2; with 2 the two lanes split the voxel's samples and sum
 * their shares, so results match one lane's to float rounding). */
int pcgb_multi_create(int n_models, const char* const* model_sources, const char* const* model_structs,
                      const int* nparam, const int* nconst, const int* ndata, int dtype, int solve_dtype, int maxrreg,
                      int block, const int* lanes, const char* cache_dir, pcgb_multi** out);
int pcgb_multi_destroy(pcgb_multi* program);
const char* pcgb_multi_log(const pcgb_multi* program);
/* Persistent grid size: resident blocks per SM x SMs. */
int pcgb_multi_grid(const pcgb_multi* program);

/* Fit all jobs (one per model, in program order) for `iters` iterations in one
 * launch. order (host, may be NULL = program order) is the order in which the
 * work queue hands out the jobs' chunks (longest work first shortens the
 * tail). work_counter: one uint32 of device scratch, zeroed by this call
 * (cudaMemsetAsync) before the launch; grid <= 0 selects the persistent grid.
 * At most 2^31 chunks of `chunk` voxels per call, summed over the jobs (the
 * counter is 32 bits wide); larger requests fail with PCGB_ERANGE before any
 * work is queued. */
int pcgb_multi_run(pcgb_multi* program, const pcgb_multi_job* jobs, int n_jobs, const int* order, int iters,
                   double tol, double mu, double eta, double acc, double dec, int chunk, int grid,
                   uint32_t* work_counter, void* stream);

/*
 * pcgb_multi_run for callers that cannot allocate device memory. No reference
 * counterpart: the reference always allocates its buffers through CuPy.
 *
 * Who needs it: hosts whose device memory belongs to another framework's pool
 * allocator (which hands out only the buffers it manages, so a side
 * cudaMalloc would fragment or exceed its budget), and embedded or
 * long-running services that reserve their device memory at start-up and may
 * not grow it afterwards. pcgb_multi_run needs one word of device scratch (the
 * work counter); this variant uses a statically allocated 256-byte array owned
 * by the library instead, so it allocates nothing and calls no allocating
 * routine. The caller still passes every input and output (the jobs' buffers).
 *
 * Limits and rules:
 *  - at most 2^31 chunks of `chunk` voxels per call (summed over the jobs);
 *    larger requests fail with PCGB_ERANGE and a message;
 *  - every GPU that loads the library holds the 256-byte array until the
 *    process exits;
 *  - all calls share the array: the counter is cleared at the start of each
 *    call (cudaMemsetAsync on the call's stream), and calls that overlap on
 *    the GPU (concurrent streams, or several host threads) race on it, so
 *    serialise them;
 *  - the first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress, with that device current) and caches it with the
 *    identity of the current CUDA context; make that first call before any
 *    stream capture. A later call under another context (after a
 *    cudaDeviceReset, or with another driver-API context current) looks the
 *    address up again, so it again must not come during a capture.
 */
int pcgb_multi_run_noalloc(pcgb_multi* program, const pcgb_multi_job* jobs, int n_jobs, const int* order, int iters,
                           double tol, double mu, double eta, double acc, double dec, int chunk, int grid,
                           void* stream);

/* Last error of pcgb_multi_run_noalloc on this host thread. */
const char* pcgb_noalloc_last_error(void);

/* ---- fit pipeline (no reference counterpart) -------------------------------
 * fp32 structure-of-arrays buffers; values/lb/ub are host arrays of nparam.
 */

/* Last error of the pipeline entry points on this host thread. */
const char* pcgb_pipeline_last_error(void);

/* Asynchronous strided copy of `rows` rows of row_bytes bytes (pitches in
 * bytes): a voxel range of a structure-of-arrays (rows, N) array in one call,
 * used to stream chunks of host-resident signals and results through the GPU.
 * direction 0 = host to device, 1 = device to host, 2 = device to device; host
 * memory should be pinned for the copy to overlap kernels. */
int pcgb_copy_rows_async(void* dst, int64_t dst_pitch, const void* src, int64_t src_pitch, int64_t row_bytes,
                         int64_t rows, int direction, void* stream);

/* The integer-pipe helpers of the FP64 GMW81 solve, elementwise, exposed so
 * callers and tests can check them on their own inputs: rcp[i] = 1/x[i] by a
 * float seed and one third-order Newton-Raphson step (within 1 ulp of 1/x;
 * zero, Inf, NaN and exponents outside the float range take the correctly
 * rounded reciprocal); narrowed[i] = x[i] rounded to float (to nearest even,
 * equal to the hardware conversion). Either output may be NULL. */
int pcgb_fp64_helpers(const double* x, double* rcp, float* narrowed, int64_t n, void* stream);

/* Constant initialisation: pars[k][v] = values[k]; a NaN entry means "the
 * voxel's largest sample" (the reference notebooks' S0 start). */
int pcgb_init_constant(const float* data, int64_t n, int m, int nparam, const double* values, float* pars,
                       void* stream);

/* Batched polynomial least squares, the reference's bpolyfit
 * (pycompute/cuda/lsq.py:18-26): per voxel, the coefficients of 1, x, ..., x^deg
 * (deg <= 3) best fitting rows [row0, row0 + rows) of y (M, n) (log y when
 * log_y), rows <= 64. x is (rows, n) device with x_stride = n, or NULL with
 * x_shared = rows host values. out is (deg + 1, n). FP64 Householder QR. */
int pcgb_bpolyfit(const float* x, int64_t x_stride, const double* x_shared, const float* y, int64_t n, int row0,
                  int rows, int deg, int log_y, float* out, void* stream);

/* The IVIM notebook's segmented initialisation (test_ivim.ipynb cells 6, 10)
 * from two degree-1 log fits (low, high: (2, n) from pcgb_bpolyfit on -b):
 * initial parameters clipped to [lb, ub] (host, 4 values) and, when lb_out /
 * ub_out are given, the notebook's per-voxel data-driven bounds. */
int pcgb_ivim_segmented_init(const float* low, const float* high, int64_t n, const double* lb, const double* ub,
                             float* pars, float* lb_out, float* ub_out, void* stream);

/* Flag voxels whose fit is not trusted (non-finite cost, cost not below
 * cost_ref, or a parameter on a bound) and append their indices to idx
 * (capacity n). count (one int32 on the device) must be zero on entry and
 * receives the number of flagged voxels. flags may be NULL. */
int pcgb_fallback_flags(const float* pars, const float* cost, const float* cost_ref, int64_t n, int nparam,
                        const double* lb, const double* ub, int8_t* flags, int32_t* idx, int32_t* count,
                        void* stream);

/* For the n_items listed voxels: save pars (P, n_items) and cost into
 * backup / cost_backup, write the constant initialisation (values as in
 * pcgb_init_constant), reset lam to lam0, step_type to 1 and f to 0. */
int pcgb_fallback_prepare(const int32_t* idx, int64_t n_items, int64_t n, int nparam, int m, const double* values,
                          float* pars, float* backup, const float* cost, float* cost_backup, const float* data,
                          float* lam, float lam0, int8_t* step_type, float* f, void* stream);

/* Keep the refit of each listed voxel only if its cost is lower than the
 * saved one, else restore the saved parameters and cost; which[v] (may be
 * NULL) = 1 where the refit was kept. */
int pcgb_fallback_select(const int32_t* idx, int64_t n_items, int64_t n, int nparam, float* pars,
                         const float* backup, float* cost, const float* cost_backup, int8_t* which, void* stream);

/* ---- warm-start network (no reference counterpart) -------------------------
 *
 * The reference starts every fit from constant parameters or from a segmented
 * log-linear fit (pycompute/cuda/lsq.py:18-26). These entry points train and
 * run a 16 -> 128 -> 128 -> 128 -> P GELU network (bf16 weights, fp32
 * accumulation, tensor cores) whose outputs replace that initialisation.
 * Weight layout per layer: (rows x ld) row-major, ld = inputs + 8, with the
 * bias in column `inputs` of the fp32 master copy. All pointers are device
 * pointers unless noted.
 */

/* Last error of the network entry points on this host thread. */
const char* pcgb_mlp_last_error(void);

/* C = A * B with bf16 operands and fp32 accumulation on the tensor cores.
 * a_layout 0: A is (M, K) row-major, 1: A is (K, M) row-major.
 * b_layout 0: B is (N, K) row-major, 1: B is (K, N) row-major.
 * epilogue 0: z = C + bias -> out_f32, gelu(z) -> out_bf16
 *          1: out_f32 = C + bias
 *          2: out_bf16 = C * gelu'(zin)
 *          3: out_f32 += C (atomic; allows split-K with k_split < K)
 *          4: out_f32 = C
 * K, lda, ldb must be multiples of 8. */
int pcgb_gemm_bf16(int a_layout, int b_layout, int epilogue, const void* A, int64_t lda, const void* B, int64_t ldb,
                   int64_t M, int64_t N, int64_t K, int64_t k_split, const float* bias, int64_t bias_stride,
                   float* out_f32, int64_t ldo, void* out_bf16, int64_t ldob, const float* zin, int64_t ldz,
                   void* stream);

/* pcgb_gemm_bf16 on the 5th-generation tensor cores (tcgen05.mma, fp32
 * accumulator in tensor memory; no reference counterpart): same arguments,
 * layouts, epilogues and results up to fp32 summation order. status (device
 * int, may be NULL) is set to 1 if a CTA gave up on a bounded wait for its
 * tensor-core work (its tile of the output is then not written). */
int pcgb_gemm_bf16_tc(int a_layout, int b_layout, int epilogue, const void* A, int64_t lda, const void* B,
                      int64_t ldb, int64_t M, int64_t N, int64_t K, int64_t k_split, const float* bias,
                      int64_t bias_stride, float* out_f32, int64_t ldo, void* out_bf16, int64_t ldob,
                      const float* zin, int64_t ldz, int* status, void* stream);

/* pcgb_gemm_bf16_tc with its failure path exposed (no reference
 * counterpart). wait_limit: mbarrier try_wait rounds before a wait for the
 * tensor cores counts as lost (0 = the default, 2^22). skip_block: a test hook
 * for that path - the CTA with this linear index (x + gx (y + gy z), -1 =
 * none) never issues its MMAs, so its first wait runs out with none of its
 * tensor-core work in flight; the CTA then sets *status to 1, writes none of
 * its output tile, still frees its tensor memory, and the call returns
 * normally. */
int pcgb_gemm_bf16_tc_ex(int a_layout, int b_layout, int epilogue, const void* A, int64_t lda, const void* B,
                         int64_t ldb, int64_t M, int64_t N, int64_t K, int64_t k_split, const float* bias,
                         int64_t bias_stride, float* out_f32, int64_t ldo, void* out_bf16, int64_t ldob,
                         const float* zin, int64_t ldz, int* status, unsigned wait_limit, int64_t skip_block,
                         void* stream);

/* Last error of pcgb_gemm_bf16_tc and pcgb_gemm_bf16_tc_ex on this host thread. */
const char* pcgb_gemm_tc_last_error(void);

/* Mean-squared-error gradient dy = 2 (y - t) / (batch * nout) (bf16, zero in
 * padding columns nout..ncols-1) and loss_sum += mean squared error. */
int pcgb_mlp_mse_grad(const float* y, const float* t, int64_t ldy, int64_t batch, int nout, int ncols, void* dy,
                      int64_t lddy, float* loss_sum, void* stream);

/* One Adam step over a (rows x ld) weight buffer; rows >= rows_live are
 * padding. corr is a device array {1 - b1^t, 1 - b2^t, s}: the bias
 * corrections of step t and a learning-rate scale (the step uses lr * s), read
 * at run time so one captured CUDA graph replays every step. Clears grad and
 * refreshes the bf16 copy. */
int pcgb_adam_step(float* master, float* m, float* v, float* grad, void* w_bf16, int64_t rows, int64_t ld,
                   int64_t rows_live, float lr, float b1, float b2, float eps, const float* corr, void* stream);

/* Training inputs x_rows (n x ldx) bf16 = signals / max per voxel (or
 * log(max(signals / max, 1e-6)) with log_in), column nin = 1; snorm[v] = that
 * maximum. With params/targets, also the normalised
 * targets (n x ldt): kind 0 p/snorm, 1 p, 2 log p, then (g - mean) / std.
 * signals (nin, n) and params (nout, n) are structure-of-arrays; kinds, mean,
 * stdv are device arrays of nout entries. */
int pcgb_mlp_prepare(const float* signals, int64_t n, int nin, int log_in, void* x_rows, int64_t ldx, float* snorm,
                     const float* params, int nout, const int* kinds, const float* mean, const float* stdv,
                     float* targets, int64_t ldt, void* stream);

/* The network's activation elementwise, for checks against other
 * implementations: gelu_out[i] = gelu(z[i]) and grad_out[i] = gelu'(z[i]) as
 * every network kernel computes them for the units of network column
 * `column` (>= 0): columns with column % 16 < 6 evaluate GELU by a polynomial
 * in f16x2 arithmetic on the FMA pipe, the others in bf16x2 arithmetic with
 * tanh.approx.bf16x2 (see the training and inference kernels). Either output
 * may be NULL. No reference counterpart. */
int pcgb_mlp_gelu(const float* z, int64_t n, int column, float* gelu_out, float* grad_out, void* stream);

/* Fused inference of all four layers: signals (nin, n) -> initial parameters
 * out (nout, n), clamped to [lb, ub]; log_in selects the input transform the
 * network was trained with. w_bf16 / w_master are host arrays of the
 * four layers' device pointers; kinds, mean, stdv, lb, ub are host arrays of
 * nout entries. nin must be 16. */
int pcgb_mlp_forward(const float* signals, int64_t n, int nin, int log_in, const void* const* w_bf16,
                     const float* const* w_master, int nout, const int* kinds, const float* mean, const float* stdv, const float* lb,
                     const float* ub, float* out, void* stream);

/* pcgb_mlp_forward on the tcgen05 tensor cores: one CTA per SM with four
 * 128-voxel tiles in flight, layer accumulators in tensor memory, operands in
 * shared memory. Same arguments and results (up to fp32 summation order);
 * status (device int, may be NULL) is set to 1 if the kernel gave up on a
 * bounded wait for its tensor-core work (its outputs are then incomplete). */
int pcgb_mlp_forward_tc(const float* signals, int64_t n, int nin, int log_in, const void* const* w_bf16,
                        const float* const* w_master, int nout, const int* kinds, const float* mean, const float* stdv,
                        const float* lb, const float* ub, float* out, int* status, void* stream);

/* pcgb_mlp_forward_tc with its failure path exposed (no reference
 * counterpart). wait_limit: mbarrier try_wait rounds before a wait for the
 * tensor cores counts as lost (0 = the default, 2^22). skip_tile: a test hook
 * for that path - the 128-voxel tile with this index (-1 = none) never has its
 * first layer issued, so its warpgroup's wait runs out with none of its
 * tensor-core work in flight; the kernel then sets *status to 1, stops that
 * warpgroup's work, still frees its tensor memory and returns normally. */
int pcgb_mlp_forward_tc_ex(const float* signals, int64_t n, int nin, int log_in, const void* const* w_bf16,
                           const float* const* w_master, int nout, const int* kinds, const float* mean,
                           const float* stdv, const float* lb, const float* ub, float* out, int* status,
                           unsigned wait_limit, int64_t skip_tile, void* stream);

/* Last error of pcgb_mlp_forward_tc on this host thread. */
const char* pcgb_mlp_tc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PCGB_H */
