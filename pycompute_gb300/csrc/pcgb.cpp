// Host side of the C ABI in include/pcgb.h.
//
// A fitter is one NVRTC-compiled program: the embedded device sources
// (lm_params.h, lm_kernel.cuh) plus the caller's generated model struct, with
// the LM, cost and GMW81 kernels instantiated for the model's P, C and M and
// the chosen precision. Programs are compiled for sm_103a to a cubin, cached
// on disk by a hash of the full source and options, and loaded with
// cudaLibraryLoadData. Only the CUDA runtime is used (cudart is linked
// statically and opens the driver on first use), so the library also loads on
// a host without a GPU.
#include "pcgb.h"

#include <cuda_runtime.h>
#include <nvrtc.h>

#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "lm_params.h"

extern const char* pcgb_embedded_lm_params_h;
extern const char* pcgb_embedded_lm_kernel_cuh;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[2048];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(PCGB_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

enum KernelSlot {
  K_LM_C1_B1, K_LM_C1_B0, K_LM_C0_B1, K_LM_C0_B0, K_COST_C1, K_COST_C0, K_GMW, K_EVAL_C1, K_EVAL_C0,
  K_SEARCH_C1, K_SEARCH_C0, K_RS_C1_B1, K_RS_C1_B0, K_RS_C0_B1, K_RS_C0_B0,
  K_LMQ_C1_B1, K_LMQ_C1_B0, K_LMQ_C0_B1, K_LMQ_C0_B0, K_CHECK_C1, K_CHECK_C0, K_SELECT_C1, K_SELECT_C0,
  K_LMC_C1_B1, K_LMC_C1_B0, K_LMC_C0_B1, K_LMC_C0_B0, K_LMS_C1_B1, K_LMS_C1_B0, K_LMS_C0_B1, K_LMS_C0_B0,
  K_LMW_C1_B1, K_LMW_C1_B0, K_LMW_C0_B1, K_LMW_C0_B0, K_COUNT
};
const char* kKernelNames[K_COUNT] = {"pcgb_lm_c1_b1", "pcgb_lm_c1_b0", "pcgb_lm_c0_b1", "pcgb_lm_c0_b0",
                                     "pcgb_cost_c1",  "pcgb_cost_c0",  "pcgb_gmw81",    "pcgb_eval_c1",
                                     "pcgb_eval_c0",  "pcgb_search_c1", "pcgb_search_c0", "pcgb_rs_c1_b1",
                                     "pcgb_rs_c1_b0", "pcgb_rs_c0_b1", "pcgb_rs_c0_b0", "pcgb_lmq_c1_b1",
                                     "pcgb_lmq_c1_b0", "pcgb_lmq_c0_b1", "pcgb_lmq_c0_b0", "pcgb_check_c1",
                                     "pcgb_check_c0", "pcgb_select_c1", "pcgb_select_c0", "pcgb_lmc_c1_b1",
                                     "pcgb_lmc_c1_b0", "pcgb_lmc_c0_b1", "pcgb_lmc_c0_b0", "pcgb_lms_c1_b1",
                                     "pcgb_lms_c1_b0", "pcgb_lms_c0_b1", "pcgb_lms_c0_b0", "pcgb_lmw_c1_b1",
                                     "pcgb_lmw_c1_b0", "pcgb_lmw_c0_b1", "pcgb_lmw_c0_b0"};

constexpr int kDefaultBlock = 128;
constexpr int kMaxBlock = 256;
// most chunks one mixed-model launch may hand out (see pcgb_multi_run)
constexpr int64_t kMaxMultiChunks = int64_t(1) << 31;

}  // namespace

struct pcgb_fitter {
  int P = 0, C = 0, M = 0, dtype = 0, sdtype = 0;
  int device = -1;
  cudaLibrary_t lib[5] = {};  // one per kernel group, loaded on first use
  int lm_min_blocks[5] = {};  // occupancy hint the group's LM kernels were built with (0: none)
  cudaKernel_t k[K_COUNT] = {};
  std::string source, structname, cache_dir;
  std::mutex mu;
  std::string log;
};

namespace {

// Kernel groups, each its own NVRTC program, compiled when a kernel of the
// group is first needed: 0 the fit itself (LM, cost, model evaluation, GMW81
// solve), 1 the searches, 2 the refill schedule and the warm-start fallback
// check (also as the LM's epilogue), 3 the fallback refit with the select as
// its epilogue, 4 the warm LM from a fresh start with the check as its
// epilogue. A group's LM kernels share one register cap (dropped when one of
// them would spill too much), so the refit and the fresh warm LM sit apart
// from the kernels whose larger state cannot take the cap.
constexpr int kGroups = 5;
int group_of(int slot) {
  switch (slot) {
    case K_LMW_C1_B1: case K_LMW_C1_B0: case K_LMW_C0_B1: case K_LMW_C0_B0:
      return 4;
    case K_SEARCH_C1: case K_SEARCH_C0: case K_RS_C1_B1: case K_RS_C1_B0: case K_RS_C0_B1: case K_RS_C0_B0:
      return 1;
    case K_LMQ_C1_B1: case K_LMQ_C1_B0: case K_LMQ_C0_B1: case K_LMQ_C0_B0: case K_CHECK_C1: case K_CHECK_C0:
    case K_SELECT_C1: case K_SELECT_C0: case K_LMC_C1_B1: case K_LMC_C1_B0: case K_LMC_C0_B1: case K_LMC_C0_B0:
      return 2;
    case K_LMS_C1_B1: case K_LMS_C1_B0: case K_LMS_C0_B1: case K_LMS_C0_B0:
      return 3;
    default:
      return 0;
  }
}

// The LM kernels for a shared protocol and shared bounds (the common case,
// the variant with the fewest registers) are first built for at least
// kLmMinBlocks resident 128-thread blocks per SM (a register cap: more warps
// to hide the FP64 pipe's latency); a model whose capped kernels would spill
// more than kLmMaxSpillBytes per thread is rebuilt without the cap.
bool is_lm_slot(int slot) {
  return slot == K_LM_C1_B1 || slot == K_LMQ_C1_B1 || slot == K_LMC_C1_B1 || slot == K_LMS_C1_B1 ||
         slot == K_LMW_C1_B1;
}

constexpr int kLmMinBlocks = 6;
// the warm LM with the check as its epilogue (group 4): two iterations and an
// epilogue per voxel gain from one more block (IVIM-16, 16.7 M voxels, whole
// warm step: 6 blocks 8.40 ms, 7 blocks 8.30 ms, 8 blocks 8.35 ms)
constexpr int kLmWarmMinBlocks = 7;
// the refit of the flagged voxels with the select as its epilogue (group 3):
// 6, 7 and 8 blocks measured within 0.3 % on the whole warm step (8.32, 8.32,
// 8.34 ms)
constexpr int kLmRefitMinBlocks = 6;
constexpr int lm_min_blocks_of(int g) {
  return g == 1 ? 0 : (g == 4 ? kLmWarmMinBlocks : (g == 3 ? kLmRefitMinBlocks : kLmMinBlocks));
}
constexpr int kLmMaxThreads = 128;
// Spilled words stay in L1 and cost less than the occupancy gain up to a few
// hundred bytes per thread (measured with the sample loops rolled, 8.4 M
// voxels: 5 -> 6 blocks per SM, 0 -> 84 bytes of spills, IVIM-16 x 8
// iterations 11.86 -> 11.68 ms, IVIM-10 x 20 flat; 7 and 8 blocks within 1 %);
// past this the cap is dropped.
constexpr size_t kLmMaxSpillBytes = 256;

std::string program_source(const char* model_source, const char* model_struct, int P, int C, int M, int dtype,
                           int sdtype, int group, int lm_min_blocks) {
  const char* ta = dtype == PCGB_DTYPE_F64 ? "double" : "float";
  const char* ts = sdtype == PCGB_DTYPE_F64 ? "double" : "float";
  std::ostringstream s;
  s << "// pcgb fitter program: P=" << P << " C=" << C << " M=" << M << " state=" << ta << " solve=" << ts
    << " group=" << group << "\n";
  s << pcgb_embedded_lm_params_h << "\n" << pcgb_embedded_lm_kernel_cuh << "\n" << model_source << "\n";
  s << "typedef " << model_struct << " PcgbModel;\n";
  s << "static_assert(PcgbModel::P == " << P << " && PcgbModel::C == " << C << ", \"model shape\");\n";
  const char* bounds = "__launch_bounds__(256)";
  const std::string lmb = lm_min_blocks > 0 ? "__launch_bounds__(" + std::to_string(kLmMaxThreads) + ", " +
                                                  std::to_string(lm_min_blocks) + ")"
                                            : std::string(bounds);
  const bool g0 = group == 0, g1 = group == 1, g2 = group == 2, g3 = group == 3, g4 = group == 4;
  for (int c = 1; c >= 0 && g0; --c)
    for (int b = 1; b >= 0; --b)
      s << "extern \"C\" __global__ void " << (c && b ? lmb : std::string(bounds)) << " pcgb_lm_c" << c << "_b" << b
        << "(const PcgbLmParams a) { pcgb::lm_grid<PcgbModel, " << M << ", " << ta << ", " << ts << ", "
        << (c ? "true" : "false") << ", " << (b ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g0; --c)
    s << "extern \"C\" __global__ void " << bounds << " pcgb_cost_c" << c
      << "(const PcgbLmParams a) { pcgb::cost_grid<PcgbModel, " << M << ", " << ta << ", " << (c ? "true" : "false")
      << ">(a); }\n";
  if (g0)
    s << "extern \"C\" __global__ void " << bounds << " pcgb_gmw81(const PcgbLmParams a) { pcgb::gmw81_grid<" << P
      << ", " << ts << ">(a); }\n";
  for (int c = 1; c >= 0 && g2; --c)
    for (int b = 1; b >= 0; --b)
      s << "extern \"C\" __global__ void " << (c && b ? lmb : std::string(bounds)) << " pcgb_lmq_c" << c << "_b" << b
        << "(const PcgbLmParams a) { pcgb::lm_refill_grid<PcgbModel, " << M << ", " << ta << ", " << ts << ", "
        << (c ? "true" : "false") << ", " << (b ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g2; --c)
    for (int b = 1; b >= 0; --b)
      s << "extern \"C\" __global__ void " << (c && b ? lmb : std::string(bounds)) << " pcgb_lmc_c" << c << "_b" << b
        << "(const PcgbLmParams a) { pcgb::lm_check_grid<PcgbModel, " << M << ", " << ta << ", " << ts << ", "
        << (c ? "true" : "false") << ", " << (b ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g3; --c)
    for (int b = 1; b >= 0; --b)
      s << "extern \"C\" __global__ void " << (c && b ? lmb : std::string(bounds)) << " pcgb_lms_c" << c << "_b" << b
        << "(const PcgbLmParams a) { pcgb::lm_select_grid<PcgbModel, " << M << ", " << ta << ", " << ts << ", "
        << (c ? "true" : "false") << ", " << (b ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g4; --c)
    for (int b = 1; b >= 0; --b)
      s << "extern \"C\" __global__ void " << (c && b ? lmb : std::string(bounds)) << " pcgb_lmw_c" << c << "_b" << b
        << "(const PcgbLmParams a) { pcgb::lm_warm_grid<PcgbModel, " << M << ", " << ta << ", " << ts << ", "
        << (c ? "true" : "false") << ", " << (b ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g1; --c)
    s << "extern \"C\" __global__ void " << bounds << " pcgb_search_c" << c
      << "(const PcgbLmParams a) { pcgb::search_step_grid<PcgbModel, " << M << ", " << ta << ", "
      << (c ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g1; --c)
    for (int b = 1; b >= 0; --b)
      s << "extern \"C\" __global__ void " << bounds << " pcgb_rs_c" << c << "_b" << b
        << "(const PcgbLmParams a) { pcgb::random_search_grid<PcgbModel, " << M << ", " << ta << ", " << ts << ", "
        << (c ? "true" : "false") << ", " << (b ? "true" : "false") << ">(a); }\n";
  for (int c = 1; c >= 0 && g2; --c) {
    s << "extern \"C\" __global__ void " << bounds << " pcgb_check_c" << c
      << "(const PcgbLmParams a) { pcgb::warm_check_grid<PcgbModel, " << M << ", " << ta << ", "
      << (c ? "true" : "false") << ">(a); }\n";
    s << "extern \"C\" __global__ void " << bounds << " pcgb_select_c" << c
      << "(const PcgbLmParams a) { pcgb::warm_select_grid<PcgbModel, " << M << ", " << ta << ", "
      << (c ? "true" : "false") << ">(a); }\n";
  }
  for (int c = 1; c >= 0 && g0; --c)
    s << "extern \"C\" __global__ void " << bounds << " pcgb_eval_c" << c
      << "(const PcgbLmParams a) { pcgb::eval_grid<PcgbModel, " << M << ", " << ta << ", " << (c ? "true" : "false")
      << ">(a); }\n";
  return s.str();
}

const std::vector<std::string>& nvrtc_options() {
  static const std::vector<std::string> opts = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo",
                                                "--ptxas-options=-v", "-default-device"};
  return opts;
}

int compile_cubin(const std::string& src, std::vector<char>& cubin, std::string& log,
                  const std::vector<std::string>& extra = {}) {
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "pcgb_fitter.cu", 0, nullptr, nullptr);
  if (r != NVRTC_SUCCESS) return fail(PCGB_ECOMPILE, "nvrtcCreateProgram: %s", nvrtcGetErrorString(r));
  std::vector<const char*> o;
  for (auto& s : nvrtc_options()) o.push_back(s.c_str());
  for (auto& s : extra) o.push_back(s.c_str());
  r = nvrtcCompileProgram(prog, int(o.size()), o.data());
  size_t ls = 0;
  nvrtcGetProgramLogSize(prog, &ls);
  log.assign(ls, '\0');
  if (ls) nvrtcGetProgramLog(prog, &log[0]);
  while (!log.empty() && log.back() == '\0') log.pop_back();
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return fail(PCGB_ECOMPILE, "NVRTC compile failed (%s):\n%s", nvrtcGetErrorString(r), log.c_str());
  }
  size_t n = 0;
  r = nvrtcGetCUBINSize(prog, &n);
  if (r != NVRTC_SUCCESS || n == 0) {
    nvrtcDestroyProgram(&prog);
    return fail(PCGB_ECOMPILE, "nvrtcGetCUBINSize: %s", nvrtcGetErrorString(r));
  }
  cubin.resize(n);
  r = nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  if (r != NVRTC_SUCCESS) return fail(PCGB_ECOMPILE, "nvrtcGetCUBIN: %s", nvrtcGetErrorString(r));
  return PCGB_OK;
}

bool read_file(const std::string& path, std::vector<char>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return !out.empty();
}

void write_file_atomic(const std::string& path, const std::vector<char>& data) {
  std::string tmp = path + ".tmp" + std::to_string(reinterpret_cast<uintptr_t>(&data));
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return;
    f.write(data.data(), std::streamsize(data.size()));
    if (!f) return;
  }
  std::rename(tmp.c_str(), path.c_str());
}

int check_device(const pcgb_fitter* ft) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (ft->device >= 0 && dev != ft->device)
    return fail(PCGB_EINVAL, "fitter was built on device %d but device %d is current", ft->device, dev);
  return PCGB_OK;
}

// The LM constants in both precisions: an fp32-state kernel reads the float
// copies instead of converting the doubles in every iteration (a double ->
// float conversion issues on the FP64 pipe).
void set_lm_constants(PcgbLmParams& p, double tol, double mu, double eta, double acc, double dec) {
  p.tol = tol;
  p.mu = mu;
  p.eta = eta;
  p.acc = acc;
  p.dec = dec;
  p.tol_f = float(tol);
  p.mu_f = float(mu);
  p.eta_f = float(eta);
  p.acc_f = float(acc);
  p.dec_f = float(dec);
}

int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > (int64_t(1) << 30)) g = int64_t(1) << 30;
  return int(g);
}

int kernel_of(pcgb_fitter* ft, int slot, cudaKernel_t* out);
int lm_block(const pcgb_fitter* ft, int slot, int block);

int launch(pcgb_fitter* ft, KernelSlot slot, PcgbLmParams prm, int64_t n, int block, void* stream) {
  cudaKernel_t kern = nullptr;
  if (int rc = kernel_of(ft, slot, &kern)) return rc;
  block = lm_block(ft, slot, block);
  if (block > kMaxBlock || block % 32) return fail(PCGB_EINVAL, "block must be a multiple of 32 up to %d", kMaxBlock);
  if (n == 0) return PCGB_OK;
  if (!prm.vox_idx) prm.n_items = n;
  void* args[] = {&prm};
  cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(kern), dim3(grid_for(n, block)),
                                   dim3(block), args, 0, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, kKernelNames[slot]);
  return PCGB_OK;
}

// launch() for work whose item count lives on the device (prm.n_items_dev,
// at most n): the kernel strides over its items, so the grid holds only as
// many blocks as are resident at once instead of one block per possible item
// (the blocks past the count would each start only to exit).
int launch_resident(pcgb_fitter* ft, KernelSlot slot, PcgbLmParams prm, int64_t n, int block, void* stream) {
  cudaKernel_t kern = nullptr;
  if (int rc = kernel_of(ft, slot, &kern)) return rc;
  block = lm_block(ft, slot, block);
  if (block > kMaxBlock || block % 32) return fail(PCGB_EINVAL, "block must be a multiple of 32 up to %d", kMaxBlock);
  if (n == 0) return PCGB_OK;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(kern), block, 0);
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  int grid = grid_for(n, block);
  if (int64_t(per_sm) * (sms > 0 ? sms : 1) < grid) grid = per_sm * (sms > 0 ? sms : 1);
  void* args[] = {&prm};
  e = cudaLaunchKernel(reinterpret_cast<const void*>(kern), dim3(grid), dim3(block), args, 0,
                       static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, kKernelNames[slot]);
  return PCGB_OK;
}

int fill_protocol(const pcgb_fitter* ft, PcgbLmParams& prm, int64_t cstride, int64_t n, const double* protocol,
                  int protocol_len) {
  if (cstride == 0) {
    const int need = ft->C * ft->M;
    if (need > PCGB_MAX_PROTOCOL) return fail(PCGB_ERANGE, "protocol of %d values exceeds %d", need, PCGB_MAX_PROTOCOL);
    if (need > 0 && (!protocol || protocol_len != need))
      return fail(PCGB_EINVAL, "shared protocol needs %d host values, got %d", need, protocol ? protocol_len : 0);
    for (int i = 0; i < need; ++i) {
      prm.protocol_d[i] = protocol[i];
      prm.protocol_f[i] = float(protocol[i]);
    }
  } else if (cstride != n) {
    return fail(PCGB_EINVAL, "consts_stride must be 0 (shared protocol) or nprobs");
  }
  prm.cstride = cstride;
  return PCGB_OK;
}

}  // namespace

namespace {

int validate_create(const char* model_source, const char* model_struct, int nparam, int nconst, int ndata, int dtype,
                    int solve_dtype) {
  if (!model_source || !model_struct || !*model_struct) return fail(PCGB_EINVAL, "model source/struct missing");
  if (nparam < 1 || nparam > PCGB_MAX_PARAMS) return fail(PCGB_ERANGE, "nparam %d outside 1..%d", nparam, PCGB_MAX_PARAMS);
  if (nconst < 0 || ndata < 1 || int64_t(nconst) * ndata > PCGB_MAX_PROTOCOL)
    return fail(PCGB_ERANGE, "nconst*ndata must fit %d (nconst=%d, ndata=%d)", PCGB_MAX_PROTOCOL, nconst, ndata);
  if ((dtype != PCGB_DTYPE_F32 && dtype != PCGB_DTYPE_F64) ||
      (solve_dtype != PCGB_DTYPE_F32 && solve_dtype != PCGB_DTYPE_F64))
    return fail(PCGB_EINVAL, "dtype must be 0 (float32) or 1 (float64)");
  if (dtype == PCGB_DTYPE_F64 && solve_dtype == PCGB_DTYPE_F32)
    return fail(PCGB_EINVAL, "a float64 state with a float32 solve is not supported");
  return PCGB_OK;
}

// Compiled cubin of a program source, from the disk cache when present.
int cubin_for_source(const std::string& src, const std::vector<std::string>& extra, const char* cache_dir,
                     std::vector<char>& cubin, std::string& log) {
  std::string key_src = src;
  for (auto& o : nvrtc_options()) key_src += "\n" + o;
  for (auto& o : extra) key_src += "\n" + o;
  int nv_major = 0, nv_minor = 0;
  nvrtcVersion(&nv_major, &nv_minor);
  key_src += "\nnvrtc " + std::to_string(nv_major) + "." + std::to_string(nv_minor);
  char keyhex[32];
  std::snprintf(keyhex, sizeof(keyhex), "%016llx", (unsigned long long)fnv1a(key_src));
  std::string cache_path;
  if (cache_dir && *cache_dir) cache_path = std::string(cache_dir) + "/pcgb_" + keyhex + ".cubin";
  if (cache_path.empty() || !read_file(cache_path, cubin)) {
    int rc = compile_cubin(src, cubin, log, extra);
    if (rc) return rc;
    if (!cache_path.empty()) write_file_atomic(cache_path, cubin);
  }
  return PCGB_OK;
}

int get_cubin(const char* model_source, const char* model_struct, int nparam, int nconst, int ndata, int dtype,
              int solve_dtype, const char* cache_dir, int group, int lm_min_blocks, std::vector<char>& cubin,
              std::string& log) {
  return cubin_for_source(
      program_source(model_source, model_struct, nparam, nconst, ndata, dtype, solve_dtype, group, lm_min_blocks),
      {}, cache_dir, cubin, log);
}

// Compile (or read from the cache) and load kernel group g of a fitter: first
// with the LM kernels' occupancy hint, again without it if any of them spills
// (local memory in use).
int load_group(pcgb_fitter* ft, int g) {
  const int tries[2] = {lm_min_blocks_of(g), 0};
  for (int t = 0; t < 2; ++t) {
    if (t == 1 && tries[0] == 0) break;
    std::vector<char> cubin;
    std::string log;
    if (int rc = get_cubin(ft->source.c_str(), ft->structname.c_str(), ft->P, ft->C, ft->M, ft->dtype, ft->sdtype,
                           ft->cache_dir.empty() ? nullptr : ft->cache_dir.c_str(), g, tries[t], cubin, log))
      return rc;
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaLibraryLoadData");
    cudaKernel_t ks[K_COUNT] = {};
    bool spills = false;
    for (int i = 0; i < K_COUNT; ++i) {
      if (group_of(i) != g) continue;
      e = cudaLibraryGetKernel(&ks[i], lib, kKernelNames[i]);
      if (e != cudaSuccess) {
        cudaLibraryUnload(lib);
        return cuda_fail(e, kKernelNames[i]);
      }
      if (tries[t] > 0 && is_lm_slot(i)) {
        cudaFuncAttributes fa{};
        e = cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(ks[i]));
        if (e != cudaSuccess) {
          cudaLibraryUnload(lib);
          return cuda_fail(e, "cudaFuncGetAttributes");
        }
        spills = spills || fa.localSizeBytes > kLmMaxSpillBytes;
      }
    }
    if (spills && t == 0) {
      cudaLibraryUnload(lib);
      continue;
    }
    for (int i = 0; i < K_COUNT; ++i)
      if (group_of(i) == g) ft->k[i] = ks[i];
    ft->lib[g] = lib;
    ft->lm_min_blocks[g] = tries[t];
    if (!log.empty()) ft->log += log;
    return PCGB_OK;
  }
  return fail(PCGB_ECOMPILE, "kernel group %d could not be loaded", g);
}

// Largest "N bytes spill stores" that ptxas reports for the register-capped
// LM kernels in a compile log (0 if the log is empty, e.g. served from cache).
size_t max_lm_spill_bytes(const std::string& log) {
  size_t worst = 0;
  for (int slot = 0; slot < K_COUNT; ++slot) {
    if (!is_lm_slot(slot)) continue;
    const std::string key = std::string("Function properties for ") + kKernelNames[slot] + "\n";
    const size_t at = log.find(key);
    if (at == std::string::npos) continue;
    const size_t sp = log.find("bytes spill stores", at);
    if (sp == std::string::npos) continue;
    size_t b = log.rfind(',', sp);
    b = b == std::string::npos ? at : b + 1;
    const size_t n = std::strtoull(log.c_str() + b, nullptr, 10);
    if (n > worst) worst = n;
  }
  return worst;
}

// Threads per block for an LM launch: kernels built with the occupancy hint
// take at most kLmMaxThreads (the per-voxel results do not depend on it).
int lm_block(const pcgb_fitter* ft, int slot, int block) {
  if (block <= 0) block = kDefaultBlock;
  if (is_lm_slot(slot) && ft->lm_min_blocks[group_of(slot)] > 0 && block > kLmMaxThreads) block = kLmMaxThreads;
  return block;
}

// The kernel of a slot, its group compiled and loaded on first use.
int kernel_of(pcgb_fitter* ft, int slot, cudaKernel_t* out) {
  std::lock_guard<std::mutex> lock(ft->mu);
  if (!ft->k[slot]) {
    if (int rc = load_group(ft, group_of(slot))) return rc;
  }
  if (!ft->k[slot]) return fail(PCGB_EINVAL, "kernel %s missing from program", kKernelNames[slot]);
  *out = ft->k[slot];
  return PCGB_OK;
}

static_assert(sizeof(PcgbMultiParams) <= 32000, "multi-model launch parameters exceed the 32 KB kernel parameter limit");

std::string multi_source(int n, const char* const* srcs, const char* const* structs, const int* P, const int* C,
                         const int* M, int dtype, int sdtype, int block, const int* lanes) {
  const char* ta = dtype == PCGB_DTYPE_F64 ? "double" : "float";
  const char* ts = sdtype == PCGB_DTYPE_F64 ? "double" : "float";
  std::ostringstream s;
  s << "// pcgb mixed-model program: " << n << " jobs, state=" << ta << " solve=" << ts << " block=" << block << "\n";
  s << pcgb_embedded_lm_params_h << "\n" << pcgb_embedded_lm_kernel_cuh << "\n";
  std::vector<std::string> seen;
  for (int k = 0; k < n; ++k) {
    bool dup = false;
    for (auto& x : seen) dup = dup || x == structs[k];
    if (!dup) {
      s << srcs[k] << "\n";
      seen.push_back(structs[k]);
    }
    s << "static_assert(" << structs[k] << "::P == " << P[k] << " && " << structs[k] << "::C == " << C[k]
      << ", \"model shape\");\n";
  }
  s << "struct PcgbDispatch {\n  static __device__ __forceinline__ void run(int k, const PcgbLmParams& a, long long base,"
       " int chunk, int lane) {\n    switch (k) {\n";
  // a model fitted with L lanes per voxel: lanes 2j, 2j + 1 (L = 2) share voxel j of each 16
  for (int k = 0; k < n; ++k) {
    const int L = lanes ? lanes[k] : 1;
    s << "      case " << k << ":\n        for (int j = lane / " << L << "; j < chunk; j += " << 32 / L << ") {\n"
      << "          const long long v = base + j;\n          if (v < a.N) pcgb::lm_fit_voxel<" << structs[k] << ", "
      << M[k] << ", " << ta << ", " << ts << ", true, true, " << L << ">(a, v, pcgb::NoEpilogue{}, lane % " << L
      << ");\n        }\n        break;\n";
  }
  s << "      default: break;\n    }\n  }\n};\n";
  s << "extern \"C\" __global__ void __launch_bounds__(" << block
    << ") pcgb_multi_lm(const PcgbMultiParams q) { pcgb::multi_grid<PcgbDispatch>(q); }\n";
  return s.str();
}

}  // namespace

struct pcgb_multi {
  int n = 0, dtype = 0, block = 128, device = -1;
  int P[PCGB_MAX_MODELS] = {}, C[PCGB_MAX_MODELS] = {}, M[PCGB_MAX_MODELS] = {};
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
  int blocks_per_sm = 0, sms = 0;
  std::string log;
};

extern "C" {

const char* pcgb_version(void) { return "pycompute-gb300 0.1 (sm_103a)"; }
int pcgb_max_params(void) { return PCGB_MAX_PARAMS; }
int pcgb_max_protocol(void) { return PCGB_MAX_PROTOCOL; }
const char* pcgb_last_error(void) { return g_err.c_str(); }

int pcgb_fitter_compile(const char* model_source, const char* model_struct, int nparam, int nconst, int ndata,
                        int dtype, int solve_dtype, const char* cache_dir, char* log_buf, size_t log_len) {
  g_err.clear();
  if (int rc = validate_create(model_source, model_struct, nparam, nconst, ndata, dtype, solve_dtype)) return rc;
  std::string all;
  for (int g = 0; g < kGroups; ++g) {
    std::vector<char> cubin;
    std::string log;
    if (int rc = get_cubin(model_source, model_struct, nparam, nconst, ndata, dtype, solve_dtype, cache_dir, g,
                           lm_min_blocks_of(g), cubin, log))
      return rc;
    // the register-capped LM kernels spill too much for this model: the
    // runtime will load the uncapped build, so compile (and cache) it too
    if (g != 1 && max_lm_spill_bytes(log) > kLmMaxSpillBytes) {
      all += log;
      log.clear();
      if (int rc = get_cubin(model_source, model_struct, nparam, nconst, ndata, dtype, solve_dtype, cache_dir, g, 0,
                             cubin, log))
        return rc;
    }
    all += log;
  }
  if (log_buf && log_len) {
    std::snprintf(log_buf, log_len, "%s", all.c_str());
  }
  return PCGB_OK;
}

int pcgb_fitter_create(const char* model_source, const char* model_struct, int nparam, int nconst, int ndata,
                       int dtype, int solve_dtype, const char* cache_dir, pcgb_fitter** out) {
  g_err.clear();
  if (!out) return fail(PCGB_EINVAL, "out is NULL");
  *out = nullptr;
  if (int rc = validate_create(model_source, model_struct, nparam, nconst, ndata, dtype, solve_dtype)) return rc;
  auto* ft = new (std::nothrow) pcgb_fitter();
  if (!ft) return fail(PCGB_ENOMEM, "out of host memory");
  ft->P = nparam;
  ft->C = nconst;
  ft->M = ndata;
  ft->dtype = dtype;
  ft->sdtype = solve_dtype;
  ft->source = model_source;
  ft->structname = model_struct;
  ft->cache_dir = cache_dir ? cache_dir : "";
  cudaError_t e = cudaGetDevice(&ft->device);
  if (e != cudaSuccess) {
    delete ft;
    return cuda_fail(e, "cudaGetDevice");
  }
  // the fit kernels now (a model that does not compile fails here); the
  // searches and the refill / fallback kernels when first used
  if (int rc = load_group(ft, 0)) {
    delete ft;
    return rc;
  }
  *out = ft;
  return PCGB_OK;
}

int pcgb_multi_create(int n_models, const char* const* model_sources, const char* const* model_structs,
                      const int* nparam, const int* nconst, const int* ndata, int dtype, int solve_dtype, int maxrreg,
                      int block, const int* lanes, const char* cache_dir, pcgb_multi** out) {
  g_err.clear();
  if (!out) return fail(PCGB_EINVAL, "out is NULL");
  *out = nullptr;
  if (n_models < 1 || n_models > PCGB_MAX_MODELS) return fail(PCGB_ERANGE, "1..%d models per program", PCGB_MAX_MODELS);
  if (!model_sources || !model_structs || !nparam || !nconst || !ndata) return fail(PCGB_EINVAL, "model arrays missing");
  if (block < 32 || block > 1024 || block % 32) return fail(PCGB_EINVAL, "block must be a multiple of 32 up to 1024");
  if (maxrreg != 0 && (maxrreg < 32 || maxrreg > 255)) return fail(PCGB_EINVAL, "maxrreg must be 0 or 32..255");
  for (int k = 0; k < n_models; ++k) {
    if (int rc = validate_create(model_sources[k], model_structs[k], nparam[k], nconst[k], ndata[k], dtype, solve_dtype))
      return rc;
    if (lanes && lanes[k] != 1 && lanes[k] != 2) return fail(PCGB_EINVAL, "lanes per voxel must be 1 or 2");
  }
  const std::string src =
      multi_source(n_models, model_sources, model_structs, nparam, nconst, ndata, dtype, solve_dtype, block, lanes);
  std::vector<std::string> extra;
  if (maxrreg) extra.push_back("--maxrregcount=" + std::to_string(maxrreg));
  std::vector<char> cubin;
  std::string log;
  if (int rc = cubin_for_source(src, extra, cache_dir, cubin, log)) return rc;
  auto* m = new (std::nothrow) pcgb_multi();
  if (!m) return fail(PCGB_ENOMEM, "out of host memory");
  m->n = n_models;
  m->dtype = dtype;
  m->block = block;
  m->log = log;
  for (int k = 0; k < n_models; ++k) {
    m->P[k] = nparam[k];
    m->C[k] = nconst[k];
    m->M[k] = ndata[k];
  }
  cudaError_t e = cudaGetDevice(&m->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->device);
  if (e == cudaSuccess) e = cudaLibraryLoadData(&m->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->kernel, m->lib, "pcgb_multi_lm");
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m->blocks_per_sm, reinterpret_cast<const void*>(m->kernel),
                                                      block, 0);
  if (e != cudaSuccess) {
    if (m->lib) cudaLibraryUnload(m->lib);
    delete m;
    return cuda_fail(e, "pcgb_multi_create");
  }
  if (m->blocks_per_sm < 1) m->blocks_per_sm = 1;
  *out = m;
  return PCGB_OK;
}

int pcgb_multi_destroy(pcgb_multi* m) {
  if (!m) return PCGB_OK;
  int rc = PCGB_OK;
  if (m->lib) {
    cudaError_t e = cudaLibraryUnload(m->lib);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaLibraryUnload");
  }
  delete m;
  return rc;
}

const char* pcgb_multi_log(const pcgb_multi* m) { return m ? m->log.c_str() : ""; }

int pcgb_multi_grid(const pcgb_multi* m) { return m ? m->blocks_per_sm * m->sms : 0; }

int pcgb_multi_run(pcgb_multi* m, const pcgb_multi_job* jobs, int n_jobs, const int* order, int iters, double tol,
                   double mu, double eta, double acc, double dec, int chunk, int grid, uint32_t* work_counter,
                   void* stream) {
  g_err.clear();
  if (!jobs || n_jobs < 1 || n_jobs > PCGB_MAX_MODELS) return fail(PCGB_EINVAL, "need 1..%d jobs", PCGB_MAX_MODELS);
  if (chunk < 32 || chunk % 32 || chunk > 4096) return fail(PCGB_EINVAL, "chunk must be a multiple of 32 up to 4096");
  // The warps claim chunk indices from a 32-bit counter up to (chunks + warps
  // of the grid); at most 2^31 chunks keep those claims below 2^32, so the
  // counter cannot wrap and hand out a chunk twice. Checked before anything
  // else touches the GPU, summing without overflow.
  {
    int64_t chunks = 0;
    for (int k = 0; k < n_jobs; ++k) {
      const int64_t n = jobs[k].nprobs;
      if (n < 0) return fail(PCGB_EINVAL, "job %d: nprobs < 0", k);
      chunks += n / chunk + (n % chunk != 0);
      if (chunks > kMaxMultiChunks)
        return fail(PCGB_ERANGE, "too many voxels for one call: at most 2^31 chunks of `chunk` voxels over all jobs "
                                 "(use a larger chunk or split the call)");
    }
  }
  if (!m) return fail(PCGB_EINVAL, "program is NULL");
  if (n_jobs != m->n) return fail(PCGB_EINVAL, "need one job per model of the program (%d)", m->n);
  if (iters < 0) return fail(PCGB_EINVAL, "iters must be >= 0");
  if (!work_counter) return fail(PCGB_EINVAL, "work_counter is NULL");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != m->device) return fail(PCGB_EINVAL, "program was built on device %d but device %d is current", m->device, dev);
  PcgbMultiParams q;
  std::memset(&q, 0, sizeof(q));
  q.counter = work_counter;
  q.njobs = n_jobs;
  q.chunk = chunk;
  bool used[PCGB_MAX_MODELS] = {};
  for (int t = 0; t < n_jobs; ++t) {
    const int k = order ? order[t] : t;
    if (k < 0 || k >= n_jobs || used[k]) return fail(PCGB_EINVAL, "order must be a permutation of 0..n_jobs-1");
    used[k] = true;
    q.order[t] = k;
  }
  for (int k = 0; k < n_jobs; ++k) {
    const pcgb_multi_job& j = jobs[k];
    PcgbLmParams& a = q.jobs[k];
    if (j.nprobs < 0) return fail(PCGB_EINVAL, "job %d: nprobs < 0", k);
    if (j.nprobs > 0 && (!j.data || !j.params || !j.lam || !j.step_type || !j.f || !j.first_f || !j.last_f))
      return fail(PCGB_EINVAL, "job %d: data, params, lam, step_type, f, first_f and last_f are required", k);
    const int need = m->C[k] * m->M[k];
    if (need > 0 && !j.protocol) return fail(PCGB_EINVAL, "job %d: protocol missing", k);
    if (!j.lb || !j.ub) return fail(PCGB_EINVAL, "job %d: bounds missing", k);
    for (int i = 0; i < need; ++i) {
      a.protocol_d[i] = j.protocol[i];
      a.protocol_f[i] = float(j.protocol[i]);
    }
    for (int p = 0; p < m->P[k]; ++p) {
      a.shared_lb_d[p] = j.lb[p];
      a.shared_ub_d[p] = j.ub[p];
      a.shared_lb_f[p] = float(j.lb[p]);
      a.shared_ub_f[p] = float(j.ub[p]);
    }
    a.pars = j.params;
    a.data = j.data;
    a.lam = j.lam;
    a.step_type = reinterpret_cast<signed char*>(j.step_type);
    a.f = j.f;
    a.first_f = j.first_f;
    a.last_f = j.last_f;
    a.iters_done = j.iters_done;
    a.N = j.nprobs;
    a.n_items = j.nprobs;
    a.iters = iters;
    set_lm_constants(a, tol, mu, eta, acc, dec);
  }
  long long off = 0;
  for (int t = 0; t < n_jobs; ++t) {
    q.chunk_off[t] = off;
    off += (jobs[q.order[t]].nprobs + chunk - 1) / chunk;
  }
  q.chunk_off[n_jobs] = off;
  if (off == 0) return PCGB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  if (grid <= 0) grid = m->blocks_per_sm * m->sms;
  void* args[] = {&q};
  e = cudaLaunchKernel(reinterpret_cast<const void*>(m->kernel), dim3(grid), dim3(m->block), args, 0, s);
  if (e != cudaSuccess) return cuda_fail(e, "pcgb_multi_lm");
  return PCGB_OK;
}

int pcgb_fitter_destroy(pcgb_fitter* ft) {
  if (!ft) return PCGB_OK;
  int rc = PCGB_OK;
  for (int g = 0; g < kGroups; ++g) {
    if (!ft->lib[g]) continue;
    cudaError_t e = cudaLibraryUnload(ft->lib[g]);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaLibraryUnload");
  }
  delete ft;
  return rc;
}

const char* pcgb_fitter_log(const pcgb_fitter* ft) { return ft ? ft->log.c_str() : ""; }

// Fallback epilogue of an LM launch: 1 = the warm fit's check (pcgb_lm_run_check),
// 2 = the refit's select (pcgb_lm_run_select).
struct FallbackArgs {
  int mode = 0;
  const double* init_values = nullptr;
  double lam0 = 5.0;
  void* cost = nullptr;
  void* pars_backup = nullptr;
  void* cost_backup = nullptr;
  int32_t* fb_idx = nullptr;
  uint32_t* fb_count = nullptr;
  int8_t* which = nullptr;
};

static int lm_run_impl(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, const int32_t* vox_idx, int64_t n_items, void* stream,
                       uint32_t* work_counter = nullptr, int grid = 0, const uint32_t* n_items_dev = nullptr,
                       const FallbackArgs* fb = nullptr, int flags = 0, double lam0 = 0.0) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0 || iters < 0) return fail(PCGB_EINVAL, "nprobs and iters must be >= 0");
  const bool fresh = flags == (PCGB_LM_FRESH | PCGB_LM_PARS_ONLY);
  if (nprobs > 0 && fresh && (!data || !params))
    return fail(PCGB_EINVAL, "data and params are required");
  if (nprobs > 0 && !fresh && (!data || !params || !lam || !step_type || !f || !first_f || !last_f))
    return fail(PCGB_EINVAL, "data, params, lam, step_type, f, first_f and last_f are required");
  if (int rc = check_device(ft)) return rc;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  if (bounds_stride == 0) {
    if (!lb_host || !ub_host) return fail(PCGB_EINVAL, "shared bounds need lb_host and ub_host");
    for (int k = 0; k < ft->P; ++k) {
      prm.shared_lb_d[k] = lb_host[k];
      prm.shared_ub_d[k] = ub_host[k];
      prm.shared_lb_f[k] = float(lb_host[k]);
      prm.shared_ub_f[k] = float(ub_host[k]);
    }
  } else if (bounds_stride != nprobs || !lower_bound || !upper_bound) {
    return fail(PCGB_EINVAL, "bounds_stride must be 0 (shared) or nprobs with device bounds");
  }
  prm.pars = params;
  prm.consts = consts;
  prm.data = data;
  prm.lb = lower_bound;
  prm.ub = upper_bound;
  prm.lam = lam;
  prm.step_type = reinterpret_cast<signed char*>(step_type);
  prm.f = f;
  prm.first_f = first_f;
  prm.last_f = last_f;
  prm.step = step;
  prm.iters_done = iters_done;
  prm.N = nprobs;
  prm.bstride = bounds_stride;
  prm.iters = iters;
  prm.flags = flags;
  if (fresh) prm.lam_start = lam0;
  set_lm_constants(prm, tol, mu, eta, acc, dec);
  const KernelSlot slot = consts_stride == 0 ? (bounds_stride == 0 ? K_LM_C1_B1 : K_LM_C1_B0)
                                             : (bounds_stride == 0 ? K_LM_C0_B1 : K_LM_C0_B0);
  if (fb) {
    if (nprobs > (int64_t(1) << 31) - 1) return fail(PCGB_ERANGE, "the fallback indexes voxels with int32");
    if (!fb->fb_count) return fail(PCGB_EINVAL, "fb_count is required");
    if (nprobs > 0 && (!fb->fb_idx || !fb->cost || !fb->pars_backup || !fb->cost_backup))
      return fail(PCGB_EINVAL, "fallback buffers (cost, backups, fb_idx) are required");
    prm.cost = fb->cost;
    prm.pars_backup = fb->pars_backup;
    prm.cost_backup = fb->cost_backup;
    prm.fb_idx = fb->fb_idx;
    prm.fb_count = fb->fb_count;
    prm.which = reinterpret_cast<signed char*>(fb->which);
    if (fb->mode == 1) {
      if (!fb->init_values) return fail(PCGB_EINVAL, "init_values are required");
      for (int k = 0; k < ft->P; ++k) prm.init_val[k] = float(fb->init_values[k]);
      prm.lam0 = fb->lam0;
      cudaError_t e = cudaMemsetAsync(fb->fb_count, 0, 2 * sizeof(uint32_t), static_cast<cudaStream_t>(stream));
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
      return launch(ft, KernelSlot(slot + (K_LMC_C1_B1 - K_LM_C1_B1)), prm, nprobs, block, stream);
    }
    prm.vox_idx = fb->fb_idx;
    prm.n_items = nprobs;
    prm.n_items_dev = fb->fb_count;
    return launch_resident(ft, KernelSlot(slot + (K_LMS_C1_B1 - K_LM_C1_B1)), prm, nprobs, block, stream);
  }
  if (work_counter) {
    // refill schedule: persistent grid, warps claim 256-item chunks from the counter
    const KernelSlot q = KernelSlot(slot + (K_LMQ_C1_B1 - K_LM_C1_B1));
    if (vox_idx) {
      if (n_items < 0) return fail(PCGB_EINVAL, "n_items must be >= 0");
      prm.vox_idx = vox_idx;
      prm.n_items = n_items;
    } else {
      prm.n_items = nprobs;
    }
    if (prm.n_items == 0) return PCGB_OK;
    if (prm.n_items / 256 >= (int64_t(1) << 31)) return fail(PCGB_ERANGE, "too many voxels for one refill launch");
    prm.work = work_counter;
    prm.n_items_dev = n_items_dev;
    if (block <= 0) block = kDefaultBlock;
    if (block > kMaxBlock || block % 32) return fail(PCGB_EINVAL, "block must be a multiple of 32 up to %d", kMaxBlock);
    cudaKernel_t kq = nullptr;
    if (int rc = kernel_of(ft, q, &kq)) return rc;
    block = lm_block(ft, q, block);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    if (grid <= 0) {
      int per_sm = 0, dev = 0, sms = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(kq), block, 0);
      if (e != cudaSuccess || per_sm < 1) per_sm = 1;
      grid = per_sm * sms;
      const int64_t need = (prm.n_items + block - 1) / block;
      if (grid > need) grid = int(need);
    }
    void* args[] = {&prm};
    e = cudaLaunchKernel(reinterpret_cast<const void*>(kq), dim3(grid), dim3(block), args, 0, st);
    if (e != cudaSuccess) return cuda_fail(e, kKernelNames[q]);
    return PCGB_OK;
  }
  if (vox_idx) {
    if (n_items < 0) return fail(PCGB_EINVAL, "n_items must be >= 0");
    prm.vox_idx = vox_idx;
    prm.n_items = n_items;
    prm.n_items_dev = n_items_dev;
    if (n_items_dev) return launch_resident(ft, slot, prm, n_items, block, stream);
    return launch(ft, slot, prm, n_items, block, stream);
  }
  return launch(ft, slot, prm, nprobs, block, stream);
}

int pcgb_lm_run(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type, void* f,
                void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host, int block,
                void* stream) {
  return lm_run_impl(ft, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride, tol, mu, eta, acc, dec,
                     params, step, lam, step_type, f, first_f, last_f, iters_done, nprobs, iters, protocol_host,
                     protocol_len, lb_host, ub_host, block, nullptr, 0, stream);
}

int pcgb_lm_run_fresh(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                      const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                      double eta, double acc, double dec, void* params, int8_t* step_type, int64_t nprobs, int iters,
                      const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                      double lam0, int block, void* stream) {
  g_err.clear();
  if (!(lam0 > 0.0)) return fail(PCGB_EINVAL, "lam0 must be > 0");
  return lm_run_impl(ft, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride, tol, mu, eta, acc, dec,
                     params, nullptr, nullptr, step_type, nullptr, nullptr, nullptr, nullptr, nprobs, iters,
                     protocol_host, protocol_len, lb_host, ub_host, block, nullptr, 0, stream, nullptr, 0, nullptr,
                     nullptr, PCGB_LM_FRESH | PCGB_LM_PARS_ONLY, lam0);
}

int pcgb_lm_run_refill(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, const int32_t* vox_idx, int64_t n_items, const uint32_t* n_items_dev,
                       uint32_t* work_counter, int grid, void* stream) {
  g_err.clear();
  if (!work_counter) return fail(PCGB_EINVAL, "work_counter is NULL");
  if (n_items_dev && !vox_idx) return fail(PCGB_EINVAL, "n_items_dev needs vox_idx");
  return lm_run_impl(ft, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride, tol, mu, eta, acc, dec,
                     params, step, lam, step_type, f, first_f, last_f, iters_done, nprobs, iters, protocol_host,
                     protocol_len, lb_host, ub_host, block, vox_idx, n_items, stream, work_counter, grid, n_items_dev);
}

int pcgb_lm_run_check(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                      const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                      double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                      void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                      const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                      int block, const double* init_values, double lam0, void* cost, void* pars_backup,
                      void* cost_backup, int32_t* fb_idx, uint32_t* fb_count, void* stream) {
  g_err.clear();
  FallbackArgs fb;
  fb.mode = 1;
  fb.init_values = init_values;
  fb.lam0 = lam0;
  fb.cost = cost;
  fb.pars_backup = pars_backup;
  fb.cost_backup = cost_backup;
  fb.fb_idx = fb_idx;
  fb.fb_count = fb_count;
  return lm_run_impl(ft, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride, tol, mu, eta, acc, dec,
                     params, step, lam, step_type, f, first_f, last_f, iters_done, nprobs, iters, protocol_host,
                     protocol_len, lb_host, ub_host, block, nullptr, 0, stream, nullptr, 0, nullptr, &fb);
}

int pcgb_lm_run_select(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, void* cost, const void* pars_backup, const void* cost_backup,
                       const int32_t* fb_idx, uint32_t* fb_count, int8_t* which, void* stream) {
  g_err.clear();
  FallbackArgs fb;
  fb.mode = 2;
  fb.cost = cost;
  fb.pars_backup = const_cast<void*>(pars_backup);
  fb.cost_backup = const_cast<void*>(cost_backup);
  fb.fb_idx = const_cast<int32_t*>(fb_idx);
  fb.fb_count = fb_count;
  fb.which = which;
  return lm_run_impl(ft, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride, tol, mu, eta, acc, dec,
                     params, step, lam, step_type, f, first_f, last_f, iters_done, nprobs, iters, protocol_host,
                     protocol_len, lb_host, ub_host, block, nullptr, 0, stream, nullptr, 0, nullptr, &fb);
}

// Launch parameters of a fallback check (pcgb_warm_check, pcgb_warm_lm_check).
static int check_params(pcgb_fitter* ft, PcgbLmParams& prm, const void* consts, int64_t consts_stride,
                        const void* data, const void* lower_bound, const void* upper_bound, int64_t bounds_stride,
                        const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                        const double* init_values, double lam0, void* params, void* lam, int8_t* step_type, void* f,
                        void* cost, void* pars_backup, void* cost_backup, int32_t* fb_idx, uint32_t* fb_count,
                        int64_t nprobs) {
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
  if (nprobs > (int64_t(1) << 31) - 1) return fail(PCGB_ERANGE, "warm check indexes voxels with int32");
  if (!fb_count || !init_values) return fail(PCGB_EINVAL, "fb_count and init_values are required");
  if (nprobs > 0 && (!data || !params || !lam || !step_type || !f || !cost || !pars_backup || !cost_backup || !fb_idx))
    return fail(PCGB_EINVAL, "data, params, lam, step_type, f, cost, backups and fb_idx are required");
  if (int rc = check_device(ft)) return rc;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  if (bounds_stride == 0) {
    if (!lb_host || !ub_host) return fail(PCGB_EINVAL, "shared bounds need lb_host and ub_host");
    for (int k = 0; k < ft->P; ++k) {
      prm.shared_lb_d[k] = lb_host[k];
      prm.shared_ub_d[k] = ub_host[k];
      prm.shared_lb_f[k] = float(lb_host[k]);
      prm.shared_ub_f[k] = float(ub_host[k]);
    }
  } else if (bounds_stride != nprobs || !lower_bound || !upper_bound) {
    return fail(PCGB_EINVAL, "bounds_stride must be 0 (shared) or nprobs with device bounds");
  }
  for (int k = 0; k < ft->P; ++k) prm.init_val[k] = float(init_values[k]);
  prm.pars = params;
  prm.consts = consts;
  prm.data = data;
  prm.lb = lower_bound;
  prm.ub = upper_bound;
  prm.bstride = bounds_stride;
  prm.lam = lam;
  prm.step_type = reinterpret_cast<signed char*>(step_type);
  prm.f = f;
  prm.cost = cost;
  prm.pars_backup = pars_backup;
  prm.cost_backup = cost_backup;
  prm.fb_idx = fb_idx;
  prm.fb_count = fb_count;
  prm.lam0 = lam0;
  prm.N = nprobs;
  prm.n_items = nprobs;
  return PCGB_OK;
}

int pcgb_warm_check(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                    const void* lower_bound, const void* upper_bound, int64_t bounds_stride,
                    const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                    const double* init_values, double lam0, void* params, void* lam, int8_t* step_type, void* f,
                    void* cost, void* pars_backup, void* cost_backup, int32_t* fb_idx, uint32_t* fb_count,
                    int64_t nprobs, void* stream) {
  g_err.clear();
  PcgbLmParams prm;
  if (int rc = check_params(ft, prm, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride,
                            protocol_host, protocol_len, lb_host, ub_host, init_values, lam0, params, lam, step_type,
                            f, cost, pars_backup, cost_backup, fb_idx, fb_count, nprobs))
    return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(fb_count, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  return launch(ft, consts_stride == 0 ? K_CHECK_C1 : K_CHECK_C0, prm, nprobs, 256, stream);
}

int pcgb_warm_lm_check(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, int iters, double lam_start, const double* protocol_host,
                       int protocol_len, const double* lb_host, const double* ub_host, const double* init_values,
                       double lam0, void* params, void* lam, int8_t* step_type, void* f, void* cost,
                       void* pars_backup, void* cost_backup, int32_t* fb_idx, uint32_t* fb_count, int64_t nprobs,
                       int block, void* stream) {
  g_err.clear();
  if (iters < 0) return fail(PCGB_EINVAL, "iters must be >= 0");
  if (!(lam_start > 0.0)) return fail(PCGB_EINVAL, "lam_start must be > 0");
  PcgbLmParams prm;
  if (int rc = check_params(ft, prm, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride,
                            protocol_host, protocol_len, lb_host, ub_host, init_values, lam0, params, lam, step_type,
                            f, cost, pars_backup, cost_backup, fb_idx, fb_count, nprobs))
    return rc;
  prm.iters = iters;
  prm.flags = PCGB_LM_FRESH | PCGB_LM_PARS_ONLY;
  prm.lam_start = lam_start;
  set_lm_constants(prm, tol, mu, eta, acc, dec);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(fb_count, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  const KernelSlot slot = consts_stride == 0 ? (bounds_stride == 0 ? K_LMW_C1_B1 : K_LMW_C1_B0)
                                             : (bounds_stride == 0 ? K_LMW_C0_B1 : K_LMW_C0_B0);
  return launch(ft, slot, prm, nprobs, block, stream);
}

int pcgb_warm_select(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                     const double* protocol_host, int protocol_len, void* params, void* cost, const void* pars_backup,
                     const void* cost_backup, const int32_t* fb_idx, uint32_t* fb_count, int8_t* which,
                     int64_t nprobs, void* stream) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
  if (!fb_count) return fail(PCGB_EINVAL, "fb_count is required");
  if (nprobs > 0 && (!data || !params || !cost || !pars_backup || !cost_backup || !fb_idx))
    return fail(PCGB_EINVAL, "data, params, cost, backups and fb_idx are required");
  if (int rc = check_device(ft)) return rc;
  if (nprobs == 0) return PCGB_OK;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  prm.pars = params;
  prm.consts = consts;
  prm.data = data;
  prm.cost = cost;
  prm.pars_backup = const_cast<void*>(pars_backup);
  prm.cost_backup = const_cast<void*>(cost_backup);
  prm.fb_idx = const_cast<int*>(fb_idx);
  prm.fb_count = fb_count;
  prm.n_items_dev = fb_count;
  prm.n_items = nprobs;
  prm.which = reinterpret_cast<signed char*>(which);
  prm.N = nprobs;
  const KernelSlot slot = consts_stride == 0 ? K_SELECT_C1 : K_SELECT_C0;
  cudaKernel_t ksel = nullptr;
  if (int rc = kernel_of(ft, slot, &ksel)) return rc;
  // the flagged count is known only on the device: a grid of 8 blocks per SM strides over it
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = 8 * (sms > 0 ? sms : 1);
  const int64_t need = (nprobs + 255) / 256;
  if (grid > need) grid = int(need);
  void* args[] = {&prm};
  cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(ksel), dim3(grid), dim3(256), args, 0,
                                   static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, kKernelNames[slot]);
  return PCGB_OK;
}

int pcgb_lm_run_subset(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, double tol, double mu,
                       double eta, double acc, double dec, void* params, void* step, void* lam, int8_t* step_type,
                       void* f, void* first_f, void* last_f, int32_t* iters_done, int64_t nprobs, int iters,
                       const double* protocol_host, int protocol_len, const double* lb_host, const double* ub_host,
                       int block, const int32_t* vox_idx, int64_t n_items, const uint32_t* n_items_dev,
                       void* stream) {
  g_err.clear();
  if (!vox_idx) return fail(PCGB_EINVAL, "vox_idx is NULL");
  return lm_run_impl(ft, consts, consts_stride, data, lower_bound, upper_bound, bounds_stride, tol, mu, eta, acc, dec,
                     params, step, lam, step_type, f, first_f, last_f, iters_done, nprobs, iters, protocol_host,
                     protocol_len, lb_host, ub_host, block, vox_idx, n_items, stream, nullptr, 0, n_items_dev);
}

int pcgb_f_run_subset(pcgb_fitter* ft, const void* params, const void* consts, int64_t consts_stride,
                      const void* data, const int8_t* step_type, void* f, int64_t nprobs, const double* protocol_host,
                      int protocol_len, const int32_t* vox_idx, int64_t n_items, void* stream);

int pcgb_f_run(pcgb_fitter* ft, const void* params, const void* consts, int64_t consts_stride, const void* data,
               const int8_t* step_type, void* f, int64_t nprobs, const double* protocol_host, int protocol_len,
               void* stream) {
  return pcgb_f_run_subset(ft, params, consts, consts_stride, data, step_type, f, nprobs, protocol_host, protocol_len,
                           nullptr, 0, stream);
}

int pcgb_f_run_subset(pcgb_fitter* ft, const void* params, const void* consts, int64_t consts_stride,
                      const void* data, const int8_t* step_type, void* f, int64_t nprobs, const double* protocol_host,
                      int protocol_len, const int32_t* vox_idx, int64_t n_items, void* stream) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
  if (nprobs > 0 && (!params || !data || !f)) return fail(PCGB_EINVAL, "params, data and f are required");
  if (int rc = check_device(ft)) return rc;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  prm.pars = const_cast<void*>(params);
  prm.consts = consts;
  prm.data = data;
  prm.step_type = const_cast<signed char*>(reinterpret_cast<const signed char*>(step_type));
  prm.f = f;
  prm.N = nprobs;
  if (vox_idx) {
    if (n_items < 0) return fail(PCGB_EINVAL, "n_items must be >= 0");
    prm.vox_idx = vox_idx;
    prm.n_items = n_items;
    return launch(ft, consts_stride == 0 ? K_COST_C1 : K_COST_C0, prm, n_items, 0, stream);
  }
  return launch(ft, consts_stride == 0 ? K_COST_C1 : K_COST_C0, prm, nprobs, 0, stream);
}

int pcgb_model_eval(pcgb_fitter* ft, const void* params, const void* consts, int64_t consts_stride, void* out,
                    int64_t nprobs, const double* protocol_host, int protocol_len, void* stream) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
  if (nprobs > 0 && (!params || !out)) return fail(PCGB_EINVAL, "params and out are required");
  if (int rc = check_device(ft)) return rc;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  prm.pars = const_cast<void*>(params);
  prm.consts = consts;
  prm.model_out = out;
  prm.N = nprobs;
  return launch(ft, consts_stride == 0 ? K_EVAL_C1 : K_EVAL_C0, prm, nprobs, 0, stream);
}

int pcgb_search_step(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data, const void* p,
                     void* f, void* best_p, void* best_f, int64_t nprobs, const double* protocol_host,
                     int protocol_len, void* stream) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
  if (nprobs > 0 && (!data || !p || !f || !best_p || !best_f))
    return fail(PCGB_EINVAL, "data, p, f, best_p and best_f are required");
  if (int rc = check_device(ft)) return rc;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  prm.pars = const_cast<void*>(p);
  prm.consts = consts;
  prm.data = data;
  prm.f = f;
  prm.best_p = best_p;
  prm.best_f = best_f;
  prm.N = nprobs;
  return launch(ft, consts_stride == 0 ? K_SEARCH_C1 : K_SEARCH_C0, prm, nprobs, 0, stream);
}

int pcgb_random_search(pcgb_fitter* ft, const void* consts, int64_t consts_stride, const void* data,
                       const void* lower_bound, const void* upper_bound, int64_t bounds_stride, void* best_p,
                       void* best_f, int64_t nprobs, int draws, int lm_iters, double tol, double mu, double eta,
                       double acc, double dec, uint64_t seed, const double* protocol_host, int protocol_len,
                       const double* lb_host, const double* ub_host, void* stream) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0 || draws < 0 || lm_iters < 0) return fail(PCGB_EINVAL, "nprobs, draws, lm_iters must be >= 0");
  if (nprobs > 0 && (!data || !best_p || !best_f)) return fail(PCGB_EINVAL, "data, best_p and best_f are required");
  if (int rc = check_device(ft)) return rc;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  if (int rc = fill_protocol(ft, prm, consts_stride, nprobs, protocol_host, protocol_len)) return rc;
  if (consts_stride != 0 && !consts) return fail(PCGB_EINVAL, "per-voxel consts pointer is NULL");
  if (bounds_stride == 0) {
    if (!lb_host || !ub_host) return fail(PCGB_EINVAL, "shared bounds need lb_host and ub_host");
    for (int k = 0; k < ft->P; ++k) {
      prm.shared_lb_d[k] = lb_host[k];
      prm.shared_ub_d[k] = ub_host[k];
      prm.shared_lb_f[k] = float(lb_host[k]);
      prm.shared_ub_f[k] = float(ub_host[k]);
    }
  } else if (bounds_stride != nprobs || !lower_bound || !upper_bound) {
    return fail(PCGB_EINVAL, "bounds_stride must be 0 (shared) or nprobs with device bounds");
  }
  prm.consts = consts;
  prm.data = data;
  prm.lb = lower_bound;
  prm.ub = upper_bound;
  prm.bstride = bounds_stride;
  prm.best_p = best_p;
  prm.best_f = best_f;
  prm.N = nprobs;
  prm.iters = draws;
  prm.lm_iters = lm_iters;
  prm.seed = seed;
  set_lm_constants(prm, tol, mu, eta, acc, dec);
  const KernelSlot slot = consts_stride == 0 ? (bounds_stride == 0 ? K_RS_C1_B1 : K_RS_C1_B0)
                                             : (bounds_stride == 0 ? K_RS_C0_B1 : K_RS_C0_B0);
  return launch(ft, slot, prm, nprobs, 0, stream);
}

int pcgb_gmw81_solve(pcgb_fitter* ft, const void* mat, const void* rhs, void* sol, int64_t nprobs, void* stream) {
  g_err.clear();
  if (!ft) return fail(PCGB_EINVAL, "fitter is NULL");
  if (nprobs < 0) return fail(PCGB_EINVAL, "nprobs must be >= 0");
  if (nprobs > 0 && (!mat || !rhs || !sol)) return fail(PCGB_EINVAL, "mat, rhs and sol are required");
  if (int rc = check_device(ft)) return rc;
  PcgbLmParams prm;
  std::memset(&prm, 0, sizeof(prm));
  prm.consts = mat;
  prm.data = rhs;
  prm.step = sol;
  prm.N = nprobs;
  return launch(ft, K_GMW, prm, nprobs, 0, stream);
}

}  // extern "C"
