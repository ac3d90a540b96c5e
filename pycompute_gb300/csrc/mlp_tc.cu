// Warm-start network inference on the 5th-generation tensor cores (tcgen05).
//
// Same network and numerics as mlp_infer_kernel in mlp.cu (16 -> 128 -> 128
// -> 128 -> P, GELU, bf16 operands, fp32 accumulation; the bf16 roundings
// happen at the same points), restructured for sm_103a:
//
//   * one CTA per SM, 16 warps = 4 warpgroups; each warpgroup owns one
//     128-voxel tile at a time (thread t of the warpgroup = voxel t = TMEM
//     lane t) and its own 128 TMEM columns for the layer accumulator, and
//     loads the next tile's signals while it works on the current one;
//   * a layer is D[128 x N] = A[128 x K] * W^T with A (activations) and W
//     (weights, N x K) in shared memory, issued as K/16 tcgen05.mma
//     (kind::f16, bf16 x bf16 -> f32, M = 128) by one thread of the
//     warpgroup and tracked by tcgen05.commit on the warpgroup's mbarrier;
//   * the bias enters the accumulator through one more MMA per layer (see
//     TcSmem), so the epilogue reads the pre-activation row of its voxel from
//     TMEM (tcgen05.ld 32x32b), applies GELU and writes the bf16 row as the
//     next layer's A operand back into shared memory (as 2 GELU, with the
//     next layer's weights staged halved: same products, one multiply fewer
//     per activation);
//   * the warpgroups run independent tiles, so one warpgroup's MMAs overlap
//     the other warpgroups' epilogues.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8 x 16-byte core matrices (8 rows x 8 bf16), element (r, k) of an R x K
// operand at byte (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (next core matrix along K) and SBO = K / 8 * 128 (next
// 8-row group). Every wait on an mbarrier is bounded: on timeout the kernel
// records an error in *status, stops issuing work and still frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "mlp_math.cuh"
#include "tc_common.cuh"
#include "pcgb.h"

namespace pcgb_mlp_tc {

using pcgb_mlp::bf16;

constexpr int NIN = 16;
constexpr int HID = 128;
constexpr int NOUT_MMA = 16;  // the last layer's N (>= P, multiple of 16)
constexpr int NOUT_MAX = 8;
constexpr int NWG = 4;        // warpgroups (tiles in flight) per CTA
constexpr int THREADS = NWG * 128;
constexpr int TMEM_COLS = 512;  // >= NWG x 128 accumulator columns, a power of 2
constexpr int LDH_G = HID + 8;  // leading dimension of the hidden weights in global memory
constexpr int LD1_G = NIN + 8;  // ... of the first layer's weights
constexpr unsigned kWaitLimit = 1u << 22;  // default try_wait rounds before a wait counts as lost

// The biases enter the accumulators through one more MMA per layer: A = a
// 128 x 16 tile whose first two columns are 1, B = the layer's bias split
// into two bf16 terms (b_hi = bf16(b), b_lo = bf16(b - b_hi): b to 2^-16
// relative) in its first two columns. The epilogue then has no bias add.
struct __align__(1024) TcSmem {
  bf16 w1[HID * NIN];
  bf16 w2[HID * HID];
  bf16 w3[HID * HID];
  bf16 w4[NOUT_MMA * HID];
  bf16 bias[3][HID * 16];   // B operands of the bias MMAs of layers 1-3
  bf16 bias4[NOUT_MMA * 16];
  bf16 ones[128 * 16];      // A operand of the bias MMAs
  // per warpgroup: the layer-1 input tile (128 x 16) at the start of its
  // activation tile (128 x 128); the first epilogue overwrites it only after
  // the layer-1 MMAs that read it have completed
  bf16 act[NWG][128 * HID];
  unsigned long long mbar[NWG];
  uint32_t tmem_base;
};

struct TcArgs {
  const float* signals;  // SoA (NIN, n)
  long long n;
  const bf16* w[4];      // bf16 weights, rows x (in + 8)
  const float* mw[4];    // fp32 master copies; column `in` holds the bias
  int nout;
  int log_in;
  int kinds[NOUT_MAX];
  float mean[NOUT_MAX], stdv[NOUT_MAX], lb[NOUT_MAX], ub[NOUT_MAX];
  float* out;            // SoA (nout, n)
  int* status;           // 0 = ok, else the kernel lost an mbarrier wait (may be null)
  unsigned wait_limit;   // try_wait rounds before a wait counts as lost
  long long skip_tile;   // failure-path test: this tile's first layer is never issued (-1 = none)
};

using namespace pcgb_tc;

// copy a rows x kdim bf16 matrix (global leading dimension ldg) into the
// core-matrix layout (rows >= rows_live are zero), halved when `halve` (the
// layers after a GELU receive 2 GELU, which keeps every product unchanged)
__device__ void stage_weights(bf16* dst, const bf16* src, int rows, int rows_live, int kdim, int ldg, bool halve) {
  const int chunks = rows * (kdim / 8);
  unsigned char* base = reinterpret_cast<unsigned char*>(dst);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    const int r = c / (kdim / 8), k = (c % (kdim / 8)) * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r < rows_live) v = *reinterpret_cast<const uint4*>(src + (long long)r * ldg + k);
    if (halve) v = pcgb_mlp::halve_bf16x8(v);
    *reinterpret_cast<uint4*>(base + core_off(r, k, kdim)) = v;
  }
}

// 2 GELU of 16 pre-activations (columns [c0, c0 + 16), bias included; c0 a
// multiple of 16, so each column's recipe is fixed at compile time), written
// as bf16 into row r of the next layer's A operand (row_base = its byte offset)
__device__ __forceinline__ void gelu_row16(const uint32_t (&acc)[16], int c0, unsigned char* row_base) {
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    uint4 o;
    uint32_t* w = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int j = q * 8 + 2 * e;
      w[e] = pcgb_mlp::gelu2x_col_pack_bf16(__uint_as_float(acc[j]), __uint_as_float(acc[j + 1]), c0 + j);
    }
    *reinterpret_cast<uint4*>(row_base + ((c0 + q * 8) >> 3) * 128) = o;
  }
}

// B operand (rows x 16, core-matrix layout) of a bias MMA: columns 0 and 1 hold
// the two bf16 terms of each row's fp32 bias, the rest is zero
__device__ void stage_bias(bf16* dst, const float* master, int rows, int rows_live, int ld, int col) {
  unsigned char* base = reinterpret_cast<unsigned char*>(dst);
  for (int c = threadIdx.x; c < rows * 2; c += blockDim.x) {
    const int r = c >> 1, k = (c & 1) * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (k == 0 && r < rows_live) {
      const float b = master[(long long)r * ld + col];
      const bf16 hi = __float2bfloat16_rn(b);
      const bf16 lo = __float2bfloat16_rn(b - __bfloat162float(hi));
      v.x = uint32_t(__bfloat16_as_ushort(hi)) | (uint32_t(__bfloat16_as_ushort(lo)) << 16);
    }
    *reinterpret_cast<uint4*>(base + core_off(r, k, 16)) = v;
  }
}

__global__ void __launch_bounds__(THREADS, 1) mlp_infer_tc_kernel(const TcArgs p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcSmem& S = *reinterpret_cast<TcSmem*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = warp >> 2;                   // warpgroup
  const int r = (warp & 3) * 32 + lane;      // voxel row of the tile = TMEM lane

  // weights, biases, barriers, TMEM
  stage_weights(S.w1, p.w[0], HID, HID, NIN, LD1_G, false);
  stage_weights(S.w2, p.w[1], HID, HID, HID, LDH_G, true);
  stage_weights(S.w3, p.w[2], HID, HID, HID, LDH_G, true);
  stage_weights(S.w4, p.w[3], NOUT_MMA, NOUT_MAX, HID, LDH_G, true);
  stage_bias(S.bias[0], p.mw[0], HID, HID, LD1_G, NIN);
  stage_bias(S.bias[1], p.mw[1], HID, HID, LDH_G, HID);
  stage_bias(S.bias[2], p.mw[2], HID, HID, LDH_G, HID);
  stage_bias(S.bias4, p.mw[3], NOUT_MMA, NOUT_MAX, LDH_G, HID);
  for (int c = threadIdx.x; c < 128 * 2; c += blockDim.x) {
    const int r = c >> 1, k = (c & 1) * 8;
    const uint32_t one2 = 0x3F803F80u;  // two bf16 ones
    const uint4 v = k == 0 ? make_uint4(one2, 0, 0, 0) : make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.ones) + core_off(r, k, 16)) = v;
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < NWG; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar[i])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();  // staged weights -> visible to the tensor cores
  fence_before_sync();
  __syncthreads();
  fence_after_sync();

  const uint32_t tbase = S.tmem_base;
  const uint32_t d_tmem = tbase + uint32_t(g * 128);                           // lane 0, this warpgroup's columns
  const uint32_t t_row = tbase + (uint32_t((warp & 3) * 32) << 16) + uint32_t(g * 128);  // this warp's lanes
  const uint32_t mbar = smem_u32(&S.mbar[g]);
  const uint32_t xs = smem_u32(S.act[g]), as = smem_u32(S.act[g]);
  const uint32_t w1s = smem_u32(S.w1), w2s = smem_u32(S.w2), w3s = smem_u32(S.w3), w4s = smem_u32(S.w4);
  const uint32_t ones_s = smem_u32(S.ones);
  const bool issuer = r == 0;
  constexpr uint32_t ID_HID = idesc_bf16(128, HID), ID_OUT = idesc_bf16(128, NOUT_MMA);
  uint32_t phase = 0;
  bool lost = false;

  const long long ntiles = (p.n + 127) / 128;
  const long long tstride = (long long)gridDim.x * NWG;
  // signals of the next tile, loaded one tile ahead of their use
  float s_next[NIN];
  {
    const long long v0 = ((long long)blockIdx.x * NWG + g) * 128 + r;
#pragma unroll
    for (int k = 0; k < NIN; ++k) s_next[k] = v0 < p.n ? p.signals[(long long)k * p.n + v0] : 0.f;
  }
  for (long long tile = (long long)blockIdx.x * NWG + g; tile < ntiles && !lost; tile += tstride) {
    const long long v = tile * 128 + r;
    // ---- inputs: 16 samples of voxel v -> bf16 row r of x
    float s[NIN];
    float mx = 0.f;
#pragma unroll
    for (int k = 0; k < NIN; ++k) {
      s[k] = s_next[k];
      mx = fmaxf(mx, s[k]);
    }
    {
      const long long vn = v + tstride * 128;
#pragma unroll
      for (int k = 0; k < NIN; ++k) s_next[k] = vn < p.n ? p.signals[(long long)k * p.n + vn] : 0.f;
    }
    mx = fmaxf(mx, 1e-20f);
    const float inv = 1.f / mx;
    {
      unsigned char* xb = reinterpret_cast<unsigned char*>(S.act[g]);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        uint4 o;
        uint32_t* w = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
        for (int e = 0; e < 4; ++e)
          w[e] = pcgb_mlp::pack_bf16(pcgb_mlp::input_transform(s[q * 8 + 2 * e], inv, p.log_in),
                                     pcgb_mlp::input_transform(s[q * 8 + 2 * e + 1], inv, p.log_in));
        *reinterpret_cast<uint4*>(xb + core_off(r, q * 8, NIN)) = o;
      }
    }
    // ---- four layers
    for (int layer = 0; layer < 4; ++layer) {
      fence_async_smem();   // this thread's A row -> visible to the tensor cores
      fence_before_sync();  // its earlier TMEM reads are done
      wg_sync(g);
      // failure-path test: the issuer skips the layer's MMAs and their commit,
      // so the mbarrier phase never completes while no tensor-core work of this
      // warpgroup is in flight, and the wait below runs out
      const bool skip = layer == 0 && tile == p.skip_tile;
      if (issuer && !skip) {
        fence_after_sync();
        if (layer == 0) {
          mma_bf16(d_tmem, smem_desc(xs, 128, 256), smem_desc(w1s, 128, 256), ID_HID, 0u);
        } else {
          const uint32_t ws = layer == 1 ? w2s : (layer == 2 ? w3s : w4s);
          const uint32_t id = layer == 3 ? ID_OUT : ID_HID;
#pragma unroll
          for (int kk = 0; kk < HID / 16; ++kk)
            mma_bf16(d_tmem, smem_desc(as + kk * 256, 128, 2048), smem_desc(ws + kk * 256, 128, 2048), id,
                     kk > 0 ? 1u : 0u);
        }
        // + bias: ones (128 x 16) times the layer's bias terms (N x 16)
        const uint32_t bs = layer < 3 ? smem_u32(S.bias[layer]) : smem_u32(S.bias4);
        mma_bf16(d_tmem, smem_desc(ones_s, 128, 256), smem_desc(bs, 128, 256), layer == 3 ? ID_OUT : ID_HID, 1u);
        mma_commit(mbar);
      }
      // one warp polls the mbarrier; the other three wait in the hardware
      // barrier below and take no issue slots from the other tiles' epilogues
      const bool ok = (warp & 3) != 0 || mbar_wait(mbar, phase, p.wait_limit);
      phase ^= 1u;
      if (wg_sync_any(g, !ok)) {
        lost = true;
        break;
      }
      fence_after_sync();
      if (layer < 3) {
        // 16 columns at a time, the next chunk's TMEM load in flight while
        // this chunk's GELU runs
        unsigned char* row_base = reinterpret_cast<unsigned char*>(S.act[g]) + core_off(r, 0, HID);
        uint32_t a0[16], a1[16];
        tmem_ld16_start(t_row, a0);
        tmem_wait16(a0);
#pragma unroll
        for (int c = 0; c < HID / 16; c += 2) {
          tmem_ld16_start(t_row + uint32_t((c + 1) * 16), a1);
          gelu_row16(a0, c * 16, row_base);
          tmem_wait16(a1);
          if (c + 2 < HID / 16) tmem_ld16_start(t_row + uint32_t((c + 2) * 16), a0);
          gelu_row16(a1, (c + 1) * 16, row_base);
          if (c + 2 < HID / 16) tmem_wait16(a0);
        }
      } else {
        float y[16];
        tmem_ld16(t_row, y);
        if (v < p.n) {
#pragma unroll
          for (int k = 0; k < NOUT_MAX; ++k) {
            if (k >= p.nout) break;
            const float t = y[k] * p.stdv[k] + p.mean[k];
            const int kind = p.kinds[k];
            float val = kind == 0 ? t * mx : (kind == 2 ? expf(t) : t);
            val = fminf(fmaxf(val, p.lb[k]), p.ub[k]);
            p.out[(long long)k * p.n + v] = val;
          }
        }
      }
    }
  }
  if (lost && issuer) {
    // the lost phase may still complete: give the warpgroup's MMAs a second
    // bounded wait before the TMEM they write is returned
    (void)mbar_wait(mbar, phase ^ 1u, p.wait_limit);
    if (p.status) atomicExch(p.status, 1);
  }
  // all TMEM reads done before the allocation is returned
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
  }
}

thread_local std::string g_err;

}  // namespace pcgb_mlp_tc

using namespace pcgb_mlp_tc;

extern "C" {

const char* pcgb_mlp_tc_last_error(void) { return g_err.c_str(); }

int pcgb_mlp_forward_tc(const float* signals, int64_t n, int nin, int log_in, const void* const* w_bf16,
                        const float* const* w_master, int nout, const int* kinds, const float* mean, const float* stdv,
                        const float* lb, const float* ub, float* out, int* status, void* stream) {
  return pcgb_mlp_forward_tc_ex(signals, n, nin, log_in, w_bf16, w_master, nout, kinds, mean, stdv, lb, ub, out,
                                status, 0u, -1, stream);
}

int pcgb_mlp_forward_tc_ex(const float* signals, int64_t n, int nin, int log_in, const void* const* w_bf16,
                           const float* const* w_master, int nout, const int* kinds, const float* mean,
                           const float* stdv, const float* lb, const float* ub, float* out, int* status,
                           unsigned wait_limit, int64_t skip_tile, void* stream) {
  g_err.clear();
  if (n < 0) {
    g_err = "n must be >= 0";
    return PCGB_EINVAL;
  }
  if (nin != NIN) {
    g_err = "the tensor-core forward is built for 16 inputs";
    return PCGB_EINVAL;
  }
  if (nout < 1 || nout > NOUT_MAX) {
    g_err = "nout must be 1..8";
    return PCGB_EINVAL;
  }
  if (!w_bf16 || !w_master || !kinds || !mean || !stdv || !lb || !ub) {
    g_err = "weights and output transforms are required";
    return PCGB_EINVAL;
  }
  if (n == 0) return PCGB_OK;
  if (!signals || !out) {
    g_err = "signals and out are required";
    return PCGB_EINVAL;
  }
  TcArgs a{};
  a.signals = signals;
  a.n = n;
  for (int l = 0; l < 4; ++l) {
    a.w[l] = static_cast<const bf16*>(w_bf16[l]);
    a.mw[l] = w_master[l];
  }
  a.nout = nout;
  a.log_in = log_in;
  for (int k = 0; k < NOUT_MAX; ++k) {
    a.kinds[k] = k < nout ? kinds[k] : 1;
    a.mean[k] = k < nout ? mean[k] : 0.f;
    a.stdv[k] = k < nout ? stdv[k] : 1.f;
    a.lb[k] = k < nout ? lb[k] : -3.0e38f;
    a.ub[k] = k < nout ? ub[k] : 3.0e38f;
  }
  a.out = out;
  a.status = status;
  a.wait_limit = wait_limit ? wait_limit : kWaitLimit;
  a.skip_tile = skip_tile;
  const int smem = int(sizeof(TcSmem));
  cudaError_t e = cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) {
    g_err = cudaGetErrorString(e);
    return PCGB_ECUDA;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;
  const long long tiles = (n + 127) / 128;
  long long blocks = (tiles + NWG - 1) / NWG;
  if (blocks > sms) blocks = sms;
  mlp_infer_tc_kernel<<<unsigned(blocks), THREADS, smem, static_cast<cudaStream_t>(stream)>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_err = cudaGetErrorString(e);
    return PCGB_ECUDA;
  }
  return PCGB_OK;
}

}  // extern "C"
