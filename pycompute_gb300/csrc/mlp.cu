// Warm-start network kernels: a 16 -> 128 -> 128 -> 128 -> P multilayer
// perceptron with GELU activations (tanh form), bf16 weights and fp32 accumulation on the
// tensor cores (mma.sync m16n8k16 bf16 -> f32, operands staged with ldmatrix).
//
// The reference has no learned component; these kernels supply the initial
// parameters of the LM fit. Layouts (row-major, voxel/sample index outermost):
//   layer l weights  W_l (out_pad x ldw) with ldw = in_l + 8; column in_l of
//                    the fp32 master copy holds the bias, the bf16 copy is the
//                    GEMM operand (bias column unused)
//   activations      (batch x (width + 8)) bf16; column `width` is 1.0 so the
//                    weight-gradient GEMM also produces the bias gradient
//   pre-activations  (batch x width) fp32
// Inference fuses all four layers in one kernel: each warp keeps a 16-voxel
// tile in registers and turns the fp32 accumulator fragments of one layer
// directly into the bf16 A fragments of the next, so activations never leave
// the SM. Training is a short sequence of GEMM launches with fused epilogues
// (bias + GELU, GELU', split-K weight-gradient accumulation) plus loss and
// Adam kernels; the host captures a whole step in a CUDA graph.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "mlp_math.cuh"
#include "pcgb.h"

namespace pcgb_mlp {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(addr));
}
// D += A(16x16, row) * B(16x8, col), bf16 inputs, fp32 accumulators
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// ---- generic bf16 GEMM with fused epilogues -------------------------------

enum Epilogue { EPI_FWD_GELU = 0, EPI_FWD_LINEAR = 1, EPI_BWD_DGELU = 2, EPI_DW_ATOMIC = 3, EPI_STORE_F32 = 4 };

struct GemmArgs {
  const bf16* A;
  long long lda;
  const bf16* B;
  long long ldb;
  long long M, N, K;
  long long k_split;      // K range per blockIdx.z (multiple of 32)
  const float* bias;      // bias[n * bias_stride]
  long long bias_stride;
  float* out_f32;         // z / y / dW
  long long ldo;
  bf16* out_bf16;         // a / dz
  long long ldob;
  const float* zin;       // pre-activation for GELU'
  long long ldz;
};

constexpr int BM = 64, BN = 64, BK = 32, PADE = 8;

// C(M x N) = A(M x K) * B(K x N).
//   A_ROW: A stored (M, K) row-major, else (K, M) row-major (read transposed)
//   B_NK : B stored (N, K) row-major, else (K, N) row-major (read transposed)
// K, lda, ldb multiples of 8 (16-byte rows); M, N arbitrary (masked).
template <bool A_ROW, bool B_NK, int EPI>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const GemmArgs g) {
  __shared__ __align__(16) bf16 sA[A_ROW ? BM : BK][(A_ROW ? BK : BM) + PADE];
  __shared__ __align__(16) bf16 sB[B_NK ? BN : BK][(B_NK ? BK : BN) + PADE];
  const long long m0 = (long long)blockIdx.y * BM, n0 = (long long)blockIdx.x * BN;
  const long long kbeg = (long long)blockIdx.z * g.k_split;
  const long long kend = kbeg + g.k_split < g.K ? kbeg + g.k_split : g.K;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

  for (long long k0 = kbeg; k0 < kend; k0 += BK) {
    // global -> shared, 16-byte chunks, zero outside the matrix
#pragma unroll
    for (int c = threadIdx.x; c < 256; c += 128) {
      uint4 v = make_uint4(0, 0, 0, 0);
      if (A_ROW) {
        const int r = c >> 2, cc = (c & 3) * 8;
        const long long gm = m0 + r, gk = k0 + cc;
        if (gm < g.M && gk < kend) v = *reinterpret_cast<const uint4*>(g.A + gm * g.lda + gk);
        *reinterpret_cast<uint4*>(&sA[r][cc]) = v;
      } else {
        const int r = c >> 3, cc = (c & 7) * 8;
        const long long gk = k0 + r, gm = m0 + cc;
        if (gk < kend && gm < g.M) v = *reinterpret_cast<const uint4*>(g.A + gk * g.lda + gm);
        *reinterpret_cast<uint4*>(&sA[r][cc]) = v;
      }
    }
#pragma unroll
    for (int c = threadIdx.x; c < 256; c += 128) {
      uint4 v = make_uint4(0, 0, 0, 0);
      if (B_NK) {
        const int r = c >> 2, cc = (c & 3) * 8;
        const long long gn = n0 + r, gk = k0 + cc;
        if (gn < g.N && gk < kend) v = *reinterpret_cast<const uint4*>(g.B + gn * g.ldb + gk);
        *reinterpret_cast<uint4*>(&sB[r][cc]) = v;
      } else {
        const int r = c >> 3, cc = (c & 7) * 8;
        const long long gk = k0 + r, gn = n0 + cc;
        if (gk < kend && gn < g.N) v = *reinterpret_cast<const uint4*>(g.B + gk * g.ldb + gn);
        *reinterpret_cast<uint4*>(&sB[r][cc]) = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bfr[2][4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (A_ROW)
          ldsm_x4(af[i], smem_u32(&sA[wm + i * 16 + (lane & 15)][kk + 8 * (lane >> 4)]));
        else
          ldsm_x4_t(af[i], smem_u32(&sA[kk + 8 * (lane >> 4) + (lane & 7)][wm + i * 16 + 8 * ((lane >> 3) & 1)]));
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        if (B_NK)
          ldsm_x4(bfr[j], smem_u32(&sB[wn + j * 16 + 8 * (lane >> 4) + (lane & 7)][kk + 8 * ((lane >> 3) & 1)]));
        else
          ldsm_x4_t(bfr[j], smem_u32(&sB[kk + 8 * ((lane >> 3) & 1) + (lane & 7)][wn + j * 16 + 8 * (lane >> 4)]));
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
          mma16816(acc[i][nt], af[i], bfr[nt >> 1][(nt & 1) * 2], bfr[nt >> 1][(nt & 1) * 2 + 1]);
    }
    __syncthreads();
  }

  const int gq = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const long long m = m0 + wm + i * 16 + gq + (e >= 2 ? 8 : 0);
        const long long n = n0 + wn + nt * 8 + 2 * tq + (e & 1);
        if (m >= g.M || n >= g.N) continue;
        const float v = acc[i][nt][e];
        if (EPI == EPI_FWD_GELU) {
          const float z = v + g.bias[n * g.bias_stride];
          g.out_f32[m * g.ldo + n] = z;
          g.out_bf16[m * g.ldob + n] = __float2bfloat16_rn(gelu_col(z, int(n)));
        } else if (EPI == EPI_FWD_LINEAR) {
          g.out_f32[m * g.ldo + n] = v + g.bias[n * g.bias_stride];
        } else if (EPI == EPI_BWD_DGELU) {
          g.out_bf16[m * g.ldob + n] = __float2bfloat16_rn(v * gelu_grad_col(g.zin[m * g.ldz + n], int(n)));
        } else if (EPI == EPI_DW_ATOMIC) {
          atomicAdd(&g.out_f32[m * g.ldo + n], v);
        } else {
          g.out_f32[m * g.ldo + n] = v;
        }
      }
}

// ---- loss gradient, Adam ----------------------------------------------------

// dy = 2 (y - t) / (batch * nout) for the first nout columns, 0 in the padding;
// loss_sum += sum (y - t)^2 / (batch * nout)
__global__ void mse_grad_kernel(const float* y, const float* t, long long ldy, long long batch, int nout, int ncols,
                                bf16* dy, long long lddy, float* loss_sum) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < batch * ncols) {
    const long long r = i / ncols;
    const int c = int(i % ncols);
    float d = 0.f;
    if (c < nout) {
      const float e = y[r * ldy + c] - t[r * ldy + c];
      d = 2.f * e / float(batch * nout);
      l = e * e / float(batch * nout);
    }
    dy[r * lddy + c] = __float2bfloat16_rn(d);
  }
  // warp reduce then one atomic per warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && loss_sum) atomicAdd(loss_sum, l);
}

// Adam (Kingma & Ba 2015) with bias correction; rows >= rows_live of the
// (rows x ld) buffer are padding and stay zero. The gradient is cleared.
// corr[0], corr[1] = 1 - b1^t, 1 - b2^t and corr[2] = learning-rate scale, in
// device memory so a captured graph can replay the step with fresh values.
__global__ void adam_kernel(float* master, float* m, float* v, float* grad, bf16* wbf, long long rows, long long ld,
                            long long rows_live, float lr, float b1, float b2, float eps, const float* corr) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * ld) return;
  const float c1 = corr[0], c2 = corr[1];
  lr *= corr[2];
  const long long r = i / ld;
  const float gi = grad[i];
  grad[i] = 0.f;
  if (r >= rows_live) return;
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float w = master[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  master[i] = w;
  wbf[i] = __float2bfloat16_rn(w);
}

// ---- training inputs and targets --------------------------------------------

// x_rows (n x ldx) bf16 = transformed signals per voxel, column nin = 1,
// remaining padding 0; snorm[v] = the per-voxel maximum. signals are SoA (nin, n).
__global__ void prepare_inputs_kernel(const float* signals, long long n, int nin, bf16* x_rows, long long ldx,
                                      float* snorm, int log_in) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  float mx = 0.f;
  for (int k = 0; k < nin; ++k) mx = fmaxf(mx, signals[(long long)k * n + v]);
  mx = fmaxf(mx, 1e-20f);
  const float inv = 1.f / mx;
  for (int k = 0; k < ldx; ++k) {
    float x = k < nin ? input_transform(signals[(long long)k * n + v], inv, log_in) : (k == nin ? 1.f : 0.f);
    x_rows[v * ldx + k] = __float2bfloat16_rn(x);
  }
  if (snorm) snorm[v] = mx;
}

// targets (n x ldt) = (g_k(p_k) - mean_k) / std_k with g_k per output kind:
// 0: p / snorm, 1: p, 2: log(p). params are SoA (nout, n).
__global__ void prepare_targets_kernel(const float* params, const float* snorm, long long n, int nout,
                                       const int* kinds, const float* mean, const float* stdv, float* targets,
                                       long long ldt) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  for (int k = 0; k < ldt; ++k) {
    float t = 0.f;
    if (k < nout) {
      const float p = params[(long long)k * n + v];
      const int kind = kinds[k];
      const float gk = kind == 0 ? p / snorm[v] : (kind == 2 ? logf(fmaxf(p, 1e-30f)) : p);
      t = (gk - mean[k]) / stdv[k];
    }
    targets[v * ldt + k] = t;
  }
}

// ---- fused inference ---------------------------------------------------------

constexpr int HID = 128;
constexpr int LDH = HID + 8;
constexpr int NOUT_PAD = 8;

struct InferArgs {
  const float* signals;  // SoA (nin, n)
  long long n;
  const bf16* w[4];      // layer weights (rows x ld), ld = in + 8
  const float* mw[4];    // fp32 master copies; column `in` = bias
  int nout;
  int log_in;
  int kinds[NOUT_PAD];
  float mean[NOUT_PAD], stdv[NOUT_PAD], lb[NOUT_PAD], ub[NOUT_PAD];
  float* out;            // SoA (nout, n)
};

template <int NIN>
struct InferSmem {
  bf16 w1[HID][NIN + 8];
  bf16 w2[HID][LDH];
  bf16 w3[HID][LDH];
  bf16 w4[NOUT_PAD][LDH];
  float b1[HID], b2[HID], b3[HID], b4[NOUT_PAD];
};

// pre-activations (16 voxels x 128 in 16 n8 tiles, bias included) -> 2 GELU ->
// bf16 A fragments of the next layer (8 k16 tiles), whose weights are staged
// halved; this lane's columns are 16 kt + 2 tq (+ 1) and 16 kt + 8 + 2 tq (+ 1)
__device__ __forceinline__ void act_to_afrag(const float (&acc)[16][4], uint32_t (&a)[8][4], int tq) {
#pragma unroll
  for (int kt = 0; kt < 8; ++kt) {
    const float* lo = acc[2 * kt];
    const float* hi = acc[2 * kt + 1];
    a[kt][0] = gelu2x_col_pack_bf16(lo[0], lo[1], 2 * tq);
    a[kt][1] = gelu2x_col_pack_bf16(lo[2], lo[3], 2 * tq);
    a[kt][2] = gelu2x_col_pack_bf16(hi[0], hi[1], 8 + 2 * tq);
    a[kt][3] = gelu2x_col_pack_bf16(hi[2], hi[3], 8 + 2 * tq);
  }
}

// accumulators start at the layer's bias (column 2t, 2t+1 of each n8 tile)
__device__ __forceinline__ void bias_init(float (&acc)[16][4], const float* bias, int tq) {
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const float b0 = bias[nt * 8 + 2 * tq], b1 = bias[nt * 8 + 2 * tq + 1];
    acc[nt][0] = b0;
    acc[nt][1] = b1;
    acc[nt][2] = b0;
    acc[nt][3] = b1;
  }
}

template <int NIN>
__device__ __forceinline__ void hidden_layer(const bf16 (*w)[LDH], const float* bias, const uint32_t (&a)[8][4],
                                             float (&acc)[16][4], int lane) {
  bias_init(acc, bias, lane & 3);
#pragma unroll
  for (int kt = 0; kt < 8; ++kt)
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      uint32_t b[4];
      ldsm_x4(b, smem_u32(&w[j * 16 + 8 * (lane >> 4) + (lane & 7)][kt * 16 + 8 * ((lane >> 3) & 1)]));
      mma16816(acc[2 * j], a[kt], b[0], b[1]);
      mma16816(acc[2 * j + 1], a[kt], b[2], b[3]);
    }
}

template <int NIN>
__global__ void __launch_bounds__(384, 1) mlp_infer_kernel(const InferArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<InferSmem<NIN>*>(smem_raw);
  // stage weights and biases; layers 2-4 halved, their inputs are 2 GELU
  for (int i = threadIdx.x; i < HID * (NIN + 8) / 8; i += blockDim.x) {
    const int r = i / ((NIN + 8) / 8), c = (i % ((NIN + 8) / 8)) * 8;
    *reinterpret_cast<uint4*>(&S.w1[r][c]) = *reinterpret_cast<const uint4*>(p.w[0] + r * (NIN + 8) + c);
  }
  for (int i = threadIdx.x; i < HID * LDH / 8; i += blockDim.x) {
    const int r = i / (LDH / 8), c = (i % (LDH / 8)) * 8;
    *reinterpret_cast<uint4*>(&S.w2[r][c]) = halve_bf16x8(*reinterpret_cast<const uint4*>(p.w[1] + r * LDH + c));
    *reinterpret_cast<uint4*>(&S.w3[r][c]) = halve_bf16x8(*reinterpret_cast<const uint4*>(p.w[2] + r * LDH + c));
  }
  for (int i = threadIdx.x; i < NOUT_PAD * LDH / 8; i += blockDim.x) {
    const int r = i / (LDH / 8), c = (i % (LDH / 8)) * 8;
    *reinterpret_cast<uint4*>(&S.w4[r][c]) = halve_bf16x8(*reinterpret_cast<const uint4*>(p.w[3] + r * LDH + c));
  }
  for (int i = threadIdx.x; i < HID; i += blockDim.x) {
    S.b1[i] = p.mw[0][i * (NIN + 8) + NIN];
    S.b2[i] = p.mw[1][i * LDH + HID];
    S.b3[i] = p.mw[2][i * LDH + HID];
  }
  if (threadIdx.x < NOUT_PAD) S.b4[threadIdx.x] = p.mw[3][threadIdx.x * LDH + HID];
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const long long ntiles = (p.n + 15) / 16;
  for (long long tile = (long long)blockIdx.x * (blockDim.x >> 5) + warp; tile < ntiles;
       tile += (long long)gridDim.x * (blockDim.x >> 5)) {
    const long long v0 = tile * 16 + gq, v1 = v0 + 8;
    // inputs: this thread holds samples {2t, 2t+1, 2t+8, 2t+9} (+16 per k16 tile) of voxels v0 and v1
    constexpr int KT1 = NIN / 16;
    float x0[KT1][4], x1[KT1][4];
    float m0 = 0.f, m1 = 0.f;
#pragma unroll
    for (int kt = 0; kt < KT1; ++kt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int k = kt * 16 + 2 * tq + (e & 1) + (e >= 2 ? 8 : 0);
        x0[kt][e] = v0 < p.n ? p.signals[(long long)k * p.n + v0] : 0.f;
        x1[kt][e] = v1 < p.n ? p.signals[(long long)k * p.n + v1] : 0.f;
        m0 = fmaxf(m0, x0[kt][e]);
        m1 = fmaxf(m1, x1[kt][e]);
      }
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 1));
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, 2));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 1));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, 2));
    m0 = fmaxf(m0, 1e-20f);
    m1 = fmaxf(m1, 1e-20f);
    const float i0 = 1.f / m0, i1 = 1.f / m1;
    float acc[16][4];
    bias_init(acc, S.b1, tq);
#pragma unroll
    for (int kt = 0; kt < KT1; ++kt) {
      uint32_t a[4];
      const int li = p.log_in;
      a[0] = pack_bf16(input_transform(x0[kt][0], i0, li), input_transform(x0[kt][1], i0, li));
      a[1] = pack_bf16(input_transform(x1[kt][0], i1, li), input_transform(x1[kt][1], i1, li));
      a[2] = pack_bf16(input_transform(x0[kt][2], i0, li), input_transform(x0[kt][3], i0, li));
      a[3] = pack_bf16(input_transform(x1[kt][2], i1, li), input_transform(x1[kt][3], i1, li));
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        uint32_t b[4];
        ldsm_x4(b, smem_u32(&S.w1[j * 16 + 8 * (lane >> 4) + (lane & 7)][kt * 16 + 8 * ((lane >> 3) & 1)]));
        mma16816(acc[2 * j], a, b[0], b[1]);
        mma16816(acc[2 * j + 1], a, b[2], b[3]);
      }
    }
    uint32_t af[8][4];
    act_to_afrag(acc, af, lane & 3);
    hidden_layer<NIN>(S.w2, S.b2, af, acc, lane);
    act_to_afrag(acc, af, lane & 3);
    hidden_layer<NIN>(S.w3, S.b3, af, acc, lane);
    act_to_afrag(acc, af, lane & 3);
    float y[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
      uint32_t b[2];
      ldsm_x2(b, smem_u32(&S.w4[lane & 7][kt * 16 + 8 * ((lane >> 3) & 1)]));
      mma16816(y, af[kt], b[0], b[1]);
    }
    // y[0], y[1]: voxel v0, outputs 2t, 2t+1; y[2], y[3]: voxel v1
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int k = 2 * tq + (e & 1);
      const long long v = e >= 2 ? v1 : v0;
      if (k >= p.nout || v >= p.n) continue;
      const float t = (y[e] + S.b4[k]) * p.stdv[k] + p.mean[k];
      const int kind = p.kinds[k];
      float val = kind == 0 ? t * (e >= 2 ? m1 : m0) : (kind == 2 ? expf(t) : t);
      val = fminf(fmaxf(val, p.lb[k]), p.ub[k]);
      p.out[(long long)k * p.n + v] = val;
    }
  }
}

thread_local std::string g_mlp_err;

int mlp_fail(int code, const char* msg) {
  g_mlp_err = msg;
  return code;
}

template <bool AR, bool BN>
cudaError_t launch_gemm(int epi, const GemmArgs& g, dim3 grid, cudaStream_t s) {
  switch (epi) {
    case EPI_FWD_GELU: gemm_bf16_kernel<AR, BN, EPI_FWD_GELU><<<grid, 128, 0, s>>>(g); break;
    case EPI_FWD_LINEAR: gemm_bf16_kernel<AR, BN, EPI_FWD_LINEAR><<<grid, 128, 0, s>>>(g); break;
    case EPI_BWD_DGELU: gemm_bf16_kernel<AR, BN, EPI_BWD_DGELU><<<grid, 128, 0, s>>>(g); break;
    case EPI_DW_ATOMIC: gemm_bf16_kernel<AR, BN, EPI_DW_ATOMIC><<<grid, 128, 0, s>>>(g); break;
    default: gemm_bf16_kernel<AR, BN, EPI_STORE_F32><<<grid, 128, 0, s>>>(g); break;
  }
  return cudaGetLastError();
}

// elementwise gelu(z) and gelu'(z) of the network's activation recipe for
// the units of network column `col`
__global__ void gelu_eval_kernel(const float* z, long long n, int col, float* g, float* dg) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (g) g[i] = gelu_col(z[i], col);
  if (dg) dg[i] = gelu_grad_col(z[i], col);
}

}  // namespace pcgb_mlp

using namespace pcgb_mlp;

extern "C" {

int pcgb_mlp_gelu(const float* z, int64_t n, int column, float* gelu_out, float* grad_out, void* stream) {
  if (n < 0 || (n > 0 && !z) || column < 0) return mlp_fail(PCGB_EINVAL, "bad gelu arguments");
  if (n == 0) return PCGB_OK;
  const long long blocks = (n + 255) / 256;
  if (blocks > 0x7fffffffLL) return mlp_fail(PCGB_ERANGE, "gelu: n too large");
  gelu_eval_kernel<<<unsigned(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(z, n, column, gelu_out,
                                                                                       grad_out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
  return PCGB_OK;
}

const char* pcgb_mlp_last_error(void) { return g_mlp_err.c_str(); }

int pcgb_gemm_bf16(int a_layout, int b_layout, int epilogue, const void* A, int64_t lda, const void* B, int64_t ldb,
                   int64_t M, int64_t N, int64_t K, int64_t k_split, const float* bias, int64_t bias_stride,
                   float* out_f32, int64_t ldo, void* out_bf16, int64_t ldob, const float* zin, int64_t ldz,
                   void* stream) {
  if (M < 0 || N < 0 || K < 0) return mlp_fail(PCGB_EINVAL, "negative GEMM size");
  if (K % 8 || lda % 8 || ldb % 8) return mlp_fail(PCGB_EINVAL, "K, lda and ldb must be multiples of 8");
  if (epilogue < 0 || epilogue > 4) return mlp_fail(PCGB_EINVAL, "unknown epilogue");
  // operands are read in 16-byte chunks
  if (reinterpret_cast<uintptr_t>(A) % 16 || reinterpret_cast<uintptr_t>(B) % 16)
    return mlp_fail(PCGB_EINVAL, "A and B must be 16-byte aligned");
  // every 16-byte operand chunk a tile reads must lie inside the stored rows
  const int64_t m8 = (M + 7) / 8 * 8, n8 = (N + 7) / 8 * 8;
  if ((a_layout == 0 && lda < K) || (a_layout != 0 && lda < m8) || (b_layout == 0 && ldb < K) ||
      (b_layout != 0 && ldb < n8))
    return mlp_fail(PCGB_EINVAL, "leading dimension smaller than the stored row");
  if (M == 0 || N == 0) return PCGB_OK;
  if (k_split <= 0 || k_split >= K) k_split = K;
  else if (k_split % BK) k_split = (k_split + BK - 1) / BK * BK;
  if (k_split > K) k_split = K;
  if (k_split != K && epilogue != EPI_DW_ATOMIC) return mlp_fail(PCGB_EINVAL, "split-K needs the atomic epilogue");
  GemmArgs g{static_cast<const bf16*>(A), lda, static_cast<const bf16*>(B), ldb, M, N, K, k_split,
             bias, bias_stride, out_f32, ldo, static_cast<bf16*>(out_bf16), ldob, zin, ldz};
  const long long splits = K == 0 ? 1 : (K + k_split - 1) / k_split;
  dim3 grid(unsigned((N + BN - 1) / BN), unsigned((M + BM - 1) / BM), unsigned(splits));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (a_layout == 0 && b_layout == 0) e = launch_gemm<true, true>(epilogue, g, grid, s);
  else if (a_layout == 0) e = launch_gemm<true, false>(epilogue, g, grid, s);
  else if (b_layout == 0) e = launch_gemm<false, true>(epilogue, g, grid, s);
  else e = launch_gemm<false, false>(epilogue, g, grid, s);
  if (e != cudaSuccess) return mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
  return PCGB_OK;
}

int pcgb_mlp_mse_grad(const float* y, const float* t, int64_t ldy, int64_t batch, int nout, int ncols, void* dy,
                      int64_t lddy, float* loss_sum, void* stream) {
  if (batch <= 0 || nout <= 0 || ncols < nout) return mlp_fail(PCGB_EINVAL, "bad mse_grad sizes");
  const long long n = batch * ncols;
  mse_grad_kernel<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      y, t, ldy, batch, nout, ncols, static_cast<bf16*>(dy), lddy, loss_sum);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PCGB_OK : mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
}

int pcgb_adam_step(float* master, float* m, float* v, float* grad, void* w_bf16, int64_t rows, int64_t ld,
                   int64_t rows_live, float lr, float b1, float b2, float eps, const float* corr, void* stream) {
  if (rows <= 0 || ld <= 0 || !corr) return mlp_fail(PCGB_EINVAL, "bad adam arguments");
  const long long n = rows * ld;
  adam_kernel<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      master, m, v, grad, static_cast<bf16*>(w_bf16), rows, ld, rows_live, lr, b1, b2, eps, corr);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PCGB_OK : mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
}

int pcgb_mlp_prepare(const float* signals, int64_t n, int nin, int log_in, void* x_rows, int64_t ldx, float* snorm,
                     const float* params, int nout, const int* kinds, const float* mean, const float* stdv,
                     float* targets, int64_t ldt, void* stream) {
  if (n < 0 || nin <= 0 || ldx < nin + 1) return mlp_fail(PCGB_EINVAL, "bad prepare sizes");
  if (n == 0) return PCGB_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  prepare_inputs_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(signals, n, nin, static_cast<bf16*>(x_rows), ldx,
                                                                   snorm, log_in);
  if (params && targets) {
    if (nout <= 0 || ldt < nout) return mlp_fail(PCGB_EINVAL, "bad target sizes");
    prepare_targets_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(params, snorm, n, nout, kinds, mean, stdv,
                                                                      targets, ldt);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PCGB_OK : mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
}

int pcgb_mlp_forward(const float* signals, int64_t n, int nin, int log_in, const void* const* w_bf16,
                     const float* const* w_master, int nout, const int* kinds, const float* mean, const float* stdv, const float* lb,
                     const float* ub, float* out, void* stream) {
  if (n < 0) return mlp_fail(PCGB_EINVAL, "n must be >= 0");
  if (nin != 16) return mlp_fail(PCGB_EINVAL, "the fused forward is built for 16 inputs");
  if (nout < 1 || nout > NOUT_PAD) return mlp_fail(PCGB_EINVAL, "nout must be 1..8");
  if (n == 0) return PCGB_OK;
  InferArgs a{};
  a.signals = signals;
  a.n = n;
  for (int l = 0; l < 4; ++l) {
    a.w[l] = static_cast<const bf16*>(w_bf16[l]);
    a.mw[l] = w_master[l];
  }
  a.nout = nout;
  a.log_in = log_in;
  for (int k = 0; k < NOUT_PAD; ++k) {
    a.kinds[k] = k < nout ? kinds[k] : 1;
    a.mean[k] = k < nout ? mean[k] : 0.f;
    a.stdv[k] = k < nout ? stdv[k] : 1.f;
    a.lb[k] = k < nout ? lb[k] : -3.0e38f;
    a.ub[k] = k < nout ? ub[k] : 3.0e38f;
  }
  a.out = out;
  const size_t smem = sizeof(InferSmem<16>);
  cudaError_t e = cudaFuncSetAttribute(mlp_infer_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (n + 15) / 16;
  long long blocks = (tiles + 11) / 12;
  if (blocks > sms) blocks = sms;
  mlp_infer_kernel<16><<<unsigned(blocks), 384, smem, static_cast<cudaStream_t>(stream)>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? PCGB_OK : mlp_fail(PCGB_ECUDA, cudaGetErrorString(e));
}

}  // extern "C"
