// Training GEMMs of the warm-start network on the 5th-generation tensor cores.
//
// C(M x N) = A(M x K) * B(K x N) with bf16 operands and an fp32 accumulator in
// tensor memory, with the epilogues of the training step fused (bias + GELU
// storing the pre-activation and the bf16 activation, bias only, GELU' times
// the incoming gradient, split-K accumulation of weight gradients with
// atomics, plain fp32 store). Same arguments, layouts and results (up to fp32
// summation order) as the warp-level mma.sync GEMM of mlp.cu:
//   a_layout 0: A stored (M, K) row-major (K-major), 1: (K, M) row-major
//   b_layout 0: B stored (N, K) row-major (K-major), 1: (K, N) row-major
//
// One CTA of 128 threads computes a 128 x 32 tile of C over its K range
// (blockIdx.z selects the split-K range); the narrow tile doubles the CTAs of
// the training step's small GEMMs and halves each thread's epilogue, which
// bounds their latency. Per 32-wide K step the threads stage both operand
// tiles into shared memory with 16-byte stores, a K-major operand in the
// canonical K-major core-matrix layout and a transposed one in the canonical
// MN-major layout (read with the MMA's transpose bit), and one thread issues two
// tcgen05.mma (M = 128, N = 32, K = 16) into the 32 accumulator columns and
// commits them to the stage's mbarrier; two stages alternate, and
// the global loads of step t + 1 are in flight while step t is staged and its
// MMAs issue. The epilogue reads row r of the accumulator (thread r = TMEM
// lane r) with tcgen05.ld and passes each warp's rows through shared memory,
// so its global stores, loads and atomics are row-contiguous. Every mbarrier
// wait is bounded: on timeout the CTA records the loss in *status, waits once
// more (bounded) for its MMAs in flight, skips its epilogue and still frees
// its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "mlp_math.cuh"
#include "pcgb.h"
#include "tc_common.cuh"

namespace pcgb_gemm_tc {

using pcgb_mlp::bf16;
using namespace pcgb_tc;

constexpr int BM = 128, BN = 32, BK = 32;
constexpr int THREADS = 128;
constexpr int TMEM_COLS = 32;  // BN fp32 accumulator columns (the minimum allocation)
constexpr unsigned kWaitLimit = 1u << 22;
// dynamic shared memory requested per CTA: at most 7 CTAs fit on an SM, so
// their 7 x 32 accumulator columns never exceed the SM's 512 and no
// tcgen05.alloc has to wait for another CTA
constexpr int kSmemBytes = 32 * 1024;

enum Epilogue { EPI_FWD_GELU = 0, EPI_FWD_LINEAR = 1, EPI_BWD_DGELU = 2, EPI_DW_ATOMIC = 3, EPI_STORE_F32 = 4 };

struct TcGemmArgs {
  const bf16* A;
  long long lda;
  const bf16* B;
  long long ldb;
  long long M, N, K;
  long long k_split;
  const float* bias;
  long long bias_stride;
  float* out_f32;
  long long ldo;
  bf16* out_bf16;
  long long ldob;
  const float* zin;
  long long ldz;
  int* status;
  unsigned wait_limit;   // try_wait rounds before a wait counts as lost
  long long skip_block;  // failure-path test: this CTA never issues its first K step (-1 = none)
};

struct __align__(1024) GemmSmem {
  bf16 a[2][BM * BK];
  bf16 b[2][BN * BK];
  unsigned long long mbar[2];
  uint32_t tmem_base;
};
static_assert(sizeof(GemmSmem) <= kSmemBytes && kSmemBytes <= 48 * 1024, "GEMM shared memory");

// One operand's rows x BK tile at (r0, k0), held in registers between its
// global loads and its shared-memory stores, so the loads of step t + 1 are
// in flight while step t is staged and its MMAs issue. KMAJOR: element (r, k)
// at src[r * ld + k], staged in the canonical K-major layout (core_off);
// else element (r, k) at src[k * ld + r], staged as it is stored, in the
// canonical MN-major layout: 16-byte rows of 8 consecutive r at one k, the
// 8 k of a core matrix 16 bytes apart, core matrices kMnSbo = 128 bytes
// apart along r and kMnLbo apart along k (the MMA reads it with the
// operand's transpose bit set). Rows >= rows_live are loaded when the stored
// row is long enough (their results are masked); k at or past kend is zero.
template <int ROWS, bool KMAJOR>
struct OperandTile {
  static constexpr int kItems = ROWS * (BK / 8);  // 16-byte chunks
  static constexpr int kPer = (kItems + THREADS - 1) / THREADS;
  static_assert(kItems % THREADS == 0 || kPer == 1, "operand tile items per thread");
  static constexpr uint32_t kMnSbo = 128;
  static constexpr uint32_t kMnLbo = uint32_t(ROWS / 8) * 128;
  // threads past the last item (kItems < THREADS) load and store nothing
  static __device__ __forceinline__ bool mine(int c) { return kItems % THREADS == 0 || c < kItems; }
  uint4 v[kPer];

  // chunk c -> (row of its first element, k): KMAJOR 8 k-values of row r;
  // else 8 rows at one k, with k % 8 varying fastest across a warp so that
  // consecutive threads fill consecutive 16-byte slots of a core matrix
  static __device__ __forceinline__ void chunk(int c, int& r, int& k) {
    if (KMAJOR) {
      r = c / (BK / 8);
      k = (c % (BK / 8)) * 8;
    } else {
      r = ((c / 8) % (ROWS / 8)) * 8;
      k = (c / (8 * (ROWS / 8))) * 8 + c % 8;
    }
  }

  __device__ __forceinline__ void load(const bf16* src, long long ld, long long r0, long long rows_live,
                                       long long k0, long long kend) {
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = threadIdx.x + i * THREADS;
      if (!mine(c)) break;
      int r, k;
      chunk(c, r, k);
      v[i] = make_uint4(0, 0, 0, 0);
      if (r0 + r < rows_live && k0 + k < kend)
        v[i] = *reinterpret_cast<const uint4*>(KMAJOR ? src + (r0 + r) * ld + k0 + k : src + (k0 + k) * ld + r0 + r);
    }
  }

  __device__ __forceinline__ void store(bf16* dst) const {
    unsigned char* base = reinterpret_cast<unsigned char*>(dst);
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = threadIdx.x + i * THREADS;
      if (!mine(c)) break;
      int r, k;
      chunk(c, r, k);
      const uint32_t off = KMAJOR ? core_off(r, k, BK) : uint32_t(r / 8) * kMnSbo + uint32_t(k / 8) * kMnLbo + (k % 8) * 16;
      *reinterpret_cast<uint4*>(base + off) = v[i];
    }
  }

  // descriptor of the K = 16 slice kk of the staged tile
  static __device__ __forceinline__ uint64_t desc(uint32_t tile, int kk) {
    return KMAJOR ? smem_desc(tile + kk * 256, 128, (BK / 8) * 128)
                  : smem_desc(tile + uint32_t(2 * kk) * kMnLbo, kMnLbo, kMnSbo);
  }
};

// Epilogue staging, one region per warp, laid over the operand buffers once
// every MMA has completed: a warp's 32 accumulator rows (one per thread) are
// written row-wise and read back column-wise, so the global stores, loads and
// atomics of a 16-column chunk touch two 64-byte row segments per
// instruction instead of 32 rows.
constexpr int kEpiPitch = 17;  // floats per staged row: odd, so the row-per-thread writes hit distinct banks
struct EpiStage {
  // fp32 outputs, or (GELU' epilogue, which stores no fp32) the
  // pre-activations it reads
  float f[THREADS / 32][32 * kEpiPitch];
  uint32_t h[THREADS / 32][32 * 9];         // bf16 outputs, as pairs (8 words per row + 1 pad)
};
static_assert(sizeof(EpiStage) <= sizeof(bf16) * 2 * (BM + BN) * BK, "epilogue staging fits the operand buffers");

template <bool A_ROW, bool B_NK, int EPI>
__global__ void __launch_bounds__(THREADS) gemm_tc_kernel(const TcGemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  GemmSmem& S = *reinterpret_cast<GemmSmem*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long m0 = (long long)blockIdx.y * BM, n0 = (long long)blockIdx.x * BN;
  const long long kbeg = (long long)blockIdx.z * g.k_split;
  const long long kend = kbeg + g.k_split < g.K ? kbeg + g.k_split : g.K;
  const int steps = int((kend - kbeg + BK - 1) / BK);

  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar[i])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  OperandTile<BM, A_ROW> ta;
  OperandTile<BN, B_NK> tb;
  if (steps > 0) {
    ta.load(g.A, g.lda, m0, g.M, kbeg, kend);
    tb.load(g.B, g.ldb, n0, g.N, kbeg, kend);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = S.tmem_base;
  // transpose bits of kind::f16: A (bit 15) and B (bit 16) MN-major
  constexpr uint32_t ID = idesc_bf16(BM, BN) | (A_ROW ? 0u : 1u << 15) | (B_NK ? 0u : 1u << 16);
  bool lost = false;
  int last_issued = -1;  // thread 0: the last K step whose MMAs it committed

  for (int t = 0; t < steps; ++t) {
    const int buf = t & 1;
    // the MMAs of step t - 2 read this buffer: wait for their commit
    if (t >= 2) {
      const bool ok = threadIdx.x != 0 || mbar_wait(smem_u32(&S.mbar[buf]), uint32_t(((t - 2) >> 1) & 1), g.wait_limit);
      if (__syncthreads_or(!ok)) {
        lost = true;
        break;
      }
    }
    ta.store(S.a[buf]);
    tb.store(S.b[buf]);
    if (t + 1 < steps) {
      const long long k1 = kbeg + (long long)(t + 1) * BK;
      ta.load(g.A, g.lda, m0, g.M, k1, kend);
      tb.load(g.B, g.ldb, n0, g.N, k1, kend);
    }
    fence_async_smem();  // staged operands -> visible to the tensor cores
    fence_before_sync();
    __syncthreads();
    // failure-path test: the CTA never issues nor commits its MMAs, so its
    // first wait on an mbarrier phase runs out while none of its tensor-core
    // work is in flight
    const bool skip = g.skip_block >= 0 && (long long)blockIdx.x +
                                                   (long long)gridDim.x *
                                                       (blockIdx.y + (long long)gridDim.y * blockIdx.z) ==
                                               g.skip_block;
    if (threadIdx.x == 0 && !skip) {
      fence_after_sync();
      const uint32_t as = smem_u32(S.a[buf]), bs = smem_u32(S.b[buf]);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)
        mma_bf16(tbase, OperandTile<BM, A_ROW>::desc(as, kk), OperandTile<BN, B_NK>::desc(bs, kk), ID,
                 (t > 0 || kk > 0) ? 1u : 0u);
      mma_commit(smem_u32(&S.mbar[buf]));
      last_issued = t;
    }
  }
  // the last commit covers every MMA of this CTA
  if (!lost && steps > 0) {
    const int last = steps - 1;
    const bool ok = threadIdx.x != 0 ||
                    mbar_wait(smem_u32(&S.mbar[last & 1]), uint32_t((last >> 1) & 1), g.wait_limit);
    lost = __syncthreads_or(!ok);
  }
  if (lost) {
    if (threadIdx.x == 0) {
      // MMAs of the lost phase may still complete: wait (bounded) for the
      // commit of the last step whose MMAs were issued (MMAs complete in
      // issue order) before the tensor memory they write is returned
      if (last_issued >= 0)
        (void)mbar_wait(smem_u32(&S.mbar[last_issued & 1]), uint32_t((last_issued >> 1) & 1), g.wait_limit);
      if (g.status) atomicExch(g.status, 1);
    }
  } else {
    fence_after_sync();
    // every MMA has completed (or none ran): the operand buffers are free
    EpiStage& E = *reinterpret_cast<EpiStage*>(smem_raw);
    float* sf = E.f[warp];
    float* sz = E.f[warp];
    uint32_t* sh = E.h[warp];
    const long long mw = m0 + warp * 32;  // first row of this warp = its TMEM lane quarter
    const uint32_t trow = tbase + (uint32_t(warp * 32) << 16);
    constexpr bool kF32 = EPI != EPI_BWD_DGELU;
    constexpr bool kBf16 = EPI == EPI_FWD_GELU || EPI == EPI_BWD_DGELU;
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 16) {
      const long long nc = n0 + c0;
      if (nc >= g.N) break;  // uniform over the CTA
      float v[16];
      if (steps > 0) {
        tmem_ld16(trow + uint32_t(c0), v);
      } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = 0.f;
      }
      if (EPI == EPI_BWD_DGELU) {
        // the chunk's pre-activations, read row segment by row segment
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int idx = j * 32 + lane, rr = idx >> 4, cc = idx & 15;
          const long long m = mw + rr, n = nc + cc;
          sz[rr * kEpiPitch + cc] = (m < g.M && n < g.N) ? g.zin[m * g.ldz + n] : 0.f;
        }
        __syncwarp();
      }
      // column nc + i has i = its position modulo 16 (nc is a multiple of 16),
      // so each pair's GELU recipe is fixed at compile time
#pragma unroll
      for (int i = 0; i < 16; i += 2) {
        float o0 = v[i], o1 = v[i + 1];
        uint32_t hb = 0;
        if (EPI == EPI_FWD_GELU || EPI == EPI_FWD_LINEAR) {
          o0 += nc + i < g.N ? g.bias[(nc + i) * g.bias_stride] : 0.f;
          o1 += nc + i + 1 < g.N ? g.bias[(nc + i + 1) * g.bias_stride] : 0.f;
        }
        if (EPI == EPI_FWD_GELU) {
          // gelu = (2 gelu) / 2, exact in bf16
          const float2 t = __bfloat1622float2(pcgb_mlp::bits_bf162(pcgb_mlp::gelu2x_col_pack_bf16(o0, o1, i)));
          hb = pcgb_mlp::pack_bf16(0.5f * t.x, 0.5f * t.y);
        } else if (EPI == EPI_BWD_DGELU) {
          hb = pcgb_mlp::pack_bf16(o0 * pcgb_mlp::gelu_grad_col(sz[lane * kEpiPitch + i], i),
                                   o1 * pcgb_mlp::gelu_grad_col(sz[lane * kEpiPitch + i + 1], i + 1));
        }
        if (kF32) {
          sf[lane * kEpiPitch + i] = o0;
          sf[lane * kEpiPitch + i + 1] = o1;
        }
        if (kBf16) sh[lane * 9 + i / 2] = hb;
      }
      __syncwarp();
      if (kF32) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int idx = j * 32 + lane, rr = idx >> 4, cc = idx & 15;
          const long long m = mw + rr, n = nc + cc;
          if (m < g.M && n < g.N) {
            const float val = sf[rr * kEpiPitch + cc];
            if (EPI == EPI_DW_ATOMIC) atomicAdd(&g.out_f32[m * g.ldo + n], val);
            else g.out_f32[m * g.ldo + n] = val;
          }
        }
      }
      if (kBf16) {
        // 32 rows x 8 words; ldob is even, so a pair at an even column is one
        // aligned 32-bit word
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int idx = j * 32 + lane, rr = idx >> 3, w = idx & 7;
          const long long m = mw + rr, n = nc + 2 * w;
          if (m < g.M && n < g.N) {
            const uint32_t pair = sh[rr * 9 + w];
            if (n + 1 < g.N) {
              *reinterpret_cast<uint32_t*>(g.out_bf16 + m * g.ldob + n) = pair;
            } else {
              g.out_bf16[m * g.ldob + n] = __ushort_as_bfloat16(uint16_t(pair & 0xffffu));
            }
          }
        }
      }
      __syncwarp();  // the next chunk reuses the staging
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(TMEM_COLS) : "memory");
  }
}

template <bool A_ROW, bool B_NK>
cudaError_t launch_tc(int epi, const TcGemmArgs& g, dim3 grid, cudaStream_t s) {
  // kSmemBytes is below the 48 KB a launch may request without opting in, so
  // no function attribute is set (the training step is captured in a graph)
  auto pick = [&](auto kern) {
    kern<<<grid, THREADS, kSmemBytes, s>>>(g);
    return cudaGetLastError();
  };
  switch (epi) {
    case EPI_FWD_GELU: return pick(gemm_tc_kernel<A_ROW, B_NK, EPI_FWD_GELU>);
    case EPI_FWD_LINEAR: return pick(gemm_tc_kernel<A_ROW, B_NK, EPI_FWD_LINEAR>);
    case EPI_BWD_DGELU: return pick(gemm_tc_kernel<A_ROW, B_NK, EPI_BWD_DGELU>);
    case EPI_DW_ATOMIC: return pick(gemm_tc_kernel<A_ROW, B_NK, EPI_DW_ATOMIC>);
    default: return pick(gemm_tc_kernel<A_ROW, B_NK, EPI_STORE_F32>);
  }
}

thread_local std::string g_err;

int fail(int code, const char* msg) {
  g_err = msg;
  return code;
}

}  // namespace pcgb_gemm_tc

using namespace pcgb_gemm_tc;

extern "C" {

const char* pcgb_gemm_tc_last_error(void) { return g_err.c_str(); }

int pcgb_gemm_bf16_tc(int a_layout, int b_layout, int epilogue, const void* A, int64_t lda, const void* B,
                      int64_t ldb, int64_t M, int64_t N, int64_t K, int64_t k_split, const float* bias,
                      int64_t bias_stride, float* out_f32, int64_t ldo, void* out_bf16, int64_t ldob,
                      const float* zin, int64_t ldz, int* status, void* stream) {
  return pcgb_gemm_bf16_tc_ex(a_layout, b_layout, epilogue, A, lda, B, ldb, M, N, K, k_split, bias, bias_stride,
                              out_f32, ldo, out_bf16, ldob, zin, ldz, status, 0u, -1, stream);
}

int pcgb_gemm_bf16_tc_ex(int a_layout, int b_layout, int epilogue, const void* A, int64_t lda, const void* B,
                         int64_t ldb, int64_t M, int64_t N, int64_t K, int64_t k_split, const float* bias,
                         int64_t bias_stride, float* out_f32, int64_t ldo, void* out_bf16, int64_t ldob,
                         const float* zin, int64_t ldz, int* status, unsigned wait_limit, int64_t skip_block,
                         void* stream) {
  g_err.clear();
  if (M < 0 || N < 0 || K < 0) return fail(PCGB_EINVAL, "negative GEMM size");
  if (K % 8 || lda % 8 || ldb % 8) return fail(PCGB_EINVAL, "K, lda and ldb must be multiples of 8");
  if (epilogue < 0 || epilogue > 4) return fail(PCGB_EINVAL, "unknown epilogue");
  if (!A || !B) return fail(PCGB_EINVAL, "A and B are required");
  // operands are read in 16-byte chunks
  if (reinterpret_cast<uintptr_t>(A) % 16 || reinterpret_cast<uintptr_t>(B) % 16)
    return fail(PCGB_EINVAL, "A and B must be 16-byte aligned");
  // every 16-byte operand chunk a tile reads must lie inside the stored rows:
  // a transposed operand is read in chunks of 8 rows up to the tile's row
  // count rounded to 8
  const int64_t m8 = (M + 7) / 8 * 8, n8 = (N + 7) / 8 * 8;
  if ((a_layout == 0 && lda < K) || (a_layout != 0 && lda < m8) || (b_layout == 0 && ldb < K) ||
      (b_layout != 0 && ldb < n8))
    return fail(PCGB_EINVAL, "leading dimension smaller than the stored row");
  const bool need_bias = epilogue == EPI_FWD_GELU || epilogue == EPI_FWD_LINEAR;
  if (!out_f32 && epilogue != EPI_BWD_DGELU) return fail(PCGB_EINVAL, "out_f32 is required");
  if ((epilogue == EPI_FWD_GELU || epilogue == EPI_BWD_DGELU) && !out_bf16)
    return fail(PCGB_EINVAL, "out_bf16 is required");
  if ((epilogue == EPI_FWD_GELU || epilogue == EPI_BWD_DGELU) &&
      (ldob % 2 || reinterpret_cast<uintptr_t>(out_bf16) % 4))
    return fail(PCGB_EINVAL, "out_bf16 must be 4-byte aligned with an even ldob");
  if (need_bias && !bias) return fail(PCGB_EINVAL, "bias is required");
  if (epilogue == EPI_BWD_DGELU && !zin) return fail(PCGB_EINVAL, "zin is required");
  if (M == 0 || N == 0) return PCGB_OK;
  if (k_split <= 0 || k_split >= K) k_split = K;
  else if (k_split % BK) k_split = (k_split + BK - 1) / BK * BK;
  if (k_split > K) k_split = K;
  if (k_split != K && epilogue != EPI_DW_ATOMIC) return fail(PCGB_EINVAL, "split-K needs the atomic epilogue");
  const long long splits = K == 0 ? 1 : (K + k_split - 1) / k_split;
  if ((N + BN - 1) / BN > 0x7fffffffLL || (M + BM - 1) / BM > 65535 || splits > 65535)
    return fail(PCGB_ERANGE, "GEMM grid too large");
  TcGemmArgs g{static_cast<const bf16*>(A), lda, static_cast<const bf16*>(B), ldb, M, N, K, k_split,
               bias, bias_stride, out_f32, ldo, static_cast<bf16*>(out_bf16), ldob, zin, ldz, status,
               wait_limit ? wait_limit : kWaitLimit, skip_block};
  dim3 grid(unsigned((N + BN - 1) / BN), unsigned((M + BM - 1) / BM), unsigned(splits));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (a_layout == 0 && b_layout == 0) e = launch_tc<true, true>(epilogue, g, grid, s);
  else if (a_layout == 0) e = launch_tc<true, false>(epilogue, g, grid, s);
  else if (b_layout == 0) e = launch_tc<false, true>(epilogue, g, grid, s);
  else e = launch_tc<false, false>(epilogue, g, grid, s);
  if (e != cudaSuccess) return fail(PCGB_ECUDA, cudaGetErrorString(e));
  return PCGB_OK;
}

}  // extern "C"
