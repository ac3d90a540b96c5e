// Elementwise math of the warm-start network, shared by its kernels: bf16
// packing, GELU (tanh form) and its derivative, and the input transform.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

namespace pcgb_mlp {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
// GELU in its tanh form (Hendrycks & Gimpel 2016),
//   gelu(z) = z/2 (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
// and its derivative 1/2 (1 + t) + z/2 (1 - t^2) sqrt(2/pi) (1 + 3 * 0.044715 z^2).
// t = tanh(u) is evaluated for two pre-activations at once: u = z (c + c' z^2)
// in f16x2 arithmetic (c = sqrt(2/pi), c' = 0.044715 c; an overflow to +-Inf
// saturates t to +-1 as it should) and tanh by one tanh.approx.f16x2 MUFU
// operation. Its error (~2^-10 relative, like tanh.approx.f32) is below the
// bf16 rounding of the activation; the rest of the GELU stays in fp32. Every
// kernel (training epilogues and both inference kernels) uses this one
// function, so training and inference see the same activation.
__device__ __forceinline__ float2 gelu_tanh2(float z0, float z1) {
  const __half2 z = __floats2half2_rn(z0, z1);
  const __half2 q = __hfma2(__hmul2(z, z), __float2half2_rn(0.0356774081363001f), __float2half2_rn(0.7978845608028654f));
  const __half2 u = __hmul2(z, q);
  uint32_t ti;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(ti) : "r"(*reinterpret_cast<const uint32_t*>(&u)));
  return __half22float2(*reinterpret_cast<const __half2*>(&ti));
}
__device__ __forceinline__ float gelu(float z) {
  const float t = gelu_tanh2(z, z).x;
  const float h = 0.5f * z;
  return fmaf(h, t, h);
}
// bf16 pair of 2 gelu(z): exactly twice the bf16 rounding of gelu(z), for a
// next layer whose weights are stored halved (the products are unchanged)
__device__ __forceinline__ uint32_t gelu2x_pack_bf16(float z0, float z1) {
  const float2 t = gelu_tanh2(z0, z1);
  return pack_bf16(fmaf(z0, t.x, z0), fmaf(z1, t.y, z1));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float z2 = z * z;
  const float t = gelu_tanh2(z, z).x;
  return fmaf(0.5f, t, 0.5f) + 0.5f * z * (1.0f - t * t) * fmaf(0.1070322244089003f, z2, 0.7978845608028654f);
}
// eight bf16 values times 1/2 (exact for normal numbers)
__device__ __forceinline__ uint4 halve_bf16x8(uint4 v) {
  uint32_t* w = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[i]));
    w[i] = pack_bf16(0.5f * f.x, 0.5f * f.y);
  }
  return v;
}

// Network input of one sample: s / max, or log(max(s / max, 1e-6)) with log_in.
__device__ __forceinline__ float input_transform(float s, float inv, int log_in) {
  const float x = s * inv;
  return log_in ? logf(fmaxf(x, 1e-6f)) : x;
}

}  // namespace pcgb_mlp
