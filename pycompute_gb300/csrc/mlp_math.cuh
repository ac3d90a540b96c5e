// Elementwise math of the warm-start network, shared by its kernels: bf16
// packing, GELU (tanh form) and its derivative, and the input transform.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace pcgb_mlp {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
// GELU in its tanh form (Hendrycks & Gimpel 2016),
//   gelu(x) = x/2 (1 + tanh(u)),  u = sqrt(2/pi) (x + 0.044715 x^3),
// with tanh from the hardware tanh.approx.f32 instruction (one MUFU op; the
// exact erf form costs ~20 instructions and dominated inference), and its
// derivative 1/2 (1 + t) + x/2 (1 - t^2) sqrt(2/pi) (1 + 3 * 0.044715 x^2).
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// u = z (c + c 0.044715 z^2) with c = sqrt(2/pi); gelu = h + h t with h = z / 2
__device__ __forceinline__ float gelu(float z) {
  const float t = tanh_approx(z * fmaf(0.0356774081363001f, z * z, 0.7978845608028654f));
  const float h = 0.5f * z;
  return fmaf(h, t, h);
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float z2 = z * z;
  const float t = tanh_approx(z * fmaf(0.0356774081363001f, z2, 0.7978845608028654f));
  return fmaf(0.5f, t, 0.5f) + 0.5f * z * (1.0f - t * t) * fmaf(0.1070322244089003f, z2, 0.7978845608028654f);
}

// Network input of one sample: s / max, or log(max(s / max, 1e-6)) with log_in.
__device__ __forceinline__ float input_transform(float s, float inv, int log_in) {
  const float x = s * inv;
  return log_in ? logf(fmaxf(x, 1e-6f)) : x;
}

}  // namespace pcgb_mlp
