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
// Evaluated for two pre-activations at once in bf16x2 arithmetic, the format
// the next layer consumes: z rounded to bf16, u = z (c + c' z^2) with
// c = bf16(sqrt(2/pi)), c' = bf16(0.044715 sqrt(2/pi)) (each product and the
// fused multiply-add rounded to bf16; an overflow to +-Inf saturates t to
// +-1), t = tanh.approx.bf16x2(u) (one MUFU operation per element), and
// 2 gelu(z) = z t + z by one fused bf16x2 multiply-add. Seven instructions per
// pair of activations; the roundings are those of the bf16 operands the
// tensor cores read anyway. Every kernel (training epilogues and both
// inference kernels) uses these functions, so training and inference see the
// same activation.
__device__ __forceinline__ uint32_t bf162_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t*>(&v); }
__device__ __forceinline__ __nv_bfloat162 bits_bf162(uint32_t v) { return *reinterpret_cast<__nv_bfloat162*>(&v); }
__device__ __forceinline__ __nv_bfloat162 tanh_bf16x2(__nv_bfloat162 z) {
  const __nv_bfloat162 c = __float2bfloat162_rn(0.7978845608028654f);
  const __nv_bfloat162 c3 = __float2bfloat162_rn(0.0356774081363001f);
  const __nv_bfloat162 u = __hmul2(z, __hfma2(__hmul2(z, z), c3, c));
  uint32_t t;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(bf162_bits(u)));
  return bits_bf162(t);
}
// bf16 pair of 2 gelu(z0), 2 gelu(z1), for a next layer whose weights are
// stored halved (the products are those of gelu with the full weights)
__device__ __forceinline__ uint32_t gelu2x_pack_bf16(float z0, float z1) {
  const __nv_bfloat162 z = __floats2bfloat162_rn(z0, z1);
  return bf162_bits(__hfma2(z, tanh_bf16x2(z), z));
}
// gelu(z) of the same recipe: half of 2 gelu(z), exact in bf16
__device__ __forceinline__ float gelu(float z) {
  return 0.5f * __low2float(bits_bf162(gelu2x_pack_bf16(z, z)));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float z2 = z * z;
  const float t = __low2float(tanh_bf16x2(__float2bfloat162_rn(z)));
  return fmaf(0.5f, t, 0.5f) + 0.5f * z * (1.0f - t * t) * fmaf(0.1070322244089003f, z2, 0.7978845608028654f);
}
// GELU on the FMA pipe for a share of the columns. The tanh of the recipe
// above takes the MUFU pipe (two MUFU operations per pair of activations,
// 16 per SM per clock); the network's columns n with n % 16 < kPolyCols
// instead evaluate the same GELU with no MUFU operation, by a polynomial in
// bf16x2 arithmetic:
//   2 gelu(z) ~ 2 relu(z) + (w e(w) - a),  a = min(|z|, 3),  w = a^2,
//   e(w) = q1 + w (q2 + w (q3 + w q4)),  w e(w) ~ |z| tanh(u(|z|)) on [0, 3],
// which is z exactly where |z| <= 3 apart from w e(w) - |z| ~ z tanh(u) - |z|,
// and 2 relu(z) - 0.011 beyond. Every operation is one bf16 rounding (fused
// multiply-adds for the Horner steps and for w e - a, the non-contracting
// forms for the product and the final sum, so the compiler cannot fuse them
// differently); the small term w e - a is formed before it is added to
// 2 relu(z), so large z see one rounding. Nine instructions per pair, the
// result already the bf16 pair the next layer reads. q1..q4 are a
// near-minimax fit of |z| tanh(u(|z|)) / w in w on [0, 9], weighted by |z|
// (Lawson's iteratively reweighted least squares, C. L. Lawson 1961), rounded
// to bf16 and adjusted by single bf16 ulps to minimise the maximum error of
// the whole recipe over every bf16 input: at most 0.0110 |z| on bf16 z and
// 0.0176 |z| on fp32 z, which adds z's rounding (the MUFU recipe: 0.0103 and
// 0.0177 |z|). The columns are fixed, so training and inference see the same
// activation per unit.
constexpr int kPolyCols = 6;
__device__ __forceinline__ bool poly_col(int n) { return (n & 15) < kPolyCols; }
__device__ __forceinline__ uint32_t gelu2x_poly_pack_bf16(float z0, float z1) {
  const __nv_bfloat162 q1 = bits_bf162(0x3f4a3f4au), q2 = bits_bf162(0xbdedbdedu), q3 = bits_bf162(0x3c373c37u),
                       q4 = bits_bf162(0xb9e7b9e7u);
  const __nv_bfloat162 three = bits_bf162(0x40404040u), two = bits_bf162(0x40004000u), zero = bits_bf162(0u);
  const __nv_bfloat162 z = __floats2bfloat162_rn(z0, z1);
  const __nv_bfloat162 a = __hmin2(__habs2(z), three);
  const __nv_bfloat162 w = __hmul2_rn(a, a);
  __nv_bfloat162 e = __hfma2(q4, w, q3);
  e = __hfma2(e, w, q2);
  e = __hfma2(e, w, q1);
  const __nv_bfloat162 t = __hfma2(e, w, __hneg2(a));
  return bf162_bits(__hadd2_rn(__hfma2_relu(z, two, zero), t));
}
// d gelu / dz of the polynomial recipe (fp32, exact derivative of the
// continuous form)
__device__ __forceinline__ float gelu_poly_grad(float z) {
  const float q1 = 0.7890625f, q2 = -0.11572265625f, q3 = 0.01116943359375f, q4 = -0.0004405975341796875f;
  const float az = fabsf(z);
  if (az >= 3.0f) return z > 0.f ? 1.0f : 0.0f;  // 1/2 (1 + 1) or 1/2 (1 - 1)
  const float w = z * z;
  const float de = fmaf(fmaf(fmaf(4.f * q4, w, 3.f * q3), w, 2.f * q2), w, q1);  // E'(w)
  return 0.5f * fmaf(2.f * z, de, 1.0f);
}
// column-aware activation: n = column of z0 (z1 is column n + 1, same choice
// for even n)
__device__ __forceinline__ uint32_t gelu2x_col_pack_bf16(float z0, float z1, int n) {
  return poly_col(n) ? gelu2x_poly_pack_bf16(z0, z1) : gelu2x_pack_bf16(z0, z1);
}
__device__ __forceinline__ float gelu_col(float z, int n) {
  return 0.5f * __low2float(bits_bf162(gelu2x_col_pack_bf16(z, z, n)));
}
__device__ __forceinline__ float gelu_grad_col(float z, int n) {
  return poly_col(n) ? gelu_poly_grad(z) : gelu_grad(z);
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
// The input is rounded to bf16 right after, so the fast logarithm (__logf,
// absolute error ~2^-21 here) loses nothing the rounding keeps.
__device__ __forceinline__ float input_transform(float s, float inv, int log_in) {
  const float x = s * inv;
  return log_in ? __logf(fmaxf(x, 1e-6f)) : x;
}

}  // namespace pcgb_mlp
