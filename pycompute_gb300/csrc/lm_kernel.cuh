// Device code of the batched second-order Levenberg-Marquardt fitter for
// sm_103a. The host library compiles it at run time together with one
// generated model struct (m, dm/dp, d2m/dp2 as straight-line code) and the
// launch parameters of lm_params.h.
//
// One thread owns one voxel for the whole fit: parameters, damping, the
// packed normal matrix, the solve and the bounds live in registers; P,
// H = P(P+1)/2 and the sample count M are compile-time constants. The loops
// over parameters unroll; the two loops over samples unroll only where
// instruction issue bounds the iteration (fp32 solve) and stay rolled where
// the FP64 pipe does (there the samples sit in L1-resident local memory; see
// sample_unroll). A voxel runs all of its iterations inside one launch and
// leaves as soon as it converges (the reference relaunches the kernel `iters`
// times and re-reads its state from global memory each time,
// pycompute/cuda/lsqnonlin.py:1058-1068).
//
// Numerics follow the reference kernel (pycompute/cuda/lsqnonlin.py:823-924)
// step for step, with two type parameters:
//   TA  state, residuals, sums over samples, convergence test
//   TS  GMW81 LDL^T factorisation and solve, gain-ratio test
// <float, double> is the FP32-bulk / FP64-solve fitter, <float, float> the
// reference's fp32 arithmetic, <double, double> the all-FP64 oracle run.
#pragma once

#define PCGB_HD __device__ __forceinline__

PCGB_HD float pcgb_exp(float x) { return expf(x); }
PCGB_HD double pcgb_exp(double x) { return exp(x); }
PCGB_HD float pcgb_log(float x) { return logf(x); }
PCGB_HD double pcgb_log(double x) { return log(x); }
PCGB_HD float pcgb_sin(float x) { return sinf(x); }
PCGB_HD double pcgb_sin(double x) { return sin(x); }
PCGB_HD float pcgb_cos(float x) { return cosf(x); }
PCGB_HD double pcgb_cos(double x) { return cos(x); }
PCGB_HD float pcgb_tan(float x) { return tanf(x); }
PCGB_HD double pcgb_tan(double x) { return tan(x); }
PCGB_HD float pcgb_asin(float x) { return asinf(x); }
PCGB_HD double pcgb_asin(double x) { return asin(x); }
PCGB_HD float pcgb_acos(float x) { return acosf(x); }
PCGB_HD double pcgb_acos(double x) { return acos(x); }
PCGB_HD float pcgb_atan(float x) { return atanf(x); }
PCGB_HD double pcgb_atan(double x) { return atan(x); }
PCGB_HD float pcgb_sinh(float x) { return sinhf(x); }
PCGB_HD double pcgb_sinh(double x) { return sinh(x); }
PCGB_HD float pcgb_cosh(float x) { return coshf(x); }
PCGB_HD double pcgb_cosh(double x) { return cosh(x); }
PCGB_HD float pcgb_tanh(float x) { return tanhf(x); }
PCGB_HD double pcgb_tanh(double x) { return tanh(x); }
PCGB_HD float pcgb_abs(float x) { return fabsf(x); }
PCGB_HD double pcgb_abs(double x) { return fabs(x); }
PCGB_HD float pcgb_erf(float x) { return erff(x); }
PCGB_HD double pcgb_erf(double x) { return erf(x); }
PCGB_HD float pcgb_sqrt(float x) { return sqrtf(x); }
PCGB_HD double pcgb_sqrt(double x) { return sqrt(x); }
PCGB_HD float pcgb_pow(float x, float y) { return powf(x, y); }
PCGB_HD double pcgb_pow(double x, double y) { return pow(x, y); }

namespace pcgb {

template <typename T> struct Num;
// sqrt(P^2 - 1), correctly rounded in each precision, for P = 2..8: the GMW81
// scale of the largest off-diagonal entry (solver.py:32-57) as a literal, so
// no square root or division of a constant runs per solve
PCGB_HD constexpr float sqrt_pm1_f(int P) {
  return P == 2 ? 1.7320507764816284f : P == 3 ? 2.8284270763397217f : P == 4 ? 3.872983455657959f
       : P == 5 ? 4.898979663848877f : P == 6 ? 5.916079998016357f : P == 7 ? 6.928203105926514f
       : 7.937253952026367f;
}
PCGB_HD constexpr double sqrt_pm1_d(int P) {
  return P == 2 ? 1.7320508075688772 : P == 3 ? 2.8284271247461903 : P == 4 ? 3.872983346207417
       : P == 5 ? 4.898979485566356 : P == 6 ? 5.916079783099616 : P == 7 ? 6.928203230275509
       : 7.937253933193772;
}
// 1 / sqrt(P^2 - 1) rounded to double
PCGB_HD constexpr double inv_sqrt_pm1_d(int P) {
  return P == 2 ? 0.5773502691896258 : P == 3 ? 0.35355339059327373 : P == 4 ? 0.2581988897471611
       : P == 5 ? 0.20412414523193154 : P == 6 ? 0.1690308509457033 : P == 7 ? 0.14433756729740646
       : 0.1259881576697424;
}

template <> struct Num<float> {
  static PCGB_HD float gmw_eps() { return 2e-7f; }    // solver.py:105
  static PCGB_HD constexpr float sqrt_pm1(int P) { return sqrt_pm1_f(P); }
  static PCGB_HD float damp_floor() { return 1e-4f; } // lsqnonlin.py:275
  static PCGB_HD float prot(const PcgbLmParams& a, int i) { return a.protocol_f[i]; }
  static PCGB_HD float slb(const PcgbLmParams& a, int k) { return a.shared_lb_f[k]; }
  static PCGB_HD float sub(const PcgbLmParams& a, int k) { return a.shared_ub_f[k]; }
  static PCGB_HD float inf() { return __int_as_float(0x7f800000); }
  static PCGB_HD float nan() { return __int_as_float(0x7fffffff); }
  // tol, mu, eta, acc, dec (k = 0..4)
  static PCGB_HD float lmc(const PcgbLmParams& a, int k) {
    return k == 0 ? a.tol_f : k == 1 ? a.mu_f : k == 2 ? a.eta_f : k == 3 ? a.acc_f : a.dec_f;
  }
};
template <> struct Num<double> {
  static PCGB_HD double gmw_eps() { return 4e-16; }   // solver.py:109
  static PCGB_HD constexpr double sqrt_pm1(int P) { return sqrt_pm1_d(P); }
  static PCGB_HD double damp_floor() { return 1e-4; } // lsqnonlin.py:278
  static PCGB_HD double prot(const PcgbLmParams& a, int i) { return a.protocol_d[i]; }
  static PCGB_HD double slb(const PcgbLmParams& a, int k) { return a.shared_lb_d[k]; }
  static PCGB_HD double sub(const PcgbLmParams& a, int k) { return a.shared_ub_d[k]; }
  static PCGB_HD double inf() { return __longlong_as_double(0x7ff0000000000000LL); }
  static PCGB_HD double nan() { return __longlong_as_double(0x7fffffffffffffffLL); }
  static PCGB_HD double lmc(const PcgbLmParams& a, int k) {
    return k == 0 ? a.tol : k == 1 ? a.mu : k == 2 ? a.eta : k == 3 ? a.acc : a.dec;
  }
};

PCGB_HD constexpr int pk(int i, int j) { return i * (i + 1) / 2 + j; }  // packed lower index, j <= i
// The reference's diagonal pivoting never picks a pivot (its max search does
// not update the running maximum, permute.py:47-58), and its swaps (i, n-1)
// for i = 0..n-1 (permute.py:185-192) compose to the fixed rotation
// perm = [n-1, 0, 1, ..., n-2]. A NaN diagonal would change the swaps, but it
// also turns every entry of the solution into NaN, which the caller zeroes.
template <int P> PCGB_HD constexpr int rot(int i) { return i == 0 ? P - 1 : i - 1; }

// GMW81 solve (solver.py:431-463) of the packed symmetric matrix A (row i,
// column j <= i) for right-hand side b: rotate, Jacobi-scale by sqrt|diag|,
// modified LDL^T with the reference's delta/beta rules (solver.py:23-95),
// L D L^T solve (solver.py:298-308, 341-350), unscale, un-rotate.
template <int P, typename T>
PCGB_HD void gmw81_solve(const T (&A)[P * (P + 1) / 2], const T (&b)[P], T (&x)[P]) {
  T L[P][P];
  T r[P], s[P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    const int pi = rot<P>(i);
    r[i] = b[pi];
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      const int pj = rot<P>(j);
      L[i][j] = pi >= pj ? A[pk(pi, pj)] : A[pk(pj, pi)];
    }
  }
#pragma unroll
  for (int i = 0; i < P; ++i) {
    s[i] = pcgb_sqrt(pcgb_abs(L[i][i]));
    r[i] /= s[i];
  }
#pragma unroll
  for (int i = 0; i < P; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) L[i][j] /= (s[i] * s[j]);

  T gam = T(0), nu = T(0);
  T beta2 = Num<T>::gmw_eps(), delta = Num<T>::gmw_eps();
#pragma unroll
  for (int i = 0; i < P; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      const T t = pcgb_abs(L[i][j]);
      if (i == j) {
        if (t > gam) gam = t;
      } else {
        if (t > nu) nu = t;
      }
    }
  if (P > 1) nu /= Num<T>::sqrt_pm1(P);
  if (beta2 < gam) beta2 = gam;
  if (beta2 < nu) beta2 = nu;
  if (gam + nu > T(1)) delta *= (gam + nu);

#pragma unroll
  for (int j = 0; j < P; ++j) {
#pragma unroll
    for (int q = 0; q < j; ++q) L[j][q] /= L[q][q];
#pragma unroll
    for (int i = j + 1; i < P; ++i) {
      T t0 = L[i][j];
#pragma unroll
      for (int q = 0; q < j; ++q) t0 -= L[j][q] * L[i][q];
      L[i][j] = t0;
    }
    T th = T(0);
#pragma unroll
    for (int i = j + 1; i < P; ++i) {
      const T t = pcgb_abs(L[i][j]);
      if (th < t) th = t;
    }
    th *= th;
    T d = pcgb_abs(L[j][j]);
    if (d < delta) d = delta;
    const T t0 = th / beta2;
    if (d < t0) d = t0;
    L[j][j] = d;
#pragma unroll
    for (int i = j + 1; i < P; ++i) {
      const T t = L[i][j];
      L[i][i] -= t * t / d;
    }
  }

  T y[P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    T t = r[i];
#pragma unroll
    for (int j = 0; j < i; ++j) t -= L[i][j] * L[j][j] * y[j];
    y[i] = t / L[i][i];
  }
#pragma unroll
  for (int i = P - 1; i >= 0; --i) {
    T t = y[i];
#pragma unroll
    for (int j = i + 1; j < P; ++j) t -= L[j][i] * y[j];
    y[i] = t;
  }
#pragma unroll
  for (int i = 0; i < P; ++i) x[rot<P>(i)] = y[i] / s[i];
}

// ---- FP64 solve for an FP32 fitter -----------------------------------------
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so the FP64 GMW81 path is
// written to spend the FP64 pipe on the factorisation and solve arithmetic
// only:
//  * the rotation and the Jacobi scaling of matrix and right-hand side are the
//    reference's own fp32 operations (solver.py:441-451); the scaled system is
//    then widened to FP64 exactly;
//  * the factorisation and the two triangular solves run in FP64 with one
//    correctly rounded reciprocal per pivot (__drcp_rn) in place of the
//    reference's per-element divisions;
//  * maxima and comparisons of non-negative doubles are taken on their bit
//    patterns (integer pipe). Like the reference's `if (t > m) m = t`, a NaN
//    candidate never wins;
//  * the unscaling multiplies by the fp32 reciprocal of the scale factor.
// Rounding therefore differs from a textbook FP64 division-based solve by a
// few FP64 ulps (and by fp32 rounding in the scale factors, which precondition
// the system and cancel out of the solution up to that rounding).

// The two 32-bit words of a double, through an opaque move: the compiler
// would otherwise recognise a masked sign bit as fabs and emit it as an FP64
// add with an absolute-value operand (a DADD per use, on the FP64 pipe).
PCGB_HD void words(double x, unsigned& lo, unsigned& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}
PCGB_HD unsigned long long abs_bits(double x) {
  unsigned lo, hi;
  words(x, lo, hi);
  return (static_cast<unsigned long long>(hi & 0x7fffffffu) << 32) | lo;
}
// m = max(m, |x|) on bit patterns, NaN skipped (bit patterns above +Inf).
PCGB_HD void max_abs_bits(unsigned long long& m, double x) {
  const unsigned long long b = abs_bits(x);
  if (b <= 0x7ff0000000000000ULL && b > m) m = b;
}
PCGB_HD double from_bits(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }

// The hardware conversions for the rare inputs of widen and narrow, kept out
// of line: an F2F issues on the FP64 pipe, and inlined into a call site the
// compiler may predicate it into the common path as well.
__device__ __noinline__ double widen_hw(float x) { return static_cast<double>(x); }
__device__ __noinline__ float narrow_hw(double x) { return __double2float_rn(x); }

// Exact float -> double widening on the integer pipe (the F2F instruction
// issues on the FP64 pipe): rebias the exponent by 1023 - 127 = 896 and move
// the 23-bit mantissa to the top of the 52-bit one. Zero keeps its sign;
// subnormal, infinite and NaN inputs take the hardware conversion.
PCGB_HD double widen(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u < 254u) {
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu);
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(u << 29));
  }
  if ((u << 1) == 0u) return __hiloint2double(static_cast<int>(u & 0x80000000u), 0);
  return widen_hw(x);
}

// Exact-rounding double -> float (to nearest, ties to even) on the integer
// pipe, for results in the normal float range: rebias the exponent, keep 23
// mantissa bits and round on the 29 dropped ones (a mantissa carry moves into
// the exponent). Zero, float subnormals, the top float binade, Inf and NaN
// take the hardware conversion.
PCGB_HD float narrow(double x) {
  unsigned lo, hi;
  words(x, lo, hi);
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 253u) {
    const unsigned long long t =
        ((static_cast<unsigned long long>(hi & 0x7fffffffu) << 32) | lo) - (896ULL << 52);
    unsigned f = static_cast<unsigned>(t >> 29);
    const unsigned rem = static_cast<unsigned>(t) & 0x1fffffffu;
    f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    return __uint_as_float(f | (hi & 0x80000000u));
  }
  return narrow_hw(x);
}

// 1/x in FP64 from a float seed and one third-order Newton-Raphson step
// (Markstein, IBM J. Res. Dev. 34, 1990): the seed is the float reciprocal of
// x's truncated high word, y0 = (1 - e)/x with |e| < 2^-19.6; with
// e = 1 - x y0, y1 = y0 (1 + e + e^2) = (1 - e^3)/x, so the remaining error
// (< 2^-58) is below double rounding. 3 DFMA in place of the ~11 FP64-pipe
// instructions of the correctly rounded reciprocal, within 1 ulp of it.
// Exponents whose float seed or its reciprocal would leave the normal float
// range (and zero, Inf, NaN) take the hardware reciprocal.
PCGB_HD double rcp64(double x) {
  const unsigned hi = static_cast<unsigned>(__double2hiint(x));
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u >= 252u) return __drcp_rn(x);
  const unsigned fb = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3);
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
  const double y = widen(r);
  const double err = fma(-x, y, 1.0);
  return fma(y, fma(err, err, err), y);
}

// A: packed fp32 matrix (row i, column j <= i), b: fp32 right-hand side.
template <int P>
PCGB_HD void gmw81_solve_f32in_f64(const float (&A)[P * (P + 1) / 2], const float (&b)[P], double (&x)[P]) {
  float s[P], r[P];
  double c[P][P];
  double y[P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    const int pi = rot<P>(i);
    s[i] = sqrtf(fabsf(A[pk(pi, pi)]));
    r[i] = 1.0f / s[i];
    y[i] = widen(b[pi] / s[i]);
  }
#pragma unroll
  for (int i = 0; i < P; ++i) {
    const int pi = rot<P>(i);
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      const int pj = rot<P>(j);
      const float a = pi >= pj ? A[pk(pi, pj)] : A[pk(pj, pi)];
      c[i][j] = widen(a / (s[i] * s[j]));
    }
  }
  // gamma = max |diag|, nu = max |offdiag| / sqrt(P^2 - 1)  (solver.py:32-57)
  unsigned long long gb = 0, nb = 0;
#pragma unroll
  for (int i = 0; i < P; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) max_abs_bits(i == j ? gb : nb, c[i][j]);
  const double gam = from_bits(gb);
  const double nu = P > 1 ? from_bits(nb) * inv_sqrt_pm1_d(P) : 0.0;
  unsigned long long bb = 0x3CBCD2B297D889BCULL;  // 4e-16, solver.py:109
  if (abs_bits(gam) > bb) bb = abs_bits(gam);
  if (abs_bits(nu) > bb) bb = abs_bits(nu);
  const double inv_beta2 = rcp64(from_bits(bb));
  const double gn = gam + nu;  // >= 0: compared with 1 on its bits
  const double delta = abs_bits(gn) > 0x3FF0000000000000ULL ? 4e-16 * gn : 4e-16;

  double inv_d[P];
  double Lr[P][P];  // L_ij = c_ij / d_j (j < i), formed once when d_j is known
#pragma unroll
  for (int j = 0; j < P; ++j) {
#pragma unroll
    for (int i = j + 1; i < P; ++i) {
      double t = c[i][j];
#pragma unroll
      for (int q = 0; q < j; ++q) t = fma(-Lr[j][q], c[i][q], t);
      c[i][j] = t;
    }
    unsigned long long tb = 0;
#pragma unroll
    for (int i = j + 1; i < P; ++i) max_abs_bits(tb, c[i][j]);
    // d = max(|c_jj|, delta, theta^2 / beta^2); a NaN c_jj falls through like the reference
    const unsigned long long cj = abs_bits(c[j][j]);
    double d = cj > 0x7ff0000000000000ULL ? c[j][j] : from_bits(cj);
    if (abs_bits(d) < abs_bits(delta)) d = delta;
    if (j + 1 < P) {  // the last column has no sub-diagonal entries: theta = 0
      const double th = from_bits(tb);
      const double th2 = (th * th) * inv_beta2;
      if (abs_bits(d) < abs_bits(th2)) d = th2;
    }
    inv_d[j] = rcp64(d);
#pragma unroll
    for (int i = j + 1; i < P; ++i) {
      Lr[i][j] = c[i][j] * inv_d[j];
      c[i][i] = fma(-c[i][j], Lr[i][j], c[i][i]);
    }
  }
  // L D y = b' with L_ij d_j = c_ij, then L^T z = y (solver.py:298-308, 341-350)
#pragma unroll
  for (int i = 0; i < P; ++i) {
    double t = y[i];
#pragma unroll
    for (int j = 0; j < i; ++j) t = fma(-c[i][j], y[j], t);
    y[i] = t * inv_d[i];
  }
#pragma unroll
  for (int i = P - 1; i >= 0; --i) {
    double t = y[i];
#pragma unroll
    for (int j = i + 1; j < P; ++j) t = fma(-Lr[j][i], y[j], t);
    y[i] = t;
  }
#pragma unroll
  for (int i = 0; i < P; ++i) x[rot<P>(i)] = y[i] * widen(r[i]);
}

template <typename T> PCGB_HD T load(const void* p, long long i) { return static_cast<const T*>(p)[i]; }
template <typename T> PCGB_HD T load_(const void* p, long long i) { return static_cast<const T*>(p)[i]; }

template <typename A, typename B> struct SameType { static constexpr bool value = false; };
template <typename A> struct SameType<A, A> { static constexpr bool value = true; };
// FP32 state with the FP64 solve / gain-ratio path above
template <typename TA, typename TS>
constexpr bool kMixed = SameType<TA, float>::value && SameType<TS, double>::value;
// unroll factor of the per-sample loops of an iteration (see lm_iterate)
template <typename TA, typename TS, int M>
constexpr int sample_unroll() { return SameType<TA, float>::value && SameType<TS, float>::value ? M : 1; }

// The iterations of one voxel on register state (lsqnonlin.py:823-924 per
// iteration). cf(k, i) returns constant k of sample i; first receives the cost
// of the first iteration; done counts the iterations run; fend receives the
// cost at the final parameters where an iteration evaluated it (the cost of
// the last iterate when its step was rejected or the voxel converged, the
// trial cost when the step was accepted and no bound moved the point), NaN
// otherwise.
//
// LANES > 1 splits a voxel's samples over LANES adjacent lanes of the warp
// (lane `sub` takes samples sub, sub + LANES, ...; d holds those): each lane
// accumulates its share of f, g, h and of the trial cost, the shares are
// summed across the lanes, and every lane then runs the same solve and
// decisions on the same sums (addition is commutative, so the lanes agree
// bit for bit). Only LANES = 1 and 2 are supported.
template <int M, int LANES> constexpr int lane_samples() { return (M + LANES - 1) / LANES; }
template <int LANES, typename T> PCGB_HD T lane_sum(T x) {
  if constexpr (LANES == 2) {
    const unsigned pair = 3u << ((threadIdx.x & 31u) & ~1u);
    x += __shfl_xor_sync(pair, x, 1);
  }
  return x;
}

template <class Model, int M, typename TA, typename TS, int LANES = 1, class CF>
PCGB_HD void lm_iterate(const CF& cf, const TA (&d)[lane_samples<M, LANES>()], TA (&p)[Model::P],
                        const TA (&lo)[Model::P], const TA (&hi)[Model::P], TA (&stp)[Model::P], TA& lam, int& st,
                        TA& f, TA& first, int& done, int iters, TA tol, TA mu, TA eta, TA acc, TA dec, TA& fend,
                        int sub = 0) {
  static_assert(LANES == 1 || LANES == 2, "one or two lanes per voxel");
  constexpr int P = Model::P, H = Model::H, C = Model::C, ML = lane_samples<M, LANES>();
  fend = Num<TA>::nan();
  for (int it = 0; it < iters; ++it) {
    if (st == 0) break;
    ++done;
    // f, g = J^T r, h = sum (J J^T + r d2m), damped diagonal (lsqnonlin.py:225-256)
    TA fa = TA(0), g[P], h[H], hd[P];
#pragma unroll
    for (int k = 0; k < P; ++k) g[k] = hd[k] = TA(0);
#pragma unroll
    for (int k = 0; k < H; ++k) h[k] = TA(0);
    // Sample loops: rolled where the FP64 pipe bounds the iteration (unrolled
    // over 16 samples it no longer fits the instruction cache: IVIM-16, 8.4 M
    // voxels x 8 iterations 13.7 ms unrolled, 11.7 ms rolled; IVIM-10 x 20:
    // 30.3 -> 28.3 ms; the samples then sit in L1-cached local memory),
    // unrolled where instruction issue bounds it (fp32 solve: IVIM-10, 1 M
    // voxels x 20 iterations 1.21 ms unrolled, 1.45 ms rolled).
#pragma unroll (sample_unroll<TA, TS, ML>())
    for (int i = 0; i < ML; ++i) {
      const int smp = i * LANES + sub;
      if (LANES > 1 && smp >= M) break;
      TA c[C > 0 ? C : 1];
#pragma unroll
      for (int k = 0; k < C; ++k) c[k] = cf(k, smp);
      TA m, J[P], Hm[H];
      Model::template all<TA>(p, c, m, J, Hm);
      const TA r = m - d[i];
      fa += r * r;
#pragma unroll
      for (int j = 0; j < P; ++j) {
#pragma unroll
        for (int k = 0; k <= j; ++k) {
          const TA jt = J[j] * J[k];
          const TA hj = Model::hnz(pk(j, k)) ? Hm[pk(j, k)] * r + jt : jt;
          h[pk(j, k)] += hj;
          if (j == k) hd[j] += hj + fmax(lam * jt, Num<TA>::damp_floor());
        }
        g[j] += J[j] * r;
      }
    }
    if constexpr (LANES > 1) {
      fa = lane_sum<LANES>(fa);
#pragma unroll
      for (int k = 0; k < P; ++k) {
        g[k] = lane_sum<LANES>(g[k]);
        hd[k] = lane_sum<LANES>(hd[k]);
      }
#pragma unroll
      for (int k = 0; k < H; ++k) h[k] = lane_sum<LANES>(h[k]);
    }
    f = fa;
    fend = f;
    if (it == 0) first = f;

    // damped solve in TS (lsqnonlin.py:848-878), then drop NaN/Inf (881-891)
    if constexpr (kMixed<TA, TS>) {
      float A[H], b[P];
      double x[P];
#pragma unroll
      for (int i = 0; i < P; ++i) {
        b[i] = g[i];
#pragma unroll
        for (int j = 0; j <= i; ++j) A[pk(i, j)] = i == j ? hd[i] : h[pk(i, j)];
      }
      gmw81_solve_f32in_f64<P>(A, b, x);
#pragma unroll
      for (int k = 0; k < P; ++k) {
        stp[k] = narrow(x[k]);
        if (!isfinite(stp[k])) stp[k] = 0.0f;
      }
    } else {
      TS A[H], b[P], x[P];
#pragma unroll
      for (int i = 0; i < P; ++i) {
        b[i] = TS(g[i]);
#pragma unroll
        for (int j = 0; j <= i; ++j) A[pk(i, j)] = TS(i == j ? hd[i] : h[pk(i, j)]);
      }
      gmw81_solve<P, TS>(A, b, x);
#pragma unroll
      for (int k = 0; k < P; ++k) {
        stp[k] = TA(x[k]);
        if (!isfinite(stp[k])) stp[k] = TA(0);
      }
    }

    // projected-gradient convergence test (lsqnonlin.py:697-723)
    {
      bool clamped = false;
      TA nrm = TA(0);
#pragma unroll
      for (int k = 0; k < P; ++k) {
        TA t2 = p[k] - g[k];
        if (t2 > hi[k]) {
          clamped = true;
          t2 = hi[k];
        } else if (t2 < lo[k]) {
          clamped = true;
          t2 = lo[k];
        }
        t2 = p[k] - t2;
        nrm += t2 * t2;
      }
      if (nrm < tol * (TA(1) + f) && ((st & 1) || clamped)) st = 0;
      if (st == 0) break;
    }

    // trial point and its cost (lsqnonlin.py:902-912, 46-67)
    TA pt[P];
#pragma unroll
    for (int k = 0; k < P; ++k) pt[k] = p[k] - stp[k];
    TA ftp = TA(0);
#pragma unroll (sample_unroll<TA, TS, ML>())
    for (int i = 0; i < ML; ++i) {
      const int smp = i * LANES + sub;
      if (LANES > 1 && smp >= M) break;
      TA c[C > 0 ? C : 1];
#pragma unroll
      for (int k = 0; k < C; ++k) c[k] = cf(k, smp);
      const TA r = Model::template value<TA>(pt, c) - d[i];
      ftp += r * r;
    }
    if constexpr (LANES > 1) ftp = lane_sum<LANES>(ftp);

    // gain ratio in TS (lsqnonlin.py:441-491)
    bool accept, very_good, pred_neg;
    if constexpr (kMixed<TA, TS>) {
      // predicted = s.g - s^T h s / 2 and the test rho = actual / predicted > mu
      // with actual = (f - ftp) / 2, evaluated without the division and with
      // the halving moved to the thresholds: for predicted > 0 it is
      // f - ftp > 2 mu predicted; predicted == +0 gives rho = +Inf.
      // f - ftp is exact in FP64, so its sign is the sign of f - ftp.
      // s^T h s = sum_i s_i (h_ii s_i + 2 sum_{j<i} h_ij s_j), the doubled
      // off-diagonal terms taken from 2 h_ij (exact in fp32).
      const double actual2 = widen(f) - widen(ftp);
      double sg = 0.0, q = 0.0, sd[P];
#pragma unroll
      for (int i = 0; i < P; ++i) sd[i] = widen(stp[i]);
#pragma unroll
      for (int i = 0; i < P; ++i) {
        double off2 = 0.0;
#pragma unroll
        for (int j = 0; j < i; ++j) off2 = fma(widen(2.0f * h[pk(i, j)]), sd[j], off2);
        const double ti = fma(widen(h[pk(i, i)]), sd[i], off2);
        q = fma(sd[i], ti, q);
        sg = fma(sd[i], widen(g[i]), sg);
      }
      const double pred = fma(-0.5, q, sg);
      // comparisons on bit patterns (integer pipe): for positive doubles the
      // order of the bits is the order of the values
      const long long pb = __double_as_longlong(pred);
      const long long ab = __double_as_longlong(actual2);
      const bool pzero = pb == 0;                         // +0: rho = +Inf
      const bool pos = pb > 0 && pb < 0x7ff0000000000000LL;  // finite, > +0
      const bool up = f > ftp;                            // actual > 0
      accept = up && ((pos && ab > __double_as_longlong(widen(2.0f * mu) * pred)) || pzero);
      // only read when accept holds: then actual > 0 and pred > 0 or +0
      very_good = pzero || ab > __double_as_longlong(widen(2.0f * eta) * pred);
      // pred < 0: sign bit set, magnitude in (0, Inf]
      pred_neg = static_cast<unsigned long long>(pb) > 0x8000000000000000ULL &&
                 static_cast<unsigned long long>(pb) <= 0xfff0000000000000ULL;
    } else {
      const TS actual = TS(0.5) * (TS(f) - TS(ftp));
      TS pred = TS(0);
#pragma unroll
      for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
          const TS e = TS(h[pk(i, j)]) * TS(stp[i]) * TS(stp[j]);
          pred -= (i == j) ? e : TS(2) * e;
        }
      pred *= TS(0.5);
#pragma unroll
      for (int i = 0; i < P; ++i) pred += TS(stp[i]) * TS(g[i]);
      const TS rho = actual / pred;
      accept = (rho > TS(mu)) && (actual > TS(0));
      very_good = rho > TS(eta);
      pred_neg = pred < TS(0);
    }
    if (accept) {
#pragma unroll
      for (int k = 0; k < P; ++k) p[k] = pt[k];
      fend = ftp;
      if (very_good) {
        lam *= acc;
        st = 1;
      } else {
        st = 2;
      }
    } else {
      lam *= dec;
      st = 4;
    }
    if (pred_neg) {
      lam *= dec;
      st |= 8;
    }
    // box projection (lsqnonlin.py:590-601)
    bool moved = false;
#pragma unroll
    for (int k = 0; k < P; ++k) {
      if (p[k] > hi[k]) {
        p[k] = hi[k];
        moved = true;
      } else if (p[k] < lo[k]) {
        p[k] = lo[k];
        moved = true;
      }
    }
    if (moved) fend = Num<TA>::nan();
  }
}

// lm_iterate for callers that do not need the cost at the final parameters
template <class Model, int M, typename TA, typename TS, class CF>
PCGB_HD void lm_iterate(const CF& cf, const TA (&d)[M], TA (&p)[Model::P], const TA (&lo)[Model::P],
                        const TA (&hi)[Model::P], TA (&stp)[Model::P], TA& lam, int& st, TA& f, TA& first, int& done,
                        int iters, TA tol, TA mu, TA eta, TA acc, TA dec) {
  TA fend;
  lm_iterate<Model, M, TA, TS>(cf, d, p, lo, hi, stp, lam, st, f, first, done, iters, tol, mu, eta, acc, dec, fend);
}

// protocol accessors for lm_iterate
template <typename TA, int M> struct SharedConsts {
  const PcgbLmParams& a;
  PCGB_HD TA operator()(int k, int i) const { return Num<TA>::prot(a, k * M + i); }
};
template <typename TA, int M, int NC> struct RegConsts {
  const TA (&cv)[NC];
  PCGB_HD TA operator()(int k, int i) const { return cv[k * M + i]; }
};

// No epilogue after a voxel's fit.
struct NoEpilogue {
  template <class PArr, class DArr, class T>
  PCGB_HD void operator()(const PArr&, const DArr&, T) const {}
  static constexpr bool kActive = false;
};

// All iterations of one voxel; then epi(p, d, fend) with the final parameters
// and the samples still in registers and the cost at the final parameters
// where the iterations evaluated it (NaN otherwise; see lm_iterate). A voxel
// converged before the call loads p and d for the epilogue.
// With LANES > 1 the voxel's samples are split over LANES adjacent lanes
// (lane `sub` of them; see lm_iterate) and lane 0 writes the results.
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B, int LANES = 1,
          class Epi = NoEpilogue>
PCGB_HD void lm_fit_voxel(const PcgbLmParams& a, long long v, const Epi& epi = Epi{}, int sub = 0) {
  static_assert(LANES == 1 || !Epi::kActive, "epilogues run with one lane per voxel");
  constexpr int P = Model::P, H = Model::H, C = Model::C, ML = lane_samples<M, LANES>();
  const long long N = a.N;
  const bool fresh = (a.flags & PCGB_LM_FRESH) != 0;
  if (!fresh && a.step_type[v] == 0) {
    // converged before this call (lsqnonlin.py:1000-1002): nothing changes,
    // first_f / last_f are copies of f as in the reference's host loop
    if (a.iters > 0 && sub == 0) {
      const TA f0 = load<TA>(a.f, v);
      static_cast<TA*>(a.first_f)[v] = f0;
      static_cast<TA*>(a.last_f)[v] = f0;
    }
    if constexpr (Epi::kActive) {
      TA p[P], d[M];
#pragma unroll
      for (int k = 0; k < P; ++k) p[k] = load<TA>(a.pars, k * N + v);
#pragma unroll
      for (int i = 0; i < M; ++i) d[i] = load<TA>(a.data, i * N + v);
      epi(p, d, Num<TA>::nan());
    }
    return;
  }
  TA p[P], lo[P], hi[P], stp[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    p[k] = load<TA>(a.pars, k * N + v);
    lo[k] = SHARED_B ? Num<TA>::slb(a, k) : load<TA>(a.lb, k * a.bstride + v);
    hi[k] = SHARED_B ? Num<TA>::sub(a, k) : load<TA>(a.ub, k * a.bstride + v);
    stp[k] = !fresh && a.step ? load<TA>(a.step, k * N + v) : TA(0);
  }
  TA d[ML];
#pragma unroll
  for (int i = 0; i < ML; ++i) {
    const int smp = i * LANES + sub;
    d[i] = LANES == 1 || smp < M ? load<TA>(a.data, smp * N + v) : TA(0);
  }
  TA cv[SHARED_C ? 1 : (C > 0 ? C * M : 1)];
  if (!SHARED_C) {
#pragma unroll
    for (int i = 0; i < C * M; ++i) cv[i] = load<TA>(a.consts, i * a.cstride + v);
  }
  TA lam = fresh ? TA(a.lam_start) : load<TA>(a.lam, v);
  int st = fresh ? 1 : a.step_type[v];
  TA f = fresh ? TA(0) : load<TA>(a.f, v);
  TA first = f;
  const TA tol = Num<TA>::lmc(a, 0), mu = Num<TA>::lmc(a, 1), eta = Num<TA>::lmc(a, 2), acc = Num<TA>::lmc(a, 3),
             dec = Num<TA>::lmc(a, 4);
  int done = 0;
  TA fend;

  if constexpr (SHARED_C) {
    lm_iterate<Model, M, TA, TS, LANES>(SharedConsts<TA, M>{a}, d, p, lo, hi, stp, lam, st, f, first, done, a.iters,
                                        tol, mu, eta, acc, dec, fend, sub);
  } else {
    lm_iterate<Model, M, TA, TS, LANES>(RegConsts<TA, M, (C > 0 ? C * M : 1)>{cv}, d, p, lo, hi, stp, lam, st, f,
                                        first, done, a.iters, tol, mu, eta, acc, dec, fend, sub);
  }
  if (LANES > 1 && sub != 0) return;

  TA* pars = static_cast<TA*>(a.pars);
#pragma unroll
  for (int k = 0; k < P; ++k) pars[k * N + v] = p[k];
  if (a.flags & PCGB_LM_PARS_ONLY) {
    if (a.step_type) a.step_type[v] = static_cast<signed char>(st);
    if constexpr (Epi::kActive) epi(p, d, fend);
    return;
  }
  if (a.step) {
#pragma unroll
    for (int k = 0; k < P; ++k) static_cast<TA*>(a.step)[k * N + v] = stp[k];
  }
  static_cast<TA*>(a.lam)[v] = lam;
  a.step_type[v] = static_cast<signed char>(st);
  static_cast<TA*>(a.f)[v] = f;
  if (a.iters > 0) {
    static_cast<TA*>(a.first_f)[v] = first;
    static_cast<TA*>(a.last_f)[v] = f;
  }
  if (a.iters_done) a.iters_done[v] += done;
  if constexpr (Epi::kActive) epi(p, d, fend);
}

// ---- refill schedule -----------------------------------------------------------
//
// One voxel per lane at a time, one LM iteration per pass: after every pass
// the warp ballots the lanes whose voxel has finished (converged or out of
// iterations), stores them, and hands those lanes the next voxels of the
// warp's chunk by their prefix-sum rank in the ballot. A warp whose chunk is
// drained claims the next chunk of the launch's work counter (one atomic per
// chunk). Lanes therefore never idle behind a slower voxel of their warp
// while work remains; each voxel's arithmetic is the grid schedule's.

template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
struct VoxelFit {
  static constexpr int P = Model::P, C = Model::C;
  TA p[P], lo[P], hi[P], stp[P], d[M];
  TA cv[SHARED_C ? 1 : (C > 0 ? C * M : 1)];
  TA lam, f, first;
  int st, done, it;

  // false when the voxel was converged before the call (its outputs are then
  // already written, as in lm_fit_voxel)
  PCGB_HD bool load(const PcgbLmParams& a, long long v) {
    const long long N = a.N;
    if (a.step_type[v] == 0) {
      if (a.iters > 0) {
        const TA f0 = load_<TA>(a.f, v);
        static_cast<TA*>(a.first_f)[v] = f0;
        static_cast<TA*>(a.last_f)[v] = f0;
      }
      return false;
    }
#pragma unroll
    for (int k = 0; k < P; ++k) {
      p[k] = load_<TA>(a.pars, k * N + v);
      lo[k] = SHARED_B ? Num<TA>::slb(a, k) : load_<TA>(a.lb, k * a.bstride + v);
      hi[k] = SHARED_B ? Num<TA>::sub(a, k) : load_<TA>(a.ub, k * a.bstride + v);
      stp[k] = a.step ? load_<TA>(a.step, k * N + v) : TA(0);
    }
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] = load_<TA>(a.data, i * N + v);
    if (!SHARED_C) {
#pragma unroll
      for (int i = 0; i < C * M; ++i) cv[i] = load_<TA>(a.consts, i * a.cstride + v);
    }
    lam = load_<TA>(a.lam, v);
    st = a.step_type[v];
    f = load_<TA>(a.f, v);
    first = f;
    done = 0;
    it = 0;
    return true;
  }

  // parameters and samples only (for a voxel converged before the call)
  PCGB_HD void load_fit(const PcgbLmParams& a, long long v) {
#pragma unroll
    for (int k = 0; k < P; ++k) p[k] = load_<TA>(a.pars, k * a.N + v);
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] = load_<TA>(a.data, i * a.N + v);
  }

  PCGB_HD bool finished(const PcgbLmParams& a) const { return st == 0 || it >= a.iters; }

  PCGB_HD void step(const PcgbLmParams& a) {
    const TA tol = Num<TA>::lmc(a, 0), mu = Num<TA>::lmc(a, 1), eta = Num<TA>::lmc(a, 2), acc = Num<TA>::lmc(a, 3),
             dec = Num<TA>::lmc(a, 4);
    TA first_it = first;
    if constexpr (SHARED_C) {
      lm_iterate<Model, M, TA, TS>(SharedConsts<TA, M>{a}, d, p, lo, hi, stp, lam, st, f, first_it, done, 1, tol, mu,
                                   eta, acc, dec);
    } else {
      lm_iterate<Model, M, TA, TS>(RegConsts<TA, M, (C > 0 ? C * M : 1)>{cv}, d, p, lo, hi, stp, lam, st, f,
                                   first_it, done, 1, tol, mu, eta, acc, dec);
    }
    if (it == 0) first = first_it;
    ++it;
  }

  PCGB_HD void store(const PcgbLmParams& a, long long v) const {
    const long long N = a.N;
    TA* pars = static_cast<TA*>(a.pars);
#pragma unroll
    for (int k = 0; k < P; ++k) pars[k * N + v] = p[k];
    if (a.step) {
#pragma unroll
      for (int k = 0; k < P; ++k) static_cast<TA*>(a.step)[k * N + v] = stp[k];
    }
    static_cast<TA*>(a.lam)[v] = lam;
    a.step_type[v] = static_cast<signed char>(st);
    static_cast<TA*>(a.f)[v] = f;
    if (a.iters > 0) {
      static_cast<TA*>(a.first_f)[v] = first;
      static_cast<TA*>(a.last_f)[v] = f;
    }
    if (a.iters_done) a.iters_done[v] += done;
  }
};

// Refill schedule over work items [begin, end) and, when `claim` is set,
// further chunks of `chunk` items claimed from a.work. The cursor `next` and
// the range are warp-uniform; idle lanes take items by their rank among the
// idle lanes.
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void lm_refill(const PcgbLmParams& a, long long begin, long long end, bool claim, long long chunk,
                          long long n_items) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  VoxelFit<Model, M, TA, TS, SHARED_C, SHARED_B> s;
  bool active = false;
  long long v = 0;
  long long next = begin;
  for (;;) {
    for (;;) {  // hand work to idle lanes while there is any
      const unsigned idle = __ballot_sync(0xffffffffu, !active);
      if (idle == 0u) break;
      if (next >= end) {
        if (!claim) break;
        unsigned int c = 0;
        if (lane == 0) c = atomicAdd(a.work, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        next = (long long)c * chunk;
        if (next >= n_items) {
          claim = false;
          break;
        }
        end = next + chunk < n_items ? next + chunk : n_items;
      }
      const long long avail = end - next;
      const int nidle = __popc(idle);
      const int take = (long long)nidle < avail ? nidle : int(avail);
      const int my = __popc(idle & lt);
      if (!active && my < take) {
        const long long item = next + my;
        v = a.vox_idx ? (long long)a.vox_idx[item] : item;
        active = s.load(a, v);  // a voxel converged before this call is done at once
      }
      next += take;
    }
    if (!__any_sync(0xffffffffu, active)) break;
    if (active) {
      if (!s.finished(a)) s.step(a);
      if (s.finished(a)) {
        s.store(a, v);
        active = false;
      }
    }
  }
}

// Single-model refill kernel body: every warp starts on an empty range and
// claims chunks of items from a.work. The item count may come from
// device memory (a compaction's counter), so the launch needs no host sync.
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void lm_refill_grid(const PcgbLmParams& a) {
  long long n = a.n_items;
  if (a.n_items_dev) {
    const long long d = (long long)*a.n_items_dev;
    n = d < n ? d : n;
  }
  // about four chunks per warp of the grid, 32..256 items each
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  long long chunk = (n + 4 * warps - 1) / (4 * warps);
  chunk = (chunk + 31) / 32 * 32;
  chunk = chunk < 32 ? 32 : (chunk > 256 ? 256 : chunk);
  lm_refill<Model, M, TA, TS, SHARED_C, SHARED_B>(a, 0, 0, true, chunk, n);
}

// Grid-stride schedule: thread t fits work items t, t + T, t + 2T, ...; an
// item is a voxel index, or an entry of the compacted list vox_idx (whose
// length may be read from device memory, a.n_items_dev).
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void lm_grid(const PcgbLmParams& a) {
  long long n = a.n_items;
  if (a.n_items_dev) {
    const long long d = (long long)*a.n_items_dev;
    n = d < n ? d : n;
  }
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += T)
    lm_fit_voxel<Model, M, TA, TS, SHARED_C, SHARED_B>(a, a.vox_idx ? (long long)a.vox_idx[i] : i);
}

// Mixed-model persistent schedule: each warp repeatedly claims the next chunk
// of voxels from the work counter and fits it with the chunk's model (FitJob<k>
// is the per-model lm_fit_voxel instantiation). A warp never mixes models, so
// models only diverge between warps; voxels of fast-converging models free
// their warp early and it takes more work.
template <class Dispatch>
__device__ void multi_grid(const PcgbMultiParams& q) {
  const int lane = threadIdx.x & 31;
  const long long total = q.chunk_off[q.njobs];
  for (;;) {
    unsigned int c = 0;
    if (lane == 0) c = atomicAdd(q.counter, 1u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if ((long long)c >= total) break;
    int t = 0;
    while (t + 1 < q.njobs && (long long)c >= q.chunk_off[t + 1]) ++t;
    const int k = q.order[t];
    const long long base = ((long long)c - q.chunk_off[t]) * q.chunk;
    Dispatch::run(k, q.jobs[k], base, q.chunk, lane);
  }
}

// Accumulating cost, the reference F kernel (lsqnonlin.py:157-177, 46-67):
// f[v] += sum_i (m(p_v; c_i) - d_i)^2, voxels with step_type == 0 skipped.
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void cost_grid(const PcgbLmParams& a) {
  constexpr int P = Model::P, C = Model::C;
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n_items; i += T) {
    const long long v = a.vox_idx ? (long long)a.vox_idx[i] : i;
    if (a.step_type && a.step_type[v] == 0) continue;
    TA p[P];
#pragma unroll
    for (int k = 0; k < P; ++k) p[k] = load<TA>(a.pars, k * a.N + v);
    TA fa = TA(0);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      TA c[C > 0 ? C : 1];
#pragma unroll
      for (int k = 0; k < C; ++k)
        c[k] = SHARED_C ? Num<TA>::prot(a, k * M + i) : load<TA>(a.consts, (k * M + i) * a.cstride + v);
      const TA r = Model::template value<TA>(p, c) - load<TA>(a.data, i * a.N + v);
      fa += r * r;
    }
    static_cast<TA*>(a.f)[v] += fa;
  }
}

// Forward model m(p_v; c_i) for every voxel and sample into model_out (M, N):
// synthetic signals, residual maps, fitted curves.
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void eval_grid(const PcgbLmParams& a) {
  constexpr int P = Model::P, C = Model::C;
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < a.n_items; v += T) {
    TA p[P];
#pragma unroll
    for (int k = 0; k < P; ++k) p[k] = load<TA>(a.pars, k * a.N + v);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      TA c[C > 0 ? C : 1];
#pragma unroll
      for (int k = 0; k < C; ++k)
        c[k] = SHARED_C ? Num<TA>::prot(a, k * M + i) : load<TA>(a.consts, (k * M + i) * a.cstride + v);
      static_cast<TA*>(a.model_out)[i * a.N + v] = Model::template value<TA>(p, c);
    }
  }
}

// ---- fallback of a warm-started fit -------------------------------------------
//
// A warm-started fit is refitted from the plain fitter's constant start where
// its cost is not finite, not below the cost at that start, or where it ends
// on a bound. The check decides this per voxel from registers (both costs),
// compacts the flagged voxels with one atomic per warp, saves their warm fits
// and resets their fitter state to the constant start; the refit runs on the
// compacted list with the count read from device memory, and the select keeps,
// per flagged voxel, whichever of the two fits has the lower cost. No step
// needs the flagged count on the host. The check runs either as its own pass
// (warm_check_grid) or as the epilogue of the warm LM (lm_check_grid), the
// select as its own pass (warm_select_grid) or as the epilogue of the refit
// (lm_select_grid).

// sum_i (m(p; c_i) - d_i)^2, in the order of cost_grid
template <class Model, int M, typename TA, class CF>
PCGB_HD TA sum_sq_residual(const CF& cf, const TA (&p)[Model::P], const TA (&d)[M]) {
  constexpr int C = Model::C;
  TA s = TA(0);
#pragma unroll
  for (int i = 0; i < M; ++i) {
    TA c[C > 0 ? C : 1];
#pragma unroll
    for (int k = 0; k < C; ++k) c[k] = cf(k, i);
    const TA r = Model::template value<TA>(p, c) - d[i];
    s += r * r;
  }
  return s;
}

template <class Model, int M, typename TA, bool SHARED_C>
PCGB_HD TA voxel_cost(const PcgbLmParams& a, long long v, const TA (&p)[Model::P], const TA (&d)[M]) {
  constexpr int C = Model::C;
  if constexpr (SHARED_C) {
    return sum_sq_residual<Model, M, TA>(SharedConsts<TA, M>{a}, p, d);
  } else {
    TA cv[C > 0 ? C * M : 1];
#pragma unroll
    for (int i = 0; i < C * M; ++i) cv[i] = load<TA>(a.consts, i * a.cstride + v);
    return sum_sq_residual<Model, M, TA>(RegConsts<TA, M, (C > 0 ? C * M : 1)>{cv}, p, d);
  }
}

// The check of one voxel from its warm fit p and samples d in registers
// (valid = the lane has a voxel; every lane of the warp calls this, for the
// ballot): cost at p into a.cost, flag, compaction into a.fb_idx, backup of
// the warm fit, state reset to the constant start.
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void warm_check_voxel(const PcgbLmParams& a, long long v, bool valid, const TA (&p)[Model::P],
                                 const TA (&d)[M]) {
  constexpr int P = Model::P;
  const long long N = a.N;
  bool flag = false;
  TA p0[P], c = TA(0);
  if (valid) {
    TA mx = -Num<TA>::inf();
#pragma unroll
    for (int i = 0; i < M; ++i) mx = fmax(mx, d[i]);
#pragma unroll
    for (int k = 0; k < P; ++k) p0[k] = isnan(a.init_val[k]) ? mx : TA(a.init_val[k]);
    c = voxel_cost<Model, M, TA, SHARED_C>(a, v, p, d);
    const TA c0 = voxel_cost<Model, M, TA, SHARED_C>(a, v, p0, d);
    flag = !isfinite(c) || !(c < c0);
#pragma unroll
    for (int k = 0; k < P; ++k) {
      const TA lo = a.bstride ? load<TA>(a.lb, k * a.bstride + v) : Num<TA>::slb(a, k);
      const TA hi = a.bstride ? load<TA>(a.ub, k * a.bstride + v) : Num<TA>::sub(a, k);
      flag = flag || !(p[k] > lo) || !(p[k] < hi);
    }
    static_cast<TA*>(a.cost)[v] = c;
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned ballot = __ballot_sync(0xffffffffu, flag);
  if (!ballot) return;
  unsigned base = 0;
  if (lane == 0) base = atomicAdd(a.fb_count, (unsigned)__popc(ballot));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (!flag) return;
  const long long i = (long long)base + __popc(ballot & ((1u << lane) - 1u));
  a.fb_idx[i] = int(v);
#pragma unroll
  for (int k = 0; k < P; ++k) {
    static_cast<TA*>(a.pars_backup)[k * N + i] = p[k];
    static_cast<TA*>(a.pars)[k * N + v] = p0[k];
  }
  static_cast<TA*>(a.cost_backup)[i] = c;
  static_cast<TA*>(a.lam)[v] = TA(a.lam0);
  a.step_type[v] = 1;
  static_cast<TA*>(a.f)[v] = TA(0);
}

// one thread per voxel, grid covering N (every lane reaches the ballot)
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void warm_check_grid(const PcgbLmParams& a) {
  constexpr int P = Model::P;
  const long long N = a.N;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  TA p[P], d[M];
  if (v < N) {
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] = load<TA>(a.data, i * N + v);
#pragma unroll
    for (int k = 0; k < P; ++k) p[k] = load<TA>(a.pars, k * N + v);
  }
  warm_check_voxel<Model, M, TA, SHARED_C>(a, v, v < N, p, d);
}

// The warm LM with the check as its epilogue: the samples and the fit are
// still in registers when the iterations end, so the check costs two model
// evaluations and no second pass over the signals. One thread per voxel,
// grid covering N. Per voxel the same arithmetic as lm_grid + warm_check_grid.
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void lm_check_grid(const PcgbLmParams& a) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = v < a.N;
  VoxelFit<Model, M, TA, TS, SHARED_C, SHARED_B> s;
  if (valid) {
    if (s.load(a, v)) {
      while (!s.finished(a)) s.step(a);
      s.store(a, v);
    } else {
      s.load_fit(a, v);  // converged before the call: the check still needs p and d
    }
  }
  warm_check_voxel<Model, M, TA, SHARED_C>(a, v, valid, s.p, s.d);
}

// The check of one voxel as the epilogue of its warm LM fit (lm_warm_grid):
// the cost at the warm fit comes from the iterations (c; NaN where they did
// not evaluate it: the last accepted step was moved by a bound, and the voxel
// is flagged for being on the bound anyway - the select evaluates that cost -
// or no iteration ran, and it is evaluated here), so in general only the
// cost at the constant start is evaluated. Same rule, compaction, backup and
// state reset as warm_check_voxel; the flagged voxels of each group of lanes
// that reaches this point together are compacted with one atomic (any
// grouping gives a valid list).
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void warm_flag_voxel(const PcgbLmParams& a, long long v, const TA (&p)[Model::P], const TA (&d)[M], TA c) {
  constexpr int P = Model::P;
  const long long N = a.N;
  if (a.iters == 0) c = voxel_cost<Model, M, TA, SHARED_C>(a, v, p, d);
  TA p0[P];
  TA mx = -Num<TA>::inf();
#pragma unroll
  for (int i = 0; i < M; ++i) mx = fmax(mx, d[i]);
#pragma unroll
  for (int k = 0; k < P; ++k) p0[k] = isnan(a.init_val[k]) ? mx : TA(a.init_val[k]);
  const TA c0 = voxel_cost<Model, M, TA, SHARED_C>(a, v, p0, d);
  bool flag = !isfinite(c) || !(c < c0);
#pragma unroll
  for (int k = 0; k < P; ++k) {
    const TA lo = a.bstride ? load<TA>(a.lb, k * a.bstride + v) : Num<TA>::slb(a, k);
    const TA hi = a.bstride ? load<TA>(a.ub, k * a.bstride + v) : Num<TA>::sub(a, k);
    flag = flag || !(p[k] > lo) || !(p[k] < hi);
  }
  static_cast<TA*>(a.cost)[v] = c;
  const unsigned m = __activemask();
  const unsigned ballot = __ballot_sync(m, flag);
  if (!ballot) return;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned leader = unsigned(__ffs(m) - 1);
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(a.fb_count, (unsigned)__popc(ballot));
  base = __shfl_sync(m, base, leader);
  if (!flag) return;
  const long long i = (long long)base + __popc(ballot & ((1u << lane) - 1u));
  a.fb_idx[i] = int(v);
#pragma unroll
  for (int k = 0; k < P; ++k) {
    static_cast<TA*>(a.pars_backup)[k * N + i] = p[k];
    static_cast<TA*>(a.pars)[k * N + v] = p0[k];
  }
  static_cast<TA*>(a.cost_backup)[i] = c;
  static_cast<TA*>(a.lam)[v] = TA(a.lam0);
  a.step_type[v] = 1;
  static_cast<TA*>(a.f)[v] = TA(0);
}

template <class Model, int M, typename TA, bool SHARED_C>
struct FlagEpilogue {
  const PcgbLmParams& a;
  long long v;
  static constexpr bool kActive = true;
  PCGB_HD void operator()(const TA (&p)[Model::P], const TA (&d)[M], TA c) const {
    warm_flag_voxel<Model, M, TA, SHARED_C>(a, v, p, d, c);
  }
};

// The warm LM (a.flags: fresh start, parameters only) with the fallback check
// as its epilogue; one thread per voxel, grid covering N.
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void lm_warm_grid(const PcgbLmParams& a) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v < a.N) lm_fit_voxel<Model, M, TA, TS, SHARED_C, SHARED_B>(a, v, FlagEpilogue<Model, M, TA, SHARED_C>{a, v});
}

// keep the refit or restore the warm fit of flagged item i (voxel v), from
// the refit's parameters and samples in registers; a warm cost saved as NaN
// (not evaluated by the warm iterations) is evaluated here
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void warm_select_voxel(const PcgbLmParams& a, long long i, long long v, const TA (&p)[Model::P],
                                  const TA (&d)[M]) {
  constexpr int P = Model::P;
  const long long N = a.N;
  const TA c = voxel_cost<Model, M, TA, SHARED_C>(a, v, p, d);
  TA cb = load<TA>(a.cost_backup, i);
  if (isnan(cb)) {
    TA pb[P];
#pragma unroll
    for (int k = 0; k < P; ++k) pb[k] = load<TA>(a.pars_backup, k * N + i);
    cb = voxel_cost<Model, M, TA, SHARED_C>(a, v, pb, d);
  }
  const bool refit = c < cb;
  if (!refit) {
#pragma unroll
    for (int k = 0; k < P; ++k) static_cast<TA*>(a.pars)[k * N + v] = load<TA>(a.pars_backup, k * N + i);
  }
  static_cast<TA*>(a.cost)[v] = refit ? c : cb;
  if (a.which) a.which[v] = refit ? 1 : 0;
  const unsigned m = __activemask();
  const unsigned kept = __ballot_sync(m, refit);
  if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1) && kept) atomicAdd(a.fb_count + 1, (unsigned)__popc(kept));
}

PCGB_HD long long device_count(const PcgbLmParams& a) {
  long long n = a.n_items;
  if (a.n_items_dev) {
    const long long d = (long long)*a.n_items_dev;
    n = d < n ? d : n;
  }
  return n;
}

// grid-stride over the flagged voxels (count from a.n_items_dev)
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void warm_select_grid(const PcgbLmParams& a) {
  constexpr int P = Model::P;
  const long long N = a.N;
  const long long n = device_count(a);
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += T) {
    const long long v = a.fb_idx[i];
    TA p[P], d[M];
#pragma unroll
    for (int k = 0; k < P; ++k) p[k] = load<TA>(a.pars, k * N + v);
#pragma unroll
    for (int q = 0; q < M; ++q) d[q] = load<TA>(a.data, q * N + v);
    warm_select_voxel<Model, M, TA, SHARED_C>(a, i, v, p, d);
  }
}

// The refit of the flagged voxels with the select as its epilogue
// (grid-stride over the compacted list, count from a.n_items_dev).
// the select of a refitted voxel as lm_fit_voxel's epilogue
template <class Model, int M, typename TA, bool SHARED_C>
struct SelectEpilogue {
  const PcgbLmParams& a;
  long long i, v;
  static constexpr bool kActive = true;
  PCGB_HD void operator()(const TA (&p)[Model::P], const TA (&d)[M], TA) const {
    warm_select_voxel<Model, M, TA, SHARED_C>(a, i, v, p, d);
  }
};

template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void lm_select_grid(const PcgbLmParams& a) {
  const long long n = device_count(a);
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += T) {
    const long long v = a.vox_idx[i];
    lm_fit_voxel<Model, M, TA, TS, SHARED_C, SHARED_B>(a, v, SelectEpilogue<Model, M, TA, SHARED_C>{a, i, v});
  }
}

// ---- searches ----------------------------------------------------------------

// splitmix64 output function (Steele, Lea & Flood, OOPSLA 2014)
PCGB_HD unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
// Counter-based uniform draw in [0, 1) with 24 random bits for component k of
// draw d of voxel v: every voxel has an independent, reproducible stream.
PCGB_HD float uniform01(unsigned long long seed, long long v, int d, int k) {
  unsigned long long z = mix64(seed + 0x9E3779B97F4A7C15ULL * (unsigned long long)(v + 1));
  z = mix64(z ^ (((unsigned long long)(unsigned)d << 8) | (unsigned)k));
  return float(z >> 40) * (1.0f / 16777216.0f);
}

// One SearchStep launch (lsqnonlin.py:1083-1105, kernel 1153-1162): f[v] +=
// cost(p_v) (accumulating, as the reference's cost function does), then keep
// (p_v, f[v]) as the best point if f[v] < best_f[v].
template <class Model, int M, typename TA, bool SHARED_C>
__device__ void search_step_grid(const PcgbLmParams& a) {
  constexpr int P = Model::P, C = Model::C;
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < a.n_items; v += T) {
    TA p[P];
#pragma unroll
    for (int k = 0; k < P; ++k) p[k] = load<TA>(a.pars, k * a.N + v);
    TA fa = TA(0);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      TA c[C > 0 ? C : 1];
#pragma unroll
      for (int k = 0; k < C; ++k)
        c[k] = SHARED_C ? Num<TA>::prot(a, k * M + i) : load<TA>(a.consts, (k * M + i) * a.cstride + v);
      const TA r = Model::template value<TA>(p, c) - load<TA>(a.data, i * a.N + v);
      fa += r * r;
    }
    TA* f = static_cast<TA*>(a.f);
    const TA fv = f[v] + fa;
    f[v] = fv;
    if (fv < load<TA>(a.best_f, v)) {
#pragma unroll
      for (int k = 0; k < P; ++k) static_cast<TA*>(a.best_p)[k * a.N + v] = p[k];
      static_cast<TA*>(a.best_f)[v] = fv;
    }
  }
}

// Random search (RandomSearch.run, lsqnonlin.py:1232-1242) and, with
// lm_iters > 0, second-order random search (SecondOrderRandomSearch.run,
// lsqnonlin.py:1277-1291): a.iters draws uniform in [lb, ub]; each draw is
// optionally refined by lm_iters LM iterations from lambda = 5, step_type = 1;
// the draw's cost at its final point is compared with the best so far.
// All draws of a voxel run in one thread with its signals in registers.
template <class Model, int M, typename TA, typename TS, bool SHARED_C, bool SHARED_B>
__device__ void random_search_grid(const PcgbLmParams& a) {
  constexpr int P = Model::P, C = Model::C;
  const long long T = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < a.n_items; v += T) {
    const long long N = a.N;
    TA lo[P], hi[P], bp[P];
#pragma unroll
    for (int k = 0; k < P; ++k) {
      lo[k] = SHARED_B ? Num<TA>::slb(a, k) : load<TA>(a.lb, k * a.bstride + v);
      hi[k] = SHARED_B ? Num<TA>::sub(a, k) : load<TA>(a.ub, k * a.bstride + v);
      bp[k] = load<TA>(a.best_p, k * N + v);
    }
    TA d[M];
#pragma unroll
    for (int i = 0; i < M; ++i) d[i] = load<TA>(a.data, i * N + v);
    TA cv[SHARED_C ? 1 : (C > 0 ? C * M : 1)];
    if (!SHARED_C) {
#pragma unroll
      for (int i = 0; i < C * M; ++i) cv[i] = load<TA>(a.consts, i * a.cstride + v);
    }
    TA bf = load<TA>(a.best_f, v);
    const TA tol = Num<TA>::lmc(a, 0), mu = Num<TA>::lmc(a, 1), eta = Num<TA>::lmc(a, 2), acc = Num<TA>::lmc(a, 3),
             dec = Num<TA>::lmc(a, 4);
    for (int dr = 0; dr < a.iters; ++dr) {
      TA p[P], stp[P];
#pragma unroll
      for (int k = 0; k < P; ++k) {
        p[k] = fma(TA(uniform01(a.seed, v, dr, k)), hi[k] - lo[k], lo[k]);  // rand * (ub - lb) + lb
        stp[k] = TA(0);
      }
      if (a.lm_iters > 0) {
        TA lam = TA(5), f = TA(0), first = TA(0);
        int st = 1, done = 0;
        if constexpr (SHARED_C)
          lm_iterate<Model, M, TA, TS>(SharedConsts<TA, M>{a}, d, p, lo, hi, stp, lam, st, f, first, done, a.lm_iters,
                                       tol, mu, eta, acc, dec);
        else
          lm_iterate<Model, M, TA, TS>(RegConsts<TA, M, (C > 0 ? C * M : 1)>{cv}, d, p, lo, hi, stp, lam, st, f, first,
                                       done, a.lm_iters, tol, mu, eta, acc, dec);
      }
      TA fa = TA(0);
#pragma unroll
      for (int i = 0; i < M; ++i) {
        TA c[C > 0 ? C : 1];
#pragma unroll
        for (int k = 0; k < C; ++k) c[k] = SHARED_C ? Num<TA>::prot(a, k * M + i) : cv[k * M + i];
        const TA r = Model::template value<TA>(p, c) - d[i];
        fa += r * r;
      }
      if (fa < bf) {
        bf = fa;
#pragma unroll
        for (int k = 0; k < P; ++k) bp[k] = p[k];
      }
    }
#pragma unroll
    for (int k = 0; k < P; ++k) static_cast<TA*>(a.best_p)[k * N + v] = bp[k];
    static_cast<TA*>(a.best_f)[v] = bf;
  }
}

// Batched GMW81 solve (the reference GMW81Solver kernel, solver.py:526-563):
// consts holds the packed (H, N) matrices, data the (P, N) right-hand sides,
// step receives the (P, N) solutions.
template <int P, typename T>
__device__ void gmw81_grid(const PcgbLmParams& a) {
  constexpr int H = P * (P + 1) / 2;
  const long long T_ = (long long)gridDim.x * blockDim.x;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < a.n_items; v += T_) {
    T A[H], b[P], x[P];
#pragma unroll
    for (int q = 0; q < H; ++q) A[q] = load<T>(a.consts, q * a.N + v);
#pragma unroll
    for (int k = 0; k < P; ++k) b[k] = load<T>(a.data, k * a.N + v);
    gmw81_solve<P, T>(A, b, x);
#pragma unroll
    for (int k = 0; k < P; ++k) static_cast<T*>(a.step)[k * a.N + v] = x[k];
  }
}

}  // namespace pcgb
