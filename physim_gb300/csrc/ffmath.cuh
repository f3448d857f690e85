// ffmath.cuh -- double-float arithmetic on the FP32 pipe, and the served path's element
// energy and gradient in it.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, about 46 bits
// of significand.  GB300 issues FP64 at 1/64 of its FP32 rate, and the element energy and
// gradient stage of the served path was bound by it; it needs about 1e-13 relative accuracy
// (the line search compares energy totals that differ by ~1e-10 of their size), which
// double-float gives.  The operations are the error-free transformations of Knuth (TwoSum),
// Dekker (FastTwoSum) and the fused-multiply-add TwoProduct, combined as in the "accurate"
// double-double addition and multiplication of Hida, Li and Bailey ("Library for
// double-double and quad-double arithmetic", 2000).  The rounded primitives are written with
// __fadd_rn / __fmul_rn so that the compiler neither contracts nor reorders them.
//
// log1p and j - log1p(j), the two transcendental terms of the Neo-Hookean energy, come from
// series in t = j / (2 + j): log1p(j) = 2 atanh(t) = 2 t sum_k t^2k / (2k + 1), and
// j - log1p(j) = 2 t sum_{n>=1} c_n t^n with c_n = 1 (n odd), n / (n + 1) (n even), which is
// free of the cancellation of j - log1p(j) near 0.  Both are used for |j| <= 1/8 (|t| <= 1/17,
// 7 and 14 terms reach 2^-48); larger volume changes take FP64 log1p.
#pragma once

#include <cuda_runtime.h>

namespace phx {

struct ff {
  float hi, lo;
};

// a double constant split into two floats at compile time (no FP64 instruction at run time)
struct ffk {
  float hi, lo;
  __host__ __device__ constexpr ffk(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

__device__ __forceinline__ ff ff_of(float a) { return ff{a, 0.f}; }
__device__ __forceinline__ ff ff_of(ffk c) { return ff{c.hi, c.lo}; }
// a compile-time constant (the split is evaluated by the compiler)
#define FFK(v) ([] { constexpr ffk k_(v); return ff{k_.hi, k_.lo}; }())
__device__ __forceinline__ ff ff_of_d(double d) {
  const float h = __double2float_rn(d);
  return ff{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  const ff t = two_sum(a.lo, b.lo);
  s = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }
__device__ __forceinline__ ff ff_sqr(ff a) { return ff_mul(a, a); }
// a / b: a float quotient refined twice against the double-float remainder
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  ff r = ff_sub(a, ff_mulf(b, q1));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  r = ff_sub(r, ff_mulf(b, q2));
  const float q3 = __fdiv_rn(r.hi, b.hi);
  return ff_add(fast_two_sum(q1, q2), ff_of(q3));
}
__device__ __forceinline__ ff ff_scale(ff a, float p2) { return ff{a.hi * p2, a.lo * p2}; }  // p2 a power of 2

// ---------------------------------------------------------------------------
// log1p(j) and j - log1p(j) for |j| <= 1/8
// ---------------------------------------------------------------------------
constexpr float kFFLogRange = 0.125f;

__device__ __forceinline__ void ff_log1p_pair(ff j, ff* l1p, ff* f) {
  const ff t = ff_div(j, ff_add(ff_of(2.f), j));
  const ff t2 = ff_sqr(t);
  // S = sum_{k=0..6} t^2k / (2k + 1)
  ff S = FFK(1.0 / 13.0);
  S = ff_fma(S, t2, FFK(1.0 / 11.0));
  S = ff_fma(S, t2, FFK(1.0 / 9.0));
  S = ff_fma(S, t2, FFK(1.0 / 7.0));
  S = ff_fma(S, t2, FFK(1.0 / 5.0));
  S = ff_fma(S, t2, FFK(1.0 / 3.0));
  S = ff_fma(S, t2, ff_of(1.f));
  *l1p = ff_mul(ff_scale(t, 2.f), S);
  // D = sum_{n=1..14} c_n t^(n-1), c_n = 1 (n odd), n / (n + 1) (n even)
  ff D = FFK(14.0 / 15.0);
  D = ff_fma(D, t, ff_of(1.f));
  D = ff_fma(D, t, FFK(12.0 / 13.0));
  D = ff_fma(D, t, ff_of(1.f));
  D = ff_fma(D, t, FFK(10.0 / 11.0));
  D = ff_fma(D, t, ff_of(1.f));
  D = ff_fma(D, t, FFK(8.0 / 9.0));
  D = ff_fma(D, t, ff_of(1.f));
  D = ff_fma(D, t, FFK(6.0 / 7.0));
  D = ff_fma(D, t, ff_of(1.f));
  D = ff_fma(D, t, FFK(4.0 / 5.0));
  D = ff_fma(D, t, ff_of(1.f));
  D = ff_fma(D, t, FFK(2.0 / 3.0));
  D = ff_fma(D, t, ff_of(1.f));
  // j - log1p(j) = 2 t (t D)
  *f = ff_mul(ff_scale(t, 2.f), ff_mul(t, D));
}

// ---------------------------------------------------------------------------
// element energy density and PK1 from H = F - I (column-major), in double-float: the same
// cancellation-free forms as material_eg in kernels.cu
//   CoNH:  psi = mu/2 (|H|^2 - 2 q + 2 f(j)) + lam/2 log(J)^2, j = tr H + q, q = I2(H) + det H,
//          P = mu F + (lam log J - mu) cof(F) / J
//   StVK:  E = (H + H^T + H^T H)/2, psi = lam/2 tr(E)^2 + mu E:E, P = F (lam tr(E) I + 2 mu E)
// ---------------------------------------------------------------------------
__device__ __forceinline__ ff ff_det3(const ff* A) {
  // A column-major: A(r, c) = A[r + 3c]
  const ff m0 = ff_sub(ff_mul(A[4], A[8]), ff_mul(A[7], A[5]));
  const ff m1 = ff_sub(ff_mul(A[1], A[8]), ff_mul(A[7], A[2]));
  const ff m2 = ff_sub(ff_mul(A[1], A[5]), ff_mul(A[4], A[2]));
  return ff_add(ff_sub(ff_mul(A[0], m0), ff_mul(A[3], m1)), ff_mul(A[6], m2));
}

// Returns false for an inverted element (J - 1 = j < -1, both models, as the FP64 kernels
// test it); psi and P are then not set.
__device__ __forceinline__ bool ff_material(int model, ff lam, ff mu, const ff* H, ff* psi, ff* P) {
  const ff trH = ff_add(ff_add(H[0], H[4]), H[8]);
  ff I2 = ff_sub(ff_mul(H[0], H[4]), ff_mul(H[3], H[1]));
  I2 = ff_add(I2, ff_sub(ff_mul(H[0], H[8]), ff_mul(H[6], H[2])));
  I2 = ff_add(I2, ff_sub(ff_mul(H[4], H[8]), ff_mul(H[7], H[5])));
  const ff q = ff_add(I2, ff_det3(H));
  const ff j = ff_add(trH, q);  // J - 1
  // J = 0 exactly: inverted for CoNH (log J), a finite StVK energy, as in FP64
  if (j.hi < -1.f || (j.hi == -1.f && (j.lo < 0.f || (j.lo == 0.f && model != 1)))) return false;
  ff F[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) F[k] = H[k];
  F[0] = ff_add(F[0], ff_of(1.f));
  F[4] = ff_add(F[4], ff_of(1.f));
  F[8] = ff_add(F[8], ff_of(1.f));
  if (model == 1) {
    ff E[9];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        ff s = ff_add(H[i + 3 * jj], H[jj + 3 * i]);
        s = ff_fma(H[3 * i], H[3 * jj], s);
        s = ff_fma(H[1 + 3 * i], H[1 + 3 * jj], s);
        s = ff_fma(H[2 + 3 * i], H[2 + 3 * jj], s);
        E[i + 3 * jj] = ff_scale(s, 0.5f);
      }
    const ff trE = ff_add(ff_add(E[0], E[4]), E[8]);
    ff ee = ff_sqr(E[0]);
#pragma unroll
    for (int k = 1; k < 9; ++k) ee = ff_fma(E[k], E[k], ee);
    *psi = ff_add(ff_scale(ff_mul(lam, ff_sqr(trE)), 0.5f), ff_mul(mu, ee));
    ff S[9];
    const ff mu2 = ff_scale(mu, 2.f), lt = ff_mul(lam, trE);
#pragma unroll
    for (int k = 0; k < 9; ++k) S[k] = ff_mul(mu2, E[k]);
    S[0] = ff_add(S[0], lt);
    S[4] = ff_add(S[4], lt);
    S[8] = ff_add(S[8], lt);
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
#pragma unroll
      for (int i = 0; i < 3; ++i)
        P[i + 3 * jj] = ff_fma(F[i + 6], S[2 + 3 * jj], ff_fma(F[i + 3], S[1 + 3 * jj], ff_mul(F[i], S[3 * jj])));
    return true;
  }
  ff hh = ff_sqr(H[0]);
#pragma unroll
  for (int k = 1; k < 9; ++k) hh = ff_fma(H[k], H[k], hh);
  ff l1p, f;
  if (fabsf(j.hi) <= kFFLogRange) {
    ff_log1p_pair(j, &l1p, &f);
  } else {  // large volume changes: FP64 log1p (no cancellation in j - log1p(j) there)
    const double jd = ff_to_d(j);
    const double ld = log1p(jd);
    l1p = ff_of_d(ld);
    f = ff_of_d(jd - ld);
  }
  const ff J = ff_add(ff_of(1.f), j);
  // psi = mu/2 (hh - 2 q + 2 f) + lam/2 l1p^2
  const ff inner = ff_add(ff_sub(hh, ff_scale(q, 2.f)), ff_scale(f, 2.f));
  *psi = ff_add(ff_scale(ff_mul(mu, inner), 0.5f), ff_scale(ff_mul(lam, ff_sqr(l1p)), 0.5f));
  // cof(F) column-major: C(r, c) = cofactor of F(r, c)
  ff C[9];
  C[0] = ff_sub(ff_mul(F[4], F[8]), ff_mul(F[7], F[5]));
  C[1] = ff_sub(ff_mul(F[5], F[6]), ff_mul(F[3], F[8]));
  C[2] = ff_sub(ff_mul(F[3], F[7]), ff_mul(F[4], F[6]));
  C[3] = ff_sub(ff_mul(F[2], F[7]), ff_mul(F[1], F[8]));
  C[4] = ff_sub(ff_mul(F[0], F[8]), ff_mul(F[2], F[6]));
  C[5] = ff_sub(ff_mul(F[1], F[6]), ff_mul(F[0], F[7]));
  C[6] = ff_sub(ff_mul(F[1], F[5]), ff_mul(F[2], F[4]));
  C[7] = ff_sub(ff_mul(F[2], F[3]), ff_mul(F[0], F[5]));
  C[8] = ff_sub(ff_mul(F[0], F[4]), ff_mul(F[1], F[3]));
  const ff c = ff_div(ff_sub(ff_mul(lam, l1p), mu), J);
#pragma unroll
  for (int k = 0; k < 9; ++k) P[k] = ff_fma(c, C[k], ff_mul(mu, F[k]));
  return true;
}

}  // namespace phx
