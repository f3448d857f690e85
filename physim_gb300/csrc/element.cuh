// element.cuh -- per-tet element arithmetic shared by the kernels.
//
// The element Hessian: the 10 node blocks of H_e = w DFDx^T dP/dF DFDx
// (EnergyElement_FEM::ComputeAndStore_Hessian_Internal,
// source/PhySim/Physics/Elements/EnergyElement_FEM.cpp:193-222) in closed form.
#pragma once

#include <cstdint>

namespace phx {

template <typename T> __device__ __forceinline__ T dlog(T x);
template <> __device__ __forceinline__ float dlog<float>(float x) { return logf(x); }
template <> __device__ __forceinline__ double dlog<double>(double x) { return log(x); }
template <typename T> __device__ __forceinline__ T dlog1p(T x);
template <> __device__ __forceinline__ float dlog1p<float>(float x) { return log1pf(x); }
template <> __device__ __forceinline__ double dlog1p<double>(double x) { return log1p(x); }

template <typename T>
__device__ __forceinline__ T det3(const T* F) {
  return F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
         F[6] * (F[1] * F[5] - F[4] * F[2]);
}

// cofactor matrix, column-major: C(i,j) = C[i + 3j]
template <typename T>
__device__ __forceinline__ void cof3(const T* F, T* C) {
  C[0] = F[4] * F[8] - F[7] * F[5];
  C[1] = F[6] * F[5] - F[3] * F[8];
  C[2] = F[3] * F[7] - F[6] * F[4];
  C[3] = F[7] * F[2] - F[1] * F[8];
  C[4] = F[0] * F[8] - F[6] * F[2];
  C[5] = F[6] * F[1] - F[0] * F[7];
  C[6] = F[1] * F[5] - F[4] * F[2];
  C[7] = F[3] * F[2] - F[0] * F[5];
  C[8] = F[0] * F[4] - F[3] * F[1];
}


// ---------------------------------------------------------------------------
static __constant__ int c_pi[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
static __constant__ int c_pj[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};

// nd: node ids; Du: displacement differences [u1-u0, u2-u0, u3-u0] (column-major, FP64);
// r64: the tet's FP64 rest record (Dm^-1, w, lambda, mu); rest: the same record in Real.
template <typename Real>
__device__ __forceinline__ void elem_blocks_core(const int (&nd)[4], const double (&Du)[9], const double* r64,
                                                 const Real* rest, int model, Real* out /* 90, stride 1 */) {
  // displacement gradient in FP64, then the element arithmetic in Real
  Real Hg[9];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      Hg[r + 3 * c] = (Real)(Du[r] * r64[0 + 3 * c] + Du[r + 3] * r64[1 + 3 * c] + Du[r + 6] * r64[2 + 3 * c]);
  Real R[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) R[k] = rest[k];
  Real F[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) F[k] = Hg[k];
  F[0] += (Real)1; F[4] += (Real)1; F[8] += (Real)1;
  const Real w = R[9], lam = R[10], mu = R[11];
  Real Bv[4][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    Bv[1][c] = R[0 + 3 * c];
    Bv[2][c] = R[1 + 3 * c];
    Bv[3][c] = R[2 + 3 * c];
    Bv[0][c] = -(Bv[1][c] + Bv[2][c] + Bv[3][c]);
  }
  Real u[4][3], beta, M[9], S[9];
  const bool stvk = model == 1;
  if (stvk) {
    Real E[9];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i)
        E[i + 3 * j] = (Real)0.5 * (Hg[i + 3 * j] + Hg[j + 3 * i] + Hg[3 * i] * Hg[3 * j] + Hg[1 + 3 * i] * Hg[1 + 3 * j] +
                                    Hg[2 + 3 * i] * Hg[2 + 3 * j]);
    Real trE = E[0] + E[4] + E[8];
#pragma unroll
    for (int k = 0; k < 9; ++k) S[k] = (Real)2 * mu * E[k];
    S[0] += lam * trE; S[4] += lam * trE; S[8] += lam * trE;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) M[i + 3 * j] = F[i] * F[j] + F[i + 3] * F[j + 3] + F[i + 6] * F[j + 6];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int m2 = 0; m2 < 3; ++m2) u[a][m2] = F[m2] * Bv[a][0] + F[m2 + 3] * Bv[a][1] + F[m2 + 6] * Bv[a][2];
    beta = mu;
  } else {
    Real C[9];
    cof3(F, C);
    const Real I2 = Hg[0] * Hg[4] - Hg[3] * Hg[1] + Hg[0] * Hg[8] - Hg[6] * Hg[2] + Hg[4] * Hg[8] - Hg[7] * Hg[5];
    const Real jm1 = Hg[0] + Hg[4] + Hg[8] + I2 + det3(Hg);  // J - 1
    const Real J = (Real)1 + jm1;
    const Real logJ2 = (jm1 > (Real)-1) ? (Real)2 * dlog1p<Real>(jm1) : dlog<Real>(J * J);
    Real invJ = (Real)1 / J;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int m2 = 0; m2 < 3; ++m2)
        u[a][m2] = (C[m2] * Bv[a][0] + C[m2 + 3] * Bv[a][1] + C[m2 + 6] * Bv[a][2]) * invJ;
    beta = mu - (Real)0.5 * lam * logJ2;
#pragma unroll
    for (int k = 0; k < 9; ++k) { M[k] = 0; S[k] = 0; }
  }
#pragma unroll
  for (int p = 0; p < 10; ++p) {
    const int li = c_pi[p], lj = c_pj[p];
    const int n = (nd[li] >= nd[lj]) ? li : lj;
    const int q = (nd[li] >= nd[lj]) ? lj : li;
    const Real bb = Bv[n][0] * Bv[q][0] + Bv[n][1] * Bv[q][1] + Bv[n][2] * Bv[q][2];
    Real s, tt;
    if (stvk) {
      Real SBq[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) SBq[r] = S[r] * Bv[q][0] + S[r + 3] * Bv[q][1] + S[r + 6] * Bv[q][2];
      s = Bv[n][0] * SBq[0] + Bv[n][1] * SBq[1] + Bv[n][2] * SBq[2];
      tt = mu * bb;
    } else {
      s = mu * bb;
      tt = 0;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        Real val = lam * u[n][a] * u[q][b] + beta * u[q][a] * u[n][b] + tt * M[a + 3 * b];
        if (a == b) val += s;
        out[p * 9 + a * 3 + b] = val * w;
      }
  }
}


}  // namespace phx
