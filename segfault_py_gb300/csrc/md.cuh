// md.cuh -- McMurchie-Davidson electron-repulsion integrals (second engine).
//
// Reference: module mmd of src/hf/core/core.f90 -- boys (:23-28),
// hermite_gauss_e (:30-61), coulomb_auxiliary_r (:64-97), eri_3d (:100-165)
// and the contraction eri (:167-198); the same maths as src/hf/mmd.py.  For a
// primitive quartet with bra pair p = a + b, centre P, ket pair q, centre Q,
// rho = pq/(p+q), T = rho |P-Q|^2:
//
//   (ab|cd) = 2 pi^{5/2} / (p q sqrt(p+q)) c_a c_b c_c c_d
//             sum_{tuv} E^{ab}_t E^{ab}_u E^{ab}_v
//             sum_{tau nu phi} (-1)^{tau+nu+phi} E^{cd}_tau E^{cd}_nu E^{cd}_phi
//             R_{t+tau, u+nu, v+phi}(rho, P-Q)
//
// with E^{ij}_t the Hermite expansion coefficients of one direction (built by
// the two-term recursions, E^{00}_0 = 1: the Gaussian product factor
// exp(-ab/p |AB|^2) lives in the pair record's K~ with the coefficients and
// the sqrt(2) pi^{5/4}/p of the prefactor) and R_{tuv} = R^0_{tuv} from
// R^n_{000} = (-2 rho)^n F_n(T) and the Hermite Coulomb recursion
//   R^n_{t+1,u,v} = t R^{n+1}_{t-1,u,v} + X_PQ R^{n+1}_{t,u,v}  (likewise u, v).
//
// The integral is evaluated in two contractions: the ket one on the CUDA
// cores, G^{cd}_{tuv} = sum (-1)^.. E^{cd} R (per primitive quartet), and the
// bra Hermite-to-Cartesian one (ab|cd) = sum_p sum_tuv E^{ab,p}_{tuv} W_p,tuv
// with W_p = sum_q prefactor G^{cd} (md_eri.cu).
#pragma once
#include "quartet.cuh"

namespace sf {

// number of Hermite functions t+u+v <= L and the index of (t,u,v) in the
// order t descending blocks: idx(t,u,v) = off(L, t+u+v) + ...; a simple
// compile-time enumeration is used instead
__host__ __device__ constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// Hermite triple of index h in the enumeration: for n = 0..L, t = n..0,
// u = n-t..0, v = n-t-u
__host__ __device__ constexpr int herm_t(int h) {
  int k = 0;
  for (int n = 0;; ++n)
    for (int t = n; t >= 0; --t)
      for (int u = n - t; u >= 0; --u) {
        if (k == h) return t;
        ++k;
      }
}
__host__ __device__ constexpr int herm_u(int h) {
  int k = 0;
  for (int n = 0;; ++n)
    for (int t = n; t >= 0; --t)
      for (int u = n - t; u >= 0; --u) {
        if (k == h) return u;
        ++k;
      }
}
__host__ __device__ constexpr int herm_v(int h) {
  int k = 0;
  for (int n = 0;; ++n)
    for (int t = n; t >= 0; --t)
      for (int u = n - t; u >= 0; --u) {
        if (k == h) return n - t - u;
        ++k;
      }
}
__host__ __device__ constexpr int herm_index(int t, int u, int v) {
  const int n = t + u + v;
  int k = nherm(n - 1 < 0 ? -1 : n - 1);
  if (n == 0) k = 0;
  for (int tt = n; tt > t; --tt) k += n - tt + 1;
  return k + (n - t - u);
}

// F_m(T), m = 0..M (series + downward recursion below T = 30, asymptotic F_0
// + upward recursion above; the same forms as the one-electron kernels)
template <int M, typename R>
__device__ __forceinline__ void md_boys(R T, R (&F)[M + 1]) {
  if (T < (R)30) {
    const R e = exp(-T);
    R term = (R)1 / (R)(2 * M + 1), sum = term;
    const R eps = sizeof(R) == 4 ? (R)1e-8 : (R)1e-17;
    for (int i = 1; i < 120; ++i) {
      term *= (R)2 * T / (R)(2 * M + 2 * i + 1);
      sum += term;
      if (term < eps * sum) break;
    }
    F[M] = e * sum;
#pragma unroll
    for (int m = M - 1; m >= 0; --m) F[m] = ((R)2 * T * F[m + 1] + e) / (R)(2 * m + 1);
  } else {
    const R e = exp(-T);
    F[0] = (R)0.5 * sqrt((R)3.14159265358979323846 / T);
#pragma unroll
    for (int m = 0; m < M; ++m) F[m + 1] = ((R)(2 * m + 1) * F[m] - e) / ((R)2 * T);
  }
}

// E[i][j][t] of one direction for i <= LI, j <= LJ (E^{00}_0 = 1)
template <int LI, int LJ, typename R>
__device__ __forceinline__ void md_hermite_e(R i2p, R xpa, R xpb, R (&E)[LI + 1][LJ + 1][LI + LJ + 1]) {
#pragma unroll
  for (int i = 0; i <= LI; ++i)
#pragma unroll
    for (int j = 0; j <= LJ; ++j)
#pragma unroll
      for (int t = 0; t <= LI + LJ; ++t) E[i][j][t] = (R)0;
  E[0][0][0] = (R)1;
#pragma unroll
  for (int i = 0; i < LI; ++i)
#pragma unroll
    for (int t = 0; t <= i + 1; ++t)
      E[i + 1][0][t] = (t > 0 ? i2p * E[i][0][t - 1] : (R)0) + xpa * E[i][0][t] +
                       (t + 1 <= i ? (R)(t + 1) * E[i][0][t + 1] : (R)0);
#pragma unroll
  for (int i = 0; i <= LI; ++i)
#pragma unroll
    for (int j = 0; j < LJ; ++j)
#pragma unroll
      for (int t = 0; t <= i + j + 1; ++t)
        E[i][j + 1][t] = (t > 0 ? i2p * E[i][j][t - 1] : (R)0) + xpb * E[i][j][t] +
                         (t + 1 <= i + j ? (R)(t + 1) * E[i][j][t + 1] : (R)0);
}

// Hermite triples of the enumeration and the inverse map, for t+u+v <= 8
// (filled by prepare_md on the host; constant memory of the MD kernels)
constexpr int kMdMaxL = 8;
struct MdTables {
  unsigned char t[nherm(kMdMaxL)], u[nherm(kMdMaxL)], v[nherm(kMdMaxL)];
  short idx[kMdMaxL + 1][kMdMaxL + 1][kMdMaxL + 1];
};

// R_{tuv} (= R^0) for t+u+v <= L into Rh[nherm(L)] (enumeration above);
// runtime loops over the Hermite index (the MD kernels are the cross-check
// engine: compact code over unrolled speed)
template <int L, typename R>
__device__ __forceinline__ void md_coulomb_r(const MdTables &tb, R rho, R T, R X, R Y, R Z, R *Rh) {
  R F[L + 1];
  md_boys<L, R>(T, F);
  R Rn[L + 1][nherm(L)];
  R f = (R)1;
#pragma unroll
  for (int n = 0; n <= L; ++n) {
    Rn[n][0] = f * F[n];
    f *= (R)-2 * rho;
  }
#pragma unroll 1
  for (int n = L - 1; n >= 0; --n) {
#pragma unroll 1
    for (int h = 1; h < nherm(L - n); ++h) {
      const int t = tb.t[h], u = tb.u[h], v = tb.v[h];
      R r;
      if (t > 0) r = (t > 1 ? (R)(t - 1) * Rn[n + 1][tb.idx[t - 2][u][v]] : (R)0) + X * Rn[n + 1][tb.idx[t - 1][u][v]];
      else if (u > 0) r = (u > 1 ? (R)(u - 1) * Rn[n + 1][tb.idx[t][u - 2][v]] : (R)0) + Y * Rn[n + 1][tb.idx[t][u - 1][v]];
      else r = (v > 1 ? (R)(v - 1) * Rn[n + 1][tb.idx[t][u][v - 2]] : (R)0) + Z * Rn[n + 1][tb.idx[t][u][v - 1]];
      Rn[n][h] = r;
    }
  }
#pragma unroll 1
  for (int h = 0; h < nherm(L); ++h) Rh[h] = Rn[0][h];
}

}  // namespace sf
