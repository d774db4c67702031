// oneint.cu -- one-electron matrices S, T, V on the GPU.
//
// Reference: src/hf/mmd2.py:14-84 (Fortran E coefficients per primitive pair)
// and src/hf/mmd.py:13-141, called per AO pair and per nucleus at
// src/hf/hf.py:266-274.  Here one thread evaluates the whole Cartesian block
// of one ordered shell pair (a, b):
//   E^{ij}_t  Hermite expansion coefficients (McMurchie-Davidson), built by
//             the two-term recursions in i and j (mmd.py:13-30 in closed form:
//             E^{i+1,j}_t = E^{ij}_{t-1}/(2p) + X_PA E^{ij}_t + (t+1) E^{ij}_{t+1})
//   S = E0 E0 E0 (pi/p)^{3/2}                       (mmd.py:32-39)
//   T = b(2 lb + 3) S - 2 b^2 sum S(lb+2) - 1/2 sum lb(lb-1) S(lb-2) (mmd.py:49-60)
//   V = -Z sum_tuv E_t E_u E_v R_tuv(p, P-C) 2 pi / p  (mmd.py:110-133)
// R_tuv by the Hermite Coulomb recursion of mmd.py:70-108 / core.f90:64-97,
// evaluated bottom-up, with the Boys function F_n(T) written from its series
// (small T) and asymptotic form with upward recursion (large T).
#include <cmath>

#include "launch.h"

namespace sf {

constexpr int kOneMaxL = 2;
constexpr int kOneMaxN = 2 * kOneMaxL;      // Boys orders needed by V

// F_n(T) for n = 0..nmax (nmax <= 8)
__device__ void boys_array(int nmax, double T, double *F) {
  if (T < 30.0) {
    // F_nmax = e^{-T} sum_i (2T)^i / ((2n+1)(2n+3)...(2n+2i+1)), then downward
    // F_m = (2T F_{m+1} + e^{-T}) / (2m+1)
    const double e = exp(-T);
    double term = 1.0 / (2.0 * nmax + 1.0), sum = term;
    for (int i = 1; i < 200; ++i) {
      term *= 2.0 * T / (2.0 * nmax + 2.0 * i + 1.0);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    F[nmax] = e * sum;
    for (int m = nmax - 1; m >= 0; --m) F[m] = (2.0 * T * F[m + 1] + e) / (2.0 * m + 1.0);
  } else {
    // F_0 = sqrt(pi/T)/2 (erfc(sqrt T) < 1e-14 here), F_{m+1} = ((2m+1) F_m - e^{-T}) / (2T)
    const double e = exp(-T);
    F[0] = 0.5 * sqrt(3.14159265358979323846 / T);
    for (int m = 0; m < nmax; ++m) F[m + 1] = ((2.0 * m + 1.0) * F[m] - e) / (2.0 * T);
  }
}

// E[i][j][t] for i <= LI, j <= LJ, t <= i+j along one direction
template <int LI, int LJ>
__device__ __forceinline__ void hermite_e(double p, double xpa, double xpb, double e0,
                                          double (&E)[LI + 1][LJ + 1][LI + LJ + 1]) {
#pragma unroll
  for (int i = 0; i <= LI; ++i)
#pragma unroll
    for (int j = 0; j <= LJ; ++j)
#pragma unroll
      for (int t = 0; t <= LI + LJ; ++t) E[i][j][t] = 0.0;
  const double h = 0.5 / p;
  E[0][0][0] = e0;
#pragma unroll
  for (int i = 0; i < LI; ++i)
#pragma unroll
    for (int t = 0; t <= i + 1; ++t)
      E[i + 1][0][t] = (t > 0 ? h * E[i][0][t - 1] : 0.0) + xpa * E[i][0][t] + (t + 1 <= i ? (t + 1) * E[i][0][t + 1] : 0.0);
#pragma unroll
  for (int i = 0; i <= LI; ++i)
#pragma unroll
    for (int j = 0; j < LJ; ++j)
#pragma unroll
      for (int t = 0; t <= i + j + 1; ++t)
        E[i][j + 1][t] = (t > 0 ? h * E[i][j][t - 1] : 0.0) + xpb * E[i][j][t] +
                         (t + 1 <= i + j ? (t + 1) * E[i][j][t + 1] : 0.0);
}


template <int LA, int LB>
__device__ void one_pair(const OneParams &P, int a, int b) {
  constexpr int NA = ncart(LA), NB = ncart(LB);
  const double A[3] = {P.sh.cx[a], P.sh.cy[a], P.sh.cz[a]};
  const double B[3] = {P.sh.cx[b], P.sh.cy[b], P.sh.cz[b]};
  const double AB2 = (A[0] - B[0]) * (A[0] - B[0]) + (A[1] - B[1]) * (A[1] - B[1]) + (A[2] - B[2]) * (A[2] - B[2]);
  double s[NA][NB], k[NA][NB], v[NA][NB];
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) s[i][j] = k[i][j] = v[i][j] = 0.0;
  const double pi = 3.14159265358979323846;
  for (int ia = P.poff[a]; ia < P.poff[a + 1]; ++ia) {
    for (int ib = P.poff[b]; ib < P.poff[b + 1]; ++ib) {
      const double al = P.exps[ia], be = P.exps[ib], p = al + be, mu = al * be / p;
      const double cc = P.coefs[ia] * P.coefs[ib];
      double Pc[3], E[3][LA + 1][LB + 3][LA + LB + 3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Pc[d] = (al * A[d] + be * B[d]) / p;
        const double X = A[d] - B[d];
        hermite_e<LA, LB + 2>(p, Pc[d] - A[d], Pc[d] - B[d], exp(-mu * X * X), E[d]);
      }
      const double sp = pow(pi / p, 1.5);
      // overlap and kinetic
#pragma unroll
      for (int i = 0; i < NA; ++i)
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          const int ax = cart_e(LA, i, 0), ay = cart_e(LA, i, 1), az = cart_e(LA, i, 2);
          const int bx = cart_e(LB, j, 0), by = cart_e(LB, j, 1), bz = cart_e(LB, j, 2);
          const double sx = E[0][ax][bx][0], sy = E[1][ay][by][0], sz = E[2][az][bz][0];
          const double s0 = sx * sy * sz * sp;
          double t = be * (2 * (bx + by + bz) + 3) * s0;
          t -= 2.0 * be * be * sp * (E[0][ax][bx + 2][0] * sy * sz + sx * E[1][ay][by + 2][0] * sz + sx * sy * E[2][az][bz + 2][0]);
          if (bx >= 2) t -= 0.5 * bx * (bx - 1) * sp * E[0][ax][bx - 2][0] * sy * sz;
          if (by >= 2) t -= 0.5 * by * (by - 1) * sp * sx * E[1][ay][by - 2][0] * sz;
          if (bz >= 2) t -= 0.5 * bz * (bz - 1) * sp * sx * sy * E[2][az][bz - 2][0];
          s[i][j] += cc * s0;
          k[i][j] += cc * t;
        }
      // nuclear attraction
      if (P.V) {
        for (int at = 0; at < P.natom; ++at) {
          const double Cc[3] = {P.atom_xyz[3 * at], P.atom_xyz[3 * at + 1], P.atom_xyz[3 * at + 2]};
          const double pc[3] = {Pc[0] - Cc[0], Pc[1] - Cc[1], Pc[2] - Cc[2]};
          const double Tb = p * (pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
          constexpr int L = LA + LB;
          double F[L + 1];
          boys_array(L, Tb, F);
          // R^n_{tuv} bottom-up: R[n][t][u][v] for t+u+v <= L-n
          double R[L + 1][L + 1][L + 1][L + 1];
          for (int n = 0; n <= L; ++n) {
            double f = F[n];
            for (int m = 0; m < n; ++m) f *= -2.0 * p;
            R[n][0][0][0] = f;
          }
          for (int n = L - 1; n >= 0; --n) {
            for (int t = 0; t <= L - n; ++t)
              for (int u = 0; u <= L - n - t; ++u)
                for (int w = 0; w <= L - n - t - u; ++w) {
                  if (t + u + w == 0) continue;
                  double r;
                  if (t > 0) r = (t > 1 ? (t - 1) * R[n + 1][t - 2][u][w] : 0.0) + pc[0] * R[n + 1][t - 1][u][w];
                  else if (u > 0) r = (u > 1 ? (u - 1) * R[n + 1][t][u - 2][w] : 0.0) + pc[1] * R[n + 1][t][u - 1][w];
                  else r = (w > 1 ? (w - 1) * R[n + 1][t][u][w - 2] : 0.0) + pc[2] * R[n + 1][t][u][w - 1];
                  R[n][t][u][w] = r;
                }
          }
          const double pre = -P.charges[at] * 2.0 * pi / p;
#pragma unroll
          for (int i = 0; i < NA; ++i)
#pragma unroll
            for (int j = 0; j < NB; ++j) {
              const int ax = cart_e(LA, i, 0), ay = cart_e(LA, i, 1), az = cart_e(LA, i, 2);
              const int bx = cart_e(LB, j, 0), by = cart_e(LB, j, 1), bz = cart_e(LB, j, 2);
              double acc = 0.0;
#pragma unroll
              for (int t = 0; t <= ax + bx; ++t)
#pragma unroll
                for (int u = 0; u <= ay + by; ++u)
#pragma unroll
                  for (int w = 0; w <= az + bz; ++w)
                    acc += E[0][ax][bx][t] * E[1][ay][by][u] * E[2][az][bz][w] * R[0][t][u][w];
              v[i][j] += cc * pre * acc;
            }
        }
      }
    }
  }
  const int a0 = P.sh.ao[a], b0 = P.sh.ao[b];
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const double nrm = cart_norm(LA, i) * cart_norm(LB, j);
      const int idx = (a0 + i) * P.nao + b0 + j;
      if (P.S) P.S[idx] = s[i][j] * nrm;
      if (P.T) P.T[idx] = k[i][j] * nrm;
      if (P.V) P.V[idx] = v[i][j] * nrm;
    }
}

__global__ void one_electron_kernel(OneParams P) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= P.nshell * P.nshell) return;
  const int a = idx / P.nshell, b = idx % P.nshell;
  const int la = P.sh.l[a], lb = P.sh.l[b];
  switch (la * 3 + lb) {
    case 0: one_pair<0, 0>(P, a, b); break;
    case 1: one_pair<0, 1>(P, a, b); break;
    case 2: one_pair<0, 2>(P, a, b); break;
    case 3: one_pair<1, 0>(P, a, b); break;
    case 4: one_pair<1, 1>(P, a, b); break;
    case 5: one_pair<1, 2>(P, a, b); break;
    case 6: one_pair<2, 0>(P, a, b); break;
    case 7: one_pair<2, 1>(P, a, b); break;
    case 8: one_pair<2, 2>(P, a, b); break;
    default: break;
  }
}

cudaError_t launch_one_electron(const OneParams &P, cudaStream_t st) {
  const int n = P.nshell * P.nshell;
  one_electron_kernel<<<(n + 63) / 64, 64, 0, st>>>(P);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Gradient of E1 = sum_ij D_ij (T_ij + V_ij) - W_ij S_ij.  With D, W and the
// operators symmetric, d/dR sum_ij D_ij O_ij = 2 sum_ij D_ij <d phi_i/dR|O|phi_j>,
// so one thread per ordered shell pair (a, b) differentiates the bra function
// only, d phi_a / dA = 2 alpha phi_{a+1} - a phi_{a-1}, and counts it twice.
// V also depends on the nucleus C: by translational invariance of
// <a|1/r_C|b>, dV/dC = -(dV/dA + dV/dB), which over all ordered pairs is
// -2 sum_ij D_ij <d phi_i/dA|1/r_C|phi_j>.
// ---------------------------------------------------------------------------
template <int LA, int LB>
__device__ void one_pair_grad(const OneParams &P, const double *Dm, const double *Wm, double *grad, int a, int b,
                              int which) {
  constexpr int NA = ncart(LA), NB = ncart(LB);
  constexpr int LE = LA + 1;                 // bra shifted up by one
  constexpr int L = LA + LB + 1;
  const double pi = 3.14159265358979323846;
  const double A[3] = {P.sh.cx[a], P.sh.cy[a], P.sh.cz[a]};
  const double B[3] = {P.sh.cx[b], P.sh.cy[b], P.sh.cz[b]};
  const int a0 = P.sh.ao[a], b0 = P.sh.ao[b], n = P.nao;
  double Dab[NA][NB], Wab[NA][NB];
  for (int i = 0; i < NA; ++i)
    for (int j = 0; j < NB; ++j) {
      const double nrm = cart_norm(LA, i) * cart_norm(LB, j);
      Dab[i][j] = Dm[(a0 + i) * n + b0 + j] * nrm;
      Wab[i][j] = Wm[(a0 + i) * n + b0 + j] * nrm;
    }
  double gA[3] = {0.0, 0.0, 0.0};
  double E[3][LE + 1][LB + 3][LE + LB + 3];
  // which == natom: overlap and kinetic (Pulay term -W dS and D dT);
  // which < natom: nuclear attraction of nucleus 'which'
  if (which == P.natom)
  for (int ia = P.poff[a]; ia < P.poff[a + 1]; ++ia)
    for (int ib = P.poff[b]; ib < P.poff[b + 1]; ++ib) {
      const double al = P.exps[ia], be = P.exps[ib], p = al + be, mu = al * be / p;
      const double cc = P.coefs[ia] * P.coefs[ib];
      for (int d = 0; d < 3; ++d) {
        const double Pd = (al * A[d] + be * B[d]) / p, X = A[d] - B[d];
        hermite_e<LE, LB + 2>(p, Pd - A[d], Pd - B[d], exp(-mu * X * X), E[d]);
      }
      const double sp = pow(pi / p, 1.5);
      for (int i = 0; i < NA; ++i)
        for (int j = 0; j < NB; ++j) {
          const int bx[3] = {cart_e(LB, j, 0), cart_e(LB, j, 1), cart_e(LB, j, 2)};
          for (int d = 0; d < 3; ++d) {
            double dS = 0.0, dT = 0.0;
            for (int sgn = 0; sgn < 2; ++sgn) {
              int ax[3] = {cart_e(LA, i, 0), cart_e(LA, i, 1), cart_e(LA, i, 2)};
              const int ad = ax[d];
              if (sgn == 1 && ad == 0) continue;
              ax[d] += sgn == 0 ? 1 : -1;
              const double f = sgn == 0 ? 2.0 * al : -(double)ad;
              const double sx = E[0][ax[0]][bx[0]][0], sy = E[1][ax[1]][bx[1]][0], sz = E[2][ax[2]][bx[2]][0];
              const double s0 = sx * sy * sz * sp;
              double t = be * (2 * (bx[0] + bx[1] + bx[2]) + 3) * s0;
              t -= 2.0 * be * be * sp *
                   (E[0][ax[0]][bx[0] + 2][0] * sy * sz + sx * E[1][ax[1]][bx[1] + 2][0] * sz +
                    sx * sy * E[2][ax[2]][bx[2] + 2][0]);
              if (bx[0] >= 2) t -= 0.5 * bx[0] * (bx[0] - 1) * sp * E[0][ax[0]][bx[0] - 2][0] * sy * sz;
              if (bx[1] >= 2) t -= 0.5 * bx[1] * (bx[1] - 1) * sp * sx * E[1][ax[1]][bx[1] - 2][0] * sz;
              if (bx[2] >= 2) t -= 0.5 * bx[2] * (bx[2] - 1) * sp * sx * sy * E[2][ax[2]][bx[2] - 2][0];
              dS += f * s0;
              dT += f * t;
            }
            gA[d] += cc * (Dab[i][j] * dT - Wab[i][j] * dS);
          }
        }
    }
  // nuclear attraction of one nucleus
  for (int at = which; at < P.natom && at == which; ++at) {
    const double Cc[3] = {P.atom_xyz[3 * at], P.atom_xyz[3 * at + 1], P.atom_xyz[3 * at + 2]};
    double gC[3] = {0.0, 0.0, 0.0};
    for (int ia = P.poff[a]; ia < P.poff[a + 1]; ++ia)
      for (int ib = P.poff[b]; ib < P.poff[b + 1]; ++ib) {
        const double al = P.exps[ia], be = P.exps[ib], p = al + be, mu = al * be / p;
        const double cc = P.coefs[ia] * P.coefs[ib];
        double Pc[3];
        for (int d = 0; d < 3; ++d) {
          Pc[d] = (al * A[d] + be * B[d]) / p;
          const double X = A[d] - B[d];
          hermite_e<LE, LB + 2>(p, Pc[d] - A[d], Pc[d] - B[d], exp(-mu * X * X), E[d]);
        }
        const double pc[3] = {Pc[0] - Cc[0], Pc[1] - Cc[1], Pc[2] - Cc[2]};
        double F[L + 1];
        boys_array(L, p * (pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]), F);
        double R[L + 1][L + 1][L + 1][L + 1];
        for (int m = 0; m <= L; ++m) {
          double f = F[m];
          for (int k = 0; k < m; ++k) f *= -2.0 * p;
          R[m][0][0][0] = f;
        }
        for (int m = L - 1; m >= 0; --m)
          for (int t = 0; t <= L - m; ++t)
            for (int u = 0; u <= L - m - t; ++u)
              for (int w = 0; w <= L - m - t - u; ++w) {
                if (t + u + w == 0) continue;
                double r;
                if (t > 0) r = (t > 1 ? (t - 1) * R[m + 1][t - 2][u][w] : 0.0) + pc[0] * R[m + 1][t - 1][u][w];
                else if (u > 0) r = (u > 1 ? (u - 1) * R[m + 1][t][u - 2][w] : 0.0) + pc[1] * R[m + 1][t][u - 1][w];
                else r = (w > 1 ? (w - 1) * R[m + 1][t][u][w - 2] : 0.0) + pc[2] * R[m + 1][t][u][w - 1];
                R[m][t][u][w] = r;
              }
        const double pre = -P.charges[at] * 2.0 * pi / p * cc;
        for (int i = 0; i < NA; ++i)
          for (int j = 0; j < NB; ++j) {
            const int bx[3] = {cart_e(LB, j, 0), cart_e(LB, j, 1), cart_e(LB, j, 2)};
            for (int d = 0; d < 3; ++d) {
              double dV = 0.0;
              for (int sgn = 0; sgn < 2; ++sgn) {
                int ax[3] = {cart_e(LA, i, 0), cart_e(LA, i, 1), cart_e(LA, i, 2)};
                const int ad = ax[d];
                if (sgn == 1 && ad == 0) continue;
                ax[d] += sgn == 0 ? 1 : -1;
                const double f = sgn == 0 ? 2.0 * al : -(double)ad;
                double acc = 0.0;
                for (int t = 0; t <= ax[0] + bx[0]; ++t)
                  for (int u = 0; u <= ax[1] + bx[1]; ++u)
                    for (int w = 0; w <= ax[2] + bx[2]; ++w)
                      acc += E[0][ax[0]][bx[0]][t] * E[1][ax[1]][bx[1]][u] * E[2][ax[2]][bx[2]][w] * R[0][t][u][w];
                dV += f * acc;
              }
              const double v = Dab[i][j] * pre * dV;
              gA[d] += v;
              gC[d] -= v;
            }
          }
      }
    for (int d = 0; d < 3; ++d) atomicAdd(grad + 3 * at + d, 2.0 * gC[d]);
  }
  const int at_a = P.sh.atom[a];
  for (int d = 0; d < 3; ++d) atomicAdd(grad + 3 * at_a + d, 2.0 * gA[d]);
}

// one thread per (ordered shell pair, nucleus or the S/T part); the
// contributions of a CTA are summed in shared memory (3 slots per atom) and
// written with one atomic per slot, because all threads add into the same
// 3*natom words
constexpr int kOneGradSmemAtoms = 512;

__global__ void one_electron_grad_kernel(OneParams P, const double *D, const double *W, double *grad) {
  extern __shared__ double sgrad[];
  const bool cta_sum = P.natom <= kOneGradSmemAtoms;
  if (cta_sum) {
    for (int i = threadIdx.x; i < 3 * P.natom; i += blockDim.x) sgrad[i] = 0.0;
    __syncthreads();
  }
  double *out = cta_sum ? sgrad : grad;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t npair = (int64_t)P.nshell * P.nshell;
  if (idx < npair * (P.natom + 1)) {
    const int which = (int)(idx / npair);
    const int ab = (int)(idx % npair);
    const int a = ab / P.nshell, b = ab % P.nshell;
    switch (P.sh.l[a] * 3 + P.sh.l[b]) {
      case 0: one_pair_grad<0, 0>(P, D, W, out, a, b, which); break;
      case 1: one_pair_grad<0, 1>(P, D, W, out, a, b, which); break;
      case 2: one_pair_grad<0, 2>(P, D, W, out, a, b, which); break;
      case 3: one_pair_grad<1, 0>(P, D, W, out, a, b, which); break;
      case 4: one_pair_grad<1, 1>(P, D, W, out, a, b, which); break;
      case 5: one_pair_grad<1, 2>(P, D, W, out, a, b, which); break;
      case 6: one_pair_grad<2, 0>(P, D, W, out, a, b, which); break;
      case 7: one_pair_grad<2, 1>(P, D, W, out, a, b, which); break;
      case 8: one_pair_grad<2, 2>(P, D, W, out, a, b, which); break;
      default: break;
    }
  }
  if (cta_sum) {
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * P.natom; i += blockDim.x)
      if (sgrad[i] != 0.0) atomicAdd(grad + i, sgrad[i]);
  }
}

cudaError_t launch_one_electron_grad(const OneParams &P, const double *D, const double *W, double *grad,
                                     cudaStream_t st) {
  const int64_t n = (int64_t)P.nshell * P.nshell * (P.natom + 1);
  const size_t smem = P.natom <= kOneGradSmemAtoms ? 3 * (size_t)P.natom * sizeof(double) : 0;
  one_electron_grad_kernel<<<(unsigned)((n + 127) / 128), 128, smem, st>>>(P, D, W, grad);
  return cudaGetLastError();
}

}  // namespace sf
