// oneint.cu -- one-electron matrices S, T, V on the GPU.
//
// Reference: src/hf/mmd2.py:14-84 (Fortran E coefficients per primitive pair)
// and src/hf/mmd.py:13-141, called per AO pair and per nucleus at
// src/hf/hf.py:266-274.  Here one CTA evaluates the whole Cartesian block of
// one canonical shell pair (a >= b) and writes it and its transpose:
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


// One CTA (kOneThreads threads) per canonical shell pair (a >= b); the
// block of (a, b) is written, and for a != b also its transpose as the block
// of (b, a) (S, T and V are symmetric).  Per primitive pair:
//  * E coefficients along x, y, z (bra to LA, ket to LB+2 for the kinetic
//    shifts) into shared memory, one direction per thread;
//  * S and T of Cartesian entry (i, j) on thread i*NB + j;
//  * V = 2 pi / p c_i c_j sum_tuv E E E S_tuv with S_tuv = sum_C -Z_C R_tuv
//    (V is linear in R): every thread takes nuclei C = t, t+kOneThreads, ...,
//    Boys values, R_tuv by the Hermite Coulomb recursion in place (level n
//    overwrites t+u+v = L-n .. 1 from the top down, then R^n_000) and adds
//    -Z_C R_tuv to its part of S_tuv; S is summed over the CTA (shuffles,
//    then the two warps) and thread i*NB + j contracts it with its E's.
// Primitive pairs whose contributions all stay below 1e-17 are skipped (the
// product Gaussian c_i c_j exp(-mu |AB|^2) (pi/p)^3/2 bounds the overlap,
// E coefficients grow at most as (|AB| + 1/sqrt(p) + 1)^L, kinetic terms as
// 3 beta (LB + 2) and attraction as 2 sqrt(p/pi) times the summed charge).
constexpr int kOneThreads = 64;

// Hermite triples t+u+v <= L, enumerated t, then u, then v ascending
__host__ __device__ constexpr int ntuv(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int tuv_index(int L, int t, int u, int v) {
  int k = 0;
  for (int t2 = 0; t2 < t; ++t2) k += (L - t2 + 1) * (L - t2 + 2) / 2;
  for (int u2 = 0; u2 < u; ++u2) k += L - t - u2 + 1;
  return k + v;
}

template <int LA, int LB>
constexpr int one_smem() {
  return 3 * (LA + 1) * (LB + 3) * (LA + LB + 3) + 2 * ntuv(LA + LB) + 2;
}
constexpr int kOneSmem = one_smem<2, 2>();   // the largest

template <int LA, int LB>
__device__ void one_pair(const OneParams &P, int a, int b, double *smem) {
  constexpr int NA = ncart(LA), NB = ncart(LB), L = LA + LB;
  constexpr int EN = (LA + 1) * (LB + 3) * (LA + LB + 3);
  using EArr = double[LA + 1][LB + 3][LA + LB + 3];
  EArr *E = reinterpret_cast<EArr *>(smem);
  constexpr int NT = ntuv(L);
  double *sred = smem + 3 * EN;              // [2 warps][NT]: S_tuv partial sums
  double *zred = smem + 3 * EN + 2 * NT;
  static_assert(3 * EN + 2 * NT + 2 == one_smem<LA, LB>(), "smem layout");
  const double pi = 3.14159265358979323846;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double A[3] = {P.sh.cx[a], P.sh.cy[a], P.sh.cz[a]};
  const double B[3] = {P.sh.cx[b], P.sh.cy[b], P.sh.cz[b]};
  double R2 = 0.0;
  for (int d = 0; d < 3; ++d) R2 += (A[d] - B[d]) * (A[d] - B[d]);
  double zs = 0.0;
  if (P.V)
    for (int k = tid; k < P.natom; k += blockDim.x) zs += fabs(P.charges[k]);
  for (int off = 16; off > 0; off >>= 1) zs += __shfl_xor_sync(0xffffffffu, zs, off);
  if (lane == 0) zred[warp] = zs;
  __syncthreads();
  zs = zred[0] + zred[1];
  const int ti = tid / NB, tj = tid % NB;   // this thread's S/T entry (tid < NA*NB)
  double s_acc = 0.0, t_acc = 0.0, v_acc = 0.0;
  for (int ia = P.poff[a]; ia < P.poff[a + 1]; ++ia)
    for (int ib = P.poff[b]; ib < P.poff[b + 1]; ++ib) {
      const double al = P.exps[ia], be = P.exps[ib], p = al + be, mu = al * be / p;
      const double cc = P.coefs[ia] * P.coefs[ib];
      const double sp = pow(pi / p, 1.5);
      {
        const double g = fabs(cc) * exp(-mu * R2) * sp;
        const double e = pow(sqrt(R2) + rsqrt(p) + 1.0, (double)L);
        const double f = 1.0 + 2.0 * sqrt(p / pi) * zs + 3.0 * be * (LB + 2);
        if (g * e * f < 1e-17) continue;   // uniform over the CTA
      }
      double Pc[3];
      for (int d = 0; d < 3; ++d) Pc[d] = (al * A[d] + be * B[d]) / p;
      __syncthreads();   // previous iteration done with E
      if (tid < 3) {
        const int d = tid;
        const double X = A[d] - B[d];
        double Et[LA + 1][LB + 3][LA + LB + 3];
        hermite_e<LA, LB + 2>(p, Pc[d] - A[d], Pc[d] - B[d], exp(-mu * X * X), Et);
        for (int i = 0; i <= LA; ++i)
          for (int j = 0; j <= LB + 2; ++j)
            for (int t = 0; t <= LA + LB + 2; ++t) E[d][i][j][t] = Et[i][j][t];
      }
      __syncthreads();
      if (tid < NA * NB) {   // overlap and kinetic
        const int ax = cart_e(LA, ti, 0), ay = cart_e(LA, ti, 1), az = cart_e(LA, ti, 2);
        const int bx = cart_e(LB, tj, 0), by = cart_e(LB, tj, 1), bz = cart_e(LB, tj, 2);
        const double sx = E[0][ax][bx][0], sy = E[1][ay][by][0], sz = E[2][az][bz][0];
        const double s0 = sx * sy * sz * sp;
        double t = be * (2 * (bx + by + bz) + 3) * s0;
        t -= 2.0 * be * be * sp *
             (E[0][ax][bx + 2][0] * sy * sz + sx * E[1][ay][by + 2][0] * sz + sx * sy * E[2][az][bz + 2][0]);
        if (bx >= 2) t -= 0.5 * bx * (bx - 1) * sp * E[0][ax][bx - 2][0] * sy * sz;
        if (by >= 2) t -= 0.5 * by * (by - 1) * sp * sx * E[1][ay][by - 2][0] * sz;
        if (bz >= 2) t -= 0.5 * bz * (bz - 1) * sp * sx * sy * E[2][az][bz - 2][0];
        s_acc += cc * s0;
        t_acc += cc * t;
      }
      if (P.V) {   // nuclear attraction, nuclei across threads
        double st[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) st[k] = 0.0;
        for (int at = tid; at < P.natom; at += blockDim.x) {
          const double pc[3] = {Pc[0] - P.atom_xyz[3 * at], Pc[1] - P.atom_xyz[3 * at + 1],
                                Pc[2] - P.atom_xyz[3 * at + 2]};
          double F[L + 1];
          boys_array(L, p * (pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]), F);
          double R[L + 1][L + 1][L + 1];
          double fm2p = 1.0;
#pragma unroll
          for (int n = 0; n < L; ++n) fm2p *= -2.0 * p;
          R[0][0][0] = F[L] * fm2p;
#pragma unroll
          for (int n = L - 1; n >= 0; --n) {
#pragma unroll
            for (int sl = L - n; sl >= 1; --sl)
#pragma unroll
              for (int t = 0; t <= sl; ++t)
#pragma unroll
                for (int u = 0; u <= sl - t; ++u) {
                  const int w = sl - t - u;
                  double r;
                  if (t > 0) r = (t > 1 ? (t - 1) * R[t - 2][u][w] : 0.0) + pc[0] * R[t - 1][u][w];
                  else if (u > 0) r = (u > 1 ? (u - 1) * R[t][u - 2][w] : 0.0) + pc[1] * R[t][u - 1][w];
                  else r = (w > 1 ? (w - 1) * R[t][u][w - 2] : 0.0) + pc[2] * R[t][u][w - 1];
                  R[t][u][w] = r;
                }
            fm2p /= -2.0 * p;
            R[0][0][0] = F[n] * fm2p;
          }
          const double z = -P.charges[at];
#pragma unroll
          for (int t = 0; t <= L; ++t)
#pragma unroll
            for (int u = 0; u <= L - t; ++u)
#pragma unroll
              for (int w = 0; w <= L - t - u; ++w) st[tuv_index(L, t, u, w)] += z * R[t][u][w];
        }
#pragma unroll
        for (int k = 0; k < NT; ++k) {
          double x = st[k];
          for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
          if (lane == 0) sred[warp * NT + k] = x;
        }
        __syncthreads();
        if (tid < NA * NB) {
          const int ax = cart_e(LA, ti, 0), ay = cart_e(LA, ti, 1), az = cart_e(LA, ti, 2);
          const int bx = cart_e(LB, tj, 0), by = cart_e(LB, tj, 1), bz = cart_e(LB, tj, 2);
          double acc = 0.0;
          for (int t = 0; t <= ax + bx; ++t)
            for (int u = 0; u <= ay + by; ++u)
              for (int w = 0; w <= az + bz; ++w) {
                const int k = tuv_index(L, t, u, w);
                acc += E[0][ax][bx][t] * E[1][ay][by][u] * E[2][az][bz][w] * (sred[k] + sred[NT + k]);
              }
          v_acc += 2.0 * pi / p * cc * acc;
        }
      }
    }
  if (tid < NA * NB) {
    const int a0 = P.sh.ao[a], b0 = P.sh.ao[b], n = P.nao;
    const double nrm = cart_norm(LA, ti) * cart_norm(LB, tj);
    const size_t ij = (size_t)(a0 + ti) * n + b0 + tj, ji = (size_t)(b0 + tj) * n + a0 + ti;
    const double vv = v_acc * nrm;
    if (P.S) P.S[ij] = s_acc * nrm;
    if (P.T) P.T[ij] = t_acc * nrm;
    if (P.V) P.V[ij] = vv;
    if (a != b) {
      if (P.S) P.S[ji] = s_acc * nrm;
      if (P.T) P.T[ji] = t_acc * nrm;
      if (P.V) P.V[ji] = vv;
    }
  }
}

// one CTA per canonical pair (a >= b): block k = a (a + 1) / 2 + b
__global__ void __launch_bounds__(kOneThreads) one_electron_kernel(OneParams P) {
  __shared__ __align__(16) double smem[kOneSmem];
  const int k = blockIdx.x;
  int a = (int)((sqrt(8.0 * k + 1.0) - 1.0) * 0.5);
  while (a * (a + 1) / 2 > k) --a;
  while ((a + 1) * (a + 2) / 2 <= k) ++a;
  const int b = k - a * (a + 1) / 2;
  switch (P.sh.l[a] * 3 + P.sh.l[b]) {
    case 0: one_pair<0, 0>(P, a, b, smem); break;
    case 1: one_pair<0, 1>(P, a, b, smem); break;
    case 2: one_pair<0, 2>(P, a, b, smem); break;
    case 3: one_pair<1, 0>(P, a, b, smem); break;
    case 4: one_pair<1, 1>(P, a, b, smem); break;
    case 5: one_pair<1, 2>(P, a, b, smem); break;
    case 6: one_pair<2, 0>(P, a, b, smem); break;
    case 7: one_pair<2, 1>(P, a, b, smem); break;
    case 8: one_pair<2, 2>(P, a, b, smem); break;
    default: break;
  }
}

cudaError_t launch_one_electron(const OneParams &P, cudaStream_t st) {
  const int n = P.nshell * (P.nshell + 1) / 2;
  if (n == 0) return cudaSuccess;
  one_electron_kernel<<<n, kOneThreads, 0, st>>>(P);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Gradient of E1 = sum_ij D_ij (T_ij + V_ij) - W_ij S_ij.  With D, W and the
// operators symmetric, d/dR sum_ij D_ij O_ij = 2 sum_ij D_ij <d phi_i/dR|O|phi_j>
// over ordered shell pairs; per canonical pair (a >= b) both the bra and the
// ket derivative are taken, d phi/dA = 2 alpha phi_{+1} - a phi_{-1}:
//  * S and T (two-centre): the ket derivative is minus the bra one;
//  * V: the bra and ket derivative share R_tuv(p, P - C) of each nucleus C,
//    which receives minus their sum (translational invariance of
//    <a|1/r_C|b>).
// CTA per canonical pair (a, b), 64 threads.  For every primitive pair whose
// bound (product Gaussian x block max of |D|, |W| x derivative, kinetic and
// attraction factors) is not below 1e-15:
//  * E coefficients (bra to LA+1, ket to LB+2) into shared memory;
//  * the S and T bra-derivative terms, one (i, j, direction) per thread;
//  * the density-contracted Hermite coefficients of the bra and the ket
//    derivative, M^d_tuv = 2pi/p c_i c_j sum_{i in a, j in b} D_ij sum_+- f
//    E.. E.. E.. (nucleus independent), cooperatively into shared memory;
//  * every thread takes nuclei C = t, t+64, ...: Boys values F_m(p |P-C|^2)
//    = sum_i w_i u_i^m from the FP64 Rys rule of floor(L/2)+1 points (exact
//    for m <= L), R_tuv by the Hermite Coulomb recursion, and
//    dV/dX_d = -Z_C sum_tuv M^d_tuv R_tuv.
constexpr int kOneGradThreads = 64;

// shared-memory doubles of one_pair_grad2<LA, LB>: E coefficients, the bra and
// ket Hermite coefficients MA, MB, the density block and the reduction rows
template <int LA, int LB>
constexpr int one_grad_smem() {
  return 3 * (LA + 2) * (LB + 3) * (LA + LB + 4) + 6 * (LA + LB + 2) * (LA + LB + 2) * (LA + LB + 2) +
         ncart(LA) * ncart(LB) + 6 * kOneGradThreads;
}
constexpr int kOneGradSmem = one_grad_smem<2, 2>();   // the largest

template <int LA, int LB>
__device__ void one_pair_grad2(const OneParams &P, const double *Dm, const double *Wm, double *grad, int a, int b,
                               double *smem) {
  constexpr int NA = ncart(LA), NB = ncart(LB);
  constexpr int LE = LA + 1, L = LA + LB + 1, NH = (L + 1) * (L + 1) * (L + 1);
  constexpr int NRT = L / 2 + 1;   // Rys points whose rule is exact for F_0 .. F_L
  constexpr int EN = (LE + 1) * (LB + 3) * (LE + LB + 3);
  const double pi = 3.14159265358979323846;
  // carved from the kernel's one shared buffer (each instantiation declaring
  // its own arrays made the kernel hold all nine sets, 79.5 KB)
  using EArr = double[LE + 1][LB + 3][LE + LB + 3];
  EArr *E = reinterpret_cast<EArr *>(smem);
  double(*MA)[NH] = reinterpret_cast<double(*)[NH]>(smem + 3 * EN);
  double(*MB)[NH] = MA + 3;
  double(*Dab)[NB] = reinterpret_cast<double(*)[NB]>(smem + 3 * EN + 6 * NH);
  double(*red)[6] = reinterpret_cast<double(*)[6]>(smem + 3 * EN + 6 * NH + NA * NB);
  static_assert(3 * EN + 6 * NH + NA * NB + 6 * kOneGradThreads == one_grad_smem<LA, LB>(), "smem layout");
  const int tid = threadIdx.x;
  const bool two = a != b;   // canonical pair with a distinct ket: ket derivative too
  const double A[3] = {P.sh.cx[a], P.sh.cy[a], P.sh.cz[a]};
  const double B[3] = {P.sh.cx[b], P.sh.cy[b], P.sh.cz[b]};
  const int a0 = P.sh.ao[a], b0 = P.sh.ao[b], n = P.nao;
  // block maximum of |D| and |W| and the summed nuclear charge: the scale of
  // everything this pair adds, for the primitive-pair screening below
  double dw = 0.0, zs = 0.0;
  for (int k = tid; k < NA * NB; k += blockDim.x) {
    const int i = k / NB, j = k % NB;
    const double nrm = cart_norm(LA, i) * cart_norm(LB, j);
    Dab[i][j] = Dm[(a0 + i) * n + b0 + j] * nrm;
    dw = fmax(dw, fmax(fabs(Dab[i][j]), fabs(Wm[(a0 + i) * n + b0 + j] * nrm)));
  }
  for (int k = tid; k < P.natom; k += blockDim.x) zs += fabs(P.charges[k]);
  for (int off = 16; off > 0; off >>= 1) {
    dw = fmax(dw, __shfl_xor_sync(0xffffffffu, dw, off));
    zs += __shfl_xor_sync(0xffffffffu, zs, off);
  }
  if ((tid & 31) == 0) {
    red[tid >> 5][0] = dw;
    red[tid >> 5][1] = zs;
  }
  __syncthreads();
  dw = 0.0;
  zs = 0.0;
  for (int w = 0; w < (int)blockDim.x / 32; ++w) {
    dw = fmax(dw, red[w][0]);
    zs += red[w][1];
  }
  __syncthreads();   // red is written again by the final reduction
  double R2 = 0.0;
  for (int d = 0; d < 3; ++d) R2 += (A[d] - B[d]) * (A[d] - B[d]);
  double gST[3] = {0.0, 0.0, 0.0}, gVA[3] = {0.0, 0.0, 0.0}, gVB[3] = {0.0, 0.0, 0.0};
  for (int ia = P.poff[a]; ia < P.poff[a + 1]; ++ia)
    for (int ib = P.poff[b]; ib < P.poff[b + 1]; ++ib) {
      const double al = P.exps[ia], be = P.exps[ib], p = al + be, mu = al * be / p;
      const double cc = P.coefs[ia] * P.coefs[ib];
      // primitive pairs whose contributions all stay below 1e-15 are skipped
      // (the same on every thread, so the barriers below stay uniform): the
      // product Gaussian c_i c_j exp(-mu |AB|^2) (pi/p)^3/2 bounds the
      // overlap; E coefficients grow at most as (|AB| + 1/sqrt(p) + 1)^(L+1),
      // derivatives as 2 max(alpha, beta) + L, kinetic terms as
      // 3 beta (LB + 2), attraction as 2 sqrt(p/pi) times the summed charge
      {
        const double g = fabs(cc) * exp(-mu * R2) * pow(pi / p, 1.5) * dw;
        const double e = pow(sqrt(R2) + rsqrt(p) + 1.0, (double)(L + 1));
        const double f = (2.0 * fmax(al, be) + L) * (1.0 + 2.0 * sqrt(p / pi) * zs + 3.0 * fmax(al, be) * (LB + 2));
        if (g * e * f < 1e-15) continue;
      }
      double Pc[3];
      for (int d = 0; d < 3; ++d) Pc[d] = (al * A[d] + be * B[d]) / p;
      __syncthreads();   // previous iteration done with E, M
      if (tid < 3) {
        const int d = tid;
        const double X = A[d] - B[d];
        double Et[LE + 1][LB + 3][LE + LB + 3];
        hermite_e<LE, LB + 2>(p, Pc[d] - A[d], Pc[d] - B[d], exp(-mu * X * X), Et);
        for (int i = 0; i <= LE; ++i)
          for (int j = 0; j <= LB + 2; ++j)
            for (int t = 0; t <= LE + LB + 2; ++t) E[d][i][j][t] = Et[i][j][t];
      }
      __syncthreads();
      // overlap / kinetic bra derivatives (Pulay -W dS, D dT), one (i, j, d)
      // per thread (gST is summed over the CTA at the end)
      {
        const double sp = pow(pi / p, 1.5);
        for (int task = tid; task < NA * NB * 3; task += blockDim.x) {
            const int i = task / (NB * 3), j = (task / 3) % NB, d = task % 3;
            const double nrm = cart_norm(LA, i) * cart_norm(LB, j);
            const double Dij = Dab[i][j], Wij = Wm[(a0 + i) * n + b0 + j] * nrm;
            const int bx[3] = {cart_e(LB, j, 0), cart_e(LB, j, 1), cart_e(LB, j, 2)};
            {
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
              gST[d] += cc * (Dij * dT - Wij * dS);
            }
          }
      }
      // density-contracted Hermite coefficients of the bra (MA) and ket (MB) derivatives
      const double pre = 2.0 * pi / p * cc;
      for (int k = tid; k < 3 * NH; k += blockDim.x) {
        const int d = k / NH, h = k % NH;
        const int t = h / ((L + 1) * (L + 1)), u = (h / (L + 1)) % (L + 1), v = h % (L + 1);
        double ma = 0.0, mb = 0.0;
        if (t + u + v <= L) {
          for (int i = 0; i < NA; ++i)
            for (int j = 0; j < NB; ++j) {
              const int ax0[3] = {cart_e(LA, i, 0), cart_e(LA, i, 1), cart_e(LA, i, 2)};
              const int bx0[3] = {cart_e(LB, j, 0), cart_e(LB, j, 1), cart_e(LB, j, 2)};
              double acca = 0.0, accb = 0.0;
              for (int sgn = 0; sgn < 2; ++sgn) {
                {
                  int ax[3] = {ax0[0], ax0[1], ax0[2]};
                  const int ad = ax[d];
                  if (!(sgn == 1 && ad == 0)) {
                    ax[d] += sgn == 0 ? 1 : -1;
                    if (t <= ax[0] + bx0[0] && u <= ax[1] + bx0[1] && v <= ax[2] + bx0[2]) {
                      const double f = sgn == 0 ? 2.0 * al : -(double)ad;
                      acca += f * E[0][ax[0]][bx0[0]][t] * E[1][ax[1]][bx0[1]][u] * E[2][ax[2]][bx0[2]][v];
                    }
                  }
                }
                if (two) {
                  int bx[3] = {bx0[0], bx0[1], bx0[2]};
                  const int bd = bx[d];
                  if (!(sgn == 1 && bd == 0)) {
                    bx[d] += sgn == 0 ? 1 : -1;
                    if (t <= ax0[0] + bx[0] && u <= ax0[1] + bx[1] && v <= ax0[2] + bx[2]) {
                      const double f = sgn == 0 ? 2.0 * be : -(double)bd;
                      accb += f * E[0][ax0[0]][bx[0]][t] * E[1][ax0[1]][bx[1]][u] * E[2][ax0[2]][bx[2]][v];
                    }
                  }
                }
              }
              ma += Dab[i][j] * acca;
              mb += Dab[i][j] * accb;
            }
        }
        MA[d][h] = pre * ma;
        MB[d][h] = pre * mb;
      }
      __syncthreads();
      for (int at = tid; at < P.natom; at += blockDim.x) {
        const double pc[3] = {Pc[0] - P.atom_xyz[3 * at], Pc[1] - P.atom_xyz[3 * at + 1],
                              Pc[2] - P.atom_xyz[3 * at + 2]};
        double F[L + 1];
        {
          double ur[NRT], wr[NRT];
          rys_roots_f64_tab<NRT>(P.tab64, P.asym, p * (pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]), ur, wr);
          double pw[NRT];
#pragma unroll
          for (int r = 0; r < NRT; ++r) pw[r] = wr[r];
#pragma unroll
          for (int m = 0; m <= L; ++m) {
            double f = 0.0;
#pragma unroll
            for (int r = 0; r < NRT; ++r) {
              f += pw[r];
              pw[r] *= ur[r];
            }
            F[m] = f;
          }
        }
        // R^m_tuv by the Hermite Coulomb recursion, in place: level m
        // overwrites t+u+w = L-m .. 1 from the top down (each entry needs
        // level m+1 at t+u+w-1 and -2, not yet overwritten), then R^m_000
        double R[L + 1][L + 1][L + 1];
        double fm2p[L + 1];
        fm2p[0] = 1.0;
#pragma unroll
        for (int m = 1; m <= L; ++m) fm2p[m] = fm2p[m - 1] * (-2.0 * p);
        R[0][0][0] = F[L] * fm2p[L];
#pragma unroll
        for (int m = L - 1; m >= 0; --m) {
#pragma unroll
          for (int sl = L - m; sl >= 1; --sl)
#pragma unroll
            for (int t = 0; t <= sl; ++t)
#pragma unroll
              for (int u = 0; u <= sl - t; ++u) {
                const int w = sl - t - u;
                double r;
                if (t > 0) r = (t > 1 ? (t - 1) * R[t - 2][u][w] : 0.0) + pc[0] * R[t - 1][u][w];
                else if (u > 0) r = (u > 1 ? (u - 1) * R[t][u - 2][w] : 0.0) + pc[1] * R[t][u - 1][w];
                else r = (w > 1 ? (w - 1) * R[t][u][w - 2] : 0.0) + pc[2] * R[t][u][w - 1];
                R[t][u][w] = r;
              }
          R[0][0][0] = F[m] * fm2p[m];
        }
        double da[3] = {0.0, 0.0, 0.0}, db[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int t = 0; t <= L; ++t)
#pragma unroll
          for (int u = 0; u <= L - t; ++u)
#pragma unroll
            for (int w = 0; w <= L - t - u; ++w) {
              const int h = (t * (L + 1) + u) * (L + 1) + w;
              const double rr = R[t][u][w];
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                da[d] += MA[d][h] * rr;
                db[d] += MB[d][h] * rr;
              }
            }
        const double z = -P.charges[at];
        for (int d = 0; d < 3; ++d) {
          gVA[d] += z * da[d];
          gVB[d] += z * db[d];
          atomicAdd(grad + 3 * at + d, -2.0 * z * (da[d] + db[d]));
        }
      }
    }
  // reduce over the CTA, one atomic per centre and direction
  for (int d = 0; d < 3; ++d) {
    red[tid][d] = gVA[d] + gST[d];
    red[tid][3 + d] = gVB[d] - gST[d];
  }
  __syncthreads();
  if (tid < 6) {
    double sacc = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) sacc += red[k][tid];
    if (tid < 3) atomicAdd(grad + 3 * P.sh.atom[a] + tid, 2.0 * sacc);
    else if (two) atomicAdd(grad + 3 * P.sh.atom[b] + tid - 3, 2.0 * sacc);
  }
}

// one CTA per canonical pair (a >= b): block k = a (a + 1) / 2 + b
__global__ void __launch_bounds__(kOneGradThreads) one_electron_grad_kernel(OneParams P, const double *D,
                                                                            const double *W, double *grad) {
  const int k = blockIdx.x;
  int a = (int)((sqrt(8.0 * k + 1.0) - 1.0) * 0.5);
  while (a * (a + 1) / 2 > k) --a;
  while ((a + 1) * (a + 2) / 2 <= k) ++a;
  const int b = k - a * (a + 1) / 2;
  __shared__ __align__(16) double smem[kOneGradSmem];
  switch (P.sh.l[a] * 3 + P.sh.l[b]) {
    case 0: one_pair_grad2<0, 0>(P, D, W, grad, a, b, smem); break;
    case 1: one_pair_grad2<0, 1>(P, D, W, grad, a, b, smem); break;
    case 2: one_pair_grad2<0, 2>(P, D, W, grad, a, b, smem); break;
    case 3: one_pair_grad2<1, 0>(P, D, W, grad, a, b, smem); break;
    case 4: one_pair_grad2<1, 1>(P, D, W, grad, a, b, smem); break;
    case 5: one_pair_grad2<1, 2>(P, D, W, grad, a, b, smem); break;
    case 6: one_pair_grad2<2, 0>(P, D, W, grad, a, b, smem); break;
    case 7: one_pair_grad2<2, 1>(P, D, W, grad, a, b, smem); break;
    case 8: one_pair_grad2<2, 2>(P, D, W, grad, a, b, smem); break;
    default: break;
  }
}

cudaError_t launch_one_electron_grad(const OneParams &P, const double *D, const double *W, double *grad,
                                     cudaStream_t st) {
  const int n = P.nshell * (P.nshell + 1) / 2;
  if (n == 0) return cudaSuccess;
  one_electron_grad_kernel<<<n, kOneGradThreads, 0, st>>>(P, D, W, grad);
  return cudaGetLastError();
}

}  // namespace sf
