// quartet.cuh -- Rys-quadrature shell-quartet kernels (sm_103a).
//
// One canonical class (la lb | lc ld), la >= lb, lc >= ld, pair class of
// (la,lb) >= pair class of (lc,ld), is one template instantiation.  A group of
// T threads evaluates one contracted shell quartet:
//
//   (ab|cd)_{ia ib ic id} = sum_{prim quartets} sum_{r < n} Ix Iy Iz
//
// with n = floor(L/2)+1 roots (the reference always uses 5: core.f90:952).
// For every primitive quartet and root the 2-D integrals of one Cartesian
// direction come from the vertical recurrence of core.f90:815-874 (B00, B10,
// B01, C00, C00') followed by the horizontal transfer of core.f90:877-899,
// written as the equivalent two-term recursion I(a,b+1) = I(a+1,b) + AB I(a,b)
// (bra) and the same on the ket.  The z direction carries the weight w_r and
// the primitive prefactor, so the innermost statement of core.f90:961
// (ix*iy*iz*w) costs one multiply and one FMA per Cartesian quadruple and root.
//
// T == 1: everything in registers, all indices compile-time.
// T  > 1: the 3n 2-D tables of a primitive quartet are computed by the T
//         threads in parallel (one (root, direction) task each), staged in
//         shared memory, and every thread accumulates the Cartesian outputs
//         o = t, t+T, t+2T, ...
//
// Epilogues: J/K digestion (fock), store (eri batch), diagonal max (Schwarz).
#pragma once
#include <cstdint>
#include <type_traits>

#include "dd.cuh"
#include "sf_internal.h"

namespace sf {

struct KParams {
  DevShells sh;
  DevPairs pr;
  DevPrims<double> p64;
  DevPrims<float> p32;
  const double *tab64;
  const float *tab32;  // FP32 kernel layout (rys_tab32v_offset)
  RysAsym asym;
  RysAsym32 asym32;
  // double-float copies: primitive-pair records (8 dd), centres, the FP64
  // Rys table as dd rows (rys_tabdd_offset) and the asymptotic constants
  DevPrims<dd> pdd;
  const float4 *pair32;   // per canonical pair: (Ax,Ay,Az,ABx) (ABy,ABz,ao_a,ao_b) (poff,np,a,b), FP32 / int bits
  const dd *cxd, *cyd, *czd;
  const float4 *tabdd;
  dd asymdd_r[kMaxRoots + 1][kMaxRoots], asymdd_w[kMaxRoots + 1][kMaxRoots];
  int nao;
  int nsm;             // multiprocessors (grid sizing of the grid-stride kernels)
  int natom;           // atoms referenced by the shells (gradient length / 3)
  int *err;            // device error flag (unused by the arithmetic kernels)
};

template <typename R>
__device__ __forceinline__ const DevPrims<R> &prims_of(const KParams &kp);
template <>
__device__ __forceinline__ const DevPrims<double> &prims_of<double>(const KParams &kp) { return kp.p64; }
template <>
__device__ __forceinline__ const DevPrims<float> &prims_of<float>(const KParams &kp) { return kp.p32; }
template <>
__device__ __forceinline__ const DevPrims<dd> &prims_of<dd>(const KParams &kp) { return kp.pdd; }

// type-generic loads, shuffles and conversions
__device__ __forceinline__ float ldg_r(const float *p) { return __ldg(p); }
__device__ __forceinline__ double ldg_r(const double *p) { return __ldg(p); }
__device__ __forceinline__ dd ldg_r(const dd *p) { return dd_ldg(p); }
__device__ __forceinline__ float shfl_xor_r(unsigned m, float v, int k) { return __shfl_xor_sync(m, v, k); }
__device__ __forceinline__ double shfl_xor_r(unsigned m, double v, int k) { return __shfl_xor_sync(m, v, k); }
__device__ __forceinline__ dd shfl_xor_r(unsigned m, dd v, int k) { return dd_shfl_xor(m, v, k); }
__device__ __forceinline__ float shfl_up_r(unsigned m, float v, int k) { return __shfl_up_sync(m, v, k); }
__device__ __forceinline__ double shfl_up_r(unsigned m, double v, int k) { return __shfl_up_sync(m, v, k); }
__device__ __forceinline__ dd shfl_up_r(unsigned m, dd v, int k) {
  return dd(__shfl_up_sync(m, v.hi, k), __shfl_up_sync(m, v.lo, k));
}

// Sums of v[0..N) over runs of equal key among the active lanes of a warp: a
// run is a maximal stretch of consecutive active lanes with one key (the
// consecutive quartets of a list that share their bra pair).  The same key
// may come back after a different one -- lists compacted on the device are
// chunks of the cost-sorted list in any order -- and then starts a new run.
// Segmented inclusive scan by shuffles, each lane taking partial sums only
// from lanes at or after the head of its own run (a lane whose left
// neighbour is inactive or has another key); returns true on the last lane of
// its run, which then holds the run's sums.  Lets one atomic per run replace
// one per lane on addresses all lanes of the run share.
template <typename R, int N>
__device__ __forceinline__ bool run_sums(int key, R (&v)[N]) {
  const unsigned mask = __activemask();
  const int lane = threadIdx.x & 31;
  const int kl = __shfl_up_sync(mask, key, 1);
  const bool head = lane == 0 || !((mask >> (lane - 1)) & 1u) || kl != key;
  const unsigned heads = __ballot_sync(mask, head);
  // highest head at or below this lane (the lowest active lane is a head)
  const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const bool take = lane - off >= start;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const R o = shfl_up_r(mask, v[i], off);
      if (take) v[i] += o;
    }
  }
  return lane == 31 || !((mask >> (lane + 1)) & 1u) || ((heads >> (lane + 1)) & 1u);
}

// 1/sqrt(a): single-precision hardware seed + two Newton-Raphson steps
// y <- y (3/2 - a/2 y^2) (quadratic convergence: 2^-23 -> 2^-46 -> rounding).
__device__ __forceinline__ double rsqrt_nr(double a) {
  double y = (double)rsqrtf((float)a);
  const double h = 0.5 * a;
  y = y * (1.5 - h * y * y);
  y = y * (1.5 - h * y * y);
  return y;
}
__device__ __forceinline__ float rsqrt_nr(float a) { return rsqrtf(a); }
__device__ __forceinline__ dd rsqrt_nr(dd a) { return dd_rsqrt(a); }

template <typename R>
struct TabDeg;
template <>
struct TabDeg<double> { static constexpr int v = kTabDeg64; };
template <>
struct TabDeg<float> { static constexpr int v = kTabDeg32; };

template <typename R>
__device__ __forceinline__ const R *tab_of(const KParams &kp);
template <>
__device__ __forceinline__ const double *tab_of<double>(const KParams &kp) { return kp.tab64; }
template <>
__device__ __forceinline__ const float *tab_of<float>(const KParams &kp) { return kp.tab32; }

// vector type of two values
template <typename R>
struct Vec2;
template <>
struct Vec2<double> { using T = double2; };
template <>
struct Vec2<float> { using T = float2; };

// FP32 register-path classes with at most this many Cartesian outputs
// evaluate two primitive quartets per loop iteration (eval_t1_x2)
constexpr int kX2MaxOutputs = 9;

// FP32: root r at x from its row of (u_k, w_k) pairs, Horner in the row's
// order k = D .. 0
__device__ __forceinline__ void rys_row_f32(const float *row, float s, float &u, float &w) {
  const float2 *c = reinterpret_cast<const float2 *>(row);
  const float2 top = __ldg(c);
  u = top.x;
  w = top.y;
#pragma unroll
  for (int k = 1; k <= kTabDeg32; ++k) {
    const float2 v = __ldg(c + k);
    u = u * s + v.x;
    w = w * s + v.y;
  }
}

// the same from a copy of the n-root block in shared memory
__device__ __forceinline__ void rys_row_f32_s(const float *row, float s, float &u, float &w) {
  const float2 *c = reinterpret_cast<const float2 *>(row);
  const float2 top = c[0];
  u = top.x;
  w = top.y;
#pragma unroll
  for (int k = 1; k <= kTabDeg32; ++k) {
    const float2 v = c[k];
    u = u * s + v.x;
    w = w * s + v.y;
  }
}

// The one-point rule in closed form (classes with L <= 1): w = F0(x),
// u = F1(x)/F0(x).  Below x = 1, F1 by its Taylor series
// F1 = sum_k (-x)^k / (k! (2k+3)) (11 terms, truncation < 1e-8) and
// F0 = 2x F1 + e^{-x} (the downward recursion); above, F0 = sqrt(pi/x)/2
// erf(sqrt x) and F1 = (F0 - e^{-x}) / (2x).  No table rows are read.  The
// square root and the quotients use the approximate reciprocal forms
// (rsqrtf, __fdividef: within 2 ulp), far inside the FP32 tier's error.
__device__ __forceinline__ void rys_n1_f32(float x, float &u, float &w) {
  const float e = expf(-x);
  float f0, f1;
  if (x < 1.0f) {
    f1 = 1.0f / 83462400.0f;
    f1 = f1 * x - 1.0f / 7620480.0f;
    f1 = f1 * x + 1.0f / 766080.0f;
    f1 = f1 * x - 1.0f / 85680.0f;
    f1 = f1 * x + 1.0f / 10800.0f;
    f1 = f1 * x - 1.0f / 1560.0f;
    f1 = f1 * x + 1.0f / 264.0f;
    f1 = f1 * x - 1.0f / 54.0f;
    f1 = f1 * x + 1.0f / 14.0f;
    f1 = f1 * x - 1.0f / 5.0f;
    f1 = f1 * x + 1.0f / 3.0f;
    f0 = 2.0f * x * f1 + e;
  } else {
    const float isx = rsqrtf(x), sx = x * isx;
    f0 = 0.886226925452758f * isx * erff(sx);   // sqrt(pi) / 2
    f1 = __fdividef(f0 - e, 2.0f * x);
  }
  w = f0;
  u = __fdividef(f1, f0);
}

template <int N>
__device__ __forceinline__ void rys_roots_all_f32_s(const KParams &kp, const float *tab_s, float x, float (&u)[N],
                                                    float (&w)[N]) {
  if constexpr (N == 1) {
    if (x < (float)kTabXmax) {
      rys_n1_f32(x, u[0], w[0]);
      return;
    }
  }
  if (x >= (float)kTabXmax) {
    const float ix = __fdividef(1.0f, x), isx = rsqrtf(x);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = kp.asym32.r[N][i] * ix;
      w[i] = kp.asym32.w[N][i] * isx;
    }
    return;
  }
  const int j = (int)x;
  const float s = 2.0f * (x - (float)j) - 1.0f;
  const float *base = tab_s + j * N * kTab32Row;
#pragma unroll
  for (int i = 0; i < N; ++i) rys_row_f32_s(base + i * kTab32Row, s, u[i], w[i]);
}

template <int N>
__device__ __forceinline__ void rys_roots_all_f32(const KParams &kp, float x, float (&u)[N], float (&w)[N]) {
  if constexpr (N == 1) {
    if (x < (float)kTabXmax) {
      rys_n1_f32(x, u[0], w[0]);
      return;
    }
  }
  if (x >= (float)kTabXmax) {
    const float ix = __fdividef(1.0f, x), isx = rsqrtf(x);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = kp.asym32.r[N][i] * ix;
      w[i] = kp.asym32.w[N][i] * isx;
    }
    return;
  }
  const int j = (int)x;
  const float s = 2.0f * (x - (float)j) - 1.0f;
  const float *base = kp.tab32 + rys_tab32v_offset(N) + j * N * kTab32Row;
#pragma unroll
  for (int i = 0; i < N; ++i) rys_row_f32(base + i * kTab32Row, s, u[i], w[i]);
}

// dd: the FP64 table's coefficients as dd rows: per n-root block, interval
// j, root r, the (D+1) coefficients from k = D down to 0, each one 16-byte
// (u_hi, u_lo, w_hi, w_lo); Horner in dd
// The leading kDDTop coefficients (k = D .. D-kDDTop+1) are summed in plain
// FP32: over every interval and root their terms add up to less than 5e-8 of
// |c_0| (Chebyshev-fitted rows decay geometrically), so FP32 rounding there
// stays below 1e-14 relative; the remaining rows run in dd.
constexpr int kDDTop = 4;
__device__ __forceinline__ void rys_row_dd(const float4 *row, dd s, dd &u, dd &w) {
  const float4 top = __ldg(row);
  float uf = top.x, wf = top.z;
#pragma unroll
  for (int k = 1; k < kDDTop; ++k) {
    const float4 c = __ldg(row + k);
    uf = fmaf(uf, s.hi, c.x);
    wf = fmaf(wf, s.hi, c.z);
  }
  u = dd(uf);
  w = dd(wf);
#pragma unroll
  for (int k = kDDTop; k <= kTabDeg64; ++k) {
    const float4 c = __ldg(row + k);
    u = dd_fma(u, s, dd(c.x, c.y));
    w = dd_fma(w, s, dd(c.z, c.w));
  }
}

template <int N>
__device__ __forceinline__ void rys_roots_all_dd(const KParams &kp, dd x, dd (&u)[N], dd (&w)[N]) {
  if (x.hi >= (float)kTabXmax) {
    const dd ix = dd_recip(x), isx = dd_rsqrt(x);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = kp.asymdd_r[N][i] * ix;
      w[i] = kp.asymdd_w[N][i] * isx;
    }
    return;
  }
  const int j = (int)x.hi;
  const dd s = (x - dd((float)j)) * 2.0f - dd(1.0f);
  const float4 *base = kp.tabdd + rys_tabdd_offset(N) + j * N * (kTabDeg64 + 1);
#pragma unroll
  for (int i = 0; i < N; ++i) rys_row_dd(base + i * (kTabDeg64 + 1), s, u[i], w[i]);
}

// all n roots (u = t^2) and weights at x.  FP64: coefficient row k of an
// interval holds the 2N values (u_0..u_{N-1}, w_0..w_{N-1}); rows are loaded
// as N two-value vectors (the table offsets are all even).
template <int N>
__device__ __forceinline__ void rys_roots_all_f64(const KParams &kp, double x, double (&u)[N], double (&w)[N]);

template <int N, typename R>
__device__ __forceinline__ void rys_roots_all(const KParams &kp, R x, R (&u)[N], R (&w)[N]) {
  if constexpr (std::is_same<R, float>::value) {
    rys_roots_all_f32<N>(kp, x, u, w);
  } else if constexpr (std::is_same<R, dd>::value) {
    rys_roots_all_dd<N>(kp, x, u, w);
  } else {
    rys_roots_all_f64<N>(kp, x, u, w);
  }
}

// the FP64 rule from an explicit table and asymptotic constants (also used by
// the one-electron kernels, whose Boys values are sum_i w_i u_i^m)
template <int N>
__device__ __forceinline__ void rys_roots_f64_tab(const double *tab64, const RysAsym &asym, double x,
                                                  double (&u)[N], double (&w)[N]) {
  using R = double;
  if (x >= (R)kTabXmax) {
    const R ix = (R)1 / x, isx = rsqrt_nr(x);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = (R)asym.r[N][i] * ix;
      w[i] = (R)asym.w[N][i] * isx;
    }
    return;
  }
  using V = typename Vec2<R>::T;
  constexpr int D = TabDeg<R>::v;
  const int j = (int)x;
  const R s = (R)2 * (x - (R)j) - (R)1;
  const V *c = reinterpret_cast<const V *>(tab64 + rys_tab_offset(N, D) + j * (D + 1) * 2 * N);
  R f[2 * N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const V v = __ldg(c + D * N + i);
    f[2 * i] = v.x;
    f[2 * i + 1] = v.y;
  }
#pragma unroll
  for (int k = D - 1; k >= 0; --k) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const V v = __ldg(c + k * N + i);
      f[2 * i] = f[2 * i] * s + v.x;
      f[2 * i + 1] = f[2 * i + 1] * s + v.y;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    u[i] = f[i];
    w[i] = f[N + i];
  }
}

template <int N>
__device__ __forceinline__ void rys_roots_all_f64(const KParams &kp, double x, double (&u)[N], double (&w)[N]) {
  rys_roots_f64_tab<N>(kp.tab64, kp.asym, x, u, w);
}

// one root r of the n-point rule
template <int N>
__device__ __forceinline__ void rys_root_one_f64(const KParams &kp, double x, int r, double &u, double &w);

template <int N, typename R>
__device__ __forceinline__ void rys_root_one(const KParams &kp, R x, int r, R &u, R &w) {
  if constexpr (std::is_same<R, float>::value) {
    if (x >= (float)kTabXmax) {
      u = __fdividef(kp.asym32.r[N][r], x);
      w = kp.asym32.w[N][r] * rsqrtf(x);
      return;
    }
    const int j = (int)x;
    const float s = 2.0f * (x - (float)j) - 1.0f;
    rys_row_f32(kp.tab32 + rys_tab32v_offset(N) + (j * N + r) * kTab32Row, s, u, w);
  } else if constexpr (std::is_same<R, dd>::value) {
    if (x.hi >= (float)kTabXmax) {
      u = kp.asymdd_r[N][r] * dd_recip(x);
      w = kp.asymdd_w[N][r] * dd_rsqrt(x);
      return;
    }
    const int j = (int)x.hi;
    const dd s = (x - dd((float)j)) * 2.0f - dd(1.0f);
    rys_row_dd(kp.tabdd + rys_tabdd_offset(N) + (j * N + r) * (kTabDeg64 + 1), s, u, w);
  } else {
    rys_root_one_f64<N>(kp, x, r, u, w);
  }
}

template <int N>
__device__ __forceinline__ void rys_root_one_f64(const KParams &kp, double x, int r, double &u, double &w) {
  using R = double;
  if (x >= (R)kTabXmax) {
    u = (R)kp.asym.r[N][r] / x;
    w = (R)kp.asym.w[N][r] * rsqrt_nr(x);
    return;
  }
  constexpr int D = TabDeg<R>::v;
  const int j = (int)x;
  const R s = (R)2 * (x - (R)j) - (R)1;
  const R *c = tab_of<R>(kp) + rys_tab_offset(N, D) + j * (D + 1) * 2 * N;
  u = __ldg(c + D * 2 * N + r);
  w = __ldg(c + D * 2 * N + N + r);
#pragma unroll
  for (int k = D - 1; k >= 0; --k) {
    u = u * s + __ldg(c + k * 2 * N + r);
    w = w * s + __ldg(c + k * 2 * N + N + r);
  }
}

template <int LA, int LB, int LC, int LD>
struct QC {
  static constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
  static constexpr int NCD = NC * ND, NABCD = NA * NB * NC * ND;
  static constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
  static constexpr int NR = L / 2 + 1;
  static constexpr int SZ = (LA + 1) * (LB + 1) * (LC + 1) * (LD + 1);
  __host__ __device__ static constexpr int ca(int o) { return o / (NB * NC * ND); }
  __host__ __device__ static constexpr int cb(int o) { return (o / (NC * ND)) % NB; }
  __host__ __device__ static constexpr int cc(int o) { return (o / ND) % NC; }
  __host__ __device__ static constexpr int cd(int o) { return o % ND; }
  // offset of output o's factor in the 2-D table of direction d
  __host__ __device__ static constexpr int toff(int o, int d) {
    return ((cart_e(LA, ca(o), d) * (LB + 1) + cart_e(LB, cb(o), d)) * (LC + 1) + cart_e(LC, cc(o), d)) * (LD + 1) +
           cart_e(LD, cd(o), d);
  }
  __host__ __device__ static constexpr double norm(int o) {
    return cart_norm(LA, ca(o)) * cart_norm(LB, cb(o)) * cart_norm(LC, cc(o)) * cart_norm(LD, cd(o));
  }
};

// Vertical recurrence + horizontal transfer for one root and one direction.
// Output I[((ia*(LB+1)+ib)*(LC+1)+ic)*(LD+1)+id].
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void rys_2d(R g0, R c00, R c00p, R b00, R b10, R b01, R ab, R cd, R *__restrict__ I) {
  constexpr int LAB = LA + LB, LCD = LC + LD;
  R G[LAB + 1][LCD + 1];
  G[0][0] = g0;
  if (LAB > 0) G[1][0] = c00 * g0;
#pragma unroll
  for (int i = 1; i < LAB; ++i) G[i + 1][0] = (R)i * b10 * G[i - 1][0] + c00 * G[i][0];
  if (LCD > 0) {
    G[0][1] = c00p * g0;
#pragma unroll
    for (int i = 1; i <= LAB; ++i) G[i][1] = (R)i * b00 * G[i - 1][0] + c00p * G[i][0];
#pragma unroll
    for (int k = 1; k < LCD; ++k) {
      G[0][k + 1] = (R)k * b01 * G[0][k - 1] + c00p * G[0][k];
#pragma unroll
      for (int i = 1; i <= LAB; ++i)
        G[i][k + 1] = (R)k * b01 * G[i][k - 1] + (R)i * b00 * G[i - 1][k] + c00p * G[i][k];
    }
  }
  // bra transfer: H[ia][ib][k]
  R H[LA + 1][LB + 1][LCD + 1];
#pragma unroll
  for (int k = 0; k <= LCD; ++k) {
    R t[LAB + 1];
#pragma unroll
    for (int i = 0; i <= LAB; ++i) t[i] = G[i][k];
#pragma unroll
    for (int ia = 0; ia <= LA; ++ia) H[ia][0][k] = t[ia];
#pragma unroll
    for (int ib = 1; ib <= LB; ++ib) {
#pragma unroll
      for (int i = 0; i <= LAB - ib; ++i) t[i] = t[i + 1] + ab * t[i];
#pragma unroll
      for (int ia = 0; ia <= LA; ++ia) H[ia][ib][k] = t[ia];
    }
  }
  // ket transfer
#pragma unroll
  for (int ia = 0; ia <= LA; ++ia) {
#pragma unroll
    for (int ib = 0; ib <= LB; ++ib) {
      R t[LCD + 1];
#pragma unroll
      for (int k = 0; k <= LCD; ++k) t[k] = H[ia][ib][k];
#pragma unroll
      for (int ic = 0; ic <= LC; ++ic) I[((ia * (LB + 1) + ib) * (LC + 1) + ic) * (LD + 1) + 0] = t[ic];
#pragma unroll
      for (int id = 1; id <= LD; ++id) {
#pragma unroll
        for (int k = 0; k <= LCD - id; ++k) t[k] = t[k + 1] + cd * t[k];
#pragma unroll
        for (int ic = 0; ic <= LC; ++ic) I[((ia * (LB + 1) + ib) * (LC + 1) + ic) * (LD + 1) + id] = t[ic];
      }
    }
  }
}

// geometry of one contracted quartet
template <typename R>
struct QGeom {
  int a, b, c, d;
  int a0, b0, c0, d0;                  // first AO of each shell
  int ab_off, ab_n, cd_off, cd_n;
  R Ax, Ay, Az, Cx, Cy, Cz;
  R ABx, ABy, ABz, CDx, CDy, CDz;
};

template <typename R>
__device__ __forceinline__ const R *centre_of(const DevShells &sh, int d);
template <>
__device__ __forceinline__ const double *centre_of<double>(const DevShells &sh, int d) {
  return d == 0 ? sh.cx : d == 1 ? sh.cy : sh.cz;
}
template <>
__device__ __forceinline__ const float *centre_of<float>(const DevShells &sh, int d) {
  return d == 0 ? sh.cx32 : d == 1 ? sh.cy32 : sh.cz32;
}
template <typename R>
__device__ __forceinline__ const R *centre_in(const KParams &kp, int d) {
  if constexpr (std::is_same<R, dd>::value) return d == 0 ? kp.cxd : d == 1 ? kp.cyd : kp.czd;
  else return centre_of<R>(kp.sh, d);
}

// geometry in the working precision R (the FP32 kernels read single-precision
// centres and never touch the FP64 pipe here)
template <typename R>
__device__ __forceinline__ QGeom<R> make_geom(const KParams &kp, int pab, int pcd, bool swap_ab, bool swap_cd) {
  QGeom<R> g;
  int a = kp.pr.a[pab], b = kp.pr.b[pab], c = kp.pr.a[pcd], d = kp.pr.b[pcd];
  if (swap_ab) { int t = a; a = b; b = t; }
  if (swap_cd) { int t = c; c = d; d = t; }
  g.a = a; g.b = b; g.c = c; g.d = d;
  g.a0 = kp.sh.ao[a]; g.b0 = kp.sh.ao[b]; g.c0 = kp.sh.ao[c]; g.d0 = kp.sh.ao[d];
  g.ab_off = kp.pr.poff[pab]; g.ab_n = kp.pr.np[pab];
  g.cd_off = kp.pr.poff[pcd]; g.cd_n = kp.pr.np[pcd];
  const R *X = centre_in<R>(kp, 0), *Y = centre_in<R>(kp, 1), *Z = centre_in<R>(kp, 2);
  g.Ax = X[a]; g.Ay = Y[a]; g.Az = Z[a];
  g.Cx = X[c]; g.Cy = Y[c]; g.Cz = Z[c];
  g.ABx = g.Ax - X[b]; g.ABy = g.Ay - Y[b]; g.ABz = g.Az - Z[b];
  g.CDx = g.Cx - X[d]; g.CDy = g.Cy - Y[d]; g.CDz = g.Cz - Z[d];
  return g;
}

// FP32 geometry of a quartet from the packed pair records (three 16-byte
// loads per pair instead of about twenty scattered loads of pair, shell and
// centre arrays; the quartet set-up is a latency chain in the light classes)
__device__ __forceinline__ QGeom<float> make_geom32(const KParams &kp, int pab, int pcd) {
  QGeom<float> g;
  const float4 *pa = kp.pair32 + 3 * (size_t)pab, *pc = kp.pair32 + 3 * (size_t)pcd;
  const float4 a0 = __ldg(pa), a1 = __ldg(pa + 1), a2 = __ldg(pa + 2);
  const float4 c0 = __ldg(pc), c1 = __ldg(pc + 1), c2 = __ldg(pc + 2);
  g.Ax = a0.x; g.Ay = a0.y; g.Az = a0.z; g.ABx = a0.w; g.ABy = a1.x; g.ABz = a1.y;
  g.a0 = __float_as_int(a1.z); g.b0 = __float_as_int(a1.w);
  g.ab_off = __float_as_int(a2.x); g.ab_n = __float_as_int(a2.y);
  g.a = __float_as_int(a2.z); g.b = __float_as_int(a2.w);
  g.Cx = c0.x; g.Cy = c0.y; g.Cz = c0.z; g.CDx = c0.w; g.CDy = c1.x; g.CDz = c1.y;
  g.c0 = __float_as_int(c1.z); g.d0 = __float_as_int(c1.w);
  g.cd_off = __float_as_int(c2.x); g.cd_n = __float_as_int(c2.y);
  g.c = __float_as_int(c2.z); g.d = __float_as_int(c2.w);
  return g;
}

// scalars of one primitive quartet
template <typename R>
struct PQ {
  R pax, pay, paz, qcx, qcy, qcz, pqx, pqy, pqz;
  R r2, aq, ap, i2p, i2q, x, pref;
};

// one primitive-pair record as (p, Px, Py, Pz) and (K~, 0.5/p)
template <typename R>
__device__ __forceinline__ void load_rec(const R *rec, R &p, R &px, R &py, R &pz, R &k, R &i2p);
template <>
__device__ __forceinline__ void load_rec<float>(const float *rec, float &p, float &px, float &py, float &pz, float &k,
                                                float &i2p) {
  const float4 a = __ldg(reinterpret_cast<const float4 *>(rec));
  const float2 b = __ldg(reinterpret_cast<const float2 *>(rec + 4));
  p = a.x; px = a.y; py = a.z; pz = a.w; k = b.x; i2p = b.y;
}
template <>
__device__ __forceinline__ void load_rec<double>(const double *rec, double &p, double &px, double &py, double &pz,
                                                 double &k, double &i2p) {
  const double2 a = __ldg(reinterpret_cast<const double2 *>(rec));
  const double2 b = __ldg(reinterpret_cast<const double2 *>(rec + 2));
  const double2 c = __ldg(reinterpret_cast<const double2 *>(rec + 4));
  p = a.x; px = a.y; py = b.x; pz = b.y; k = c.x; i2p = c.y;
}

template <>
__device__ __forceinline__ void load_rec<dd>(const dd *rec, dd &p, dd &px, dd &py, dd &pz, dd &k, dd &i2p) {
  const float4 *r4 = reinterpret_cast<const float4 *>(rec);
  const float4 a = __ldg(r4), b = __ldg(r4 + 1), c = __ldg(r4 + 2);
  p = dd(a.x, a.y); px = dd(a.z, a.w); py = dd(b.x, b.y); pz = dd(b.z, b.w); k = dd(c.x, c.y); i2p = dd(c.z, c.w);
}

template <typename R>
__device__ __forceinline__ void load_prim_ab(const KParams &kp, const QGeom<R> &g, int ip, PQ<R> &s, R &p, R &px,
                                             R &py, R &pz, R &kab) {
  load_rec<R>(prims_of<R>(kp).rec + (size_t)(g.ab_off + ip) * kPrimRec, p, px, py, pz, kab, s.i2p);
  s.pax = px - g.Ax; s.pay = py - g.Ay; s.paz = pz - g.Az;
}

// one ket primitive-pair record held in registers (loaded an iteration ahead)
template <typename R>
struct KetRec {
  R q, qx, qy, qz, kcd, i2q;
};
template <typename R>
__device__ __forceinline__ void load_ket(const KParams &kp, const QGeom<R> &g, int iq, KetRec<R> &k) {
  load_rec<R>(prims_of<R>(kp).rec + (size_t)(g.cd_off + iq) * kPrimRec, k.q, k.qx, k.qy, k.qz, k.kcd, k.i2q);
}

// primitive-quartet scalars from the bra values and a ket record
template <typename R>
__device__ __forceinline__ void set_prim_cd(const QGeom<R> &g, const KetRec<R> &k, PQ<R> &s, R p, R px, R py, R pz,
                                            R kab) {
  const R q = k.q, qx = k.qx, qy = k.qy, qz = k.qz, kcd = k.kcd;
  s.i2q = k.i2q;
  s.qcx = qx - g.Cx; s.qcy = qy - g.Cy; s.qcz = qz - g.Cz;
  s.pqx = px - qx; s.pqy = py - qy; s.pqz = pz - qz;
  const R rr = rsqrt_nr(p + q);
  s.r2 = rr * rr;
  s.aq = q * s.r2;
  s.ap = p * s.r2;
  const R rho = p * s.aq;
  s.x = rho * (s.pqx * s.pqx + s.pqy * s.pqy + s.pqz * s.pqz);
  s.pref = kab * kcd * rr;
}

template <typename R>
__device__ __forceinline__ void load_prim_cd(const KParams &kp, const QGeom<R> &g, int iq, PQ<R> &s, R p, R px, R py,
                                             R pz, R kab) {
  R q, qx, qy, qz, kcd;
  load_rec<R>(prims_of<R>(kp).rec + (size_t)(g.cd_off + iq) * kPrimRec, q, qx, qy, qz, kcd, s.i2q);
  s.qcx = qx - g.Cx; s.qcy = qy - g.Cy; s.qcz = qz - g.Cz;
  s.pqx = px - qx; s.pqy = py - qy; s.pqz = pz - qz;
  const R rr = rsqrt_nr(p + q);
  s.r2 = rr * rr;
  s.aq = q * s.r2;
  s.ap = p * s.r2;
  const R rho = p * s.aq;
  s.x = rho * (s.pqx * s.pqx + s.pqy * s.pqy + s.pqz * s.pqz);
  s.pref = kab * kcd * rr;
}

// float -> double without the FP64 pipe: re-pack sign, exponent (rebias
// 127 -> 1023, i.e. + 896 << 20 in the high word) and mantissa with five
// 32-bit integer operations, no branches.  Exact for normal floats.  A zero
// or single-precision subnormal becomes a number of magnitude below
// 1.2e-38 (a zero: +-2^-127) instead of +-0, which adds nothing measurable
// to the FP64 sums it feeds; the FP32 kernels produce no inf or nan.  (The
// version with those special cases cost 3-6 % of the FP32 + double-float
// build: (H2O)8 1.43 -> 1.35 ms, (H2O)16 6.71 -> 6.48 ms.)
__device__ __forceinline__ double f2d_alu(float f) {
  const unsigned u = __float_as_uint(f);
  return __hiloint2double((int)((u & 0x80000000u) | (((u >> 3) & 0x0fffffffu) + 0x38000000u)), (int)(u << 29));
}
__device__ __forceinline__ double to_f64(float f) { return f2d_alu(f); }
__device__ __forceinline__ double to_f64(double f) { return f; }
__device__ __forceinline__ double to_f64(dd f) { return f2d_alu(f.hi) + f2d_alu(f.lo); }

// advance the (ab, cd) primitive indices of a flattened index by step
__device__ __forceinline__ void prim_advance(int &ip, int &iq, int step, int cd_n) {
  iq += step;
  if (iq >= cd_n) {
    const int k = iq / cd_n;
    ip += k;
    iq -= k * cd_n;
  }
}

// bra primitive-pair values cached across primitive quartets
template <typename R>
struct BraRec {
  R p, px, py, pz, kab, i2p;
};
template <typename R>
__device__ __forceinline__ void load_bra(const KParams &kp, const QGeom<R> &g, int ip, BraRec<R> &b) {
  load_rec<R>(prims_of<R>(kp).rec + (size_t)(g.ab_off + ip) * kPrimRec, b.p, b.px, b.py, b.pz, b.kab, b.i2p);
}
template <typename R>
__device__ __forceinline__ void set_pq(const QGeom<R> &g, const BraRec<R> &b, const KetRec<R> &k, PQ<R> &s) {
  s.i2p = b.i2p;
  s.pax = b.px - g.Ax; s.pay = b.py - g.Ay; s.paz = b.pz - g.Az;
  set_prim_cd<R>(g, k, s, b.p, b.px, b.py, b.pz, b.kab);
}

// all roots, from the shared-memory copy of the FP32 table when given
template <int N, typename R>
__device__ __forceinline__ void roots_t1(const KParams &kp, const float *tab_s, R x, R (&u)[N], R (&w)[N]) {
  if constexpr (std::is_same<R, float>::value) {
    if (tab_s) {
      rys_roots_all_f32_s<N>(kp, tab_s, x, u, w);
      return;
    }
  }
  rys_roots_all<N, R>(kp, x, u, w);
}

// Rys assembly of one primitive quartet into acc (roots already evaluated)
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void assemble_pq(const QGeom<R> &g, const PQ<R> &s, const R *u, const R *w,
                                            R (&acc)[QC<LA, LB, LC, LD>::NABCD]) {
  using Q = QC<LA, LB, LC, LD>;
  constexpr int NR = Q::NR, SZ = Q::SZ;
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    const R uu = u[r];
    const R b00 = (R)0.5 * s.r2 * uu;
    const R b10 = s.i2p * ((R)1 - s.aq * uu);
    const R b01 = s.i2q * ((R)1 - s.ap * uu);
    const R tq = s.aq * uu, tp = s.ap * uu;
    R Ix[SZ], Iy[SZ], Iz[SZ];
    rys_2d<LA, LB, LC, LD, R>((R)1, s.pax - tq * s.pqx, s.qcx + tp * s.pqx, b00, b10, b01, g.ABx, g.CDx, Ix);
    rys_2d<LA, LB, LC, LD, R>((R)1, s.pay - tq * s.pqy, s.qcy + tp * s.pqy, b00, b10, b01, g.ABy, g.CDy, Iy);
    rys_2d<LA, LB, LC, LD, R>(s.pref * w[r], s.paz - tq * s.pqz, s.qcz + tp * s.pqz, b00, b10, b01, g.ABz, g.CDz,
                              Iz);
#pragma unroll
    for (int o = 0; o < Q::NABCD; ++o) acc[o] += Ix[Q::toff(o, 0)] * Iy[Q::toff(o, 1)] * Iz[Q::toff(o, 2)];
  }
}

// T == 1, FP32, few outputs: two primitive quartets per iteration, their
// record and table loads issued before either is consumed (the low-L FP32
// kernels are bound by the latency of these dependent loads); an odd tail
// repeats the last quartet with a zero prefactor
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void eval_t1_x2(const KParams &kp, const QGeom<R> &g,
                                           R (&acc)[QC<LA, LB, LC, LD>::NABCD], int p, int P, const float *tab_s) {
  using Q = QC<LA, LB, LC, LD>;
  constexpr int NR = Q::NR;
#pragma unroll
  for (int o = 0; o < Q::NABCD; ++o) acc[o] = (R)0;
  const int nprim = g.ab_n * g.cd_n;
  int cur = -1;
  BraRec<R> br;
  // (ab, cd) primitive indices of idx advanced incrementally: a division
  // only when the cd index wraps
  int ip1 = p / g.cd_n, iq1 = p - ip1 * g.cd_n;
  for (int idx = p; idx < nprim; idx += 2 * P) {
    const bool two = idx + P < nprim;
    int ip2 = ip1, iq2 = iq1;
    if (two) prim_advance(ip2, iq2, P, g.cd_n);
    KetRec<R> k1, k2;
    load_ket<R>(kp, g, iq1, k1);
    load_ket<R>(kp, g, iq2, k2);
    if (ip1 != cur) {
      load_bra<R>(kp, g, ip1, br);
      cur = ip1;
    }
    BraRec<R> b2 = br;
    if (ip2 != ip1) {
      load_bra<R>(kp, g, ip2, b2);
    }
    PQ<R> s1, s2;
    set_pq<R>(g, br, k1, s1);
    set_pq<R>(g, b2, k2, s2);
    if (!two) s2.pref = (R)0;
    if (ip2 != ip1) {
      br = b2;
      cur = ip2;
    }
    R u1[NR], w1[NR], u2[NR], w2[NR];
    roots_t1<NR, R>(kp, tab_s, s1.x, u1, w1);
    roots_t1<NR, R>(kp, tab_s, s2.x, u2, w2);
    assemble_pq<LA, LB, LC, LD, R>(g, s1, u1, w1, acc);
    assemble_pq<LA, LB, LC, LD, R>(g, s2, u2, w2, acc);
    prim_advance(ip1, iq1, 2 * P, g.cd_n);
  }
}

// ---------------------------------------------------------------------------
// T == 1: whole quartet in registers; acc[o] unnormalised
// ---------------------------------------------------------------------------
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void eval_t1(const KParams &kp, const QGeom<R> &g, R (&acc)[QC<LA, LB, LC, LD>::NABCD],
                                        int p = 0, int P = 1, const float *tab_s = nullptr) {
  using Q = QC<LA, LB, LC, LD>;
  constexpr int NR = Q::NR, SZ = Q::SZ;
  if constexpr (std::is_same<R, float>::value && Q::NABCD <= kX2MaxOutputs) {
    eval_t1_x2<LA, LB, LC, LD, R>(kp, g, acc, p, P, tab_s);
    return;
  }
#pragma unroll
  for (int o = 0; o < Q::NABCD; ++o) acc[o] = (R)0;
  const int nprim = g.ab_n * g.cd_n;
  int cur = -1;
  PQ<R> s;
  // primitive quartets idx = p, p+P, ... of the ab-major flattened loop; the
  // ket record of the next one, and its bra record when the bra index
  // changes, are loaded while this one is evaluated
  KetRec<R> kn;
  BraRec<R> bn, b;
  int ip = p / g.cd_n, iq = p - ip * g.cd_n;   // (ab, cd) indices of idx
  if (p < nprim) {
    load_ket<R>(kp, g, iq, kn);
    load_bra<R>(kp, g, ip, bn);
  }
  for (int idx = p; idx < nprim; idx += P) {
    const KetRec<R> kc = kn;
    if (ip != cur) {
      b = bn;
      cur = ip;
      s.i2p = b.i2p;
      s.pax = b.px - g.Ax; s.pay = b.py - g.Ay; s.paz = b.pz - g.Az;
    }
    int ipn = ip, iqn = iq;
    prim_advance(ipn, iqn, P, g.cd_n);
    if (idx + P < nprim) {
      load_ket<R>(kp, g, iqn, kn);
      if (ipn != ip) load_bra<R>(kp, g, ipn, bn);
    }
    set_prim_cd<R>(g, kc, s, b.p, b.px, b.py, b.pz, b.kab);
    ip = ipn;
    iq = iqn;
    R u[NR], w[NR];
    roots_t1<NR, R>(kp, tab_s, s.x, u, w);
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const R uu = u[r];
      const R b00 = (R)0.5 * s.r2 * uu;
      const R b10 = s.i2p * ((R)1 - s.aq * uu);
      const R b01 = s.i2q * ((R)1 - s.ap * uu);
      const R tq = s.aq * uu, tp = s.ap * uu;
      R Ix[SZ], Iy[SZ], Iz[SZ];
      rys_2d<LA, LB, LC, LD, R>((R)1, s.pax - tq * s.pqx, s.qcx + tp * s.pqx, b00, b10, b01, g.ABx, g.CDx, Ix);
      rys_2d<LA, LB, LC, LD, R>((R)1, s.pay - tq * s.pqy, s.qcy + tp * s.pqy, b00, b10, b01, g.ABy, g.CDy, Iy);
      rys_2d<LA, LB, LC, LD, R>(s.pref * w[r], s.paz - tq * s.pqz, s.qcz + tp * s.pqz, b00, b10, b01, g.ABz,
                                g.CDz, Iz);
#pragma unroll
      for (int o = 0; o < Q::NABCD; ++o) acc[o] += Ix[Q::toff(o, 0)] * Iy[Q::toff(o, 1)] * Iz[Q::toff(o, 2)];
    }
  }
}

// ---------------------------------------------------------------------------
// T > 1: group of T lanes (inside one warp); tab = 3*NR*SZ shared values
// ---------------------------------------------------------------------------
template <int LA, int LB, int LC, int LD, typename R, int T>
struct Grp {
  using Q = QC<LA, LB, LC, LD>;
  // Outputs per lane.  FP32 groups own whole rows: the INNER outputs that
  // differ only in the components of the last shell with l > 0 (d, or c when
  // l_d = 0).  A row's 2-D factors in each direction are the LI+1 consecutive
  // table entries of that shell's exponents, loaded once per root and shared
  // by its INNER outputs (3 (LI+1) shared loads per root instead of 3 INNER:
  // the FP32 contraction is bound by shared-memory loads, FP64 by its pipe).
  // Otherwise output o = t + k T.
  static constexpr bool ROWWISE = std::is_same<R, float>::value && (LD > 0 || LC > 0);
  static constexpr int LI = LD > 0 ? LD : LC;
  static constexpr int INNER = ROWWISE ? (LD > 0 ? Q::ND : Q::NC) : 1;
  static constexpr int ROWS = Q::NABCD / INNER;
  static constexpr int RPER = (ROWS + T - 1) / T;
  static constexpr int NPER = RPER * INNER;
  // output of lane t's k-th accumulator (>= NABCD past the last row)
  __device__ static __forceinline__ int out(int t, int k) { return (t + (k / INNER) * T) * INNER + k % INNER; }
  static constexpr int TABN = 3 * Q::NR * Q::SZ;            // 2-D tables of one primitive quartet
  static constexpr int ROOTS = TABN;                         // then u_r, w_r
  static constexpr int NEED = (TABN + 2 * Q::NR) > Q::NABCD ? (TABN + 2 * Q::NR) : Q::NABCD;
  // odd stride (in elements) between the buffers of neighbouring groups so
  // that equal offsets of different groups fall into different banks
  static constexpr int BUFN = NEED | 1;
};

template <int LA, int LB, int LC, int LD, typename R, int T>
__device__ __forceinline__ void eval_grp(const KParams &kp, const QGeom<R> &g, R *tab, int t, unsigned gmask,
                                         R (&acc)[Grp<LA, LB, LC, LD, R, T>::NPER], int p = 0, int P = 1) {
  using Q = QC<LA, LB, LC, LD>;
  using GP = Grp<LA, LB, LC, LD, R, T>;
  constexpr int NR = Q::NR, SZ = Q::SZ, NPER = GP::NPER, RPER = GP::RPER, INNER = GP::INNER, LI = GP::LI;
#pragma unroll
  for (int k = 0; k < NPER; ++k) acc[k] = (R)0;
  // per row: the table offsets of its first output in the three directions,
  // less the inner shell's exponent of component 0 (the row's base)
  int off[RPER];
#pragma unroll
  for (int j = 0; j < RPER; ++j) {
    const int o = (t + j * T) * INNER;
    const int i0 = INNER > 1 ? cart_e(LI, 0, 0) : 0, i1 = INNER > 1 ? cart_e(LI, 0, 1) : 0,
              i2 = INNER > 1 ? cart_e(LI, 0, 2) : 0;
    off[j] = o < Q::NABCD ? ((Q::toff(o, 0) - i0) | ((NR * SZ + Q::toff(o, 1) - i1) << 10) |
                             ((2 * NR * SZ + Q::toff(o, 2) - i2) << 20))
                          : 0;
  }
  const int nprim = g.ab_n * g.cd_n;
  int cur = -1;
  PQ<R> s;
  R pp, px, py, pz, kab;
  KetRec<R> kn;
  int ip = p / g.cd_n, iq = p - ip * g.cd_n;   // (ab, cd) indices of idx
  if (p < nprim) load_ket<R>(kp, g, iq, kn);
  for (int idx = p; idx < nprim; idx += P) {
    const KetRec<R> kc = kn;
    int ipn = ip, iqn = iq;
    prim_advance(ipn, iqn, P, g.cd_n);
    if (idx + P < nprim) load_ket<R>(kp, g, iqn, kn);
    if (ip != cur) {
      load_prim_ab<R>(kp, g, ip, s, pp, px, py, pz, kab);
      cur = ip;
    }
    set_prim_cd<R>(g, kc, s, pp, px, py, pz, kab);
    ip = ipn;
    iq = iqn;
    // each root once: lane t evaluates roots t, t+T, ... into the group buffer
    for (int r = t; r < NR; r += T) {
      R uu, ww;
      rys_root_one<NR, R>(kp, s.x, r, uu, ww);
      tab[GP::ROOTS + r] = uu;
      tab[GP::ROOTS + NR + r] = ww;
    }
    __syncwarp(gmask);
    for (int task = t; task < 3 * NR; task += T) {
      const int r = task % NR, d = task / NR;
      const R uu = tab[GP::ROOTS + r], ww = tab[GP::ROOTS + NR + r];
      const R b00 = (R)0.5 * s.r2 * uu;
      const R b10 = s.i2p * ((R)1 - s.aq * uu);
      const R b01 = s.i2q * ((R)1 - s.ap * uu);
      const R tq = s.aq * uu, tp = s.ap * uu;
      const R pa = d == 0 ? s.pax : d == 1 ? s.pay : s.paz;
      const R qc = d == 0 ? s.qcx : d == 1 ? s.qcy : s.qcz;
      const R pq = d == 0 ? s.pqx : d == 1 ? s.pqy : s.pqz;
      const R ab = d == 0 ? g.ABx : d == 1 ? g.ABy : g.ABz;
      const R cd = d == 0 ? g.CDx : d == 1 ? g.CDy : g.CDz;
      const R g0 = d == 2 ? s.pref * ww : (R)1;
      rys_2d<LA, LB, LC, LD, R>(g0, pa - tq * pq, qc + tp * pq, b00, b10, b01, ab, cd, tab + (d * NR + r) * SZ);
    }
    __syncwarp(gmask);
#pragma unroll
    for (int j = 0; j < RPER; ++j) {
      if (t + j * T < GP::ROWS) {
        const int ox = off[j] & 1023, oy = (off[j] >> 10) & 1023, oz = off[j] >> 20;
        if constexpr (INNER == 1) {
          R v = (R)0;
#pragma unroll
          for (int r = 0; r < NR; ++r) v += tab[ox + r * SZ] * tab[oy + r * SZ] * tab[oz + r * SZ];
          acc[j] += v;
        } else {
          R v[INNER];
#pragma unroll
          for (int e = 0; e < INNER; ++e) v[e] = (R)0;
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            R X[LI + 1], Y[LI + 1], Z[LI + 1];
#pragma unroll
            for (int i = 0; i <= LI; ++i) {
              X[i] = tab[ox + r * SZ + i];
              Y[i] = tab[oy + r * SZ + i];
              Z[i] = tab[oz + r * SZ + i];
            }
#pragma unroll
            for (int e = 0; e < INNER; ++e)
              v[e] += X[cart_e(LI, e, 0)] * Y[cart_e(LI, e, 1)] * Z[cart_e(LI, e, 2)];
          }
#pragma unroll
          for (int e = 0; e < INNER; ++e) acc[j * INNER + e] += v[e];
        }
      }
    }
    __syncwarp(gmask);
  }
}

// sum acc over the P primitive sub-groups of a quartet (lanes T apart)
template <typename R, int N, int T>
__device__ __forceinline__ void reduce_psplit(R (&acc)[N], int P, unsigned qmask) {
  for (int sft = T; sft < T * P; sft <<= 1) {
#pragma unroll
    for (int k = 0; k < N; ++k) acc[k] += shfl_xor_r(qmask, acc[k], sft);
  }
}

// ---------------------------------------------------------------------------
// J/K digestion.  With v = degeneracy-scaled normalised integral of the
// component quadruple (i,j,k,l) of a canonical shell quartet, the eight index
// permutations of hf.py:49-60 give J = Jh + Jh^T and K = Kh + Kh^T with
//   Jh_ij += 2 v D_kl, Jh_kl += 2 v D_ij,
//   Kh_ik += v D_jl, Kh_jk += v D_il, Kh_il += v D_jk, Kh_jl += v D_ik.
// ---------------------------------------------------------------------------
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void digest_t1(const KParams &kp, const QGeom<R> &g, const R (&acc)[QC<LA, LB, LC, LD>::NABCD],
                                          R scale, const R *__restrict__ D, double *Jh, double *Kh, int bra_key = -1) {
  using Q = QC<LA, LB, LC, LD>;
  const int n = kp.nao;
  const int a0 = g.a0, b0 = g.b0, c0 = g.c0, d0 = g.d0;
  R v[Q::NABCD];
#pragma unroll
  for (int o = 0; o < Q::NABCD; ++o) v[o] = acc[o] * (R)Q::norm(o);
  // J_ab and K blocks need D of the other pairs.  J_ab: with one quartet per
  // lane (bra_key >= 0) the lanes sharing the bra pair add their J_ab first
  R sj[Q::NA * Q::NB];
#pragma unroll
  for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
    for (int ib = 0; ib < Q::NB; ++ib) {
      R s = 0;
#pragma unroll
      for (int ic = 0; ic < Q::NC; ++ic)
#pragma unroll
        for (int id = 0; id < Q::ND; ++id)
          s += v[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id] * ldg_r(D + (c0 + ic) * n + d0 + id);
      sj[ia * Q::NB + ib] = (R)2 * scale * s;
    }
  const bool write_j = bra_key < 0 ? true : run_sums<R, Q::NA * Q::NB>(bra_key, sj);
  if (write_j) {
#pragma unroll
    for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
      for (int ib = 0; ib < Q::NB; ++ib) atomicAdd(Jh + (a0 + ia) * n + b0 + ib, to_f64(sj[ia * Q::NB + ib]));
  }
#pragma unroll
  for (int ic = 0; ic < Q::NC; ++ic)
#pragma unroll
    for (int id = 0; id < Q::ND; ++id) {
      R s = 0;
#pragma unroll
      for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
        for (int ib = 0; ib < Q::NB; ++ib)
          s += v[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id] * ldg_r(D + (a0 + ia) * n + b0 + ib);
      atomicAdd(Jh + (c0 + ic) * n + d0 + id, to_f64((R)2 * scale * s));
    }
#pragma unroll
  for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
    for (int ic = 0; ic < Q::NC; ++ic) {
      R s = 0;
#pragma unroll
      for (int ib = 0; ib < Q::NB; ++ib)
#pragma unroll
        for (int id = 0; id < Q::ND; ++id)
          s += v[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id] * ldg_r(D + (b0 + ib) * n + d0 + id);
      atomicAdd(Kh + (a0 + ia) * n + c0 + ic, to_f64(scale * s));
    }
#pragma unroll
  for (int ib = 0; ib < Q::NB; ++ib)
#pragma unroll
    for (int ic = 0; ic < Q::NC; ++ic) {
      R s = 0;
#pragma unroll
      for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
        for (int id = 0; id < Q::ND; ++id)
          s += v[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id] * ldg_r(D + (a0 + ia) * n + d0 + id);
      atomicAdd(Kh + (b0 + ib) * n + c0 + ic, to_f64(scale * s));
    }
#pragma unroll
  for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
    for (int id = 0; id < Q::ND; ++id) {
      R s = 0;
#pragma unroll
      for (int ib = 0; ib < Q::NB; ++ib)
#pragma unroll
        for (int ic = 0; ic < Q::NC; ++ic)
          s += v[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id] * ldg_r(D + (b0 + ib) * n + c0 + ic);
      atomicAdd(Kh + (a0 + ia) * n + d0 + id, to_f64(scale * s));
    }
#pragma unroll
  for (int ib = 0; ib < Q::NB; ++ib)
#pragma unroll
    for (int id = 0; id < Q::ND; ++id) {
      R s = 0;
#pragma unroll
      for (int ia = 0; ia < Q::NA; ++ia)
#pragma unroll
        for (int ic = 0; ic < Q::NC; ++ic)
          s += v[((ia * Q::NB + ib) * Q::NC + ic) * Q::ND + id] * ldg_r(D + (a0 + ia) * n + c0 + ic);
      atomicAdd(Kh + (b0 + ib) * n + d0 + id, to_f64(scale * s));
    }
}

// group version: normalised integrals are staged in buf (shared), then the
// 6 blocks' entries are distributed over the T lanes
template <int LA, int LB, int LC, int LD, typename R, int T>
__device__ __forceinline__ void digest_grp(const KParams &kp, const QGeom<R> &g,
                                           const R (&acc)[Grp<LA, LB, LC, LD, R, T>::NPER], R *buf, int t,
                                           unsigned gmask, R scale, const R *__restrict__ D, double *Jh,
                                           double *Kh) {
  using Q = QC<LA, LB, LC, LD>;
  constexpr int NA = Q::NA, NB = Q::NB, NC = Q::NC, ND = Q::ND;
  const int n = kp.nao;
  const int a0 = g.a0, b0 = g.b0, c0 = g.c0, d0 = g.d0;
  __syncwarp(gmask);
#pragma unroll
  for (int k = 0; k < Grp<LA, LB, LC, LD, R, T>::NPER; ++k) {
    const int o = Grp<LA, LB, LC, LD, R, T>::out(t, k);
    if (o < Q::NABCD) buf[o] = acc[k] * (R)Q::norm(o);
  }
  __syncwarp(gmask);
  constexpr int E0 = NA * NB, E1 = E0 + NC * ND, E2 = E1 + NA * NC, E3 = E2 + NB * NC, E4 = E3 + NA * ND,
                E5 = E4 + NB * ND;
#define V4(ia, ib, ic, id) buf[(((ia) * NB + (ib)) * NC + (ic)) * ND + (id)]
  for (int e = t; e < E5; e += T) {
    R s = 0;
    if (e < E0) {
      const int ia = e / NB, ib = e % NB;
      for (int ic = 0; ic < NC; ++ic)
        for (int id = 0; id < ND; ++id) s += V4(ia, ib, ic, id) * ldg_r(D + (c0 + ic) * n + d0 + id);
      atomicAdd(Jh + (a0 + ia) * n + b0 + ib, to_f64((R)2 * scale * s));
    } else if (e < E1) {
      const int ic = (e - E0) / ND, id = (e - E0) % ND;
      for (int ia = 0; ia < NA; ++ia)
        for (int ib = 0; ib < NB; ++ib) s += V4(ia, ib, ic, id) * ldg_r(D + (a0 + ia) * n + b0 + ib);
      atomicAdd(Jh + (c0 + ic) * n + d0 + id, to_f64((R)2 * scale * s));
    } else if (e < E2) {
      const int ia = (e - E1) / NC, ic = (e - E1) % NC;
      for (int ib = 0; ib < NB; ++ib)
        for (int id = 0; id < ND; ++id) s += V4(ia, ib, ic, id) * ldg_r(D + (b0 + ib) * n + d0 + id);
      atomicAdd(Kh + (a0 + ia) * n + c0 + ic, to_f64(scale * s));
    } else if (e < E3) {
      const int ib = (e - E2) / NC, ic = (e - E2) % NC;
      for (int ia = 0; ia < NA; ++ia)
        for (int id = 0; id < ND; ++id) s += V4(ia, ib, ic, id) * ldg_r(D + (a0 + ia) * n + d0 + id);
      atomicAdd(Kh + (b0 + ib) * n + c0 + ic, to_f64(scale * s));
    } else if (e < E4) {
      const int ia = (e - E3) / ND, id = (e - E3) % ND;
      for (int ib = 0; ib < NB; ++ib)
        for (int ic = 0; ic < NC; ++ic) s += V4(ia, ib, ic, id) * ldg_r(D + (b0 + ib) * n + c0 + ic);
      atomicAdd(Kh + (a0 + ia) * n + d0 + id, to_f64(scale * s));
    } else {
      const int ib = (e - E4) / ND, id = (e - E4) % ND;
      for (int ia = 0; ia < NA; ++ia)
        for (int ic = 0; ic < NC; ++ic) s += V4(ia, ib, ic, id) * ldg_r(D + (a0 + ia) * n + c0 + ic);
      atomicAdd(Kh + (b0 + ib) * n + d0 + id, to_f64(scale * s));
    }
  }
#undef V4
}

// ---------------------------------------------------------------------------
// work description of one (class, precision) launch: an explicit list of
// (bra pair index in class X, ket pair index in class Y), sorted on the host
// by primitive cost so that the lanes / groups of a warp run identical loops
// ---------------------------------------------------------------------------
struct ClassWork {
  const int2 *list;
  int64_t n;               // quartets in the list (with count: the list's capacity)
  int x0, y0;              // first global pair index of class X / Y
  int same;                // X == Y
  int psplit;              // P: primitive sub-groups per quartet inside one group of T*P <= 32 lanes
  int wsplit;              // W: groups per quartet; group c of W runs primitive sub-groups c*P .. c*P+P-1
                           // of W*P and digests its partial integrals itself (digestion is linear)
  int max_cost = 1;        // K_ab K_cd of the list's first (costliest) quartet
  // device count of the quartets actually in the list (lists compacted on the
  // device by the density-weighted classification); nullptr: n
  const unsigned long long *count = nullptr;
  int wide = 0;            // double-float: the tdd_wide lanes per quartet (host-side choice)
};

// quartets of a work list: the device count when the list was compacted on
// the device, else the host count
__device__ __forceinline__ int64_t work_count(const ClassWork &w) {
  return w.count ? (int64_t)__ldg(w.count) : w.n;
}

constexpr int kBlock = 128;
constexpr int kMaxWsplit = 64;

// One quartet group of the FP32 register path (one lane per quartet and
// primitive sub-group): group gid of the list's W*P sub-groups per quartet,
// Rys table rows read from the shared-memory copy tab_s of the class's root
// block.  Returns false past the end of the list (nq quartets).  Used by the
// class kernel's grid-stride loop and by the persistent multi-class kernel.
template <int LA, int LB, int LC, int LD>
__device__ __forceinline__ bool jk_f32_t1_step(const KParams &kp, const ClassWork &w, int64_t gid, int64_t nq,
                                               const float *tab_s, const float *__restrict__ D, double *Jh,
                                               double *Kh) {
  using R = float;
  const int P = w.psplit, W = w.wsplit;
  const int p = threadIdx.x % P;
  const int64_t q = gid / W;
  if (q >= nq) return false;
  const int sub = (int)(gid - q * W) * P + p;
  const int2 ij = __ldg(w.list + q);
  const QGeom<R> g = make_geom32(kp, w.x0 + ij.x, w.y0 + ij.y);
  R scale = (R)1;
  if (g.a == g.b) scale *= (R)0.5;
  if (g.c == g.d) scale *= (R)0.5;
  if (w.same && ij.x == ij.y) scale *= (R)0.5;
  const int lane = threadIdx.x & 31;
  const unsigned qmask = (P == 32) ? 0xffffffffu : (((1u << P) - 1u) << (lane & ~(P - 1)));
  R acc[QC<LA, LB, LC, LD>::NABCD];
  eval_t1<LA, LB, LC, LD, R>(kp, g, acc, sub, W * P, tab_s);
  if (P > 1) reduce_psplit<R, QC<LA, LB, LC, LD>::NABCD, 1>(acc, P, qmask);
  if (p == 0) digest_t1<LA, LB, LC, LD, R>(kp, g, acc, scale, D, Jh, Kh, P == 1 ? ij.x : -1);
  return true;
}

// copy the n-root block of the FP32 Rys table to shared memory (its rows are
// read at lane-dependent intervals: divergent global loads)
__device__ __forceinline__ void load_tab32_block(const KParams &kp, int nr, float4 *tab4) {
  const int ntab4 = kTabNint * nr * kTab32Row / 4;
  const float4 *src = reinterpret_cast<const float4 *>(kp.tab32 + rys_tab32v_offset(nr));
  for (int k = threadIdx.x; k < ntab4; k += blockDim.x) tab4[k] = __ldg(src + k);
}

template <int LA, int LB, int LC, int LD, typename R, int T>
__global__ void __launch_bounds__(kBlock) jk_kernel(KParams kp, ClassWork w, const R *__restrict__ D, double *Jh,
                                                    double *Kh) {
  const int P = w.psplit, W = w.wsplit;
  const int TP = T * P;
  const int grp = threadIdx.x / TP, p = (threadIdx.x / T) % P, t = threadIdx.x % T;
  if constexpr (T == 1 && std::is_same<R, float>::value) {
    // FP32 register path: the n-root block of the Rys table is copied to
    // shared memory once per CTA and the CTA strides over the list
    extern __shared__ __align__(16) unsigned char smem_raw[];
    load_tab32_block(kp, QC<LA, LB, LC, LD>::NR, reinterpret_cast<float4 *>(smem_raw));
    __syncthreads();
    const float *tab_s = reinterpret_cast<const float *>(smem_raw);
    const int64_t nq = work_count(w);
    for (int64_t gid = (int64_t)blockIdx.x * (kBlock / TP) + grp;; gid += (int64_t)gridDim.x * (kBlock / TP))
      if (!jk_f32_t1_step<LA, LB, LC, LD>(kp, w, gid, nq, tab_s, D, Jh, Kh)) return;
  }
  const int64_t gid = (int64_t)blockIdx.x * (kBlock / TP) + grp;
  const int64_t q = gid / W;
  const int sub = (int)(gid - q * W) * P + p;   // primitive sub-group of the W*P
  if (q >= work_count(w)) return;
  const int2 ij = __ldg(w.list + q);
  const int i = ij.x, j = ij.y;
  const int pab = w.x0 + i, pcd = w.y0 + j;
  QGeom<R> g;
  if constexpr (std::is_same<R, float>::value) g = make_geom32(kp, pab, pcd);
  else g = make_geom<R>(kp, pab, pcd, false, false);
  R scale = (R)1;
  if (g.a == g.b) scale *= (R)0.5;
  if (g.c == g.d) scale *= (R)0.5;
  if (w.same && i == j) scale *= (R)0.5;
  const int lane = threadIdx.x & 31;
  const unsigned qmask = (TP == 32) ? 0xffffffffu : (((1u << TP) - 1u) << (lane & ~(TP - 1)));
  if constexpr (T == 1) {
    R acc[QC<LA, LB, LC, LD>::NABCD];
    eval_t1<LA, LB, LC, LD, R>(kp, g, acc, sub, W * P);
    if (P > 1) reduce_psplit<R, QC<LA, LB, LC, LD>::NABCD, 1>(acc, P, qmask);
    if (p == 0) digest_t1<LA, LB, LC, LD, R>(kp, g, acc, scale, D, Jh, Kh, P == 1 ? i : -1);
  } else {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using GP = Grp<LA, LB, LC, LD, R, T>;
    R *buf = reinterpret_cast<R *>(smem_raw) + (threadIdx.x / T) * GP::BUFN;
    const unsigned gmask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));
    R acc[GP::NPER];
    eval_grp<LA, LB, LC, LD, R, T>(kp, g, buf, t, gmask, acc, sub, W * P);
    if (P > 1) reduce_psplit<R, GP::NPER, T>(acc, P, qmask);
    if (p == 0) digest_grp<LA, LB, LC, LD, R, T>(kp, g, acc, buf, t, gmask, scale, D, Jh, Kh);
  }
}

// raw integrals of an explicit quartet list (one class); perm packs, per
// canonical slot s (a,b,c,d), the original position (2 bits each) plus the
// swap flags of the bra / ket shells (bits 8, 9)
struct EriWork {
  const int *pab, *pcd;        // canonical pair indices
  const int *flags;            // bit0 swap a<->b, bit1 swap c<->d (within the pair record)
  const int64_t *out_off;      // output offset per quartet
  const int *strides;          // 4 output strides per quartet (canonical slot order)
  int64_t n;
  double *out;
  int psplit;                  // P primitive sub-groups per quartet (T*P <= 32)
};

// one quartet of the one-lane (T == 1) raw-integral path: P lanes share it
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void eri_t1_quartet(const KParams &kp, const EriWork &w, int64_t q, int p, int P,
                                               unsigned qmask, const float *tab_s) {
  using Q = QC<LA, LB, LC, LD>;
  const int fl = w.flags[q];
  const QGeom<R> g = make_geom<R>(kp, w.pab[q], w.pcd[q], fl & 1, fl & 2);
  R acc[Q::NABCD];
  eval_t1<LA, LB, LC, LD, R>(kp, g, acc, p, P, tab_s);
  if (P > 1) reduce_psplit<R, Q::NABCD, 1>(acc, P, qmask);
  if (p != 0) return;
  const int s0 = w.strides[4 * q], s1 = w.strides[4 * q + 1], s2 = w.strides[4 * q + 2], s3 = w.strides[4 * q + 3];
  double *out = w.out + w.out_off[q];
#pragma unroll
  for (int o = 0; o < Q::NABCD; ++o)
    out[Q::ca(o) * s0 + Q::cb(o) * s1 + Q::cc(o) * s2 + Q::cd(o) * s3] = to_f64(acc[o] * (R)Q::norm(o));
}

template <int LA, int LB, int LC, int LD, typename R, int T>
__global__ void __launch_bounds__(kBlock) eri_kernel(KParams kp, EriWork w) {
  using Q = QC<LA, LB, LC, LD>;
  const int P = w.psplit;
  const int TP = T * P;
  const int grp = threadIdx.x / TP, p = (threadIdx.x / T) % P, t = threadIdx.x % T;
  const int lane = threadIdx.x & 31;
  const unsigned qmask = (TP == 32) ? 0xffffffffu : (((1u << TP) - 1u) << (lane & ~(TP - 1)));
  if constexpr (T == 1) {
    // one lane group per quartet, grid-stride over the list; the FP32 path
    // copies the n-root block of the Rys table to shared memory once per CTA
    // (its rows are read at lane-dependent intervals)
    const float *tab_s = nullptr;
    if constexpr (std::is_same<R, float>::value) {
      extern __shared__ __align__(16) unsigned char smem_t[];
      load_tab32_block(kp, Q::NR, reinterpret_cast<float4 *>(smem_t));
      __syncthreads();
      tab_s = reinterpret_cast<const float *>(smem_t);
    }
    const int64_t stride = (int64_t)gridDim.x * (kBlock / TP);
    for (int64_t q = (int64_t)blockIdx.x * (kBlock / TP) + grp; q < w.n; q += stride)
      eri_t1_quartet<LA, LB, LC, LD, R>(kp, w, q, p, P, qmask, tab_s);
  } else {
    const int64_t q = (int64_t)blockIdx.x * (kBlock / TP) + grp;
    if (q >= w.n) return;
    const int fl = w.flags[q];
    const QGeom<R> g = make_geom<R>(kp, w.pab[q], w.pcd[q], fl & 1, fl & 2);
    const int s0 = w.strides[4 * q], s1 = w.strides[4 * q + 1], s2 = w.strides[4 * q + 2], s3 = w.strides[4 * q + 3];
    double *out = w.out + w.out_off[q];
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using GP = Grp<LA, LB, LC, LD, R, T>;
    R *buf = reinterpret_cast<R *>(smem_raw) + (threadIdx.x / T) * GP::BUFN;
    const unsigned gmask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));
    R acc[GP::NPER];
    eval_grp<LA, LB, LC, LD, R, T>(kp, g, buf, t, gmask, acc, p, P);
    if (P > 1) reduce_psplit<R, GP::NPER, T>(acc, P, qmask);
    if (p != 0) return;
#pragma unroll
    for (int k = 0; k < GP::NPER; ++k) {
      const int o = GP::out(t, k);
      if (o < Q::NABCD)
        out[Q::ca(o) * s0 + Q::cb(o) * s1 + Q::cc(o) * s2 + Q::cd(o) * s3] = to_f64(acc[k] * (R)Q::norm(o));
    }
  }
}

// Schwarz: Q_ab = sqrt(max_{ia,ib} |(ia ib|ia ib)|) over the pairs
// [p0, p0 + n) of one pair class; class (X|X)
template <int LA, int LB, typename R, int T>
__global__ void __launch_bounds__(kBlock) schwarz_kernel(KParams kp, int p0, int n, double *qout) {
  using Q = QC<LA, LB, LA, LB>;
  constexpr int G = kBlock / T;
  const int grp = threadIdx.x / T, t = threadIdx.x % T;
  const int i = blockIdx.x * G + grp;
  if (i >= n) return;
  const QGeom<R> g = make_geom<R>(kp, p0 + i, p0 + i, false, false);
  double m = 0.0;
  if constexpr (T == 1) {
    R acc[Q::NABCD];
    eval_t1<LA, LB, LA, LB, R>(kp, g, acc);
#pragma unroll
    for (int o = 0; o < Q::NABCD; ++o)
      if (Q::ca(o) == Q::cc(o) && Q::cb(o) == Q::cd(o)) m = fmax(m, fabs((double)(acc[o] * (R)Q::norm(o))));
  } else {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using GP = Grp<LA, LB, LA, LB, R, T>;
    R *buf = reinterpret_cast<R *>(smem_raw) + grp * GP::BUFN;
    const unsigned gmask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << ((threadIdx.x & 31) & ~(T - 1)));
    R acc[GP::NPER];
    eval_grp<LA, LB, LA, LB, R, T>(kp, g, buf, t, gmask, acc);
#pragma unroll
    for (int k = 0; k < GP::NPER; ++k) {
      const int o = GP::out(t, k);
      if (o < Q::NABCD && Q::ca(o) == Q::cc(o) && Q::cb(o) == Q::cd(o))
        m = fmax(m, fabs((double)(acc[k] * (R)Q::norm(o))));
    }
#pragma unroll
    for (int sft = T / 2; sft > 0; sft >>= 1) m = fmax(m, __shfl_xor_sync(gmask, m, sft, T));
  }
  if (t == 0) qout[p0 + i] = sqrt(m);
}

}  // namespace sf
