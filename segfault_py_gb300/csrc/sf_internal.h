// sf_internal.h -- shared definitions of libsegfock (host + device).
//
// Data layout in device memory (all owned by the sf_handle):
//   shells   : SoA  l, nprim, ao_offset, atom, centre x/y/z
//   pairs    : canonical shell pairs (a,b) with l_a >= l_b (a >= b when
//              l_a == l_b), grouped by pair class ss,ps,pp,ds,dp,dd and, after
//              sf_schwarz, sorted by Schwarz bound Q_ab descending inside each
//              class.  A pair record holds a, b, the offset and count of its
//              primitive pairs, and Q_ab.
//   prims    : one 8-value record per primitive pair (alpha_i, beta_j):
//              p = alpha+beta, P = (alpha A + beta B)/p, 0.5/p and
//              K~ = c_i c_j exp(-alpha beta/p |AB|^2) sqrt(2) pi^(5/4) / p,
//              in FP64 and FP32.  K~_ab K~_cd / sqrt(p+q) is the full
//              prefactor 2 pi^(5/2) / (p q sqrt(p+q)) E_ab E_cd of a primitive
//              quartet.
//   rys      : root/weight tables, see rys_table.cpp.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sf {

constexpr int kMaxL = 2;
constexpr int kMaxPrim = 16;
constexpr int kNumPairClass = 6;   // ss ps pp ds dp dd
constexpr int kNumClass = 21;      // canonical (pair class X >= pair class Y)
constexpr int kMaxRoots = 5;       // L <= 8 -> 5 roots (4 for L<=7 ...)

// Rys root tables: x in [0, kTabXmax) split into unit intervals; on each a
// polynomial in s = 2 (x - j) - 1 per root u_i (= t_i^2) and weight w_i.
constexpr int kTabNint = 64;
constexpr double kTabXmax = 64.0;
constexpr int kTabDeg64 = 11;
constexpr int kTabDeg32 = 6;

// offset (in elements) of the n-root block of a table of degree deg
__host__ __device__ constexpr int rys_tab_offset(int n, int deg) {
  // blocks for n = 1..n-1 precede: sum_{m<n} kTabNint*(deg+1)*2m
  return kTabNint * (deg + 1) * (n - 1) * n;
}
__host__ __device__ constexpr int rys_tab_size(int deg) { return rys_tab_offset(kMaxRoots + 1, deg); }

// Layout of the FP32 table read by the kernels: per n-root block, interval j,
// root r, one row of kTab32Row floats holding the coefficient pairs
// (u_k, w_k) from k = kTabDeg32 down to 0 (the Horner order): one root costs
// kTabDeg32+1 eight-byte loads of one contiguous row (no padding: the
// kernels that read it are bound by L1 bytes).
constexpr int kTab32Row = 2 * (kTabDeg32 + 1);
__host__ __device__ constexpr int rys_tab32v_offset(int n) { return kTabNint * kTab32Row * ((n - 1) * n / 2); }
__host__ __device__ constexpr int rys_tab32v_size() { return rys_tab32v_offset(kMaxRoots + 1); }

// Layout of the double-float copy of the FP64 table (in 16-byte units): per
// n-root block, interval j, root r, the kTabDeg64+1 coefficients from
// k = kTabDeg64 down to 0, each (u_hi, u_lo, w_hi, w_lo).
__host__ __device__ constexpr int rys_tabdd_offset(int n) { return kTabNint * (kTabDeg64 + 1) * ((n - 1) * n / 2); }
__host__ __device__ constexpr int rys_tabdd_size() { return rys_tabdd_offset(kMaxRoots + 1); }

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int pair_class_of(int la, int lb) {  // la >= lb
  return la * (la + 1) / 2 + lb;
}

// Cartesian exponents of component i of shell l, reference order
// (molecule.py:138-153): s; x,y,z; xx,xy,xz,yy,yz,zz
__host__ __device__ constexpr int cart_e(int l, int i, int d) {
  return l == 0 ? 0
       : l == 1 ? (i == d ? 1 : 0)
       : /* l == 2 */ (d == 0 ? (i == 0 ? 2 : (i == 1 || i == 2) ? 1 : 0)
                    : d == 1 ? (i == 3 ? 2 : (i == 1 || i == 4) ? 1 : 0)
                             : (i == 5 ? 2 : (i == 2 || i == 4) ? 1 : 0));
}
// sqrt((2l-1)!! / prod (2l_d - 1)!!): 1 for s, p; d: xx,yy,zz -> 1, xy,xz,yz -> sqrt(3)
__host__ __device__ constexpr double cart_norm(int l, int i) {
  return (l == 2 && (i == 1 || i == 2 || i == 4)) ? 1.7320508075688772935 : 1.0;
}

struct DevShells {
  const int *l, *nprim, *ao, *atom;
  const double *cx, *cy, *cz;
  const float *cx32, *cy32, *cz32;   // single-precision copies for the FP32 kernels
};

struct DevPairs {
  const int *a, *b, *poff, *np;
  const double *q;
};

// primitive-pair records (array of structures, 8 values each so that a
// record is read with two vector loads in FP32 and three in FP64; the
// exponents alpha, beta of the two primitives are read only by gradients):
//   [p, Px, Py, Pz, K~, 0.5/p, alpha, beta]
constexpr int kPrimRec = 8;
template <typename R>
struct DevPrims {
  const R *rec;
};

struct RysAsym {
  double r[kMaxRoots + 1][kMaxRoots];   // u_i * x as x -> inf
  double w[kMaxRoots + 1][kMaxRoots];   // w_i * sqrt(x) as x -> inf
};
struct RysAsym32 {                      // the same constants rounded to FP32
  float r[kMaxRoots + 1][kMaxRoots];
  float w[kMaxRoots + 1][kMaxRoots];
};

// host-side: build tables (rys_table.cpp)
void rys_build_tables(double *tab64, float *tab32, RysAsym *asym);
void rys_eval_host(const double *tab64, const float *tab32, const RysAsym &as, int n, double x, int fp32,
                   double *u, double *w);

}  // namespace sf
