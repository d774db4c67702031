// grad.cuh -- two-electron part of the analytic RHF nuclear gradient.
//
// The reference has no gradients.  With E2 = 1/2 sum (pq|rs) [D_pq D_rs -
// 1/2 D_pr D_qs] the derivative with respect to a nuclear coordinate, at fixed
// density (the Pulay term -sum W dS is added by the one-electron part), is
//
//   dE2/dR = sum_{canonical shell quartets} m(ab,cd) sum_{ijkl} G_ijkl d(ij|kl)/dR
//   G_ijkl = 1/2 D_ij D_kl - 1/8 (D_ik D_jl + D_il D_jk),
//
// m = 8 / 2^(d_ab + d_cd + d_(ab,cd)) the number of index permutations of the
// quartet.  A Cartesian Gaussian on centre A obeys
// d phi_a / dA_x = 2 alpha phi_{a+1x} - a_x phi_{a-1x}, so in the Rys
// factorisation only the x 2-D integral changes:
//   dIx/dA_x = 2 alpha Ix(a_x+1, ...) - a_x Ix(a_x-1, ...).
// The 2-D tables are therefore built for the class extended by one unit on A,
// B and C ((la+1 lb+1 | lc+1 ld), same recurrences as the energy kernels, one
// more root when the total angular momentum becomes odd), and G is contracted
// on the fly:  g_A,x += 2 alpha sum_o w_o Ix(+A) - sum_o a_x(o) w_o Ix(-A) with
// w_o = G_o Iy Iz, likewise B and C; centre D follows from translational
// invariance, g_D = -(g_A + g_B + g_C).
#pragma once
#include "quartet.cuh"

namespace sf {

template <int LA, int LB, int LC, int LD>
struct QG {
  using Q = QC<LA, LB, LC, LD>;
  static constexpr int SZE = (LA + 2) * (LB + 2) * (LC + 2) * (LD + 1);   // extended 2-D table
  static constexpr int NRG = (Q::L + 1) / 2 + 1;                          // roots for degree L+1
  static constexpr int SA = (LB + 2) * (LC + 2) * (LD + 1), SB = (LC + 2) * (LD + 1), SC = LD + 1;
  __host__ __device__ static constexpr int eoff(int o, int d) {
    return ((cart_e(LA, Q::ca(o), d) * (LB + 2) + cart_e(LB, Q::cb(o), d)) * (LC + 2) + cart_e(LC, Q::cc(o), d)) *
               (LD + 1) +
           cart_e(LD, Q::cd(o), d);
  }
};

// lanes per quartet of the gradient kernels (bigger tables than the energy);
// T = 1 keeps everything in registers
__host__ __device__ constexpr int tgrad(int nabcd) {
  return nabcd <= 18 ? 1 : nabcd <= 27 ? 4 : nabcd <= 81 ? 8 : nabcd <= 216 ? 16 : 32;
}

// per arithmetic: FP32 values take half the registers, so the FP32 kernels
// keep quartets of up to 27 outputs in one lane (measured: faster up to 27,
// slower with fewer lanes beyond)
template <typename R>
__host__ __device__ constexpr int tgrad_r(int nabcd) {
  if constexpr (sizeof(R) == sizeof(float)) return nabcd <= 27 ? 1 : tgrad(nabcd);
  else return tgrad(nabcd);
}

template <int LA, int LB, int LC, int LD, typename R, int T>
struct GGrp {
  using Q = QC<LA, LB, LC, LD>;
  using G = QG<LA, LB, LC, LD>;
  static constexpr int NPER = (Q::NABCD + T - 1) / T;
  static constexpr int TABN = 3 * G::NRG * G::SZE;
  static constexpr int ROOTS = TABN;
  static constexpr int BUFN = (TABN + 2 * G::NRG) | 1;
};

template <typename R>
__device__ __forceinline__ void load_exps(const KParams &kp, int prim, R &e0, R &e1) {
  const R *rec = prims_of<R>(kp).rec + (size_t)prim * kPrimRec + 6;
  e0 = ldg_r(rec);
  e1 = ldg_r(rec + 1);
}

// T == 1: one lane per quartet, every table in registers, compile-time indices
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void grad_t1(const KParams &kp, const QGeom<R> &g, const R (&gam)[QC<LA, LB, LC, LD>::NABCD],
                                        int p, int P, R (&gA)[3], R (&gB)[3], R (&gC)[3]) {
  using Q = QC<LA, LB, LC, LD>;
  using G = QG<LA, LB, LC, LD>;
  constexpr int NR = G::NRG, SZ = G::SZE;
  const int nprim = g.ab_n * g.cd_n;
  int cur = -1;
  PQ<R> s;
  R pp, px, py, pz, kab, al = 0, be = 0;
  for (int idx = p; idx < nprim; idx += P) {
    const int ip = idx / g.cd_n, iq = idx - ip * g.cd_n;
    if (ip != cur) {
      load_prim_ab<R>(kp, g, ip, s, pp, px, py, pz, kab);
      load_exps<R>(kp, g.ab_off + ip, al, be);
      cur = ip;
    }
    load_prim_cd<R>(kp, g, iq, s, pp, px, py, pz, kab);
    R ga, gd;
    load_exps<R>(kp, g.cd_off + iq, ga, gd);
    R u[NR], wr[NR];
    rys_roots_all<NR, R>(kp, s.x, u, wr);
    R sp[3][3], sm[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) sp[c][d] = sm[c][d] = (R)0;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const R uu = u[r];
      const R b00 = (R)0.5 * s.r2 * uu;
      const R b10 = s.i2p * ((R)1 - s.aq * uu);
      const R b01 = s.i2q * ((R)1 - s.ap * uu);
      const R tq = s.aq * uu, tp = s.ap * uu;
      R I[3][SZ];
      rys_2d<LA + 1, LB + 1, LC + 1, LD, R>((R)1, s.pax - tq * s.pqx, s.qcx + tp * s.pqx, b00, b10, b01, g.ABx,
                                            g.CDx, I[0]);
      rys_2d<LA + 1, LB + 1, LC + 1, LD, R>((R)1, s.pay - tq * s.pqy, s.qcy + tp * s.pqy, b00, b10, b01, g.ABy,
                                            g.CDy, I[1]);
      rys_2d<LA + 1, LB + 1, LC + 1, LD, R>(s.pref * wr[r], s.paz - tq * s.pqz, s.qcz + tp * s.pqz, b00, b10, b01,
                                            g.ABz, g.CDz, I[2]);
#pragma unroll
      for (int o = 0; o < Q::NABCD; ++o) {
        const R ix = I[0][G::eoff(o, 0)], iy = I[1][G::eoff(o, 1)], iz = I[2][G::eoff(o, 2)];
        const R wd[3] = {gam[o] * iy * iz, gam[o] * ix * iz, gam[o] * ix * iy};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int e = G::eoff(o, d);
          const int ea = cart_e(LA, Q::ca(o), d), eb = cart_e(LB, Q::cb(o), d), ec = cart_e(LC, Q::cc(o), d);
          sp[0][d] += wd[d] * I[d][e + G::SA];
          sp[1][d] += wd[d] * I[d][e + G::SB];
          sp[2][d] += wd[d] * I[d][e + G::SC];
          if (ea) sm[0][d] += (R)ea * wd[d] * I[d][e - G::SA];
          if (eb) sm[1][d] += (R)eb * wd[d] * I[d][e - G::SB];
          if (ec) sm[2][d] += (R)ec * wd[d] * I[d][e - G::SC];
        }
      }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gA[d] += (R)2 * al * sp[0][d] - sm[0][d];
      gB[d] += (R)2 * be * sp[1][d] - sm[1][d];
      gC[d] += (R)2 * ga * sp[2][d] - sm[2][d];
    }
  }
}

template <int LA, int LB, int LC, int LD, typename R, int T, typename A>
__device__ __forceinline__ void grad_quartet(const KParams &kp, const ClassWork &w, const R *__restrict__ D, A *grad);

// Gradient contributions of a CTA are summed in shared memory (3 slots per
// atom) and written with one atomic per slot at the end: all quartets add
// into the same 3*natom words, so per-quartet global atomics serialise.
constexpr int kGradSmemAtoms = 512;   // larger molecules add to global memory directly

// Per-CTA sums: FP32 for the FP32 kernels (shared-memory FP32 atomic adds are
// native; FP64 ones are compare-and-swap loops whose FP64 adds, retried on
// every collision of the lanes' atoms, kept the 1/64-rate FP64 pipe a third
// to half busy), FP64 for the FP64 and double-float kernels.
template <typename R>
using GradAcc = typename std::conditional<std::is_same<R, float>::value, float, double>::type;

__device__ __forceinline__ double acc_to_f64(float v) { return f2d_alu(v); }
__device__ __forceinline__ double acc_to_f64(double v) { return v; }
__device__ __forceinline__ float acc_value(float v, float) { return v; }
template <typename V>
__device__ __forceinline__ double acc_value(V v, double) { return to_f64(v); }

template <int LA, int LB, int LC, int LD, typename R, int T>
__global__ void __launch_bounds__(kBlock) grad_kernel(KParams kp, ClassWork w, const R *__restrict__ D, double *grad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using GP0 = GGrp<LA, LB, LC, LD, R, T>;
  using A = GradAcc<R>;
  const bool cta_sum = kp.natom <= kGradSmemAtoms;
  A *sgrad = reinterpret_cast<A *>(smem_raw + (T == 1 ? 0 : (size_t)(kBlock / T) * GP0::BUFN * sizeof(R)));
  const int TP0 = T * w.psplit;
  const int64_t nq = work_count(w);
  const int64_t qfirst = ((int64_t)blockIdx.x * (kBlock / TP0)) / w.wsplit;
  if (qfirst >= nq) return;   // the whole CTA is past the end of the list
  if (cta_sum) {
    for (int i = threadIdx.x; i < 3 * kp.natom; i += blockDim.x) sgrad[i] = (A)0;
    __syncthreads();
  }
  const int64_t q0 = ((int64_t)blockIdx.x * (kBlock / TP0) + threadIdx.x / TP0) / w.wsplit;
  if (q0 < nq) {
    if (cta_sum) grad_quartet<LA, LB, LC, LD, R, T, A>(kp, w, D, sgrad);
    else grad_quartet<LA, LB, LC, LD, R, T, double>(kp, w, D, grad);
  }
  if (cta_sum) {
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * kp.natom; i += blockDim.x)
      if (sgrad[i] != (A)0) atomicAdd(grad + i, acc_to_f64(sgrad[i]));
  }
}

template <int LA, int LB, int LC, int LD, typename R, int T, typename A>
__device__ __forceinline__ void grad_quartet(const KParams &kp, const ClassWork &w, const R *__restrict__ D,
                                             A *grad) {
  using Q = QC<LA, LB, LC, LD>;
  using G = QG<LA, LB, LC, LD>;
  using GP = GGrp<LA, LB, LC, LD, R, T>;
  constexpr int NR = G::NRG, SZ = G::SZE, NPER = GP::NPER;
  const int P = w.psplit, W = w.wsplit;
  const int TP = T * P;
  const int grp = threadIdx.x / TP, t = threadIdx.x % T;
  const int64_t gid = (int64_t)blockIdx.x * (kBlock / TP) + grp;
  const int64_t q = gid / W;
  const int pl = (threadIdx.x / T) % P;
  const int sub = (int)(gid - q * W) * P + pl;   // primitive sub-group of the W*P
  const int2 ij = __ldg(w.list + q);
  const int pab = w.x0 + ij.x, pcd = w.y0 + ij.y;
  const QGeom<R> g = make_geom<R>(kp, pab, pcd, false, false);
  R scale = (R)8;
  if (g.a == g.b) scale *= (R)0.5;
  if (g.c == g.d) scale *= (R)0.5;
  if (w.same && ij.x == ij.y) scale *= (R)0.5;
  const int lane = threadIdx.x & 31;
  const unsigned qmask = (TP == 32) ? 0xffffffffu : (((1u << TP) - 1u) << (lane & ~(TP - 1)));
  const unsigned gmask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *tab = reinterpret_cast<R *>(smem_raw) + (threadIdx.x / T) * GP::BUFN;

  // G_o of this lane's outputs (normalised, permutation count folded in),
  // packed table offsets and Cartesian exponents of a, b, c per direction
  const int n = kp.nao;
  const int a0 = g.a0, b0 = g.b0, c0 = g.c0, d0 = g.d0;
  R gam[NPER];
  int off[NPER], ex[NPER];
#pragma unroll
  for (int k = 0; k < NPER; ++k) {
    const int o = t + k * T;
    gam[k] = (R)0;
    off[k] = 0;
    ex[k] = 0;
    if (o < Q::NABCD) {
      const int i = a0 + Q::ca(o), j = b0 + Q::cb(o), kk = c0 + Q::cc(o), l = d0 + Q::cd(o);
      const R Dij = ldg_r(D + i * n + j), Dkl = ldg_r(D + kk * n + l), Dik = ldg_r(D + i * n + kk);
      const R Djl = ldg_r(D + j * n + l), Dil = ldg_r(D + i * n + l), Djk = ldg_r(D + j * n + kk);
      gam[k] = scale * (R)Q::norm(o) * ((R)0.5 * Dij * Dkl - (R)0.125 * (Dik * Djl + Dil * Djk));
      off[k] = G::eoff(o, 0) | (G::eoff(o, 1) << 10) | (G::eoff(o, 2) << 20);
#pragma unroll
      for (int d = 0; d < 3; ++d)
        ex[k] |= (cart_e(LA, Q::ca(o), d) | (cart_e(LB, Q::cb(o), d) << 2) | (cart_e(LC, Q::cc(o), d) << 4)) << (6 * d);
    }
  }
  R gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0}, gC[3] = {0, 0, 0};
  if constexpr (T == 1) {
    grad_t1<LA, LB, LC, LD, R>(kp, g, gam, sub, W * P, gA, gB, gC);
  } else {
  const int nprim = g.ab_n * g.cd_n;
  int cur = -1;
  PQ<R> s;
  R pp, px, py, pz, kab, al = 0, be = 0;
  for (int idx = sub; idx < nprim; idx += W * P) {
    const int ip = idx / g.cd_n, iq = idx - ip * g.cd_n;
    if (ip != cur) {
      load_prim_ab<R>(kp, g, ip, s, pp, px, py, pz, kab);
      load_exps<R>(kp, g.ab_off + ip, al, be);
      cur = ip;
    }
    load_prim_cd<R>(kp, g, iq, s, pp, px, py, pz, kab);
    R ga, gd;
    load_exps<R>(kp, g.cd_off + iq, ga, gd);
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
      rys_2d<LA + 1, LB + 1, LC + 1, LD, R>(g0, pa - tq * pq, qc + tp * pq, b00, b10, b01, ab, cd,
                                            tab + (d * NR + r) * SZ);
    }
    __syncwarp(gmask);
    R sp[3][3], sm[3][3];   // [centre A,B,C][direction]: + and - shift sums
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d) sp[c][d] = sm[c][d] = (R)0;
#pragma unroll
    for (int k = 0; k < NPER; ++k) {
      if (t + k * T < Q::NABCD) {
        const int o3[3] = {off[k] & 1023, (off[k] >> 10) & 1023, off[k] >> 20};
#pragma unroll
        for (int r = 0; r < NR; ++r) {
          const R *tx = tab + r * SZ + o3[0];
          const R *ty = tab + (NR + r) * SZ + o3[1];
          const R *tz = tab + (2 * NR + r) * SZ + o3[2];
          const R ix = tx[0], iy = ty[0], iz = tz[0];
          const R wd[3] = {gam[k] * iy * iz, gam[k] * ix * iz, gam[k] * ix * iy};
          const R *td[3] = {tx, ty, tz};
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const int e = ex[k] >> (6 * d);
            const int ea = e & 3, eb = (e >> 2) & 3, ec = (e >> 4) & 3;
            sp[0][d] += wd[d] * td[d][G::SA];
            sp[1][d] += wd[d] * td[d][G::SB];
            sp[2][d] += wd[d] * td[d][G::SC];
            if (ea) sm[0][d] += (R)ea * wd[d] * td[d][-G::SA];
            if (eb) sm[1][d] += (R)eb * wd[d] * td[d][-G::SB];
            if (ec) sm[2][d] += (R)ec * wd[d] * td[d][-G::SC];
          }
        }
      }
    }
    __syncwarp(gmask);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gA[d] += (R)2 * al * sp[0][d] - sm[0][d];
      gB[d] += (R)2 * be * sp[1][d] - sm[1][d];
      gC[d] += (R)2 * ga * sp[2][d] - sm[2][d];
    }
  }
  }
  // sum over the T x P lanes of the quartet
#pragma unroll
  for (int d = 0; d < 3; ++d)
    for (int sft = 1; sft < TP; sft <<= 1) {
      gA[d] += shfl_xor_r(qmask, gA[d], sft);
      gB[d] += shfl_xor_r(qmask, gB[d], sft);
      gC[d] += shfl_xor_r(qmask, gC[d], sft);
    }
  if (t == 0 && pl == 0) {
    const int at_a = kp.sh.atom[g.a], at_b = kp.sh.atom[g.b], at_c = kp.sh.atom[g.c], at_d = kp.sh.atom[g.d];
    R gD[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gD[d] = -(gA[d] + gB[d] + gC[d]);
      atomicAdd(grad + 3 * at_c + d, acc_value(gC[d], A()));
      atomicAdd(grad + 3 * at_d + d, acc_value(gD[d], A()));
    }
    // centres a, b: with one quartet per lane, the lanes sharing the bra pair
    // (consecutive in the cost-sorted list) add their forces first
    R gab[6] = {gA[0], gA[1], gA[2], gB[0], gB[1], gB[2]};
    const bool write = TP > 1 ? true : run_sums<R, 6>(ij.x, gab);
    if (write) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        atomicAdd(grad + 3 * at_a + d, acc_value(gab[d], A()));
        atomicAdd(grad + 3 * at_b + d, acc_value(gab[3 + d], A()));
      }
    }
  }
}

// Primitive split of one gradient launch.  The energy kernel's split S = P*W
// of the list is re-cut for this kernel's T (as many sub-groups inside the
// T*P <= 32 lanes as fit, the rest as separate groups) and then doubled while
// the list's lanes stay below 8 resident warps per SM sub-partition: a
// derivative quartet costs several energy quartets, so the few-quartet
// launches (the accurate tier above all) otherwise run at the latency of one
// quartet's primitive loop on a fraction of the SMs.  Every sub-group keeps at
// least one primitive quartet of the list's costliest quartet.
inline ClassWork grad_work(const ClassWork &w, int T, int nsm) {
  int S = (w.psplit < 1 ? 1 : w.psplit) * (w.wsplit < 1 ? 1 : w.wsplit);
  const int64_t fill = (int64_t)(nsm < 1 ? 1 : nsm) * 4 * 8 * 32;
  while (w.n * T * S < fill && 2 * S <= w.max_cost && 2 * S <= (32 / T) * kMaxWsplit) S *= 2;
  int P = S;
  while (T * P > 32) P >>= 1;
  ClassWork w2 = w;
  w2.psplit = P;
  w2.wsplit = S / P < kMaxWsplit ? S / P : kMaxWsplit;
  return w2;
}

template <int LA, int LB, int LC, int LD, typename R>
constexpr size_t grad_smem() {
  constexpr int T = tgrad_r<R>(QC<LA, LB, LC, LD>::NABCD);
  return (T == 1 ? 0 : (size_t)(kBlock / T) * GGrp<LA, LB, LC, LD, R, T>::BUFN * sizeof(R)) +
         3 * kGradSmemAtoms * sizeof(double);
}

}  // namespace sf
