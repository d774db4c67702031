// md_eri.cu -- raw contracted ERIs by McMurchie-Davidson (md.cuh), FP64, one
// thread per contracted shell quartet: the second ERI engine, an independent
// cross-check of the Rys kernels on the same plans (sf_eri_plan_run_md).
#include "classes.h"
#include "launch.h"
#include "md.cuh"

namespace sf {

__constant__ MdTables c_md;

template <int LA, int LB, int LC, int LD, typename R>
__global__ void __launch_bounds__(kBlock) md_eri_kernel(KParams kp, EriWork w) {
  using Q = QC<LA, LB, LC, LD>;
  constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
  constexpr int NHAB = nherm(LAB);
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= w.n) return;
  const int fl = w.flags[q];
  const QGeom<R> g = make_geom<R>(kp, w.pab[q], w.pcd[q], fl & 1, fl & 2);
  R acc[Q::NABCD];
#pragma unroll 1
  for (int o = 0; o < Q::NABCD; ++o) acc[o] = (R)0;
  const R *recs = prims_of<R>(kp).rec;
#pragma unroll 1
  for (int ip = 0; ip < g.ab_n; ++ip) {
    R p, Px, Py, Pz, kab, i2p;
    load_rec<R>(recs + (size_t)(g.ab_off + ip) * kPrimRec, p, Px, Py, Pz, kab, i2p);
    const R PA[3] = {Px - g.Ax, Py - g.Ay, Pz - g.Az};
    const R AB[3] = {g.ABx, g.ABy, g.ABz};
    R Eab[3][LA + 1][LB + 1][LAB + 1];
#pragma unroll
    for (int d = 0; d < 3; ++d) md_hermite_e<LA, LB, R>(i2p, PA[d], PA[d] + AB[d], Eab[d]);
#pragma unroll 1
    for (int iq = 0; iq < g.cd_n; ++iq) {
      R qq, Qx, Qy, Qz, kcd, i2q;
      load_rec<R>(recs + (size_t)(g.cd_off + iq) * kPrimRec, qq, Qx, Qy, Qz, kcd, i2q);
      const R QC_[3] = {Qx - g.Cx, Qy - g.Cy, Qz - g.Cz};
      const R CD[3] = {g.CDx, g.CDy, g.CDz};
      R Ecd[3][LC + 1][LD + 1][LCD + 1];
#pragma unroll
      for (int d = 0; d < 3; ++d) md_hermite_e<LC, LD, R>(i2q, QC_[d], QC_[d] + CD[d], Ecd[d]);
      const R pq = p + qq;
      const R rho = p * qq / pq;
      const R X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
      R Rh[nherm(L)];
      md_coulomb_r<L, R>(c_md, rho, rho * (X * X + Y * Y + Z * Z), X, Y, Z, Rh);
      const R pref = kab * kcd / sqrt(pq);
#pragma unroll 1
      for (int oc = 0; oc < Q::NC * Q::ND; ++oc) {
        const int ic = oc / Q::ND, id = oc % Q::ND;
        const int cx = cart_e(LC, ic, 0), cy = cart_e(LC, ic, 1), cz = cart_e(LC, ic, 2);
        const int dx = cart_e(LD, id, 0), dy = cart_e(LD, id, 1), dz = cart_e(LD, id, 2);
        // ket contraction G_h = sum (-1)^{tau+nu+phi} E^cd E^cd E^cd R_{h + (tau,nu,phi)}
        R G[NHAB];
#pragma unroll 1
        for (int h = 0; h < NHAB; ++h) {
          const int t = c_md.t[h], u = c_md.u[h], v = c_md.v[h];
          R s = (R)0;
#pragma unroll 1
          for (int ta = 0; ta <= cx + dx; ++ta)
#pragma unroll 1
            for (int nu = 0; nu <= cy + dy; ++nu)
#pragma unroll 1
              for (int ph = 0; ph <= cz + dz; ++ph) {
                const R e = Ecd[0][cx][dx][ta] * Ecd[1][cy][dy][nu] * Ecd[2][cz][dz][ph];
                const R r = Rh[c_md.idx[t + ta][u + nu][v + ph]];
                s += ((ta + nu + ph) & 1) ? -e * r : e * r;
              }
          G[h] = s;
        }
        // bra Hermite-to-Cartesian contraction
#pragma unroll 1
        for (int oab = 0; oab < Q::NA * Q::NB; ++oab) {
          const int ia = oab / Q::NB, ib = oab % Q::NB;
          const int ax = cart_e(LA, ia, 0), ay = cart_e(LA, ia, 1), az = cart_e(LA, ia, 2);
          const int bx = cart_e(LB, ib, 0), by = cart_e(LB, ib, 1), bz = cart_e(LB, ib, 2);
          R s = (R)0;
#pragma unroll 1
          for (int t = 0; t <= ax + bx; ++t)
#pragma unroll 1
            for (int u = 0; u <= ay + by; ++u)
#pragma unroll 1
              for (int v = 0; v <= az + bz; ++v)
                s += Eab[0][ax][bx][t] * Eab[1][ay][by][u] * Eab[2][az][bz][v] * G[c_md.idx[t][u][v]];
          acc[oab * Q::NC * Q::ND + oc] += pref * s;
        }
      }
    }
  }
  const int s0 = w.strides[4 * q], s1 = w.strides[4 * q + 1], s2 = w.strides[4 * q + 2], s3 = w.strides[4 * q + 3];
  double *out = w.out + w.out_off[q];
#pragma unroll 1
  for (int o = 0; o < Q::NABCD; ++o)
    out[Q::ca(o) * s0 + Q::cb(o) * s1 + Q::cc(o) * s2 + Q::cd(o) * s3] = to_f64(acc[o] * (R)Q::norm(o));
}

// host copy of the Hermite tables into constant memory (once per device)
cudaError_t prepare_md() {
  MdTables tb{};
  for (int h = 0; h < nherm(kMdMaxL); ++h) {
    tb.t[h] = (unsigned char)herm_t(h);
    tb.u[h] = (unsigned char)herm_u(h);
    tb.v[h] = (unsigned char)herm_v(h);
  }
  for (int t = 0; t <= kMdMaxL; ++t)
    for (int u = 0; u <= kMdMaxL; ++u)
      for (int v = 0; v <= kMdMaxL; ++v) tb.idx[t][u][v] = (short)(t + u + v <= kMdMaxL ? herm_index(t, u, v) : 0);
  return cudaMemcpyToSymbol(c_md, &tb, sizeof(tb));
}

template <int LA, int LB, int LC, int LD>
static cudaError_t run_md_eri(const KParams &kp, const EriWork &w, cudaStream_t st) {
  if (w.n <= 0) return cudaSuccess;
  md_eri_kernel<LA, LB, LC, LD, double><<<(unsigned)((w.n + kBlock - 1) / kBlock), kBlock, 0, st>>>(kp, w);
  return cudaGetLastError();
}

cudaError_t launch_md_eri(int cls, const KParams &kp, const EriWork &w, cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_md_eri<la, lb, lc, ld>(kp, w, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sf
