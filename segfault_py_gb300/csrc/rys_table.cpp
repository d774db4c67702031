// rys_table.cpp -- Rys quadrature root/weight tables for the GPU kernels.
//
// The reference evaluates one fixed 5-point rule from fitted formulas
// (root5, src/hf/core/core.f90:232-812) for every primitive quartet, whatever
// its angular momentum.  The kernels here use the n = floor(L/2)+1 point rule
// (exact for the degree-L polynomial integrand, so identical integrals to
// rounding) and need it for n = 1..5, so the rules are generated here from the
// definition:
//
//   sum_i w_i u_i^m = F_m(x) = int_0^1 t^(2m) exp(-x t^2) dt,   m < 2n,
//
// i.e. the Gauss rule of the measure exp(-x t^2) dt on [0,1] in u = t^2.
// Generation: the measure is discretised with M-point Gauss-Legendre in t on
// [0, T] (T = 1, or 10/sqrt(x) for x > 100 where exp(-100) is negligible);
// the Stieltjes procedure gives the recurrence coefficients; the nodes are
// the eigenvalues of the Jacobi matrix (Sturm-sequence bisection to full
// precision); the weights follow from the Christoffel function
// 1/w_i = sum_j p_j(u_i)^2 / ||p_j||^2.
//
// Tables: for x in [0, 64) on unit intervals a Chebyshev interpolant of degree
// 11 (FP64) or 6 (FP32) per function, stored as monomial coefficients in
// s = 2(x-j)-1 so that the device evaluates it by Horner.  For x >= 64 the
// rule is the large-x limit u_i = r_i / x, w_i = W_i / sqrt(x) (the half-range
// Gauss-Hermite rule; the neglected terms are O(exp(-x))).
#include <cmath>
#include <cstring>
#include <vector>

#include "sf_internal.h"

namespace sf {
namespace {

constexpr int kGL = 200;

struct GaussLegendre {
  double x[kGL], w[kGL];
  GaussLegendre() {
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < (kGL + 1) / 2; ++i) {
      double z = std::cos(pi * (i + 0.75) / (kGL + 0.5)), dp = 1.0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = 0.0;
        for (int k = 1; k <= kGL; ++k) {
          double p2 = p1;
          p1 = p0;
          p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
        }
        dp = kGL * (z * p0 - p1) / (z * z - 1.0);
        double dz = p0 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-16) break;
      }
      x[i] = -z;
      x[kGL - 1 - i] = z;
      w[i] = w[kGL - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
  }
};

const GaussLegendre &gl() {
  static GaussLegendre g;
  return g;
}

// exact n-point rule at x (u ascending)
void rys_exact(int n, double x, double *u, double *w) {
  const GaussLegendre &G = gl();
  const double T = (x <= 100.0) ? 1.0 : 10.0 / std::sqrt(x);
  double uu[kGL], om[kGL], p0[kGL], p1[kGL];
  for (int k = 0; k < kGL; ++k) {
    double t = 0.5 * T * (G.x[k] + 1.0);
    uu[k] = t * t;
    om[k] = 0.5 * T * G.w[k] * std::exp(-x * t * t);
    p0[k] = 1.0;
    p1[k] = 0.0;
  }
  double al[kMaxRoots], be[kMaxRoots], hprev = 1.0;
  for (int j = 0; j < n; ++j) {
    double h = 0.0, hu = 0.0;
    for (int k = 0; k < kGL; ++k) {
      double v = om[k] * p0[k] * p0[k];
      h += v;
      hu += v * uu[k];
    }
    al[j] = hu / h;
    be[j] = (j == 0) ? h : h / hprev;
    hprev = h;
    for (int k = 0; k < kGL; ++k) {
      double pn = (uu[k] - al[j]) * p0[k] - (j ? be[j] : 0.0) * p1[k];
      p1[k] = p0[k];
      p0[k] = pn;
    }
  }
  auto below = [&](double lam) {  // eigenvalues of the Jacobi matrix below lam
    int c = 0;
    double d = al[0] - lam;
    if (d < 0) ++c;
    for (int i = 1; i < n; ++i) {
      if (d == 0.0) d = 1e-300;
      d = al[i] - lam - be[i] / d;
      if (d < 0) ++c;
    }
    return c;
  };
  for (int i = 0; i < n; ++i) {
    double lo = 0.0, hi = 1.0;
    for (int it = 0; it < 300; ++it) {
      double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (below(mid) > i) hi = mid; else lo = mid;
    }
    double z = 0.5 * (lo + hi);
    u[i] = z;
    double s = 0.0, q0 = 1.0, q1 = 0.0, hj = 1.0;
    for (int j = 0; j < n; ++j) {
      hj *= be[j];
      s += q0 * q0 / hj;
      double qn = (z - al[j]) * q0 - (j ? be[j] : 0.0) * q1;
      q1 = q0;
      q0 = qn;
    }
    w[i] = 1.0 / s;
  }
}

// Chebyshev coefficients -> monomial coefficients in s (degree D)
void cheb_to_mono(const double *c, int D, double *m) {
  std::vector<double> tm1(D + 2, 0.0), t0(D + 2, 0.0), tp1(D + 2, 0.0);
  tm1[0] = 1.0;
  t0[1] = 1.0;
  for (int i = 0; i <= D; ++i) m[i] = 0.0;
  m[0] += c[0];
  if (D >= 1) m[1] += c[1];
  for (int k = 1; k < D; ++k) {
    for (int i = 0; i <= D; ++i) tp1[i] = -tm1[i] + (i > 0 ? 2.0 * t0[i - 1] : 0.0);
    for (int i = 0; i <= D; ++i) m[i] += c[k + 1] * tp1[i];
    tm1 = t0;
    t0 = tp1;
  }
}

template <typename T>
void fill_table(T *tab, int deg) {
  const double pi = 3.14159265358979323846;
  std::vector<double> sk(deg + 1), vals((deg + 1) * 2 * kMaxRoots), c(deg + 1), m(deg + 1);
  for (int k = 0; k <= deg; ++k) sk[k] = std::cos(pi * (k + 0.5) / (deg + 1));
  for (int n = 1; n <= kMaxRoots; ++n) {
    T *blk = tab + rys_tab_offset(n, deg);
    for (int j = 0; j < kTabNint; ++j) {
      for (int k = 0; k <= deg; ++k) {
        double x = j + 0.5 * (sk[k] + 1.0);
        rys_exact(n, x, &vals[k * 2 * n], &vals[k * 2 * n + n]);
      }
      for (int f = 0; f < 2 * n; ++f) {
        for (int i = 0; i <= deg; ++i) {
          double s = 0.0;
          for (int k = 0; k <= deg; ++k) s += vals[k * 2 * n + f] * std::cos(i * std::acos(sk[k]));
          c[i] = s * 2.0 / (deg + 1) * (i == 0 ? 0.5 : 1.0);
        }
        cheb_to_mono(c.data(), deg, m.data());
        for (int i = 0; i <= deg; ++i) blk[(j * (deg + 1) + i) * 2 * n + f] = (T)m[i];
      }
    }
  }
}

}  // namespace

void rys_build_tables(double *tab64, float *tab32, RysAsym *asym) {
  fill_table<double>(tab64, kTabDeg64);
  fill_table<float>(tab32, kTabDeg32);
  const double X = 1e7;
  for (int n = 1; n <= kMaxRoots; ++n) {
    double u[kMaxRoots], w[kMaxRoots];
    rys_exact(n, X, u, w);
    for (int i = 0; i < n; ++i) {
      asym->r[n][i] = u[i] * X;
      asym->w[n][i] = w[i] * std::sqrt(X);
    }
  }
}

void rys_eval_host(const double *tab64, const float *tab32, const RysAsym &as, int n, double x, int fp32,
                   double *u, double *w) {
  if (x >= kTabXmax) {
    for (int i = 0; i < n; ++i) {
      u[i] = as.r[n][i] / x;
      w[i] = as.w[n][i] / std::sqrt(x);
    }
    return;
  }
  int j = (int)x;
  double s = 2.0 * (x - j) - 1.0;
  int deg = fp32 ? kTabDeg32 : kTabDeg64;
  for (int f = 0; f < 2 * n; ++f) {
    double v;
    if (fp32) {
      const float *c = tab32 + rys_tab_offset(n, deg) + j * (deg + 1) * 2 * n + f;
      float vf = c[deg * 2 * n], sf_ = (float)s;
      for (int i = deg - 1; i >= 0; --i) vf = vf * sf_ + c[i * 2 * n];
      v = vf;
    } else {
      const double *c = tab64 + rys_tab_offset(n, deg) + j * (deg + 1) * 2 * n + f;
      v = c[deg * 2 * n];
      for (int i = deg - 1; i >= 0; --i) v = v * s + c[i * 2 * n];
    }
    if (f < n) u[f] = v; else w[f - n] = v;
  }
}

}  // namespace sf
