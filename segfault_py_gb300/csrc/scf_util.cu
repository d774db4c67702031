// scf_util.cu -- device-side helpers that keep an SCF iteration free of host
// synchronisation (so that it can be captured in a CUDA graph).
//
// sf_small_solve: x = A^-1 b for a small dense system (the Pulay/DIIS system
// of src/hf/hf.py:330-343, at most 8 x 8 there) by Gaussian elimination with
// partial pivoting in one thread.  A singular pivot (|pivot| below 1e-300 or
// not finite) sets *ok = 0 instead of raising, so the caller can fall back to
// the un-extrapolated Fock matrix as hf.py:344-346 does.
#include <cmath>
#include <cstdint>

#include "segfock.h"

namespace {

constexpr int kMaxSolve = 32;

__global__ void small_solve_kernel(int n, const double *A, const double *b, double *x, double *ok) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double M[kMaxSolve][kMaxSolve + 1];
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) M[i][j] = A[i * n + j];
    M[i][n] = b[i];
  }
  double good = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    double best = fabs(M[c][c]);
    for (int r = c + 1; r < n; ++r)
      if (fabs(M[r][c]) > best) { best = fabs(M[r][c]); piv = r; }
    if (!(best > 1e-300) || !isfinite(best)) { good = 0.0; break; }
    if (piv != c)
      for (int j = 0; j <= n; ++j) { const double t = M[c][j]; M[c][j] = M[piv][j]; M[piv][j] = t; }
    for (int r = c + 1; r < n; ++r) {
      const double f = M[r][c] / M[c][c];
      for (int j = c; j <= n; ++j) M[r][j] -= f * M[c][j];
    }
  }
  if (good != 0.0) {
    for (int i = n - 1; i >= 0; --i) {
      double s = M[i][n];
      for (int j = i + 1; j < n; ++j) s -= M[i][j] * x[j];
      x[i] = s / M[i][i];
      if (!isfinite(x[i])) good = 0.0;
    }
  }
  if (good == 0.0)
    for (int i = 0; i < n; ++i) x[i] = 0.0;
  *ok = good;
}

}  // namespace

extern "C" int sf_small_solve(int32_t n, const double *A, const double *b, double *x, double *ok, void *stream) {
  if (n < 1 || n > kMaxSolve || !A || !b || !x || !ok) return SF_EINVAL;
  small_solve_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(n, A, b, x, ok);
  return cudaGetLastError() == cudaSuccess ? SF_OK : SF_ECUDA;
}
