// jk_dd.cu -- double-float (dd) J/K kernels, per class: the accurate tier of
// the SF_PREC_MIXED_DF / SF_PREC_DF modes.  Lanes per quartet as the FP64
// kernels (same register footprint per value); the tdd_wide instantiations
// for the accurate tier of a mixed build are in jk_dd_wide.cu.
#include "classes.h"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD, int T>
static cudaError_t run_jk_dd(const KParams &kp, const ClassWork &w, const dd *D, double *Jh, double *Kh,
                             cudaStream_t st) {
  const int64_t n = w.n;
  if (n <= 0) return cudaSuccess;
  const int P = w.psplit < 1 ? 1 : w.psplit, W = w.wsplit < 1 ? 1 : w.wsplit;
  if (T * P > 32 || (P & (P - 1)) || W > kMaxWsplit) return cudaErrorInvalidValue;
  const int G = kBlock / (T * P);
  constexpr size_t smem = grp_smem<LA, LB, LC, LD, dd, T>();
  const int64_t grid = (n * W + G - 1) / G;
  jk_kernel<LA, LB, LC, LD, dd, T><<<(unsigned)grid, kBlock, smem, st>>>(kp, w, D, Jh, Kh);
  return cudaGetLastError();
}

// w.wide selects the tdd_wide lanes per quartet (the accurate tier of a mixed
// build; compiled in jk_dd_wide.cu), else the FP64 lanes
cudaError_t launch_jk_dd(int cls, const KParams &kp, const ClassWork &w, const dd *D, double *Jh, double *Kh,
                         cudaStream_t st) {
  if (w.wide) return launch_jk_dd_wide(cls, kp, w, D, Jh, Kh, st);
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_jk_dd<la, lb, lc, ld, t64>(kp, w, D, Jh, Kh, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_jk_dd() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32)                                                           \
  if (e == cudaSuccess) e = prep_smem(jk_kernel<la, lb, lc, ld, dd, t64>, grp_smem<la, lb, lc, ld, dd, t64>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  if (e == cudaSuccess) e = prepare_jk_dd_wide();
  return e;
}

}  // namespace sf
