// jk_dd_wide.cu -- double-float J/K kernels with tdd_wide lanes per quartet
// (classes.h): the accurate tier of the SF_PREC_MIXED_DF mode, whose few long
// quartets run latency-bound with the FP64 lane count.  Its own translation
// unit so that the build compiles it beside jk_dd.cu.
#include "classes.h"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD, int T>
static cudaError_t run_jk_dd_wide(const KParams &kp, const ClassWork &w, const dd *D, double *Jh, double *Kh,
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

cudaError_t launch_jk_dd_wide(int cls, const KParams &kp, const ClassWork &w, const dd *D, double *Jh, double *Kh,
                              cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_jk_dd_wide<la, lb, lc, ld, tdd_wide(la, lb, lc, ld, t64)>(kp, w, D, Jh, Kh, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_jk_dd_wide() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32)                                       \
  if (e == cudaSuccess)                                                             \
    e = prep_smem(jk_kernel<la, lb, lc, ld, dd, tdd_wide(la, lb, lc, ld, t64)>,     \
                  grp_smem<la, lb, lc, ld, dd, tdd_wide(la, lb, lc, ld, t64)>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  return e;
}

}  // namespace sf
