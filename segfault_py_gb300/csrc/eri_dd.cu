// eri_dd.cu -- double-float (dd) raw-ERI kernels (sf_eri_batch / plans in
// the SF_PREC_DF mode), one instantiation per class.
#include "classes.h"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD, int T>
static cudaError_t run_eri_dd(const KParams &kp, const EriWork &w, cudaStream_t st) {
  if (w.n <= 0) return cudaSuccess;
  const int P = w.psplit < 1 ? 1 : w.psplit;
  if (T * P > 32 || (P & (P - 1))) return cudaErrorInvalidValue;
  EriWork w2 = w;
  w2.psplit = P;
  const int G = kBlock / (T * P);
  constexpr size_t smem = grp_smem<LA, LB, LC, LD, dd, T>();
  eri_kernel<LA, LB, LC, LD, dd, T><<<(unsigned)((w.n + G - 1) / G), kBlock, smem, st>>>(kp, w2);
  return cudaGetLastError();
}

cudaError_t launch_eri_dd(int cls, const KParams &kp, const EriWork &w, cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_eri_dd<la, lb, lc, ld, t64>(kp, w, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_eri_dd() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32) \
  if (e == cudaSuccess) e = prep_smem(eri_kernel<la, lb, lc, ld, dd, t64>, grp_smem<la, lb, lc, ld, dd, t64>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  return e;
}

}  // namespace sf
