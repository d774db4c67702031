// jk_f32.cu -- FP32 J/K kernels (FP64 accumulation), one instantiation per class.
#include <algorithm>

#include "classes.h"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD, int T>
static cudaError_t run_jk32(const KParams &kp, const ClassWork &w, const float *D, double *Jh, double *Kh,
                            cudaStream_t st) {
  const int64_t n = w.n;
  if (n <= 0) return cudaSuccess;
  const int P = w.psplit < 1 ? 1 : w.psplit, W = w.wsplit < 1 ? 1 : w.wsplit;
  if (T * P > 32 || (P & (P - 1)) || W > kMaxWsplit) return cudaErrorInvalidValue;
  const int G = kBlock / (T * P);
  auto kern = jk_kernel<LA, LB, LC, LD, float, T>;
  int64_t grid = (n * W + G - 1) / G;
  size_t smem = grp_smem<LA, LB, LC, LD, float, T>();
  if (T == 1) {   // Rys table block in shared memory, grid-stride over the list
    smem = (size_t)kTabNint * QC<LA, LB, LC, LD>::NR * kTab32Row * sizeof(float);
    grid = std::min<int64_t>(grid, (int64_t)std::max(kp.nsm, 1) * 16);
  }
  kern<<<(unsigned)grid, kBlock, smem, st>>>(kp, w, D, Jh, Kh);
  return cudaGetLastError();
}

cudaError_t launch_jk_f32(int cls, const KParams &kp, const ClassWork &w, const float *D, double *Jh, double *Kh,
                          cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_jk32<la, lb, lc, ld, t32>(kp, w, D, Jh, Kh, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

// raise the dynamic shared-memory limit of every group kernel on the current
// device (called once per device by sf_create)
cudaError_t prepare_jk_f32() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32)                                                      \
  if (e == cudaSuccess)                                                                            \
    e = prep_smem(jk_kernel<la, lb, lc, ld, float, t32>, grp_smem<la, lb, lc, ld, float, t32>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  return e;
}

}  // namespace sf
