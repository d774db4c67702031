// grad_f32.cu -- FP32 two-electron gradient kernels (FP64 accumulation), one per class.
#include <algorithm>

#include "classes.h"
#include "grad.cuh"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD>
static cudaError_t run_grad32(const KParams &kp, const ClassWork &w, const float *D, double *grad, cudaStream_t st) {
  constexpr int T = tgrad_r<float>(QC<LA, LB, LC, LD>::NABCD);
  if (w.n <= 0) return cudaSuccess;
  const ClassWork w2 = grad_work(w, T, kp.nsm);
  const int G = kBlock / (T * w2.psplit);
  constexpr size_t smem = grad_smem<LA, LB, LC, LD, float>();
  grad_kernel<LA, LB, LC, LD, float, T><<<(unsigned)((w.n * w2.wsplit + G - 1) / G), kBlock, smem, st>>>(kp, w2, D, grad);
  return cudaGetLastError();
}

cudaError_t launch_grad_f32(int cls, const KParams &kp, const ClassWork &w, const float *D, double *grad,
                            cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_grad32<la, lb, lc, ld>(kp, w, D, grad, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_grad_f32() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32)                                                               \
  if (e == cudaSuccess)                                                                                     \
    e = prep_smem(grad_kernel<la, lb, lc, ld, float, tgrad_r<float>(QC<la, lb, lc, ld>::NABCD)>,                    \
                  grad_smem<la, lb, lc, ld, float>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  return e;
}

}  // namespace sf
