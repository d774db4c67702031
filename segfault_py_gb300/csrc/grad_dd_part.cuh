// grad_dd_part.cuh -- double-float two-electron gradient kernels (the accurate
// tier of the gradient in the SF_PREC_MIXED_DF / SF_PREC_DF modes), split over
// four translation units by class id modulo 4 so that they compile in
// parallel; each unit defines SF_DD_PART and includes this file.
#pragma once
#include <algorithm>

#include "classes.h"
#include "grad.cuh"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD>
static cudaError_t run_grad_dd(const KParams &kp, const ClassWork &w, const dd *D, double *grad, cudaStream_t st) {
  constexpr int T = tgrad(QC<LA, LB, LC, LD>::NABCD);
  if (w.n <= 0) return cudaSuccess;
  const ClassWork w2 = grad_work(w, T, kp.nsm);
  const int G = kBlock / (T * w2.psplit);
  constexpr size_t smem = grad_smem<LA, LB, LC, LD, dd>();
  grad_kernel<LA, LB, LC, LD, dd, T><<<(unsigned)((w.n * w2.wsplit + G - 1) / G), kBlock, smem, st>>>(kp, w2, D, grad);
  return cudaGetLastError();
}

#define SF_DD_JOIN2(a, b) a##b
#define SF_DD_JOIN(a, b) SF_DD_JOIN2(a, b)

cudaError_t SF_DD_JOIN(launch_grad_dd_part, SF_DD_PART)(int cls, const KParams &kp, const ClassWork &w, const dd *D,
                                                         double *grad, cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id:                                    \
    if constexpr (id % 4 == SF_DD_PART) return run_grad_dd<la, lb, lc, ld>(kp, w, D, grad, st); \
    else return cudaErrorInvalidValue;
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t SF_DD_JOIN(prepare_grad_dd_part, SF_DD_PART)() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32)                                                    \
  if constexpr (id % 4 == SF_DD_PART)                                                            \
    if (e == cudaSuccess)                                                                        \
      e = prep_smem(grad_kernel<la, lb, lc, ld, dd, tgrad(QC<la, lb, lc, ld>::NABCD)>,           \
                    grad_smem<la, lb, lc, ld, dd>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  return e;
}

}  // namespace sf
