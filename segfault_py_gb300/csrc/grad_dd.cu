// grad_dd.cu -- dispatch of the double-float gradient kernels, whose classes
// are compiled in four units (grad_dd_0.cu .. grad_dd_3.cu, class id modulo 4).
#include "launch.h"

namespace sf {

cudaError_t launch_grad_dd_part0(int, const KParams &, const ClassWork &, const dd *, double *, cudaStream_t);
cudaError_t launch_grad_dd_part1(int, const KParams &, const ClassWork &, const dd *, double *, cudaStream_t);
cudaError_t launch_grad_dd_part2(int, const KParams &, const ClassWork &, const dd *, double *, cudaStream_t);
cudaError_t launch_grad_dd_part3(int, const KParams &, const ClassWork &, const dd *, double *, cudaStream_t);
cudaError_t prepare_grad_dd_part0();
cudaError_t prepare_grad_dd_part1();
cudaError_t prepare_grad_dd_part2();
cudaError_t prepare_grad_dd_part3();

cudaError_t launch_grad_dd(int cls, const KParams &kp, const ClassWork &w, const dd *D, double *grad,
                           cudaStream_t st) {
  switch (cls % 4) {
    case 0: return launch_grad_dd_part0(cls, kp, w, D, grad, st);
    case 1: return launch_grad_dd_part1(cls, kp, w, D, grad, st);
    case 2: return launch_grad_dd_part2(cls, kp, w, D, grad, st);
    default: return launch_grad_dd_part3(cls, kp, w, D, grad, st);
  }
}

cudaError_t prepare_grad_dd() {
  cudaError_t e = prepare_grad_dd_part0();
  if (e == cudaSuccess) e = prepare_grad_dd_part1();
  if (e == cudaSuccess) e = prepare_grad_dd_part2();
  if (e == cudaSuccess) e = prepare_grad_dd_part3();
  return e;
}

}  // namespace sf
