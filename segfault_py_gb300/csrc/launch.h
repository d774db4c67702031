// launch.h -- host-side launchers implemented in the kernel translation units.
#pragma once
#include "quartet.cuh"

namespace sf {
// J/K digestion kernels of class cls (0..20) over one work slice
cudaError_t launch_jk_f64(int cls, const KParams &kp, const ClassWork &w, const double *D, double *Jh, double *Kh,
                          cudaStream_t st);
cudaError_t launch_jk_f32(int cls, const KParams &kp, const ClassWork &w, const float *D, double *Jh, double *Kh,
                          cudaStream_t st);
cudaError_t launch_jk_dd(int cls, const KParams &kp, const ClassWork &w, const dd *D, double *Jh, double *Kh,
                         cudaStream_t st);
// the same with tdd_wide lanes per quartet (jk_dd_wide.cu)
cudaError_t launch_jk_dd_wide(int cls, const KParams &kp, const ClassWork &w, const dd *D, double *Jh, double *Kh,
                              cudaStream_t st);
cudaError_t prepare_jk_dd_wide();
// persistent multi-class FP32 J/K kernels (jk_persist.cu): one launch per
// register tier runs the tiles of every list of the tier's classes, taken
// from a device work queue
constexpr int kPersistTiers = 4;
struct PersistWork {
  const ClassWork *works;   // the tier's lists
  const int *cls;           // class of each list
  const int2 *tiles;        // (list, tile index in the list), heaviest first
  int ntiles;
  unsigned *next;           // queue counter (zeroed by the launcher)
};
// tier of a class whose FP32 kernel runs in the register path, else -1
int persist_tier_of(int cls);
cudaError_t persist_blocks_per_sm(int tier, int *blocks);
cudaError_t launch_jk_persist_f32(int tier, const KParams &kp, const PersistWork &pw, int grid, const float *D,
                                  double *Jh, double *Kh, cudaStream_t st);
// raw integrals of one class (fp32: FP32 evaluation, else FP64)
cudaError_t launch_eri(int cls, int fp32, const KParams &kp, const EriWork &w, cudaStream_t st);
cudaError_t launch_eri_dd(int cls, const KParams &kp, const EriWork &w, cudaStream_t st);
// raw integrals of one class by McMurchie-Davidson (FP64)
cudaError_t launch_md_eri(int cls, const KParams &kp, const EriWork &w, cudaStream_t st);
cudaError_t prepare_md();
// the same with the bra E contraction on the tensor cores (FP32 MD, 3-pass TF32)
cudaError_t launch_md_tc(int cls, const KParams &kp, const EriWork &w, int nsm, cudaStream_t st);
cudaError_t prepare_md_tc();
// polls of md_tc's bounded MMA waits (0: out before the first poll, < 0: the
// default); a test hook
void md_tc_set_wait_limit(int iterations);
// Schwarz bounds of pair class pc (0..5) over pairs [p0, p0+n)
cudaError_t launch_schwarz(int pc, const KParams &kp, int p0, int n, double *qout, cudaStream_t st);

cudaError_t launch_grad_f64(int cls, const KParams &kp, const ClassWork &w, const double *D, double *grad,
                            cudaStream_t st);
cudaError_t launch_grad_f32(int cls, const KParams &kp, const ClassWork &w, const float *D, double *grad,
                            cudaStream_t st);
cudaError_t launch_grad_dd(int cls, const KParams &kp, const ClassWork &w, const dd *D, double *grad,
                           cudaStream_t st);
cudaError_t prepare_grad_f64();
cudaError_t prepare_grad_dd();
cudaError_t prepare_grad_f32();
cudaError_t prepare_jk_f64();
cudaError_t prepare_jk_f32();
cudaError_t prepare_jk_dd();
cudaError_t prepare_eri_dd();
cudaError_t prepare_eri();

// one-electron kernel parameters (oneint.cu)
struct OneParams {
  DevShells sh;
  const double *exps, *coefs;   // per shell primitives (shell prim offsets in poff)
  const int *poff;
  int nshell, nao;
  const double *atom_xyz, *charges;
  int natom;
  double *S, *T, *V;
  const double *tab64;          // FP64 Rys rule (Boys values of the gradient kernel)
  RysAsym asym;
};

cudaError_t launch_one_electron(const OneParams &P, cudaStream_t st);
// gradient of sum_ij D_ij (T+V)_ij - W_ij S_ij (derivatives of the basis
// centres and, for V, of the nuclei), accumulated into grad[3*natom]
cudaError_t launch_one_electron_grad(const OneParams &P, const double *D, const double *W, double *grad,
                                     cudaStream_t st);

// smem bytes of a group kernel
template <int LA, int LB, int LC, int LD, typename R, int T>
constexpr size_t grp_smem() {
  return T == 1 ? 0 : (size_t)(kBlock / T) * Grp<LA, LB, LC, LD, R, T>::BUFN * sizeof(R);
}

template <typename K>
inline cudaError_t prep_smem(K kern, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}
}  // namespace sf
