// eri.cu -- raw contracted ERIs (FP64 / FP32) and Schwarz bounds (FP64).
#include <algorithm>
#include "classes.h"
#include "launch.h"

namespace sf {

template <int LA, int LB, int LC, int LD, typename R, int T>
static cudaError_t run_eri(const KParams &kp, const EriWork &w, cudaStream_t st) {
  if (w.n <= 0) return cudaSuccess;
  const int P = w.psplit < 1 ? 1 : w.psplit;
  if (T * P > 32 || (P & (P - 1))) return cudaErrorInvalidValue;
  EriWork w2 = w;
  w2.psplit = P;
  const int G = kBlock / (T * P);
  size_t smem = grp_smem<LA, LB, LC, LD, R, T>();
  int64_t grid = (w.n + G - 1) / G;
  if (T == 1 && std::is_same<R, float>::value) {   // Rys table block in shared memory, grid-stride
    smem = (size_t)kTabNint * QC<LA, LB, LC, LD>::NR * kTab32Row * sizeof(float);
    grid = std::min<int64_t>(grid, (int64_t)std::max(kp.nsm, 1) * 16);
  }
  eri_kernel<LA, LB, LC, LD, R, T><<<(unsigned)grid, kBlock, smem, st>>>(kp, w2);
  return cudaGetLastError();
}

cudaError_t launch_eri(int cls, int fp32, const KParams &kp, const EriWork &w, cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32)                                                    \
  case id:                                                                                       \
    return fp32 ? run_eri<la, lb, lc, ld, float, t32>(kp, w, st) : run_eri<la, lb, lc, ld, double, t64>(kp, w, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

// pair class pc -> diagonal class (X|X) and its thread-group size
template <int LA, int LB, int T>
static cudaError_t run_schwarz(const KParams &kp, int p0, int n, double *qout, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  constexpr int G = kBlock / T;
  constexpr size_t smem = grp_smem<LA, LB, LA, LB, double, T>();
  schwarz_kernel<LA, LB, double, T><<<(n + G - 1) / G, kBlock, smem, st>>>(kp, p0, n, qout);
  return cudaGetLastError();
}

cudaError_t launch_schwarz(int pc, const KParams &kp, int p0, int n, double *qout, cudaStream_t st) {
  switch (pc) {
    case 0: return run_schwarz<0, 0, kClassInfo[0].t64>(kp, p0, n, qout, st);
    case 1: return run_schwarz<1, 0, kClassInfo[2].t64>(kp, p0, n, qout, st);
    case 2: return run_schwarz<1, 1, kClassInfo[5].t64>(kp, p0, n, qout, st);
    case 3: return run_schwarz<2, 0, kClassInfo[9].t64>(kp, p0, n, qout, st);
    case 4: return run_schwarz<2, 1, kClassInfo[14].t64>(kp, p0, n, qout, st);
    case 5: return run_schwarz<2, 2, kClassInfo[20].t64>(kp, p0, n, qout, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_eri() {
  cudaError_t e = cudaSuccess;
#define SF_PREP(id, la, lb, lc, ld, t64, t32)                                                           \
  if (e == cudaSuccess)                                                                                 \
    e = prep_smem(eri_kernel<la, lb, lc, ld, double, t64>, grp_smem<la, lb, lc, ld, double, t64>());    \
  if (e == cudaSuccess)                                                                                 \
    e = prep_smem(eri_kernel<la, lb, lc, ld, float, t32>, grp_smem<la, lb, lc, ld, float, t32>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  if (e == cudaSuccess) e = prep_smem(schwarz_kernel<1, 1, double, kClassInfo[5].t64>, grp_smem<1, 1, 1, 1, double, kClassInfo[5].t64>());
  if (e == cudaSuccess) e = prep_smem(schwarz_kernel<2, 0, double, kClassInfo[9].t64>, grp_smem<2, 0, 2, 0, double, kClassInfo[9].t64>());
  if (e == cudaSuccess) e = prep_smem(schwarz_kernel<2, 1, double, kClassInfo[14].t64>, grp_smem<2, 1, 2, 1, double, kClassInfo[14].t64>());
  if (e == cudaSuccess) e = prep_smem(schwarz_kernel<2, 2, double, kClassInfo[20].t64>, grp_smem<2, 2, 2, 2, double, kClassInfo[20].t64>());
  return e;
}

}  // namespace sf
