// jk_persist.cu -- persistent multi-class FP32 J/K kernels.
//
// One launch per register tier runs every quartet list of the tier's classes:
// each CTA takes tiles from a device work queue (an atomic counter over a
// tile table sorted by estimated cost, heaviest first) until the table is
// exhausted.  A tile is what one CTA of the class kernel does in one trip of
// its grid-stride loop: kBlock / P quartet groups of one list, in that list's
// primitive split (P, W).  The class is dispatched at compile time among the
// tier's classes.  A kernel holding several classes' code needs far more
// registers than the largest of them (ptxas, FP32 register path, class kernel
// alone -> inlined together): (00|00) 48 + (10|00) 64 -> 96; (10|10) 96,
// (11|00) 96, (20|00) 80, (20|10) 96 -> 162; (11|10) 126, (20|20) 125,
// (21|00) 108 -> 207; (11|11) 240, (20|11) 164, (21|10) 164, (22|00) 147 ->
// 254 (a real call per class instead of inlining did not lower them), so the
// classes are grouped in four tiers of similar register use and every tier
// runs as one launch.
// The queue has no waits: a CTA that finds the counter past the end returns.
// This replaces, for these classes, the reference's scheduler of independent
// integral tasks (Pool(8).map over AO quartets, src/hf/hf.py:45-47) with
// dynamically balanced launches.
#include "classes.h"
#include "launch.h"

namespace sf {

namespace {
// class ids: (00|00) 0, (10|00) 1, (10|10) 2, (11|00) 3, (11|10) 4,
// (11|11) 5, (20|00) 6, (20|10) 7, (20|11) 8, (20|20) 9, (21|00) 10,
// (21|10) 11, (22|00) 15
constexpr unsigned kTierMask[kPersistTiers] = {(1u << 0) | (1u << 1), (1u << 2) | (1u << 3) | (1u << 6) | (1u << 7),
                                               (1u << 4) | (1u << 9) | (1u << 10),
                                               (1u << 5) | (1u << 8) | (1u << 11) | (1u << 15)};
// largest root count of each tier's classes: its Rys table block in shared memory
constexpr int kTierMaxNR[kPersistTiers] = {1, 2, 3, 3};
constexpr size_t persist_smem(int tier) { return (size_t)kTabNint * kTierMaxNR[tier] * kTab32Row * sizeof(float); }

template <unsigned MASK>
__global__ void __launch_bounds__(kBlock) jk_persist_f32_kernel(KParams kp, PersistWork pw, const float *__restrict__ D,
                                                                double *Jh, double *Kh) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4 *tab4 = reinterpret_cast<float4 *>(smem_raw);
  const float *tab_s = reinterpret_cast<const float *>(smem_raw);
  __shared__ int s_tile;
  int cur_nr = 0;   // root block in shared memory (uniform over the CTA)
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(pw.next, 1u);
    __syncthreads();   // also: every thread is done with the previous tile
    const int t = s_tile;
    __syncthreads();   // s_tile read before thread 0 takes the next one
    if (t >= pw.ntiles) return;
    const int2 tl = __ldg(pw.tiles + t);
    const int cls = __ldg(pw.cls + tl.x);
    const ClassWork w = pw.works[tl.x];
    const int P = w.psplit;
    const int64_t gid = (int64_t)tl.y * (kBlock / P) + threadIdx.x / P;
    const int64_t nq = work_count(w);
    switch (cls) {
#define SF_PCASE(id, la, lb, lc, ld, t64, t32)                                      \
  case id:                                                                          \
    if constexpr (((MASK >> id) & 1u) && t32 == 1) {                               \
      constexpr int NR = QC<la, lb, lc, ld>::NR;                                    \
      if (NR != cur_nr) {                                                           \
        load_tab32_block(kp, NR, tab4);                                             \
        __syncthreads();                                                            \
        cur_nr = NR;                                                                \
      }                                                                             \
      jk_f32_t1_step<la, lb, lc, ld>(kp, w, gid, nq, tab_s, D, Jh, Kh);            \
    }                                                                               \
    break;
      SF_CLASS_LIST(SF_PCASE)
#undef SF_PCASE
      default: break;
    }
  }
}

template <int TIER>
cudaError_t occupancy(int *blocks) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, jk_persist_f32_kernel<kTierMask[TIER]>, kBlock,
                                                       persist_smem(TIER));
}

template <int TIER>
void launch_tier(const KParams &kp, const PersistWork &pw, int grid, const float *D, double *Jh, double *Kh,
                 cudaStream_t st) {
  jk_persist_f32_kernel<kTierMask[TIER]><<<(unsigned)grid, kBlock, persist_smem(TIER), st>>>(kp, pw, D, Jh, Kh);
}
}  // namespace

int persist_tier_of(int cls) {
  for (int t = 0; t < kPersistTiers; ++t)
    if ((kTierMask[t] >> cls) & 1u) return t;
  return -1;
}

cudaError_t persist_blocks_per_sm(int tier, int *blocks) {
  *blocks = 0;
  switch (tier) {
    case 0: return occupancy<0>(blocks);
    case 1: return occupancy<1>(blocks);
    case 2: return occupancy<2>(blocks);
    case 3: return occupancy<3>(blocks);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_jk_persist_f32(int tier, const KParams &kp, const PersistWork &pw, int grid, const float *D,
                                  double *Jh, double *Kh, cudaStream_t st) {
  if (pw.ntiles <= 0) return cudaSuccess;
  if (grid < 1) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(pw.next, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  switch (tier) {
    case 0: launch_tier<0>(kp, pw, grid, D, Jh, Kh, st); break;
    case 1: launch_tier<1>(kp, pw, grid, D, Jh, Kh, st); break;
    case 2: launch_tier<2>(kp, pw, grid, D, Jh, Kh, st); break;
    case 3: launch_tier<3>(kp, pw, grid, D, Jh, Kh, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace sf
