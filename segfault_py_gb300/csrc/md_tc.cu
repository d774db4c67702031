// md_tc.cu -- McMurchie-Davidson raw ERIs whose bra Hermite-to-Cartesian
// E-coefficient contraction runs on the fifth-generation tensor cores.
//
// For one contracted quartet and one bra primitive pair p (md.cuh):
//   W_p[cd][h]  = sum_q K~_p K~_q / sqrt(p+q) sum_{tau nu phi} (-1)^{..}
//                 E^{cd,q} R_{h+(tau,nu,phi)}(p,q)          (CUDA cores, FP32)
//   (ab|cd)    += sum_h E^{ab,p}[ab][h] W_p[cd][h]           (tensor cores)
// The second line is a GEMM D[128 x N] += A[128 x K] B[N x K]^T with the
// ab components as rows of A (padded to M = 128), the Hermite functions h of
// the bra as K (padded to 40) and the cd components as rows of B (padded to
// N = 48), issued as tcgen05.mma kind::tf32 from shared-memory operands in the
// canonical K-major layout without swizzle (8-row x 16-byte core matrices,
// K-adjacent core matrices 128 bytes apart, 8-row groups 1280 bytes apart),
// accumulating in tensor memory over the bra primitives.  FP32 accuracy from
// TF32 inputs by the three-pass split x = hi + lo (hi rounded to TF32):
// A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi.  One elected thread issues the
// MMAs and commits them to an mbarrier; every wait is bounded and a timeout
// sets the handle's error flag, after which the CTA frees its tensor memory
// and stops.
#include <cstdint>

#include "classes.h"
#include "launch.h"
#include "md.cuh"

namespace sf {

__constant__ MdTables c_md_tc;

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcM = 128;                 // MMA M (ab components padded)
constexpr int kTcK = 40;                  // Hermite functions of the bra (<= 35) padded to 8
constexpr int kTcN = 48;                  // cd components (<= 36) padded to 16 (M = 128 needs N % 16 == 0)
constexpr int kTcCols = 64;               // tensor-memory columns allocated (power of two >= 32)
constexpr uint32_t kCoreBytes = 128;      // one 8 x 16-byte core matrix
constexpr uint32_t kLBO = kCoreBytes;     // K-adjacent core matrices
constexpr uint32_t kSBO = (kTcK / 4) * kCoreBytes;   // adjacent 8-row groups (1280 B)
constexpr uint32_t kABytes = (kTcM / 8) * kSBO;      // 20480
constexpr uint32_t kBBytes = (kTcN / 8) * kSBO;      // 7680
constexpr int kMaxWait = 1 << 24;

// instruction descriptor: D F32, A and B TF32, both K-major, N, M
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                            ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in a K-major operand without swizzle
__device__ __forceinline__ uint32_t op_off(int r, int k) {
  return (uint32_t)(r >> 3) * kSBO + (uint32_t)(k >> 2) * kCoreBytes + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((kLBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version; base offset 0, no swizzle
  return d;
}

__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  lo = x - hi;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(kTcThreads) md_tc_kernel(KParams kp, EriWork w, int wait_limit) {
  using Q = QC<LA, LB, LC, LD>;
  constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
  constexpr int NHAB = nherm(LAB), NHL = nherm(L);
  constexpr int NAB = Q::NA * Q::NB, NCD = Q::NC * Q::ND;
  constexpr int NW = (NHAB * NCD + kTcThreads - 1) / kTcThreads;   // W entries per thread
  static_assert(NHAB <= kTcK && NCD <= kTcN && NAB <= kTcM, "class exceeds the MMA tile");

  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *a_hi = smem, *a_lo = smem + kABytes;
  unsigned char *b_hi = smem + 2 * kABytes, *b_lo = b_hi + kBBytes;
  float *rlev = reinterpret_cast<float *>(b_lo + kBBytes);          // 2 x NHL: R^n by level
  uint64_t *mbar = reinterpret_cast<uint64_t *>(rlev + 2 * NHL + 2);  // 8-byte aligned (NHL even or padded)
  uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
  int *abort_flag = reinterpret_cast<int *>(tslot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // zero both operands once: padding rows / columns are never written again
  for (int i = tid; i < (int)(2 * kABytes + 2 * kBBytes) / 4; i += kTcThreads) reinterpret_cast<float *>(smem)[i] = 0.f;
  if (tid == 0) {
    mbar_init(mbar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  uint32_t phase = 0;
  const uint32_t a_hi_s = smem_addr(a_hi), a_lo_s = smem_addr(a_lo), b_hi_s = smem_addr(b_hi), b_lo_s = smem_addr(b_lo);

  for (int64_t qi = blockIdx.x; qi < w.n; qi += gridDim.x) {
    const int fl = w.flags[qi];
    const QGeom<float> g = make_geom<float>(kp, w.pab[qi], w.pcd[qi], fl & 1, fl & 2);
    const float *recs = kp.p32.rec;
    bool failed = false;
    for (int ip = 0; ip < g.ab_n && !failed; ++ip) {
      float p, Px, Py, Pz, kab, i2p;
      load_rec<float>(recs + (size_t)(g.ab_off + ip) * kPrimRec, p, Px, Py, Pz, kab, i2p);
      const float PA[3] = {Px - g.Ax, Py - g.Ay, Pz - g.Az};
      const float AB[3] = {g.ABx, g.ABy, g.ABz};
      float Eab[3][LA + 1][LB + 1][LAB + 1];
#pragma unroll
      for (int d = 0; d < 3; ++d) md_hermite_e<LA, LB, float>(i2p, PA[d], PA[d] + AB[d], Eab[d]);
      // A operand: E^{ab,p}[ab][h]
      for (int e = tid; e < NAB * NHAB; e += kTcThreads) {
        const int r = e / NHAB, h = e % NHAB;
        const int ia = r / Q::NB, ib = r % Q::NB;
        const int t = c_md_tc.t[h], u = c_md_tc.u[h], v = c_md_tc.v[h];
        const int ax = cart_e(LA, ia, 0), ay = cart_e(LA, ia, 1), az = cart_e(LA, ia, 2);
        const int bx = cart_e(LB, ib, 0), by = cart_e(LB, ib, 1), bz = cart_e(LB, ib, 2);
        const float val = (t <= ax + bx && u <= ay + by && v <= az + bz)
                              ? Eab[0][ax][bx][t] * Eab[1][ay][by][u] * Eab[2][az][bz][v]
                              : 0.f;
        float hi, lo;
        split_tf32(val, hi, lo);
        *reinterpret_cast<float *>(a_hi + op_off(r, h)) = hi;
        *reinterpret_cast<float *>(a_lo + op_off(r, h)) = lo;
      }
      // W_p[cd][h] over the ket primitives
      float Wacc[NW];
#pragma unroll
      for (int j = 0; j < NW; ++j) Wacc[j] = 0.f;
      for (int iq = 0; iq < g.cd_n; ++iq) {
        float qq, Qx, Qy, Qz, kcd, i2q;
        load_rec<float>(recs + (size_t)(g.cd_off + iq) * kPrimRec, qq, Qx, Qy, Qz, kcd, i2q);
        const float QC_[3] = {Qx - g.Cx, Qy - g.Cy, Qz - g.Cz};
        const float CD[3] = {g.CDx, g.CDy, g.CDz};
        float Ecd[3][LC + 1][LD + 1][LCD + 1];
#pragma unroll
        for (int d = 0; d < 3; ++d) md_hermite_e<LC, LD, float>(i2q, QC_[d], QC_[d] + CD[d], Ecd[d]);
        const float pq = p + qq, rho = p * qq / pq;
        const float X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
        float F[L + 1];
        md_boys<L, float>(rho * (X * X + Y * Y + Z * Z), F);
        // R^n_h level by level (n = L .. 0), ping-pong between two smem rows
        __syncthreads();   // the previous primitive's R is no longer read
        if (tid == 0) {
          float f = 1.f;
          for (int n = 0; n < L; ++n) f *= -2.f * rho;
          rlev[(L & 1) * NHL] = f * F[L];
        }
        __syncthreads();
        float fpow = 1.f;
        for (int n = 0; n < L; ++n) fpow *= -2.f * rho;   // (-2 rho)^L
        for (int n = L - 1; n >= 0; --n) {
          fpow /= -2.f * rho;
          const float *up = rlev + ((n + 1) & 1) * NHL;
          float *cur = rlev + (n & 1) * NHL;
          for (int h = tid; h < nherm(L - n); h += kTcThreads) {
            float r;
            if (h == 0) {
              r = fpow * F[n];
            } else {
              const int t = c_md_tc.t[h], u = c_md_tc.u[h], v = c_md_tc.v[h];
              if (t > 0) r = (t > 1 ? (float)(t - 1) * up[c_md_tc.idx[t - 2][u][v]] : 0.f) + X * up[c_md_tc.idx[t - 1][u][v]];
              else if (u > 0) r = (u > 1 ? (float)(u - 1) * up[c_md_tc.idx[t][u - 2][v]] : 0.f) + Y * up[c_md_tc.idx[t][u - 1][v]];
              else r = (v > 1 ? (float)(v - 1) * up[c_md_tc.idx[t][u][v - 2]] : 0.f) + Z * up[c_md_tc.idx[t][u][v - 1]];
            }
            cur[h] = r;
          }
          __syncthreads();
        }
        const float *R0 = rlev;   // level 0 lives in row 0
        const float pref = kab * kcd * rsqrtf(pq);
#pragma unroll
        for (int j = 0; j < NW; ++j) {
          const int e = tid + j * kTcThreads;
          if (e < NHAB * NCD) {
            const int cdi = e / NHAB, h = e % NHAB;
            const int ic = cdi / Q::ND, id = cdi % Q::ND;
            const int cx = cart_e(LC, ic, 0), cy = cart_e(LC, ic, 1), cz = cart_e(LC, ic, 2);
            const int dx = cart_e(LD, id, 0), dy = cart_e(LD, id, 1), dz = cart_e(LD, id, 2);
            const int t = c_md_tc.t[h], u = c_md_tc.u[h], v = c_md_tc.v[h];
            float s = 0.f;
            for (int ta = 0; ta <= cx + dx; ++ta)
              for (int nu = 0; nu <= cy + dy; ++nu)
                for (int ph = 0; ph <= cz + dz; ++ph) {
                  const float ev = Ecd[0][cx][dx][ta] * Ecd[1][cy][dy][nu] * Ecd[2][cz][dz][ph];
                  const float rv = R0[c_md_tc.idx[t + ta][u + nu][v + ph]];
                  s += ((ta + nu + ph) & 1) ? -ev * rv : ev * rv;
                }
            Wacc[j] += pref * s;
          }
        }
      }
      // B operand: W_p[cd][h]
#pragma unroll
      for (int j = 0; j < NW; ++j) {
        const int e = tid + j * kTcThreads;
        if (e < NHAB * NCD) {
          const int cdi = e / NHAB, h = e % NHAB;
          float hi, lo;
          split_tf32(Wacc[j], hi, lo);
          *reinterpret_cast<float *>(b_hi + op_off(cdi, h)) = hi;
          *reinterpret_cast<float *>(b_lo + op_off(cdi, h)) = lo;
        }
      }
      // operands visible to the tensor core, then one thread issues the MMAs
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
#pragma unroll 1
        for (int s = 0; s < kTcK / 8; ++s) {
          const uint32_t koff = (uint32_t)s * 2u * kCoreBytes;
          const uint32_t acc0 = (ip > 0 || s > 0) ? 1u : 0u;
          mma_tf32(tmem, smem_desc(a_hi_s + koff), smem_desc(b_hi_s + koff), acc0);
          mma_tf32(tmem, smem_desc(a_hi_s + koff), smem_desc(b_lo_s + koff), 1u);
          mma_tf32(tmem, smem_desc(a_lo_s + koff), smem_desc(b_hi_s + koff), 1u);
        }
        mma_commit(mbar);
      }
      // every thread waits (bounded) for the MMAs before the operands are rewritten
      bool done = false;
      for (int it = 0; it < wait_limit && !done; ++it) done = mbar_try_wait(mbar, phase);
      if (!done) {
        atomicExch(abort_flag, 1);
        if (kp.err) atomicExch(kp.err, 2);
      }
      phase ^= 1u;
      __syncthreads();
      failed = *abort_flag != 0;
    }
    if (failed) {
      // the commit that timed out may still have MMAs writing the tensor
      // memory: wait once more (bounded) for that phase before the memory is
      // freed below; if it never completes the flag says so (the results of
      // the whole launch are discarded by the host either way)
      if (tid == 0) {
        int it2 = 0;
        while (!mbar_try_wait(mbar, phase ^ 1u) && ++it2 < kMaxWait) {
        }
        if (it2 >= kMaxWait && kp.err) atomicExch(kp.err, 3);
      }
      __syncthreads();
      break;
    }
    // accumulator rows (ab) -> output; warp w holds lanes 32w .. 32w+31
    tc_fence_after();
    float dv[kTcN];
#pragma unroll
    for (int c = 0; c < kTcN; c += 16) {
      float v16[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v16);
#pragma unroll
      for (int i = 0; i < 16; ++i) dv[c + i] = v16[i];
    }
    const int r = warp * 32 + lane;
    if (r < NAB) {
      const int s0 = w.strides[4 * qi], s1 = w.strides[4 * qi + 1], s2 = w.strides[4 * qi + 2], s3 = w.strides[4 * qi + 3];
      double *out = w.out + w.out_off[qi];
      const int ia = r / Q::NB, ib = r % Q::NB;
#pragma unroll 1
      for (int c = 0; c < NCD; ++c) {
        const int ic = c / Q::ND, id = c % Q::ND;
        const int o = r * NCD + c;
        out[ia * s0 + ib * s1 + ic * s2 + id * s3] = (double)(dv[c] * (float)Q::norm(o));
      }
    }
    tc_fence_before();
    __syncthreads();   // the accumulator is read before the next quartet overwrites it
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
  }
}

template <int LA, int LB, int LC, int LD>
constexpr size_t md_tc_smem() {
  return 2 * kABytes + 2 * kBBytes + (2 * nherm(LA + LB + LC + LD) + 2) * sizeof(float) + 32;
}

// polls of the bounded wait on each MMA commit: kMaxWait unless a test
// shortens it to make the wait run out (0: out before the first poll); the
// wait after a timeout, which drains the MMAs before the tensor memory is
// freed, always allows kMaxWait
static int g_wait_limit = kMaxWait;

void md_tc_set_wait_limit(int iterations) { g_wait_limit = iterations >= 0 ? iterations : kMaxWait; }

template <int LA, int LB, int LC, int LD>
static cudaError_t run_md_tc(const KParams &kp, const EriWork &w, int nsm, cudaStream_t st) {
  if (w.n <= 0) return cudaSuccess;
  const int64_t grid = std::min<int64_t>(w.n, (int64_t)std::max(nsm, 1) * 2);
  md_tc_kernel<LA, LB, LC, LD><<<(unsigned)grid, kTcThreads, md_tc_smem<LA, LB, LC, LD>(), st>>>(kp, w,
                                                                                                  g_wait_limit);
  return cudaGetLastError();
}

cudaError_t launch_md_tc(int cls, const KParams &kp, const EriWork &w, int nsm, cudaStream_t st) {
  switch (cls) {
#define SF_CASE(id, la, lb, lc, ld, t64, t32) \
  case id: return run_md_tc<la, lb, lc, ld>(kp, w, nsm, st);
    SF_CLASS_LIST(SF_CASE)
#undef SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_md_tc() {
  MdTables tb{};
  for (int h = 0; h < nherm(kMdMaxL); ++h) {
    tb.t[h] = (unsigned char)herm_t(h);
    tb.u[h] = (unsigned char)herm_u(h);
    tb.v[h] = (unsigned char)herm_v(h);
  }
  for (int t = 0; t <= kMdMaxL; ++t)
    for (int u = 0; u <= kMdMaxL; ++u)
      for (int v = 0; v <= kMdMaxL; ++v) tb.idx[t][u][v] = (short)(t + u + v <= kMdMaxL ? herm_index(t, u, v) : 0);
  cudaError_t e = cudaMemcpyToSymbol(c_md_tc, &tb, sizeof(tb));
#define SF_PREP(id, la, lb, lc, ld, t64, t32) \
  if (e == cudaSuccess) e = prep_smem(md_tc_kernel<la, lb, lc, ld>, md_tc_smem<la, lb, lc, ld>());
  SF_CLASS_LIST(SF_PREP)
#undef SF_PREP
  return e;
}

}  // namespace sf
