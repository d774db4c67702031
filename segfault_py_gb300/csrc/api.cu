// api.cu -- C ABI of libsegfock (declared in include/segfock.h) and the host
// logic behind it: shell / pair tables, Schwarz ordering, the implicit
// screened quartet lists and the launch sequence of one Fock build.
//
// Quartet enumeration.  The reference enumerates every unique AO quartet
// i>=j, k>=l, ij>=kl (src/hf/hf.py:37-43).  Here the unit is the canonical
// shell quartet: pairs (a,b) with l_a >= l_b (a >= b if equal), classes
// (X|Y) with pair class X >= Y, and for X == Y the ket pair index <= the bra
// pair index.  After sf_schwarz the pairs of each class are sorted by Q
// descending, so for bra pair i the ket pairs that pass Q_i Q_j >= cutoff are
// a prefix of the ket list (found by binary search); in the mixed mode that
// prefix splits at Q_i Q_j >= fp32_cutoff into an FP64 head and an FP32 tail.
// The surviving quartets of each (class, precision) are then listed
// explicitly, ordered by primitive cost (see build_work).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <atomic>
#include <numeric>
#include <string>
#include <vector>

#include "classes.h"
#include "launch.h"
#include "segfock.h"

using namespace sf;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define SF_CK(call)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return fail(SF_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t m) {
    if (m <= n && p) return cudaSuccess;
    reset();
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(m, 1) * sizeof(T));
    if (e == cudaSuccess) n = m;
    return e;
  }
  cudaError_t upload(const std::vector<T> &v) {
    cudaError_t e = alloc(v.size());
    if (e != cudaSuccess) return e;
    if (v.empty()) return cudaSuccess;
    return cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
};

struct HostTables {
  std::vector<double> t64;
  std::vector<float> t32, t32v;   // t32v: the FP32 kernels' layout (sf_internal.h)
  std::vector<float4> tdd;         // the FP64 table as dd rows (sf_internal.h)
  RysAsym asym;
  RysAsym32 asym32;
};

// split of a double into the float pair hi + lo (round to nearest twice)
inline void dd_split(double d, float &hi, float &lo) {
  hi = (float)d;
  lo = (float)(d - (double)hi);
}

const HostTables &host_tables() {
  static HostTables T;
  static std::once_flag once;
  std::call_once(once, [] {
    T.t64.assign(rys_tab_size(kTabDeg64), 0.0);
    T.t32.assign(rys_tab_size(kTabDeg32), 0.0f);
    std::memset(&T.asym, 0, sizeof(T.asym));
    rys_build_tables(T.t64.data(), T.t32.data(), &T.asym);
    constexpr int D = kTabDeg32;
    T.t32v.assign(rys_tab32v_size(), 0.0f);
    for (int n = 1; n <= kMaxRoots; ++n)
      for (int j = 0; j < kTabNint; ++j)
        for (int r = 0; r < n; ++r) {
          float *row = T.t32v.data() + rys_tab32v_offset(n) + (j * n + r) * kTab32Row;
          const float *src = T.t32.data() + rys_tab_offset(n, D) + j * (D + 1) * 2 * n;
          for (int k = D; k >= 0; --k) {
            row[2 * (D - k)] = src[k * 2 * n + r];
            row[2 * (D - k) + 1] = src[k * 2 * n + n + r];
          }
        }
    for (int n = 0; n <= kMaxRoots; ++n)
      for (int i = 0; i < kMaxRoots; ++i) {
        T.asym32.r[n][i] = (float)T.asym.r[n][i];
        T.asym32.w[n][i] = (float)T.asym.w[n][i];
      }
    constexpr int D64 = kTabDeg64;
    T.tdd.assign(rys_tabdd_size(), make_float4(0.f, 0.f, 0.f, 0.f));
    for (int n = 1; n <= kMaxRoots; ++n)
      for (int j = 0; j < kTabNint; ++j)
        for (int r = 0; r < n; ++r) {
          float4 *row = T.tdd.data() + rys_tabdd_offset(n) + (j * n + r) * (D64 + 1);
          const double *src = T.t64.data() + rys_tab_offset(n, D64) + j * (D64 + 1) * 2 * n;
          for (int k = D64; k >= 0; --k) {
            float4 &c = row[D64 - k];
            dd_split(src[k * 2 * n + r], c.x, c.y);
            dd_split(src[k * 2 * n + n + r], c.z, c.w);
          }
        }
  });
  return T;
}

constexpr int kPairL[6][2] = {{0, 0}, {1, 0}, {1, 1}, {2, 0}, {2, 1}, {2, 2}};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

__global__ void symmetrize_kernel(const double *Jh, const double *Kh, double *J, double *K, int n) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * n) return;
  const int i = (int)(idx / n), j = (int)(idx % n);
  const int64_t t = (int64_t)j * n + i;
  J[idx] = Jh[idx] + Jh[t];
  K[idx] = Kh[idx] + Kh[t];
}

__global__ void to_float_kernel(const double *D, float *Df, int64_t n) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) Df[idx] = (float)D[idx];
}

// D as float pairs (hi, lo) for the dd kernels
__global__ void to_dd_kernel(const double *D, float2 *Dd, int64_t n) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) {
    const double d = D[idx];
    const float hi = __double2float_rn(d);
    Dd[idx] = make_float2(hi, __double2float_rn(d - (double)hi));
  }
}

// ---------------------------------------------------------------------------
// Density-weighted classification of the quartet lists, on the device, once
// per Fock build or gradient (the density changes between calls).  With M_xy
// the largest |D| element of the shell block (x, y):
//  * Fock build: a quartet adds at most Q_ab Q_cd * max(2 M_ab, 2 M_cd, M_ac,
//    M_bd, M_ad, M_bc) to any element of J or K (the eight index
//    permutations of hf.py:49-60); the mixed modes keep a quartet of the
//    accurate tier (Q_ab Q_cd >= fp32 cutoff) there only while this bound is
//    >= its cutoff, else it runs in FP32 (demoted);
//  * gradient: every contraction coefficient is bounded by
//    G = M_ab M_cd / 2 + (M_ac M_bd + M_ad M_bc) / 8, so a quartet whose
//    Q_ab Q_cd G is below the drop cutoff is left out (density screening).
//    A derivative integral is larger than the Schwarz bound of its integral
//    by about the square root of the differentiated exponent (d/dA_x of a
//    primitive is 2 alpha x_A times it, whose norm grows as sqrt(alpha)), so
//    one of the accurate tier runs in FP32 when
//    Q_ab Q_cd G (s_a + s_b + s_c + s_d), s = sqrt of the shell's largest
//    exponent, is below the accurate cutoff: quartets of tight core shells
//    stay accurate.
// Every list is compacted into a "kept" and a "demoted" list at the same
// offsets (d_keep, d_dem), order kept within each chunk of 1024 entries, with
// device counts read by the kernels, so nothing synchronises with the host.
struct ClassifySlice {
  int64_t off, n;        // offset in the quartet-list buffer, length
  int x0, y0;            // first global pair of the bra / ket pair class
  int acc;               // accurate tier (FP64 or double-float launch)
  int pad;
};
constexpr int kClsThreads = 256, kClsPer = 4, kClsChunk = kClsThreads * kClsPer;
// default gradient FP32 cutoff / the call's fp32_cutoff, measured against
// FP64 gradients (6-31G* (H2O)16 / 6-31G** C20H42, FP32 cutoff 1e-2): 3e-4
// gives 6.9e-8 / 4.5e-7 Eh/bohr, 1e-3 1.4e-7 / 1.05e-6, 1e-2 1.4e-6 / 9.8e-6
// (the FP32 tier alone leaves 7e-8 / 3e-7)
constexpr double kGradFp32Scale = 3e-2;

// M_xy = max |D| over the Cartesian block of shells x, y (FP32 is enough for a bound)
__global__ void shell_dmax_kernel(const double *D, int n, const int *l, const int *ao, int ns, float *dm) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ns * ns) return;
  const int a = idx / ns, b = idx % ns;
  const int la = l[a], lb = l[b], a0 = ao[a], b0 = ao[b];
  const int na = (la + 1) * (la + 2) / 2, nb = (lb + 1) * (lb + 2) / 2;
  double m = 0.0;
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) m = fmax(m, fabs(D[(int64_t)(a0 + i) * n + b0 + j]));
  dm[idx] = (float)m;
}

__global__ void __launch_bounds__(kClsThreads) classify_kernel(
    const int2 *list, const ClassifySlice *sl, const int2 *blk, const int *pa, const int *pb, const int *pnp,
    const double *pq, const float *dm, const float *sqa, int ns, int grad_mode, double t_drop, double t_acc,
    int2 *keep, int2 *dem, unsigned long long *cnt) {
  const int2 bk = blk[blockIdx.x];
  const ClassifySlice S = sl[bk.x];
  const int64_t e0 = (int64_t)bk.y * kClsChunk + (int64_t)threadIdx.x * kClsPer;
  int2 v[kClsPer];
  int where[kClsPer];   // 0 kept, 1 demoted, 2 left out
  int nk = 0, nd = 0;
  unsigned long long pk = 0, pd = 0;
#pragma unroll
  for (int k = 0; k < kClsPer; ++k) {
    where[k] = 2;
    const int64_t e = e0 + k;
    if (e >= S.n) continue;
    v[k] = list[S.off + e];
    const int pab = S.x0 + v[k].x, pcd = S.y0 + v[k].y;
    const int a = pa[pab], b = pb[pab], c = pa[pcd], d = pb[pcd];
    const float mab = dm[a * ns + b], mcd = dm[c * ns + d], mac = dm[a * ns + c], mbd = dm[b * ns + d],
                mad = dm[a * ns + d], mbc = dm[b * ns + c];
    const double q = pq[pab] * pq[pcd];
    double bound, bound_acc;
    if (grad_mode) {
      bound = q * (double)(0.5f * mab * mcd + 0.125f * (mac * mbd + mad * mbc));
      bound_acc = bound * (double)(sqa[a] + sqa[b] + sqa[c] + sqa[d]);
    } else {
      bound = q * (double)fmaxf(2.0f * fmaxf(mab, mcd), fmaxf(fmaxf(mac, mbd), fmaxf(mad, mbc)));
      bound_acc = bound;
    }
    where[k] = bound < t_drop ? 2 : (S.acc && bound_acc < t_acc) ? 1 : 0;
    const unsigned long long c0 = (unsigned long long)pnp[pab] * (unsigned long long)pnp[pcd];
    if (where[k] == 0) { ++nk; pk += c0; }
    if (where[k] == 1) { ++nd; pd += c0; }
  }
  // exclusive scan of (nk, nd) over the CTA: warp shuffles, then the warp totals
  __shared__ int s_wk[kClsThreads / 32], s_wd[kClsThreads / 32];
  __shared__ unsigned long long s_base[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int ik = nk, id = nd;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int tk = __shfl_up_sync(0xffffffffu, ik, off), td = __shfl_up_sync(0xffffffffu, id, off);
    if (lane >= off) { ik += tk; id += td; }
  }
  unsigned long long sk = pk, sd = pd;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    sk += __shfl_xor_sync(0xffffffffu, sk, off);
    sd += __shfl_xor_sync(0xffffffffu, sd, off);
  }
  if (lane == 31) { s_wk[warp] = ik; s_wd[warp] = id; }
  if (lane == 0) {
    if (sk) atomicAdd(cnt + 4 * bk.x + 2, sk);
    if (sd) atomicAdd(cnt + 4 * bk.x + 3, sd);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int tk = 0, td = 0;
    for (int w = 0; w < kClsThreads / 32; ++w) {
      const int a = s_wk[w], b = s_wd[w];
      s_wk[w] = tk;
      s_wd[w] = td;
      tk += a;
      td += b;
    }
    s_base[0] = tk ? atomicAdd(cnt + 4 * bk.x, (unsigned long long)tk) : 0ull;
    s_base[1] = td ? atomicAdd(cnt + 4 * bk.x + 1, (unsigned long long)td) : 0ull;
  }
  __syncthreads();
  int64_t ok = (int64_t)s_base[0] + s_wk[warp] + ik - nk, od = (int64_t)s_base[1] + s_wd[warp] + id - nd;
#pragma unroll
  for (int k = 0; k < kClsPer; ++k) {
    if (where[k] == 0) keep[S.off + ok++] = v[k];
    else if (where[k] == 1) dem[S.off + od++] = v[k];
  }
}

}  // namespace

struct sf_handle {
  int device = 0;
  int nsm = 0;                     // multiprocessors of the device
  int nshell = 0, nao = 0, natom = 0;
  std::vector<int> l, nprim, atom, ao, spoff;
  std::vector<double> cx, cy, cz, exps, coefs;
  int cstart[kNumPairClass + 1] = {0};
  std::vector<int> pa, pb, ppoff, pnp;
  std::vector<double> pq;
  std::vector<int> pairmap;   // a*nshell+b -> pair index (a,b canonical)
  DBuf<int> d_l, d_nprim, d_ao, d_atom, d_spoff;
  DBuf<double> d_cx, d_cy, d_cz, d_exps, d_coefs;
  DBuf<int> d_pa, d_pb, d_ppoff, d_pnp;
  DBuf<double> d_pq;
  DBuf<double> d_pp64;
  DBuf<float> d_pp32;
  DBuf<float> d_ppdd;              // records as (hi, lo) float pairs
  DBuf<float> d_cdd;               // centres x, y, z as dd: 3 blocks of nshell (hi, lo)
  DBuf<float4> d_tabdd;
  DBuf<float4> d_pair32;           // packed FP32 pair geometry (KParams::pair32)
  DBuf<float> d_Ddd;               // density as dd (per build)
  DBuf<float> d_cx32, d_cy32, d_cz32;
  DBuf<double> d_tab64;
  DBuf<float> d_tab32;
  DBuf<double> d_Jh, d_Kh;
  DBuf<float> d_D32;
  DBuf<int> d_err;
  bool have_schwarz = false;
  // work cache
  struct Slice {
    int cls, prec;
    ClassWork w;
    int64_t quartets, prims;
    double flops;
    int64_t cost_hi;               // primitive cost of the segment's first quartet (tuning key)
  };
  // autotuned primitive splits S = P*W, keyed by (class, precision, cost_hi)
  std::vector<sf_tune_entry> tune;
  int profiling = 0;              // 1: per-slice events; 2: also serialise launches
  std::vector<cudaEvent_t> ev;   // 2 per slice while profiling
  cudaEvent_t prof_t0 = nullptr;  // start of the last profiled build (launch start offsets)
  // side streams: the class launches of one build are independent (they only
  // add into Jh/Kh with atomics), so they are spread over kSideStreams
  // streams forked from and joined back into the caller's stream
  // one hardware work queue per side stream needs CUDA_DEVICE_MAX_CONNECTIONS
  // >= kSideStreams when the context is created (default 8: streams then
  // share queues, and a launch waits behind another stream's launch)
  static constexpr int kSideStreams = 16;
  static constexpr int kHiStreams = 6;   // high-priority side streams (accurate tier of a mixed build)
  cudaStream_t side[kSideStreams] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kSideStreams] = {};
  std::vector<int> slice_stream;   // side stream of each slice (greedy by cost)
  std::vector<Slice> slices;
  DBuf<int2> d_list;
  double c_cut = -1, c_cut32 = -1;
  int c_prec = -1, c_part = -1, c_nparts = -1;
  int64_t st_q[2] = {0, 0}, st_pq[2] = {0, 0}, st_total = 0;
  double st_f[2] = {0, 0};
  int part = 0, nparts = 1;
  // launch-fill target per precision mode, in quarters of "8 resident warps
  // per SM sub-partition" (0: no extra primitive split); set by sf_autotune
  int fill_x4[5] = {4, 4, 4, 4, 4};
  // fill target of the accurate tier of a mixed mode (-1: fill_x4 of the mode)
  int fill_acc_x4[5] = {-1, -1, -1, -1, -1};
  KParams kp;
  // density-weighted classification (see classify_kernel); cutoffs < 0 mean
  // the call's own: fp32_cutoff for the accurate tiers, the Schwarz cutoff
  // for the gradient's drop bound
  int dens_flags = SF_DENS_GRAD;   // SF_DENS_FOCK | SF_DENS_GRAD
  double dens_fock_acc = -1.0, dens_grad_drop = -1.0, dens_grad_acc = -1.0;
  DBuf<float> d_dmax;                      // nshell^2 block maxima of |D|
  DBuf<float> d_sqa;                       // per shell: sqrt of its largest primitive exponent
  DBuf<int2> d_keep, d_dem;                // compacted lists at the offsets of d_list
  DBuf<unsigned long long> d_cnt;          // per slice: kept, demoted quartets; kept, demoted primitive quartets
  DBuf<ClassifySlice> d_csl;
  DBuf<int2> d_blk_acc, d_blk_all;         // classification CTAs (slice, chunk): accurate-tier slices / all
  int nblk_acc = 0, nblk_all = 0;
  // the launches of the last Fock build or gradient: one per slice, plus one
  // FP32 launch per accurate-tier slice for its demoted quartets
  struct Launch {
    int slice, kind, stream, demoted;
    ClassWork w;
    int covered = 0;                       // run by a persistent tier launch, not by its own
  };
  std::vector<Launch> plan;
  bool plan_counts = false;                // quartet counts of the plan live on the device
  bool plan_grad = false;                  // the last plan was a gradient's
  // launch mode SF_LAUNCH_PERSISTENT: the FP32 register-path lists of a Fock
  // build run as one persistent launch per register tier (jk_persist.cu)
  cudaStream_t cap_st = nullptr;           // stream that sf_fock_jk_graph_create captures on
  int launch_mode = SF_LAUNCH_STREAMS;
  int persist_ctas_per_sm = 0;             // 0: the occupancy limit of each tier kernel
  int lists_version = 0, persist_version = -1;
  DBuf<ClassWork> d_pworks;                // the covered lists
  DBuf<int> d_pcls;
  DBuf<int2> d_ptiles;                     // per tier, heaviest first
  DBuf<unsigned> d_pnext;                  // one queue counter per tier
  int ptile_off[kPersistTiers + 1] = {0};
  std::vector<char> slice_covered;
  struct TierLaunch {
    int tier, stream, grid;
  };
  std::vector<TierLaunch> pplan;
};

namespace {

void fill_kparams(sf_handle *h) {
  KParams &k = h->kp;
  k.sh = DevShells{h->d_l.p,  h->d_nprim.p, h->d_ao.p,   h->d_atom.p, h->d_cx.p,
                   h->d_cy.p, h->d_cz.p,    h->d_cx32.p, h->d_cy32.p, h->d_cz32.p};
  k.pr = DevPairs{h->d_pa.p, h->d_pb.p, h->d_ppoff.p, h->d_pnp.p, h->d_pq.p};
  k.p64 = DevPrims<double>{h->d_pp64.p};
  k.p32 = DevPrims<float>{h->d_pp32.p};
  k.tab64 = h->d_tab64.p;
  k.tab32 = h->d_tab32.p;
  k.asym = host_tables().asym;
  k.asym32 = host_tables().asym32;
  k.pdd = DevPrims<dd>{reinterpret_cast<const dd *>(h->d_ppdd.p)};
  k.pair32 = h->d_pair32.p;
  k.cxd = reinterpret_cast<const dd *>(h->d_cdd.p);
  k.cyd = k.cxd + h->nshell;
  k.czd = k.cyd + h->nshell;
  k.tabdd = h->d_tabdd.p;
  for (int n = 0; n <= kMaxRoots; ++n)
    for (int i = 0; i < kMaxRoots; ++i) {
      float a, b;
      dd_split(host_tables().asym.r[n][i], a, b);
      k.asymdd_r[n][i] = dd(a, b);
      dd_split(host_tables().asym.w[n][i], a, b);
      k.asymdd_w[n][i] = dd(a, b);
    }
  k.nao = h->nao;
  k.nsm = h->nsm;
  k.natom = h->natom;
  k.err = h->d_err.p;
}

int upload_pairs(sf_handle *h) {
  {
    std::vector<float4> pg(3 * h->pa.size());
    for (size_t i = 0; i < h->pa.size(); ++i) {
      const int a = h->pa[i], b = h->pb[i];
      pg[3 * i] = make_float4((float)h->cx[a], (float)h->cy[a], (float)h->cz[a], (float)(h->cx[a] - h->cx[b]));
      float ao_a, ao_b, poff, np, fa, fb;
      const int ia = h->ao[a], ib = h->ao[b], ip = h->ppoff[i], inp = h->pnp[i];
      std::memcpy(&ao_a, &ia, 4); std::memcpy(&ao_b, &ib, 4);
      std::memcpy(&poff, &ip, 4); std::memcpy(&np, &inp, 4);
      std::memcpy(&fa, &a, 4); std::memcpy(&fb, &b, 4);
      pg[3 * i + 1] = make_float4((float)(h->cy[a] - h->cy[b]), (float)(h->cz[a] - h->cz[b]), ao_a, ao_b);
      pg[3 * i + 2] = make_float4(poff, np, fa, fb);
    }
    SF_CK(h->d_pair32.upload(pg));
  }
  SF_CK(h->d_pa.upload(h->pa));
  SF_CK(h->d_pb.upload(h->pb));
  SF_CK(h->d_ppoff.upload(h->ppoff));
  SF_CK(h->d_pnp.upload(h->pnp));
  SF_CK(h->d_pq.upload(h->pq));
  h->pairmap.assign((size_t)h->nshell * h->nshell, -1);
  for (size_t i = 0; i < h->pa.size(); ++i) h->pairmap[(size_t)h->pa[i] * h->nshell + h->pb[i]] = (int)i;
  fill_kparams(h);
  return SF_OK;
}

// number of leading ket pairs j (Q sorted descending) with qi * Q_j >= cut
int64_t count_pass(const double *qy, int ny, double qi, double cut) {
  const double *e = std::partition_point(qy, qy + ny, [&](double qj) { return qi * qj >= cut; });
  return e - qy;
}

// greedy longest-processing-time assignment of jobs (cost descending) to
// the side streams
std::vector<int> lpt_streams(const std::vector<double> &cost_desc, int first = 0,
                             int last = sf_handle::kSideStreams) {
  double load[sf_handle::kSideStreams] = {0};
  std::vector<int> s(cost_desc.size(), first);
  for (size_t k = 0; k < cost_desc.size(); ++k) {
    int best = first;
    for (int j = first + 1; j < last; ++j)
      if (load[j] < load[best]) best = j;
    s[k] = best;
    load[best] += cost_desc[k];
  }
  return s;
}

// Quartet lists of every (class, precision) launch for the given cutoffs.
// Each list holds the surviving canonical quartets (bra i, ket j) of one
// class, ordered by decreasing primitive cost K_ab K_cd (then K_ab), stable,
// so consecutive quartets -- the lanes and groups of one warp -- run the same
// number of primitive iterations; inside a cost bucket the (i, j) order of the
// Schwarz-sorted pair lists is kept.  A partition (part, nparts) keeps every
// nparts-th quartet of each sorted list, which balances cost across parts.
// lanes per quartet of a launch of class ci in kind (0 FP64, 1 FP32, 2 dd)
inline int kind_lanes(const ClassInfo &ci, int kind, int wide) {
  return kind == 1 ? ci.t32 : (kind == 2 && wide) ? tdd_wide(ci.la, ci.lb, ci.lc, ci.ld, ci.t64) : ci.t64;
}

int build_work(sf_handle *h, int prec, double cut, double cut32) {
  if (h->c_prec == prec && h->c_cut == cut && h->c_cut32 == cut32 && h->c_part == h->part &&
      h->c_nparts == h->nparts)
    return SF_OK;
  h->slices.clear();
  std::vector<int2> all;
  struct Pending {
    int cls, prec;
    size_t off;
    int64_t n, prims;
    double flops;
    int x0, y0, same;
    int psplit, wsplit;
    int64_t cost_hi;
    int wide;
  };
  std::vector<Pending> pend;
  h->st_q[0] = h->st_q[1] = h->st_pq[0] = h->st_pq[1] = 0;
  h->st_f[0] = h->st_f[1] = 0.0;
  h->st_total = 0;
  constexpr int KB = kMaxPrim * kMaxPrim + 1;   // primitive pairs per shell pair <= 256
  // every class's lists are cut independently, on host threads, then
  // concatenated in class order (the result does not depend on the threads)
  struct Part {   // the list of one (class, tier), offsets relative to it
    std::vector<int2> lst;
    std::vector<Pending> segs;
    int64_t q = 0, pq = 0;
    double f = 0.0;
  };
  std::vector<Part> parts(2 * kNumClass);
  std::vector<int64_t> totals(kNumClass, 0);
  auto build_class = [&](int cls, std::vector<int64_t> &hist) {
    const ClassInfo &ci = kClassInfo[cls];
    const int X = pair_class_of(ci.la, ci.lb), Y = pair_class_of(ci.lc, ci.ld);
    const int x0 = h->cstart[X], y0 = h->cstart[Y];
    const int nX = h->cstart[X + 1] - x0, nY = h->cstart[Y + 1] - y0;
    const int same = X == Y;
    totals[cls] = same ? (int64_t)nX * (nX + 1) / 2 : (int64_t)nX * nY;
    if (nX == 0 || nY == 0) return;
    const double *qx = h->pq.data() + x0, *qy = h->pq.data() + y0;
    std::vector<int64_t> m(nX), m64(nX);
    for (int i = 0; i < nX; ++i) {
      int64_t mi = count_pass(qy, nY, qx[i], cut);
      if (same) mi = std::min<int64_t>(mi, i + 1);
      int64_t m6;
      if (prec == SF_PREC_FP64 || prec == SF_PREC_DF) m6 = mi;
      else if (prec == SF_PREC_FP32) m6 = 0;
      else m6 = std::min<int64_t>(mi, count_pass(qy, nY, qx[i], std::max(cut32, cut)));
      m[i] = mi;
      m64[i] = m6;
    }
    const int nr = (ci.la + ci.lb + ci.lc + ci.ld) / 2 + 1;
    const double nabcd = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
    // launch kind of tier pr: 0 FP64, 1 FP32, 2 double-float
    const int hi_kind = (prec == SF_PREC_MIXED_DF || prec == SF_PREC_DF) ? 2 : 0;
    for (int pr = 0; pr < 2; ++pr) {
      const int kind = pr == 0 ? hi_kind : 1;
      // counting sort on (K_ab, K_cd)
      std::fill(hist.begin(), hist.end(), 0);
      int64_t n = 0;
      for (int i = 0; i < nX; ++i) {
        const int64_t lo = pr == 0 ? 0 : m64[i], hi = pr == 0 ? m64[i] : m[i];
        const int ka = h->pnp[x0 + i];
        for (int64_t j = lo; j < hi; ++j) ++hist[(size_t)ka * KB + h->pnp[y0 + j]];
        n += hi - lo;
      }
      if (n == 0) continue;
      std::vector<int> keys;
      for (int k = 0; k < KB * KB; ++k)
        if (hist[k]) keys.push_back(k);
      std::sort(keys.begin(), keys.end(), [&](int a, int b) {
        const int ca = (a / KB) * (a % KB), cb = (b / KB) * (b % KB);
        return ca != cb ? ca > cb : a > b;
      });
      std::vector<int64_t> pos((size_t)KB * KB, 0);
      int64_t run = 0, prims = 0;
      for (int k : keys) {
        pos[k] = run;
        run += hist[k];
        prims += hist[k] * (int64_t)(k / KB) * (k % KB);
      }
      std::vector<int2> lst(n);
      for (int i = 0; i < nX; ++i) {
        const int64_t lo = pr == 0 ? 0 : m64[i], hi = pr == 0 ? m64[i] : m[i];
        const int ka = h->pnp[x0 + i];
        for (int64_t j = lo; j < hi; ++j) lst[pos[(size_t)ka * KB + h->pnp[y0 + j]]++] = make_int2(i, (int)j);
      }
      Pending p;
      // the double-float accurate tier of a mixed build runs its wide kernels
      p.wide = (kind == 2 && prec == SF_PREC_MIXED_DF) ? 1 : 0;
      p.cost_hi = 0;
      p.psplit = 1;
      p.wsplit = 1;
      p.cls = cls;
      p.prec = kind;
      p.off = 0;
      p.x0 = x0;
      p.y0 = y0;
      p.same = same;
      if (h->nparts > 1) {
        int64_t kept = 0;
        for (int64_t q = h->part; q < n; q += h->nparts) lst[kept++] = lst[q];
        lst.resize(kept);
      }
      const double frac = (double)lst.size() / (double)n;
      p.n = (int64_t)lst.size();
      p.prims = (int64_t)(prims * frac);
      p.flops = ((double)prims * nr * 4.0 * nabcd + 12.0 * nabcd * (double)n) * frac;
      Part &part = parts[2 * cls + pr];
      part.q = p.n;
      part.pq = p.prims;
      part.f = p.flops;
      // split the cost-sorted list into launches with P primitive sub-groups
      // per quartet: heavy quartets (many primitive quartets) get more lanes
      const int T = kind_lanes(ci, kind, p.wide);
      const int pmax = 32 / T;
      auto psplit = [&](int64_t cost) {
        if (pmax > 1 && cost >= 4 * pmax) return pmax;
        if (pmax > 8 && cost >= 32) return 8;
        return 1;
      };
      // a list with fewer lanes than 8 resident warps per SM sub-partition
      // leaves most of the GPU idle and runs at the latency of one warp's
      // instruction stream (an FP64 instruction of one warp occupies its
      // sub-partition's FP64 unit for 64 cycles): its quartets' primitive
      // loops are split further, up to S_fill = P*W sub-groups per quartet,
      // each sub-group keeping at least one primitive quartet
      const int fx4 = (pr == 0 && h->fill_acc_x4[prec] >= 0) ? h->fill_acc_x4[prec] : h->fill_x4[prec];
      const int64_t fill = (int64_t)std::max(h->nsm, 1) * 4 * 8 * 32 * fx4 / 4;
      int sfill = 1;
      while (p.n * T * sfill < fill && sfill < pmax * kMaxWsplit) sfill *= 2;
      auto split_of = [&](int64_t cost) {
        int sc = 1;
        while (2 * sc <= cost && 2 * sc <= sfill) sc *= 2;
        return std::max(psplit(cost), sc);
      };
      int64_t q0 = 0;
      while (q0 < p.n) {
        const auto cost_of = [&](int64_t q) {
          return (int64_t)h->pnp[x0 + lst[q].x] * h->pnp[y0 + lst[q].y];
        };
        const int S = split_of(cost_of(q0));
        int64_t q1 = q0 + 1;
        while (q1 < p.n && split_of(cost_of(q1)) == S) ++q1;
        Pending seg = p;
        seg.off = q0;
        seg.n = q1 - q0;
        seg.cost_hi = cost_of(q0);
        int St = S;
        for (const sf_tune_entry &e : h->tune)
          if (e.cls == cls && e.precision == kind && e.cost == seg.cost_hi) St = e.split;
        seg.psplit = std::min(St, pmax);
        seg.wsplit = std::max(1, std::min(St / seg.psplit, kMaxWsplit));
        int64_t sp = 0;
        for (int64_t q = q0; q < q1; ++q) sp += cost_of(q);
        seg.prims = sp;
        seg.flops = (double)sp * nr * 4.0 * nabcd + 12.0 * nabcd * (double)seg.n;
        part.segs.push_back(seg);
        q0 = q1;
      }
      part.lst = std::move(lst);
    }
    };
  {
    const unsigned hw = std::thread::hardware_concurrency();
    const int nthr = std::max(1, std::min<int>(kNumClass, hw ? (int)hw : 1));
    std::atomic<int> next{0};
    auto worker = [&]() {
      std::vector<int64_t> hist((size_t)KB * KB);
      for (int c = next++; c < kNumClass; c = next++) build_class(c, hist);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthr; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
  }
  for (int cls = 0; cls < kNumClass; ++cls) {
    h->st_total += totals[cls];
    for (int pr = 0; pr < 2; ++pr) {
      Part &part = parts[2 * cls + pr];
      for (Pending seg : part.segs) {
        seg.off += all.size();
        pend.push_back(seg);
      }
      all.insert(all.end(), part.lst.begin(), part.lst.end());
      h->st_q[pr] += part.q;
      h->st_pq[pr] += part.pq;
      h->st_f[pr] += part.f;
    }
  }
  SF_CK(h->d_list.upload(all));
  for (const Pending &p : pend) {
    ClassWork w;
    w.list = h->d_list.p + p.off;
    w.n = p.n;
    w.x0 = p.x0;
    w.y0 = p.y0;
    w.same = p.same;
    w.psplit = p.psplit;
    w.wsplit = p.wsplit;
    w.max_cost = (int)std::max<int64_t>(p.cost_hi, 1);
    w.wide = p.wide;
    h->slices.push_back({p.cls, p.prec, w, p.n, p.prims, p.flops, p.cost_hi});
  }
  // greedy longest-processing-time assignment of slices to side streams;
  // cost estimate: primitive quartets x roots x Cartesian outputs, FP64 work
  // weighted by the FP64:FP32 throughput ratio of the part
  {
    std::vector<int> order(h->slices.size());
    std::vector<double> cost(h->slices.size());
    for (size_t k = 0; k < h->slices.size(); ++k) {
      const auto &sl = h->slices[k];
      const ClassInfo &ci = kClassInfo[sl.cls];
      const double nr = (ci.la + ci.lb + ci.lc + ci.ld) / 2 + 1;
      const double nc = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
      cost[k] = (double)sl.prims * (nr * (nc + 30.0) + 40.0) * (sl.prec == 0 ? 16.0 : sl.prec == 2 ? 5.0 : 1.0);
    }
    // launches timed by the autotuner: their measured times (a latency-bound
    // launch of few quartets costs far more than its work suggests)
    bool all_timed = !h->slices.empty();
    std::vector<double> timed(h->slices.size(), 0.0);
    for (size_t k = 0; k < h->slices.size() && all_timed; ++k) {
      const auto &sl = h->slices[k];
      bool found = false;
      for (const sf_tune_entry &e : h->tune)
        if (e.cls == sl.cls && e.precision == sl.prec && e.cost == sl.cost_hi && e.ms_tuned > 0.f) {
          timed[k] = e.ms_tuned;
          found = true;
        }
      all_timed = found;
    }
    if (all_timed) cost = timed;
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<sf_handle::Slice> sorted;
    for (int k : order) sorted.push_back(h->slices[k]);
    h->slices.swap(sorted);
    std::sort(cost.begin(), cost.end(), std::greater<double>());
    bool has32 = false, hasacc = false;
    for (const auto &sl : h->slices) (sl.prec == 1 ? has32 : hasacc) = true;
    if (has32 && hasacc) {
      // mixed build: accurate-tier launches on the high-priority streams,
      // FP32 launches on the others, each group balanced by LPT
      std::vector<double> ca, cf;
      for (size_t k = 0; k < h->slices.size(); ++k) (h->slices[k].prec == 1 ? cf : ca).push_back(cost[k]);
      const std::vector<int> sa = lpt_streams(ca, 0, sf_handle::kHiStreams);
      const std::vector<int> sf = lpt_streams(cf, sf_handle::kHiStreams, sf_handle::kSideStreams);
      h->slice_stream.assign(h->slices.size(), 0);
      size_t ia = 0, ifp = 0;
      for (size_t k = 0; k < h->slices.size(); ++k)
        h->slice_stream[k] = h->slices[k].prec == 1 ? sf[ifp++] : sa[ia++];
    } else {
      h->slice_stream = lpt_streams(cost);
    }
  }
  // tables of the density-weighted classification
  {
    std::vector<ClassifySlice> csl(h->slices.size());
    std::vector<int2> ba, bl;
    for (size_t k = 0; k < h->slices.size(); ++k) {
      const auto &sl = h->slices[k];
      csl[k] = ClassifySlice{(int64_t)(sl.w.list - h->d_list.p), sl.w.n, sl.w.x0, sl.w.y0, sl.prec != 1 ? 1 : 0, 0};
      for (int64_t c = 0; c * kClsChunk < sl.w.n; ++c) {
        bl.push_back(make_int2((int)k, (int)c));
        if (sl.prec != 1) ba.push_back(make_int2((int)k, (int)c));
      }
    }
    SF_CK(h->d_csl.upload(csl));
    SF_CK(h->d_blk_acc.upload(ba));
    SF_CK(h->d_blk_all.upload(bl));
    h->nblk_acc = (int)ba.size();
    h->nblk_all = (int)bl.size();
    SF_CK(h->d_keep.alloc(all.size()));
    SF_CK(h->d_dem.alloc(all.size()));
    SF_CK(h->d_cnt.alloc(4 * std::max<size_t>(h->slices.size(), 1)));
    SF_CK(h->d_dmax.alloc((size_t)h->nshell * h->nshell));
  }
  ++h->lists_version;
  h->c_prec = prec;
  h->c_cut = cut;
  h->c_cut32 = cut32;
  h->c_part = h->part;
  h->c_nparts = h->nparts;
  return SF_OK;
}

// Classify the current lists against the density D (see classify_kernel):
// for a Fock build only in the mixed modes (demotion of the accurate tier),
// for a gradient always (drop bound; demotion too in the mixed modes).
// Returns 1 when the launches must read the compacted lists, 0 when the
// lists are used as they are.
int density_classify(sf_handle *h, const double *D, bool grad, double cut, double cut32, cudaStream_t st,
                     int *launches, int *active) {
  *active = 0;
  if (!(h->dens_flags & (grad ? SF_DENS_GRAD : SF_DENS_FOCK)) || h->slices.empty()) return SF_OK;
  bool has32 = false, hasacc = false;
  for (const auto &sl : h->slices) (sl.prec == 1 ? has32 : hasacc) = true;
  const bool mixed = has32 && hasacc;
  if (!grad && !mixed) return SF_OK;
  // default FP32 cutoffs: the call's own for the Fock build, kGradFp32Scale
  // times it for the gradient
  const double t_acc = !mixed ? -1.0
                       : grad ? (h->dens_grad_acc >= 0.0 ? h->dens_grad_acc : cut32 * kGradFp32Scale)
                              : (h->dens_fock_acc >= 0.0 ? h->dens_fock_acc : cut32);
  const double t_drop = grad ? (h->dens_grad_drop >= 0.0 ? h->dens_grad_drop : cut) : -1.0;
  const int nb = grad ? h->nblk_all : h->nblk_acc;
  const int ns = h->nshell;
  SF_CK(cudaMemsetAsync(h->d_cnt.p, 0, 4 * h->slices.size() * sizeof(unsigned long long), st));
  shell_dmax_kernel<<<(unsigned)((ns * ns + 255) / 256), 256, 0, st>>>(D, h->nao, h->d_l.p, h->d_ao.p, ns,
                                                                       h->d_dmax.p);
  SF_CK(cudaGetLastError());
  if (nb > 0) {
    classify_kernel<<<(unsigned)nb, kClsThreads, 0, st>>>(
        h->d_list.p, h->d_csl.p, grad ? h->d_blk_all.p : h->d_blk_acc.p, h->d_pa.p, h->d_pb.p, h->d_pnp.p, h->d_pq.p,
        h->d_dmax.p, h->d_sqa.p, ns, grad ? 1 : 0, t_drop, t_acc, h->d_keep.p, h->d_dem.p, h->d_cnt.p);
    SF_CK(cudaGetLastError());
  }
  if (launches) *launches += nb > 0 ? 2 : 1;
  *active = 1;
  return SF_OK;
}

// Tile tables of the persistent tier launches for the current lists: every
// FP32 slice of a class in a register tier is cut into tiles of kBlock / P
// quartet groups (one CTA trip of the class kernel); a tier's tiles are
// ordered by estimated cost, heaviest first (primitive quartets x roots x
// (outputs + 30) per tile, from the slice's mean cost), so the long tiles
// start first and the short ones fill the end.
int build_persist(sf_handle *h) {
  std::vector<ClassWork> works;
  std::vector<int> cls;
  struct T {
    double cost;
    int tier, work, tile;
  };
  std::vector<T> tiles;
  h->slice_covered.assign(h->slices.size(), 0);
  for (size_t k = 0; k < h->slices.size(); ++k) {
    const auto &sl = h->slices[k];
    const int tier = sl.prec == 1 ? persist_tier_of(sl.cls) : -1;
    if (tier < 0 || sl.w.n <= 0) continue;
    h->slice_covered[k] = 1;
    const int P = std::max(1, sl.w.psplit), W = std::max(1, sl.w.wsplit);
    const int64_t groups = sl.w.n * W, per = kBlock / P;
    const int64_t nt = (groups + per - 1) / per;
    const ClassInfo &ci = kClassInfo[sl.cls];
    const double nr = (ci.la + ci.lb + ci.lc + ci.ld) / 2 + 1;
    const double nc = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
    const double per_q = (double)sl.prims / (double)std::max<int64_t>(sl.quartets, 1) * nr * (nc + 30.0);
    const int widx = (int)works.size();
    works.push_back(sl.w);
    cls.push_back(sl.cls);
    for (int64_t c = 0; c < nt; ++c) {
      const int64_t g0 = c * per, g1 = std::min(groups, g0 + per);
      tiles.push_back(T{per_q * (double)(g1 - g0) / W, tier, widx, (int)c});
    }
  }
  std::stable_sort(tiles.begin(), tiles.end(), [](const T &a, const T &b) {
    return a.tier != b.tier ? a.tier < b.tier : a.cost > b.cost;
  });
  std::vector<int2> tl(tiles.size());
  for (int t = 0; t <= kPersistTiers; ++t) h->ptile_off[t] = 0;
  for (size_t i = 0; i < tiles.size(); ++i) {
    tl[i] = make_int2(tiles[i].work, tiles[i].tile);
    ++h->ptile_off[tiles[i].tier + 1];
  }
  for (int t = 0; t < kPersistTiers; ++t) h->ptile_off[t + 1] += h->ptile_off[t];
  SF_CK(h->d_pworks.upload(works));
  SF_CK(h->d_pcls.upload(cls));
  SF_CK(h->d_ptiles.upload(tl));
  SF_CK(h->d_pnext.alloc(kPersistTiers));
  h->persist_version = h->lists_version;
  return SF_OK;
}

// The launches of one call: one per slice (reading its compacted list when
// the classification ran for it) and, for a classified accurate-tier slice of
// a mixed mode, one FP32 launch of its demoted quartets on the next FP32
// stream.  In the persistent launch mode (Fock builds, profiling off) the
// slices of the register tiers are marked covered and one launch per tier
// runs them, on the FP32 streams.
int make_plan(sf_handle *h, bool grad, int active) {
  h->plan.clear();
  h->pplan.clear();
  h->plan_grad = grad;
  const bool persist = h->launch_mode == SF_LAUNCH_PERSISTENT && !grad && h->profiling == 0;
  if (persist && h->persist_version != h->lists_version) {
    const int rc = build_persist(h);
    if (rc) return rc;
  }
  h->plan_counts = active != 0;
  bool has32 = false, hasacc = false;
  for (const auto &sl : h->slices) (sl.prec == 1 ? has32 : hasacc) = true;
  const bool mixed = has32 && hasacc;
  int rr = 0;
  for (size_t k = 0; k < h->slices.size(); ++k) {
    const auto &sl = h->slices[k];
    const bool cl = active && (grad || sl.prec != 1);
    const int64_t off = sl.w.list - h->d_list.p;
    sf_handle::Launch L{(int)k, sl.prec, h->slice_stream[k], 0, sl.w};
    if (cl) {
      L.w.list = h->d_keep.p + off;
      L.w.count = h->d_cnt.p + 4 * k;
    }
    h->plan.push_back(L);
    if (cl && mixed && sl.prec != 1) {
      sf_handle::Launch Dm{(int)k, 1, sf_handle::kHiStreams + rr, 1, sl.w};
      rr = (rr + 1) % (sf_handle::kSideStreams - sf_handle::kHiStreams);
      Dm.w.list = h->d_dem.p + off;
      Dm.w.count = h->d_cnt.p + 4 * k + 1;
      const int S = std::max(1, sl.w.psplit) * std::max(1, sl.w.wsplit);
      const int pmax = 32 / kClassInfo[sl.cls].t32;
      Dm.w.psplit = std::min(S, pmax);
      Dm.w.wsplit = std::max(1, std::min(S / Dm.w.psplit, kMaxWsplit));
      h->plan.push_back(Dm);
    }
  }
  if (persist) {
    for (auto &L : h->plan)
      if (!L.demoted && L.kind == 1 && h->slice_covered[L.slice]) L.covered = 1;
    for (int t = 0; t < kPersistTiers; ++t) {
      if (h->ptile_off[t + 1] == h->ptile_off[t]) continue;
      int bps = h->persist_ctas_per_sm;
      if (bps <= 0) SF_CK(persist_blocks_per_sm(t, &bps));
      const int grid = std::max(1, h->nsm) * std::max(1, bps);
      h->pplan.push_back(sf_handle::TierLaunch{t, sf_handle::kHiStreams + t, grid});
    }
  }
  return SF_OK;
}

// Run fn(k, stream) for every slice k on its side stream (forked from st,
// joined back into st).
template <typename F>
int fan_out_list(sf_handle *h, cudaStream_t st, const std::vector<int> &stream_of, F &&fn) {
  SF_CK(cudaEventRecord(h->fork_ev, st));
  bool used[sf_handle::kSideStreams] = {false};
  for (int j : stream_of) used[j] = true;
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) SF_CK(cudaStreamWaitEvent(h->side[j], h->fork_ev, 0));
  for (size_t k = 0; k < stream_of.size(); ++k) SF_CK(fn(k, h->side[stream_of[k]]));
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) {
      SF_CK(cudaEventRecord(h->join_ev[j], h->side[j]));
      SF_CK(cudaStreamWaitEvent(st, h->join_ev[j], 0));
    }
  return SF_OK;
}



// one launch of the current quartet lists, in its kind's arithmetic
cudaError_t launch_slice(sf_handle *h, const sf_handle::Slice &s, const ClassWork &w, const double *D,
                         const float *D32, double *Jh, double *Kh, cudaStream_t st) {
  if (s.prec == 0) return launch_jk_f64(s.cls, h->kp, w, D, Jh, Kh, st);
  if (s.prec == 1) return launch_jk_f32(s.cls, h->kp, w, D32, Jh, Kh, st);
  return launch_jk_dd(s.cls, h->kp, w, reinterpret_cast<const dd *>(h->d_Ddd.p), Jh, Kh, st);
}

int profiling_events(sf_handle *h, cudaStream_t st);

// one launch of the plan: J/K digestion (Jh, Kh) or gradient (g) kernels in
// the launch's arithmetic
cudaError_t launch_one(sf_handle *h, const sf_handle::Launch &L, bool grad, const double *D, const float *D32,
                       double *Jh, double *Kh, double *g, cudaStream_t st) {
  const int cls = h->slices[L.slice].cls;
  const dd *Ddd = reinterpret_cast<const dd *>(h->d_Ddd.p);
  if (grad) {
    if (L.kind == 0) return launch_grad_f64(cls, h->kp, L.w, D, g, st);
    if (L.kind == 1) return launch_grad_f32(cls, h->kp, L.w, D32, g, st);
    return launch_grad_dd(cls, h->kp, L.w, Ddd, g, st);
  }
  if (L.kind == 0) return launch_jk_f64(cls, h->kp, L.w, D, Jh, Kh, st);
  if (L.kind == 1) return launch_jk_f32(cls, h->kp, L.w, D32, Jh, Kh, st);
  return launch_jk_dd(cls, h->kp, L.w, Ddd, Jh, Kh, st);
}

// Run every launch of the plan on its side stream (forked from st, joined
// back into st); profiling 1: events bracket each launch on its own stream;
// profiling 2: the launches are serialised on st, each between two events.
int run_plan(sf_handle *h, bool grad, const double *D, const float *D32, double *Jh, double *Kh, double *g,
             cudaStream_t st, int profiling, int *launches) {
  if (profiling == 2) {
    for (size_t k = 0; k < h->plan.size(); ++k) {
      SF_CK(cudaEventRecord(h->ev[2 * k], st));
      SF_CK(launch_one(h, h->plan[k], grad, D, D32, Jh, Kh, g, st));
      SF_CK(cudaEventRecord(h->ev[2 * k + 1], st));
      if (launches) ++*launches;
    }
    return SF_OK;
  }
  SF_CK(cudaEventRecord(h->fork_ev, st));
  bool used[sf_handle::kSideStreams] = {false};
  for (const auto &L : h->plan)
    if (!L.covered) used[L.stream] = true;
  for (const auto &T : h->pplan) used[T.stream] = true;
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) SF_CK(cudaStreamWaitEvent(h->side[j], h->fork_ev, 0));
  for (size_t k = 0; k < h->plan.size(); ++k) {
    const auto &L = h->plan[k];
    if (L.covered) continue;
    cudaStream_t ss = h->side[L.stream];
    if (profiling) SF_CK(cudaEventRecord(h->ev[2 * k], ss));
    SF_CK(launch_one(h, L, grad, D, D32, Jh, Kh, g, ss));
    if (profiling) SF_CK(cudaEventRecord(h->ev[2 * k + 1], ss));
    if (launches) ++*launches;
  }
  // the persistent tier launches last: they take the SM slots the others leave
  for (const auto &T : h->pplan) {
    PersistWork pw{h->d_pworks.p, h->d_pcls.p, h->d_ptiles.p + h->ptile_off[T.tier],
                   h->ptile_off[T.tier + 1] - h->ptile_off[T.tier], h->d_pnext.p + T.tier};
    SF_CK(launch_jk_persist_f32(T.tier, h->kp, pw, T.grid, D32, Jh, Kh, h->side[T.stream]));
    if (launches) ++*launches;
  }
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) {
      SF_CK(cudaEventRecord(h->join_ev[j], h->side[j]));
      SF_CK(cudaStreamWaitEvent(st, h->join_ev[j], 0));
    }
  return SF_OK;
}

// classification, plan and launches of one Fock build (Jh, Kh) or gradient (g)
int run_call(sf_handle *h, bool grad, const double *D, const float *D32, double *Jh, double *Kh, double *g,
             double cut, double cut32, cudaStream_t st, int profiling, int *launches) {
  int active = 0;
  int rc = density_classify(h, D, grad, cut, cut32, st, launches, &active);
  if (rc) return rc;
  rc = make_plan(h, grad, active);
  if (rc) return rc;
  if (profiling) {
    rc = profiling_events(h, st);
    if (rc) return rc;
  }
  return run_plan(h, grad, D, D32, Jh, Kh, g, st, profiling, launches);
}

// events of the profiling modes: two per launch plus the build's start,
// recorded on the caller's stream before the launches fork
int profiling_events(sf_handle *h, cudaStream_t st) {
  while (h->ev.size() < 2 * h->plan.size()) {
    cudaEvent_t e;
    SF_CK(cudaEventCreate(&e));
    h->ev.push_back(e);
  }
  if (!h->prof_t0) SF_CK(cudaEventCreate(&h->prof_t0));
  SF_CK(cudaEventRecord(h->prof_t0, st));
  return SF_OK;
}

// FP32 / double-float copies of D needed by the current launch list
int convert_density(sf_handle *h, const double *D, float *D32, cudaStream_t st, int *launches) {
  const size_t nn = (size_t)h->nao * h->nao;
  bool need32 = false, needdd = false;
  for (const auto &s : h->slices) {
    need32 |= s.prec == 1;
    needdd |= s.prec == 2;
  }
  if (need32) {
    to_float_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(D, D32, (int64_t)nn);
    SF_CK(cudaGetLastError());
    if (launches) ++*launches;
  }
  if (needdd) {
    to_dd_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(D, reinterpret_cast<float2 *>(h->d_Ddd.p),
                                                                (int64_t)nn);
    SF_CK(cudaGetLastError());
    if (launches) ++*launches;
  }
  return SF_OK;
}

// work counters of the last plan: the host counts of the lists, or, when the
// lists were classified on the device, the device counts (the stream must be
// synchronised)
// grad: the algorithmic FLOPs of derivative quartets instead, per surviving
// quartet K_aK_bK_cK_d n' 36 N_c (nine derivative components -- centres A,
// B, C times x, y, z -- each a 4-FLOP assembly Ix' Iy Iz w per output, root
// and primitive quartet; n' = floor((L+1)/2) + 1 roots)
int plan_stats(sf_handle *h, sf_stats *stats, bool grad = false) {
  stats->quartets_total = h->st_total;
  stats->reserved = 0;
  if (!h->plan_counts && !grad) {
    stats->quartets_fp64 = h->st_q[0];
    stats->quartets_fp32 = h->st_q[1];
    stats->prim_quartets_fp64 = h->st_pq[0];
    stats->prim_quartets_fp32 = h->st_pq[1];
    stats->flop_alg_fp64 = h->st_f[0];
    stats->flop_alg_fp32 = h->st_f[1];
    return SF_OK;
  }
  std::vector<unsigned long long> c(4 * h->slices.size());
  if (h->plan_counts)
    SF_CK(cudaMemcpy(c.data(), h->d_cnt.p, c.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  int64_t q[2] = {0, 0}, pq[2] = {0, 0};
  double f[2] = {0.0, 0.0};
  for (const auto &L : h->plan) {
    const auto &sl = h->slices[L.slice];
    const ClassInfo &ci = kClassInfo[sl.cls];
    const int lsum = ci.la + ci.lb + ci.lc + ci.ld;
    const double nr = grad ? (lsum + 1) / 2 + 1 : lsum / 2 + 1;
    const double nabcd = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
    int64_t nq = sl.quartets, np = sl.prims;
    if (L.w.count) {
      const size_t o = 4 * (size_t)L.slice + (L.demoted ? 1 : 0);
      nq = (int64_t)c[o];
      np = (int64_t)c[o + 2];
    }
    const int t = L.kind == 1 ? 1 : 0;
    q[t] += nq;
    pq[t] += np;
    f[t] += grad ? (double)np * nr * 36.0 * nabcd : (double)np * nr * 4.0 * nabcd + 12.0 * nabcd * (double)nq;
  }
  stats->quartets_fp64 = q[0];
  stats->quartets_fp32 = q[1];
  stats->prim_quartets_fp64 = pq[0];
  stats->prim_quartets_fp32 = pq[1];
  stats->flop_alg_fp64 = f[0];
  stats->flop_alg_fp32 = f[1];
  return SF_OK;
}

}  // namespace

// A raw-ERI batch prepared once and run any number of times: the quartets,
// canonicalised (l_a >= l_b, l_c >= l_d, pair class of ab >= cd) and grouped
// by class, each class list ordered by primitive cost K_ab K_cd descending so
// that the lanes of a warp run equal primitive loops; cut into launches by
// the primitive split P of each precision; launches spread over the side
// streams.  Outputs stay in input order (offsets as given, or packed).
struct sf_eri_plan {
  sf_handle *h = nullptr;
  int64_t nq = 0, total = 0, prims = 0;
  double flops = 0.0;
  std::vector<int64_t> offsets;
  struct Seg {
    int cls, psplit;
    int64_t n;
    size_t off;
  };
  std::vector<Seg> segs[2];          // [FP64 and double-float (same lanes per quartet), FP32]
  std::vector<int> seg_stream[2];
  DBuf<int> d_pab, d_pcd, d_fl, d_str;
  DBuf<int64_t> d_off;
};

namespace {

int build_eri_plan(sf_handle *h, const int32_t *hq, int64_t nq, const int64_t *hoff, sf_eri_plan *pl) {
  pl->h = h;
  pl->nq = nq;
  pl->offsets.assign(nq, 0);
  struct Item {
    int pab, pcd;
    int64_t off;
    int str[4];
    int cost;
  };
  std::vector<std::vector<Item>> byc(kNumClass);
  int64_t run = 0, maxend = 0;
  for (int64_t q = 0; q < nq; ++q) {
    int s[4], pos[4] = {0, 1, 2, 3};
    for (int k = 0; k < 4; ++k) {
      s[k] = hq[4 * q + k];
      if (s[k] < 0 || s[k] >= h->nshell) return fail(SF_EINVAL, "sf_eri_plan: shell index out of range");
    }
    int nc[4], so[4];
    for (int k = 0; k < 4; ++k) nc[k] = ncart(h->l[s[k]]);
    so[3] = 1;
    so[2] = nc[3];
    so[1] = nc[2] * nc[3];
    so[0] = nc[1] * nc[2] * nc[3];
    const int64_t size = (int64_t)nc[0] * so[0];
    const int64_t off = hoff ? hoff[q] : run;
    if (off < 0) return fail(SF_EINVAL, "sf_eri_plan: negative output offset");
    pl->offsets[q] = off;
    run += size;
    maxend = std::max(maxend, off + size);
    auto before = [&](int x, int y) { return h->l[x] < h->l[y] || (h->l[x] == h->l[y] && x < y); };
    if (before(s[0], s[1])) { std::swap(s[0], s[1]); std::swap(pos[0], pos[1]); }
    if (before(s[2], s[3])) { std::swap(s[2], s[3]); std::swap(pos[2], pos[3]); }
    const int X = pair_class_of(h->l[s[0]], h->l[s[1]]), Y = pair_class_of(h->l[s[2]], h->l[s[3]]);
    int x = X, y = Y;
    if (X < Y) {
      std::swap(s[0], s[2]); std::swap(s[1], s[3]);
      std::swap(pos[0], pos[2]); std::swap(pos[1], pos[3]);
      std::swap(x, y);
    }
    Item it;
    it.pab = h->pairmap[(size_t)s[0] * h->nshell + s[1]];
    it.pcd = h->pairmap[(size_t)s[2] * h->nshell + s[3]];
    if (it.pab < 0 || it.pcd < 0) return fail(SF_EINVAL, "sf_eri_plan: internal pair lookup failed");
    it.off = off;
    for (int k = 0; k < 4; ++k) it.str[k] = so[pos[k]];
    it.cost = h->pnp[it.pab] * h->pnp[it.pcd];
    byc[x * (x + 1) / 2 + y].push_back(it);
  }
  pl->total = maxend;
  std::vector<int> pab, pcd, fl, str;
  std::vector<int64_t> off;
  pab.reserve(nq); pcd.reserve(nq); fl.reserve(nq); off.reserve(nq); str.reserve(4 * nq);
  std::vector<double> cost[2];
  for (int cls = 0; cls < kNumClass; ++cls) {
    auto &v = byc[cls];
    if (v.empty()) continue;
    std::stable_sort(v.begin(), v.end(), [](const Item &a, const Item &b) { return a.cost > b.cost; });
    const size_t base = pab.size();
    const ClassInfo &ci = kClassInfo[cls];
    const int nr = (ci.la + ci.lb + ci.lc + ci.ld) / 2 + 1;
    const double nabcd = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
    for (const Item &it : v) {
      pab.push_back(it.pab); pcd.push_back(it.pcd); fl.push_back(0); off.push_back(it.off);
      for (int k = 0; k < 4; ++k) str.push_back(it.str[k]);
      pl->prims += it.cost;
      pl->flops += (double)it.cost * nr * 4.0 * nabcd;
    }
    for (int pr = 0; pr < 2; ++pr) {
      const int T = pr == 0 ? ci.t64 : ci.t32;
      const int pmax = 32 / T;
      auto psplit = [&](int64_t c) {
        if (pmax > 1 && c >= 4 * pmax) return pmax;
        if (pmax > 8 && c >= 32) return 8;
        return 1;
      };
      size_t q0 = 0;
      while (q0 < v.size()) {
        const int P = psplit(v[q0].cost);
        size_t q1 = q0 + 1;
        double c = v[q0].cost;
        while (q1 < v.size() && psplit(v[q1].cost) == P) c += v[q1++].cost;
        pl->segs[pr].push_back({cls, P, (int64_t)(q1 - q0), base + q0});
        cost[pr].push_back(c * nr * (nabcd + 30.0));
        q0 = q1;
      }
    }
  }
  for (int pr = 0; pr < 2; ++pr) {
    std::vector<int> order(pl->segs[pr].size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[pr][a] > cost[pr][b]; });
    std::vector<sf_eri_plan::Seg> sorted;
    std::vector<double> cs;
    for (int k : order) {
      sorted.push_back(pl->segs[pr][k]);
      cs.push_back(cost[pr][k]);
    }
    pl->segs[pr].swap(sorted);
    pl->seg_stream[pr] = lpt_streams(cs);
  }
  SF_CK(pl->d_pab.upload(pab));
  SF_CK(pl->d_pcd.upload(pcd));
  SF_CK(pl->d_fl.upload(fl));
  SF_CK(pl->d_str.upload(str));
  SF_CK(pl->d_off.upload(off));
  return SF_OK;
}

int run_eri_plan(sf_eri_plan *pl, int precision, double *out, cudaStream_t st) {
  sf_handle *h = pl->h;
  const int pr = precision == SF_PREC_FP32 ? 1 : 0;
  const auto &segs = pl->segs[pr];
  if (segs.empty()) return SF_OK;
  return fan_out_list(h, st, pl->seg_stream[pr], [&](size_t k, cudaStream_t ss) {
    const sf_eri_plan::Seg &sg = segs[k];
    EriWork w{pl->d_pab.p + sg.off, pl->d_pcd.p + sg.off, pl->d_fl.p + sg.off, pl->d_off.p + sg.off,
              pl->d_str.p + 4 * sg.off, sg.n, out, sg.psplit};
    if (precision == SF_PREC_DF) return launch_eri_dd(sg.cls, h->kp, w, ss);
    return launch_eri(sg.cls, pr, h->kp, w, ss);
  });
}

}  // namespace

// Scratch of sf_fock_jk_noalloc: Jh and Kh (nao^2 doubles each) followed by
// the single-precision copy of D (nao^2 floats), for nao <= SF_NOALLOC_MAX_NAO.
static constexpr size_t kNoAllocNN = (size_t)SF_NOALLOC_MAX_NAO * SF_NOALLOC_MAX_NAO;
static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocNN + (kNoAllocNN + 1) / 2];

namespace {
// device address of g_noalloc_scratch per device (host code cannot use the
// symbol itself as a device pointer)
std::mutex g_noalloc_mu;
double *g_noalloc_dev[128] = {nullptr};
}  // namespace

extern "C" {

int sf_version(void) { return 100; }

const char *sf_last_error(void) { return g_err.c_str(); }

int32_t sf_nao(const sf_handle *h) { return h ? h->nao : -1; }

int64_t sf_npairs(const sf_handle *h) { return h ? (int64_t)h->pa.size() : -1; }

int sf_create(const sf_shell_desc *shells, int32_t nshell, sf_handle **out) {
  if (!out) return fail(SF_EINVAL, "sf_create: out is NULL");
  *out = nullptr;
  if (!shells || nshell <= 0) return fail(SF_EINVAL, "sf_create: no shells");
  for (int s = 0, ao = 0; s < nshell; ++s) {
    const sf_shell_desc &d = shells[s];
    if (d.l < 0 || d.l > SF_MAX_L) return fail(SF_EUNSUPPORTED, "sf_create: shell " + std::to_string(s) + " has l > 2");
    if (d.nprim < 1 || d.nprim > SF_MAX_PRIM)
      return fail(SF_EUNSUPPORTED, "sf_create: shell " + std::to_string(s) + " has an unsupported contraction length");
    if (!d.exps || !d.coefs) return fail(SF_EINVAL, "sf_create: NULL primitive arrays");
    if (d.ao_offset != ao) return fail(SF_EINVAL, "sf_create: ao_offset of shell " + std::to_string(s) + " is not contiguous");
    for (int k = 0; k < d.nprim; ++k)
      if (!(d.exps[k] > 0.0) || !std::isfinite(d.exps[k]) || !std::isfinite(d.coefs[k]))
        return fail(SF_EINVAL, "sf_create: bad exponent/coefficient in shell " + std::to_string(s));
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(d.center[k])) return fail(SF_EINVAL, "sf_create: non-finite centre of shell " + std::to_string(s));
    if (d.atom < 0) return fail(SF_EINVAL, "sf_create: negative atom index of shell " + std::to_string(s));
    ao += ncart(d.l);
  }
  sf_handle *h = new sf_handle();
  std::unique_ptr<sf_handle> guard(h);
  SF_CK(cudaGetDevice(&h->device));
  SF_CK(cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device));
  h->nshell = nshell;
  h->spoff.push_back(0);
  int nao = 0;
  for (int s = 0; s < nshell; ++s) {
    const sf_shell_desc &d = shells[s];
    h->l.push_back(d.l);
    h->nprim.push_back(d.nprim);
    h->atom.push_back(d.atom);
    h->ao.push_back(d.ao_offset);
    h->cx.push_back(d.center[0]);
    h->cy.push_back(d.center[1]);
    h->cz.push_back(d.center[2]);
    for (int k = 0; k < d.nprim; ++k) {
      h->exps.push_back(d.exps[k]);
      h->coefs.push_back(d.coefs[k]);
    }
    h->spoff.push_back((int)h->exps.size());
    nao += ncart(d.l);
  }
  h->nao = nao;
  for (int s = 0; s < nshell; ++s) h->natom = std::max(h->natom, h->atom[s] + 1);
  // canonical shell pairs, grouped by pair class
  const double kpre = std::sqrt(2.0) * std::pow(3.14159265358979323846, 1.25);
  std::vector<double> pp[8];
  for (int pc = 0; pc < kNumPairClass; ++pc) {
    h->cstart[pc] = (int)h->pa.size();
    const int la = kPairL[pc][0], lb = kPairL[pc][1];
    for (int a = 0; a < nshell; ++a) {
      if (h->l[a] != la) continue;
      for (int b = 0; b < nshell; ++b) {
        if (h->l[b] != lb || (la == lb && b > a)) continue;
        h->pa.push_back(a);
        h->pb.push_back(b);
        h->ppoff.push_back((int)pp[0].size());
        h->pnp.push_back(h->nprim[a] * h->nprim[b]);
        h->pq.push_back(0.0);
        const double ABx = h->cx[a] - h->cx[b], ABy = h->cy[a] - h->cy[b], ABz = h->cz[a] - h->cz[b];
        const double AB2 = ABx * ABx + ABy * ABy + ABz * ABz;
        for (int i = h->spoff[a]; i < h->spoff[a + 1]; ++i)
          for (int j = h->spoff[b]; j < h->spoff[b + 1]; ++j) {
            const double al = h->exps[i], be = h->exps[j], p = al + be;
            pp[0].push_back(p);
            pp[1].push_back((al * h->cx[a] + be * h->cx[b]) / p);
            pp[2].push_back((al * h->cy[a] + be * h->cy[b]) / p);
            pp[3].push_back((al * h->cz[a] + be * h->cz[b]) / p);
            pp[4].push_back(h->coefs[i] * h->coefs[j] * std::exp(-al * be / p * AB2) * kpre / p);
            pp[5].push_back(0.5 / p);
            pp[6].push_back(al);   // exponents of the two primitives (gradients)
            pp[7].push_back(be);
          }
      }
    }
  }
  h->cstart[kNumPairClass] = (int)h->pa.size();
  {
    const size_t npp = pp[0].size();
    std::vector<double> rec(npp * kPrimRec, 0.0);
    for (size_t i = 0; i < npp; ++i)
      for (int f = 0; f < kPrimRec; ++f) rec[i * kPrimRec + f] = pp[f][i];
    SF_CK(h->d_pp64.upload(rec));
    std::vector<float> rec32(rec.begin(), rec.end());
    SF_CK(h->d_pp32.upload(rec32));
    std::vector<float> recdd(2 * rec.size());
    for (size_t i = 0; i < rec.size(); ++i) dd_split(rec[i], recdd[2 * i], recdd[2 * i + 1]);
    SF_CK(h->d_ppdd.upload(recdd));
    std::vector<float> cdd(6 * (size_t)nshell);
    for (int a = 0; a < nshell; ++a) {
      dd_split(h->cx[a], cdd[2 * a], cdd[2 * a + 1]);
      dd_split(h->cy[a], cdd[2 * (nshell + a)], cdd[2 * (nshell + a) + 1]);
      dd_split(h->cz[a], cdd[2 * (2 * nshell + a)], cdd[2 * (2 * nshell + a) + 1]);
    }
    SF_CK(h->d_cdd.upload(cdd));
    std::vector<float> c32(h->cx.begin(), h->cx.end());
    SF_CK(h->d_cx32.upload(c32));
    c32.assign(h->cy.begin(), h->cy.end());
    SF_CK(h->d_cy32.upload(c32));
    c32.assign(h->cz.begin(), h->cz.end());
    SF_CK(h->d_cz32.upload(c32));
  }
  SF_CK(h->d_l.upload(h->l));
  SF_CK(h->d_nprim.upload(h->nprim));
  SF_CK(h->d_ao.upload(h->ao));
  SF_CK(h->d_atom.upload(h->atom));
  SF_CK(h->d_spoff.upload(h->spoff));
  SF_CK(h->d_cx.upload(h->cx));
  SF_CK(h->d_cy.upload(h->cy));
  SF_CK(h->d_cz.upload(h->cz));
  SF_CK(h->d_exps.upload(h->exps));
  {
    std::vector<float> sqa(h->nshell);
    for (int a = 0; a < h->nshell; ++a) {
      double m = 0.0;
      for (int i = h->spoff[a]; i < h->spoff[a + 1]; ++i) m = std::max(m, h->exps[i]);
      sqa[a] = (float)std::sqrt(m);
    }
    SF_CK(h->d_sqa.upload(sqa));
  }
  SF_CK(h->d_coefs.upload(h->coefs));
  const HostTables &T = host_tables();
  SF_CK(h->d_tab64.upload(T.t64));
  SF_CK(h->d_tab32.upload(T.t32v));
  SF_CK(h->d_tabdd.upload(T.tdd));
  SF_CK(h->d_Ddd.alloc(2 * (size_t)nao * nao));
  SF_CK(h->d_Jh.alloc((size_t)nao * nao));
  SF_CK(h->d_Kh.alloc((size_t)nao * nao));
  SF_CK(h->d_D32.alloc((size_t)nao * nao));
  SF_CK(h->d_err.alloc(4));
  SF_CK(cudaMemset(h->d_err.p, 0, 4 * sizeof(int)));
  int rc = upload_pairs(h);
  if (rc) return rc;
  {
    // the first kHiStreams side streams run at the device's highest priority:
    // in the mixed modes they carry the accurate tier's few, long-running
    // CTAs, which then start as soon as an SM frees up instead of queueing
    // behind the FP32 launches
    int lo = 0, hi = 0;
    SF_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int k = 0; k < sf_handle::kSideStreams; ++k) {
      SF_CK(cudaStreamCreateWithPriority(&h->side[k], cudaStreamNonBlocking, k < sf_handle::kHiStreams ? hi : lo));
      SF_CK(cudaEventCreateWithFlags(&h->join_ev[k], cudaEventDisableTiming));
    }
  }
  SF_CK(cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming));
  SF_CK(prepare_jk_f64());
  SF_CK(prepare_jk_f32());
  SF_CK(prepare_jk_dd());
  SF_CK(prepare_eri());
  SF_CK(prepare_eri_dd());
  SF_CK(prepare_md());
  SF_CK(prepare_md_tc());
  SF_CK(prepare_grad_f64());
  SF_CK(prepare_grad_f32());
  SF_CK(prepare_grad_dd());
  *out = guard.release();
  g_err.clear();
  return SF_OK;
}

int sf_build_shells(const sf_shell_desc *shells, int32_t nshell, sf_handle **out) {
  return sf_create(shells, nshell, out);
}

void sf_destroy(sf_handle *h) {
  if (!h) return;
  DeviceGuard g(h->device);
  for (cudaEvent_t e : h->ev) cudaEventDestroy(e);
  if (h->prof_t0) cudaEventDestroy(h->prof_t0);
  for (int k = 0; k < sf_handle::kSideStreams; ++k) {
    if (h->side[k]) cudaStreamDestroy(h->side[k]);
    if (h->join_ev[k]) cudaEventDestroy(h->join_ev[k]);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->cap_st) cudaStreamDestroy(h->cap_st);
  delete h;
}

int sf_set_profiling(sf_handle *h, int32_t on) {
  if (!h) return fail(SF_EINVAL, "sf_set_profiling: NULL handle");
  h->profiling = on < 0 ? 0 : on > 2 ? 2 : on;
  return SF_OK;
}

int32_t sf_slice_count(const sf_handle *h) {
  return h ? (int32_t)(h->plan.empty() ? h->slices.size() : h->plan.size()) : -1;
}

int sf_get_slice_info(sf_handle *h, int32_t idx, sf_slice_info *out) {
  if (!h || !out || idx < 0 || idx >= sf_slice_count(h)) return fail(SF_EINVAL, "sf_get_slice_info: bad index");
  DeviceGuard g(h->device);
  // a launch of the last call's plan (before any call: the slices themselves)
  sf_handle::Launch L{idx, 0, 0, 0, ClassWork{}};
  if (h->plan.empty()) {
    L.kind = h->slices[idx].prec;
    L.stream = (size_t)idx < h->slice_stream.size() ? h->slice_stream[idx] : -1;
    L.w = h->slices[idx].w;
  } else {
    L = h->plan[idx];
  }
  const auto &s = h->slices[L.slice];
  const ClassInfo &ci = kClassInfo[s.cls];
  out->cls = s.cls;
  out->precision = L.kind;
  out->la = ci.la; out->lb = ci.lb; out->lc = ci.lc; out->ld = ci.ld;
  out->quartets = s.quartets;
  out->prim_quartets = s.prims;
  out->flop_alg = s.flops;
  if (L.w.count) {   // classified on the device: its counts
    unsigned long long c[2] = {0, 0};
    SF_CK(cudaDeviceSynchronize());
    SF_CK(cudaMemcpy(&c[0], L.w.count, sizeof(c[0]), cudaMemcpyDeviceToHost));
    SF_CK(cudaMemcpy(&c[1], L.w.count + 2, sizeof(c[1]), cudaMemcpyDeviceToHost));
    const double nr = (ci.la + ci.lb + ci.lc + ci.ld) / 2 + 1;
    const double nabcd = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
    out->quartets = (int64_t)c[0];
    out->prim_quartets = (int64_t)c[1];
    out->flop_alg = (double)c[1] * nr * 4.0 * nabcd + 12.0 * nabcd * (double)c[0];
  }
  out->threads_per_quartet = kind_lanes(ci, L.kind, L.w.wide) * L.w.psplit * L.w.wsplit;
  out->ms = -1.0f;
  out->start_ms = -1.0f;
  out->stream = h->profiling == 2 ? -1 : L.stream;
  if (h->profiling && h->ev.size() >= 2 * (size_t)sf_slice_count(h)) {
    SF_CK(cudaEventSynchronize(h->ev[2 * idx + 1]));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, h->ev[2 * idx], h->ev[2 * idx + 1]) == cudaSuccess) out->ms = ms;
    else cudaGetLastError();
    if (h->prof_t0 && cudaEventElapsedTime(&ms, h->prof_t0, h->ev[2 * idx]) == cudaSuccess) out->start_ms = ms;
    else cudaGetLastError();
  }
  return SF_OK;
}

int sf_schwarz(sf_handle *h, double *q_out, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_schwarz: NULL handle");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  DBuf<double> dq;
  const int np = (int)h->pa.size();
  SF_CK(dq.alloc(np));
  for (int pc = 0; pc < kNumPairClass; ++pc)
    SF_CK(launch_schwarz(pc, h->kp, h->cstart[pc], h->cstart[pc + 1] - h->cstart[pc], dq.p, st));
  std::vector<double> q(np);
  SF_CK(cudaMemcpyAsync(q.data(), dq.p, np * sizeof(double), cudaMemcpyDeviceToHost, st));
  SF_CK(cudaStreamSynchronize(st));
  for (double v : q)
    if (!std::isfinite(v)) return fail(SF_EINVAL, "sf_schwarz: non-finite Schwarz bound (bad basis data?)");
  // sort every pair class by Q descending (stable)
  for (int pc = 0; pc < kNumPairClass; ++pc) {
    const int s0 = h->cstart[pc], s1 = h->cstart[pc + 1];
    std::vector<int> idx(s1 - s0);
    std::iota(idx.begin(), idx.end(), s0);
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return q[x] > q[y]; });
    std::vector<int> a(idx.size()), b(idx.size()), po(idx.size()), n(idx.size());
    std::vector<double> qq(idx.size());
    for (size_t k = 0; k < idx.size(); ++k) {
      a[k] = h->pa[idx[k]];
      b[k] = h->pb[idx[k]];
      po[k] = h->ppoff[idx[k]];
      n[k] = h->pnp[idx[k]];
      qq[k] = q[idx[k]];
    }
    std::copy(a.begin(), a.end(), h->pa.begin() + s0);
    std::copy(b.begin(), b.end(), h->pb.begin() + s0);
    std::copy(po.begin(), po.end(), h->ppoff.begin() + s0);
    std::copy(n.begin(), n.end(), h->pnp.begin() + s0);
    std::copy(qq.begin(), qq.end(), h->pq.begin() + s0);
  }
  int rc = upload_pairs(h);
  if (rc) return rc;
  h->have_schwarz = true;
  h->c_prec = -1;   // invalidate quartet lists
  if (q_out) {
    std::fill(q_out, q_out + (size_t)h->nshell * h->nshell, 0.0);
    for (int i = 0; i < np; ++i) {
      q_out[(size_t)h->pa[i] * h->nshell + h->pb[i]] = h->pq[i];
      q_out[(size_t)h->pb[i] * h->nshell + h->pa[i]] = h->pq[i];
    }
  }
  g_err.clear();
  return SF_OK;
}

int sf_set_density_screening(sf_handle *h, int32_t flags, double fock_fp32_cutoff, double grad_drop_cutoff,
                             double grad_fp32_cutoff) {
  if (!h) return fail(SF_EINVAL, "sf_set_density_screening: NULL handle");
  if (flags & ~(SF_DENS_FOCK | SF_DENS_GRAD)) return fail(SF_EINVAL, "sf_set_density_screening: unknown flag");
  if (std::isnan(fock_fp32_cutoff) || std::isnan(grad_drop_cutoff) || std::isnan(grad_fp32_cutoff))
    return fail(SF_EINVAL, "sf_set_density_screening: NaN cutoff");
  h->dens_flags = flags;
  h->dens_fock_acc = fock_fp32_cutoff;
  h->dens_grad_drop = grad_drop_cutoff;
  h->dens_grad_acc = grad_fp32_cutoff;
  return SF_OK;
}

int sf_set_launch_mode(sf_handle *h, int32_t mode, int32_t ctas_per_sm) {
  if (!h) return fail(SF_EINVAL, "sf_set_launch_mode: NULL handle");
  if (mode != SF_LAUNCH_STREAMS && mode != SF_LAUNCH_PERSISTENT) return fail(SF_EINVAL, "sf_set_launch_mode: bad mode");
  if (ctas_per_sm < 0 || ctas_per_sm > 64) return fail(SF_EINVAL, "sf_set_launch_mode: bad CTAs per SM");
  h->launch_mode = mode;
  h->persist_ctas_per_sm = ctas_per_sm;
  return SF_OK;
}

int sf_set_partition(sf_handle *h, int32_t part, int32_t nparts) {
  if (!h || nparts < 1 || part < 0 || part >= nparts) return fail(SF_EINVAL, "sf_set_partition: bad slice");
  h->part = part;
  h->nparts = nparts;
  return SF_OK;
}

int sf_fock_jk(sf_handle *h, const double *D, double *J, double *K, int32_t precision, double cutoff,
               double fp32_cutoff, sf_stats *stats, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_fock_jk: NULL handle");
  if (!D || !J || !K) return fail(SF_EINVAL, "sf_fock_jk: NULL matrix");
  if (precision < SF_PREC_FP64 || precision > SF_PREC_DF) return fail(SF_EINVAL, "sf_fock_jk: bad precision");
  if (!(cutoff >= 0.0) || !(fp32_cutoff >= 0.0)) return fail(SF_EINVAL, "sf_fock_jk: bad cutoff");
  if (!h->have_schwarz) return fail(SF_ESTATE, "sf_fock_jk: call sf_schwarz first");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  int rc = build_work(h, precision, cutoff, fp32_cutoff);
  if (rc) return rc;
  const int n = h->nao;
  const size_t nn = (size_t)n * n;
  SF_CK(cudaMemsetAsync(h->d_Jh.p, 0, nn * sizeof(double), st));
  SF_CK(cudaMemsetAsync(h->d_Kh.p, 0, nn * sizeof(double), st));
  int launches = 0;
  rc = convert_density(h, D, h->d_D32.p, st, &launches);
  if (rc) return rc;
  rc = run_call(h, false, D, h->d_D32.p, h->d_Jh.p, h->d_Kh.p, nullptr, cutoff, fp32_cutoff, st, h->profiling,
                &launches);
  if (rc) return rc;
  symmetrize_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(h->d_Jh.p, h->d_Kh.p, J, K, n);
  SF_CK(cudaGetLastError());
  ++launches;
  if (stats) {
    SF_CK(cudaStreamSynchronize(st));
    rc = plan_stats(h, stats);
    if (rc) return rc;
    stats->launches = launches;
  }
  return SF_OK;
}

struct sf_fock_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
};

int sf_fock_jk_graph_create(sf_handle *h, const double *D, double *J, double *K, int32_t precision, double cutoff,
                            double fp32_cutoff, int32_t node_priority, void *stream, sf_fock_graph **out) {
  if (!out) return fail(SF_EINVAL, "sf_fock_jk_graph_create: out is NULL");
  *out = nullptr;
  if (!h) return fail(SF_EINVAL, "sf_fock_jk_graph_create: NULL handle");
  // one ordinary build first: it cuts the quartet lists (and the persistent
  // tile tables), which allocates -- nothing allocates inside the capture
  int rc = sf_fock_jk(h, D, J, K, precision, cutoff, fp32_cutoff, nullptr, stream);
  if (rc) return rc;
  DeviceGuard g(h->device);
  SF_CK(cudaStreamSynchronize((cudaStream_t)stream));
  if (!h->cap_st) SF_CK(cudaStreamCreateWithFlags(&h->cap_st, cudaStreamNonBlocking));
  SF_CK(cudaStreamBeginCapture(h->cap_st, cudaStreamCaptureModeThreadLocal));
  rc = sf_fock_jk(h, D, J, K, precision, cutoff, fp32_cutoff, nullptr, h->cap_st);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(h->cap_st, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(SF_ECUDA, std::string("sf_fock_jk_graph_create: ") + cudaGetErrorString(e));
  auto *fg = new sf_fock_graph;
  fg->graph = graph;
  fg->device = h->device;
  const cudaError_t ei =
      cudaGraphInstantiateWithFlags(&fg->exec, graph, node_priority ? cudaGraphInstantiateFlagUseNodePriority : 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(graph);
    delete fg;
    return fail(SF_ECUDA, std::string("sf_fock_jk_graph_create: ") + cudaGetErrorString(ei));
  }
  *out = fg;
  return SF_OK;
}

int sf_graph_instantiate(void *graph, int32_t node_priority, sf_fock_graph **out) {
  if (!out) return fail(SF_EINVAL, "sf_graph_instantiate: out is NULL");
  *out = nullptr;
  if (!graph) return fail(SF_EINVAL, "sf_graph_instantiate: NULL graph");
  auto *fg = new sf_fock_graph;
  SF_CK(cudaGetDevice(&fg->device));
  const cudaError_t e = cudaGraphInstantiateWithFlags(&fg->exec, (cudaGraph_t)graph,
                                                      node_priority ? cudaGraphInstantiateFlagUseNodePriority : 0);
  if (e != cudaSuccess) {
    delete fg;
    return fail(SF_ECUDA, std::string("sf_graph_instantiate: ") + cudaGetErrorString(e));
  }
  *out = fg;   // fg->graph stays null: the caller owns the graph
  return SF_OK;
}

int sf_fock_graph_launch(sf_fock_graph *g, void *stream) {
  if (!g || !g->exec) return fail(SF_EINVAL, "sf_fock_graph_launch: NULL graph");
  DeviceGuard dg(g->device);
  SF_CK(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return SF_OK;
}

void sf_fock_graph_destroy(sf_fock_graph *g) {
  if (!g) return;
  DeviceGuard dg(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

int sf_autotune(sf_handle *h, const double *D, int32_t precision, double cutoff, double fp32_cutoff, int32_t reps,
                void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_autotune: NULL handle");
  if (!D) return fail(SF_EINVAL, "sf_autotune: NULL density");
  if (precision < SF_PREC_FP64 || precision > SF_PREC_DF) return fail(SF_EINVAL, "sf_autotune: bad precision");
  if (!(cutoff >= 0.0) || !(fp32_cutoff >= 0.0)) return fail(SF_EINVAL, "sf_autotune: bad cutoff");
  if (reps < 1 || reps > 1000) return fail(SF_EINVAL, "sf_autotune: reps must be in 1..1000");
  if (!h->have_schwarz) return fail(SF_ESTATE, "sf_autotune: call sf_schwarz first");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  int rc = build_work(h, precision, cutoff, fp32_cutoff);
  if (rc) return rc;
  rc = convert_density(h, D, h->d_D32.p, st, nullptr);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  SF_CK(cudaEventCreate(&e0));
  SF_CK(cudaEventCreate(&e1));
  // every candidate adds into the handle's scratch Jh/Kh, which the next
  // Fock build clears; the caller's matrices are not touched
  auto time_split = [&](const sf_handle::Slice &sl, int S, float *ms) -> cudaError_t {
    const ClassInfo &ci = kClassInfo[sl.cls];
    const int pmax = 32 / kind_lanes(ci, sl.prec, sl.w.wide);
    ClassWork w = sl.w;
    w.psplit = std::min(S, pmax);
    w.wsplit = S / w.psplit;
    auto launch = [&]() { return launch_slice(h, sl, w, D, h->d_D32.p, h->d_Jh.p, h->d_Kh.p, st); };
    cudaError_t e = launch();   // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    *ms /= (float)reps;
    return e;
  };
  // whole-build time of the current lists, launches concurrent as in a build
  auto time_build = [&](float *ms) -> int {
    int r2 = build_work(h, precision, cutoff, fp32_cutoff);
    if (r2) return r2;
    r2 = run_call(h, false, D, h->d_D32.p, h->d_Jh.p, h->d_Kh.p, nullptr, cutoff, fp32_cutoff, st, 0,
                  nullptr);   // warm-up
    if (r2) return r2;
    SF_CK(cudaEventRecord(e0, st));
    for (int r = 0; r < reps; ++r) {
      r2 = run_call(h, false, D, h->d_D32.p, h->d_Jh.p, h->d_Kh.p, nullptr, cutoff, fp32_cutoff, st, 0, nullptr);
      if (r2) return r2;
    }
    SF_CK(cudaEventRecord(e1, st));
    SF_CK(cudaEventSynchronize(e1));
    SF_CK(cudaEventElapsedTime(ms, e0, e1));
    *ms /= (float)reps;
    return SF_OK;
  };
  auto drop_entries = [&]() {
    std::vector<sf_tune_entry> keep;
    const int kinds[2] = {(precision == SF_PREC_MIXED_DF || precision == SF_PREC_DF) ? 2 : 0, 1};
    for (const auto &x : h->tune) {
      bool mine = x.cls < 0 ? x.precision == precision : false;
      if (x.cls >= 0)
        for (int k : kinds)
          if (x.precision == k &&
              ((k == 1 && precision != SF_PREC_FP64 && precision != SF_PREC_DF) ||
               (k != 1 && precision != SF_PREC_FP32)))
            mine = true;
      if (!mine) keep.push_back(x);
    }
    h->tune.swap(keep);
  };
  // 1. the launch-fill target of this mode, by whole-build time (per-launch
  // splits of this mode cleared first)
  drop_entries();
  h->fill_acc_x4[precision] = -1;
  int best_fill = h->fill_x4[precision];
  float best_ms = 1e30f;
  for (int f : {0, 1, 4, 16}) {
    h->fill_x4[precision] = f;
    h->c_prec = -1;
    float ms = 0.f;
    rc = time_build(&ms);
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    if (ms < best_ms) {
      best_ms = ms;
      best_fill = f;
    }
  }
  h->fill_x4[precision] = best_fill;
  // mixed modes: the accurate tier's few quartets fill the GPU at another
  // target than the FP32 tier's many; searched with the FP32 tier's fixed
  int best_acc = -1;
  if (precision == SF_PREC_MIXED || precision == SF_PREC_MIXED_DF) {
    for (int f : {0, 1, 4, 16, 64}) {
      if (f == best_fill) continue;   // already timed: the mode's target for both tiers
      h->fill_acc_x4[precision] = f;
      h->c_prec = -1;
      float ms = 0.f;
      rc = time_build(&ms);
      if (rc) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best_acc = f;
      }
    }
    h->fill_acc_x4[precision] = best_acc;
  }
  h->c_prec = -1;
  rc = build_work(h, precision, cutoff, fp32_cutoff);
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  // 2. per-launch splits, each launch timed alone
  int tuned = 0;
  for (auto &sl : h->slices) {
    const ClassInfo &ci = kClassInfo[sl.cls];
    const int pmax = 32 / kind_lanes(ci, sl.prec, sl.w.wide);
    const int S0 = sl.w.psplit * sl.w.wsplit;
    float ms0 = 0.f;
    cudaError_t e = time_split(sl, S0, &ms0);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail(SF_ECUDA, std::string("sf_autotune: ") + cudaGetErrorString(e));
    }
    int best = S0;
    float bms = ms0;
    for (int S : {S0 / 4, S0 / 2, S0 * 2, S0 * 4}) {
      if (S < 1 || S > pmax * kMaxWsplit || S > 2 * std::max<int64_t>(sl.cost_hi, 1)) continue;
      float ms = 0.f;
      e = time_split(sl, S, &ms);
      if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return fail(SF_ECUDA, std::string("sf_autotune: ") + cudaGetErrorString(e));
      }
      if (ms < 0.97f * bms) {   // keep the heuristic unless a split is clearly faster
        bms = ms;
        best = S;
      }
    }
    sl.w.psplit = std::min(best, pmax);
    sl.w.wsplit = best / sl.w.psplit;
    sf_tune_entry te{sl.cls, sl.prec, sl.cost_hi, best, ms0, bms};
    bool found = false;
    for (auto &x : h->tune)
      if (x.cls == te.cls && x.precision == te.precision && x.cost == te.cost) {
        x = te;
        found = true;
      }
    if (!found) h->tune.push_back(te);
    ++tuned;
  }
  // 3. keep the per-launch splits (and the stream assignment by their
  // measured times) only if the whole build got faster
  h->c_prec = -1;
  float tuned_ms = 0.f;
  rc = time_build(&tuned_ms);
  if (rc) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  if (tuned_ms > best_ms) {
    drop_entries();
    tuned = 0;
  }
  h->tune.push_back(sf_tune_entry{-1, precision, 0, best_fill, best_ms, std::min(best_ms, tuned_ms)});
  if (best_acc >= 0)
    h->tune.push_back(sf_tune_entry{-2, precision, 0, best_acc, best_ms, std::min(best_ms, tuned_ms)});
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->c_prec = -1;   // the next build re-cuts the lists and assigns streams by the measured times
  return tuned;
}

int32_t sf_tuning_count(const sf_handle *h) { return h ? (int32_t)h->tune.size() : -1; }

int sf_get_tuning(const sf_handle *h, int32_t idx, sf_tune_entry *out) {
  if (!h || !out || idx < 0 || idx >= (int32_t)h->tune.size()) return fail(SF_EINVAL, "sf_get_tuning: bad arguments");
  *out = h->tune[idx];
  return SF_OK;
}

int sf_set_tuning(sf_handle *h, const sf_tune_entry *entries, int32_t n) {
  if (!h || n < 0 || (n > 0 && !entries)) return fail(SF_EINVAL, "sf_set_tuning: bad arguments");
  for (int32_t i = 0; i < n; ++i) {
    const sf_tune_entry &e = entries[i];
    const bool fill_entry = (e.cls == -1 || e.cls == -2) && e.precision >= 0 && e.precision <= SF_PREC_DF &&
                            e.split >= 0 && e.split <= 64;
    if (fill_entry) continue;
    if (e.cls < 0 || e.cls >= kNumClass || e.precision < 0 || e.precision > 2 || e.split < 1 ||
        e.split > 32 * kMaxWsplit || (e.split & (e.split - 1)))
      return fail(SF_EINVAL, "sf_set_tuning: bad entry " + std::to_string(i));
  }
  h->tune.assign(entries, entries + n);
  for (int m = 0; m <= SF_PREC_DF; ++m) {
    h->fill_x4[m] = 4;
    h->fill_acc_x4[m] = -1;
  }
  for (const auto &e : h->tune) {
    if (e.cls == -1) h->fill_x4[e.precision] = e.split;
    if (e.cls == -2) h->fill_acc_x4[e.precision] = e.split;
  }
  h->c_prec = -1;   // rebuild the launch list with the new splits
  return SF_OK;
}

int sf_fock_jk_noalloc(sf_handle *h, const double *D, double *J, double *K, int32_t precision, double cutoff,
                       double fp32_cutoff, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_fock_jk_noalloc: NULL handle");
  if (!D || !J || !K) return fail(SF_EINVAL, "sf_fock_jk_noalloc: NULL matrix");
  if (precision == SF_PREC_MIXED_DF || precision == SF_PREC_DF)
    return fail(SF_EUNSUPPORTED, "sf_fock_jk_noalloc: the double-float modes need the handle's scratch (sf_fock_jk)");
  if (precision < SF_PREC_FP64 || precision > SF_PREC_MIXED) return fail(SF_EINVAL, "sf_fock_jk_noalloc: bad precision");
  if (h->nao > SF_NOALLOC_MAX_NAO)
    return fail(SF_EINVAL, "sf_fock_jk_noalloc: nao = " + std::to_string(h->nao) +
                               " exceeds the static scratch limit SF_NOALLOC_MAX_NAO = " +
                               std::to_string(SF_NOALLOC_MAX_NAO) + "; use sf_fock_jk");
  if (!h->have_schwarz) return fail(SF_ESTATE, "sf_fock_jk_noalloc: call sf_schwarz first");
  if (!(h->c_prec == precision && h->c_cut == cutoff && h->c_cut32 == fp32_cutoff && h->c_part == h->part &&
        h->c_nparts == h->nparts))
    return fail(SF_ESTATE,
                "sf_fock_jk_noalloc: the quartet lists for this precision and these cutoffs are not built; "
                "call sf_fock_jk once with the same arguments first (that call allocates)");
  if (h->device < 0 || h->device >= 128) return fail(SF_EINVAL, "sf_fock_jk_noalloc: device index out of range");
  if (h->launch_mode == SF_LAUNCH_PERSISTENT && h->profiling == 0 && h->persist_version != h->lists_version)
    return fail(SF_ESTATE,
                "sf_fock_jk_noalloc: the persistent launch tables are not built; call sf_fock_jk once in this launch "
                "mode first (that call allocates)");
  DeviceGuard g(h->device);
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_dev[h->device]) {
      void *p = nullptr;
      SF_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      g_noalloc_dev[h->device] = static_cast<double *>(p);
    }
    scratch = g_noalloc_dev[h->device];
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int n = h->nao;
  const size_t nn = (size_t)n * n;
  double *Jh = scratch, *Kh = scratch + nn;
  float *D32 = reinterpret_cast<float *>(scratch + 2 * nn);
  SF_CK(cudaMemsetAsync(scratch, 0, 2 * nn * sizeof(double), st));
  bool need32 = false;
  for (const auto &s : h->slices) need32 |= s.prec == 1;
  if (need32) {
    to_float_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(D, D32, (int64_t)nn);
    SF_CK(cudaGetLastError());
  }
  int rc = run_call(h, false, D, D32, Jh, Kh, nullptr, cutoff, fp32_cutoff, st, 0, nullptr);
  if (rc) return rc;
  symmetrize_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(Jh, Kh, J, K, n);
  SF_CK(cudaGetLastError());
  return SF_OK;
}

int sf_grad_jk(sf_handle *h, const double *D, double *grad, int32_t precision, double cutoff, double fp32_cutoff,
               void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_grad_jk: NULL handle");
  if (!D || !grad) return fail(SF_EINVAL, "sf_grad_jk: NULL pointer");
  if (precision < SF_PREC_FP64 || precision > SF_PREC_DF) return fail(SF_EINVAL, "sf_grad_jk: bad precision");
  if (!(cutoff >= 0.0) || !(fp32_cutoff >= 0.0)) return fail(SF_EINVAL, "sf_grad_jk: bad cutoff");
  if (!h->have_schwarz) return fail(SF_ESTATE, "sf_grad_jk: call sf_schwarz first");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  int rc = build_work(h, precision, cutoff, fp32_cutoff);
  if (rc) return rc;
  rc = convert_density(h, D, h->d_D32.p, st, nullptr);
  if (rc) return rc;
  // per-launch events in the profiling modes (serialised in mode 2), read by sf_get_slice_info
  return run_call(h, true, D, h->d_D32.p, nullptr, nullptr, grad, cutoff, fp32_cutoff, st, h->profiling, nullptr);
}

int sf_grad_stats(sf_handle *h, sf_stats *stats, void *stream) {
  if (!h || !stats) return fail(SF_EINVAL, "sf_grad_stats: NULL argument");
  if (!h->plan_grad || h->plan.empty()) return fail(SF_ESTATE, "sf_grad_stats: no gradient call on this handle yet");
  DeviceGuard g(h->device);
  SF_CK(cudaStreamSynchronize((cudaStream_t)stream));
  const int rc = plan_stats(h, stats, true);
  if (rc) return rc;
  stats->launches = (int32_t)h->plan.size();
  return SF_OK;
}

int sf_grad_one_electron(sf_handle *h, const double *atom_xyz, const double *charges, int32_t natom, const double *D,
                         const double *W, double *grad, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_grad_one_electron: NULL handle");
  if (!D || !W || !grad || natom < 0 || (natom > 0 && (!atom_xyz || !charges)))
    return fail(SF_EINVAL, "sf_grad_one_electron: bad arguments");
  if (natom < h->natom)
    return fail(SF_EINVAL, "sf_grad_one_electron: the shells reference atom " + std::to_string(h->natom - 1) +
                               " but only " + std::to_string(natom) + " nuclei were given");
  DeviceGuard g(h->device);
  OneParams P;
  P.sh = h->kp.sh;
  P.exps = h->d_exps.p;
  P.coefs = h->d_coefs.p;
  P.poff = h->d_spoff.p;
  P.nshell = h->nshell;
  P.nao = h->nao;
  P.atom_xyz = atom_xyz;
  P.charges = charges;
  P.natom = natom;
  P.S = P.T = P.V = nullptr;
  P.tab64 = h->kp.tab64;
  P.asym = h->kp.asym;
  SF_CK(launch_one_electron_grad(P, D, W, grad, (cudaStream_t)stream));
  return SF_OK;
}

int sf_eri_batch(sf_handle *h, const int32_t *quartets, int64_t nq, int32_t precision, double *out,
                 const int64_t *out_offsets, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_eri_batch: NULL handle");
  if (nq < 0 || (nq > 0 && (!quartets || !out || !out_offsets))) return fail(SF_EINVAL, "sf_eri_batch: bad arguments");
  if (precision != SF_PREC_FP64 && precision != SF_PREC_FP32 && precision != SF_PREC_DF)
    return fail(SF_EINVAL, "sf_eri_batch: bad precision");
  if (nq == 0) return SF_OK;
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<int32_t> hq((size_t)nq * 4);
  std::vector<int64_t> hoff(nq);
  SF_CK(cudaMemcpyAsync(hq.data(), quartets, hq.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  SF_CK(cudaMemcpyAsync(hoff.data(), out_offsets, hoff.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  SF_CK(cudaStreamSynchronize(st));
  sf_eri_plan pl;
  int rc = build_eri_plan(h, hq.data(), nq, hoff.data(), &pl);
  if (rc) return rc;
  rc = run_eri_plan(&pl, precision, out, st);
  if (rc) return rc;
  SF_CK(cudaStreamSynchronize(st));   // the plan's device lists are freed on return
  return SF_OK;
}

int sf_eri_plan_create(sf_handle *h, const int32_t *quartets, int64_t nq, sf_eri_plan **out) {
  if (!out) return fail(SF_EINVAL, "sf_eri_plan_create: out is NULL");
  *out = nullptr;
  if (!h) return fail(SF_EINVAL, "sf_eri_plan_create: NULL handle");
  if (nq < 0 || (nq > 0 && !quartets)) return fail(SF_EINVAL, "sf_eri_plan_create: bad arguments");
  DeviceGuard g(h->device);
  std::unique_ptr<sf_eri_plan> pl(new sf_eri_plan);
  int rc = build_eri_plan(h, quartets, nq, nullptr, pl.get());
  if (rc) return rc;
  *out = pl.release();
  return SF_OK;
}

int sf_eri_plan_info(const sf_eri_plan *pl, int64_t *outputs, int64_t *prim_quartets, double *flop_alg) {
  if (!pl) return fail(SF_EINVAL, "sf_eri_plan_info: NULL plan");
  if (outputs) *outputs = pl->total;
  if (prim_quartets) *prim_quartets = pl->prims;
  if (flop_alg) *flop_alg = pl->flops;
  return SF_OK;
}

int sf_eri_plan_offsets(const sf_eri_plan *pl, int64_t *offsets) {
  if (!pl || (pl->nq > 0 && !offsets)) return fail(SF_EINVAL, "sf_eri_plan_offsets: bad arguments");
  if (pl->nq > 0) std::memcpy(offsets, pl->offsets.data(), (size_t)pl->nq * sizeof(int64_t));
  return SF_OK;
}

int sf_eri_plan_run(sf_eri_plan *pl, int32_t precision, double *out, void *stream) {
  if (!pl) return fail(SF_EINVAL, "sf_eri_plan_run: NULL plan");
  if (precision != SF_PREC_FP64 && precision != SF_PREC_FP32 && precision != SF_PREC_DF)
    return fail(SF_EINVAL, "sf_eri_plan_run: bad precision");
  if (pl->nq > 0 && !out) return fail(SF_EINVAL, "sf_eri_plan_run: NULL output");
  DeviceGuard g(pl->h->device);
  return run_eri_plan(pl, precision, out, (cudaStream_t)stream);
}

int sf_eri_plan_run_md(sf_eri_plan *pl, int32_t precision, double *out, void *stream) {
  if (!pl) return fail(SF_EINVAL, "sf_eri_plan_run_md: NULL plan");
  if (precision != SF_PREC_FP64 && precision != SF_PREC_FP32)
    return fail(SF_EUNSUPPORTED, "sf_eri_plan_run_md: the MD engine runs in FP64 or FP32 (tensor cores)");
  if (pl->nq > 0 && !out) return fail(SF_EINVAL, "sf_eri_plan_run_md: NULL output");
  DeviceGuard g(pl->h->device);
  sf_handle *h = pl->h;
  cudaStream_t st = (cudaStream_t)stream;
  const auto &segs = pl->segs[0];
  if (segs.empty()) return SF_OK;
  const bool tc = precision == SF_PREC_FP32;
  if (tc) SF_CK(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), st));
  int rc = fan_out_list(h, st, pl->seg_stream[0], [&](size_t k, cudaStream_t ss) {
    const sf_eri_plan::Seg &sg = segs[k];
    EriWork w{pl->d_pab.p + sg.off, pl->d_pcd.p + sg.off, pl->d_fl.p + sg.off, pl->d_off.p + sg.off,
              pl->d_str.p + 4 * sg.off, sg.n, out, 1};
    return tc ? launch_md_tc(sg.cls, h->kp, w, h->nsm, ss) : launch_md_eri(sg.cls, h->kp, w, ss);
  });
  if (rc || !tc) return rc;
  // the tensor-core kernels bound every wait on their MMAs and flag a timeout
  int flag = 0;
  SF_CK(cudaMemcpyAsync(&flag, h->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  SF_CK(cudaStreamSynchronize(st));
  if (flag) return fail(SF_ECUDA, "sf_eri_plan_run_md: a tensor-core MMA wait timed out");
  return SF_OK;
}

int sf_debug_tc_wait_limit(int32_t iterations) {
  if (iterations < -1) return fail(SF_EINVAL, "sf_debug_tc_wait_limit: limit below -1");
  md_tc_set_wait_limit(iterations);
  return SF_OK;
}

void sf_eri_plan_destroy(sf_eri_plan *pl) {
  if (!pl) return;
  DeviceGuard g(pl->h->device);
  cudaDeviceSynchronize();   // runs in flight still read the plan's lists
  delete pl;
}

int sf_one_electron(sf_handle *h, const double *atom_xyz, const double *charges, int32_t natom, double *S, double *T,
                    double *V, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_one_electron: NULL handle");
  if (V && (natom < 0 || (natom > 0 && (!atom_xyz || !charges)))) return fail(SF_EINVAL, "sf_one_electron: bad atoms");
  DeviceGuard g(h->device);
  OneParams P;
  P.sh = h->kp.sh;
  P.exps = h->d_exps.p;
  P.coefs = h->d_coefs.p;
  P.poff = h->d_spoff.p;
  P.nshell = h->nshell;
  P.nao = h->nao;
  P.atom_xyz = atom_xyz;
  P.charges = charges;
  P.natom = V ? natom : 0;
  P.S = S;
  P.T = T;
  P.V = V;
  P.tab64 = h->kp.tab64;
  P.asym = h->kp.asym;
  SF_CK(launch_one_electron(P, (cudaStream_t)stream));
  return SF_OK;
}

int sf_rys_roots_host(int32_t n, double x, int32_t fp32, double *u, double *w) {
  if (n < 1 || n > kMaxRoots || !(x >= 0.0) || !u || !w) return fail(SF_EINVAL, "sf_rys_roots_host: bad arguments");
  const HostTables &T = host_tables();
  rys_eval_host(T.t64.data(), T.t32.data(), T.asym, n, x, fp32, u, w);
  return SF_OK;
}

}  // extern "C"
