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
  std::vector<float> t32;
  RysAsym asym;
};

const HostTables &host_tables() {
  static HostTables T;
  static std::once_flag once;
  std::call_once(once, [] {
    T.t64.assign(rys_tab_size(kTabDeg64), 0.0);
    T.t32.assign(rys_tab_size(kTabDeg32), 0.0f);
    std::memset(&T.asym, 0, sizeof(T.asym));
    rys_build_tables(T.t64.data(), T.t32.data(), &T.asym);
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

}  // namespace

struct sf_handle {
  int device = 0;
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
  };
  int profiling = 0;              // 1: per-slice events; 2: also serialise launches
  std::vector<cudaEvent_t> ev;   // 2 per slice while profiling
  // side streams: the class launches of one build are independent (they only
  // add into Jh/Kh with atomics), so they are spread over kSideStreams
  // streams forked from and joined back into the caller's stream
  static constexpr int kSideStreams = 8;
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
  KParams kp;
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
  k.nao = h->nao;
  k.natom = h->natom;
  k.err = h->d_err.p;
}

int upload_pairs(sf_handle *h) {
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

// Quartet lists of every (class, precision) launch for the given cutoffs.
// Each list holds the surviving canonical quartets (bra i, ket j) of one
// class, ordered by decreasing primitive cost K_ab K_cd (then K_ab), stable,
// so consecutive quartets -- the lanes and groups of one warp -- run the same
// number of primitive iterations; inside a cost bucket the (i, j) order of the
// Schwarz-sorted pair lists is kept.  A partition (part, nparts) keeps every
// nparts-th quartet of each sorted list, which balances cost across parts.
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
    int psplit;
  };
  std::vector<Pending> pend;
  h->st_q[0] = h->st_q[1] = h->st_pq[0] = h->st_pq[1] = 0;
  h->st_f[0] = h->st_f[1] = 0.0;
  h->st_total = 0;
  constexpr int KB = kMaxPrim * kMaxPrim + 1;   // primitive pairs per shell pair <= 256
  std::vector<int64_t> hist((size_t)KB * KB);
  for (int cls = 0; cls < kNumClass; ++cls) {
    const ClassInfo &ci = kClassInfo[cls];
    const int X = pair_class_of(ci.la, ci.lb), Y = pair_class_of(ci.lc, ci.ld);
    const int x0 = h->cstart[X], y0 = h->cstart[Y];
    const int nX = h->cstart[X + 1] - x0, nY = h->cstart[Y + 1] - y0;
    const int same = X == Y;
    h->st_total += same ? (int64_t)nX * (nX + 1) / 2 : (int64_t)nX * nY;
    if (nX == 0 || nY == 0) continue;
    const double *qx = h->pq.data() + x0, *qy = h->pq.data() + y0;
    std::vector<int64_t> m(nX), m64(nX);
    for (int i = 0; i < nX; ++i) {
      int64_t mi = count_pass(qy, nY, qx[i], cut);
      if (same) mi = std::min<int64_t>(mi, i + 1);
      int64_t m6;
      if (prec == SF_PREC_FP64) m6 = mi;
      else if (prec == SF_PREC_FP32) m6 = 0;
      else m6 = std::min<int64_t>(mi, count_pass(qy, nY, qx[i], std::max(cut32, cut)));
      m[i] = mi;
      m64[i] = m6;
    }
    const int nr = (ci.la + ci.lb + ci.lc + ci.ld) / 2 + 1;
    const double nabcd = (double)ncart(ci.la) * ncart(ci.lb) * ncart(ci.lc) * ncart(ci.ld);
    for (int pr = 0; pr < 2; ++pr) {
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
      p.psplit = 1;
      p.cls = cls;
      p.prec = pr;
      p.off = all.size();
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
      h->st_q[pr] += p.n;
      h->st_pq[pr] += p.prims;
      h->st_f[pr] += p.flops;
      // split the cost-sorted list into launches with P primitive sub-groups
      // per quartet: heavy quartets (many primitive quartets) get more lanes
      const int T = pr == 0 ? ci.t64 : ci.t32;
      const int pmax = 32 / T;
      auto psplit = [&](int64_t cost) {
        if (pmax > 1 && cost >= 4 * pmax) return pmax;
        if (pmax > 8 && cost >= 32) return 8;
        return 1;
      };
      int64_t q0 = 0;
      while (q0 < p.n) {
        const auto cost_of = [&](int64_t q) {
          return (int64_t)h->pnp[x0 + lst[q].x] * h->pnp[y0 + lst[q].y];
        };
        const int P = psplit(cost_of(q0));
        int64_t q1 = q0 + 1;
        while (q1 < p.n && psplit(cost_of(q1)) == P) ++q1;
        Pending seg = p;
        seg.off = all.size() + q0;
        seg.n = q1 - q0;
        int64_t sp = 0;
        for (int64_t q = q0; q < q1; ++q) sp += cost_of(q);
        seg.prims = sp;
        seg.flops = (double)sp * nr * 4.0 * nabcd + 12.0 * nabcd * (double)seg.n;
        seg.psplit = P;
        pend.push_back(seg);
        q0 = q1;
      }
      all.insert(all.end(), lst.begin(), lst.end());
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
    h->slices.push_back({p.cls, p.prec, w, p.n, p.prims, p.flops});
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
      cost[k] = (double)sl.prims * (nr * (nc + 30.0) + 40.0) * (sl.prec == 0 ? 16.0 : 1.0);
    }
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<sf_handle::Slice> sorted;
    for (int k : order) sorted.push_back(h->slices[k]);
    h->slices.swap(sorted);
    std::sort(cost.begin(), cost.end(), std::greater<double>());
    double load[sf_handle::kSideStreams] = {0};
    h->slice_stream.assign(h->slices.size(), 0);
    for (size_t k = 0; k < h->slices.size(); ++k) {
      int best = 0;
      for (int j = 1; j < sf_handle::kSideStreams; ++j)
        if (load[j] < load[best]) best = j;
      h->slice_stream[k] = best;
      load[best] += cost[k];
    }
  }
  h->c_prec = prec;
  h->c_cut = cut;
  h->c_cut32 = cut32;
  h->c_part = h->part;
  h->c_nparts = h->nparts;
  return SF_OK;
}

// Run fn(k, stream) for every slice k on its side stream (forked from st,
// joined back into st).
template <typename F>
int fan_out(sf_handle *h, cudaStream_t st, F &&fn) {
  SF_CK(cudaEventRecord(h->fork_ev, st));
  bool used[sf_handle::kSideStreams] = {false};
  for (size_t k = 0; k < h->slices.size(); ++k) used[h->slice_stream[k]] = true;
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) SF_CK(cudaStreamWaitEvent(h->side[j], h->fork_ev, 0));
  for (size_t k = 0; k < h->slices.size(); ++k) SF_CK(fn(k, h->side[h->slice_stream[k]]));
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) {
      SF_CK(cudaEventRecord(h->join_ev[j], h->side[j]));
      SF_CK(cudaStreamWaitEvent(st, h->join_ev[j], 0));
    }
  return SF_OK;
}

// Launch every slice of the current quartet lists on the side streams
// (forked from st, joined back into st).  Events of the profiling mode
// bracket each launch on its own stream.
int launch_slices(sf_handle *h, const double *D, const float *D32, double *Jh, double *Kh, cudaStream_t st,
                  int profiling, int *launches) {
  if (profiling == 2) {   // serialised on the caller's stream
    for (size_t k = 0; k < h->slices.size(); ++k) {
      const auto &s = h->slices[k];
      SF_CK(cudaEventRecord(h->ev[2 * k], st));
      if (s.prec == 0) SF_CK(launch_jk_f64(s.cls, h->kp, s.w, D, Jh, Kh, st));
      else SF_CK(launch_jk_f32(s.cls, h->kp, s.w, D32, Jh, Kh, st));
      SF_CK(cudaEventRecord(h->ev[2 * k + 1], st));
      if (launches) ++*launches;
    }
    return SF_OK;
  }
  SF_CK(cudaEventRecord(h->fork_ev, st));
  bool used[sf_handle::kSideStreams] = {false};
  for (size_t k = 0; k < h->slices.size(); ++k) used[h->slice_stream[k]] = true;
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) SF_CK(cudaStreamWaitEvent(h->side[j], h->fork_ev, 0));
  for (size_t k = 0; k < h->slices.size(); ++k) {
    const auto &s = h->slices[k];
    cudaStream_t ss = h->side[h->slice_stream[k]];
    if (profiling) SF_CK(cudaEventRecord(h->ev[2 * k], ss));
    if (s.prec == 0) SF_CK(launch_jk_f64(s.cls, h->kp, s.w, D, Jh, Kh, ss));
    else SF_CK(launch_jk_f32(s.cls, h->kp, s.w, D32, Jh, Kh, ss));
    if (profiling) SF_CK(cudaEventRecord(h->ev[2 * k + 1], ss));
    if (launches) ++*launches;
  }
  for (int j = 0; j < sf_handle::kSideStreams; ++j)
    if (used[j]) {
      SF_CK(cudaEventRecord(h->join_ev[j], h->side[j]));
      SF_CK(cudaStreamWaitEvent(st, h->join_ev[j], 0));
    }
  return SF_OK;
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
  SF_CK(h->d_coefs.upload(h->coefs));
  const HostTables &T = host_tables();
  SF_CK(h->d_tab64.upload(T.t64));
  SF_CK(h->d_tab32.upload(T.t32));
  SF_CK(h->d_Jh.alloc((size_t)nao * nao));
  SF_CK(h->d_Kh.alloc((size_t)nao * nao));
  SF_CK(h->d_D32.alloc((size_t)nao * nao));
  SF_CK(h->d_err.alloc(4));
  SF_CK(cudaMemset(h->d_err.p, 0, 4 * sizeof(int)));
  int rc = upload_pairs(h);
  if (rc) return rc;
  for (int k = 0; k < sf_handle::kSideStreams; ++k) {
    SF_CK(cudaStreamCreateWithFlags(&h->side[k], cudaStreamNonBlocking));
    SF_CK(cudaEventCreateWithFlags(&h->join_ev[k], cudaEventDisableTiming));
  }
  SF_CK(cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming));
  SF_CK(prepare_jk_f64());
  SF_CK(prepare_jk_f32());
  SF_CK(prepare_eri());
  SF_CK(prepare_grad_f64());
  SF_CK(prepare_grad_f32());
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
  for (int k = 0; k < sf_handle::kSideStreams; ++k) {
    if (h->side[k]) cudaStreamDestroy(h->side[k]);
    if (h->join_ev[k]) cudaEventDestroy(h->join_ev[k]);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  delete h;
}

int sf_set_profiling(sf_handle *h, int32_t on) {
  if (!h) return fail(SF_EINVAL, "sf_set_profiling: NULL handle");
  h->profiling = on < 0 ? 0 : on > 2 ? 2 : on;
  return SF_OK;
}

int32_t sf_slice_count(const sf_handle *h) { return h ? (int32_t)h->slices.size() : -1; }

int sf_get_slice_info(sf_handle *h, int32_t idx, sf_slice_info *out) {
  if (!h || !out || idx < 0 || idx >= (int32_t)h->slices.size()) return fail(SF_EINVAL, "sf_get_slice_info: bad index");
  DeviceGuard g(h->device);
  const auto &s = h->slices[idx];
  const ClassInfo &ci = kClassInfo[s.cls];
  out->cls = s.cls;
  out->precision = s.prec == 0 ? SF_PREC_FP64 : SF_PREC_FP32;
  out->la = ci.la; out->lb = ci.lb; out->lc = ci.lc; out->ld = ci.ld;
  out->quartets = s.quartets;
  out->prim_quartets = s.prims;
  out->flop_alg = s.flops;
  out->threads_per_quartet = (s.prec == 0 ? ci.t64 : ci.t32) * s.w.psplit;
  out->ms = -1.0f;
  if (h->profiling && h->ev.size() >= 2 * h->slices.size()) {
    SF_CK(cudaEventSynchronize(h->ev[2 * idx + 1]));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, h->ev[2 * idx], h->ev[2 * idx + 1]) == cudaSuccess) out->ms = ms;
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
  if (precision < SF_PREC_FP64 || precision > SF_PREC_MIXED) return fail(SF_EINVAL, "sf_fock_jk: bad precision");
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
  bool need32 = false;
  for (const auto &s : h->slices) need32 |= s.prec == 1;
  if (need32) {
    to_float_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(D, h->d_D32.p, (int64_t)nn);
    SF_CK(cudaGetLastError());
    ++launches;
  }
  if (h->profiling && h->ev.size() < 2 * h->slices.size()) {
    while (h->ev.size() < 2 * h->slices.size()) {
      cudaEvent_t e;
      SF_CK(cudaEventCreate(&e));
      h->ev.push_back(e);
    }
  }
  rc = launch_slices(h, D, h->d_D32.p, h->d_Jh.p, h->d_Kh.p, st, h->profiling, &launches);
  if (rc) return rc;
  symmetrize_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(h->d_Jh.p, h->d_Kh.p, J, K, n);
  SF_CK(cudaGetLastError());
  ++launches;
  if (stats) {
    stats->quartets_fp64 = h->st_q[0];
    stats->quartets_fp32 = h->st_q[1];
    stats->quartets_total = h->st_total;
    stats->prim_quartets_fp64 = h->st_pq[0];
    stats->prim_quartets_fp32 = h->st_pq[1];
    stats->flop_alg_fp64 = h->st_f[0];
    stats->flop_alg_fp32 = h->st_f[1];
    stats->launches = launches;
    stats->reserved = 0;
    SF_CK(cudaStreamSynchronize(st));
  }
  return SF_OK;
}

int sf_fock_jk_noalloc(sf_handle *h, const double *D, double *J, double *K, int32_t precision, double cutoff,
                       double fp32_cutoff, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_fock_jk_noalloc: NULL handle");
  if (!D || !J || !K) return fail(SF_EINVAL, "sf_fock_jk_noalloc: NULL matrix");
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
  DeviceGuard g(h->device);
  if (h->device < 0 || h->device >= 128) return fail(SF_EINVAL, "sf_fock_jk_noalloc: device index out of range");
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
  int rc = launch_slices(h, D, D32, Jh, Kh, st, 0, nullptr);
  if (rc) return rc;
  symmetrize_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(Jh, Kh, J, K, n);
  SF_CK(cudaGetLastError());
  return SF_OK;
}

int sf_grad_jk(sf_handle *h, const double *D, double *grad, int32_t precision, double cutoff, double fp32_cutoff,
               void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_grad_jk: NULL handle");
  if (!D || !grad) return fail(SF_EINVAL, "sf_grad_jk: NULL pointer");
  if (precision < SF_PREC_FP64 || precision > SF_PREC_MIXED) return fail(SF_EINVAL, "sf_grad_jk: bad precision");
  if (!(cutoff >= 0.0) || !(fp32_cutoff >= 0.0)) return fail(SF_EINVAL, "sf_grad_jk: bad cutoff");
  if (!h->have_schwarz) return fail(SF_ESTATE, "sf_grad_jk: call sf_schwarz first");
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  int rc = build_work(h, precision, cutoff, fp32_cutoff);
  if (rc) return rc;
  const size_t nn = (size_t)h->nao * h->nao;
  bool need32 = false;
  for (const auto &s : h->slices) need32 |= s.prec == 1;
  if (need32) {
    to_float_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(D, h->d_D32.p, (int64_t)nn);
    SF_CK(cudaGetLastError());
  }
  auto launch = [&](size_t k, cudaStream_t ss) {
    const auto &s = h->slices[k];
    return s.prec == 0 ? launch_grad_f64(s.cls, h->kp, s.w, D, grad, ss)
                       : launch_grad_f32(s.cls, h->kp, s.w, h->d_D32.p, grad, ss);
  };
  if (h->profiling) {   // per-launch events (serialised in mode 2), read by sf_get_slice_info
    while (h->ev.size() < 2 * h->slices.size()) {
      cudaEvent_t e;
      SF_CK(cudaEventCreate(&e));
      h->ev.push_back(e);
    }
    if (h->profiling == 2) {
      for (size_t k = 0; k < h->slices.size(); ++k) {
        SF_CK(cudaEventRecord(h->ev[2 * k], st));
        SF_CK(launch(k, st));
        SF_CK(cudaEventRecord(h->ev[2 * k + 1], st));
      }
      return SF_OK;
    }
    return fan_out(h, st, [&](size_t k, cudaStream_t ss) {
      cudaError_t e = cudaEventRecord(h->ev[2 * k], ss);
      if (e == cudaSuccess) e = launch(k, ss);
      if (e == cudaSuccess) e = cudaEventRecord(h->ev[2 * k + 1], ss);
      return e;
    });
  }
  return fan_out(h, st, launch);
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
  SF_CK(launch_one_electron_grad(P, D, W, grad, (cudaStream_t)stream));
  return SF_OK;
}

int sf_eri_batch(sf_handle *h, const int32_t *quartets, int64_t nq, int32_t precision, double *out,
                 const int64_t *out_offsets, void *stream) {
  if (!h) return fail(SF_EINVAL, "sf_eri_batch: NULL handle");
  if (nq < 0 || (nq > 0 && (!quartets || !out || !out_offsets))) return fail(SF_EINVAL, "sf_eri_batch: bad arguments");
  if (precision != SF_PREC_FP64 && precision != SF_PREC_FP32) return fail(SF_EINVAL, "sf_eri_batch: bad precision");
  if (nq == 0) return SF_OK;
  DeviceGuard g(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<int32_t> hq((size_t)nq * 4);
  std::vector<int64_t> hoff(nq);
  SF_CK(cudaMemcpyAsync(hq.data(), quartets, hq.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  SF_CK(cudaMemcpyAsync(hoff.data(), out_offsets, hoff.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  SF_CK(cudaStreamSynchronize(st));
  struct Item { int pab, pcd, flags; int64_t off; int str[4]; };
  std::vector<std::vector<Item>> byc(kNumClass);
  for (int64_t q = 0; q < nq; ++q) {
    int s[4], pos[4] = {0, 1, 2, 3};
    for (int k = 0; k < 4; ++k) {
      s[k] = hq[4 * q + k];
      if (s[k] < 0 || s[k] >= h->nshell) return fail(SF_EINVAL, "sf_eri_batch: shell index out of range");
    }
    int nc[4], so[4];
    for (int k = 0; k < 4; ++k) nc[k] = ncart(h->l[s[k]]);
    so[3] = 1;
    so[2] = nc[3];
    so[1] = nc[2] * nc[3];
    so[0] = nc[1] * nc[2] * nc[3];
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
    if (it.pab < 0 || it.pcd < 0) return fail(SF_EINVAL, "sf_eri_batch: internal pair lookup failed");
    it.flags = 0;
    it.off = hoff[q];
    for (int k = 0; k < 4; ++k) it.str[k] = so[pos[k]];
    byc[x * (x + 1) / 2 + y].push_back(it);
  }
  for (int cls = 0; cls < kNumClass; ++cls) {
    const auto &v = byc[cls];
    if (v.empty()) continue;
    std::vector<int> pab(v.size()), pcd(v.size()), fl(v.size()), str(4 * v.size());
    std::vector<int64_t> off(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      pab[i] = v[i].pab; pcd[i] = v[i].pcd; fl[i] = v[i].flags; off[i] = v[i].off;
      for (int k = 0; k < 4; ++k) str[4 * i + k] = v[i].str[k];
    }
    DBuf<int> dpab, dpcd, dfl, dstr;
    DBuf<int64_t> doff;
    SF_CK(dpab.upload(pab)); SF_CK(dpcd.upload(pcd)); SF_CK(dfl.upload(fl)); SF_CK(dstr.upload(str));
    SF_CK(doff.upload(off));
    EriWork w{dpab.p, dpcd.p, dfl.p, doff.p, dstr.p, (int64_t)v.size(), out};
    SF_CK(launch_eri(cls, precision == SF_PREC_FP32, h->kp, w, st));
    SF_CK(cudaStreamSynchronize(st));
  }
  return SF_OK;
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
