/*
 * segfock.h -- C ABI of libsegfock.so, the GB300 direct-SCF Fock builder.
 *
 * It replaces the ERI/Fock boundary of lyuhang428/SegFault_py (src/hf):
 *
 *   reference                                         here
 *   --------------------------------------------------------------------------
 *   rys.eri_rys(c1..c4, e1..e4, s1..s4, n1..n4,       sf_eri_batch: contracted
 *     r1..r4) -> float, one Cartesian AO quartet        shell quartets, all
 *     (src/hf/core/core.f90:967-1002, called at         Cartesian components
 *     src/hf/hf.py:26-30 and :100-104)                  at once
 *   build_eri_parallel: unique quartets i>=j, k>=l,   sf_fock_jk: the same
 *     ij>=kl over Pool(8), dense N^4 tensor             unique (shell) quartets,
 *     (src/hf/hf.py:33-61) + per-iteration J/K          Schwarz-screened, digested
 *     einsums G = J - K/2 (src/hf/hf.py:300)            into J and K on the GPU
 *   mmd2.overlap/kinetic/potential per AO pair        sf_one_electron
 *     (src/hf/mmd2.py:14-84, hf.py:266-274)
 *   Molecule/Atom/ContractedGaussianFunction          sf_create (shell table)
 *     (src/hf/molecule.py:51-226)
 *
 * Conventions
 *   - All compute entry points take DEVICE pointers and a cudaStream_t passed
 *     as void* (NULL = legacy default stream).  Work is stream-ordered; the
 *     host is not synchronised unless stated.
 *   - AO order: shells in the order given, Cartesian components of a shell in
 *     the reference order s; x,y,z; xx,xy,xz,yy,yz,zz (molecule.py:138-153).
 *   - Matrices are row-major nao x nao doubles.
 *   - Every function returns 0 on success or a negative SF_E* code; the text of
 *     the last error of the calling thread is returned by sf_last_error().
 *     Nothing traps or aborts on the device.
 *   - Thread safety: one handle may be used by one host thread at a time.
 */
#ifndef SEGFOCK_H
#define SEGFOCK_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SF_OK 0
#define SF_EINVAL (-1)      /* bad argument                                  */
#define SF_EUNSUPPORTED (-2)/* l > 2, contraction > SF_MAX_PRIM, ...        */
#define SF_ECUDA (-3)       /* a CUDA runtime call failed                    */
#define SF_ESTATE (-4)      /* call order (e.g. Fock build before Schwarz)   */
#define SF_ENOMEM (-5)

#define SF_MAX_L 2
#define SF_MAX_PRIM 16

/* precision modes of sf_fock_jk / sf_eri_batch */
#define SF_PREC_FP64 0      /* every quartet in FP64                          */
#define SF_PREC_FP32 1      /* every quartet in FP32 (FP64 accumulation)      */
#define SF_PREC_MIXED 2     /* FP64 above the FP32 cutoff, FP32 below it      */
#define SF_PREC_MIXED_DF 3  /* double-float (FP32 pairs, ~2^-44 relative) above
                               the FP32 cutoff, FP32 below it                 */
#define SF_PREC_DF 4        /* every quartet in double-float                  */
/* kind of one launch (sf_slice_info.precision, sf_tune_entry.precision):
 * 0 FP64, 1 FP32, 2 double-float */

typedef struct sf_handle sf_handle;

/* One contracted Cartesian shell.  coefs are the contraction coefficients of
 * the x^l component including its primitive normalisation; component
 * (lx,ly,lz) is scaled by sqrt((2l-1)!! / ((2lx-1)!!(2ly-1)!!(2lz-1)!!)), so
 * every Cartesian function is normalised individually as in
 * src/hf/molecule.py:210-226. */
typedef struct {
    int32_t l;
    int32_t nprim;
    int32_t atom;
    int32_t ao_offset;
    double center[3];        /* bohr */
    const double *exps;      /* host pointer, nprim values */
    const double *coefs;     /* host pointer, nprim values */
} sf_shell_desc;

/* counters of the last sf_fock_jk call */
typedef struct {
    int64_t quartets_fp64;        /* canonical shell quartets done in FP64     */
    int64_t quartets_fp32;        /* ... in FP32                               */
    int64_t quartets_total;       /* canonical shell quartets before screening */
    int64_t prim_quartets_fp64;
    int64_t prim_quartets_fp32;
    double flop_alg_fp64;         /* algorithmic FLOPs (Rys assembly + digestion) */
    double flop_alg_fp32;
    int32_t launches;             /* kernel launches issued by the call        */
    int32_t reserved;
} sf_stats;

/* library version (major*10000 + minor*100 + patch) */
int sf_version(void);

/* text of the last error on this host thread ("" if none) */
const char *sf_last_error(void);

/* Build the shell table, primitive-pair data and Rys root tables on the
 * current device.  Replaces Molecule/Atom/ContractedGaussianFunction set-up
 * (src/hf/molecule.py:51-226).  Allocates device memory owned by the handle. */
int sf_create(const sf_shell_desc *shells, int32_t nshell, sf_handle **out);

/* Same as sf_create (name used by earlier drafts of the interface). */
int sf_build_shells(const sf_shell_desc *shells, int32_t nshell, sf_handle **out);

void sf_destroy(sf_handle *h);

/* number of Cartesian AOs and shell pairs of the handle */
int32_t sf_nao(const sf_handle *h);
int64_t sf_npairs(const sf_handle *h);

/* Schwarz bounds Q_ab = sqrt(max |(ab|ab)|) for every shell pair a >= b,
 * computed on the GPU in FP64 and kept in the handle (needed by sf_fock_jk).
 * q_out (optional, host pointer, nshell*nshell doubles, symmetric) receives
 * them.  Synchronises the stream.  The reference has no screening
 * (hf.py:37-43 enumerates every quartet). */
int sf_schwarz(sf_handle *h, double *q_out, void *stream);

/* Coulomb and exchange matrices for a symmetric density D (device, nao*nao):
 *   J_pq = sum_rs (pq|rs) D_rs,  K_pq = sum_rs (pr|qs) D_rs
 * (the two einsums of src/hf/hf.py:300), over the canonical shell quartets
 * with Q_ab Q_cd >= cutoff.  In SF_PREC_MIXED and SF_PREC_MIXED_DF, quartets
 * with Q_ab Q_cd < fp32_cutoff are evaluated in FP32, the others in FP64
 * (MIXED) or double-float (MIXED_DF); J and K are accumulated in FP64 in
 * every mode.  sf_stats counts the FP64 / double-float tier as "fp64".
 * J, K: device, nao*nao, overwritten.
 * stats (optional, host) receives counters.  Does not synchronise unless
 * stats is given. */
int sf_fock_jk(sf_handle *h, const double *D, double *J, double *K, int32_t precision,
               double cutoff, double fp32_cutoff, sf_stats *stats, void *stream);

/* Autotuner of the launch shapes.  Each launch of a Fock build (one class,
 * one precision, one cost segment of the quartet list) maps a quartet onto
 * T x P x W lanes: T lanes share its Cartesian outputs (fixed per class),
 * its primitive loop is split S = P*W ways (P lane groups inside a warp, W
 * separate groups whose partial integrals are digested separately).  The
 * library picks S by a cost rule: enough sub-groups that a launch covers
 * the GPU ("fill" target), at least one primitive quartet each.  sf_autotune,
 * for the given precision mode and cutoffs, on `stream` (adding into the
 * handle's scratch only; the caller's matrices are not touched):
 *   1. times whole builds (launches concurrent) with fill targets 0, 1/4, 1
 *      and 4 times 8 warps per SM sub-partition and keeps the fastest; in
 *      the mixed modes it then times the accurate tier (few, long quartets)
 *      at its own targets 0 .. 16 times, keeping one only if faster;
 *   2. times every launch alone (reps times) with S/4, S/2, S, 2S, 4S and
 *      records the fastest; streams are then assigned by measured times;
 *   3. keeps the step-2 splits only if the whole build got faster.
 * Later builds with the same work lists use the recorded shapes.  Returns the
 * number of launches tuned (>= 0) or an error code.  The table can be read
 * out and loaded again (e.g. from a file): sf_set_tuning replaces it (n = 0
 * clears it).  Entries with cls = -1 hold the fill target of precision mode
 * `precision` in `split` (quarters; 0 = no extra split), entries with
 * cls = -2 that of the accurate tier of a mixed mode when it differs. */
typedef struct {
    int32_t cls;           /* canonical class 0..20 (ss|ss .. dd|dd); -1 / -2: fill target */
    int32_t precision;     /* launch kind: 0 FP64, 1 FP32, 2 double-float; precision mode for cls < 0 */
    int64_t cost;          /* K_ab*K_cd of the launch's first (costliest) quartet */
    int32_t split;         /* chosen S = P*W (power of two)                   */
    float ms_default;      /* measured time with the rule's S                 */
    float ms_tuned;        /* measured time with the chosen S                 */
} sf_tune_entry;
int sf_autotune(sf_handle *h, const double *D, int32_t precision, double cutoff, double fp32_cutoff,
                int32_t reps, void *stream);
int32_t sf_tuning_count(const sf_handle *h);
int sf_get_tuning(const sf_handle *h, int32_t idx, sf_tune_entry *out);
int sf_set_tuning(sf_handle *h, const sf_tune_entry *entries, int32_t n);

/* Density-weighted classification of the quartet lists, redone on the device
 * by every sf_fock_jk / sf_grad_jk call from its density D (no counterpart in
 * the reference, which computes every quartet in FP64).  With M_xy the
 * largest |D| element of the block of shells x, y:
 *  - SF_DENS_FOCK, Fock build, mixed modes: a quartet of the accurate tier
 *    (Q_ab Q_cd >= fp32_cutoff) stays there only while Q_ab Q_cd max(2M_ab,
 *    2M_cd, M_ac, M_bd, M_ad, M_bc) -- a bound on what it adds to any element
 *    of J or K -- is >= fock_fp32_cutoff; otherwise it runs in FP32.  Off by
 *    default: the split then moves with D from one SCF iteration to the next,
 *    which makes F(D) jump by the FP32 rounding of the quartets that change
 *    tier and stalls the last decades of an SCF's convergence, for a gain of
 *    about 1 % of the build time on water clusters;
 *  - SF_DENS_GRAD, gradient: a quartet whose bound B = Q_ab Q_cd (M_ab
 *    M_cd/2 + (M_ac M_bd + M_ad M_bc)/8) is below grad_drop_cutoff is left
 *    out; in the mixed modes one of the accurate tier runs in FP32 when
 *    B (s_a + s_b + s_c + s_d) is below grad_fp32_cutoff, s_x the square root
 *    of shell x's largest exponent (a derivative integral outgrows the
 *    Schwarz bound of its integral by about that factor).  On by default.
 * A negative cutoff means the default: the call's fp32_cutoff for the Fock
 * build's FP32 cutoff, 3e-2 times it for the gradient's (measured against
 * FP64 with fp32_cutoff 1e-2: 6.9e-8 Eh/bohr on (H2O)16 in 6-31G*, 4.5e-7 on
 * C20H42 in 6-31G**), the Schwarz cutoff for the drop cutoff.  flags = 0
 * turns the classification off (every call then uses the Schwarz-sorted
 * lists as cut).
 * Default: SF_DENS_GRAD, all three cutoffs negative. */
#define SF_DENS_FOCK 1
#define SF_DENS_GRAD 2
int sf_set_density_screening(sf_handle *h, int32_t flags, double fock_fp32_cutoff, double grad_drop_cutoff,
                             double grad_fp32_cutoff);

/* One Fock build captured as a CUDA graph, for callers that replay it (an SCF
 * iteration on a fixed geometry): sf_fock_jk_graph_create runs one ordinary
 * sf_fock_jk (which cuts and caches the quartet lists), then captures a
 * second one on an internal stream (the class launches and their fork/join
 * over the side streams become graph nodes) and instantiates it.  With
 * node_priority != 0 the graph runs each launch at the priority of the side
 * stream it was captured from (cudaGraphInstantiateFlagUseNodePriority): the
 * accurate tier of a mixed build keeps its high priority, as in an eager
 * build; with 0 every node runs at the priority of the launching stream.
 * sf_fock_graph_launch replays it on a stream for the current contents of D
 * (same pointers, same precision and cutoffs); nothing allocates.  Changing
 * the handle's lists (sf_autotune, sf_set_tuning, sf_set_partition,
 * sf_schwarz) invalidates the graph.  No counterpart in the reference. */
typedef struct sf_fock_graph sf_fock_graph;
int sf_fock_jk_graph_create(sf_handle *h, const double *D, double *J, double *K, int32_t precision, double cutoff,
                            double fp32_cutoff, int32_t node_priority, void *stream, sf_fock_graph **out);
int sf_fock_graph_launch(sf_fock_graph *g, void *stream);
/* Instantiate a graph the caller captured and owns (a cudaGraph_t, e.g. the
 * whole SCF iteration captured by torch.cuda.CUDAGraph(keep_graph=True)),
 * with node priorities when node_priority != 0, on the current device; launch
 * and free it with sf_fock_graph_launch / sf_fock_graph_destroy (which leaves
 * the caller's graph alone).  The graph must outlive the instance. */
int sf_graph_instantiate(void *graph, int32_t node_priority, sf_fock_graph **out);
void sf_fock_graph_destroy(sf_fock_graph *g);

/* How a Fock build launches its class kernels (no counterpart in the
 * reference, whose scheduler is Pool(8).map over AO quartets, hf.py:45-47):
 *  - SF_LAUNCH_STREAMS (default): one launch per (class, precision, primitive
 *    split) slice, spread over 16 side streams forked from the caller's
 *    stream and joined back;
 *  - SF_LAUNCH_PERSISTENT: the FP32 register-path classes run as one
 *    persistent launch per register tier (four tiers of similar register
 *    use), each CTA taking CTA-sized tiles of the tier's lists from a device
 *    work queue, heaviest first, until it is empty; the other lists keep their
 *    own launches.  ctas_per_sm sets the persistent grid (0: the occupancy
 *    limit of each tier kernel).  Profiling modes and gradients use the
 *    stream launches.  The first build in this mode after the lists change
 *    allocates the tile tables.
 * The measured comparison is in the design notes; the default is the faster. */
#define SF_LAUNCH_STREAMS 0
#define SF_LAUNCH_PERSISTENT 1
int sf_set_launch_mode(sf_handle *h, int32_t mode, int32_t ctas_per_sm);

/* Restrict sf_fock_jk to the slice [part, part+1) of nparts equal-work slices
 * of every quartet class (replica / multi-GPU partitioning hook; 0,1 = all). */
int sf_set_partition(sf_handle *h, int32_t part, int32_t nparts);

/* Raw contracted ERIs of nq shell quartets (device int32[nq*4] shell ids, any
 * order of angular momenta).  out (device) receives, for quartet q at
 * out_offsets[q] (device int64[nq]), the ncart(a)*ncart(b)*ncart(c)*ncart(d)
 * integrals (ab|cd) in row-major component order.  precision: SF_PREC_FP64,
 * SF_PREC_FP32 or SF_PREC_DF (evaluated in that arithmetic, stored as
 * double). */
int sf_eri_batch(sf_handle *h, const int32_t *quartets, int64_t nq, int32_t precision,
                 double *out, const int64_t *out_offsets, void *stream);

/* The same raw-ERI batch prepared once and run many times (replaces the
 * per-AO-quartet rys.eri_rys calls of src/hf/hf.py:26-30 as one batched
 * evaluation).  sf_eri_plan_create takes the shell quartets on the HOST
 * (int32[nq*4]); the plan owns the class-sorted device work lists; outputs are
 * packed in input order (quartet q at offsets[q], ncart(a)*ncart(b)*ncart(c)*
 * ncart(d) values, row-major).  sf_eri_plan_run launches every class on the
 * handle's side streams, forked from and joined back into `stream`; it
 * allocates nothing and can be captured in a CUDA graph.  A plan belongs to
 * its handle and must be destroyed before it. */
typedef struct sf_eri_plan sf_eri_plan;
int sf_eri_plan_create(sf_handle *h, const int32_t *quartets, int64_t nq, sf_eri_plan **out);
/* total output doubles, primitive quartets and algorithmic FLOPs of one run */
int sf_eri_plan_info(const sf_eri_plan *plan, int64_t *outputs, int64_t *prim_quartets, double *flop_alg);
/* host int64[nq]: output offset of every quartet */
int sf_eri_plan_offsets(const sf_eri_plan *plan, int64_t *offsets);
int sf_eri_plan_run(sf_eri_plan *plan, int32_t precision, double *out, void *stream);
/* The same plan evaluated by the McMurchie-Davidson engine instead of Rys
 * quadrature (Hermite expansion coefficients, Boys function and Hermite
 * Coulomb integrals R_tuv: module mmd of src/hf/core/core.f90:23-198, the
 * reference's second integral engine): an independent cross-check of the
 * production Rys kernels.  SF_PREC_FP64: everything on the CUDA cores in
 * FP64.  SF_PREC_FP32: FP32 MD whose bra Hermite-to-Cartesian E contraction
 * runs on the tcgen05 tensor cores (kind::tf32, three-pass hi/lo split for
 * FP32 accuracy); synchronises the stream and returns SF_ECUDA if a bounded
 * wait on the tensor cores timed out.  Other precisions: SF_EUNSUPPORTED. */
int sf_eri_plan_run_md(sf_eri_plan *plan, int32_t precision, double *out, void *stream);
/* Test hook for the error path of the tensor-core McMurchie-Davidson kernels
 * (sf_eri_plan_run_md in FP32): every wait for their MMAs is bounded, and a
 * wait that runs out sets a device flag, waits (again bounded) for the MMAs
 * in flight, frees the tensor memory and returns; the run then fails with
 * SF_ECUDA and its outputs are not to be used.  This sets the bound of the
 * first wait to `iterations` polls: 0 makes it count as run out before its
 * first poll, so a test can take that path without any fault; -1 restores
 * the default (2^24 polls).  Process-wide; not for production use.  No
 * counterpart in the reference. */
int sf_debug_tc_wait_limit(int32_t iterations);
void sf_eri_plan_destroy(sf_eri_plan *plan);

/* One-electron matrices (device, nao*nao each): overlap S, kinetic T and
 * nuclear attraction V = sum_C -Z_C <a|1/r_C|b> for natom point charges
 * (atom_xyz device [natom*3] bohr, charges device [natom]).
 * src/hf/mmd2.py:14-84 with hf.py:266-274.  Any of S, T, V may be NULL. */
int sf_one_electron(sf_handle *h, const double *atom_xyz, const double *charges,
                    int32_t natom, double *S, double *T, double *V, void *stream);

/* Two-electron part of the analytic RHF nuclear gradient (no counterpart in
 * the reference, which has no gradients):
 *   grad[3*A + d] += sum_{pqrs} G_pqrs d(pq|rs)/dR_{A,d},
 *   G_pqrs = 1/2 D_pq D_rs - 1/8 (D_pr D_qs + D_ps D_qr),
 * i.e. the derivative of 1/2 sum_pq D_pq (J - K/2)_pq at fixed D, over the
 * same screened quartets and precision split as sf_fock_jk (FP64, FP32 and
 * double-float derivative kernels).  grad (device, 3 doubles per atom index
 * used by the shells) is accumulated, not zeroed. */
int sf_grad_jk(sf_handle *h, const double *D, double *grad, int32_t precision, double cutoff,
               double fp32_cutoff, void *stream);

/* Counters of the last sf_grad_jk call on this handle, after the
 * density-weighted screening (synchronises `stream` first): surviving
 * quartets and primitive quartets of the accurate tier ("fp64": FP64 or
 * double-float) and of the FP32 tier, and their algorithmic FLOPs for
 * derivative quartets, per quartet K_aK_bK_cK_d n' 36 N_c (nine derivative
 * components, centres A, B, C times x, y, z, each a 4-FLOP assembly
 * Ix' Iy Iz w per output, root and primitive quartet; n' = floor((L+1)/2)+1
 * roots; root, recurrence and contraction work excluded); launches = the
 * call's class launches.  No counterpart in the reference. */
int sf_grad_stats(sf_handle *h, sf_stats *stats, void *stream);

/* One-electron part of the gradient: derivatives of sum_pq D_pq (T+V)_pq
 * - W_pq S_pq with respect to the basis centres and, for V, the nuclei
 * (W = energy-weighted density 2 sum_occ e_i C_pi C_qi).  atom_xyz/charges as
 * in sf_one_electron; grad accumulated. */
int sf_grad_one_electron(sf_handle *h, const double *atom_xyz, const double *charges, int32_t natom,
                         const double *D, const double *W, double *grad, void *stream);

/* Per-launch profiling of sf_fock_jk.  on = 1: every class kernel of a Fock
 * build is bracketed by CUDA events on the stream it runs on (class launches
 * run concurrently on streams forked from the caller's, so these times
 * overlap); on = 2: the launches are also serialised on the caller's stream,
 * so each time is that kernel alone; 0: off.  sf_slice_info
 * then reports, per launch ("slice" = one class in one precision), the work,
 * the device time of the last profiled build (waits for its events) and the
 * launch's start after the build's start (a timeline of the concurrent build).
 * No counterpart in the reference (it only times whole SCF runs,
 * src/hf/utils.py:76-83). */
typedef struct {
    int32_t cls;              /* canonical class id 0..20                      */
    int32_t precision;        /* launch kind: 0 FP64, 1 FP32, 2 double-float   */
    int32_t la, lb, lc, ld;
    int64_t quartets;
    int64_t prim_quartets;
    double flop_alg;
    float ms;                 /* device time of the last profiled launch      */
    int32_t threads_per_quartet;   /* lanes per quartet: Cartesian split T x primitive split (P lane groups x W groups) */
    float start_ms;           /* start of the launch after the start of its build */
    int32_t stream;           /* side stream of the launch (-1: serialised)     */
} sf_slice_info;

int sf_set_profiling(sf_handle *h, int32_t on);
int32_t sf_slice_count(const sf_handle *h);
int sf_get_slice_info(sf_handle *h, int32_t idx, sf_slice_info *out);

/* FMA-throughput microbenchmark of the FP64 (precision 0) or FP32 (1)
 * CUDA-core pipe on the current device: *flops executed in *ms.  It is the
 * peak the roofline fractions are quoted against.  No counterpart in the
 * reference.  Synchronises the stream. */
int sf_fma_peak(int32_t precision, double *flops, float *ms, void *stream);

/* Allocation-free Fock build.  No counterpart in the reference.
 *
 * Same result and arguments as sf_fock_jk (without stats), for callers that
 * cannot call cudaMalloc when they build a Fock matrix: code that runs where
 * another component owns all device memory (a framework's memory pool, a
 * fixed memory budget) or a time-critical loop that must not enter the CUDA
 * allocator.  The scratch sf_fock_jk keeps in the handle (the half matrices
 * Jh, Kh and the single-precision copy of D) lives here in one static device
 * array of the library, sized for nao <= SF_NOALLOC_MAX_NAO (2.5 * 1024^2
 * doubles = 20 MiB, held on every GPU that loads the library until the
 * process exits).  Larger handles are rejected with SF_EINVAL.
 *
 * The call allocates nothing: no cudaMalloc, cudaFree or allocating library
 * routine.  Set-up that does allocate must happen before it: sf_create,
 * sf_schwarz, and one sf_fock_jk call with the same precision and cutoffs,
 * which builds the quartet lists of the handle (otherwise SF_ESTATE).
 * sf_schwarz, sf_autotune, sf_set_tuning and sf_set_partition discard those
 * lists (the next sf_fock_jk re-cuts them with the new bounds, splits or
 * partition), so after any of them one more allocating sf_fock_jk call with
 * the same arguments must come before the next sf_fock_jk_noalloc.  The
 * first call on a device looks up the device address of the static array
 * (cudaGetSymbolAddress) with that device current; make that first call before
 * any stream capture.  The address is kept for the life of the process: it
 * assumes the device's primary context is never reset (cudaDeviceReset) while
 * the library is loaded.  Every call shares the one array: calls that overlap on
 * the GPU (other streams, other threads, other handles) race and must be
 * serialised by the caller.  The array is cleared by each call before use. */
#define SF_NOALLOC_MAX_NAO 1024
int sf_fock_jk_noalloc(sf_handle *h, const double *D, double *J, double *K, int32_t precision,
                       double cutoff, double fp32_cutoff, void *stream);

/* x = A^-1 b for a small dense system (n <= 32; device row-major A[n*n],
 * b[n], x[n]), Gaussian elimination with partial pivoting on the device;
 * *ok (device double) = 1, or 0 with x = 0 when A is singular.  Used for the
 * DIIS system (src/hf/hf.py:330-346) inside a captured SCF iteration, where a
 * host-side check is not possible. */
int sf_small_solve(int32_t n, const double *A, const double *b, double *x, double *ok, void *stream);

/* Host evaluation of the library's Rys root table (for checks without a GPU):
 * n-point rule at x, u[i] = t_i^2, w[i] weights; fp32 != 0 selects the
 * single-precision table. */
int sf_rys_roots_host(int32_t n, double x, int32_t fp32, double *u, double *w);

#ifdef __cplusplus
}
#endif
#endif /* SEGFOCK_H */
