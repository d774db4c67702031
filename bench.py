"""Benchmark: Fock builds/s of the GPU direct-SCF J/K build.

Workload (N=1): seeded (H2O)_8 water cluster, 6-31G* (Cartesian d), 152 AOs,
80 shells; Schwarz cutoff 1e-12; FP32 cutoff 1e-2 for the mixed path.  The
density is the converged FP64 RHF density of that cluster (computed once,
outside the timed region).  One step = one Fock build J, K = jk(D) (the two
einsums of the reference's hf.py:300 without the N^4 tensor), mixed precision:
quartets with Q_ab Q_cd < 1e-2 in FP32, the others in double-float (FP32
pairs, ~2^-44 relative per operation), J/K accumulated in FP64.  Launch shapes
are autotuned for every timed mode before the timed region.

Reported:
* value        Fock builds/s, mixed path (FP32 + double-float), D/J/K resident
               in HBM; L2 flushed (256 MB write) before every step, each step
               timed by CUDA events; each build replayed from the library's own
               capture of it (FockBuilder.capture_jk(native=True):
               sf_fock_jk_graph_create / sf_fock_graph_launch, node priorities
               kept) -- the way an SCF iteration runs it; the same build issued
               eagerly through FockBuilder.jk is eager_value (graph_replay_value:
               replayed from a torch.cuda.CUDAGraph; persistent_launch_value:
               the FP32 register-path classes as one persistent launch per
               register tier, fed by a device work queue)
* e2e          same metric through the public API with host buffers: pinned D
               -> device, Fock build, J and K -> pinned host, every step
* fp64         the all-FP64 build, same protocol (the plain FP64 GPU baseline)
* mixed_fp32_fp64  the mixed build with native FP64 above the cutoff
* roofline     dominant class kernel (the (class, precision) kernel with the
               most device time over its launches in one build): algorithmic
               FLOPs / event time of its largest launch vs the FMA peak of its
               precision measured live by an FMA-chain kernel
* cpu_baseline the oracle's restatement of the reference algorithm (one call
               per unique AO quartet, 5 Rys roots, no screening, OpenMP over
               all host cores) on a bounded stride sample, extrapolated
* clocks       nvidia-smi samples taken during the timed region
* secondary    (H2O)16 6-31G*: mixed vs FP64 Fock builds/s and forces/s
* eri_batch    1e6 random shell quartets over all 21 classes: raw-ERI
               quartets/s in FP64 and FP32 through one prepared plan
* alkane       C20H42 6-31G** (510 AOs): graph-captured mixed SCF wall time
               and errors against FP64, Fock builds/s and forces/s

``--impl reference`` times the reference's CPU algorithm (oracle port, all host
cores, the reference's root5 fits where transcribed) on the same workload and
prints the same metric; every timed step there is one whole Fock build.
Multi-GPU (torchrun, N ranks): replicas -- every rank builds the same Fock
matrix; value = sum over ranks of builds / max-over-ranks time (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = ("Fock builds/s ((H2O)8 6-31G*, mixed precision: FP32 below Q_abQ_cd 1e-2, double-float above, "
          "FP64 accumulation; Schwarz 1e-12)")
HEADLINE = "mixed_df"
CUTOFF = 1e-12
FP32_CUTOFF = 1e-2
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes (read + write) per quartet of the J/K class kernels of this
# workload, from one ncu capture (segfault_py_gb300/profile_traffic.py) committed
# as a text table under profiles/ together with a hash of the kernel sources
# it was measured on; a table whose hash does not match the sources being run
# gives traffic = null (stale)
TRAFFIC_TABLE = os.path.join(REPO, "profiles", "ncu_dram_bytes_water8_631gs.txt")


def csrc_hash():
    """sha256 (first 16 hex digits) over the library's CUDA/C++ sources."""
    from segfault_py_gb300.profile_traffic import csrc_hash as h
    return h()


def ncu_traffic(kernel):
    """(DRAM bytes per quartet, source note) of a kernel family from the committed table."""
    if not os.path.exists(TRAFFIC_TABLE):
        return None, "no ncu table"
    table, src_hash = {}, None
    for line in open(TRAFFIC_TABLE):
        t = line.split()
        if not t:
            continue
        if t[0] == "#" and len(t) >= 3 and t[1] == "csrc_sha16":
            src_hash = t[2]
        elif t[0] != "#" and len(t) >= 2:
            table[t[0]] = float(t[1])
    if src_hash != csrc_hash():
        return None, "ncu table measured on other kernel sources (stale)"
    if kernel not in table:
        return None, "kernel not in the ncu table"
    return table[kernel], "ncu capture, " + os.path.relpath(TRAFFIC_TABLE, REPO) + " (bytes per quartet x quartets of the launch)"


def workload(nwater=8, basis="6-31g*", seed=0):
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.molecule import Molecule
    s, x = G.water_cluster(nwater, seed=seed)
    return Molecule.from_geometry(s, x, basis)


def cfg_dict(mol, nwater, basis):
    return {"workload": "(H2O)%d water cluster, %s, seed 0" % (nwater, basis.upper()), "nao": mol.nao,
            "nshell": len(mol.shells), "schwarz_cutoff": CUTOFF, "fp32_cutoff": FP32_CUTOFF,
            "density": "converged FP64 RHF", "l2": "flushed before every step (256 MB write)",
            "parallelism": "replicas"}


# ----------------------------------------------------------------------------
def clock_sampler_start(path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                stdout=f, stderr=subprocess.DEVNULL)
    except Exception:
        return None, None
    # wait (at most 5 s) for the first sample: nvidia-smi's start-up, which
    # initialises NVML, must not fall into the timed steps
    t0 = time.time()
    while time.time() - t0 < 5.0 and proc.poll() is None:
        f.flush()
        if os.path.getsize(path) > 0:
            break
        time.sleep(0.05)
    time.sleep(0.3)
    return proc, f


def clock_sampler_stop(proc, f, path, device_index=0):
    if proc is None:
        return None
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except Exception:
        proc.kill()
    f.close()
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        t = [v.strip() for v in line.split(",")]
        if len(t) < 9 or t[0] != str(device_index):
            continue
        try:
            sm.append(float(t[1]))
            smax.append(float(t[2]))
        except ValueError:
            continue
        for nm, v in zip(names, t[5:9]):
            if v.lower() == "active":
                reasons.add(nm)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
            "samples": len(sm)}


# ----------------------------------------------------------------------------
def fma_peaks(dev):
    """Live FMA-throughput peaks (TFLOP/s) of the FP64 and FP32 CUDA-core pipes."""
    import torch
    from segfault_py_gb300 import _lib
    import ctypes as C
    L = _lib.lib()
    out = {}
    for prec, name in ((0, "fp64"), (1, "fp32")):
        flops = C.c_double(0.0)
        ms = C.c_float(0.0)
        _lib.check(L.sf_fma_peak(prec, C.byref(flops), C.byref(ms), C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        out[name] = flops.value / (ms.value * 1e-3) / 1e12
    return out


def time_steps(fn, steps, warmup, flush, stream):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        fn()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def dominant_kernel(slices):
    """The J/K class kernel with the most device time over its launches of one
    build (launches of one class and precision run the same kernel), its
    largest launch and its name: (largest launch, all its launches, name)."""
    groups = {}
    for sl in slices:
        groups.setdefault((sl["la"], sl["lb"], sl["lc"], sl["ld"], sl["precision"]), []).append(sl)
    group = max(groups.values(), key=lambda g: sum(sl["ms"] for sl in g))
    top = max(group, key=lambda sl: sl["ms"])
    name = "jk_kernel<%d,%d,%d,%d,%s>" % (top["la"], top["lb"], top["lc"], top["ld"],
                                          ("fp64", "fp32", "dd")[top["precision"]])
    return top, group, name


def run_ours(args):
    import torch
    import torch.distributed as dist
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.scf import scf_diis

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nwater, basis = args.nwater, args.basis
    mol = workload(nwater, basis)
    fb = FockBuilder(mol, device=dev, cutoff=CUTOFF, fp32_cutoff=FP32_CUTOFF, precision="mixed")
    r = scf_diis(mol, tol=1e-9, fb=fb, device=dev, precision="fp64")
    D = r.D.contiguous()
    H = r.H
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    J = torch.empty_like(D)
    K = torch.empty_like(D)

    # launch shapes autotuned for every mode that is timed (outside the timed region)
    t0 = time.time()
    if args.tuning and os.path.exists(args.tuning):
        fb.load_tuning(args.tuning)
    else:
        for prec in (HEADLINE, "mixed", "fp64"):
            fb.autotune(D, precision=prec, reps=3)
        if args.tuning and rank == 0:
            fb.save_tuning(args.tuning)
    tune_s = time.time() - t0

    # error of the mixed builds against the FP64 build at the converged density
    def energy(prec):
        fb.jk(D, precision=prec, out=(J, K))
        F = H + J - 0.5 * K
        return float(0.5 * torch.sum(D * (H + F)))
    e64, ehl, emx = energy("fp64"), energy(HEADLINE), energy("mixed")
    vs_oracle = oracle_energy_errors(fb, mol, nwater, basis, dev)

    # stats + per-launch profile of one build per mode
    prof = {}
    for prec in ("fp64", HEADLINE):
        fb.set_profiling(2)       # launches serialised on one stream: isolated per-kernel times
        fb.jk(D, precision=prec, out=(J, K), stats=True)
        prof[prec] = (dict(fb.last_stats), fb.slice_info())
        fb.set_profiling(False)
    st_hl, slices_hl = prof[HEADLINE]
    st_64, slices_64 = prof["fp64"]

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    if args.clocks_log:
        clk_path = args.clocks_log
    else:
        import tempfile
        clk_path = os.path.join(tempfile.gettempdir(), "segfock_bench_clocks_rank%d.csv" % rank)
    os.makedirs(os.path.dirname(os.path.abspath(clk_path)), exist_ok=True)
    proc, fh = clock_sampler_start(clk_path) if rank == 0 else (None, None)
    t_hl = time_steps(lambda: fb.jk(D, precision=HEADLINE, out=(J, K)), args.steps, args.warmup, flush, stream)
    t_mx = time_steps(lambda: fb.jk(D, precision="mixed", out=(J, K)), args.steps, args.warmup, flush, stream)
    t_64 = time_steps(lambda: fb.jk(D, precision="fp64", out=(J, K)), args.steps, args.warmup, flush, stream)
    # the same build replayed from a captured CUDA graph, reported beside
    g_hl = fb.capture_jk(D, J, K, precision=HEADLINE)
    t_hl_graph = time_steps(g_hl.replay, args.steps, args.warmup, flush, stream)
    # the library's own capture, replayed with the side streams' priorities
    g_nat = fb.capture_jk(D, J, K, precision=HEADLINE, native=True)
    t_hl_native = time_steps(g_nat.replay, args.steps, args.warmup, flush, stream)
    g_nat.close()
    # the same build with the FP32 register-path classes as persistent tier
    # launches fed by a device work queue (sf_set_launch_mode), reported beside
    fb.set_launch_mode("persistent")
    t_hl_persist = time_steps(lambda: fb.jk(D, precision=HEADLINE, out=(J, K)), args.steps, args.warmup, flush,
                              stream)
    fb.set_launch_mode("streams")
    # e2e through the public API with host buffers
    Dh = D.cpu().pin_memory()
    Jh = torch.empty_like(Dh).pin_memory()
    Kh = torch.empty_like(Dh).pin_memory()
    Dd = torch.empty_like(D)

    def e2e_step():
        Dd.copy_(Dh, non_blocking=True)
        fb.jk(Dd, precision=HEADLINE, out=(J, K))
        Jh.copy_(J, non_blocking=True)
        Kh.copy_(K, non_blocking=True)
    t_e2e = time_steps(e2e_step, args.steps, args.warmup, flush, stream)
    torch.cuda.synchronize()
    clocks = clock_sampler_stop(proc, fh, clk_path) if rank == 0 else None
    if world > 1:
        dist.barrier()
    # forces: one complete nuclear gradient (backward from the converged SCF)
    from segfault_py_gb300.grad import rhf_gradient
    t_f = {}
    for prec in (HEADLINE, "fp64"):
        t_f[prec] = time_steps(lambda: rhf_gradient(mol, r, fb, precision=prec), max(3, args.steps // 4),
                               args.warmup, flush, stream)
    g64 = rhf_gradient(mol, r, fb, precision="fp64")
    ghl = rhf_gradient(mol, r, fb, precision=HEADLINE)
    grad_err = float((ghl - g64).abs().max())
    # the headline: the build replayed as the library's own captured graph
    # (one launch per step, node priorities kept); the eager build beside it
    t_val = t_hl_native
    ms_hl, ms_mx, ms_64, ms_e2e = (float(np.sum(t)) for t in (t_val, t_mx, t_64, t_e2e))
    ms_eager = float(np.sum(t_hl))
    if world > 1:
        tt = torch.tensor([ms_hl, ms_mx, ms_64, ms_e2e, ms_eager], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_hl, ms_mx, ms_64, ms_e2e, ms_eager = tt.tolist()
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    steps = args.steps
    value = world * steps / (ms_hl * 1e-3)
    peaks = fma_peaks(dev)
    forces_roof = {prec: grad_roofline(fb, D, prec, peaks, max(3, steps // 4), args.warmup, flush, stream)
                   for prec in (HEADLINE, "fp64")}
    # roofline of the dominant class kernel of the headline build (double-float
    # kernels run on the FP32 pipe: their FP64-equivalent algorithmic FLOPs are
    # set against the FP32 FMA peak)
    dom, dom_group, dom_name = dominant_kernel(slices_hl)
    dom_ms = sum(sl["ms"] for sl in dom_group)
    kind = ("fp64", "fp32", "dd")[dom["precision"]]
    pipe = "fp64" if kind == "fp64" else "fp32"
    achieved = dom["flop_alg"] / (dom["ms"] * 1e-3) / 1e12 if dom["ms"] > 0 else 0.0
    total_ms = sum(s["ms"] for s in slices_hl)
    comb = st_hl["flop_alg_fp32"] / (peaks["fp32"] * 1e12) + st_hl["flop_alg_fp64"] / (peaks["fp32"] * 1e12)
    build_frac = comb / (float(np.mean(t_val)) * 1e-3)
    bpq, traffic_src = ncu_traffic(dom_name)
    traffic = bpq * dom["quartets"] if bpq is not None else None
    setup = setup_costs(mol, dev, D, J, K)
    nn = mol.nao * mol.nao * 8
    secondary = None
    if args.nwater2 > 0:
        secondary = secondary_config(args.nwater2, basis, max(5, args.steps // 2), args.warmup, flush, dev)
    alkane = alkane_config(dev, flush, args.warmup) if args.alkane else None
    eri = None
    if args.eri_quartets > 0:
        eri = eri_batch_config(args.eri_quartets, 3, args.warmup, flush, dev, peaks)
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(mol, args.cpu_seconds)
    rec = {
        "metric": METRIC, "value": value, "unit": "Fock builds/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms_hl / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 + double-float (fp32 pairs); fp64 accumulation", "data": "synthetic",
        "config": cfg_dict(mol, nwater, basis),
        "e2e": {"value": world * steps / (ms_e2e * 1e-3), "unit": "Fock builds/s",
                "h2d_bytes_per_step": nn, "d2h_bytes_per_step": 2 * nn},
        "fp64": {"value": world * steps / (ms_64 * 1e-3), "unit": "Fock builds/s", "ms_per_step": ms_64 / steps,
                 "quartets_per_s": st_64["quartets_fp64"] * steps / (ms_64 * 1e-3),
                 "flop_alg": st_64["flop_alg_fp64"],
                 # algorithmic FLOPs per build over its time against the FP64 FMA peak (a lower
                 # bound: ncu puts the FP64 pipe of its largest kernels at 88-89 % busy)
                 "frac_of_fp64_peak": st_64["flop_alg_fp64"] / (ms_64 / steps * 1e-3) / (peaks["fp64"] * 1e12)},
        "mixed_speedup_vs_fp64": ms_64 / ms_eager,   # both issued eagerly
        "mixed_fp32_fp64": {"value": world * steps / (ms_mx * 1e-3), "unit": "Fock builds/s",
                            "note": "FP32 below the cutoff, native FP64 above",
                            "energy_error_vs_fp64": emx - e64, "speedup_vs_fp64": ms_64 / ms_mx},
        "step_ms": {"min": float(np.min(t_val)), "median": float(np.median(t_val)), "max": float(np.max(t_val))},
        "eager_value": world * steps / (ms_eager * 1e-3),
        "eager_step_ms": {"min": float(np.min(t_hl)), "median": float(np.median(t_hl)), "max": float(np.max(t_hl))},
        "graph_replay_value": world * steps / (float(np.sum(t_hl_graph)) * 1e-3),
        "persistent_launch_value": world * steps / (float(np.sum(t_hl_persist)) * 1e-3),
        "graph_native_value": world * steps / (ms_hl * 1e-3),
        "quartets_per_s": (st_hl["quartets_fp64"] + st_hl["quartets_fp32"]) * world * steps / (ms_hl * 1e-3),
        "prim_quartets_per_s": (st_hl["prim_quartets_fp64"] + st_hl["prim_quartets_fp32"]) * world * steps
                               / (ms_hl * 1e-3),
        "quartets": {"double_float": st_hl["quartets_fp64"], "fp32": st_hl["quartets_fp32"],
                     "unscreened": st_hl["quartets_total"]},
        "energy_error_mixed_vs_fp64": ehl - e64,
        "energy_error_vs_oracle": vs_oracle,
        "forces": {"value": world * 1e3 / float(np.mean(t_f[HEADLINE])), "unit": "forces/s",
                   "fp64": world * 1e3 / float(np.mean(t_f["fp64"])),
                   "max_grad_error_mixed_vs_fp64": grad_err, "unit_error": "Eh/bohr",
                   "note": "derivative integrals: FP32 below the cutoff, double-float above",
                   "roofline": forces_roof},
        "autotune_s": tune_s,
        "setup": setup,
        "gpu_launches": (int(st_hl["launches"]) * 3 + int(st_64["launches"])) * steps,
        "roofline": {"bound": pipe, "achieved": achieved, "peak": peaks[pipe], "unit": "TFLOP/s",
                     "frac": achieved / peaks[pipe] if peaks[pipe] else None,
                     "traffic": traffic, "traffic_unit": "bytes per launch (ncu)", "traffic_source": traffic_src,
                     "kernel": dom_name, "kernel_launches": len(dom_group),
                     "lanes_per_quartet": dom["threads_per_quartet"],
                     "kernel_share": dom_ms / total_ms if total_ms else None,
                     "peak_source": "live FMA-chain kernel (sf_fma_peak), this run",
                     "build_combined_frac": build_frac},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "secondary": secondary,
        "eri_batch": eri,
        "alkane": alkane,
    }
    print(json.dumps(rec))
    if world > 1:
        dist.destroy_process_group()


# ----------------------------------------------------------------------------
def grad_roofline(fb, D, precision, peaks, steps, warmup, flush, stream):
    """Two-electron gradient (sf_grad_jk) alone: CUDA-event time per call and
    the algorithmic FLOPs of its surviving derivative quartets (sf_grad_stats:
    K_aK_bK_cK_d n' 36 N_c per quartet) against the FMA peak of the pipe each
    tier runs on (FP32 pipe for FP32 and double-float, FP64 pipe for FP64)."""
    import ctypes as C
    import torch
    from segfault_py_gb300 import _lib
    from segfault_py_gb300.fock import _ptr, _stream_ptr
    L = _lib.lib()
    g = torch.zeros(3 * fb.mol.natom, dtype=torch.float64, device=D.device)

    def run():
        _lib.check(L.sf_grad_jk(fb.handle, _ptr(D), _ptr(g), _lib.PRECISION[precision], fb.cutoff, fb.fp32_cutoff,
                                _stream_ptr()))
    t = time_steps(run, steps, warmup, flush, stream)
    st = _lib.Stats()
    _lib.check(L.sf_grad_stats(fb.handle, C.byref(st), _stream_ptr()))
    d = st.as_dict()
    ms = float(np.mean(t))
    acc_pipe = "fp64" if precision in ("fp64", "mixed") else "fp32"
    t_acc = d["flop_alg_fp64"] / (peaks[acc_pipe] * 1e12)
    t_32 = d["flop_alg_fp32"] / (peaks["fp32"] * 1e12)
    return {"precision": precision, "two_electron_ms": ms, "launches": d["launches"],
            "quartets_accurate": d["quartets_fp64"], "quartets_fp32": d["quartets_fp32"],
            "flop_alg_accurate": d["flop_alg_fp64"], "flop_alg_fp32": d["flop_alg_fp32"],
            "achieved_tflops": (d["flop_alg_fp64"] + d["flop_alg_fp32"]) / (ms * 1e-3) / 1e12,
            "combined_frac": (t_acc + t_32) / (ms * 1e-3),
            "unit": "TFLOP/s", "peak_source": "live FMA-chain kernel (sf_fma_peak), this run",
            "flop_alg": "per surviving derivative quartet K_aK_bK_cK_d n' 36 N_c (n' = floor((L+1)/2)+1)"}


ORACLE_FIXTURE = os.path.join(REPO, "tests", "golden", "water8_631gs.npz")


def oracle_energy_errors(fb, mol, nwater, basis, dev):
    """Energy errors against the all-FP64 oracle at the oracle's converged
    density, for the (H2O)8 6-31G* workload: the committed fixture holds the
    oracle's D, H and E(D) = 1/2 sum D (2H + J - K/2) + E_nuc (the reference's
    Rys algorithm with its root5 fits, every unique AO quartet).  Each build's
    E(D) uses the fixture's H, so the error is the two-electron part's."""
    import torch
    if nwater != 8 or basis.lower() != "6-31g*" or not os.path.exists(ORACLE_FIXTURE):
        return None
    z = np.load(ORACLE_FIXTURE)
    n = int(z["nao"])
    from segfault_py_gb300 import geometry as G
    _, xyz = G.water_cluster(8, seed=0)
    if n != mol.nao or np.abs(xyz - z["xyz_angstrom"]).max() > 1e-10:
        return None

    def sym(t):
        M = np.zeros((n, n))
        M[np.tril_indices(n)] = t
        return M + np.tril(M, -1).T
    Dn, Hn = sym(z["D"]), sym(z["H"])
    e_ref = float(z["e_elec_at_D"]) + float(z["e_nuc"])
    Dt = torch.tensor(Dn, device=dev)
    out = {"reference": "oracle fixture tests/golden/water8_631gs.npz (E(D) at the oracle's converged D, roots: %s)"
                        % str(z["roots"])}
    for prec in ("fp64", "mixed_df", "mixed"):
        J, K = fb.jk(Dt, precision=prec)
        J, K = J.cpu().numpy(), K.cpu().numpy()
        out[prec] = 0.5 * float(np.sum(Dn * (2.0 * Hn + J - 0.5 * K))) + float(z["e_nuc"]) - e_ref
    return out


def setup_costs(mol, dev, D, J, K, reps=3):
    """Per-geometry cost, paid once per geometry (each step of an optimisation
    or MD loop), outside the Fock-build timing: a new handle (shell and pair
    tables, device upload), the Schwarz bounds (GPU kernels, then the pair
    sort on the host) and the quartet lists the first build cuts on the host."""
    import torch
    from segfault_py_gb300.fock import FockBuilder
    out = {"handle_and_schwarz_ms": [], "first_build_ms": [], "steady_build_ms": []}
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fb = FockBuilder(mol, device=dev, cutoff=CUTOFF, fp32_cutoff=FP32_CUTOFF, precision=HEADLINE)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        fb.jk(D, out=(J, K))
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        fb.jk(D, out=(J, K))
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        fb.close()
        out["handle_and_schwarz_ms"].append((t1 - t0) * 1e3)
        out["first_build_ms"].append((t2 - t1) * 1e3)
        out["steady_build_ms"].append((t3 - t2) * 1e3)
    m = {k: float(np.median(v)) for k, v in out.items()}
    return {"handle_and_schwarz_ms": m["handle_and_schwarz_ms"],
            "quartet_lists_ms": m["first_build_ms"] - m["steady_build_ms"],
            "note": "per geometry, host wall clock (median of %d): sf_create + sf_schwarz, then the quartet lists "
                    "cut by the first sf_fock_jk (first build minus a steady build, %s mode, untuned)"
                    % (reps, HEADLINE)}


def secondary_config(nwater, basis, steps, warmup, flush, dev):
    """Mixed (FP32 + double-float, and FP32 + FP64) vs FP64 Fock builds and
    forces on a second cluster size, launch shapes autotuned first."""
    import torch
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.grad import rhf_gradient
    from segfault_py_gb300.scf import scf_diis
    mol = workload(nwater, basis)
    fb = FockBuilder(mol, device=dev, cutoff=CUTOFF, fp32_cutoff=FP32_CUTOFF, precision=HEADLINE)
    r = scf_diis(mol, tol=1e-9, fb=fb, device=dev, precision="fp64")
    D, H = r.D.contiguous(), r.H
    J, K = torch.empty_like(D), torch.empty_like(D)
    stream = torch.cuda.current_stream()
    modes = (HEADLINE, "mixed", "fp64")
    for p in modes:
        fb.autotune(D, precision=p, reps=3)

    def energy(prec):
        fb.jk(D, precision=prec, out=(J, K))
        return float(0.5 * torch.sum(D * (H + H + J - 0.5 * K)))
    e = {p: energy(p) for p in modes}
    t = {p: time_steps(lambda: fb.jk(D, precision=p, out=(J, K)), steps, warmup, flush, stream) for p in modes}
    tf = {p: time_steps(lambda: rhf_gradient(mol, r, fb, precision=p), max(3, steps // 4), warmup, flush, stream)
          for p in (HEADLINE, "fp64")}
    gerr = float((rhf_gradient(mol, r, fb, precision=HEADLINE) - rhf_gradient(mol, r, fb, precision="fp64")).abs().max())
    m = {p: float(np.mean(t[p])) for p in modes}
    mf = {p: float(np.mean(tf[p])) for p in tf}
    out = {"workload": "(H2O)%d water cluster, %s, seed 0" % (nwater, basis.upper()), "nao": mol.nao,
           "fock_builds_per_s_mixed": 1e3 / m[HEADLINE],
           "fock_builds_per_s_mixed_fp32_fp64": 1e3 / m["mixed"],
           "fock_builds_per_s_fp64": 1e3 / m["fp64"],
           "mixed_speedup_vs_fp64": m["fp64"] / m[HEADLINE],
           "forces_per_s_mixed": 1e3 / mf[HEADLINE],
           "forces_per_s_fp64": 1e3 / mf["fp64"],
           "mixed_fock_plus_forces_speedup_vs_fp64": (m["fp64"] + mf["fp64"]) / (m[HEADLINE] + mf[HEADLINE]),
           "energy_error_mixed_vs_fp64": e[HEADLINE] - e["fp64"],
           "energy_error_mixed_fp32_fp64_vs_fp64": e["mixed"] - e["fp64"],
           "max_grad_error_mixed_vs_fp64": gerr,
           "scf_energy_fp64": r.energy}
    fb.close()
    return out


def alkane_config(dev, flush, warmup):
    """C20H42 all-trans, 6-31G** (510 AOs): the full mixed-precision SCF
    captured as one CUDA graph per iteration, plus forces, against the
    all-FP64 GPU path (energy and gradient errors), and Fock builds/s of both."""
    import torch
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.grad import rhf_gradient
    from segfault_py_gb300.molecule import Molecule
    from segfault_py_gb300.scf import scf_diis
    from segfault_py_gb300.scf_graph import GraphSCF
    sym, xyz = G.alkane(20, seed=0)
    mol = Molecule.from_geometry(sym, xyz, "6-31g**")
    fb = FockBuilder(mol, device=dev, cutoff=CUTOFF, fp32_cutoff=FP32_CUTOFF, precision=HEADLINE)
    torch.cuda.synchronize()
    t0 = time.time()
    ref = scf_diis(mol, tol=1e-9, dtol=1e-7, fb=fb, precision="fp64")
    torch.cuda.synchronize()
    t_ref = time.time() - t0
    fb.autotune(ref.D.contiguous(), precision=HEADLINE, reps=2)
    g = GraphSCF(mol, fb=fb, precision=HEADLINE, fp32_cutoff=FP32_CUTOFF).capture()
    torch.cuda.synchronize()
    t0 = time.time()
    r = g.run(tol=1e-9)
    torch.cuda.synchronize()
    t_graph = time.time() - t0
    stream = torch.cuda.current_stream()
    D = ref.D.contiguous()
    J, K = torch.empty_like(D), torch.empty_like(D)
    t = {p: time_steps(lambda: fb.jk(D, precision=p, out=(J, K)), 3, warmup, flush, stream) for p in (HEADLINE, "fp64")}
    tf = {p: time_steps(lambda: rhf_gradient(mol, ref, fb, precision=p), 3, 1, flush, stream) for p in (HEADLINE, "fp64")}
    g64 = rhf_gradient(mol, ref, fb, precision="fp64")
    gmx = rhf_gradient(mol, ref, fb, precision=HEADLINE)
    out = {"workload": "C20H42 all-trans, 6-31G**, seed 0", "nao": mol.nao,
           "scf_graph_mixed_s": t_graph, "scf_graph_iterations": r.iterations, "scf_graph_converged": r.converged,
           "scf_fp64_eager_s": t_ref, "energy_error_mixed_vs_fp64": r.energy - ref.energy,
           "fock_builds_per_s_mixed": 1e3 / float(np.mean(t[HEADLINE])),
           "fock_builds_per_s_fp64": 1e3 / float(np.mean(t["fp64"])),
           "forces_per_s_mixed": 1e3 / float(np.mean(tf[HEADLINE])),
           "forces_per_s_fp64": 1e3 / float(np.mean(tf["fp64"])),
           "max_grad_error_mixed_vs_fp64": float((gmx - g64).abs().max()),
           "scf_energy_fp64": ref.energy}
    fb.close()
    return out


def eri_batch_config(nq, steps, warmup, flush, dev, peaks):
    """Raw-ERI stress batch: nq random contracted shell quartets, class
    uniform over ss|ss .. dd|dd, contraction 1-6, exponents log-uniform in
    [0.05, 1e4], centres in a 10 A box (seed 0); one prepared plan, every class
    launched on the side streams; FP64 and FP32 outputs (stored as float64)."""
    import torch
    from segfault_py_gb300 import geometry as G
    from segfault_py_gb300.fock import FockBuilder
    table, q = G.random_quartet_batch(nq, seed=0)
    fb = FockBuilder(table, device=dev)
    plan = fb.eri_plan(q)
    stream = torch.cuda.current_stream()
    out64 = torch.empty(plan.outputs, dtype=torch.float64, device=dev)
    out32 = torch.empty_like(out64)
    t = {"fp64": time_steps(lambda: plan.run("fp64", out64), steps, warmup, flush, stream),
         "fp32": time_steps(lambda: plan.run("fp32", out32), steps, warmup, flush, stream)}
    diff = float((out32 - out64).abs().max())
    amax = float(out64.abs().max())
    res = {"workload": "%d random contracted shell quartets, classes ss|ss..dd|dd uniform, K 1-6, "
                       "exponents log-uniform [0.05, 1e4], 10 A box, seed 0" % nq,
           "outputs": plan.outputs, "prim_quartets": plan.prim_quartets, "flop_alg": plan.flop_alg}
    for p in ("fp64", "fp32"):
        ms = float(np.mean(t[p]))
        res[p] = {"ms": ms, "quartets_per_s": nq / (ms * 1e-3), "prim_quartets_per_s": plan.prim_quartets / (ms * 1e-3),
                  "tflops_alg": plan.flop_alg / (ms * 1e-3) / 1e12,
                  "frac_of_fma_peak": plan.flop_alg / (ms * 1e-3) / 1e12 / peaks[p] if peaks.get(p) else None}
    res["max_abs_diff_fp32_vs_fp64"] = diff
    res["max_abs_fp64"] = amax
    plan.close()
    fb.close()
    return res


def cpu_baseline(mol, seconds=15.0):
    """Oracle port of the reference algorithm on a bounded stride sample of the
    unique AO quartets (rows ij of the packed pair index with ij % stride == 0)."""
    from oracle import oracle as O
    n = mol.nao
    cg = O.cgf_array(mol.cgfs)
    D = np.eye(n) * 0.1
    npair = n * (n + 1) // 2
    tot = npair * (npair + 1) // 2
    threads = os.cpu_count() or 1
    stride = 4000
    while True:
        rows = np.arange(0, npair, stride)
        cov = int(np.sum(rows + 1))
        t = time.time()
        O.jk_direct(cg, D, nthreads=threads, stride=stride, phase=0)
        dt = time.time() - t
        if dt * 3 > seconds or stride <= 1:
            break
        stride = max(1, int(stride * dt / seconds * 1.5) if dt > 0.05 else stride // 8)
    full = dt * tot / cov
    root = "reference root5 (transcribed)" if O.use_reference_root5(True) else "oracle root table"
    O.use_reference_root5(False)
    return {"value": 1.0 / full, "unit": "Fock builds/s", "cores": threads, "kind": "port",
            "sample": "%d of %d unique AO quartets (stride %d over packed pair rows), %.1f s, extrapolated"
                      % (cov, tot, stride, dt),
            "algorithm": "reference rys.eri_rys per AO quartet, 5 roots, no screening, direct J/K digestion",
            "roots": root}


def run_reference(args):
    """The reference's CPU algorithm (oracle port of core.f90 rys.eri_rys per
    unique AO quartet, hf.py:33-61, with the reference's own root5 fits where
    they were transcribed) on all host cores.  Every timed step is one whole
    Fock build: all N(N+1)/2 x (N(N+1)/2 + 1)/2 unique AO quartets digested
    into J and K.  The untimed warm-up steps run a 1/40 row sample each (they
    only bring the code and tables into the caches)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    mol = workload(args.nwater, args.basis)
    n = mol.nao
    cg = O.cgf_array(mol.cgfs)
    D = np.eye(n) * 0.1
    npair = n * (n + 1) // 2
    tot = npair * (npair + 1) // 2
    threads = os.cpu_count() or 1
    use_ref = O.use_reference_root5(True)
    for i in range(args.warmup):
        O.jk_direct(cg, D, nthreads=threads, stride=40, phase=i % 40)
    times = []
    for _ in range(args.steps):
        t = time.time()
        O.jk_direct(cg, D, nthreads=threads)
        times.append(time.time() - t)
    full = float(np.mean(times))
    value = 1.0 / full
    rec = {"metric": METRIC, "value": value, "unit": "Fock builds/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": full * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic", "impl": "reference",
           "config": dict(cfg_dict(mol, args.nwater, args.basis),
                          density="0.1 I (the reference's algorithm evaluates every unique AO quartet "
                                  "whatever the density)", l2="not flushed (CPU arm)"),
           "cpu_baseline": {"value": value, "unit": "Fock builds/s", "cores": threads, "kind": "port",
                            "sample": "each timed step: one whole Fock build, all %d unique AO quartets "
                                      "(warm-up steps: 1/40 of the pair rows)" % tot,
                            "step_s": [round(v, 3) for v in times],
                            "roots": "reference root5 (transcribed)" if use_ref else "oracle root table"},
           "e2e": {"value": value, "unit": "Fock builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(rec))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nwater", type=int, default=8)
    ap.add_argument("--basis", default="6-31g*")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nwater2", type=int, default=16, help="second cluster size reported beside (0: off)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--eri-quartets", type=int, default=1_000_000, help="raw-ERI stress batch size (0: off)")
    ap.add_argument("--no-alkane", dest="alkane", action="store_false", help="skip the C20H42 6-31G** block")
    ap.add_argument("--clocks-log", default=None,
                    help="CSV of the nvidia-smi clock samples taken during the timed region (default: a temporary file)")
    ap.add_argument("--tuning", default=None,
                    help="launch-shape table of the headline cluster: loaded when the file exists (no autotuning), "
                         "else written after autotuning")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
