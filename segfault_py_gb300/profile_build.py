"""Per-launch device times of one Fock build (or two-electron gradient).

    python -m segfault_py_gb300.profile_build --nwater 8 --precision mixed --fp32-cutoff 1e-2

Builds the seeded water cluster (6-31G* by default), forms the core-Hamiltonian
guess density (the work of a build does not depend on the density values, only
on the Schwarz bounds) and runs `--builds` Fock builds.  With `--slices` the
library serialises its launches on one stream and times each with CUDA events;
the table lists, per launch (one class, precision and lanes-per-quartet
segment), the quartets, primitive quartets, device time, share of the build
and algorithmic GFLOP/s.  With `--timeline` the launches stay concurrent and
each one's start and end after the start of the build are listed, with the
number of launches in flight over time.  Without either it only runs the
builds (the command to put under a profiler).
"""
from __future__ import annotations

import argparse
import json

import torch

from . import geometry
from .fock import FockBuilder
from .molecule import Molecule
from .scf import preload_torch_linalg


def guess_density(fb: FockBuilder, nocc: int) -> torch.Tensor:
    S, T, V = fb.one_electron()
    w, U = torch.linalg.eigh(S)
    X = U @ torch.diag(w.rsqrt()) @ U.T
    _, Cp = torch.linalg.eigh(X @ (T + V) @ X)
    C = (X @ Cp)[:, :nocc]
    return 2.0 * C @ C.T


def slice_table(fb: FockBuilder):
    sl = fb.slice_info()
    tot = sum(q["ms"] for q in sl)
    rows = []
    for q in sorted(sl, key=lambda q: -q["ms"]):
        rows.append("(%d%d|%d%d) %s T=%2d q=%9d pq=%11d ms=%8.4f share=%5.1f%% GF/s=%8.1f" % (
            q["la"], q["lb"], q["lc"], q["ld"], ("f64", "f32", "dd")[q["precision"]],
            q["threads_per_quartet"], q["quartets"], q["prim_quartets"], q["ms"],
            100.0 * q["ms"] / max(tot, 1e-30), q["flop_alg"] / max(q["ms"], 1e-30) / 1e6))
    return tot, rows


def timeline_table(fb: FockBuilder, bin_ms: float = 0.05):
    sl = sorted(fb.slice_info(), key=lambda q: q["start_ms"])
    span = max(q["start_ms"] + q["ms"] for q in sl)
    busy = sum(q["ms"] for q in sl)
    rows = ["build span %.4f ms, launch time summed %.4f ms (mean launches in flight %.2f)" % (span, busy, busy / span)]
    for kind, name in ((0, "f64"), (1, "f32"), (2, "dd")):
        k = [q for q in sl if q["precision"] == kind]
        if k:
            rows.append("  %s: %d launches, first start %.4f ms, last end %.4f ms, summed %.4f ms" % (
                name, len(k), min(q["start_ms"] for q in k), max(q["start_ms"] + q["ms"] for q in k),
                sum(q["ms"] for q in k)))
    nb = int(span / bin_ms) + 1
    occ = []
    for b in range(nb):
        t0, t1 = b * bin_ms, (b + 1) * bin_ms
        occ.append(sum(max(0.0, min(t1, q["start_ms"] + q["ms"]) - max(t0, q["start_ms"])) for q in sl) / bin_ms)
    rows.append("launches in flight per %.3f ms bin: %s" % (bin_ms, " ".join("%.1f" % o for o in occ)))
    for q in sl:
        rows.append("start=%8.4f end=%8.4f stream=%2d (%d%d|%d%d) %s T=%2d q=%9d ms=%8.4f" % (
            q["start_ms"], q["start_ms"] + q["ms"], q["stream"], q["la"], q["lb"], q["lc"], q["ld"],
            ("f64", "f32", "dd")[q["precision"]], q["threads_per_quartet"], q["quartets"], q["ms"]))
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nwater", type=int, default=8)
    ap.add_argument("--basis", default="6-31g*")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "fp32", "mixed", "mixed_df", "df"])
    ap.add_argument("--cutoff", type=float, default=1e-12)
    ap.add_argument("--fp32-cutoff", type=float, default=1e-2)
    ap.add_argument("--builds", type=int, default=3)
    ap.add_argument("--slices", action="store_true")
    ap.add_argument("--timeline", action="store_true",
                    help="concurrent launches with start/end times (last build)")
    ap.add_argument("--time", action="store_true",
                    help="also time --builds normal (concurrent) builds (or gradients) with events")
    ap.add_argument("--autotune", action="store_true", help="autotune the launch shapes first")
    ap.add_argument("--launch", default="streams", choices=["streams", "persistent"],
                    help="launch mode of the Fock build (sf_set_launch_mode)")
    ap.add_argument("--ctas-per-sm", type=int, default=0, help="persistent grid: CTAs per SM (0: occupancy)")
    ap.add_argument("--density", default="grad", choices=["none", "grad", "fock", "both"],
                    help="density-weighted classification of the quartet lists (sf_set_density_screening)")
    ap.add_argument("--graph", action="store_true",
                    help="also time --builds replays of the build captured as a CUDA graph: torch.cuda.CUDAGraph "
                         "and the library's own capture with and without node priorities")
    ap.add_argument("--grad", action="store_true",
                    help="profile the two-electron gradient (sf_grad_jk) instead of the Fock build")
    ap.add_argument("--one-electron", action="store_true",
                    help="only the one-electron kernels: S, T, V (sf_one_electron) and their gradient "
                         "(sf_grad_one_electron), --builds times each")
    a = ap.parse_args(argv)
    preload_torch_linalg()
    sym, xyz = geometry.water_cluster(a.nwater)
    mol = Molecule.from_geometry(sym, xyz, a.basis)
    fb = FockBuilder(mol, cutoff=a.cutoff, fp32_cutoff=a.fp32_cutoff, precision=a.precision)
    D = guess_density(fb, mol.nelectron // 2)
    fb.set_density_screening(fock=a.density in ("fock", "both"), grad=a.density in ("grad", "both"))
    fb.set_launch_mode(a.launch, a.ctas_per_sm)
    if a.one_electron:
        from . import _lib
        from .fock import _ptr, _stream_ptr
        xyz, Z = mol.atom_table()
        xyz_d = torch.as_tensor(xyz, device=fb.device)
        Z_d = torch.as_tensor(Z, device=fb.device)
        g = torch.zeros(3 * mol.natom, dtype=torch.float64, device=fb.device)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        for _ in range(a.builds):
            fb.one_electron()
        ev[1].record()
        for _ in range(a.builds):
            _lib.check(_lib.lib().sf_grad_one_electron(fb.handle, _ptr(xyz_d), _ptr(Z_d), mol.natom, _ptr(D),
                                                       _ptr(D), _ptr(g), _stream_ptr()))
        ev[2].record()
        torch.cuda.synchronize()
        print("== one-electron nao=%d natom=%d: S,T,V %.4f ms, gradient %.4f ms (mean of %d)"
              % (fb.nao, mol.natom, ev[0].elapsed_time(ev[1]) / a.builds, ev[1].elapsed_time(ev[2]) / a.builds,
                 a.builds))
        return
    if a.autotune:
        tab = fb.autotune(D, reps=3)
        gain = sum(e["ms_default"] - e["ms_tuned"] for e in tab)
        print("autotuned %d launches, serialised time saved %.4f ms" % (len(tab), gain))
    if a.slices:
        fb.set_profiling(2)
    elif a.timeline:
        fb.set_profiling(1)
    if a.grad:
        from . import _lib
        from .fock import _ptr, _stream_ptr
        fb.jk(D, stats=True)   # work counters; the slice times below are the gradient's
        g = torch.zeros(3 * mol.natom, dtype=torch.float64, device=fb.device)
        for _ in range(a.builds):
            _lib.check(_lib.lib().sf_grad_jk(fb.handle, _ptr(D), _ptr(g), _lib.PRECISION[a.precision], a.cutoff,
                                             a.fp32_cutoff, _stream_ptr()))
    else:
        for _ in range(a.builds):
            fb.jk(D, stats=True)
    torch.cuda.synchronize()
    print("== %s nao=%d builds=%d stats %s" % (a.precision, fb.nao, a.builds, json.dumps(fb.last_stats)))
    if a.slices:
        tot, rows = slice_table(fb)
        print("serialised kernel time of one build: %.4f ms" % tot)
        print("\n".join(rows))
    if a.timeline and not a.slices:
        print("\n".join(timeline_table(fb)))
    if a.time and a.grad:
        from . import _lib
        from .fock import _ptr, _stream_ptr
        fb.set_profiling(0)
        g = torch.zeros(3 * mol.natom, dtype=torch.float64, device=fb.device)
        run = lambda: _lib.check(_lib.lib().sf_grad_jk(fb.handle, _ptr(D), _ptr(g), _lib.PRECISION[a.precision],
                                                       a.cutoff, a.fp32_cutoff, _stream_ptr()))
        for _ in range(3):
            run()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(a.builds):
            run()
        ev[1].record()
        torch.cuda.synchronize()
        print("wall time of one two-electron gradient (mean of %d back to back): %.4f ms"
              % (a.builds, ev[0].elapsed_time(ev[1]) / a.builds))
    if a.time and not a.grad:
        fb.set_profiling(0)
        J = torch.empty_like(D)
        K = torch.empty_like(D)
        for _ in range(3):
            fb.jk(D, out=(J, K))
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(a.builds):
            fb.jk(D, out=(J, K))
        ev[1].record()
        torch.cuda.synchronize()
        print("wall time of one build (mean of %d back to back): %.4f ms" % (a.builds, ev[0].elapsed_time(ev[1]) / a.builds))

    if a.graph and not a.grad:
        fb.set_profiling(0)
        J = torch.empty_like(D)
        K = torch.empty_like(D)
        for name, kw in (("torch.cuda.CUDAGraph", {}), ("library graph, node priorities", {"native": True}),
                         ("library graph, stream priority", {"native": True, "node_priority": False})):
            g = fb.capture_jk(D, J, K, **kw)
            for _ in range(3):
                g.replay()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            for _ in range(a.builds):
                g.replay()
            ev[1].record()
            torch.cuda.synchronize()
            print("graph replay (%s): %.4f ms per build (mean of %d)" % (name, ev[0].elapsed_time(ev[1]) / a.builds,
                                                                        a.builds))
            if hasattr(g, "close"):
                g.close()


if __name__ == "__main__":
    main()
