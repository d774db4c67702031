"""Time raw-ERI batches (the random stress batch over all 21 classes).

    python -m segfault_py_gb300.profile_eri --quartets 1000000 --precision fp32 --engine rys

Builds `--quartets` random contracted shell quartets (class uniform over
ss|ss .. dd|dd, contraction 1-6, exponents log-uniform in [0.05, 1e4], centres
in a 10 A box, seed 0), prepares one plan and runs it `--runs` times after one
warm-up, timing each run with CUDA events.  Engines: "rys" (production
kernels; fp64, fp32, df) and "md" (McMurchie-Davidson: fp64 on the CUDA cores,
fp32 with the bra E contraction on the tensor cores).
"""
from __future__ import annotations

import argparse

import torch

from . import geometry
from .fock import FockBuilder


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--quartets", type=int, default=1_000_000)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32", "df"])
    ap.add_argument("--engine", default="rys", choices=["rys", "md"])
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    table, q = geometry.random_quartet_batch(a.quartets, seed=a.seed)
    fb = FockBuilder(table)
    plan = fb.eri_plan(q)
    out = torch.empty(plan.outputs, dtype=torch.float64, device=fb.device)
    plan.run(a.precision, out, engine=a.engine)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(a.runs):
        plan.run(a.precision, out, engine=a.engine)
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / a.runs
    print("%s %s: %d quartets, %d primitive quartets, %.3f ms per batch, %.4g quartets/s, %.4g TFLOP/s (alg)"
          % (a.engine, a.precision, a.quartets, plan.prim_quartets, ms, a.quartets / (ms * 1e-3),
             plan.flop_alg / (ms * 1e-3) / 1e12))
    plan.close()
    fb.close()


if __name__ == "__main__":
    main()
