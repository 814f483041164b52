"""Times the multigrid kernels of one level with CUDA events.

    python -m curvib_old_gb300.kernel_timer [--cells 256x128x128] [--level -1] [--reps 20]
                                            [--grid channel|box] [KERNEL ...]

KERNEL is one of line_sweep_f32, line_sweep_f64 (a damped-Jacobi y-line sweep),
residual_f32, residual_f64, zebra_f32, zebra_f64 (one half-sweep of the zebra
smoother: residual on one color, then its line solves), vcycle_f32, vcycle_f64
(one V-cycle with the default options from the level down, replayed from a
CUDA graph; no byte count), contra2cart, ghost_nodes, convection
(Contra2Cart, GhostNodeVelocity and Convection; finest level only), viscous,
momentum_rhs (Viscous, and CalcRHS with FormFunction1's Convection and
pressure gradient; finest level only), imp_rk (one pseudo-time iteration of
ImpRK -- the boundary conditions and CalcRHS, then four Runge-Kutta stages --
on the box with a sphere of radius 0.25, an inlet on k = 0 and an outlet on
the last k face, Re 300, dt 2e-3, cfl 0.05, from a uniform stream; the call
is timed on the host, twice, the second inside the NVTX range); default: all
but imp_rk.  ``--grid channel`` (the
default) is the periodic channel (x and z periodic, tanh-stretched walls in y,
factor 2.5) at the given cell counts, whose operator is 7-point; ``--grid box``
is a walled box of the same cell counts (tanh 2.0 in y, nodes moved by sine
waves in x and z), so
every level keeps the 19-point operator with its cross-derivative terms.
Convection, viscous and momentum_rhs always run on the box: the momentum
right-hand side does not cover periodic faces.  Each kernel's
timed launches run inside an NVTX range named ``timed:<kernel>``, so a profiler
can be pointed at exactly those launches (``ncu --nvtx --nvtx-include
"timed:line_sweep_f32/"``) and skip the set-up autotuner's launches.  Prints one
JSON object per kernel: microseconds per launch, algorithmic bytes per launch
(every array the kernel needs, read or written once) and the GB/s they imply.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import workload as W
from ._lib import KERNELS
from .solver import PoissonContext


def _cells(text):
    parts = [int(v) for v in text.lower().split("x")]
    if len(parts) != 3 or min(parts) < 4:
        raise argparse.ArgumentTypeError("cells must look like 256x128x128")
    return tuple(parts)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("kernels", nargs="*", default=list(KERNELS))
    extra = {"imp_rk"}
    ap.add_argument("--cells", type=_cells, default=(256, 128, 128))
    ap.add_argument("--level", type=int, default=-1, help="multigrid level (0 coarsest, -1 finest)")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--grid", choices=["channel", "box"], default="channel")
    a = ap.parse_args(argv)
    for k in a.kernels:
        if k not in KERNELS and k not in extra:
            ap.error(f"unknown kernel {k!r}; choose from {sorted(set(KERNELS) | extra)}")
    import torch  # NVTX ranges only; the kernels themselves come from libcvb.so

    ctx = box = None
    on_box = {"convection", "viscous", "momentum_rhs"}
    for k in a.kernels:
        if k == "imp_rk":
            _imp_rk_iteration(a.cells, torch)
            continue
        if k in on_box or a.grid == "box":
            box = box or PoissonContext().setup(W.make_problem(a.cells, (1.0, 1.0, 1.0), 2.0, True,
                                                               (False, False, False), [], name="box"))
            c = box
        else:
            ctx = ctx or PoissonContext().setup(W.config1_problem(cells=a.cells))
            c = ctx
        torch.cuda.nvtx.range_push(f"timed:{k}")
        ms, nbytes = c.time_kernel(k, level=a.level, reps=a.reps)
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"kernel": k, "level": a.level % c.nlevels, "cells": int(np.prod(c.shapes[a.level])),
                          "us": round(ms * 1e3, 2), "bytes": int(nbytes),
                          "gbs": round(nbytes / (ms * 1e-3) / 1e9, 1)}))
    for c in (ctx, box):
        if c:
            c.close()


def _imp_rk_iteration(cells, torch):
    import time
    P = W.make_problem(cells, (1.0, 1.0, 1.0), 2.0, True, (False, False, False), [(0.5, 0.5, 0.5, 0.25)],
                       name="box-inout")
    P.bctype = [1, 1, 1, 1, 5, 4]
    c = PoissonContext().setup(P)
    sh = P.nvert.shape
    zet, nv = P.metrics[-1]["Zet"], P.nvert
    u0 = np.zeros(sh + (3,))
    fluid = (nv[:-1] < 0.1) & (nv[1:] < 0.1)
    u0[:-1, 1:-1, 1:-1, 2] = np.where(fluid[:, 1:-1, 1:-1], 2.0 * np.sqrt((zet[:-1, 1:-1, 1:-1] ** 2).sum(-1)), 0.0)
    z3, z1 = np.zeros(sh + (3,)), np.zeros(sh)
    for rep in range(2):
        if rep:
            torch.cuda.nvtx.range_push("timed:imp_rk")
        t0 = time.perf_counter()
        out = c.imp_rk(u0, u0, u0, z3, z1, z3, 300.0, 2e-3, 1.0, 0.05, 1, 0, 0, 1e-7, 1e-4, 1, 1, 0.0)
        ms = (time.perf_counter() - t0) * 1e3
        if rep:
            torch.cuda.nvtx.range_pop()
    print(json.dumps({"kernel": "imp_rk", "cells": int(np.prod(sh)), "ms_per_call": round(ms, 2),
                      "pseudo_iterations": out[3]["pseudo_iterations"], "stages": 5}))
    c.close()


if __name__ == "__main__":
    main()
