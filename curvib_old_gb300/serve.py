"""Served solve stream: a request loop with continuous batching on one GPU.

    python -m curvib_old_gb300.serve [--requests 200] [--load 0.8] [--budget-gb 150] [--max-cells 256]

Requests arrive as a Poisson process at a share (0.8) of the batched capacity
of this workload, measured first by queueing the whole stream at once.  Each
request is a pressure solve on a
[0,1]^3 box (tanh stretching 2.0 in y, sin distortion) of n^3 cells, with
n^3 log-uniform between 32^3 and max-cells^3 unknowns and n rounded to the
nearest multigrid-friendly size of SIZE_LADDER, 0-3 seeded spheres (one union
of immersed bodies: codes 1 and 3 only) and a noisy-divergence right-hand side.
30 % of the requests are follow-ups on one of the last few new problems: its
right-hand side
perturbed by 1 %, made compatible again, solved from the previous pressure
(warm start) while that problem is still resident.

The server keeps admitted problems resident on the device (metrics, multigrid
hierarchy, pressure).  A new problem takes an idle resident context of its
size (its operators rebuilt for the new bodies, cvb_set_nvert) or a new one,
evicting the least recently used idle context when the device memory of the
resident contexts would leave the HBM budget.  Every admitted solve goes to
one batch engine (cvb_batch_*): solves that arrive while others run join at
the next FGMRES iteration.  Latency runs from a request's arrival to its
pressure back in host memory; the report gives p50/p99 and solves/s.

The right-hand sides are the clients' input: they are computed before the
stream starts, so the clock measures the server only.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import time
from collections import OrderedDict

import numpy as np

from . import _lib
from . import workload as W
from .solver import PoissonContext, SolveBatch

# cells per direction a request is rounded to; each coarsens to a box of at
# most 600 cells
SIZE_LADDER = (32, 40, 48, 64, 80, 96, 128, 160, 192, 256)
DT, ST = 1e-3, 1.0
FOLLOWUP_SHARE = 0.3
PERTURB = 0.01
RECENT = 8        # follow-ups pick their problem among the last RECENT new ones


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float            # seconds after the stream starts
    n: int                    # cells per direction
    spheres: tuple            # ((cx, cy, cz, r), ...)
    seed: int
    base: int = -1            # follow-up of this request id (-1: a new problem)


def make_stream(count, rate, seed=4, max_cells=256):
    """`count` requests with Poisson arrivals at `rate` per second.  The draws
    do not depend on the rate, so streams of equal seed hold the same problems."""
    rng = np.random.default_rng(seed)
    ladder = [n for n in SIZE_LADDER if n <= max_cells]
    lo, hi = np.log(32.0 ** 3), np.log(float(max_cells) ** 3)
    t = 0.0
    out, news = [], []
    for rid in range(count):
        t += float(rng.exponential(1.0)) / rate
        if news and rng.uniform() < FOLLOWUP_SHARE:
            # a follow-up on one of the last few new problems (likely still resident)
            base = news[-1 - int(rng.integers(min(len(news), RECENT)))]
            out.append(Request(rid, t, out[base].n, out[base].spheres, int(rng.integers(1 << 30)), base))
            continue
        cells = float(np.exp(rng.uniform(lo, hi))) ** (1.0 / 3.0)
        n = min(ladder, key=lambda v: abs(np.log(v / cells)))
        k = int(rng.integers(0, 4))
        sph = tuple((float(a), float(b), float(c), float(r)) for a, b, c, r in
                    zip(rng.uniform(0.25, 0.75, k), rng.uniform(0.25, 0.75, k), rng.uniform(0.25, 0.75, k),
                        rng.uniform(0.08, 0.2, k)))
        out.append(Request(rid, t, n, sph, int(rng.integers(1 << 30))))
        news.append(rid)
    return out


def own_bytes_estimate(n):
    """Device bytes one n^3 problem holds alone: operators and vectors of every
    level and the FGMRES(30) basis (about 0.9 KB per finest cell)."""
    return int(0.9e3 * (n + 2) ** 3)


def geometry_bytes_estimate(n):
    """Device bytes of an n^3 grid's metrics, shared by its problems (~0.32 KB/cell)."""
    return int(0.32e3 * (n + 2) ** 3)


def bytes_estimate(n):
    """Device bytes of a lone n^3 problem: its own arrays and its grid's metrics."""
    return own_bytes_estimate(n) + geometry_bytes_estimate(n)


class Inputs:
    """The clients' data: box metrics per size, nvert and rhs per request."""

    def __init__(self, stream, device=0):
        self.geo = {}
        self.nvert = {}
        self.rhs = {}
        scratch = {}
        try:
            for req in stream:
                if req.n not in self.geo:
                    self.geo[req.n] = W.box_geometry((req.n, req.n, req.n))
                mets, uc = self.geo[req.n]
                aj = mets[-1]["Aj"]
                if req.base >= 0:
                    nv = self.nvert[req.base]
                    rng = np.random.default_rng(req.seed)
                    b = self.rhs[req.base] * (1.0 + PERTURB * rng.uniform(-1.0, 1.0, self.rhs[req.base].shape))
                    self.nvert[req.rid] = nv
                    self.rhs[req.rid] = W.compatible(b, aj, nv)
                    continue
                nv = W.sphere_nvert(mets[-1]["Cent"], list(req.spheres))
                if req.n not in scratch:
                    scratch[req.n] = PoissonContext(device).setup(self.problem(req.n, nv))
                else:
                    scratch[req.n].set_nvert(nv)
                ctx = scratch[req.n]
                ucc, _, _ = ctx.volume_flux_rev(uc, 0.0, 1)
                b, _ = ctx.poisson_rhs(ucc, DT, ST)
                self.nvert[req.rid] = nv
                self.rhs[req.rid] = W.noisy_rhs(b, nv, aj, DT, seed=req.seed)
        finally:
            for c in scratch.values():
                c.close()

    def problem(self, n, nv):
        mets, uc = self.geo[n]
        return W.Problem(mets, nv, uc, [1] * 6, (0, 0, 0), (False, False, False), f"box{n}")


class Server:
    """Request loop over one batch engine.  Contexts are prepared (operators
    rebuilt for a new problem's bodies, or a new context set up on its grid's
    resident metrics) on a worker thread while the main loop keeps the batch's
    rounds flowing; every piece of bookkeeping stays on the main thread."""

    def __init__(self, inputs, device=0, budget_bytes=150e9, precision=_lib.MIXED, rtol=1e-8, max_it=200,
                 restart=30, keep_results=False, workers=4):
        from concurrent.futures import ThreadPoolExecutor
        self.inp = inputs
        self.results = {} if keep_results else None
        self.trace = []             # (request id, warm start, request whose pressure was the initial guess)
        self.device = device
        self.budget = float(budget_bytes)
        self.batch = SolveBatch(device, precision=precision, rtol=rtol, max_it=max_it, restart=restart)
        self.ctxs = OrderedDict()   # context id -> dict(ctx, n, bytes, busy, owner, last): LRU order
        self.owner = {}             # problem (first request id) -> context id holding it
        self.holders = OrderedDict()  # grid size -> dict(ctx, bytes, ready future): resident metrics, LRU
        self.peak = 0
        self._next = 0
        self.pool = ThreadPoolExecutor(max_workers=workers)

    @property
    def used(self):
        return sum(c["bytes"] for c in self.ctxs.values()) + sum(h["bytes"] for h in self.holders.values())

    def close(self):
        self.pool.shutdown(wait=True)
        for c in self.ctxs.values():
            c["ctx"].close()
        for h in self.holders.values():
            h["ctx"].close()
        self.ctxs.clear()
        self.holders.clear()
        self.batch.close()

    def _evict_one(self, keep_n):
        """Free the least recently used idle context, else an unused grid's
        metrics; False when nothing can go."""
        for cid, c in self.ctxs.items():
            if not c["busy"]:
                self.ctxs.pop(cid)
                if c["owner"] is not None:
                    self.owner.pop(c["owner"], None)
                c["ctx"].close()
                return True
        for n, h in self.holders.items():
            if n != keep_n and h["ready"].done() and not any(c["n"] == n for c in self.ctxs.values()):
                self.holders.pop(n)
                h["ctx"].close()
                return True
        return False

    def _holder(self, n):
        h = self.holders.get(n)
        if h is None:
            ctx = PoissonContext(self.device)
            mets = self.inp.geo[n][0]
            P = W.Problem(mets, np.zeros(mets[-1]["Aj"].shape[:3]), None, [1] * 6)
            h = {"ctx": ctx, "bytes": geometry_bytes_estimate(n)}
            h["ready"] = self.pool.submit(ctx.setup_geometry, P)
            self.holders[n] = h
        self.holders.move_to_end(n)
        return h

    def _prepare(self, n, problem_id):
        """A context for a new problem: (context id, evictions, reused) or
        (None, evictions, False) while the budget has no room.  The context is
        busy until its preparation future completes."""
        nv = self.inp.nvert[problem_id]
        for cid, c in self.ctxs.items():
            if not c["busy"] and c["n"] == n:
                if c["owner"] is not None:
                    self.owner.pop(c["owner"], None)
                c.update(owner=problem_id, busy=True, last=None)
                c["ready"] = self.pool.submit(c["ctx"].set_nvert, nv)
                self.ctxs.move_to_end(cid)
                return cid, 0, True
        evicted = 0

        def need():
            return own_bytes_estimate(n) + (0 if n in self.holders else geometry_bytes_estimate(n))
        while self.used + need() > self.budget:
            if not self._evict_one(n):
                return None, evicted, False
            evicted += 1
        h = self._holder(n)
        ctx = PoissonContext(self.device)

        def job():
            h["ready"].result()
            ctx.setup_like(h["ctx"], nv)
        cid = self._next
        self._next += 1
        self.ctxs[cid] = {"ctx": ctx, "n": n, "bytes": own_bytes_estimate(n), "busy": True, "owner": problem_id,
                          "last": None, "ready": self.pool.submit(job)}
        self.peak = max(self.peak, self.used)
        return cid, evicted, False

    def run(self, stream, time_limit=600.0):
        """Serve `stream` (sorted by arrival); returns the statistics."""
        queue, inflight, preparing = [], {}, []
        lat, warm, cold_followups, evictions, reused = [], 0, 0, 0, 0
        prep = []  # set-up phases (ms) of every problem prepared for the stream
        spent = {"admit_s": 0.0, "step_s": 0.0, "result_s": 0.0, "rounds": 0}
        nxt = 0
        t0 = time.perf_counter()

        def submit(req, cid, ws):
            c = self.ctxs[cid]
            self.trace.append((req.rid, ws, c.get("last") if ws else None))
            c["last"] = req.rid
            t = self.batch.submit(c["ctx"], b=self.inp.rhs[req.rid], warm_start=ws)
            inflight[t] = (req, cid)

        while nxt < len(stream) or queue or inflight or preparing:
            now = time.perf_counter() - t0
            if now > time_limit:
                break
            ts = time.perf_counter()
            while nxt < len(stream) and stream[nxt].arrival <= now:
                queue.append(stream[nxt])
                nxt += 1
            still = []
            for req in queue:
                pid = req.base if req.base >= 0 else req.rid
                cid = self.owner.get(pid) if req.base >= 0 else None
                if cid is not None:
                    c = self.ctxs[cid]
                    if c["busy"]:
                        still.append(req)
                        continue
                    c["busy"] = True
                    self.ctxs.move_to_end(cid)
                    warm += 1
                    submit(req, cid, True)
                    continue
                cid, ev, was_reused = self._prepare(req.n, pid)
                evictions += ev
                if cid is None:
                    still.append(req)
                    continue
                reused += int(was_reused)
                self.owner[pid] = cid
                cold_followups += int(req.base >= 0)
                preparing.append((req, cid))
            queue = still
            left = []
            for req, cid in preparing:
                c = self.ctxs[cid]
                if c["ready"].done():
                    c["ready"].result()           # re-raise a failed preparation
                    prep.append(c["ctx"].setup_times())
                    c["bytes"] = max(c["ctx"].device_bytes(), own_bytes_estimate(c["n"]))
                    submit(req, cid, False)
                else:
                    left.append((req, cid))
            preparing = left
            spent["admit_s"] += time.perf_counter() - ts
            if inflight:
                ts = time.perf_counter()
                self.batch.step()
                spent["step_s"] += time.perf_counter() - ts
                spent["rounds"] += 1
                ts = time.perf_counter()
                for t, st in self.batch.poll():
                    req, cid = inflight.pop(t)
                    if st["status"] != 0:
                        raise RuntimeError(f"request {req.rid}: {st}")
                    c = self.ctxs[cid]
                    phi = self.batch.read_phi(c["ctx"])    # the result back to the client
                    if self.results is not None:
                        self.results[req.rid] = (phi, st)
                    c["busy"] = False
                    lat.append((time.perf_counter() - t0 - req.arrival) * 1e3)
                spent["result_s"] += time.perf_counter() - ts
            else:
                wait = 0.002 if preparing else (stream[nxt].arrival - (time.perf_counter() - t0)
                                                 if nxt < len(stream) else 0.002)
                time.sleep(max(0.0, min(0.005, wait)))
        wall = time.perf_counter() - t0
        return {"requests": len(stream), "served": len(lat), "wall_s": wall,
                "solves_per_s": len(lat) / wall if wall > 0 else 0.0,
                "p50_ms": float(np.percentile(lat, 50)) if lat else None,
                "p99_ms": float(np.percentile(lat, 99)) if lat else None,
                "warm_followups": warm, "cold_followups": cold_followups, "contexts_reused": reused,
                "evictions": evictions, "peak_resident_bytes": int(self.peak), "budget_bytes": int(self.budget),
                "loop": spent,
                "setup_ms_mean": {k: float(np.mean([q[k] for q in prep])) for k in prep[0]} if prep else None,
                "setups": len(prep)}


def capacity(inputs, stream, device=0, precision=_lib.MIXED, rtol=1e-8, budget_bytes=150e9):
    """Batched solves/s of the new problems of `stream` (as many as the HBM
    budget holds), all solved at once."""
    reqs, need = [], 0
    for r in stream:
        if r.base < 0 and need + bytes_estimate(r.n) <= budget_bytes:
            reqs.append(r)
            need += bytes_estimate(r.n)   # (no metrics sharing here: an upper bound)
    ctxs = []
    B = SolveBatch(device, precision=precision, rtol=rtol, max_it=200)
    try:
        for req in reqs:
            c = PoissonContext(device).setup(inputs.problem(req.n, inputs.nvert[req.rid]))
            c.set_rhs(inputs.rhs[req.rid])
            ctxs.append(c)
        B.solve(ctxs)
        for c, req in zip(ctxs, reqs):
            c.set_rhs(inputs.rhs[req.rid])
        t0 = time.perf_counter()
        B.solve(ctxs)
        wall = time.perf_counter() - t0
    finally:
        B.close()
        for c in ctxs:
            c.close()
    return len(ctxs) / wall


def serve(requests=200, load=0.8, budget_gb=150.0, max_cells=256, precision=_lib.MIXED, device=0,
          time_limit=600.0, probe=24, inputs=None, results=None):
    """Measure the batched capacity of the served workload -- the whole stream
    queued at once, set-ups included -- then serve the stream with Poisson
    arrivals at `load` times that rate.  Returns the report, with the solve-only
    batched capacity of the stream's first problems beside it.  `inputs`: the
    prepared Inputs of make_stream(requests, 1.0, 4, max_cells), to reuse.
    `results`: a dict to fill with request id -> (pressure, statistics) of the
    paced run."""
    proto = make_stream(requests, 1.0, seed=4, max_cells=max_cells)
    t0 = time.perf_counter()
    if inputs is None:
        inputs = Inputs(proto, device)
    prep = time.perf_counter() - t0
    solve_cap = capacity(inputs, proto[:probe], device, precision, budget_bytes=budget_gb * 1e9)
    saturated = [dataclasses.replace(r, arrival=0.0) for r in proto]
    srv = Server(inputs, device, budget_gb * 1e9, precision)
    try:
        sat = srv.run(saturated, time_limit)
    finally:
        srv.close()
    cap = sat["solves_per_s"]
    rate = load * cap
    stream = [dataclasses.replace(r, arrival=r.arrival / rate) for r in proto]
    srv = Server(inputs, device, budget_gb * 1e9, precision, keep_results=results is not None)
    try:
        out = srv.run(stream, time_limit)
        if results is not None:
            results.update(srv.results)
    finally:
        srv.close()
    sizes = [r.n for r in stream]
    out.update({"capacity_solves_per_s": cap,
                "capacity_sample": "the whole stream queued at once (set-ups, evictions and solves)",
                "solve_only_capacity_solves_per_s": solve_cap,
                "solve_only_capacity_sample": f"the first {probe} requests' new problems, resident, in one batch",
                "arrival_rate_per_s": rate, "load": load, "max_cells": max_cells,
                "size_mix": {str(n): sizes.count(n) for n in sorted(set(sizes))},
                "inputs_prepared_s": prep})
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description="served solve stream on one GPU")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--load", type=float, default=0.8, help="arrival rate as a share of batched capacity")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--max-cells", type=int, default=256)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--time-limit", type=float, default=600.0)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    out = serve(a.requests, a.load, a.budget_gb, a.max_cells, _lib.MIXED if a.precision == "mixed" else _lib.FP64,
                a.device, a.time_limit)
    out["precision"] = a.precision
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
