"""Many independent SIMP parts on one GPU.

    python -m anneal_gb300.batch [--parts 32] [--iters 30] [--seed 0] [--lanes auto|N]

Runs a set of independent voxel SIMP problems (the many-part batching configuration: seeded
cantilevers with nx in [32, 128], ny, nz in [16, 64], volume fraction in [0.2, 0.4], filter
radius in [1.2, 2.5], p = 3, FP32 operator with FP64 CG scalars) as concurrent lanes. Each
lane is a host thread that owns one part at a time, its SIMP state and its own CUDA stream.
The library releases the GIL in every call, so the lanes' kernels overlap on the GPU. Small
parts are latency-bound (each kernel a few microseconds, one CG chunk a few hundred), and
overlapping them fills the 152 SMs that one part alone leaves idle. Parts are handed to lanes
largest first (longest-processing-time order), which balances the lanes.

The lane count is tuned: ``lanes="auto"`` times two SIMP iterations of the largest parts at a
few lane counts and keeps the fastest. The reference has no counterpart; it optimises one part
per process.
"""
import argparse
import concurrent.futures as cf
import json
import threading
import time

import numpy as np
import torch

from . import optimize as OPT
from . import problems as P
from .fem import Grid


def seeded_parts(n, seed=0):
    """The many-part set: cantilevers of seeded sizes, volume fractions and filter radii."""
    rng = np.random.default_rng(seed)
    parts = []
    for _ in range(n):
        nx = int(rng.integers(32, 129))
        ny = int(rng.integers(16, 65))
        nz = int(rng.integers(16, 65))
        vf = float(rng.uniform(0.2, 0.4))
        r = float(rng.uniform(1.2, 2.5))
        parts.append(P.cantilever(nx, ny, nz, vf=vf, r_vox=r, emin=1e-9))
    return parts


def _runner(w, iters):
    grid = Grid(w.shape, w.h, (0, 0, 0))
    return OPT.SimpRunner(grid, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu, w.vf,
                          iters=iters, r_mm=w.r_vox, p_final=3.0, move=0.2, x0=np.full(w.nelem, w.vf),
                          beta_max=0.0, rtol=1e-6, log=lambda *a: None)


def run_parts(parts, iters, lanes):
    """SIMP on every part, `lanes` at a time. Returns (seconds, per-part results)."""
    dev = torch.cuda.current_device()
    order = sorted(range(len(parts)), key=lambda i: -parts[i].nelem)
    queue = list(order)
    qlock = threading.Lock()
    results = [None] * len(parts)
    OPT.EMIN = 1e-9  # the parts share it (optimize.py:18 is a module constant)

    def lane(k):
        torch.cuda.set_device(dev)
        stream = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(stream):
            while True:
                with qlock:
                    if not queue:
                        return
                    i = queue.pop(0)
                run = _runner(parts[i], iters)
                cg = []
                for _ in range(iters):
                    rec = run.step()
                    cg.append(rec["cgIters"][0])
                stream.synchronize()
                results[i] = {"shape": list(parts[i].shape), "compliance": rec["compliance"][0],
                              "cg_mean": float(np.mean(cg)), "volume": rec["volumeFraction"]}
                run.close()

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if lanes == 1:
        lane(0)
    else:
        with cf.ThreadPoolExecutor(max_workers=lanes) as ex:
            list(ex.map(lane, range(lanes)))
    torch.cuda.synchronize()
    return time.perf_counter() - t0, results


def tune_lanes(parts, candidates=(1, 2, 4, 8)):
    """Lane count with the best throughput on two SIMP iterations of the largest parts."""
    probe = sorted(parts, key=lambda w: -w.nelem)[:max(candidates)]
    best, best_rate, rates = 1, 0.0, {}
    for n in candidates:
        t, _ = run_parts(probe, 2, n)
        rates[n] = len(probe) * 2 / t
        if rates[n] > best_rate:
            best, best_rate = n, rates[n]
    return best, rates


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--parts", type=int, default=32)
    ap.add_argument("--iters", type=int, default=30)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--lanes", default="auto")
    ap.add_argument("--compare", action="store_true", help="also time one lane (parts one after another)")
    a = ap.parse_args()
    parts = seeded_parts(a.parts, a.seed)
    tuned = None
    if a.lanes == "auto":
        lanes, tuned = tune_lanes(parts)
    else:
        lanes = int(a.lanes)
    t, res = run_parts(parts, a.iters, lanes)
    out = {"parts": a.parts, "iters": a.iters, "lanes": lanes, "seconds": t,
           "part_iters_per_s": a.parts * a.iters / t, "dofs_total": int(sum(w.ndof for w in parts)),
           "tuning_parts_per_s": tuned, "results": res[:4]}
    if a.compare:
        t1, _ = run_parts(parts, a.iters, 1)
        out["seconds_one_lane"] = t1
        out["speedup"] = t1 / t
    print(json.dumps(out))


if __name__ == "__main__":
    main()
