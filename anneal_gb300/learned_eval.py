"""Trains the warm-start U-Net on GPU SIMP snapshots and measures what it gains.

    python -m anneal_gb300.learned_eval [--train-shape NX NY NZ] [--seeds S] [--iters I]
        [--epochs E] [--base B] [--eval-shape NX NY NZ ...] [--eval-iters N]

Training pairs come from SIMP histories of seeded cantilevers and L-brackets (the
learned-warm-start configuration; the default sizes are scaled down from 128x64x64 to keep
training to a few minutes with the direct-convolution kernels). Evaluation runs the SIMP
loop twice on unseen seeds, once with the previous iterate as the CG start (the reference's
choice, optimize.py:122) and once with the learned start, to the same relative residual
1e-6, and prints one JSON line: CG iterations and wall time per SIMP iteration for both,
the network's share of the time, and the training losses.
"""
import argparse
import json
import time

import numpy as np
import torch

from . import learned as LW
from . import optimize as OPT
from .fem import Grid


def run_loop(work, iters, warm=None):
    grid = Grid(work.shape, work.h, (0, 0, 0))
    old = OPT.EMIN
    OPT.EMIN = work.emin
    try:
        run = OPT.SimpRunner(grid, work.fill, work.active, work.frozen, work.fixed, work.loads, work.weights,
                             work.E0, work.nu, work.vf, iters=iters, r_mm=work.r_vox, p_final=3.0, move=0.2,
                             x0=np.full(work.nelem, work.vf), beta_max=0.0, rtol=1e-6, log=lambda *a: None,
                             warm_start=warm)
        times, cg, comp = [], [], []
        for _ in range(iters):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rec = run.step()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            cg.append(rec["cgIters"][0])
            comp.append(rec["compliance"][0])
        dropped = warm is not None and run.warm_start is None
        gains = list(run.ws_gain)
        ledger = [(round(a_, 5), round(b_, 5)) for a_, b_ in run.ws_ledger]
        run.close()
    finally:
        OPT.EMIN = old
    return {"ms": 1e3 * float(np.mean(times[1:])), "cg": float(np.mean(cg[1:])), "cg_list": cg,
            "compliance_last": comp[-1], "dropped": dropped, "gains": [round(g, 6) for g in gains],
            "saved_s_vs_predict_s": ledger}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-shape", type=int, nargs=3, default=[64, 32, 32])
    ap.add_argument("--seeds", type=int, default=12)
    ap.add_argument("--iters", type=int, default=12)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--base", type=int, default=16)
    ap.add_argument("--eval-shape", type=int, nargs=3, action="append")
    ap.add_argument("--eval-iters", type=int, default=10)
    a = ap.parse_args()
    shape = tuple(a.train_shape)
    t0 = time.time()
    samples = []
    for seed in range(a.seeds):
        w = LW.seeded_problem(seed, shape)
        snaps, fixed, free = LW.simp_snapshots(w, a.iters)
        for esc, u, F in snaps:
            x, mask, dims, _ = LW.node_features(shape, esc, w.E0, w.emin, 3.0, F, fixed, free)
            tgt, _ = LW.node_target(shape, u, dims)
            samples.append((x, tgt, mask, dims))
    t_data = time.time() - t0
    net = LW.UNet(base=a.base, levels=4, seed=0)
    t0 = time.time()
    hist = LW.train(samples, net, epochs=a.epochs, lr=1e-3, log=lambda *m: None)
    t_train = time.time() - t0
    out = {"train_shape": list(shape), "pairs": len(samples), "params": net.nparam, "epochs": a.epochs,
           "loss_first": hist[0], "loss_last": hist[-1], "data_s": t_data, "train_s": t_train, "eval": []}
    for es in (a.eval_shape or [list(shape), [2 * s for s in shape]]):
        es = tuple(es)
        for seed in (1001, 1002):
            w = LW.seeded_problem(seed, es)
            plain = run_loop(w, a.eval_iters)
            ws = LW.WarmStart(net, es, w.E0, w.emin, 3.0)
            # time of one prediction at this size
            esc = torch.full((w.nelem,), 0.3 ** 3, device="cuda")
            F = torch.zeros(w.ndof, dtype=torch.float64, device="cuda")
            m8 = torch.zeros(w.ndof, dtype=torch.uint8, device="cuda")
            ws.predict(esc, F, m8, m8)
            torch.cuda.synchronize()
            tp = time.perf_counter()
            for _ in range(3):
                ws.predict(esc, F, m8, m8)
            torch.cuda.synchronize()
            t_pred = (time.perf_counter() - tp) / 3
            learned = run_loop(w, a.eval_iters, warm=ws)
            out["eval"].append({"shape": list(es), "seed": seed, "plain": plain, "learned": learned,
                                "predict_ms": 1e3 * t_pred,
                                "cg_ratio": plain["cg"] / max(learned["cg"], 1e-9),
                                "time_ratio": plain["ms"] / max(learned["ms"], 1e-9)})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
