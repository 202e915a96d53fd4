"""SIMP iterations per second on the 256x128x128 L-bracket (12.8M DOF), one GB300.

A step is one SIMP iteration of the GPU loop (filter + projection, stiffness scale,
multigrid-preconditioned CG to relative residual 1e-6 warm-started from the previous
displacement, sensitivity, two filter backward passes, OC bisection, history values).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

After W warm-up steps, K device-timed steps (design resident in HBM) alternate with K
end-to-end steps (design copied host -> device before and device -> host after, inside the
timed region), so both numbers sample the same SIMP iterations. ``learned_vs_plain`` then
compares the first 5 SIMP iterations with the learned CG start and with the plain
previous-iterate start (the network trained in the run; ``--no-learned`` skips it).

N > 1 runs under torchrun with one independent replica per GPU (the solve has no
cross-GPU exchange): value = total iterations / max rank time. ``--impl reference`` times
the FP64 CPU oracle (the restatement of the reference's solver) on the host cores: W
untimed and K timed SIMP iterations, each a full iteration with its PCG run to 1e-6.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SIMP iters/s at 12.8M DOF; learned vs plain GPU PCG at rel. residual 1e-6"
UNIT = "iter/s"
SCALE = 4.0 / 3.0          # 256 x 128 x 128 voxels
RTOL = 1e-6


# FP32 operations per element of K u: the dense 24 x 24 product, and the modal form (forward
# transform from edge differences, the sparse modal stiffness times E, the inverse transform)
KU_DENSE_FLOPS = 2 * 24 * 24
KU_MODAL_FLOPS = 210

# finest-level solve passes: (profile id, name, launches per CG iteration, algorithmic bytes(N_n, N_e))
# K u reads u and E and writes y; the residual also reads b; the last Chebyshev step of a sweep
# reads x, b, the direction and the inverse diagonal and writes x (the first step of the
# post-smoothing reads x, b and the inverse diagonal and writes x and the direction); the fused
# first two steps read b and the inverse diagonal and write x
PASSES = [
    (1, "K u with u.Ku (CG q = K p)", 1, lambda nn, ne: 24 * nn + 4 * ne),
    (2, "residual b - K x", 1, lambda nn, ne: 36 * nn + 4 * ne),
    (3, "last Chebyshev step of a sweep", 1, lambda nn, ne: 52 * nn + 4 * ne),
    (5, "first Chebyshev step after the prolongation", 1, lambda nn, ne: 52 * nn + 4 * ne),
    (4, "first two Chebyshev steps", 1, lambda nn, ne: 28 * nn + 4 * ne),
    (0, "K u", 0, lambda nn, ne: 24 * nn + 4 * ne),
]


def workload_config():
    return {"workload": "lbracket-256x128x128", "dofs": 3 * 257 * 129 * 129, "elements": 256 * 128 * 128,
            "penalty": 3.0, "filter_r": 2.0, "vf": 0.25, "emin": 1e-9, "rtol": RTOL,
            "l2": "flushed (512 MB write) between timed steps"}


def make_workload():
    from anneal_gb300 import problems as P
    return P.lbracket(scale=SCALE, vf=0.25, r_vox=2.0, emin=1e-9)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of the SM clock during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""
        return False

    def summary(self):
        if self.proc is None:
            return None
        rows = []
        for line in getattr(self, "out", "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                rows.append((float(f[0]), float(f[1]), f[3:7]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": reasons}


# ------------------------------------------------------------------ CPU oracle

def oracle_run(w, iters):
    """The FP64 oracle's SIMP loop on the workload, set up (FEM, filter) but not stepped:
    each step() is one full iteration (filter, stiffness, multigrid set-up, PCG to RTOL from
    the previous displacement, sensitivity, two filter backward passes, OC bisection)."""
    from oracle import oracle as O
    O.build()
    return O.SimpRun(w.shape, w.h, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu, w.vf,
                     iters=iters, r_mm=w.r_vox, p_final=3.0, move=0.2, x0=np.full(w.nelem, w.vf), beta_max=0.0,
                     rtol=RTOL, emin=w.emin, log=lambda *a: None), O.num_threads()


def cpu_sample(w):
    """One full SIMP iteration of the FP64 oracle at full size (the first, from the initial
    design). Returns (seconds, CG iterations, threads, description)."""
    t_all = time.perf_counter()
    run, threads = oracle_run(w, 1)
    t0 = time.perf_counter()
    rec = run.step()
    t = time.perf_counter() - t0
    cg = rec["cgIters"][0]
    desc = (f"one full SIMP iteration (the first) of the FP64 oracle at 256x128x128: filter, stiffness, "
            f"multigrid set-up, PCG to rel. residual {RTOL:g} ({cg} CG iterations), sensitivity, 2 filter "
            f"backward passes, OC bisection; {t:.1f} s, {time.perf_counter() - t_all:.1f} s with set-up")
    return t, cg, threads, desc


# ------------------------------------------------------------------ arms

def run_reference(args):
    """The reference arm: the FP64 oracle's own SIMP loop on the host cores, W untimed
    iterations, then K timed ones (wall clock per iteration; each a full iteration)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    w = make_workload()
    run, threads = oracle_run(w, args.warmup + args.steps)
    for _ in range(args.warmup):
        run.step()
    times, cgs = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rec = run.step()
        times.append(time.perf_counter() - t0)
        cgs.append(rec["cgIters"][0])
    ttot = float(np.sum(times))
    value = args.steps / ttot
    desc = (f"SIMP iterations {args.warmup + 1}-{args.warmup + args.steps} of the FP64 oracle at 256x128x128, "
            f"each in full: PCG to rel. residual {RTOL:g} from the previous displacement "
            f"({np.mean(cgs):.1f} CG iterations per solve), filter, sensitivity, OC")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * ttot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(), "cg_iters_per_solve": float(np.mean(cgs)),
            "cg_start": "previous displacement (the reference's start)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def replica_rate(local_ms, steps, world, device):
    """Whole-job rate of `world` independent replicas that each ran `steps` steps in
    local_ms: the slowest rank's time (max over ranks) bounds the job. Returns (rate in
    steps/s, max ms)."""
    t = float(local_ms)
    if world > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([t], device=device, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return world * steps / (t / 1e3), t


def learned_vs_plain(w, iters=5):
    """The metric's second half: the first `iters` SIMP iterations of the workload from the same
    start, with the learned CG start (a U-Net trained here on GPU SIMP snapshots of seeded
    64x32x32 cantilevers and L-brackets, then combined with the previous iterate by the Galerkin
    step and dropped once it stops paying) against the plain previous-iterate start (the start of
    the timed steps), and the Galerkin combination of the last two displacements
    (cg_start="history") as a third arm. Each iteration is timed with CUDA events, prediction
    included."""
    import torch
    from anneal_gb300 import learned as LW
    from anneal_gb300 import optimize as OPT
    from anneal_gb300.fem import Grid

    t0 = time.time()
    shape = (64, 32, 32)
    samples = []
    for seed in range(12):
        pw = LW.seeded_problem(seed, shape)
        snaps, fixed, free = LW.simp_snapshots(pw, 12)
        for esc, u, F in snaps:
            x, mask, dims, _ = LW.node_features(shape, esc, pw.E0, pw.emin, 3.0, F, fixed, free)
            tgt, _ = LW.node_target(shape, u, dims)
            samples.append((x, tgt, mask, dims))
    net = LW.UNet(base=16, levels=4, seed=0)
    hist = LW.train(samples, net, epochs=8, lr=1e-3, log=lambda *m: None)
    t_train = time.time() - t0
    grid = Grid(w.shape, w.h, (0, 0, 0))
    OPT.EMIN = w.emin
    out = {"iterations": iters, "train": {"pairs": len(samples), "shape": list(shape), "epochs": 8,
                                          "params": net.nparam, "loss_first": hist[0], "loss_last": hist[-1],
                                          "seconds": t_train}}
    for arm in ("plain", "learned", "history"):
        ws = None
        if arm == "learned":  # its buffers allocated by one untimed prediction
            ws = LW.WarmStart(net, w.shape, w.E0, w.emin, 3.0)
            m8 = torch.zeros(w.ndof, dtype=torch.uint8, device="cuda")
            ws.predict(torch.full((w.nelem,), w.vf ** 3, device="cuda"),
                       torch.zeros(w.ndof, dtype=torch.float64, device="cuda"), m8, m8)
            torch.cuda.synchronize()
        run = OPT.SimpRunner(grid, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu, w.vf,
                             iters=10 ** 6, r_mm=w.r_vox, p_final=3.0, move=0.2, x0=np.full(w.nelem, w.vf),
                             beta_max=0.0, rtol=RTOL, log=lambda *a: None, warm_start=ws,
                             cg_start="history" if arm == "history" else "previous")
        ms, cg, used = [], [], []
        for _ in range(iters):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            active = run.warm_start is not None
            e0.record()
            rec = run.step()
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            cg.append(rec["cgIters"][0])
            used.append(active)
        out[arm] = {"ms_per_iteration": ms, "cg_iters": cg, "value": iters / (sum(ms) / 1e3), "unit": UNIT}
        if arm == "learned":
            out[arm]["network_used"] = used
            out[arm]["initial_error_gain"] = [round(g, 6) for g in run.ws_gain]
        run.close()
        del ws
        torch.cuda.empty_cache()
    out["time_ratio_plain_over_learned"] = sum(out["plain"]["ms_per_iteration"]) / sum(
        out["learned"]["ms_per_iteration"])
    out["time_ratio_plain_over_history"] = sum(out["plain"]["ms_per_iteration"]) / sum(
        out["history"]["ms_per_iteration"])
    return out


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from anneal_gb300 import _native as N
    from anneal_gb300 import optimize as OPT
    from anneal_gb300.fem import Grid

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = make_workload()
    grid = Grid(w.shape, w.h, (0, 0, 0))
    OPT.EMIN = w.emin
    run = OPT.SimpRunner(grid, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu, w.vf,
                         iters=10 ** 6, r_mm=w.r_vox, p_final=3.0, move=0.2, x0=np.full(w.nelem, w.vf),
                         beta_max=0.0, rtol=RTOL, log=lambda *a: None)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        run.step()
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    barrier()
    lib = N.load()
    # Device-timed steps and end-to-end steps alternate, so both sample the same stretch of
    # SIMP iterations (the CG count per solve drifts as the design develops). An end-to-end
    # step copies the current design into pinned host memory first (untimed), then times
    # host -> device, the step and device -> host.
    x_in = torch.empty(w.nelem, dtype=torch.float32).pin_memory()
    x_out = torch.empty_like(x_in).pin_memory()
    total_ms = e2e_ms = 0.0
    launches = 0
    cg_dev, cg_e2e = [], []
    solve_ev = []
    with ClockSampler(local) as clk:
        for s in range(2 * args.steps):
            device = s % 2 == 0
            if not device:
                x_in.copy_(run.x_t.cpu())
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            n0, c0 = lib.anl_launch_count(), len(run.fem.cg_iters)
            run.solve_events = solve_ev if device else None
            e0.record(stream)
            if device:
                run.step()
            else:
                run.step_host(x_in, x_out)
            e1.record(stream)
            e1.synchronize()
            if device:
                total_ms += e0.elapsed_time(e1)
                launches += lib.anl_launch_count() - n0
                cg_dev += run.fem.cg_iters[c0:]
            else:
                e2e_ms += e0.elapsed_time(e1)
                cg_e2e += run.fem.cg_iters[c0:]
    barrier()
    run.solve_events = None
    solve_ms = sum(a.elapsed_time(b) for a, b in solve_ev)
    cg_counts = cg_dev
    value, t_max = replica_rate(total_ms, args.steps, world, "cuda")
    e2e, e2e_ms = replica_rate(e2e_ms, args.steps, world, "cuda")

    # The finest level's K u passes, each launch timed alone with CUDA events on this stream
    # (the solver's own launch path and work vectors) right after a 512 MB L2 flush, with their
    # algorithmic bytes; `roofline` reports the one that takes the largest share of a CG
    # iteration. The back-to-back figure (20 launches, part of the working set left in L2 by the
    # launch before) is kept beside it as `ms_per_launch_warm`.
    ctx = run.ctx
    nn, ne = ctx.nn, ctx.ne
    peak, peak_kind = read_peaks()
    passes = []
    for pid, name, per_it, nbytes in PASSES:
        cold = []
        for _ in range(20):
            flush.zero_()
            cold.append(ctx.profile_pass(pid, 1))
        ms = float(np.median(cold))
        b = nbytes(nn, ne)
        passes.append({"pass": name, "launches_per_cg_iteration": per_it, "ms_per_launch": ms,
                       "ms_per_launch_warm": ctx.profile_pass(pid, 20),
                       "algorithmic_bytes": b, "GBps": b / (ms * 1e-3) / 1e9,
                       "frac": b / (ms * 1e-3) / 1e9 / peak})
    dom = max(passes, key=lambda q: q["ms_per_launch"] * q["launches_per_cg_iteration"])
    # K u in DOF/s and as a FLOP fraction: the dense-equivalent 1,152 flops per element (the
    # 24 x 24 Ke times u_e) and the ~210 FP32 operations the modal form executes, against the
    # FP32 CUDA-core peak (SMs x 128 lanes x 2 flops x the sampled SM clock)
    clocks = clk.summary()
    ku_ms = next(q["ms_per_launch"] for q in passes if q["pass"] == "K u")
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sms * 128 * 2 * ((clocks or {}).get("sm_mhz") or 2070.0) * 1e6 / 1e12
    ku_line = {"dofs_per_s": 3 * nn / (ku_ms * 1e-3), "ms_per_launch": ku_ms,
               "tflops_dense_equivalent": KU_DENSE_FLOPS * ne / (ku_ms * 1e-3) / 1e12,
               "tflops_executed": KU_MODAL_FLOPS * ne / (ku_ms * 1e-3) / 1e12,
               "fp32_peak_tflops": fp32_peak,
               "executed_frac": KU_MODAL_FLOPS * ne / (ku_ms * 1e-3) / 1e12 / fp32_peak}
    # PCG solves of the device-timed steps (CUDA events around each solve: set-up of the
    # hierarchy and the coarsest factor, the CG iterations, the accurate residuals)
    nsolve = len(solve_ev)
    pcg_line = {"solves_per_s": nsolve / (solve_ms / 1e3) if solve_ms > 0 else None,
                "ms_per_solve": solve_ms / nsolve if nsolve else None,
                "ms_per_cg_iteration": solve_ms / sum(cg_dev) if cg_dev else None,
                "share_of_step": solve_ms / total_ms if total_ms > 0 else None}
    traffic = None  # DRAM bytes come from an ncu capture (profiles/), never from this timed run
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (FP64 CG scalars and solution)",
                "data": "synthetic", "config": workload_config(), "parallelism": f"replicas x{world}",
                "cg_start": "previous displacement (the reference's start)",
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * w.nelem,
                        "d2h_bytes_per_step": 4 * w.nelem},
                "gpu_launches": int(launches),
                "cg_iters_per_solve": float(np.mean(cg_counts)) if cg_counts else None,
                "cg_iters_per_solve_e2e": float(np.mean(cg_e2e)) if cg_e2e else None,
                "roofline": {"kernel": f"fine-level {dom['pass']}", "bound": "hbm", "achieved": dom["GBps"],
                             "peak": peak, "unit": "GB/s", "frac": dom["frac"], "peak_kind": peak_kind,
                             "traffic": traffic, "algorithmic_bytes": dom["algorithmic_bytes"],
                             "ms_per_launch": dom["ms_per_launch"],
                             "timing": "one launch after a 512 MB L2 flush, median of 20"},
                "roofline_passes": passes,
                "ku": ku_line,
                "pcg": pcg_line,
                "ku_engine": "tensor cores (tcgen05, 3xTF32)" if os.environ.get("ANL_TC", "0") not in ("", "0")
                else "SIMT (modal FP32)",
                "clocks": clocks}
    run.close()
    if rank == 0:
        if world == 1 and not args.no_learned:
            line["learned_vs_plain"] = learned_vs_plain(w)
        if world == 1 and not args.no_cpu_baseline:
            t, cg, threads, desc = cpu_sample(w)
            line["cpu_baseline"] = {"value": 1.0 / t, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": desc, "cg_iters": cg}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-start comparison (training takes about 15 s)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
