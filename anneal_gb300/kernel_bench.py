"""Microbenchmark of the matrix-free K u kernel on a clamped box.

    python -m anneal_gb300.kernel_bench [--shape NX NY NZ] [--reps R] [--fp64]
    python -m anneal_gb300.kernel_bench --export [--shape NX NY NZ] [--reps R]
    python -m anneal_gb300.kernel_bench --voxel [--shape NX NY NZ] [--reps R] [--subdiv N]
    python -m anneal_gb300.kernel_bench --simp [--scale S] [--reps R] [--six]

--export times the iso-surface export instead: zoom (x2), classify, scan, emit, 10 Taubin
steps and the component labels on a smooth synthetic density field.
--voxel times the voxeliser (s = 3) on a sphere of 20 * 4^subdiv triangles filling most of the
grid's short side (h = 1) plus a rotated box.
--simp runs R SIMP iterations of the L-bracket (scale S: 1 is 192x96x96, 4/3 the 256x128x128
bench workload; --six: the six-load-case variant) on the FP32 path and prints their wall times
and CG iterations (a driver for profiling the kernels of a SIMP step).

Prints one JSON line: milliseconds per launch (CUDA events, after warm-up), the
algorithmic bytes (24 per node + 4 per element: read u, write y, read the element
scale) and the achieved GB/s and FP32 TFLOP/s (210 flop per element in the modal form of the
element product, against 1152 for the dense 24 x 24 product).
"""
import argparse
import json

import numpy as np
import torch

from .context import Context, to_dev

# FP32 operations per element of the modal K u (transforms, modal stiffness, node sums)
MODAL_FLOPS = 210.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", type=int, nargs=3, default=[320, 160, 160])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--export", action="store_true")
    ap.add_argument("--voxel", action="store_true")
    ap.add_argument("--subdiv", type=int, default=6)
    ap.add_argument("--tc", action="store_true", help="the tensor-core K u kernel (FP32)")
    ap.add_argument("--simp", action="store_true")
    ap.add_argument("--scale", type=float, default=4.0 / 3.0)
    ap.add_argument("--six", action="store_true")
    a = ap.parse_args()
    if a.simp:
        return simp_bench(a.scale, a.reps, a.six)
    if a.tc:
        import os
        os.environ["ANL_TC"] = "1"
    if a.export:
        return export_bench(a.shape, a.reps)
    if a.voxel:
        return voxel_bench(a.shape, a.reps, a.subdiv)
    nx, ny, nz = a.shape
    ctx = Context((nx, ny, nz), 1.0, 0.3, fp64=a.fp64)
    ne, nn = ctx.ne, ctx.nn
    fixed = np.zeros(3 * nn, np.uint8)
    clamp = np.arange(0, nn, nx + 1)          # the nodes of the x = 0 face
    for c in range(3):
        fixed[3 * clamp + c] = 1
    ctx.set_domain(torch.ones(ne, dtype=torch.uint8, device="cuda"), to_dev(fixed, torch.uint8))
    g = torch.Generator(device="cuda").manual_seed(0)
    E = torch.rand(ne, device="cuda", generator=g, dtype=torch.float32) + 1e-3
    dt = torch.float64 if a.fp64 else torch.float32
    mask = ctx.free_mask().to(dt)
    u = torch.randn(ctx.ndof, device="cuda", generator=g, dtype=dt) * mask
    y = torch.empty_like(u)
    ctx.apply_K(E, u, y)
    ms = ctx.profile_apply(u, y, a.reps)
    alg = 24 * nn + 4 * ne
    print(json.dumps({"kernel": "K u (APPLY)" + (" tensor cores" if a.tc else ""), "shape": [nx, ny, nz],
                      "precision": "fp64" if a.fp64 else "fp32",
                      "ms_per_launch": ms, "algorithmic_bytes": alg, "GBps": alg / (ms * 1e-3) / 1e9,
                      "tflops": MODAL_FLOPS * ne / (ms * 1e-3) / 1e12}))
    ctx.close()


def export_bench(shape, reps):
    """Iso-surface export of a lattice-like field (0.5 + 0.5 sin sin sin, period 16 voxels)."""
    from . import export as X
    nx, ny, nz = shape
    i = torch.arange(nx, device="cuda", dtype=torch.float32)
    j = torch.arange(ny, device="cuda", dtype=torch.float32)
    k = torch.arange(nz, device="cuda", dtype=torch.float32)
    w = 2 * np.pi / 16
    f = 0.5 + 0.5 * (torch.sin(w * k)[:, None, None] * torch.sin(w * j)[None, :, None] * torch.sin(w * i)[None, None, :])
    f = f.reshape(-1).contiguous()
    mc = X.MarchingCubes()
    res = {}
    for phase in ("extract", "all"):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for r in range(reps + 2):
            if r == 2:
                e0.record()
            nv, nf = mc.extract(f, shape, 0.5, 1.0, (0.0, 0.0, 0.0), 2)
            if phase == "all":
                mc.smooth(10)
                mc.components()
        e1.record()
        e1.synchronize()
        res[phase] = e0.elapsed_time(e1) / reps
    mc.close()
    ns = (nx + 2) * (ny + 2) * (nz + 2) * 8
    print(json.dumps({"kernel": "iso-surface export", "shape": [nx, ny, nz], "upsample": 2, "samples": ns,
                      "vertices": nv, "faces": nf, "ms_extract": res["extract"], "ms_with_smooth_and_labels": res["all"],
                      "samples_per_s": ns / (res["extract"] * 1e-3)}))


def voxel_tris(shape, subdiv):
    """The voxeliser workload: a sphere (20 * 4^subdiv triangles) and a rotated box inside an
    nx x ny x nz grid of unit elements at the origin."""
    from . import geometry as G
    nx, ny, nz = shape
    r = 0.45 * min(shape)
    V, F = G.icosphere(subdiv, r, (0.3 * nx, 0.5 * ny, 0.5 * nz))
    rot = np.linalg.qr(np.random.default_rng(1).normal(size=(3, 3)))[0]
    Vb, Fb = G.box((0.3 * nx, 0.5 * ny, 0.3 * nz), (0.75 * nx, 0.5 * ny, 0.5 * nz), rot)
    return np.concatenate([V[F], Vb[Fb]])


def voxel_bench(shape, reps, subdiv):
    from . import geometry as G
    tri = torch.as_tensor(voxel_tris(shape, subdiv), device="cuda")
    vox = G.Voxeliser()
    vox.fill_device(tri, shape, 1.0, (0.0, 0.0, 0.0), stats=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for r in range(reps + 3):
        if r == 3:
            e0.record()
        f = vox.fill_device(tri, shape, 1.0, (0.0, 0.0, 0.0))
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    ne = int(np.prod(shape))
    print(json.dumps({"kernel": "voxeliser (s=3)", "shape": list(shape), "triangles": int(tri.shape[0]),
                      "pairs": vox.pairs, "crossings": vox.hits, "ms_per_call": ms,
                      "elements_per_s": ne / (ms * 1e-3), "fill_sum": float(f.sum())}))
    vox.close()


def simp_bench(scale, reps, six):
    import time
    from . import optimize as O, problems as P
    from .fem import Grid
    w = (P.six_case_bracket if six else P.lbracket)(scale=scale, vf=0.25, r_vox=2.0, emin=1e-9)
    O.EMIN = 1e-9
    run = O.SimpRunner(Grid(w.shape, 1.0, (0.0, 0.0, 0.0)), w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights,
                       w.E0, w.nu, w.vf, iters=max(reps, 1), r_mm=w.r_vox, x0=np.full(w.nelem, w.vf), beta_max=0.0,
                       log=lambda *a: None, precision="fp32")
    ms, cg = [], []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = run.step()
        torch.cuda.synchronize()
        ms.append(1e3 * (time.perf_counter() - t0))
        cg.append(h["cgIters"])
    print(json.dumps({"workload": f"{'sixcase' if six else 'lbracket'}-{w.shape[0]}x{w.shape[1]}x{w.shape[2]}",
                      "ms_per_iteration": ms, "cg_iters": cg}))
    run.close()


if __name__ == "__main__":
    main()
