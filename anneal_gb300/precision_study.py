"""Precision study at 256x128x128 (12.8M DOF): the FP32 operator against FP64.

    python -m anneal_gb300.precision_study [--scale 1.3333] [--iters 30]

For each density field, the load case of the 256x128x128 L-bracket is solved twice:
- in FP32 (modal K u and smoothers in FP32, CG scalars and solution in FP64), to relative
  residual 1e-7, the floor this path certifies;
- with the FP64 operator to 1e-10. The FP64 operator is checked against the FP64 CPU oracle
  and the reference's own solves by the GPU tests.
It compares the compliance, max |u| and the design after one full OC step (sensitivity,
filter, bisection) from each solution.

The fields are the SIMP iterates 1, 10 and 30 of the FP32 loop, and the seeded random fields
rho = clip(0.3 exp(N(0, 1)), 1e-3, 1) for seeds 0 and 1. Prints one JSON line.
"""
import argparse
import json

import numpy as np
import torch

from . import optimize as OPT
from . import problems as P
from .fem import Grid

F32 = torch.float32


def one_case(run, xphys, rtol32=1e-7, rtol64=1e-10):
    """FP32 and FP64 solves of run's load on `xphys`, then one OC step from each."""
    ctx, fem = run.ctx, run.fem
    ctx.stiffness_scale(xphys, run.phi_t, run.E0, run.emin, 3.0, run.escale_t)
    out = {}
    U = {}
    for name, rtol in (("fp32", rtol32), ("fp64", rtol64)):
        X = torch.zeros_like(run.F_t)
        fem.solve_device(run.escale_t, run.F_t, X, rtol=rtol, maxiter=5000, rebuild=True)
        U[name] = X
        out[f"cg_{name}"] = fem.cg_iters[-1]
    c = {k: ctx.dot(run.F_t[0], U[k][0]) for k in U}
    umax = {k: float(U[k][0].abs().max()) for k in U}
    out["compliance_rel_err"] = abs(c["fp32"] / c["fp64"] - 1)
    out["max_u_rel_err"] = abs(umax["fp32"] / umax["fp64"] - 1)
    out["u_linf_rel_err"] = float((U["fp32"][0] - U["fp64"][0]).abs().max()) / umax["fp64"]
    # one OC step from each solution, from the same design
    xnew = {}
    for k in U:
        dc, dv, dcx, dvx = (torch.empty_like(xphys) for _ in range(4))
        ctx.sensitivity(U[k], [1.0], xphys, None, run.phi_t, 3.0, run.emin, run.E0, dc, dv)
        ctx.filter_bwd(dc, dcx)
        ctx.filter_bwd(dv, dvx)
        xn = torch.empty_like(xphys)
        ctx.oc_update(xphys, dcx, dvx, run.phi_t, run.frz_t, run.move, 0.0, 0.5, run.Vtarget, xn)
        xnew[k] = xn
    out["oc_density_linf"] = float((xnew["fp32"] - xnew["fp64"]).abs().max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=float, default=4.0 / 3.0)
    ap.add_argument("--iters", type=int, default=30)
    a = ap.parse_args()
    w = P.lbracket(scale=a.scale, vf=0.25, r_vox=2.0, emin=1e-9)
    grid = Grid(w.shape, w.h, (0, 0, 0))
    OPT.EMIN = w.emin
    run = OPT.SimpRunner(grid, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu, w.vf,
                         iters=a.iters, r_mm=w.r_vox, p_final=3.0, move=0.2, x0=np.full(w.nelem, w.vf),
                         beta_max=0.0, rtol=1e-6, log=lambda *m: None)
    fields = {}
    for it in range(1, a.iters + 1):
        run.ctx.physical(run.x_t, run.frz_t, 0.0, 0.5, run.xphys_t, None)
        if it in (1, 10, 30):
            fields[f"simp_iter_{it}"] = run.xphys_t.clone()
        run.step()
    act = torch.as_tensor(w.active, device="cuda")
    for seed in (0, 1):
        rho = P.random_density(w.shape, seed, w.active)
        fields[f"random_seed_{seed}"] = torch.as_tensor(rho, dtype=F32, device="cuda") * act
    res = {}
    for name, xp in fields.items():
        res[name] = one_case(run, xp)
    run.close()
    print(json.dumps({"workload": f"lbracket-{w.shape[0]}x{w.shape[1]}x{w.shape[2]}", "dofs": w.ndof,
                      "fp32_rtol": 1e-7, "fp64_rtol": 1e-10, "fields": res}))


if __name__ == "__main__":
    main()
