"""SIMP topology optimisation with the interface of anneal's optimize.py (anneal 0.3.0).

``simp`` keeps the reference's signature, continuation schedule, OC update, history
records and per-iteration log line (optimize.py:50-180); ``Filter`` keeps the density
filter interface (optimize.py:24-47). Every array operation of the loop runs in the CUDA
library: the filter, projection, stiffness scale, solve, sensitivity, OC bisection and the
history statistics. Design fields stay on the device between iterations; the host sees
only scalars (compliances, the bisection's volumes, the history values).
"""
import time

import numpy as np
import torch

from .context import Context, to_dev
from .fem import FEM, FP32_RTOL_FLOOR

EMIN = 1e-6       # optimize.py:18
PNORM = 8.0       # optimize.py:19
ETA = 0.5         # optimize.py:20
BETA_MAX = 4.0    # optimize.py:21
CG_RTOL = 1e-6    # the tolerance simp gives every solve (optimize.py:122)


class Filter:
    """Cone-weight density filter on the active voxels (optimize.py:24-47)."""

    def __init__(self, grid, active, r_vox):
        self.g = grid
        self.act = np.flatnonzero(active)
        R = max(int(np.ceil(r_vox)) - 1, 1)
        ax = np.arange(-R, R + 1)
        X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
        self.k = np.maximum(0.0, r_vox - np.sqrt(X ** 2 + Y ** 2 + Z ** 2))
        self.ctx = Context(grid.shape, grid.h, 0.3)
        a = np.zeros(grid.nelem, np.uint8)
        a[self.act] = 1
        self.ctx.set_domain(to_dev(a, torch.uint8), torch.zeros(3 * grid.nnode, dtype=torch.uint8, device="cuda"))
        self.ctx.filter_init(r_vox)

    def _run(self, v_act, forward):
        full = np.zeros(self.g.nelem)
        full[self.act] = v_act
        out = torch.empty(self.g.nelem, dtype=torch.float32, device="cuda")
        (self.ctx.filter_fwd if forward else self.ctx.filter_bwd)(to_dev(full, torch.float32), out)
        return out.cpu().numpy().astype(float)[self.act]

    def forward(self, x_act):
        return self._run(x_act, True)

    def backward(self, d_act):
        return self._run(d_act, False)


def _continuation(it, iters, p_final, warm):
    """Penalty of iteration `it` (optimize.py:107-110)."""
    hold = max(1, min(3, int(0.4 * iters / max((p_final - 1.0) / 0.25, 1))))
    return p_final if warm else min(p_final, 1.0 + 0.25 * ((it - 1) // hold))


def simp(grid, fill, active, frozen, fixed, loads, weights, E0, nu, vf,
         iters=80, r_mm=None, p_final=3.0, move=0.2, combine="sum", log=print, tol=0.01, x0=None,
         beta_max=BETA_MAX, rtol=None, maxiter=2000):
    """optimize.py:50-180 on the GPU. ``rtol`` overrides the CG tolerance (default CG_RTOL,
    the reference's hard-coded 1e-6); the void stiffness is the module constant EMIN."""
    t_start = time.time()
    emin = EMIN
    rtol = CG_RTOL if rtol is None else float(rtol)
    fem = FEM(grid, active, fixed, nu, log=log)
    ctx = fem._ctx(fp64=False)
    act = fem.act
    ne = grid.nelem
    fill = np.asarray(fill, float)
    frozen = np.asarray(frozen, bool)
    phi = fill[act]
    frz = frozen[act]
    des = ~frz
    h = grid.h
    r_vox = max((r_mm or 1.5 * h) / h, 1.5)
    ctx.filter_init(r_vox)
    cases = list(loads)
    F_host = np.stack([np.where(fem._mask_t.cpu().numpy(), np.asarray(loads[c], float), 0.0) for c in cases])
    w = np.array([weights[c] for c in cases], float)
    if all(np.allclose(f[fem.free], 0) for f in F_host):
        raise ValueError("All loads are zero after mapping onto the grid. Check the load anchors' regions.")

    Vtot = phi.sum()
    Vtarget = vf * Vtot
    Vfrozen = phi[frz].sum()
    x = np.ones(act.size)
    x[des] = np.clip((Vtarget - Vfrozen) / max(phi[des].sum(), 1e-12), 0.01, 1.0)
    warm = x0 is not None
    if warm:
        xs = np.clip(np.asarray(x0, float)[act], 0.0, 1.0)
        cur = (phi[des] * xs[des]).sum()
        if cur > 0:
            x[des] = np.clip(xs[des] * (Vtarget - Vfrozen) / cur, 0.001, 1.0)

    def full(v_act):
        f = np.zeros(ne)
        f[act] = v_act
        return f

    f32 = torch.float32
    phi_t = to_dev(full(phi), f32)
    frz_t = to_dev(full(frz).astype(np.uint8), torch.uint8)
    x_t = to_dev(full(x), f32)
    xnew_t = torch.empty_like(x_t)
    xphys_t = torch.empty_like(x_t)
    dxp_t = torch.empty_like(x_t)
    escale_t = torch.empty_like(x_t)
    dc_t = torch.empty_like(x_t)
    dcx_t = torch.empty_like(x_t)
    dv_t = torch.empty_like(x_t)
    dvx_t = torch.empty_like(x_t)
    F_t = to_dev(F_host, torch.float64)
    U_t = torch.zeros_like(F_t)

    beta = 0.0
    hist = []
    c0 = None
    base_iters = None
    p = 1.0
    if warm:
        beta = beta_max / 2
    beta_step = max(5, int(0.12 * iters))
    beta_since = 0
    for it in range(1, iters + 1):
        t0 = time.time()
        p = _continuation(it, iters, p_final, warm)
        if p >= p_final and not warm and beta_max > 0:   # optimize.py:111-116
            if beta == 0:
                beta, beta_since = 1.0, 0
            elif beta_since >= beta_step and beta < beta_max:
                beta, beta_since = min(beta_max, 2 * beta), 0
            beta_since += 1
        ctx.physical(x_t, frz_t, beta, ETA, xphys_t, dxp_t)
        ctx.stiffness_scale(xphys_t, phi_t, E0, emin, p, escale_t)
        last = fem.cg_iters[-1] if fem.cg_iters else None
        rebuild = base_iters is None or (last is not None and last > 1.6 * base_iters)
        fem.solve_device(escale_t, F_t, U_t, rtol=rtol, maxiter=maxiter, rebuild=rebuild)
        if rebuild:
            base_iters = fem.cg_iters[-1]
        cs = np.array([ctx.dot(F_t[c], U_t[c]) for c in range(len(cases))])
        if c0 is None:
            c0 = cs.copy()
        if combine == "sum" or len(cases) == 1:
            obj = float(w @ cs)
            coef = w
        else:   # optimize.py:136-139
            r = w * cs / c0
            obj = float((r ** PNORM).sum() ** (1 / PNORM))
            coef = (r / obj) ** (PNORM - 1) * w / c0
        ctx.sensitivity(U_t, coef, xphys_t, dxp_t, phi_t, p, emin, E0, dc_t, dv_t)
        ctx.filter_bwd(dc_t, dcx_t)
        ctx.filter_bwd(dv_t, dvx_t)
        ctx.oc_update(x_t, dcx_t, dvx_t, phi_t, frz_t, move, beta, ETA, Vtarget, xnew_t)
        ctx.physical(xnew_t, frz_t, beta, ETA, xphys_t, None)
        change, grey, vol, ndes = ctx.design_stats(x_t, xnew_t, xphys_t, phi_t, frz_t)
        if ndes == 0:
            change, grey = 0.0, 0.0
        x_t, xnew_t = xnew_t, x_t
        hist.append({"iter": it, "objective": obj, "compliance": cs.tolist(), "p": p, "beta": beta,
                     "volumeFraction": float(vol / Vtot), "change": change,
                     "grey": grey, "cgIters": fem.cg_iters[-len(cases):], "amgRebuilt": bool(rebuild),
                     "seconds": time.time() - t0})
        log(f"  it {it:3d}  p {p:.2f}  b {beta:.0f}  obj {obj:.4g}  vol {hist[-1]['volumeFraction']:.3f}  "
            f"change {change:.3f}  grey {grey:.2f}  cg {fem.cg_iters[-1]}{' amg' if rebuild else ''}  "
            f"{hist[-1]['seconds']:.1f}s")
        if p >= p_final and beta >= beta_max and it > (5 if warm else 10) and change < tol:
            log(f"  converged at iteration {it}")
            break

    xout = np.zeros(ne)
    xout[act] = xphys_t.cpu().numpy().astype(float)[act]
    res = {"x": xout, "history": hist, "fem_builds": fem.amg_builds, "rMM": r_vox * h,
           "seconds": time.time() - t_start, "cases": cases}
    fem.close()
    return res


def benchmark_cantilever(log=lambda *a: None):
    """V6 (optimize.py:183-210): an optimised cantilever must beat a uniform design at
    equal mass and equal penalty."""
    from .fem import Grid
    g = Grid((32, 8, 12), 1.0, (0, 0, 0))
    fill = np.ones(g.nelem)
    active = np.ones(g.nelem, bool)
    frozen = np.zeros(g.nelem, bool)
    n = np.arange(g.nnode)
    pc = g.node_coords(n)
    clamp = n[pc[:, 0] < 1e-9]
    fixed = (3 * clamp[:, None] + np.arange(3)).ravel()
    tip = n[(abs(pc[:, 0] - 32) < 1e-9) & (abs(pc[:, 2] - 6) < 1e-9)]
    F = np.zeros(3 * g.nnode)
    F[3 * tip + 2] = -1.0 / tip.size
    vf = 0.3
    r = simp(g, fill, active, frozen, fixed, {"c": F}, {"c": 1.0}, 1000.0, 0.3, vf, iters=40, r_mm=1.6, log=log)
    fem = FEM(g, active, fixed, 0.3)
    Fr = fem.reduce_load(F)

    def comp(xp):
        u = fem.solve(fem.assemble(1000.0 * (EMIN + xp ** 3 * (1 - EMIN))), [Fr], rebuild=True)[0]
        return float(Fr @ u)
    c_opt = comp(r["x"])
    c_uni = comp(np.full(g.nelem, vf))
    fem.close()
    return {"stiffer_pct": 100 * (1 - c_opt / c_uni), "vol_err": r["history"][-1]["volumeFraction"] - vf}
