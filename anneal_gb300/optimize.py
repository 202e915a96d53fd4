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
from .fem import FEM

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


def galerkin_coefficients(g11, g12, g22, r1, r2):
    """(a, b) minimising the energy x.Kx/2 - F.x of x = a u1 + b d over the two directions, from
    g11 = u1.Ku1, g12 = u1.Kd, g22 = d.Kd, r1 = F.u1 and r2 = F.d; None where the start should
    stay u1: a non-finite or degenerate matrix (d too small or too close to u1's direction
    for FP32 entries to resolve), or a combination whose energy is not below u1's."""
    if not all(np.isfinite(v) for v in (g11, g12, g22, r1, r2)) or not (g11 > 0 and g22 > 1e-12 * g11):
        return None
    det = g11 * g22 - g12 * g12
    if not det > 1e-4 * g11 * g22:  # the FP32 entries resolve the two directions
        return None
    a, b = (r1 * g22 - r2 * g12) / det, (g11 * r2 - g12 * r1) / det
    # Pi(x0) = -(a r1 + b r2) / 2 against Pi(u1) = g11 / 2 - r1
    if not (np.isfinite(a) and np.isfinite(b) and -0.5 * (a * r1 + b * r2) <= 0.5 * g11 - r1):
        return None
    return a, b


class SimpRunner:
    """The device-resident state of one SIMP run and one ``step()`` per iteration.

    ``simp`` drives it for the reference's interface; benchmarks and services that step
    the loop themselves use it directly (``step_host`` exchanges the design with pinned
    host memory around a step)."""

    def __init__(self, grid, fill, active, frozen, fixed, loads, weights, E0, nu, vf, iters=80, r_mm=None,
                 p_final=3.0, move=0.2, combine="sum", log=print, x0=None, beta_max=BETA_MAX, rtol=None,
                 maxiter=2000, warm_start=None, precision="auto", multi="batch", cg_start="previous"):
        if cg_start not in ("history", "previous"):
            raise ValueError(f"cg_start must be 'history' or 'previous', not {cg_start!r}")
        self.grid = grid
        self.cg_start = cg_start
        self.E0, self.vf, self.iters, self.p_final, self.move = float(E0), float(vf), int(iters), p_final, move
        self.combine, self.log, self.beta_max, self.maxiter = combine, log, beta_max, maxiter
        self.emin = EMIN
        self.rtol = CG_RTOL if rtol is None else float(rtol)
        self.fem = fem = FEM(grid, active, fixed, nu, log=log, precision=precision, multi=multi)
        self.ctx = ctx = fem._ctx(fp64=False)
        act = self.act = fem.act
        ne = grid.nelem
        fill = np.asarray(fill, float)
        frozen = np.asarray(frozen, bool)
        phi = fill[act]
        frz = frozen[act]
        des = ~frz
        self.r_vox = max((r_mm or 1.5 * grid.h) / grid.h, 1.5)
        ctx.filter_init(self.r_vox)
        self.cases = list(loads)
        mask = fem._mask_t.cpu().numpy()
        F_host = np.stack([np.where(mask, np.asarray(loads[c], float), 0.0) for c in self.cases])
        self.w = np.array([weights[c] for c in self.cases], float)
        if all(np.allclose(f[fem.free], 0) for f in F_host):
            raise ValueError("All loads are zero after mapping onto the grid. Check the load anchors' regions.")
        # optimize.py:67-77
        self.Vtot = phi.sum()
        self.Vtarget = vf * self.Vtot
        Vfrozen = phi[frz].sum()
        x = np.ones(act.size)
        x[des] = np.clip((self.Vtarget - Vfrozen) / max(phi[des].sum(), 1e-12), 0.01, 1.0)
        self.warm = x0 is not None
        if self.warm:
            xs = np.clip(np.asarray(x0, float)[act], 0.0, 1.0)
            cur = (phi[des] * xs[des]).sum()
            if cur > 0:
                x[des] = np.clip(xs[des] * (self.Vtarget - Vfrozen) / cur, 0.001, 1.0)

        def full(v_act):
            f = np.zeros(ne)
            f[act] = v_act
            return f

        f32 = torch.float32
        self.phi_t = to_dev(full(phi), f32)
        self.frz_t = to_dev(full(frz).astype(np.uint8), torch.uint8)
        self.x_t = to_dev(full(x), f32)
        self.xnew_t = torch.empty_like(self.x_t)
        self.xphys_t = torch.empty_like(self.x_t)
        self.dxp_t = torch.empty_like(self.x_t)
        self.escale_t = torch.empty_like(self.x_t)
        self.dc_t = torch.empty_like(self.x_t)
        self.dcx_t = torch.empty_like(self.x_t)
        self.dv_t = torch.empty_like(self.x_t)
        self.dvx_t = torch.empty_like(self.x_t)
        self.F_t = to_dev(F_host, torch.float64)
        self.U_t = torch.zeros_like(self.F_t)
        self._U_prev = None     # the solutions of the solve before the last (cg_start "history")
        # a list makes step() record a pair of CUDA events around each solve into it
        self.solve_events = None
        self.beta = beta_max / 2 if self.warm else 0.0
        self.beta_step = max(5, int(0.12 * iters))
        self.beta_since = 0
        self.c0 = None
        self.base_iters = None
        self.it = 0
        self.hist = []
        self.p = 1.0
        # optional learned start (anneal_gb300.learned.WarmStart); dropped once its Galerkin
        # combination stops lowering the energy of the previous iterate
        self.warm_start = warm_start
        self.ws_gain = []
        self.ws_ledger = []
        if warm_start is not None:
            fx = torch.zeros(3 * grid.nnode, dtype=torch.uint8, device="cuda")
            fx[torch.as_tensor(np.asarray(fixed, np.int64), device="cuda")] = 1
            self._ws_fixed = fx
            self._ws_free = fem._mask_t.to(torch.uint8)

    def step(self):
        """One SIMP iteration (optimize.py:105-172); returns its history record."""
        t0 = time.time()
        ctx, fem = self.ctx, self.fem
        self.it += 1
        it = self.it
        p, beta = self._advance_continuation(it)
        ctx.physical(self.x_t, self.frz_t, beta, ETA, self.xphys_t, self.dxp_t)
        ctx.stiffness_scale(self.xphys_t, self.phi_t, self.E0, self.emin, p, self.escale_t)
        last = fem.cg_iters[-1] if fem.cg_iters else None
        rebuild = self.base_iters is None or (last is not None and last > 1.6 * self.base_iters)
        ws = self._learned_start() if self.warm_start is not None else None
        if ws is not None:
            self._U_prev = None  # the history restarts once the network is dropped
        elif self.cg_start == "history" and it > 1:
            self._history_start()
        t_solve = time.perf_counter()
        if self.solve_events is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record()
        fem.solve_device(self.escale_t, self.F_t, self.U_t, rtol=self.rtol, maxiter=self.maxiter, rebuild=rebuild)
        if self.solve_events is not None:
            ev[1].record()
            self.solve_events.append(ev)
        if ws is not None:
            self._assess_learned_start(ws, time.perf_counter() - t_solve)
        if rebuild:
            self.base_iters = fem.cg_iters[-1]
        nc = len(self.cases)
        cs = np.array([ctx.dot(self.F_t[c], self.U_t[c]) for c in range(nc)])
        if self.c0 is None:
            self.c0 = cs.copy()
        if self.combine == "sum" or nc == 1:
            obj = float(self.w @ cs)
            coef = self.w
        else:   # optimize.py:136-139
            r = self.w * cs / self.c0
            obj = float((r ** PNORM).sum() ** (1 / PNORM))
            coef = (r / obj) ** (PNORM - 1) * self.w / self.c0
        ctx.sensitivity(self.U_t, coef, self.xphys_t, self.dxp_t, self.phi_t, p, self.emin, self.E0, self.dc_t,
                        self.dv_t)
        ctx.filter_bwd(self.dc_t, self.dcx_t)
        ctx.filter_bwd(self.dv_t, self.dvx_t)
        ctx.oc_update(self.x_t, self.dcx_t, self.dvx_t, self.phi_t, self.frz_t, self.move, beta, ETA, self.Vtarget,
                      self.xnew_t)
        ctx.physical(self.xnew_t, self.frz_t, beta, ETA, self.xphys_t, None)
        change, grey, vol, ndes = ctx.design_stats(self.x_t, self.xnew_t, self.xphys_t, self.phi_t, self.frz_t)
        if ndes == 0:
            change, grey = 0.0, 0.0
        self.x_t, self.xnew_t = self.xnew_t, self.x_t
        rec = {"iter": it, "objective": obj, "compliance": cs.tolist(), "p": p, "beta": beta,
               "volumeFraction": float(vol / self.Vtot), "change": change, "grey": grey,
               "cgIters": fem.cg_iters[-nc:], "amgRebuilt": bool(rebuild), "seconds": time.time() - t0}
        self.hist.append(rec)
        self.log(f"  it {it:3d}  p {p:.2f}  b {beta:.0f}  obj {obj:.4g}  vol {rec['volumeFraction']:.3f}  "
                 f"change {change:.3f}  grey {grey:.2f}  cg {fem.cg_iters[-1]}{' amg' if rebuild else ''}  "
                 f"{rec['seconds']:.1f}s")
        return rec

    def _advance_continuation(self, it):
        """Penalty and projection sharpness of iteration `it` (optimize.py:105-116): p from the
        ramp, beta from 1 once p is final, doubled every beta_step iterations up to beta_max.
        Advances the beta state; returns (p, beta)."""
        p = self.p = _continuation(it, self.iters, self.p_final, self.warm)
        if p >= self.p_final and not self.warm and self.beta_max > 0:   # optimize.py:111-116
            if self.beta == 0:
                self.beta, self.beta_since = 1.0, 0
            elif self.beta_since >= self.beta_step and self.beta < self.beta_max:
                self.beta, self.beta_since = min(self.beta_max, 2 * self.beta), 0
            self.beta_since += 1
        return p, self.beta

    def _history_start(self):
        """CG start from the last two solutions. The reference starts each solve from the
        previous solution u1 (optimize.py:122); here the start is the energy-optimal
        combination x0 = a u1 + b d, d = u1 - u2 (u2 the solution before), under the new
        stiffness: [u1.Ku1 u1.Kd; d.Ku1 d.Kd] [a b] = [F.u1 F.d]. The loads do not change, so
        F.u1 and F.u2 are the last two compliances; the 2x2 matrix takes two FP32 K u and three
        FP32 dot products (the start only has to be close: every solve still runs to the same
        relative residual). Its energy x0.Kx0/2 - F.x0 is never above that of u1, so the start
        is at least as close to the solution in the energy norm. On the 256x128x128 L-bracket it
        saves 2-3 CG iterations a solve while the design moves fast (SIMP iterations 3-5) and
        about 0.5 later, where its set-up (about 0.4 ms) costs as much as it saves; hence
        opt-in (cg_start="history"). The first call only keeps the previous solutions."""
        n_keep = len(self.hist)
        if self._U_prev is None or n_keep < 2:
            if self._U_prev is None:
                self._U_prev = torch.empty_like(self.U_t)
                n = self.U_t.shape[1]
                self._hs = [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(4)]
            self._U_prev.copy_(self.U_t)
            self._U_prev_it = self.it - 1
            return
        if self._U_prev_it != self.it - 2:  # the kept solutions are not the last two
            self._U_prev.copy_(self.U_t)
            self._U_prev_it = self.it - 1
            return
        U1, U2 = self.U_t, self._U_prev
        f1, f2, k1, k2 = self._hs
        nc = len(self.cases)
        c1 = self.hist[-1]["compliance"]
        c2 = self.hist[-2]["compliance"]
        vals = torch.empty((nc, 3), dtype=torch.float32, device="cuda")
        for c in range(nc):
            f1.copy_(U1[c])
            f2.copy_(U2[c])
            torch.sub(f1, f2, out=f2)
            self.ctx.apply_K(self.escale_t, f1, k1)
            self.ctx.apply_K(self.escale_t, f2, k2)
            vals[c, 0] = torch.dot(f1, k1)
            vals[c, 1] = torch.dot(f1, k2)
            vals[c, 2] = torch.dot(f2, k2)
        v = vals.cpu().numpy().astype(np.float64)
        for c in range(nc):
            g11, g12, g22 = v[c]
            coef = galerkin_coefficients(g11, g12, g22, float(c1[c]), float(c1[c]) - float(c2[c]))
            if coef is None:
                U2[c].copy_(U1[c])
            else:   # x0 = (a + b) u1 - b u2, into the older solution's storage
                U2[c].mul_(-coef[1]).add_(U1[c], alpha=coef[0] + coef[1])
        self.U_t, self._U_prev = U2, U1
        self._U_prev_it = self.it - 1

    def _learned_start(self):
        """Replaces each case's start by the energy-optimal combination of the previous
        iterate and the network's prediction (anneal_gb300.learned.galerkin_start). Returns
        what the assessment after the solve needs."""
        from . import learned as LW
        ctx = self.ctx
        free = self._ws_free.double()
        t0 = time.perf_counter()
        info = []
        for c in range(len(self.cases)):
            F = self.F_t[c]
            u_prev = self.U_t[c].clone()
            u_net = self.warm_start.predict(self.escale_t, F, self._ws_fixed, self._ws_free)
            x0, a, b, gain = LW.galerkin_start(ctx, self.escale_t, F, u_prev, u_net, free, with_gain=True)
            info.append((LW.energy(ctx, self.escale_t, F, u_prev), LW.energy(ctx, self.escale_t, F, x0)))
            self.U_t[c].copy_(x0)
            self.ws_gain.append(gain)
        torch.cuda.synchronize()
        return info, time.perf_counter() - t0

    def _assess_learned_start(self, ws, t_solve):
        """After the solve, Pi(u) = u.Ku/2 - F.u of the solution gives the initial energy
        errors of both starts (Pi(x) - Pi(u*) = |x - u*|_K^2 / 2). CG needs iterations in
        proportion to log(initial / final energy error), the final one being about
        rtol^2 |Pi(u*)|, so the previous iterate would have needed about
        it * log(e_prev / e_fin) / log(e_new / e_fin) iterations. The network is dropped after
        two SIMP iterations in a row where the saved iterations cost less than the prediction."""
        from . import learned as LW
        info, t_pred = ws
        nc = len(self.cases)
        its = self.fem.cg_iters[-nc:]
        saved_s = 0.0
        for c in range(nc):
            pi_star = LW.energy(self.ctx, self.escale_t, self.F_t[c], self.U_t[c])
            e_fin = max(self.rtol ** 2 * abs(pi_star), 1e-300)
            e_prev = max(info[c][0] - pi_star, e_fin)
            e_new = max(info[c][1] - pi_star, e_fin)
            it = max(its[c], 1)
            if e_new > e_fin:
                would = it * np.log(e_prev / e_fin) / np.log(e_new / e_fin)
                saved_s += max(0.0, would - it) * t_solve / (nc * it)
        self.ws_ledger.append((saved_s, t_pred))
        recent = self.ws_ledger[-2:]
        if len(recent) == 2 and all(sv < tp for sv, tp in recent):
            self.warm_start = None

    def step_host(self, x_in, x_out):
        """One iteration with the design exchanged through host memory: x_in (host float32,
        full grid) is copied in, the updated design is copied to x_out (host float32)."""
        self.x_t.copy_(x_in, non_blocking=True)
        rec = self.step()
        x_out.copy_(self.x_t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return rec

    def converged(self, tol):
        rec = self.hist[-1]
        return (rec["p"] >= self.p_final and rec["beta"] >= self.beta_max
                and self.it > (5 if self.warm else 10) and rec["change"] < tol)

    def result(self, t_start):
        xout = np.zeros(self.grid.nelem)
        xout[self.act] = self.xphys_t.cpu().numpy().astype(float)[self.act]
        return {"x": xout, "history": self.hist, "fem_builds": self.fem.amg_builds, "rMM": self.r_vox * self.grid.h,
                "seconds": time.time() - t_start, "cases": self.cases}

    def close(self):
        self.fem.close()


def simp(grid, fill, active, frozen, fixed, loads, weights, E0, nu, vf,
         iters=80, r_mm=None, p_final=3.0, move=0.2, combine="sum", log=print, tol=0.01, x0=None,
         beta_max=BETA_MAX, rtol=None, maxiter=2000, precision="auto", multi="batch", cg_start="previous"):
    """optimize.py:50-180 on the GPU. ``rtol`` overrides the CG tolerance (default CG_RTOL,
    the reference's hard-coded 1e-6); the void stiffness is the module constant EMIN.
    ``precision`` ("auto", "fp32", "fp64") picks the solver's operator arithmetic,
    ``multi`` ("batch", "lanes") how several load cases are solved (FEM) and ``cg_start``
    each solve's start: "previous" (the last solution, as the reference) or "history" (the
    Galerkin combination of the last two solutions, SimpRunner._history_start)."""
    t_start = time.time()
    run = SimpRunner(grid, fill, active, frozen, fixed, loads, weights, E0, nu, vf, iters=iters, r_mm=r_mm,
                     p_final=p_final, move=move, combine=combine, log=log, x0=x0, beta_max=beta_max, rtol=rtol,
                     maxiter=maxiter, precision=precision, multi=multi, cg_start=cg_start)
    for _ in range(iters):
        run.step()
        if run.converged(tol):
            log(f"  converged at iteration {run.it}")
            break
    res = run.result(t_start)
    run.close()
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
