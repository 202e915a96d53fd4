"""FP64 CPU oracle for the voxel SIMP hot path of anneal 0.3.0.

TEST INFRASTRUCTURE ONLY: the checker for the GPU library (tests/, the smoke check in
__graft_entry__) and the timed CPU baseline in bench.py. The product never imports it.

The heavy loops (element-by-element K u, PCG, filter, OC) are C in anneal_oracle.c;
this module restates the Python logic of the reference around them:

* ``OracleFEM``  -- fem.py:130-242 (free-DOF rule, solve semantics, element energy)
* ``OracleFilter`` -- optimize.py:24-47
* ``simp`` -- optimize.py:50-180 (continuation, Heaviside projection, combine, OC, history)

Vectors use the full-grid DOF layout (3*node + c) with zeros on non-free DOFs; the
reference's reduced vectors are ``u_full[free]``.
"""
import ctypes
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

EMIN = 1e-6      # optimize.py:18
PNORM = 8.0      # optimize.py:19
ETA = 0.5        # optimize.py:20
BETA_MAX = 4.0   # optimize.py:21

LOCAL = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])

_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_u8 = ctypes.POINTER(ctypes.c_uint8)
_i64 = ctypes.POINTER(ctypes.c_int64)


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        I, D = ctypes.c_int, ctypes.c_double
        _lib.orc_hex8_ke.argtypes = [D, D, _d]
        _lib.orc_apply_K.argtypes = [I, I, I, _d, _d, _u8, _d, _d]
        _lib.orc_diag.argtypes = [I, I, I, _d, _d, _u8, _d]
        _lib.orc_element_energy.argtypes = [I, I, I, _d, _u8, _d, _d]
        _lib.orc_filter.argtypes = [I, I, I, D, _u8, _d, _d, _d, I]
        _lib.orc_pcg.argtypes = [I, I, I, _d, _d, _u8, _d, _d, D, I, I, I,
                                 ctypes.POINTER(I), ctypes.POINTER(D)]
        _lib.orc_pcg.restype = I
        _lib.orc_oc.argtypes = [I, I, I, D, _u8, _d, ctypes.c_int64, _i64, _d, _d, _d, _d, _u8,
                                D, D, D, D, _d]
        _lib.orc_oc.restype = I
        _lib.orc_num_threads.restype = I
    return _lib


def build(force=False):
    """Compile anneal_oracle.c with gcc (OpenMP) into oracle/_build/liboracle.so."""
    import subprocess
    src = os.path.join(HERE, "anneal_oracle.c")
    if not force and os.path.isfile(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c99", src, "-lm",
                           "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _p(a, t=_d):
    return a.ctypes.data_as(t)


def num_threads():
    return lib().orc_num_threads()


def hex8_ke(nu, h=1.0):
    """fem.py:71-84 (Ke only)."""
    ke = np.zeros(576)
    lib().orc_hex8_ke(nu, h, _p(ke))
    return ke.reshape(24, 24)


def element_nodes(shape, e):
    """fem.py:100-107."""
    nx, ny, nz = shape
    e = np.asarray(e)
    i, j, k = e % nx, (e // nx) % ny, e // (nx * ny)
    base = i + (nx + 1) * (j + (ny + 1) * k)
    noff = LOCAL[:, 0] + (nx + 1) * (LOCAL[:, 1] + (ny + 1) * LOCAL[:, 2])
    return base[:, None] + noff[None, :]


def free_dof_mask(shape, active, fixed_dofs):
    """fem.py:142-150: DOFs of nodes touched by an active element, minus fixed DOFs."""
    nx, ny, nz = shape
    nnode = (nx + 1) * (ny + 1) * (nz + 1)
    act = np.flatnonzero(active)
    used = np.unique(element_nodes(shape, act))
    m = np.zeros(3 * nnode, dtype=bool)
    m[(3 * used[:, None] + np.arange(3)).ravel()] = True
    m[np.asarray(fixed_dofs, dtype=np.int64)] = False
    return m


class SolverError(RuntimeError):
    """fem.py:24-25."""


class OracleFEM:
    """fem.py:130-242 restated matrix-free (the same linear operator, no CSR)."""

    def __init__(self, shape, h, active, fixed_dofs, nu):
        self.shape = tuple(int(s) for s in shape)
        self.nelem = int(np.prod(self.shape))
        self.nnode = int(np.prod([s + 1 for s in self.shape]))
        self.act = np.flatnonzero(active)
        if self.act.size == 0:
            raise SolverError("No active voxels: the design space is empty.")
        self.active = np.zeros(self.nelem, np.uint8)
        self.active[self.act] = 1
        self.ke = hex8_ke(nu, h).ravel().copy()
        self.mask = free_dof_mask(self.shape, active, fixed_dofs)
        self.mask_u8 = self.mask.astype(np.uint8)
        self.free = np.flatnonzero(self.mask)
        self.nfree = self.free.size
        self.cg_iters = []

    def full_E(self, Ee):
        E = np.zeros(self.nelem)
        E[self.act] = Ee
        return E

    def apply(self, Ee, u_full):
        y = np.zeros(3 * self.nnode)
        lib().orc_apply_K(*self.shape, _p(self.ke), _p(self.full_E(Ee)), _p(self.mask_u8, _u8),
                          _p(np.ascontiguousarray(u_full, float)), _p(y))
        return y

    def solve(self, Ee, F_list, x0_list=None, rtol=1e-8, maxiter=2000, precond="mg", degree=2):
        """fem.py:206-232; returns full-layout solutions; raises SolverError like :225-229."""
        E = self.full_E(Ee)
        out = []
        for i, F in enumerate(F_list):
            b = np.where(self.mask, F, 0.0)
            x = np.zeros(3 * self.nnode) if x0_list is None else np.where(self.mask, x0_list[i], 0.0)
            it = ctypes.c_int(0)
            rr = ctypes.c_double(0.0)
            st = lib().orc_pcg(*self.shape, _p(self.ke), _p(E), _p(self.mask_u8, _u8), _p(b), _p(x),
                               rtol, maxiter, 1 if precond == "mg" else 0, degree,
                               ctypes.byref(it), ctypes.byref(rr))
            if st != 0 or not np.all(np.isfinite(x)):
                raise SolverError(
                    f"The solver did not converge in {maxiter} iterations. Usual causes: the part can move "
                    f"or turn freely (add a fixed anchor, or fix more directions on one), or the design has "
                    f"pieces held only by near-empty voxels (raise volumeFraction or iterations).")
            self.cg_iters.append(it.value)
            out.append(x)
        return out

    def element_energy(self, u_full):
        """fem.py:239-242, returned for the active elements."""
        ce = np.zeros(self.nelem)
        lib().orc_element_energy(*self.shape, _p(self.ke), _p(self.active, _u8),
                                 _p(np.ascontiguousarray(u_full, float)), _p(ce))
        return ce[self.act]


class OracleFilter:
    """optimize.py:24-47."""

    def __init__(self, shape, active, r_vox):
        self.shape = tuple(int(s) for s in shape)
        self.nelem = int(np.prod(self.shape))
        self.r = float(r_vox)
        self.act = np.flatnonzero(active)
        self.active = np.zeros(self.nelem, np.uint8)
        self.active[self.act] = 1
        self.Hs = np.zeros(self.nelem)
        lib().orc_filter(*self.shape, self.r, _p(self.active, _u8), _p(self.Hs), _p(self.Hs),
                         _p(self.Hs), 0)

    def _run(self, v_act, mode):
        full = np.zeros(self.nelem)
        full[self.act] = v_act
        out = np.zeros(self.nelem)
        lib().orc_filter(*self.shape, self.r, _p(self.active, _u8), _p(self.Hs), _p(full), _p(out), mode)
        return out[self.act]

    def forward(self, x_act):
        return self._run(x_act, 1)

    def backward(self, d_act):
        return self._run(d_act, 2)


def oc_update(filt, x, dcx, dvx, phi, frz, move, beta, vtarget):
    """optimize.py:144-161 (the bisection); returns (xd, steps)."""
    xd = np.zeros(x.size)
    steps = lib().orc_oc(*filt.shape, filt.r, _p(filt.active, _u8), _p(filt.Hs), x.size,
                         _p(filt.act.astype(np.int64), _i64), _p(np.ascontiguousarray(x)),
                         _p(np.ascontiguousarray(dcx)), _p(np.ascontiguousarray(dvx)),
                         _p(np.ascontiguousarray(phi, float)), _p(frz.astype(np.uint8), _u8),
                         move, beta, ETA, vtarget, _p(xd))
    return xd, steps


class SimpRun:
    """The state of one oracle SIMP run (optimize.py:50-104) and one ``step()`` per iteration
    (optimize.py:105-172). ``simp`` drives it; the CPU baseline of the benchmark times
    ``step()`` directly."""

    def __init__(self, shape, h, fill, active, frozen, fixed, loads, weights, E0, nu, vf, iters=80, r_mm=None,
                 p_final=3.0, move=0.2, combine="sum", log=print, x0=None, beta_max=BETA_MAX, rtol=1e-6,
                 emin=None, precond="mg", maxiter=2000):
        self.EM = EMIN if emin is None else emin
        self.shape, self.h = tuple(int(s) for s in shape), h
        self.E0, self.vf, self.iters, self.p_final, self.move = E0, vf, iters, p_final, move
        self.combine, self.log, self.beta_max, self.rtol = combine, log, beta_max, rtol
        self.precond, self.maxiter = precond, maxiter
        self.fem = fem = OracleFEM(shape, h, active, fixed, nu)
        act = self.act = fem.act
        self.phi = phi = np.asarray(fill, float)[act]
        self.frz = frz = np.asarray(frozen)[act].astype(bool)
        self.des = des = ~frz
        self.r_vox = max((r_mm or 1.5 * h) / h, 1.5)
        self.filt = OracleFilter(shape, active, self.r_vox)
        self.cases = cases = list(loads)
        self.Fr = [np.where(fem.mask, loads[c], 0.0) for c in cases]
        self.w = np.array([weights[c] for c in cases])
        if all(np.allclose(f, 0) for f in self.Fr):
            raise ValueError("All loads are zero after mapping onto the grid. Check the load anchors' regions.")
        self.Vtot = phi.sum()
        self.Vtarget = vf * self.Vtot
        Vfrozen = phi[frz].sum()
        x = np.ones(act.size)
        x[des] = np.clip((self.Vtarget - Vfrozen) / max(phi[des].sum(), 1e-12), 0.01, 1.0)
        self.warm = x0 is not None
        if self.warm:
            xs = np.clip(np.asarray(x0)[act], 0.0, 1.0)
            cur = (phi[des] * xs[des]).sum()
            if cur > 0:
                x[des] = np.clip(xs[des] * (self.Vtarget - Vfrozen) / cur, 0.001, 1.0)
        self.x = x
        self.beta = beta_max / 2 if self.warm else 0.0
        self.hist = []
        self.U = [None] * len(cases)
        self.c0 = None
        self.p = 1.0
        self.xPhys = self.physical(x)
        self.beta_step = max(5, int(0.12 * iters))
        self.beta_since = 0
        self.it = 0

    def project(self, xt):
        b = self.beta
        if b <= 0:
            return xt, np.ones_like(xt)
        t0, t1 = np.tanh(b * ETA), np.tanh(b * (1 - ETA))
        th = np.tanh(b * (xt - ETA))
        return (t0 + th) / (t0 + t1), b * (1 - th ** 2) / (t0 + t1)

    def physical(self, xd, with_grad=False):
        xt = self.filt.forward(xd)
        xp, dxp = self.project(xt)
        xp[self.frz] = 1.0
        return (xp, dxp) if with_grad else xp

    def step(self):
        t0 = time.time()
        self.it += 1
        it, iters, p_final, EM, E0 = self.it, self.iters, self.p_final, self.EM, self.E0
        fem, phi, frz, des, w = self.fem, self.phi, self.frz, self.des, self.w
        hold = max(1, min(3, int(0.4 * iters / max((p_final - 1.0) / 0.25, 1))))
        p = self.p = p_final if self.warm else min(p_final, 1.0 + 0.25 * ((it - 1) // hold))
        if p >= p_final and not self.warm and self.beta_max > 0:
            if self.beta == 0:
                self.beta, self.beta_since = 1.0, 0
            elif self.beta_since >= self.beta_step and self.beta < self.beta_max:
                self.beta, self.beta_since = min(self.beta_max, 2 * self.beta), 0
            self.beta_since += 1
        xPhys, dxp = self.physical(self.x, with_grad=True)
        Ee = E0 * phi * (EM + xPhys ** p * (1 - EM))
        U = self.U = fem.solve(Ee, self.Fr, x0_list=None if self.U[0] is None else self.U, rtol=self.rtol,
                               maxiter=self.maxiter, precond=self.precond)
        cs = np.array([f @ u for f, u in zip(self.Fr, U)])
        dce = []
        for u in U:
            ce = fem.element_energy(u)
            dce.append(-p * xPhys ** (p - 1) * (1 - EM) * E0 * phi * ce)
        if self.c0 is None:
            self.c0 = cs.copy()
        if self.combine == "sum" or len(self.cases) == 1:
            obj = float(w @ cs)
            dc = sum(wi * d for wi, d in zip(w, dce))
        else:
            r = w * cs / self.c0
            obj = float((r ** PNORM).sum() ** (1 / PNORM))
            coef = (r / obj) ** (PNORM - 1) * w / self.c0
            dc = sum(ci * d for ci, d in zip(coef, dce))
        dc = np.minimum(dc, 0.0)
        dcx = self.filt.backward(dc * dxp)
        dvx = self.filt.backward(phi * dxp)
        xd, _ = oc_update(self.filt, self.x, dcx, dvx, phi, frz, self.move, self.beta, self.Vtarget)
        change = float(np.abs(xd - self.x)[des].max()) if des.any() else 0.0
        self.x = xd
        self.xPhys = xPhys = self.physical(xd)
        grey = float(((xPhys > 0.1) & (xPhys < 0.9))[des].mean()) if des.any() else 0.0
        rec = {"iter": it, "objective": obj, "compliance": cs.tolist(), "p": p, "beta": self.beta,
               "volumeFraction": float((phi * xPhys).sum() / self.Vtot), "change": change,
               "grey": grey, "cgIters": fem.cg_iters[-len(self.cases):], "amgRebuilt": True,
               "seconds": time.time() - t0}
        self.hist.append(rec)
        self.log(f"  it {it:3d}  p {p:.2f}  b {self.beta:.0f}  obj {obj:.4g}  vol {rec['volumeFraction']:.3f}  "
                 f"change {change:.3f}  grey {grey:.2f}  cg {fem.cg_iters[-1]} amg  {rec['seconds']:.1f}s")
        return rec

    def converged(self, tol):
        rec = self.hist[-1]
        return (rec["p"] >= self.p_final and rec["beta"] >= self.beta_max
                and self.it > (5 if self.warm else 10) and rec["change"] < tol)

    def full_x(self):
        full = np.zeros(int(np.prod(self.shape)))
        full[self.act] = self.xPhys
        return full


def simp(shape, h, fill, active, frozen, fixed, loads, weights, E0, nu, vf, iters=80, r_mm=None,
         p_final=3.0, move=0.2, combine="sum", log=print, tol=0.01, x0=None, beta_max=BETA_MAX,
         rtol=1e-6, emin=None, precond="mg", maxiter=2000):
    """optimize.py:50-180 restated. ``rtol`` is the CG tolerance the reference hard-codes
    at optimize.py:122 (1e-6); ``emin`` overrides EMIN (optimize.py:18)."""
    t_start = time.time()
    run = SimpRun(shape, h, fill, active, frozen, fixed, loads, weights, E0, nu, vf, iters=iters, r_mm=r_mm,
                  p_final=p_final, move=move, combine=combine, log=log, x0=x0, beta_max=beta_max, rtol=rtol,
                  emin=emin, precond=precond, maxiter=maxiter)
    for _ in range(iters):
        run.step()
        if run.converged(tol):
            log(f"  converged at iteration {run.it}")
            break
    return {"x": run.full_x(), "history": run.hist, "fem_builds": len(run.hist), "rMM": run.r_vox * h,
            "seconds": time.time() - t_start, "cases": run.cases, "U": run.U}
