"""GPU kernels against the FP64 oracle and the reference's golden vectors, through the C ABI.

Tolerances: FP64 paths agree to ~1e-12 relative; FP32 paths to a few 1e-6 of the field's
largest magnitude (FP32 arithmetic with FP64 accumulation where the kernel reduces)."""
import os

import numpy as np
import pytest
import torch

from anneal_gb300.context import Context, to_dev

pytestmark = pytest.mark.gpu

F32, F64, U8 = torch.float32, torch.float64, torch.uint8


def _domain(shape, seed, hole_frac=0.1, clamp_x0=True):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    ne = nx * ny * nz
    e = np.arange(ne)
    i, k = e % nx, e // (nx * ny)
    active = ~((i >= nx // 2) & (k >= nz // 2)) & (rng.random(ne) > hole_frac)
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    n = np.arange(nn)
    fixed = np.zeros(3 * nn, np.uint8)
    if clamp_x0:
        c = n[n % (nx + 1) == 0]
        fixed[3 * c] = fixed[3 * c + 1] = fixed[3 * c + 2] = 1
    E = np.exp(rng.normal(0.0, 1.0, ne))
    E[rng.random(ne) < 0.2] = 1e-9
    E[~active] = 0.0
    return active, fixed, E


def _ctx(shape, active, fixed, fp64, h=1.0, nu=0.3):
    c = Context(shape, h, nu, fp64=fp64)
    c.set_domain(to_dev(active.astype(np.uint8), U8), to_dev(fixed, U8))
    return c


@pytest.mark.parametrize("shape", [(7, 5, 4), (13, 7, 5), (40, 11, 19), (33, 9, 17), (61, 31, 23), (70, 33, 40)])
@pytest.mark.parametrize("fp64", [False, True])
def test_apply_K_matches_oracle(oracle, shape, fp64):
    active, fixed, E = _domain(shape, seed=sum(shape))
    fem = oracle.OracleFEM(shape, 1.0, active, np.flatnonzero(fixed), 0.3)
    rng = np.random.default_rng(1)
    u = np.where(fem.mask, rng.normal(0.0, 1.0, 3 * fem.nnode), 0.0)
    want = fem.apply(E[fem.act], u)
    c = _ctx(shape, active, fixed, fp64)
    assert c.nfree == fem.nfree
    assert np.array_equal(c.free_mask().cpu().numpy().astype(bool), fem.mask)
    dt = F64 if fp64 else F32
    y = torch.empty(c.ndof, dtype=dt, device="cuda")
    c.apply_K(to_dev(E, F32), to_dev(u, dt), y)
    got = y.cpu().numpy().astype(float)
    scale = np.abs(want).max()
    tol = 1e-6 if fp64 else 2e-6   # E is rounded to FP32 on input in both modes
    assert np.abs(got - want).max() <= tol * scale


def test_apply_K_matches_reference_csr(golden):
    g = golden("fem_small.npz")
    shape = tuple(int(s) for s in g["shape"])
    fixed = np.zeros(3 * np.prod([s + 1 for s in shape]), np.uint8)
    fixed[g["fixed"]] = 1
    c = _ctx(shape, g["active"], fixed, True)
    E = np.zeros(np.prod(shape))
    E[np.flatnonzero(g["active"])] = g["Ee"]
    u = np.zeros(c.ndof)
    u[g["free"]] = g["u_red"]
    y = torch.empty(c.ndof, dtype=F64, device="cuda")
    c.apply_K(to_dev(E, F32), to_dev(u, F64), y)
    got = y.cpu().numpy()[g["free"]]
    # the element scales enter as FP32: compare against the reference within that rounding
    assert np.abs(got - g["y_red"]).max() <= 1e-6 * np.abs(g["y_red"]).max()


def test_element_energy_matches_reference(golden):
    g = golden("fem_small.npz")
    shape = tuple(int(s) for s in g["shape"])
    fixed = np.zeros(3 * np.prod([s + 1 for s in shape]), np.uint8)
    fixed[g["fixed"]] = 1
    c = _ctx(shape, g["active"], fixed, False)
    u = np.zeros(c.ndof)
    u[g["free"]] = g["u_red"]
    ce = torch.empty(c.ne, dtype=F32, device="cuda")
    c.element_energy(to_dev(u, F64), ce)
    got = ce.cpu().numpy()[np.flatnonzero(g["active"])]
    assert np.abs(got - g["ce"]).max() <= 2e-6 * np.abs(g["ce"]).max()


@pytest.mark.parametrize("tag,r", [("r15", 1.5), ("r20", 2.0), ("r26", 2.6), ("r31", 3.1)])
def test_filter_matches_reference(golden, tag, r):
    f = golden("filter.npz")
    shape = tuple(int(s) for s in f["shape"])
    act = np.flatnonzero(f["active"])
    c = _ctx(shape, f["active"], np.zeros(3 * np.prod([s + 1 for s in shape]), np.uint8), False)
    c.filter_init(r)
    ne = int(np.prod(shape))
    for src, fn, key in ((f["x"], c.filter_fwd, "fwd"), (f["d"], c.filter_bwd, "bwd")):
        full = np.zeros(ne)
        full[act] = src
        out = torch.empty(ne, dtype=F32, device="cuda")
        fn(to_dev(full, F32), out)
        got = out.cpu().numpy()[act]
        assert np.abs(got - f[f"{key}_{tag}"]).max() <= 2e-6 * max(1.0, np.abs(f[f"{key}_{tag}"]).max())


@pytest.mark.parametrize("beta", [0.0, 2.0])
def test_physical_and_oc_match_oracle(oracle, beta):
    shape = (21, 10, 9)
    rng = np.random.default_rng(5)
    active, fixed, _ = _domain(shape, seed=9)
    ne = int(np.prod(shape))
    frozen = (rng.random(ne) < 0.05) & active
    phi = np.where(active, np.clip(rng.random(ne) + 0.3, 0, 1), 0.0)
    x = np.where(active, np.clip(rng.random(ne), 0.05, 1.0), 0.0)
    dcx = np.where(active, -np.exp(rng.normal(0, 1, ne)) * 1e-3, 0.0)
    dcx[rng.random(ne) < 0.05] = 0.0
    r = 2.0
    F = oracle.OracleFilter(shape, active, r)
    act = F.act
    dvx_act = F.backward(phi[act])
    dvx = np.zeros(ne)
    dvx[act] = dvx_act
    vtarget = 0.3 * phi[act].sum()
    want, steps = oracle.oc_update(F, x[act], dcx[act], dvx[act], phi[act], frozen[act], 0.2, beta, vtarget)

    c = _ctx(shape, active, fixed, False)
    c.filter_init(r)
    xn = torch.empty(ne, dtype=F32, device="cuda")
    got_steps, _ = c.oc_update(to_dev(x, F32), to_dev(dcx, F32), to_dev(dvx, F32), to_dev(phi, F32),
                               to_dev(frozen.astype(np.uint8), U8), 0.2, beta, 0.5, vtarget, xn)
    got = xn.cpu().numpy()[act]
    assert abs(got_steps - steps) <= 2
    assert np.abs(got - want).max() < 1e-4

    # physical(): filter + projection + frozen
    xp = torch.empty(ne, dtype=F32, device="cuda")
    dxp = torch.empty(ne, dtype=F32, device="cuda")
    c.physical(to_dev(x, F32), to_dev(frozen.astype(np.uint8), U8), beta, 0.5, xp, dxp)
    xt = F.forward(x[act])
    if beta > 0:
        t0, t1 = np.tanh(beta * 0.5), np.tanh(beta * 0.5)
        th = np.tanh(beta * (xt - 0.5))
        wp, wd = (t0 + th) / (t0 + t1), beta * (1 - th ** 2) / (t0 + t1)
    else:
        wp, wd = xt.copy(), np.ones_like(xt)
    wp[frozen[act]] = 1.0
    assert np.abs(xp.cpu().numpy()[act] - wp).max() < 2e-6
    assert np.abs(dxp.cpu().numpy()[act] - wd).max() < 2e-6


def test_sensitivity_matches_oracle(oracle):
    shape = (12, 7, 6)
    active, fixed, E = _domain(shape, seed=3)
    ne = int(np.prod(shape))
    fem = oracle.OracleFEM(shape, 1.0, active, np.flatnonzero(fixed), 0.3)
    rng = np.random.default_rng(8)
    U = [np.where(fem.mask, rng.normal(0, 1e-2, 3 * fem.nnode), 0.0) for _ in range(2)]
    xphys = np.where(active, rng.random(ne), 0.0)
    dxp = np.where(active, rng.random(ne) + 0.5, 0.0)
    phi = np.where(active, 1.0, 0.0)
    coef = [1.0, 0.5]
    p, emin, E0 = 3.0, 1e-9, 2.0
    act = fem.act
    dc = sum(w * (-p * xphys[act] ** (p - 1) * (1 - emin) * E0 * phi[act] * fem.element_energy(u))
             for w, u in zip(coef, U))
    want = np.minimum(dc, 0.0) * dxp[act]
    c = _ctx(shape, active, fixed, False)
    out = torch.empty(ne, dtype=F32, device="cuda")
    dv = torch.empty(ne, dtype=F32, device="cuda")
    c.sensitivity(to_dev(np.stack(U), F64), coef, to_dev(xphys, F32), to_dev(dxp, F32), to_dev(phi, F32),
                  p, emin, E0, out, dv)
    got = out.cpu().numpy()[act]
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()
    assert np.abs(dv.cpu().numpy()[act] - phi[act] * dxp[act]).max() < 1e-6


def test_stress_and_von_mises_match_reference(golden):
    """FEM.stress / von_mises / normal_stress against the reference's own values
    (fem.py:244-263) on a cantilever solution, per-element and scalar modulus."""
    from anneal_gb300 import fem as G
    g = golden("stress.npz")
    grid = G.Grid(tuple(int(s) for s in g["shape"]), float(g["h"]), g["origin"])
    fem = G.FEM(grid, g["active"], g["fixed"], 0.3)
    sig = fem.stress(g["u"], g["Emat"])
    assert np.abs(sig - g["sig"]).max() <= 1e-10 * np.abs(g["sig"]).max()
    vm = fem.von_mises(g["u"], g["Emat"])
    assert np.abs(vm - g["vm"]).max() <= 1e-10 * np.abs(g["vm"]).max()
    vs = fem.von_mises(g["u"], 1500.0)
    assert np.abs(vs - g["vm_scalar"]).max() <= 1e-10 * np.abs(g["vm_scalar"]).max()
    sn = fem.normal_stress(sig, (0.2, -0.3, 1.0))
    assert np.abs(sn - g["sn"]).max() <= 1e-10 * np.abs(g["sn"]).max()
    fem.close()


def test_bounds_checks_match_the_loaded_library():
    """The bounds-checked build (ANL_DEBUG_LIB=1) reports a count (0 here: the tests before
    it are checked by the conftest fixture); the normal build reports -1 (no checks)."""
    import ctypes
    from anneal_gb300 import _native as N
    lib = N.load()
    count, first = ctypes.c_longlong(0), (ctypes.c_longlong * 3)()
    N.check(lib.anl_debug_oob(ctypes.byref(count), first), "anl_debug_oob")
    assert N.LIB_PATH.endswith(os.path.join("_lib_debug" if N.DEBUG_LIB else "_lib", "libanneal_gb300.so"))
    assert count.value == (0 if N.DEBUG_LIB else -1)
