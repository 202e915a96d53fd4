"""Solver validation gate on the GPU path (anneal's validate.py V1-V6, validate.py:38-143).

Each check compares the solver with a closed-form answer and uses the same grids, loads,
tolerances and pass bands as the reference, so ``run_all`` is a drop-in for
``anneal validate``.
"""
import hashlib

import numpy as np

from .fem import FEM, Grid, hex8_matrices

E0, NU = 1000.0, 0.3


def _face_load(grid, elems, weights, total, comp, face_nodes):
    """Spread `total` over one face of each listed element, in proportion to weights."""
    F = np.zeros(3 * grid.nnode)
    en = grid.element_nodes(elems)
    share = total * weights / weights.sum()
    for k in face_nodes:
        np.add.at(F, 3 * en[:, k] + comp, share / 4.0)
    return F


def _bar(nx, ny, nz, h):
    g = Grid((nx, ny, nz), h, (0, 0, 0))
    e = np.arange(g.nelem)
    i, j, k = g.elem_ijk(e)
    return g, e, i, j, k


def _nodes(grid, pred):
    n = np.arange(grid.nnode)
    return n[pred(grid.node_coords(n))]


def check_rigid_body():
    """V1: translations and rotations of one element store no energy."""
    ke, _, _ = hex8_matrices(NU, 1.0)
    xyz = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    t = np.tile([1.0, 0, 0], 8)
    rot = np.stack([-xyz[:, 1], xyz[:, 0], np.zeros(8)], axis=1).ravel()
    et, er = float(t @ ke @ t), float(rot @ ke @ rot)
    return "V1 rigid body stores no energy", max(abs(et), abs(er)) < 1e-10, f"translation {et:.2e}, rotation {er:.2e}"


def _tension(fill_layer=None, nz=4, L=10, ny=2, h=1.0, F=100.0):
    g, e, i, j, k = _bar(L, ny, nz, h)
    fill = np.ones(g.nelem) if fill_layer is None else np.where(k == nz - 1, fill_layer, 1.0)
    fixed = [3 * n for n in _nodes(g, lambda p: p[:, 0] < 1e-9)]
    n0 = _nodes(g, lambda p: (p[:, 0] < 1e-9) & (p[:, 1] < 1e-9) & (p[:, 2] < 1e-9))[0]
    n1 = _nodes(g, lambda p: (p[:, 0] < 1e-9) & (abs(p[:, 1] - ny * h) < 1e-9) & (p[:, 2] < 1e-9))[0]
    fixed += [3 * n0 + 1, 3 * n0 + 2, 3 * n1 + 2]
    fem = FEM(g, np.ones(g.nelem, bool), fixed, NU)
    end = e[i == L - 1]
    Fg = _face_load(g, end, fill[end], F, 0, [1, 2, 5, 6])
    u = fem.expand(fem.solve(fem.assemble(E0 * fill), [fem.reduce_load(Fg)], rtol=1e-12)[0])
    fem.close()
    tip = _nodes(g, lambda p: abs(p[:, 0] - L * h) < 1e-9)
    return u[3 * tip].mean(), g


def check_tension():
    """V2: a uniform bar in tension stretches by exactly F L / (A E)."""
    ux, _ = _tension()
    exact = 100.0 * 10 / (2 * 4 * 1.0 * E0)
    err = abs(ux - exact) / exact
    return "V2 uniform tension = FL/(AE)", err < 1e-8, f"relative error {err:.2e}"


def check_cantilever():
    """V3: tip deflection against Timoshenko beam theory, inside the shear-locking bands."""
    res, ok = [], True
    bands = {2: (0.84, 0.90), 4: (0.93, 0.98), 8: (0.97, 0.995)}
    for nd in (2, 4, 8):
        d, b, L, P = 4.0, 4.0, 40.0, 10.0
        h = d / nd
        g, e, i, j, k = _bar(10 * nd, nd, nd, h)
        clamp = _nodes(g, lambda p: p[:, 0] < 1e-9)
        fem = FEM(g, np.ones(g.nelem, bool), (3 * clamp[:, None] + np.arange(3)).ravel(), NU)
        end = e[i == g.nx - 1]
        Fg = _face_load(g, end, np.ones(end.size), -P, 2, [1, 2, 5, 6])
        u = fem.expand(fem.solve(fem.assemble(E0 * np.ones(g.nelem)), [fem.reduce_load(Fg)], rtol=1e-12)[0])
        fem.close()
        tip = _nodes(g, lambda p: abs(p[:, 0] - L) < 1e-9)
        uz = -u[3 * tip + 2].mean()
        I = b * d ** 3 / 12
        G = E0 / (2 * (1 + NU))
        timo = P * L ** 3 / (3 * E0 * I) + P * L / (5 / 6 * G * b * d)
        r = uz / timo
        lo, hi = bands[nd]
        ok &= lo <= r <= hi
        res.append(f"{nd} deep {100 * r:.1f}%")
    return "V3 cantilever vs Timoshenko (shear locking expected)", bool(ok), " · ".join(res)


def check_partial_volume():
    """V4: a partially filled layer (fill as stiffness scale) is exact; binary voxels are not."""
    ux_partial, _ = _tension(fill_layer=0.4, nz=7)
    ux_binary, _ = _tension(fill_layer=None, nz=6)
    exact = 100.0 * 10 / (2 * 6.4 * E0)
    ep = abs(ux_partial - exact) / exact
    eb = abs(ux_binary - exact) / exact
    return "V4 partial volume beats binary (bar 6.4 cells deep)", ep < 1e-8 and eb > 0.05, \
        f"binary {100 * eb:.2f}% error, partial {ep:.1e}"


def check_determinism():
    """V5: two identical solves give bit-identical displacements."""
    hashes = []
    for _ in range(2):
        g, e, i, j, k = _bar(20, 4, 4, 1.0)
        clamp = _nodes(g, lambda p: p[:, 0] < 1e-9)
        fem = FEM(g, np.ones(g.nelem, bool), (3 * clamp[:, None] + np.arange(3)).ravel(), NU)
        end = e[i == g.nx - 1]
        Fg = _face_load(g, end, np.ones(end.size), -1.0, 2, [1, 2, 5, 6])
        u = fem.solve(fem.assemble(E0 * np.ones(g.nelem)), [fem.reduce_load(Fg)])[0]
        fem.close()
        hashes.append(hashlib.sha256(u.tobytes()).hexdigest())
    return "V5 deterministic reruns", hashes[0] == hashes[1], f"sha256 {hashes[0][:12]}…"


def check_simp():
    """V6: SIMP beats a uniform design at equal mass."""
    from .optimize import benchmark_cantilever
    r = benchmark_cantilever()
    ok = r["stiffer_pct"] > 20 and abs(r["vol_err"]) < 1e-3
    return "V6 SIMP beats uniform at equal mass", ok, f"{r['stiffer_pct']:.1f}% stiffer, volume error {r['vol_err']:.1e}"


CHECKS = [check_rigid_body, check_tension, check_cantilever, check_partial_volume, check_determinism, check_simp]


def run_all(log=print):
    passed = 0
    for fn in CHECKS:
        name, ok, detail = fn()
        passed += ok
        log(f"  [{'PASS' if ok else 'FAIL'}] {name}: {detail}")
    log(f"  GATE: {'OPEN' if passed == len(CHECKS) else 'CLOSED'} - {passed} of {len(CHECKS)} checks pass")
    return passed == len(CHECKS)
