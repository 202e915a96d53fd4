"""The GPU solve and SIMP loop against the reference's golden runs and the FP64 oracle.

Parity bars: compliance within 1e-5 relative per solve; final density L-inf within 1e-3."""
import numpy as np
import pytest

from anneal_gb300 import fem as G
from anneal_gb300 import optimize as O
from anneal_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _grid(shape):
    return G.Grid(shape, 1.0, (0, 0, 0))


@pytest.mark.parametrize("rtol", [1e-12, 1e-6])
def test_solve_matches_reference(golden, rtol):
    g = golden("fem_small.npz")
    grid = _grid(tuple(int(s) for s in g["shape"]))
    fem = G.FEM(grid, g["active"], g["fixed"], 0.3)
    assert np.array_equal(fem.free, g["free"])
    Fr = fem.reduce_load(g["F"])
    u = fem.solve(fem.assemble(g["Ee_solve"]), [Fr], rtol=rtol)[0]
    c = float(Fr @ u)
    assert abs(c / float(g["compliance"]) - 1) < (1e-6 if rtol < 1e-7 else 1e-5)
    assert fem.relres[-1] <= rtol * 1.0001
    if rtol < 1e-7:
        assert np.abs(u - g["u_sol"]).max() <= 1e-6 * np.abs(g["u_sol"]).max()
    fem.close()


@pytest.mark.parametrize("seed", [0, 1])
def test_fp32_path_certifies_the_fp64_operator(seed):
    """The FP32 solver certifies on the accurate residual of the FP64 operator: its solution at
    rtol 1e-7 matches the FP64 solver's at 1e-11 (random SIMP-like densities, penalty 3, on a
    64 x 32 x 32 cantilever), and its reported residual is the FP64 operator's."""
    w = P.cantilever(64, 32, 32)
    fem = G.FEM(_grid(w.shape), w.active, w.fixed, 0.3)
    rho = P.random_density(w.shape, seed)
    Ee = 1e-9 + rho[fem.act] ** 3 * (1 - 1e-9)
    K = fem.assemble(Ee)
    Fr = fem.reduce_load(w.loads["c"])
    u32 = fem.solve(K, [Fr], rtol=1e-7)[0]
    rel32 = fem.relres[-1]
    u64 = fem.solve(K, [Fr], rtol=1e-11)[0]
    assert rel32 <= 1e-7 * 1.0001
    r = Fr - K @ u32  # the operator product on the host-facing side is the FP64 one
    assert np.linalg.norm(r) <= 1.5e-7 * np.linalg.norm(Fr)
    assert abs(float(Fr @ u32) / float(Fr @ u64) - 1) < 1e-8
    fem.close()


def test_operator_matmul_on_reduced_vectors(golden):
    g = golden("fem_small.npz")
    grid = _grid(tuple(int(s) for s in g["shape"]))
    fem = G.FEM(grid, g["active"], g["fixed"], 0.3)
    y = fem.assemble(g["Ee"]) @ g["u_red"]
    assert np.abs(y - g["y_red"]).max() <= 1e-6 * np.abs(g["y_red"]).max()
    fem.close()


def test_unsupported_part_raises_solver_error():
    """No fixed DOF: K is singular; the reference raises SolverError (fem.py:225-229)."""
    w = P.cantilever(8, 4, 4)
    fem = G.FEM(_grid(w.shape), w.active, np.zeros(0, int), 0.3)
    with pytest.raises(G.SolverError, match="did not converge"):
        fem.solve(fem.assemble(np.ones(w.nelem)), [fem.reduce_load(w.loads["c"])], rtol=1e-6, maxiter=200)
    fem.close()


def test_nonfinite_load_raises_solver_error():
    w = P.cantilever(8, 4, 4)
    fem = G.FEM(_grid(w.shape), w.active, w.fixed, 0.3)
    F = fem.reduce_load(w.loads["c"]).copy()
    F[len(F) // 2] = np.nan
    with pytest.raises(G.SolverError):
        fem.solve(fem.assemble(np.ones(w.nelem)), [F], rtol=1e-6, maxiter=200)
    fem.close()


def _simp_fixture(s, **kw):
    grid = _grid(tuple(int(v) for v in s["shape"]))
    return O.simp(grid, s["fill"], s["active"], s["frozen"], s["fixed"], {"down": s["F"]}, {"down": 1.0},
                  float(s["E0"]), float(s["nu"]), float(s["vf"]), iters=int(s["iters"]), log=lambda *a: None,
                  rtol=float(s["rtol"]), **kw)


def test_simp_default_path_matches_reference(golden):
    """Penalty ramp, projection continuation, frozen and partial-fill voxels (24 iterations)."""
    s = golden("simp_small_tight.npz")
    r = _simp_fixture(s)
    c = np.array([h["compliance"][0] for h in r["history"]])
    assert np.abs(c / s["h_compliance"][:, 0] - 1).max() < 1e-5
    assert np.abs(r["x"] - s["x"]).max() < 1e-3
    for k in ("p", "beta"):
        assert np.array_equal(np.array([h[k] for h in r["history"]]), s[f"h_{k}"])
    vol = np.array([h["volumeFraction"] for h in r["history"]])
    assert np.abs(vol - s["h_volumeFraction"]).max() < 1e-5


def test_simp_stock_tolerance_fp32_path(golden):
    """The reference's own CG tolerance (1e-6) on the FP32 solver, at the parity bars."""
    s = golden("simp_small.npz")
    r = _simp_fixture(s, precision="fp32")
    c = np.array([h["compliance"][0] for h in r["history"]])
    assert np.abs(c / s["h_compliance"][:, 0] - 1).max() < 1e-5
    assert np.abs(r["x"] - s["x"]).max() < 1e-3


def test_simp_worst_case_combine(golden):
    s = golden("simp_worst.npz")
    grid = _grid(tuple(int(v) for v in s["shape"]))
    r = O.simp(grid, s["fill"], s["active"], s["frozen"], s["fixed"], {"a": s["F1"], "b": s["F2"]},
               {"a": 1.0, "b": 2.0}, 1.0, 0.3, float(s["vf"]), iters=int(s["iters"]), r_mm=2.0,
               combine="worst", x0=s["x0"], log=lambda *a: None, rtol=1e-10)
    c = np.array([h["compliance"] for h in r["history"]])
    assert np.abs(c / s["h_compliance"] - 1).max() < 1e-5
    assert np.abs(r["x"] - s["x"]).max() < 1e-3


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_config1_cantilever_50_iterations(golden, precision):
    """48x24x24 cantilever, E_min 1e-9, p = 3, r = 1.5, vf = 0.3, CG rtol 1e-8, 50 iterations:
    compliance of every iteration within 1e-5 and the final density within 1e-3 (L-inf) of
    the reference's own run, on the FP32 operator (certified on the FP64 operator's residual)
    and on the FP64 operator."""
    s = golden("simp_config1.npz")
    w = P.cantilever(48, 24, 24)
    old = O.EMIN
    O.EMIN = 1e-9
    try:
        r = O.simp(_grid(w.shape), w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, 1.0, 0.3, 0.3,
                   iters=50, r_mm=1.5, p_final=3.0, move=0.2, tol=0.0, x0=np.full(w.nelem, 0.3),
                   beta_max=0.0, log=lambda *a: None, rtol=1e-8, precision=precision)
    finally:
        O.EMIN = old
    c = np.array([h["compliance"][0] for h in r["history"]])
    assert np.abs(c / s["h_compliance"][:, 0] - 1).max() < 1e-5
    assert np.abs(r["x"] - s["x"]).max() < 1e-3


def _lbracket_run(golden, name, scale):
    """The FP32 SimpRunner (the benchmarked path: FP32 operator and smoothers, FP64 CG scalars,
    solution and certification) on an L-bracket against the FP64 oracle's fixture."""
    import torch
    s = golden(name)
    w = P.lbracket(scale=scale, vf=0.25, r_vox=2.0, emin=1e-9)
    assert tuple(s["shape"]) == w.shape
    old = O.EMIN
    O.EMIN = 1e-9
    try:
        run = O.SimpRunner(_grid(w.shape), w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu,
                           w.vf, iters=int(s["iters"]), r_mm=w.r_vox, p_final=3.0, move=0.2,
                           x0=np.full(w.nelem, w.vf), beta_max=0.0, rtol=float(s["rtol"]), log=lambda *a: None,
                           precision="fp32")
        hist = [run.step() for _ in range(int(s["iters"]))]
        x = np.zeros(w.nelem)
        x[run.act] = run.xphys_t.cpu().numpy().astype(float)[run.act]
        assert not run.fem._ctxs.get(("fp64", 0, 1)), "an FP32 solve fell back to FP64"
        run.close()
        torch.cuda.empty_cache()
    finally:
        O.EMIN = old
    c = np.array([h["compliance"][0] for h in hist])
    vol = np.array([h["volumeFraction"] for h in hist])
    return s, c, vol, x


def test_history_start_saves_cg_iterations_at_the_same_results():
    """The opt-in CG start from the last two solutions (their Galerkin combination) against the
    reference's previous-solution start (optimize.py:122) on the FP32 path: fewer CG iterations
    over SIMP iterations 3-10, the same compliances and design within the parity bars."""
    import torch
    w = P.lbracket(scale=1 / 3, vf=0.25, r_vox=2.0, emin=1e-9)
    old = O.EMIN
    O.EMIN = 1e-9
    out = {}
    try:
        for start in ("previous", "history"):
            run = O.SimpRunner(_grid(w.shape), w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0,
                               w.nu, w.vf, iters=10, r_mm=w.r_vox, p_final=3.0, move=0.2,
                               x0=np.full(w.nelem, w.vf), beta_max=0.0, rtol=1e-6, log=lambda *a: None,
                               precision="fp32", cg_start=start)
            hist = [run.step() for _ in range(10)]
            out[start] = (np.array([h["cgIters"][0] for h in hist]), np.array([h["compliance"][0] for h in hist]),
                          run.xphys_t.cpu().numpy().astype(float))
            run.close()
            torch.cuda.empty_cache()
    finally:
        O.EMIN = old
    (cg_p, c_p, x_p), (cg_h, c_h, x_h) = out["previous"], out["history"]
    assert np.array_equal(cg_p[:2], cg_h[:2])  # the same start until two solutions exist
    assert cg_h[2:].sum() < cg_p[2:].sum(), (cg_h, cg_p)
    assert np.abs(c_h / c_p - 1).max() < 1e-5
    assert np.abs(x_h - x_p).max() < 1e-3


def test_config2_lbracket_192_fp32_30_iterations_match_oracle(golden):
    """Config 2: the 192x96x96 L-bracket (5.45M DOF), 30 iterations at CG rtol 1e-6: compliance
    of every iteration within 1e-5 and the final density within 1e-3 (L-inf) of the oracle."""
    s, c, vol, x = _lbracket_run(golden, "lbracket192_30it.npz", 1.0)
    assert np.abs(c / s["h_compliance"] - 1).max() < 1e-5
    assert np.abs(vol - s["h_volumeFraction"]).max() < 1e-5
    assert np.abs(x - s["x_q16"] / 65535.0).max() < 1e-3


def test_bench_workload_lbracket_256_fp32_first_iterations_match_oracle(golden):
    """The benchmarked workload: the 256x128x128 L-bracket (12.8M DOF) at CG rtol 1e-6, its first
    3 SIMP iterations against the oracle (compliance 1e-5, density 1e-3)."""
    s, c, vol, x = _lbracket_run(golden, "lbracket256_3it.npz", 4.0 / 3.0)
    assert np.abs(c / s["h_compliance"] - 1).max() < 1e-5
    assert np.abs(vol - s["h_volumeFraction"]).max() < 1e-5
    # every 17th element at the density bar; every element through its x-row's sum
    assert np.abs(x[::17] - s["x_q16_stride17"] / 65535.0).max() < 1e-3
    nx = int(s["shape"][0])
    assert np.abs(x.reshape(-1, nx).sum(axis=1) - s["row_sums"]).max() < 1e-3 * nx


def test_log_line_format_matches_reference(golden):
    """The per-iteration line is parsed by the reference GUI (gui/server.py:38-40)."""
    import os
    import re
    ref = open(os.path.join(os.path.dirname(__file__), "golden", "simp_small_tight_log.txt")).read().splitlines()
    pat = re.compile(r"^  it +(\d+)  p ([\d.]+)  b (\d+)  obj (\S+)  vol ([\d.]+)  change ([\d.]+)  "
                     r"grey ([\d.]+)  cg (\d+)( amg)?  ([\d.]+)s$")
    s = golden("simp_small_tight.npz")
    lines = []
    grid = _grid(tuple(int(v) for v in s["shape"]))
    O.simp(grid, s["fill"], s["active"], s["frozen"], s["fixed"], {"down": s["F"]}, {"down": 1.0},
           float(s["E0"]), float(s["nu"]), float(s["vf"]), iters=3, log=lines.append, rtol=1e-6)
    its = [l for l in lines if l.startswith("  it ")]
    assert len(its) == 3 and all(pat.match(l) for l in its)
    assert all(pat.match(l) for l in ref if l.startswith("  it "))


def test_six_load_cases_batched_match_one_by_one():
    """The batched multi-case solve (scalar-multiple cases folded, the rest solved at the
    same time on separate streams) against one solve per case."""
    import torch
    w = P.six_case_bracket(scale=1.0 / 6.0)
    grid = _grid(w.shape)
    fem = G.FEM(grid, w.active, w.fixed, 0.3)
    rng = np.random.default_rng(3)
    E = np.exp(rng.normal(0.0, 1.0, w.nelem)) * w.active
    escale = torch.as_tensor(E, dtype=torch.float32, device="cuda")
    mask = fem._mask_t.double()
    F = torch.stack([torch.as_tensor(w.loads[k], device="cuda") * mask for k in w.loads])
    X = torch.zeros_like(F)
    fem.solve_device(escale, F, X, rtol=1e-10)
    for i in range(F.shape[0]):
        Xi = torch.zeros_like(F[i:i + 1])
        fem.solve_device(escale, F[i:i + 1].clone(), Xi, rtol=1e-10)
        assert float((X[i] - Xi[0]).abs().max()) <= 1e-7 * float(Xi.abs().max())
    # the -x case is the +x solution negated, exactly
    assert torch.equal(X[1], -X[0])
    fem.close()


def test_fp32_batch_is_the_one_by_one_solve():
    """FP32 cases solved together in one context (a slot per case, every kernel advancing all
    of them) take exactly the iterates of their own solves: bit-identical solutions and the
    same CG iterations as one solve per case and as concurrent lanes. A zero load among them
    returns a zero solution in 0 iterations."""
    import torch
    w = P.six_case_bracket(scale=1.0 / 6.0)
    grid = _grid(w.shape)
    rng = np.random.default_rng(11)
    E = np.exp(rng.normal(0.0, 1.0, w.nelem)) * w.active
    escale = torch.as_tensor(E, dtype=torch.float32, device="cuda")
    res = {}
    for multi in ("batch", "lanes"):
        fem = G.FEM(grid, w.active, w.fixed, 0.3, precision="fp32", multi=multi)
        mask = fem._mask_t.double()
        F = torch.stack([torch.as_tensor(w.loads[k], device="cuda") * mask for k in w.loads] +
                        [torch.zeros_like(mask)])
        X = torch.zeros_like(F)
        its = fem.solve_device(escale, F, X, rtol=1e-6)
        res[multi] = (X, its, fem)
    Xb, itb, fem = res["batch"]
    Xl, itl, _ = res["lanes"]
    assert any(k[2] > 1 for k in fem._ctxs)  # the batched context was used
    assert itb == itl and torch.equal(Xb, Xl)
    assert itb[-1] == 0 and float(Xb[-1].abs().max()) == 0.0
    for i in range(Xb.shape[0] - 1):
        Xi = torch.zeros_like(Xb[i:i + 1])
        it = fem.solve_device(escale, (torch.as_tensor(w.loads[list(w.loads)[i]], device="cuda") *
                                       fem._mask_t.double())[None], Xi, rtol=1e-6)
        assert it[0] == itb[i] and torch.equal(Xi[0], Xb[i]), i
    for _, _, f in res.values():
        f.close()


def test_six_case_bracket_160_fp32_batch_matches_oracle(golden):
    """The six-case bracket at full size (160x80x80, 3.17M DOF per case) through the FP32
    batch (the three distinct cases in one context), its first 3 SIMP iterations against the
    oracle, which solves all six cases one after another: every case's compliance within
    1e-5, the density within 1e-3."""
    import torch
    s = golden("sixcase160_3it.npz")
    w = P.six_case_bracket(scale=5.0 / 6.0, vf=0.25, r_vox=2.0, emin=1e-9)
    assert tuple(s["shape"]) == w.shape
    old = O.EMIN
    O.EMIN = 1e-9
    try:
        run = O.SimpRunner(_grid(w.shape), w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu,
                           w.vf, iters=int(s["iters"]), r_mm=w.r_vox, p_final=3.0, move=0.2,
                           x0=np.full(w.nelem, w.vf), beta_max=0.0, rtol=float(s["rtol"]), log=lambda *a: None,
                           precision="fp32", multi="batch")
        hist = [run.step() for _ in range(int(s["iters"]))]
        x = np.zeros(w.nelem)
        x[run.act] = run.xphys_t.cpu().numpy().astype(float)[run.act]
        assert ("fp32", 0, 3) in run.fem._ctxs, "the three distinct cases were not batched"
        assert not run.fem._ctxs.get(("fp64", 0, 1)), "an FP32 solve fell back to FP64"
        run.close()
        torch.cuda.empty_cache()
    finally:
        O.EMIN = old
    c = np.array([h["compliance"] for h in hist])
    assert c.shape == s["h_compliance_cases"].shape
    assert np.abs(c / s["h_compliance_cases"] - 1).max() < 1e-5
    assert np.abs(np.array([h["volumeFraction"] for h in hist]) - s["h_volumeFraction"]).max() < 1e-5
    assert np.abs(x[::17] - s["x_q16_stride17"] / 65535.0).max() < 1e-3
    nx = int(s["shape"][0])
    assert np.abs(x.reshape(-1, nx).sum(axis=1) - s["row_sums"]).max() < 1e-3 * nx


def test_fp32_batch_is_the_one_by_one_solve_on_a_larger_grid():
    """At 128x64x64 the finest K u grid no longer fits one wave per right-hand side: each slot of
    a batch still gets the CTA partition of a single solve (its p.Kp sums follow the CTAs), so the
    batch stays bit-identical to one solve per case."""
    import torch
    w = P.six_case_bracket(scale=2.0 / 3.0)
    fem = G.FEM(_grid(w.shape), w.active, w.fixed, 0.3, precision="fp32")
    rho = P.random_density(w.shape, 12, active=w.active)
    E = torch.as_tensor((1e-9 + rho ** 3) * w.active, dtype=torch.float32, device="cuda")
    mask = fem._mask_t.double()
    keys = list(w.loads)[::2][:2]
    F = torch.stack([torch.as_tensor(w.loads[k], device="cuda") * mask for k in keys])
    X = torch.zeros_like(F)
    its = fem.solve_device(E, F, X, rtol=1e-6)
    for i in range(2):
        Xi = torch.zeros_like(F[i:i + 1])
        it = fem.solve_device(E, F[i:i + 1].clone(), Xi, rtol=1e-6)
        assert it[0] == its[i] and torch.equal(Xi[0], X[i]), i
    fem.close()


@pytest.mark.parametrize("precision,rtol", [("auto", 1e-8), ("fp32", 1e-6)])
def test_six_case_simp_matches_oracle(oracle, precision, rtol):
    """Six load cases (+-x, +-y, +-z: each negative case folded onto its positive one, the
    three distinct cases solved together) through four SIMP iterations: FP64 lanes at rtol
    1e-8 and the FP32 batch at rtol 1e-6."""
    w = P.six_case_bracket(scale=1.0 / 6.0)
    kw = dict(iters=4, r_mm=1.5, p_final=3.0, move=0.2, tol=0.0, x0=np.full(w.nelem, 0.25), beta_max=0.0,
              log=lambda *a: None, rtol=rtol)
    old = O.EMIN
    O.EMIN = 1e-9
    try:
        got = O.simp(_grid(w.shape), w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, 1.0, 0.3, 0.25,
                     precision=precision, **kw)
    finally:
        O.EMIN = old
    want = oracle.simp(w.shape, 1.0, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, 1.0, 0.3, 0.25,
                       emin=1e-9, **kw)
    cg = np.array([h["compliance"] for h in got["history"]])
    co = np.array([h["compliance"] for h in want["history"]])
    assert np.abs(cg / co - 1).max() < 1e-5
    assert np.abs(got["x"] - want["x"]).max() < 1e-3


def test_many_parts_in_lanes_match_one_by_one():
    """Independent parts run as concurrent lanes give exactly the results of running them one
    after another (the kernels are deterministic; lanes only overlap them)."""
    from anneal_gb300 import batch as B
    parts = B.seeded_parts(4, seed=5)
    parts = [P.cantilever(min(w.shape[0], 40), min(w.shape[1], 20), min(w.shape[2], 20), vf=w.vf, r_vox=w.r_vox,
                          emin=1e-9) for w in parts]
    _, seq = B.run_parts(parts, 3, 1)
    _, par = B.run_parts(parts, 3, 3)
    for a, b in zip(seq, par):
        assert a["compliance"] == b["compliance"] and a["shape"] == b["shape"]


def test_box_smoother_levels_match_the_marching_kernel(monkeypatch):
    """The V-cycle with the box kernels on the coarse levels (the default) against the same
    V-cycle on the z-marching K u kernel everywhere: the same solution to the tolerance and
    about the same CG iterations (only the summation order of the smoother's forces differs)."""
    import torch
    w = P.lbracket(scale=0.5, vf=0.25, r_vox=2.0, emin=1e-9)
    rho = P.random_density(w.shape, 7, active=w.active)
    out = {}
    for tag, box_from in (("box", "2"), ("march", "99")):
        monkeypatch.setenv("ANL_BOX_FROM", box_from)
        fem = G.FEM(_grid(w.shape), w.active, w.fixed, 0.3, precision="fp32")
        Ee = 1e-9 + rho[fem.act] ** 3 * (1 - 1e-9)
        K = fem.assemble(Ee)
        u = fem.solve(K, [fem.reduce_load(w.loads["down"])], rtol=1e-8)[0]
        out[tag] = (u, fem.cg_iters[-1], len(fem._ctx(False).mg_info()))
        fem.close()
        torch.cuda.empty_cache()
    (ub, ib, nlev), (um, im, _) = out["box"], out["march"]
    assert nlev >= 4
    assert np.abs(ub - um).max() <= 1e-6 * np.abs(um).max()
    assert abs(ib - im) <= max(2, im // 10), (ib, im)


def test_one_cta_vcycle_tail_matches_per_level_launches(monkeypatch):
    """The smallest multigrid levels and the coarsest solve in one CTA (the default) against the
    same levels as separate launches: the same solution to the tolerance and about the same CG
    iterations, on two grids (a cantilever and the L-bracket with its void)."""
    import torch
    for w in (P.cantilever(128, 64, 32), P.lbracket(scale=0.5, vf=0.25, r_vox=2.0, emin=1e-9)):
        rho = P.random_density(w.shape, 9, active=w.active)
        case = next(iter(w.loads))
        out = {}
        for tag, on in (("tail", "1"), ("launches", "0")):
            monkeypatch.setenv("ANL_TAIL", on)
            fem = G.FEM(_grid(w.shape), w.active, w.fixed, 0.3, precision="fp32")
            Ee = 1e-9 + rho[fem.act] ** 3 * (1 - 1e-9)
            u = fem.solve(fem.assemble(Ee), [fem.reduce_load(w.loads[case])], rtol=1e-8)[0]
            out[tag] = (u, fem.cg_iters[-1])
            fem.close()
            torch.cuda.empty_cache()
        (ut, it_t), (ul, it_l) = out["tail"], out["launches"]
        assert np.abs(ut - ul).max() <= 1e-6 * np.abs(ul).max()
        assert abs(it_t - it_l) <= max(2, it_l // 10), (w.name, it_t, it_l)
