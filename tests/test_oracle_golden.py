"""The CPU oracle against the golden fixtures generated by running the reference
(tests/golden/make_golden.py). These pin the oracle before it checks the GPU path."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_ke_matches_reference(golden, oracle):
    g = golden("ke.npz")
    for t in "abc":
        ke = oracle.hex8_ke(float(g[f"nu_{t}"]), float(g[f"h_{t}"]))
        assert np.abs(ke - g[f"ke_{t}"]).max() < 1e-14


def test_free_dofs_match_reference(golden, oracle):
    g = golden("fem_small.npz")
    fem = oracle.OracleFEM(tuple(g["shape"]), 1.0, g["active"], g["fixed"], 0.3)
    assert np.array_equal(fem.free, g["free"])


def test_operator_and_energy_match_reference(golden, oracle):
    g = golden("fem_small.npz")
    fem = oracle.OracleFEM(tuple(g["shape"]), 1.0, g["active"], g["fixed"], 0.3)
    u = np.zeros(3 * fem.nnode)
    u[fem.free] = g["u_red"]
    y = fem.apply(g["Ee"], u)
    assert np.abs(y[fem.free] - g["y_red"]).max() <= 1e-13 * np.abs(g["y_red"]).max()
    ce = fem.element_energy(u)
    assert np.abs(ce - g["ce"]).max() <= 1e-13 * np.abs(g["ce"]).max()


@pytest.mark.parametrize("precond", ["jacobi", "mg"])
def test_solve_matches_reference(golden, oracle, precond):
    g = golden("fem_small.npz")
    fem = oracle.OracleFEM(tuple(g["shape"]), 1.0, g["active"], g["fixed"], 0.3)
    u = fem.solve(g["Ee_solve"], [g["F"]], rtol=1e-12, maxiter=20000, precond=precond)[0]
    c = float(np.where(fem.mask, g["F"], 0.0) @ u)
    assert abs(c / float(g["compliance"]) - 1) < 1e-10
    assert np.abs(u[fem.free] - g["u_sol"]).max() <= 1e-10 * np.abs(g["u_sol"]).max()


@pytest.mark.parametrize("tag,r", [("r15", 1.5), ("r20", 2.0), ("r26", 2.6), ("r31", 3.1)])
def test_filter_matches_reference(golden, oracle, tag, r):
    f = golden("filter.npz")
    F = oracle.OracleFilter(tuple(f["shape"]), f["active"], r)
    assert np.abs(F.Hs - f[f"Hs_{tag}"]).max() < 1e-12
    assert np.abs(F.forward(f["x"]) - f[f"fwd_{tag}"]).max() < 1e-13
    assert np.abs(F.backward(f["d"]) - f[f"bwd_{tag}"]).max() < 1e-13


def _run_simp_fixture(oracle, s, **kw):
    return oracle.simp(tuple(s["shape"]), 1.0, s["fill"], s["active"], s["frozen"], s["fixed"],
                       {"down": s["F"]}, {"down": 1.0}, float(s["E0"]), float(s["nu"]), float(s["vf"]),
                       iters=int(s["iters"]), log=lambda *a: None, rtol=float(s["rtol"]), **kw)


def test_simp_default_path_tight(golden, oracle):
    """Penalty ramp, projection continuation, frozen and partial-fill voxels; CG at 1e-10."""
    s = golden("simp_small_tight.npz")
    r = _run_simp_fixture(oracle, s)
    c = np.array([h["compliance"][0] for h in r["history"]])
    assert np.abs(c / s["h_compliance"][:, 0] - 1).max() < 1e-8
    assert np.abs(r["x"] - s["x"]).max() < 1e-7
    for k in ("p", "beta"):
        assert np.array_equal(np.array([h[k] for h in r["history"]]), s[f"h_{k}"])


def test_simp_default_path_stock_rtol(golden, oracle):
    """The reference's own tolerance (1e-6) with a different preconditioner."""
    s = golden("simp_small.npz")
    r = _run_simp_fixture(oracle, s)
    c = np.array([h["compliance"][0] for h in r["history"]])
    assert np.abs(c / s["h_compliance"][:, 0] - 1).max() < 1e-5
    assert np.abs(r["x"] - s["x"]).max() < 1e-3


def test_simp_worst_case_combine(golden, oracle):
    s = golden("simp_worst.npz")
    r = oracle.simp(tuple(s["shape"]), 1.0, s["fill"], s["active"], s["frozen"], s["fixed"],
                    {"a": s["F1"], "b": s["F2"]}, {"a": 1.0, "b": 2.0}, 1.0, 0.3, float(s["vf"]),
                    iters=int(s["iters"]), r_mm=2.0, combine="worst", x0=s["x0"], log=lambda *a: None,
                    rtol=1e-10)
    c = np.array([h["compliance"] for h in r["history"]])
    assert np.abs(c / s["h_compliance"] - 1).max() < 1e-8
    assert np.abs(np.array([h["objective"] for h in r["history"]]) / s["h_objective"] - 1).max() < 1e-8
    assert np.abs(r["x"] - s["x"]).max() < 1e-7


@pytest.mark.skipif(not os.path.isfile(os.path.join(GOLDEN, "simp_config1.npz")), reason="fixture absent")
def test_config1_cantilever_50_iterations(golden, oracle):
    """48x24x24 cantilever, 50 iterations, CG rtol 1e-8: the reference's own run."""
    from anneal_gb300 import problems as P
    s = golden("simp_config1.npz")
    w = P.cantilever(48, 24, 24)
    assert np.array_equal(np.sort(w.fixed), np.sort(s["fixed"]))
    assert np.array_equal(w.loads["c"], s["F"])
    r = oracle.simp(w.shape, 1.0, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, 1.0, 0.3, 0.3,
                    iters=50, r_mm=1.5, p_final=3.0, move=0.2, tol=0.0, x0=np.full(w.nelem, 0.3),
                    beta_max=0.0, log=lambda *a: None, rtol=1e-8, emin=1e-9)
    c = np.array([h["compliance"][0] for h in r["history"]])
    assert np.abs(c / s["h_compliance"][:, 0] - 1).max() < 1e-6
    assert np.abs(r["x"] - s["x"]).max() < 1e-4


def test_validation_values_recorded():
    with open(os.path.join(GOLDEN, "validate.json")) as fh:
        v = json.load(fh)
    assert all(v[k]["ok"] for k in v if k.startswith("check_"))
    assert abs(v["_tension_ux"] - 0.125) < 1e-10
