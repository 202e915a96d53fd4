"""Host-side logic on the CPU: the continuation schedule against the reference's recorded runs,
the CG start's Galerkin rule, the synthetic workloads' sizes, the benchmark's byte counts, the
element matrices against the reference's golden values and the grid against the reference's
own Grid (where its source tree is present)."""
import numpy as np
import pytest

from anneal_gb300 import optimize as O
from anneal_gb300 import problems as P


def _schedule(iters, warm, beta_max, n, p_final=3.0):
    """(p, beta) of SIMP iterations 1..n through SimpRunner's own state machine."""
    r = O.SimpRunner.__new__(O.SimpRunner)
    r.iters, r.p_final, r.warm, r.beta_max = iters, p_final, warm, beta_max
    r.beta = beta_max / 2 if warm else 0.0
    r.beta_since = 0
    r.beta_step = max(5, int(0.12 * iters))
    out = [r._advance_continuation(it) for it in range(1, n + 1)]
    return np.array([p for p, _ in out]), np.array([b for _, b in out])


@pytest.mark.parametrize("name, warm, beta_max", [
    ("simp_small.npz", False, O.BETA_MAX),        # penalty ramp, then projection continuation
    ("simp_small_tight.npz", False, O.BETA_MAX),
    ("simp_worst.npz", True, O.BETA_MAX),         # warm start: p final, beta_max / 2 throughout
    ("simp_config1.npz", True, 0.0),              # warm start without projection
])
def test_continuation_matches_the_reference_history(golden, name, warm, beta_max):
    """optimize.py:105-116: the p and beta of every iteration of the reference's own runs."""
    g = golden(name)
    n = len(g["h_p"])
    p, beta = _schedule(int(g["iters"]), warm, beta_max, n)
    assert np.array_equal(p, g["h_p"])
    assert np.array_equal(beta, g["h_beta"])


def test_galerkin_coefficients_minimise_the_energy():
    rng = np.random.default_rng(3)
    for _ in range(200):
        A = rng.normal(size=(2, 2))
        G = A @ A.T + 0.05 * np.eye(2)
        r = rng.normal(size=2)
        c = O.galerkin_coefficients(G[0, 0], G[0, 1], G[1, 1], r[0], r[1])
        pi_u1 = 0.5 * G[0, 0] - r[0]
        best = np.linalg.solve(G, r)
        if -0.5 * best @ r <= pi_u1 and np.linalg.det(G) > 1e-4 * G[0, 0] * G[1, 1]:
            assert c is not None and np.allclose(c, best, rtol=1e-10, atol=1e-12)
            assert -0.5 * np.dot(c, r) <= pi_u1 + 1e-12
    # the start stays u1 where the two directions cannot be resolved or a value is not finite
    assert O.galerkin_coefficients(1.0, 0.0, 1e-13, 1.0, 0.0) is None
    assert O.galerkin_coefficients(1.0, 0.99999, 1.0, 1.0, 1.0) is None
    assert O.galerkin_coefficients(1.0, 0.0, 1.0, float("nan"), 0.0) is None
    assert O.galerkin_coefficients(-1.0, 0.0, 1.0, 1.0, 0.0) is None
    # d orthogonal to u1 in the K inner product: each direction takes its own projection
    assert np.allclose(O.galerkin_coefficients(2.0, 0.0, 4.0, 1.0, 2.0), (0.5, 0.5))


def test_workloads_have_the_stated_sizes():
    """The configurations' sizes: 48x24x24 cantilever (27,648 elements, 91,875 DOF), the
    192x96x96 L-bracket (1,327,104 of 1,769,472 elements active, 5,447,811 DOF), the same at
    256x128x128 (3,145,728 of 4,194,304, 12,830,211 DOF), the six-case bracket at 160x80x80
    (1,024,000 elements, 3,168,963 DOF, six load cases)."""
    c = P.cantilever()
    assert c.shape == (48, 24, 24) and c.nelem == 27648 and c.ndof == 91875
    for scale, shape, act, dof in ((1.0, (192, 96, 96), 1327104, 5447811),
                                   (4 / 3, (256, 128, 128), 3145728, 12830211)):
        w = P.lbracket(scale=scale)
        assert w.shape == shape and int(np.asarray(w.active).sum()) == act and w.ndof == dof
        assert len(w.loads) == 1
        F = next(iter(w.loads.values()))
        assert abs(F.sum() + 1.0) < 1e-12 and np.all(F[0::3] == 0) and np.all(F[1::3] == 0)
    s = P.six_case_bracket()
    assert s.shape == (160, 80, 80) and s.nelem == 1024000 and s.ndof == 3168963 and len(s.loads) == 6


def test_bench_byte_counts():
    """The benchmark's algorithmic bytes per finest-level pass at 256x128x128: K u is
    24 N_n + 4 N_e = 119.4 MB (u and y as FP32 nodes, E as FP32 elements)."""
    import bench
    nn, ne = 257 * 129 * 129, 256 * 128 * 128
    by = {name: f(nn, ne) for _, name, _, f in bench.PASSES}
    assert by["K u"] == 24 * nn + 4 * ne and abs(by["K u"] / 1e6 - 119.4) < 0.05
    assert by["residual b - K x"] == 36 * nn + 4 * ne
    assert by["last Chebyshev step of a sweep"] == by["first Chebyshev step after the prolongation"] == 52 * nn + 4 * ne
    assert by["first two Chebyshev steps"] == 28 * nn + 4 * ne
    assert bench.KU_DENSE_FLOPS == 1152


def test_hex8_matrices_match_the_reference_golden(golden):
    """fem.py:71-84: Ke, B0 and D of the reference for three (nu, h)."""
    from anneal_gb300 import fem
    g = golden("ke.npz")
    for t in "abc":
        ke, B0, D = fem.hex8_matrices(float(g[f"nu_{t}"]), float(g[f"h_{t}"]))
        for got, key in ((ke, "ke"), (B0, "B0"), (D, "D")):
            want = g[f"{key}_{t}"]
            assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max(), (key, t)


REF = "/root/reference"


@pytest.mark.skipif(not __import__("os").path.isfile(REF + "/anneal/fem.py"),
                    reason="reference tree not present on this machine")
def test_grid_matches_the_reference_grid():
    """fem.py:87-127: element nodes, node coordinates, element centres and the flat <-> [i, j, k]
    maps of the reference's own Grid, on a ragged grid with an offset origin."""
    import os
    import sys
    from anneal_gb300 import fem
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    saved = {k: sys.modules[k] for k in list(sys.modules) if k == "anneal" or k.startswith("anneal.")
             or k in ("pyamg", "trimesh")}
    try:
        import make_golden
        rfem, _, _ = make_golden.install_stubs(REF)
        shape, h, origin = (7, 5, 4), 0.37, (1.5, -2.0, 0.25)
        a, b = fem.Grid(shape, h, origin), rfem.Grid(shape, h, origin)
        assert (a.nelem, a.nnode, a.shape) == (b.nelem, b.nnode, b.shape)
        e = np.arange(a.nelem)
        n = np.arange(a.nnode)
        assert np.array_equal(a.element_nodes(e), b.element_nodes(e))
        assert np.array_equal(a.node_coords(n), b.node_coords(n))
        assert np.array_equal(a.elem_centers(), b.elem_centers())
        f = np.random.default_rng(0).random(a.nelem)
        assert np.array_equal(a.to3d(f), b.to3d(f)) and np.array_equal(a.to1d(a.to3d(f)), f)
    finally:
        for k in [k for k in sys.modules if k == "anneal" or k.startswith("anneal.") or k in ("pyamg", "trimesh")]:
            del sys.modules[k]
        sys.modules.update(saved)


def test_many_part_set_is_seeded_and_in_range():
    """The many-part set: 32 seeded cantilevers, nx in [32, 128], ny and nz in [16, 64], volume
    fraction in [0.2, 0.4], filter radius in [1.2, 2.5]; 16.0M DOF in total for seed 0."""
    from anneal_gb300 import batch as B
    a, b = B.seeded_parts(32, 0), B.seeded_parts(32, 0)
    assert [p.shape for p in a] == [p.shape for p in b]
    for p in a:
        nx, ny, nz = p.shape
        assert 32 <= nx <= 128 and 16 <= ny <= 64 and 16 <= nz <= 64
        assert 0.2 <= p.vf <= 0.4 and 1.2 <= p.r_vox <= 2.5
    assert abs(sum(p.ndof for p in a) / 1e6 - 16.0) < 0.05
