"""Generate the golden fixtures in this folder by running the reference implementation.

The reference is anneal 0.3.0 (pure Python). Its hot path lives in ``anneal/fem.py`` and
``anneal/optimize.py``. Two of its third-party imports are absent here and get stubs:

* ``pyamg`` (>=5.0, pyproject.toml:14): only a CG preconditioner
  (fem.py:212-215). The stub returns a Jacobi preconditioner. CG is still run to the
  reference's own relative residual, so converged answers do not depend on the stub
  beyond that tolerance.
* ``trimesh`` (>=4.0): imported at module level by geometry.py. The hot path never
  calls it, so the stub is an empty module.

Everything else (Ke, CSR assembly, scipy CG, the ndimage filter, the SIMP loop, OC,
the validation checks V1-V6) is the reference's unchanged code.

Run from the repository root, in a container that holds the reference tree:

    python tests/golden/make_golden.py [--ref /path/to/reference] [--skip-config1]

The config-1 fixture (48x24x24, 50 SIMP iterations, CG at rtol 1e-8 with Jacobi) takes
several minutes of CPU time. The other fixtures take seconds.
"""
import argparse
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def install_stubs(ref_root):
    import scipy.sparse.linalg as spla

    pyamg = types.ModuleType("pyamg")

    class _Jacobi:
        def __init__(self, K):
            self.d = K.diagonal().copy()

        def aspreconditioner(self, cycle="V"):
            d = self.d
            return spla.LinearOperator((d.size, d.size), matvec=lambda x: x / d)

    pyamg.smoothed_aggregation_solver = lambda K, **kw: _Jacobi(K)
    sys.modules["pyamg"] = pyamg
    sys.modules["trimesh"] = types.ModuleType("trimesh")
    sys.path.insert(0, ref_root)
    import anneal.fem as fem
    import anneal.optimize as optimize
    import anneal.validate as validate
    return fem, optimize, validate


def patch_simp_rtol(fem_mod, rtol):
    """simp() hard-codes rtol=1e-6 (optimize.py:122); wrap FEM.solve to force another rtol.
    Returns a callable that restores the original method."""
    orig = fem_mod.FEM.solve

    def wrapper(self, K, F_list, x0_list=None, rebuild=True, rtol=None, maxiter=None):
        return orig(self, K, F_list, x0_list=x0_list, rebuild=rebuild, rtol=rtol_forced,
                    maxiter=20000)

    rtol_forced = rtol
    fem_mod.FEM.solve = wrapper

    def restore():
        fem_mod.FEM.solve = orig
    return restore


def cantilever(fem_mod, nx, ny, nz, edge_z=0.0):
    """Clamp every node on x=0; total -1 in z spread over the nodes of the x=nx, z=edge_z line."""
    g = fem_mod.Grid((nx, ny, nz), 1.0, (0, 0, 0))
    n = np.arange(g.nnode)
    p = g.node_coords(n)
    clamp = n[p[:, 0] < 1e-9]
    fixed = (3 * clamp[:, None] + np.arange(3)).ravel()
    tip = n[(abs(p[:, 0] - nx) < 1e-9) & (abs(p[:, 2] - edge_z) < 1e-9)]
    F = np.zeros(3 * g.nnode)
    F[3 * tip + 2] = -1.0 / tip.size
    return g, fixed, F


def gen_ke(fem):
    out = {}
    for tag, nu, h in (("a", 0.3, 1.0), ("b", 0.3, 0.5), ("c", 0.25, 2.0)):
        ke, B0, D = fem.hex8_matrices(nu, h)
        out[f"ke_{tag}"] = ke
        out[f"B0_{tag}"] = B0
        out[f"D_{tag}"] = D
        out[f"nu_{tag}"] = nu
        out[f"h_{tag}"] = h
    np.savez_compressed(os.path.join(HERE, "ke.npz"), **out)


def gen_fem_small(fem):
    """Assembled K @ u, element energy and a tight solve on a small ragged domain."""
    rng = np.random.default_rng(7)
    g = fem.Grid((7, 5, 4), 1.0, (0, 0, 0))
    i, j, k = g.elem_ijk(np.arange(g.nelem))
    active = ~((i >= 4) & (k >= 2))            # an L-shaped domain: inactive voids
    active &= rng.random(g.nelem) > 0.08        # plus a few random holes
    act = np.flatnonzero(active)
    n = np.arange(g.nnode)
    p = g.node_coords(n)
    clamp = n[(p[:, 0] < 1e-9) & (p[:, 2] < 2.5)]
    fixed = np.concatenate([3 * clamp, 3 * clamp + 1, 3 * clamp + 2,
                            3 * n[(p[:, 0] < 1e-9) & (p[:, 2] > 2.5)] + 2])
    model = fem.FEM(g, active, fixed, 0.3)
    Ee = np.exp(rng.normal(0.0, 1.0, act.size)) * 0.5
    Ee[rng.random(act.size) < 0.2] = 1e-9      # some near-void elements
    K = model.assemble(Ee)
    u_red = rng.normal(0.0, 1.0, model.nfree)
    y_red = K @ u_red
    ce = model.element_energy(model.expand(u_red))
    F = np.zeros(3 * g.nnode)
    tip = n[(abs(p[:, 0] - 7) < 1e-9) & (p[:, 2] < 1e-9)]
    F[3 * tip + 2] = -1.0 / tip.size
    F[3 * tip + 1] = 0.25 / tip.size
    Fr = model.reduce_load(F)
    Ks = model.assemble(np.where(Ee < 1e-6, 1e-3, Ee))
    sol = model.solve(Ks, [Fr], rtol=1e-12, maxiter=20000)[0]
    np.savez_compressed(os.path.join(HERE, "fem_small.npz"), shape=np.array(g.shape), h=g.h,
                        active=active, fixed=fixed, Ee=Ee, free=model.free, u_red=u_red,
                        y_red=y_red, ce=ce, F=F, Ee_solve=np.where(Ee < 1e-6, 1e-3, Ee),
                        u_sol=sol, compliance=float(Fr @ sol), nnz=model.nnz)


def gen_filter(optimize, fem):
    rng = np.random.default_rng(11)
    g = fem.Grid((9, 7, 6), 1.0, (0, 0, 0))
    active = rng.random(g.nelem) > 0.15
    act = np.flatnonzero(active)
    out = {"shape": np.array(g.shape), "active": active}
    x = rng.random(act.size)
    d = rng.normal(0, 1, act.size)
    out["x"] = x
    out["d"] = d
    for tag, r in (("r15", 1.5), ("r20", 2.0), ("r26", 2.6), ("r31", 3.1)):
        f = optimize.Filter(g, active, r)
        out[f"fwd_{tag}"] = f.forward(x)
        out[f"bwd_{tag}"] = f.backward(d)
        out[f"k_{tag}"] = f.k
        out[f"Hs_{tag}"] = g.to1d(f.Hs)
    np.savez_compressed(os.path.join(HERE, "filter.npz"), **out)


def _hist_arrays(hist):
    keys = ("objective", "p", "beta", "volumeFraction", "change", "grey")
    out = {f"h_{k}": np.array([h[k] for h in hist], float) for k in keys}
    out["h_compliance"] = np.array([h["compliance"] for h in hist], float)
    out["h_amg"] = np.array([h["amgRebuilt"] for h in hist], bool)
    return out


def gen_simp_small(fem, optimize, rtol=None):
    """Default SIMP path (penalty ramp, projection continuation, frozen, partial fill).
    With ``rtol`` set, every CG solve inside simp runs to that tolerance instead of 1e-6."""
    restore = patch_simp_rtol(fem, rtol) if rtol else (lambda: None)
    tag = "simp_small_tight" if rtol else "simp_small"
    g, fixed, F = cantilever(fem, 16, 8, 8, edge_z=0.0)
    i, j, k = g.elem_ijk(np.arange(g.nelem))
    active = ~((i >= 10) & (k >= 5))
    fill = np.ones(g.nelem)
    fill[(k == 7) & active] = 0.6
    fill[~active] = 0.0
    frozen = (i == 15) & (k <= 1)
    logs = []
    res = optimize.simp(g, fill, active, frozen, fixed, {"down": F}, {"down": 1.0}, 70000.0, 0.33, 0.3,
                        iters=24, r_mm=None, log=logs.append)
    restore()
    np.savez_compressed(os.path.join(HERE, f"{tag}.npz"), shape=np.array(g.shape), fill=fill,
                        active=active, frozen=frozen, fixed=fixed, F=F, E0=70000.0, nu=0.33, vf=0.3,
                        iters=24, x=res["x"], rMM=res["rMM"], rtol=rtol or 1e-6,
                        **_hist_arrays(res["history"]))
    with open(os.path.join(HERE, f"{tag}_log.txt"), "w") as fh:
        fh.write("\n".join(logs) + "\n")


def gen_simp_worst(fem, optimize):
    """Two load cases combined by the p-norm ('worst'), warm start from a previous design.
    CG runs to rtol 1e-10 so the fixture pins the loop, not the preconditioner."""
    restore = patch_simp_rtol(fem, 1e-10)
    g, fixed, F1 = cantilever(fem, 12, 6, 6, edge_z=0.0)
    n = np.arange(g.nnode)
    p = g.node_coords(n)
    tip = n[(abs(p[:, 0] - 12) < 1e-9) & (abs(p[:, 2] - 6) < 1e-9)]
    F2 = np.zeros(3 * g.nnode)
    F2[3 * tip + 1] = 0.5 / tip.size
    active = np.ones(g.nelem, bool)
    fill = np.ones(g.nelem)
    frozen = np.zeros(g.nelem, bool)
    rng = np.random.default_rng(3)
    x0 = np.clip(0.3 + 0.2 * rng.normal(size=g.nelem), 0.0, 1.0)
    res = optimize.simp(g, fill, active, frozen, fixed, {"a": F1, "b": F2}, {"a": 1.0, "b": 2.0},
                        1.0, 0.3, 0.35, iters=16, r_mm=2.0, combine="worst", x0=x0,
                        log=lambda *a: None)
    restore()
    np.savez_compressed(os.path.join(HERE, "simp_worst.npz"), shape=np.array(g.shape), fill=fill,
                        active=active, frozen=frozen, fixed=fixed, F1=F1, F2=F2, x0=x0, vf=0.35,
                        iters=16, x=res["x"], **_hist_arrays(res["history"]))


def gen_config1(fem, optimize, iters=50):
    """The 48x24x24 cantilever in FP64: E0=1, Emin=1e-9, nu=0.3, p=3 from iteration 1
    (warm path with x0 = 0.3), no projection, r=1.5, vf=0.3, CG rtol 1e-8, 50 iterations."""
    optimize.EMIN = 1e-9
    restore = patch_simp_rtol(fem, 1e-8)
    g, fixed, F = cantilever(fem, 48, 24, 24, edge_z=0.0)
    active = np.ones(g.nelem, bool)
    fill = np.ones(g.nelem)
    frozen = np.zeros(g.nelem, bool)
    logs = []
    t0 = time.time()
    res = optimize.simp(g, fill, active, frozen, fixed, {"c": F}, {"c": 1.0}, 1.0, 0.3, 0.3,
                        iters=iters, r_mm=1.5, p_final=3.0, move=0.2, tol=0.0,
                        x0=np.full(g.nelem, 0.3), beta_max=0.0, log=logs.append)
    print(f"config1: {time.time() - t0:.0f} s")
    np.savez_compressed(os.path.join(HERE, "simp_config1.npz"), shape=np.array(g.shape),
                        fixed=fixed, F=F, iters=iters, x=res["x"], **_hist_arrays(res["history"]))
    with open(os.path.join(HERE, "simp_config1_log.txt"), "w") as fh:
        fh.write("\n".join(logs) + "\n")
    optimize.EMIN = 1e-6
    restore()


def gen_validate(validate):
    out = {}
    for fn in validate.CHECKS:
        name, ok, detail = fn()
        out[fn.__name__] = {"name": name, "ok": bool(ok), "detail": detail}
    ux, _ = validate._tension()
    out["_tension_ux"] = float(ux)
    ux_p, _ = validate._tension(fill_layer=0.4, nz=7)
    out["_partial_ux"] = float(ux_p)
    with open(os.path.join(HERE, "validate.json"), "w") as fh:
        json.dump(out, fh, indent=1)


def gen_stress(fem):
    """FEM.stress / von_mises / normal_stress (fem.py:244-263) on a cantilever solution, with
    a per-element modulus (h = 0.5) and a scalar one."""
    rng = np.random.default_rng(11)
    g = fem.Grid((9, 4, 5), 0.5, (1.0, -2.0, 0.5))
    active = rng.random(g.nelem) > 0.1
    n = np.arange(g.nnode)
    p = g.node_coords(n)
    clamp = n[p[:, 0] < 1.0 + 1e-9]
    fixed = (3 * clamp[:, None] + np.arange(3)).ravel()
    model = fem.FEM(g, active, fixed, 0.3)
    act = np.flatnonzero(active)
    Ee = np.exp(rng.normal(0.0, 0.5, act.size))
    F = np.zeros(3 * g.nnode)
    tip = n[(abs(p[:, 0] - (1.0 + 9 * 0.5)) < 1e-9)]
    F[3 * tip + 2] = -1.0 / tip.size
    F[3 * tip] = 0.3 / tip.size
    u = model.expand(model.solve(model.assemble(Ee), [model.reduce_load(F)], rtol=1e-12, maxiter=20000)[0])
    Emat = np.exp(rng.normal(0.0, 0.3, act.size)) * 2000.0
    sig = model.stress(u, Emat)
    np.savez_compressed(os.path.join(HERE, "stress.npz"), shape=np.array(g.shape), h=g.h, origin=g.origin,
                        active=active, fixed=fixed, u=u, Emat=Emat, sig=sig, vm=model.von_mises(u, Emat),
                        vm_scalar=model.von_mises(u, 1500.0), sn=model.normal_stress(sig, (0.2, -0.3, 1.0)))


def gen_voxel(ref_root):
    """geometry.voxel_fill (geometry.py:89-149) on closed meshes, an axis-aligned box whose top
    face lies on a sample plane, a seeded triangle soup and several sub-sample counts. The
    meshes come from anneal_gb300.geometry (icosphere, box), which stand in for
    trimesh.creation (absent here); voxel_fill reads only ``mesh.triangles``."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import anneal.fem as fem
    import anneal.geometry as geometry
    from anneal_gb300 import geometry as G

    class _M:
        def __init__(self, tri):
            self.triangles = tri

    def grid_around(V, h):  # test_core.py:31-36
        lo, hi = V.min(axis=0), V.max(axis=0)
        return fem.Grid(np.ceil((hi - lo + 2 * h) / h).astype(int), h, lo - h)

    rot = np.linalg.qr(np.random.default_rng(3).normal(size=(3, 3)))[0]
    cases = {}
    V, F = G.icosphere(4, 10.0)
    cases["sphere"] = (V[F], grid_around(V, 0.75), 3)
    V, F = G.box((5.0, 3.0, 2.0), (1.3, -0.7, 0.4), rot)
    cases["box_rot"] = (V[F], grid_around(V, 0.5), 3)
    V, F = G.box((3.0, 3.0, 1.5), (1.5, 1.5, 0.75))
    cases["box_plane"] = (V[F], fem.Grid((5, 5, 4), 1.0, (-1.0, -1.0, -1.0)), 3)
    tri = np.random.default_rng(5).uniform(-2.0, 2.0, size=(300, 3, 3))
    cases["soup"] = (tri, fem.Grid((11, 11, 11), 0.4, (-2.2, -2.2, -2.2)), 3)
    V, F = G.icosphere(3, 4.0, (0.3, -0.2, 0.1))
    cases["sphere_s2"] = (V[F], grid_around(V, 0.6), 2)
    cases["sphere_s5"] = (V[F], grid_around(V, 0.9), 5)
    out = {}
    for name, (tri, g, s) in cases.items():
        out[name + "_tri"] = tri
        out[name + "_shape"] = np.array(g.shape)
        out[name + "_h"] = g.h
        out[name + "_origin"] = np.asarray(g.origin, float)
        out[name + "_s"] = s
        out[name + "_fill"] = geometry.voxel_fill(_M(tri), g, s=s)
    out["names"] = np.array(list(cases))
    # a larger case kept as SHA-256 digests: the mesh (rebuilt by the test) and the fill bytes
    import hashlib
    V, F = G.icosphere(5, 0.45 * 64, (0.3 * 128, 32.0, 32.0))
    g = fem.Grid((128, 64, 64), 1.0, (0.0, 0.0, 0.0))
    fill = geometry.voxel_fill(_M(V[F]), g)
    out["big_tri_sha256"] = hashlib.sha256(np.ascontiguousarray(V[F]).tobytes()).hexdigest()
    out["big_fill_sha256"] = hashlib.sha256(fill.tobytes()).hexdigest()
    out["big_fill_sum"] = fill.sum()
    np.savez_compressed(os.path.join(HERE, "voxel.npz"), **out)


def post_problem(fem, bar, seed=0):
    """A small stand-in for the reference's Problem as export.py reads it: a 24 x 12 x 10 grid, a
    fixed sphere anchor at x = 2 and a load sphere anchor at x = 21 joined by a bar of density
    `bar` through a void-ish field; a keep-out slab and a frozen patch."""
    rng = np.random.default_rng(seed)
    g = fem.Grid((24, 12, 10), 1.0, (0.0, 0.0, 0.0))
    c = g.elem_centers()
    f = 0.3 * rng.random(g.nelem)
    blob_a = np.linalg.norm(c - np.array([2.0, 6.0, 5.0]), axis=1) < 3.0
    blob_b = np.linalg.norm(c - np.array([21.0, 6.0, 5.0]), axis=1) < 3.0
    bar_m = (np.abs(c[:, 1] - 6.0) < 1.0) & (np.abs(c[:, 2] - 5.0) < 1.0)
    f[blob_a | blob_b] = 0.9
    f[bar_m & ~(blob_a | blob_b)] = bar
    fill = np.where(rng.random(g.nelem) < 0.05, 0.5, 1.0)
    active = ~((c[:, 2] > 8.0) & (c[:, 0] > 10.0) & (c[:, 0] < 14.0))
    solid = np.where((c[:, 2] < 1.0) & (c[:, 0] < 3.0), 0.7, 0.0)
    void = np.where(c[:, 2] > 9.0, 0.4, 0.0)
    frozen = blob_a & (c[:, 0] < 1.0)
    sdfs = [np.linalg.norm(c - np.array([2.0, 6.0, 5.0]), axis=1) - 1.5,
            np.linalg.norm(c - np.array([21.0, 6.0, 5.0]), axis=1) - 1.5]
    return g, dict(f=f, fill=fill, active=active, solid_fill=solid, void_fill=void, frozen=frozen,
                   sdf_fixed=sdfs[0], sdf_load=sdfs[1], x=np.clip(f + 0.05, 0.0, 1.0))


def gen_post(ref_root):
    """export.output_field, choose_level and keep_load_paths (export.py:8-118) on small
    stand-in problems: stage 1 (level lowered), stage 2 (path repair), repair off, and an
    already connected part."""
    import types as T
    sk = T.ModuleType("skimage")
    sk.measure = T.ModuleType("skimage.measure")
    sys.modules.setdefault("skimage", sk)
    sys.modules.setdefault("skimage.measure", sk.measure)
    import anneal.fem as fem
    import anneal.export as export
    out = {}
    cases = {"stage1": (0.45, True), "stage2": (0.2, True), "norepair": (0.2, False), "connected": (0.8, True)}
    for name, (bar, repair) in cases.items():
        g, d = post_problem(fem, bar)
        prob = T.SimpleNamespace(grid=g, fill=d["fill"], active=d["active"], solid_fill=d["solid_fill"],
                                 void_fill=d["void_fill"], frozen=d["frozen"], anchors=[
                                     T.SimpleNamespace(name="clamp", role="fixed",
                                                       region=T.SimpleNamespace(sdf=lambda p, s=d["sdf_fixed"]: s)),
                                     T.SimpleNamespace(name="tip", role="load",
                                                       region=T.SimpleNamespace(sdf=lambda p, s=d["sdf_load"]: s))])
        fo = export.output_field(prob, d["x"])
        level = export.choose_level(prob, d["f"], d["x"])
        logs = []
        f2, level2 = export.keep_load_paths(prob, d["f"], 0.5, log=logs.append, repair=repair)
        for k, v in d.items():
            out[f"{name}_{k}"] = v
        out[f"{name}_output_field"] = fo
        out[f"{name}_level"] = level
        out[f"{name}_repair"] = repair
        out[f"{name}_kept_f"] = f2
        out[f"{name}_kept_level"] = level2
        out[f"{name}_log"] = np.array(logs if logs else [""])
    out["names"] = np.array(list(cases))
    out["shape"] = np.array([24, 12, 10])
    rng = np.random.default_rng(7)   # unclamped levels: targets near 0.45 and 0.62
    for i, scale in enumerate((0.9, 0.75)):
        lf, lx = rng.random(20000), rng.random(20000) * scale
        lfill = np.where(rng.random(20000) < 0.1, 0.5, 1.0)
        out[f"level{i}_f"], out[f"level{i}_x"], out[f"level{i}_fill"] = lf, lx, lfill
        out[f"level{i}_out"] = export.choose_level(T.SimpleNamespace(fill=lfill), lf, lx)
    np.savez_compressed(os.path.join(HERE, "post.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--skip-config1", action="store_true")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    fem, optimize, validate = install_stubs(a.ref)
    jobs = {"ke": lambda: gen_ke(fem), "fem_small": lambda: gen_fem_small(fem),
            "filter": lambda: gen_filter(optimize, fem),
            "simp_small": lambda: gen_simp_small(fem, optimize),
            "simp_small_tight": lambda: gen_simp_small(fem, optimize, rtol=1e-10),
            "simp_worst": lambda: gen_simp_worst(fem, optimize),
            "validate": lambda: gen_validate(validate), "stress": lambda: gen_stress(fem),
            "voxel": lambda: gen_voxel(a.ref), "post": lambda: gen_post(a.ref)}
    if not a.skip_config1:
        jobs["config1"] = lambda: gen_config1(fem, optimize)
    for name, fn in jobs.items():
        if a.only and name not in a.only.split(","):
            continue
        t0 = time.time()
        fn()
        print(f"{name}: {time.time() - t0:.1f} s")


if __name__ == "__main__":
    main()
