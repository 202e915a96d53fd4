"""anneal_gb300.integrate.install swaps every hot-path name in a reference-shaped package: a
stand-in package with the module layout and the names run.py, problem.py and validate.py bind at
import, and, where the reference tree is present on this machine, the reference package itself
(imported with its absent third-party modules stubbed, as tests/golden/make_golden.py does).
Neither test runs a solve: they check the wiring only."""
import os
import sys
import types

import pytest

import anneal_gb300.integrate as gi


def _fake_package(name):
    pkg = types.ModuleType(name)
    pkg.__path__ = []
    sys.modules[name] = pkg
    mods = {}
    for m in ("fem", "optimize", "export", "geometry", "problem", "run", "validate"):
        mod = types.ModuleType(f"{name}.{m}")
        sys.modules[f"{name}.{m}"] = mod
        setattr(pkg, m, mod)
        mods[m] = mod
    mods["optimize"].EMIN = 1e-9
    mods["validate"].CHECKS = ["stays"]
    return mods


def test_install_replaces_every_name():
    mods = _fake_package("fake_anneal_pkg")
    try:
        assert gi.install("fake_anneal_pkg")
        from anneal_gb300 import export, fem, geometry, optimize
        assert mods["fem"].FEM is fem.FEM and mods["optimize"].simp is optimize.simp
        assert mods["optimize"].Filter is optimize.Filter
        for n in ("surface", "output_field", "choose_level", "keep_load_paths", "member_thickness"):
            assert getattr(mods["export"], n) is getattr(export, n)
            assert getattr(mods["run"], n) is getattr(export, n)
        for m in ("geometry", "problem", "run"):
            assert mods[m].voxel_fill is geometry.voxel_fill
        assert mods["run"].FEM is fem.FEM and mods["run"].simp is optimize.simp
        # the gate keeps its own checks; only the solver names it bound are swapped
        assert mods["validate"].CHECKS == ["stays"]
        assert mods["validate"].FEM is fem.FEM and mods["validate"].hex8_matrices is fem.hex8_matrices
    finally:
        for k in [k for k in sys.modules if k.startswith("fake_anneal_pkg")]:
            del sys.modules[k]


REF = "/root/reference"


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "anneal", "validate.py")),
                    reason="reference tree not present on this machine")
def test_install_on_the_reference_package():
    """The reference's own validate module, after install(), reaches the GPU FEM through the
    names it bound at import; its check functions and CHECKS list are untouched."""
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    saved = {k: sys.modules[k] for k in list(sys.modules) if k == "anneal" or k.startswith("anneal.")
             or k in ("pyamg", "trimesh")}
    try:
        import make_golden
        _, _, validate = make_golden.install_stubs(REF)
        checks = list(validate.CHECKS)
        assert gi.install("anneal")
        from anneal_gb300 import fem, optimize
        import anneal.optimize as ropt
        assert validate.FEM is fem.FEM and validate.Grid is fem.Grid
        assert validate.hex8_matrices is fem.hex8_matrices
        assert ropt.simp is optimize.simp and ropt.benchmark_cantilever is optimize.benchmark_cantilever
        assert validate.CHECKS == checks and all(c.__module__ == "anneal.validate" for c in checks)
    finally:
        for k in [k for k in sys.modules if k == "anneal" or k.startswith("anneal.") or k in ("pyamg", "trimesh")]:
            del sys.modules[k]
        sys.modules.update(saved)
        if REF in sys.path:
            sys.path.remove(REF)
        sys.path.pop(0)
