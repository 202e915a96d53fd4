"""anneal_gb300.integrate.install swaps every hot-path name in a reference-shaped package
(a stand-in package here: the module layout and the names run.py, problem.py bind at import)."""
import sys
import types

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
    mods["validate"].CHECKS = []
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
        assert len(mods["validate"].CHECKS) == 6
    finally:
        for k in [k for k in sys.modules if k.startswith("fake_anneal_pkg")]:
            del sys.modules[k]
