"""Route an installed anneal (0.3.0) through the GPU path.

    import anneal_gb300.integrate as gi
    gi.install()          # before `anneal run` / `anneal validate` does its work

``install`` swaps the reference's solve and optimise entry points for the GPU ones in the
already imported (or importable) ``anneal`` package: ``anneal.fem.FEM`` / ``SolverError``,
``anneal.optimize.simp`` / ``Filter``, ``anneal.export.surface`` / ``output_field`` /
``choose_level`` / ``keep_load_paths`` / ``member_thickness``, the voxeliser
(``anneal.geometry.voxel_fill`` and the names ``problem.py`` and ``run.py`` bound), the names ``run.py`` bound
at import (``anneal.run.FEM``, ``anneal.run.simp`` and the export functions) and the solver
names the validation gate bound at import (``anneal.validate.FEM`` / ``Grid`` /
``hex8_matrices``), so the reference's own checks V1-V6 run against the GPU solver. Spec
parsing, the other export steps, the gate itself, reports and the database stay the
reference's.
"""
import importlib


_EXPORT_NAMES = ("surface", "output_field", "choose_level", "keep_load_paths", "member_thickness")


def install(anneal_pkg="anneal"):
    from . import fem as gfem
    from . import optimize as gopt
    fem = importlib.import_module(f"{anneal_pkg}.fem")
    opt = importlib.import_module(f"{anneal_pkg}.optimize")
    fem.FEM = gfem.FEM
    fem.SolverError = gfem.SolverError
    fem.hex8_matrices = gfem.hex8_matrices
    opt.FEM = gfem.FEM
    opt.simp = gopt.simp
    opt.Filter = gopt.Filter
    opt.benchmark_cantilever = gopt.benchmark_cantilever
    from . import export as gexp
    try:
        exp = importlib.import_module(f"{anneal_pkg}.export")
        for name in _EXPORT_NAMES:
            setattr(exp, name, getattr(gexp, name))
    except ImportError:   # export.py needs trimesh / skimage
        pass
    try:
        run = importlib.import_module(f"{anneal_pkg}.run")
        run.FEM = gfem.FEM
        run.simp = gopt.simp
        for name in _EXPORT_NAMES:   # run.py:16 binds them by name
            setattr(run, name, getattr(gexp, name))
    except ImportError:   # run.py needs trimesh / skimage / matplotlib
        pass
    from . import geometry as ggeo
    for mod in ("geometry", "problem", "run"):   # problem.py:16 and run.py:13 bind voxel_fill by name
        try:
            m = importlib.import_module(f"{anneal_pkg}.{mod}")
            m.voxel_fill = ggeo.voxel_fill
        except ImportError:   # geometry.py needs trimesh
            pass
    try:
        val = importlib.import_module(f"{anneal_pkg}.validate")   # validate.py:8 binds these by name
        val.FEM = gfem.FEM
        val.Grid = gfem.Grid
        val.hex8_matrices = gfem.hex8_matrices
    except ImportError:
        pass
    # keep the EMIN constant shared: the GPU simp reads anneal_gb300.optimize.EMIN
    gopt.EMIN = getattr(opt, "EMIN", gopt.EMIN)
    return True
