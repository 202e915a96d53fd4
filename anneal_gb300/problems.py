"""Synthetic voxel SIMP workloads.

These stand in for the spec files a user gives ``anneal run``: each builds the arrays
that the reference's ``Problem.build()`` / ``Problem.boundary()`` hand to ``simp``
(problem.py:168-326): element fill, active and frozen masks, fixed DOFs and one nodal
load vector per case. Grid conventions follow fem.py:87-127 (x fastest, DOF = 3*node+c).

Workloads:

* ``cantilever(nx, ny, nz)`` -- every node of the x=0 face clamped, a total force of -1
  in z spread equally over the nodes of the (x=nx, z=0) edge line.
* ``lbracket(scale)`` -- at scale 1: 192x96x96 voxels, passive void x>96 and z>48
  (inactive), clamped nodes in two round patches of radius 6 on the x=0 face centred at
  (y=24, z=48) and (y=72, z=48), each wrapped by a 2-voxel frozen (keep-solid) shell,
  a total force of -1 in z over a round patch of radius 4 on the top of the lower arm
  centred at (x=180, y=48). Every length scales with ``scale`` (4/3 gives 256x128x128).
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    shape: tuple
    h: float
    fill: np.ndarray
    active: np.ndarray
    frozen: np.ndarray
    fixed: np.ndarray
    loads: dict
    weights: dict
    E0: float = 1.0
    nu: float = 0.3
    vf: float = 0.3
    r_vox: float = 1.5
    emin: float = 1e-9
    extra: dict = field(default_factory=dict)

    @property
    def nelem(self):
        return int(np.prod(self.shape))

    @property
    def nnode(self):
        return int(np.prod([s + 1 for s in self.shape]))

    @property
    def ndof(self):
        return 3 * self.nnode


def _node_ijk(shape):
    nx, ny, nz = shape
    n = np.arange((nx + 1) * (ny + 1) * (nz + 1))
    return n, n % (nx + 1), (n // (nx + 1)) % (ny + 1), n // ((nx + 1) * (ny + 1))


def _elem_ijk(shape):
    nx, ny, nz = shape
    e = np.arange(nx * ny * nz)
    return e, e % nx, (e // nx) % ny, e // (nx * ny)


def used_nodes(shape, active):
    """Nodes touched by at least one active element (fem.py:145)."""
    nx, ny, nz = shape
    a3 = np.asarray(active, bool).reshape(nz, ny, nx)
    u = np.zeros((nz + 1, ny + 1, nx + 1), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                u[dz:dz + nz, dy:dy + ny, dx:dx + nx] |= a3
    return u.ravel()


def cantilever(nx=48, ny=24, nz=24, vf=0.3, r_vox=1.5, E0=1.0, nu=0.3, emin=1e-9):
    shape = (nx, ny, nz)
    n, i, j, k = _node_ijk(shape)
    clamp = n[i == 0]
    fixed = (3 * clamp[:, None] + np.arange(3)).ravel()
    tip = n[(i == nx) & (k == 0)]
    F = np.zeros(3 * n.size)
    F[3 * tip + 2] = -1.0 / tip.size
    ne = nx * ny * nz
    return Workload(f"cantilever-{nx}x{ny}x{nz}", shape, 1.0, np.ones(ne), np.ones(ne, bool),
                    np.zeros(ne, bool), fixed, {"c": F}, {"c": 1.0}, E0=E0, nu=nu, vf=vf,
                    r_vox=r_vox, emin=emin)


def _disc_sdf_x0(px, py, pz, cy, cz, r):
    """Distance to the disc {x = 0, (y-cy)^2 + (z-cz)^2 <= r^2}."""
    rho = np.sqrt((py - cy) ** 2 + (pz - cz) ** 2)
    return np.sqrt(px ** 2 + np.maximum(rho - r, 0.0) ** 2)


def lbracket(scale=1.0, vf=0.25, r_vox=2.0, E0=1.0, nu=0.3, emin=1e-9, load_dirs=None):
    """L-bracket; ``load_dirs`` (list of 3-vectors) makes one load case per direction on the
    same top patch instead of the single -z case."""
    s = float(scale)
    nx, ny, nz = int(round(192 * s)), int(round(96 * s)), int(round(96 * s))
    shape = (nx, ny, nz)
    xv, zv = 96 * s, 48 * s
    e, ei, ej, ek = _elem_ijk(shape)
    cx, cy, cz = ei + 0.5, ej + 0.5, ek + 0.5
    active = ~((cx > xv) & (cz > zv))
    n, ni, nj, nk = _node_ijk(shape)
    used = used_nodes(shape, active)
    patches = [(24 * s, 48 * s), (72 * s, 48 * s)]
    r_clamp = 6 * s
    clamp = np.zeros(n.size, bool)
    for (py, pz) in patches:
        clamp |= (ni == 0) & ((nj - py) ** 2 + (nk - pz) ** 2 <= r_clamp ** 2 + 1e-9)
    clamp &= used
    fixed = (3 * n[clamp][:, None] + np.arange(3)).ravel()
    shell = 2 * s
    frozen = np.zeros(e.size, bool)
    for (py, pz) in patches:
        frozen |= _disc_sdf_x0(cx, cy, cz, py, pz, r_clamp) <= shell
    frozen &= active
    lx, ly, r_load = 180 * s, 48 * s, 4 * s
    top = (nk == int(round(zv))) & ((ni - lx) ** 2 + (nj - ly) ** 2 <= r_load ** 2 + 1e-9) & used
    tn = n[top]
    dirs = load_dirs if load_dirs is not None else [(0.0, 0.0, -1.0)]
    loads, weights = {}, {}
    for c, d in enumerate(dirs):
        F = np.zeros(3 * n.size)
        for comp in range(3):
            F[3 * tn + comp] = d[comp] / tn.size
        name = "down" if load_dirs is None else f"case{c}"
        loads[name] = F
        weights[name] = 1.0
    fill = active.astype(float)
    return Workload(f"lbracket-{nx}x{ny}x{nz}", shape, 1.0, fill, active, frozen, fixed, loads, weights,
                    E0=E0, nu=nu, vf=vf, r_vox=r_vox, emin=emin,
                    extra={"clamp_nodes": int(clamp.sum()), "load_nodes": int(tn.size)})


def six_case_bracket(scale=5.0 / 6.0, **kw):
    """Six load cases (unit force along +-x, +-y, +-z on the top patch) on the bracket grid;
    scale 5/6 gives 160x80x80."""
    dirs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    return lbracket(scale=scale, load_dirs=[tuple(float(v) for v in d) for d in dirs], **kw)


def random_density(shape, seed, active=None):
    """rho = clip(0.3 * exp(N(0, 1)), 1e-3, 1) with numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    rho = np.clip(0.3 * np.exp(rng.normal(0.0, 1.0, int(np.prod(shape)))), 1e-3, 1.0)
    if active is not None:
        rho = np.where(active, rho, 0.0)
    return rho
