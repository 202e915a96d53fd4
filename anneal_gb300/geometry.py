"""Voxelisation with the interface of anneal's geometry.voxel_fill (geometry.py:89-149).

``voxel_fill(mesh, grid, s=3, chunk=...)`` returns the fill fraction (0..1) of every grid
element inside a closed triangle mesh, by ray parity along z at s x s x s sample points per
element: the reference's method and its rounding, so the result is bit-identical. The work
runs in the CUDA library (``anl_voxel_fill``): a per-triangle count of the sample columns in
its bounding box, a scan, one thread per (triangle, column) pair for the barycentric test,
crossings recorded as bit flips and a prefix XOR per column. ``chunk`` is accepted for the
reference's signature; the GPU needs no chunking.

``icosphere`` and ``box`` build the closed meshes that ``trimesh.creation`` gives the
reference's tests (trimesh is not needed here).
"""
import ctypes
import math
import threading

import numpy as np
import torch

from . import _native as N
from .context import require_cuda


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Voxeliser:
    """The device workspace of the voxeliser (anl_vox): it keeps its buffers between calls."""

    def __init__(self):
        require_cuda()
        h = ctypes.c_void_p()
        N.call("anl_vox_create", ctypes.byref(h))
        self.h = h
        self.pairs = 0
        self.hits = 0

    def close(self):
        if self.h:
            N.load().anl_vox_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fill_device(self, tri, shape, h, origin, s=3, stats=False):
        """tri: (n, 3, 3) float64 CUDA tensor. Returns the (nx*ny*nz,) float64 fill fractions
        (x fastest) as a CUDA tensor. With stats, also records the pair and crossing counts
        (one synchronisation)."""
        nx, ny, nz = (int(v) for v in shape)
        tri = tri.contiguous()
        if tri.dtype != torch.float64 or tri.dim() != 3 or tuple(tri.shape[1:]) != (3, 3):
            raise ValueError("triangles must be an (n, 3, 3) float64 tensor")
        if tri.shape[0] == 0:
            raise ValueError("the mesh has no triangles")
        out = torch.empty(nx * ny * nz, dtype=torch.float64, device=tri.device)
        org = (ctypes.c_double * 3)(*[float(o) for o in origin])
        st = (ctypes.c_int64 * 2)() if stats else None
        N.call("anl_voxel_fill", self.h, ctypes.c_void_p(tri.data_ptr()), int(tri.shape[0]), nx, ny, nz,
               float(h), org, int(s), ctypes.c_void_p(out.data_ptr()), st, _stream())
        if stats:
            self.pairs, self.hits = int(st[0]), int(st[1])
        return out


_local = threading.local()


def _voxeliser():
    v = getattr(_local, "vox", None)
    if v is None:
        v = _local.vox = Voxeliser()
    return v


def triangles_of(mesh):
    """(n, 3, 3) float64 vertex coordinates of a mesh object (``.triangles``, or ``.vertices``
    and ``.faces``) or of an array that already has that shape."""
    if hasattr(mesh, "triangles"):
        t = mesh.triangles
    elif hasattr(mesh, "vertices") and hasattr(mesh, "faces"):
        t = np.asarray(mesh.vertices, float)[np.asarray(mesh.faces, np.int64)]
    else:
        t = mesh
    t = np.ascontiguousarray(np.asarray(t, dtype=np.float64))
    if t.ndim != 3 or t.shape[1:] != (3, 3):
        raise ValueError("expected triangles of shape (n, 3, 3)")
    return t


def voxel_fill(mesh, grid, s=3, chunk=4_000_000):
    """Fill fraction (0..1) per grid element of a closed mesh, as a flat float64 element array
    (geometry.py:89-149; the same values bit for bit)."""
    del chunk
    tri = triangles_of(mesh)
    if tri.shape[0] == 0:
        raise ValueError("zero-size array to reduction operation minimum which has no identity")
    t = torch.as_tensor(tri, device="cuda")
    out = _voxeliser().fill_device(t, (grid.nx, grid.ny, grid.nz), grid.h, grid.origin, s)
    return out.cpu().numpy()


# ------------------------------------------------------------------ test meshes

def _unit(p):
    # plain IEEE operations only (no BLAS), so the mesh is the same on every machine
    return p / math.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2])


def icosphere(subdivisions=2, radius=1.0, center=(0.0, 0.0, 0.0)):
    """A closed, outward-wound sphere: the icosahedron with every face split into four
    `subdivisions` times and the new vertices pushed onto the sphere. Returns (vertices, faces)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [_unit(np.asarray(p, float)) for p in v]
    faces = list(f)
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                verts.append(_unit(verts[a] + verts[b]))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.asarray(verts) * float(radius) + np.asarray(center, float)
    return V, np.asarray(faces, np.int64)


def box(extents=(1.0, 1.0, 1.0), center=(0.0, 0.0, 0.0), rotation=None):
    """A closed, outward-wound box (12 triangles), optionally rotated by a 3x3 matrix about its
    centre. Returns (vertices, faces)."""
    e = np.asarray(extents, float) / 2.0
    corners = np.array([[x, y, z] for z in (-1, 1) for y in (-1, 1) for x in (-1, 1)], float) * e
    if rotation is not None:
        corners = corners @ np.asarray(rotation, float).T
    V = corners + np.asarray(center, float)
    # corner index = x + 2 y + 4 z (bits); two triangles per face, normals outward
    F = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6],      # z- , z+
                  [0, 1, 4], [1, 5, 4], [2, 6, 3], [3, 6, 7],      # y- , y+
                  [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]], np.int64)  # x- , x+
    return V, F


def mesh_volume(vertices, faces):
    """Signed volume of a closed mesh (positive when the faces wind outward)."""
    t = np.asarray(vertices, float)[np.asarray(faces, np.int64)]
    return float(np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2])).sum() / 6.0)
