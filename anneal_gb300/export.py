"""Iso-surface export with the interface of anneal's export.surface (export.py:121-147).

``surface(grid, f, level, upsample=2, smooth=10, log=print)`` pads the element field by one
element, upsamples it linearly, extracts the level set by marching cubes, applies Taubin
smoothing and drops floating fragments under 1 % of the main body's volume, as the
reference does with ndimage.zoom, skimage and trimesh. The field work, the extraction (a
stream compaction over the sample grid), the smoothing and the component labelling run in
the CUDA library (``anl_mc_*``); the host keeps the per-component volume bookkeeping and the
final orientation check. The result is a ``trimesh.Trimesh`` when trimesh is installed (the
reference's return type), else a ``Mesh`` with the attributes the reference's callers read.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .context import require_cuda, to_dev

TAUBIN_LAMBDA = 0.5    # export.py:134
TAUBIN_MU = -0.53      # export.py:134 (passed as nu)
FRAGMENT_FRACTION = 0.01  # export.py:138


class Mesh:
    """Indexed triangle mesh: vertices (nv, 3) float64, faces (nf, 3) int64, outward-facing."""

    def __init__(self, vertices, faces):
        self.vertices = np.asarray(vertices, float)
        self.faces = np.asarray(faces, np.int64)

    @property
    def triangles(self):
        return self.vertices[self.faces]

    @property
    def volume(self):
        t = self.triangles
        return float(np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2])).sum() / 6.0)

    @property
    def area(self):
        t = self.triangles
        return float(0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1).sum())

    @property
    def is_watertight(self):
        """Every directed edge appears once and its reverse once (closed, consistently wound)."""
        f = self.faces
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        n = max(int(self.vertices.shape[0]), 1)
        fwd = e[:, 0] * n + e[:, 1]
        rev = e[:, 1] * n + e[:, 0]
        if np.unique(fwd).size != fwd.size:
            return False
        return bool(np.array_equal(np.sort(fwd), np.sort(rev)))

    @property
    def bounds(self):
        return np.stack([self.vertices.min(axis=0), self.vertices.max(axis=0)])

    def export(self, path):
        """Binary STL."""
        t = self.triangles.astype(np.float32)
        nrm = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
        ln = np.linalg.norm(nrm, axis=1, keepdims=True)
        nrm = np.where(ln > 0, nrm / np.maximum(ln, 1e-30), 0.0).astype(np.float32)
        rec = np.zeros(t.shape[0], dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
        rec["n"] = nrm
        rec["v"] = t
        with open(path, "wb") as fh:
            fh.write(b"anneal_gb300 binary STL".ljust(80, b" "))
            fh.write(np.uint32(t.shape[0]).tobytes())
            fh.write(rec.tobytes())


class MarchingCubes:
    """The device workspace of the export (anl_mc): it keeps its buffers between calls."""

    def __init__(self):
        require_cuda()
        h = ctypes.c_void_p()
        N.call("anl_mc_create", ctypes.byref(h))
        self.h = h

    def close(self):
        if self.h:
            N.load().anl_mc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def extract(self, field, shape, level, h, origin, upsample=2):
        """field: (nx*ny*nz,) float32 CUDA tensor. Returns (nverts, nfaces)."""
        nx, ny, nz = shape
        nv, nf = ctypes.c_int64(), ctypes.c_int64()
        org = (ctypes.c_double * 3)(*[float(o) for o in origin])
        N.call("anl_mc_extract", self.h, ctypes.c_void_p(field.data_ptr()), nx, ny, nz, int(upsample),
               float(level), float(h), org, ctypes.byref(nv), ctypes.byref(nf), _stream())
        self.nv, self.nf = nv.value, nf.value
        return self.nv, self.nf

    def smooth(self, iterations, lamb=TAUBIN_LAMBDA, mu=TAUBIN_MU):
        N.call("anl_mc_smooth", self.h, int(iterations), float(lamb), float(mu), _stream())

    def components(self):
        lab = torch.empty(max(self.nf, 1), dtype=torch.int32, device="cuda")
        rounds = ctypes.c_int()
        N.call("anl_mc_components", self.h, ctypes.c_void_p(lab.data_ptr()), ctypes.byref(rounds), _stream())
        return lab[:self.nf]

    def mesh_device(self):
        v = torch.empty((max(self.nv, 1), 3), dtype=torch.float32, device="cuda")
        f = torch.empty((max(self.nf, 1), 3), dtype=torch.int32, device="cuda")
        N.call("anl_mc_copy", self.h, ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(f.data_ptr()), _stream())
        return v[:self.nv], f[:self.nf]


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def case_table():
    """The library's derived marching-cubes case table (no GPU needed)."""
    ntri = np.zeros(256, np.uint8)
    tri = np.zeros(256 * 24, np.int8)
    N.call("anl_mc_table", ntri.ctypes.data_as(ctypes.c_void_p), tri.ctypes.data_as(ctypes.c_void_p))
    return ntri, tri.reshape(256, 24)


def surface(grid, f, level, upsample=2, smooth=10, log=print):
    """export.py:121-147 on the GPU."""
    field = to_dev(np.asarray(f, float), torch.float32) if not torch.is_tensor(f) else \
        f.to(device="cuda", dtype=torch.float32).contiguous()
    if float(field.max()) <= level:
        raise RuntimeError("The optimized field is empty at the chosen level. Raise volumeFraction.")
    mc = MarchingCubes()
    try:
        mc.extract(field, grid.shape, level, grid.h, grid.origin, upsample)
        if smooth > 0:
            mc.smooth(int(smooth))
        lab = mc.components()
        v, fc = mc.mesh_device()
        verts = v.double().cpu().numpy()
        faces = fc.long().cpu().numpy()
        labels = lab.long().cpu().numpy()
    finally:
        mc.close()
    # export.py:135-141: drop fragments under 1 % of the largest component's volume
    uniq, comp = np.unique(labels, return_inverse=True)
    if uniq.size > 1:
        t = verts[faces]
        tv = np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2])) / 6.0
        vols = np.abs(np.bincount(comp, weights=tv, minlength=uniq.size))
        keep = vols >= FRAGMENT_FRACTION * vols.max()
        if not keep.all():
            log(f"  removed {int((~keep).sum())} floating fragment(s) under 1 % of the main body")
            faces = faces[keep[comp]]
            used, inv = np.unique(faces.ravel(), return_inverse=True)
            verts = verts[used]
            faces = inv.reshape(-1, 3)
    mesh = Mesh(verts, faces)
    if mesh.volume < 0:   # export.py:145-146
        mesh = Mesh(verts, faces[:, ::-1])
    try:
        import trimesh
        return trimesh.Trimesh(mesh.vertices, mesh.faces, process=False)
    except ImportError:
        return mesh
