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


# ------------------------------------------------------------------ from design to surface

def _f64(a):
    """CUDA float64 copy (or view) of a numpy array or tensor."""
    if torch.is_tensor(a):
        return a.to(device="cuda", dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(a, np.float64)), device="cuda")


def _u8(a):
    if torch.is_tensor(a):
        return a.to(device="cuda", dtype=torch.uint8).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(a).astype(np.uint8)), device="cuda")


def output_field(prob, x):
    """export.py:8-14 on the GPU: the printed field from the design x. Returns the type of x
    (a numpy array, or a CUDA tensor)."""
    xd = _f64(x)
    n = xd.numel()
    f = torch.empty_like(xd)
    keep = (_f64(prob.fill), _u8(prob.active), _f64(prob.solid_fill), _f64(prob.void_fill), _u8(prob.frozen))
    N.call("anl_output_field", *[ctypes.c_void_p(t.data_ptr()) for t in (xd,) + keep], n,
           ctypes.c_void_p(f.data_ptr()), _stream())
    return f if torch.is_tensor(x) else f.cpu().numpy()


def level_bisection(f, target, lo=0.05, hi=0.95, steps=40):
    """The [lo, hi] bracket after `steps` halvings that keep count(f > t) > target below
    (export.py:20-27), on the GPU. f: numpy array or tensor."""
    fd = _f64(f)
    state = torch.empty(2, dtype=torch.float64, device="cuda")
    hist = torch.empty(256, dtype=torch.int64, device="cuda")
    out = (ctypes.c_double * 2)()
    N.call("anl_choose_level", ctypes.c_void_p(fd.data_ptr()), fd.numel(), float(target), float(lo), float(hi),
           int(steps), ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(hist.data_ptr()), out, _stream())
    return out[0], out[1]


def choose_level(prob, f, x):
    """export.py:17-28: the iso level that keeps the optimised material volume, clamped to
    0.3..0.7. The target volume is the reference's float((x fill).sum()) (numpy inputs: the
    same summation; CUDA tensors: torch's)."""
    if torch.is_tensor(x):
        target = float((x.double() * _f64(prob.fill)).sum())
    else:
        target = float((x * prob.fill).sum())
    lo, hi = level_bisection(f, target)
    return float(np.clip(0.5 * (lo + hi), 0.3, 0.7))


def label_above(f, shape, thr):
    """Components of {f > thr} (6-connectivity) on the GPU: int32 CUDA tensor, each element's
    component named by its smallest element index, -1 outside."""
    fd = _f64(f)
    nx, ny, nz = shape
    lab = torch.empty(fd.numel(), dtype=torch.int32, device="cuda")
    N.call("anl_label_above", ctypes.c_void_p(fd.data_ptr()), int(nx), int(ny), int(nz), float(thr),
           ctypes.c_void_p(lab.data_ptr()), _stream())
    return lab


def keep_load_paths(prob, f, level, log=print, margin=0.1, max_drop=0.15, repair=True):
    """export.py:31-118: every load anchor must reach a fixed anchor through material at least
    `margin` above the iso level. Stage 1 lowers the level by up to max_drop (0.02 a step); stage
    2 adds material along the cheapest voxel path. The component labelling runs on the GPU;
    the anchor groups (the anchors' own distance functions) and the Dijkstra repair run on the
    host as in the reference. Returns (field, level)."""
    g = prob.grid
    centres = g.elem_centers()
    groups = []
    for a in prob.anchors:
        sel = (a.region.sdf(centres) <= 2.5 * g.h) & prob.active
        if sel.any():
            groups.append((a.name, a.role, np.flatnonzero(sel)))
    f = np.array(f, dtype=np.float64, copy=True)
    shape = (g.nx, g.ny, g.nz)
    members = np.concatenate([e for _, _, e in groups]) if groups else np.zeros(0, np.int64)
    bounds = np.cumsum([0] + [e.size for _, _, e in groups])
    members_d = torch.as_tensor(members, device="cuda")
    state = {"need": min(level + margin, 0.95), "f": _f64(f)}

    def broken():
        lab = label_above(state["f"], shape, state["need"])
        at = lab[members_d].cpu().numpy() if members.size else np.zeros(0, np.int32)
        sets = [set(at[bounds[i]:bounds[i + 1]].tolist()) for i in range(len(groups))]
        fixed = set()
        for (n, r, e), s in zip(groups, sets):
            if r == "fixed":
                fixed |= {v for v in s if v >= 0}
        return [(n, e) for (n, r, e), s in zip(groups, sets) if r == "load" and not (s & fixed)]

    level0 = level
    cut = broken()
    while cut and level > level0 - max_drop + 1e-9:
        level = max(0.1, level - 0.02)
        state["need"] = min(level + margin, 0.95)
        cut = broken()
        if level <= 0.1:
            break
    if level < level0:
        log(f"  iso level lowered {level0:.2f} -> {level:.2f} to keep load paths connected")
    if not cut:
        return f, level
    if not repair:
        log(f"  WARNING: anchor(s) {[n for n, _ in cut]} are not connected to a support and path repair is off. "
            f"Turn repair on, or raise volumeFraction or iterations.")
        return f, level
    f = _repair_paths(prob, f, level, state["need"], groups, cut, log)
    state["f"] = _f64(f)
    still = [n for n, _ in broken()]
    if still:
        log(f"  WARNING: anchor(s) {still} are still thinly connected. Raise volumeFraction or iterations.")
    return f, level


def _repair_paths(prob, f, level, need, groups, cut, log):
    """Stage 2 of keep_load_paths (export.py:71-118), host side: shortest paths from the fixed
    anchors over the active elements (6-neighbour graph, entering an element costs the density
    it lacks below `need` plus 1e-3), then every cut load anchor's path is made solid and
    wrapped in a shell at need + 0.05. The shell takes the +-1, +-nx, +-nx ny flat-index
    neighbours of the path, as the reference does."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import dijkstra
    g = prob.grid
    nx, nxy = g.nx, g.nx * g.ny
    act = np.flatnonzero(prob.active)
    slot = np.full(g.nelem, -1)
    slot[act] = np.arange(act.size)
    i, j, k = g.elem_ijk(act)
    src, dst = [], []
    for inside, step in ((i + 1 < g.nx, 1), (j + 1 < g.ny, nx), (k + 1 < g.nz, nxy)):
        a = act[inside]
        b = slot[a + step]
        ok = b >= 0
        src.append(slot[a[ok]])
        dst.append(b[ok])
    src = np.concatenate(src)
    dst = np.concatenate(dst)
    cost = np.maximum(0.0, need - f[act]) + 1e-3
    rows = np.concatenate([src, dst])
    cols = np.concatenate([dst, src])
    graph = csr_matrix((cost[cols], (rows, cols)), shape=(act.size, act.size))
    sources = np.unique(np.concatenate([slot[e] for _, r, e in groups if r == "fixed"]))
    sources = sources[sources >= 0]
    dist, pred, _ = dijkstra(graph, indices=sources, min_only=True, return_predecessors=True)
    added = 0
    offsets = (1, -1, nx, -nx, nxy, -nxy)
    for name, e in cut:
        targets = slot[e]
        targets = targets[targets >= 0]
        start = targets[np.argmin(dist[targets])]
        if not np.isfinite(dist[start]):
            log(f"  WARNING: anchor '{name}' cannot be reached from any support inside the design space.")
            continue
        path = []
        v = start
        while v >= 0:
            path.append(act[v])
            v = pred[v]
        path = np.array(path)
        shell = np.unique(np.concatenate([path + d for d in offsets]))
        shell = shell[(shell >= 0) & (shell < g.nelem)]
        shell = shell[prob.active[shell]]
        before = int((f > level).sum())
        f[shell] = np.maximum(f[shell], np.minimum(need + 0.05, prob.fill[shell]))
        f[path] = np.maximum(f[path], np.minimum(1.0, prob.fill[path]))
        added += int((f > level).sum()) - before
        log(f"  reconnected anchor '{name}' to the supports along a {path.size}-voxel path "
            f"({added} voxels of material added)")
    return f


def distance_transform(solid, shape):
    """Exact Euclidean distance of every element to the nearest non-solid one, with the grid
    padded by one empty layer (ndimage.distance_transform_edt(np.pad(b, 1)) cropped back, as in
    export.py:155). solid: flat x-fastest bool/uint8 (numpy or tensor). FP64 CUDA tensor, flat."""
    nx, ny, nz = shape
    b = _u8(solid).reshape(nz, ny, nx)
    p = torch.nn.functional.pad(b, (1, 1, 1, 1, 1, 1)).contiguous()
    px, py, pz = nx + 2, ny + 2, nz + 2
    n = px * py * pz
    need = ((4 * n + 15) & ~15) + 16 * n + 8 * max(py * pz, px * pz, px * py)
    scratch = torch.empty(need, dtype=torch.uint8, device="cuda")
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    N.call("anl_edt", ctypes.c_void_p(p.data_ptr()), px, py, pz, ctypes.c_void_p(d.data_ptr()),
           ctypes.c_void_p(scratch.data_ptr()), ctypes.c_size_t(need), _stream())
    return d.reshape(pz, py, px)[1:-1, 1:-1, 1:-1].reshape(-1)


def member_thickness(grid, fill_b):
    """export.py:150-158: member thickness in voxels along the skeleton of the as-built part,
    2 x the distance to the nearest empty voxel at the skeleton's voxels. The distance transform
    runs on the GPU; the skeleton is skimage.morphology.skeletonize on the host, as in the
    reference (which also needs skimage)."""
    from skimage.morphology import skeletonize
    solid = np.asarray(fill_b) >= 0.5
    if not solid.any():
        return np.zeros(0)
    edt = grid.to3d(distance_transform(solid, (grid.nx, grid.ny, grid.nz)).cpu().numpy())
    sk = skeletonize(grid.to3d(solid))
    return 2.0 * edt[sk > 0]
