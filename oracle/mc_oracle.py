"""FP64 CPU oracle of the iso-surface export (export.py:121-147 of anneal 0.3.0).

TEST INFRASTRUCTURE ONLY: the checker for the GPU marching cubes in tests/. The product
never imports it.

The reference calls skimage.measure.marching_cubes and trimesh, neither of which is in this
image, so vertex-level parity with them cannot be pinned ("parity unpinned" for the
triangulation and the smoothing). This module restates, in numpy:

* ``zoomed`` -- np.pad(f, 1) and ndimage.zoom(order=1) exactly as export.py:122-126 does
  (scipy is present, so this step IS the reference's own call);
* ``case_table`` -- the face-consistent cube triangulation rule (inside = value > level;
  on a face whose inside corners sit on a diagonal, each inside corner is cut off alone;
  segments keep the inside on their left seen from outside the cube; each loop is fanned
  from its first position, counted from its smallest edge, none of whose diagonals lies on
  a cube face);
* ``marching_cubes`` -- one vertex per crossed grid edge (ordered by sample, then axis),
  triangles per cell in cell order, spacing and the origin - h/2 shift of export.py:126-131;
* ``taubin`` -- Taubin's lambda|mu smoothing with the equal-weight umbrella operator;
* ``components`` -- connected components labelled by their smallest vertex.
"""
import numpy as np
from scipy import ndimage
from scipy.sparse import coo_matrix
from scipy.sparse.csgraph import connected_components

MAXTRI = 8


def _corner(c):
    return np.array([c & 1, (c >> 1) & 1, (c >> 2) & 1], float)


def _edge(axis, corner):
    """Cube edge id along `axis` from `corner` (its bit `axis` clear)."""
    others = [d for d in range(3) if d != axis]
    bits = [(corner >> d) & 1 for d in others]
    return 4 * axis + bits[0] + 2 * bits[1]


def _edge_low_corner(e):
    axis, q = e >> 2, e & 3
    others = [d for d in range(3) if d != axis]
    return ((q & 1) << others[0]) | (((q >> 1) & 1) << others[1])


def _faces(e):
    axis, q = e >> 2, e & 3
    others = [d for d in range(3) if d != axis]
    return {(others[0], q & 1), (others[1], (q >> 1) & 1)}


def _share_face(e, f):
    return bool(_faces(e) & _faces(f))


def _edge_mid(e):
    p = _corner(_edge_low_corner(e))
    p[e >> 2] += 0.5
    return p


def case_table():
    """(ntri[256], tri[256, 24]) of cube edges, by the rule in the module docstring."""
    ntri = np.zeros(256, np.uint8)
    tri = np.zeros((256, 3 * MAXTRI), np.int8)
    for case in range(256):
        inside = [(case >> c) & 1 for c in range(8)]
        succ = {}
        for axis in range(3):
            u, v = [d for d in range(3) if d != axis]
            for side in (0, 1):
                ring = [(side << axis) | (bu << u) | (bv << v) for bu, bv in ((0, 0), (1, 0), (1, 1), (0, 1))]
                ring_edges = []
                for k in range(4):
                    a, b = ring[k], ring[(k + 1) % 4]
                    ring_edges.append(_edge(u if (a ^ b) == (1 << u) else v, a & b))
                crossed = [k for k in range(4) if inside[ring[k]] != inside[ring[(k + 1) % 4]]]
                if not crossed:
                    continue
                if len(crossed) == 2:
                    pairs = [((ring_edges[crossed[0]], ring_edges[crossed[1]]),
                              next(c for c in ring if inside[c]))]
                else:
                    pairs = [((ring_edges[(k + 3) % 4], ring_edges[k]), ring[k]) for k in range(4) if inside[ring[k]]]
                normal = np.zeros(3)
                normal[axis] = 1.0 if side else -1.0
                for (e0, e1), corner in pairs:
                    p, q = _edge_mid(e0), _edge_mid(e1)
                    if np.cross(q - p, normal) @ (_corner(corner) - 0.5 * (p + q)) < 0:
                        e0, e1 = e1, e0
                    assert e0 not in succ
                    succ[e0] = e1
        tris = []
        seen = set()
        for start in sorted(succ):
            if start in seen:
                continue
            loop, e = [], start
            while e not in seen:
                seen.add(e)
                loop.append(e)
                e = succ[e]
            assert e == start and len(loop) >= 3
            n = len(loop)
            # fan from the first position none of whose diagonals lies on a cube face
            apex = next(i for i in range(n)
                        if not any(_share_face(loop[i], loop[k]) for k in range(n)
                                   if k not in (i, (i + 1) % n, (i - 1) % n)))
            tris += [(loop[apex], loop[(apex + k) % n], loop[(apex + k + 1) % n]) for k in range(1, n - 1)]
        ntri[case] = len(tris)
        for t, (a, b, c) in enumerate(tris):
            tri[case, 3 * t:3 * t + 3] = (a, b, c)
    return ntri, tri


def zoomed(f3, upsample):
    """export.py:122-126: the padded, upsampled sample grid and its spacing (units of h)."""
    g = np.pad(np.asarray(f3, float), 1)
    n_in = np.array(g.shape)
    if upsample > 1:
        g = ndimage.zoom(g, upsample, order=1)
    n_out = np.array(g.shape)
    return g, (n_in - 1) / (n_out - 1)


def marching_cubes(g, level, spacing, shift, table=None):
    """g indexed [i, j, k] (x first). Returns (verts (nv, 3), faces (nf, 3))."""
    ntri, tri = case_table() if table is None else table
    nx, ny, nz = g.shape
    above = g > level
    # crossed forward edges per sample, vertex ids in (sample, axis) order with x fastest
    cross = np.zeros((3, nx, ny, nz), bool)
    cross[0, :-1] = above[:-1] != above[1:]
    cross[1, :, :-1] = above[:, :-1] != above[:, 1:]
    cross[2, :, :, :-1] = above[:, :, :-1] != above[:, :, 1:]
    # flatten with x fastest: sample s = i + nx (j + ny k); edge id = 3 s + axis
    cflat = np.stack([cross[a].transpose(2, 1, 0).ravel() for a in range(3)], axis=1).ravel()
    vid = np.full(cflat.size, -1, np.int64)
    vid[cflat] = np.arange(int(cflat.sum()))
    eids = np.flatnonzero(cflat)
    s, axis = eids // 3, eids % 3
    i, j, k = s % nx, (s // nx) % ny, s // (nx * ny)
    p0 = np.stack([i, j, k], 1).astype(float)
    st = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]])
    q = p0 + st[axis]
    f0 = g[i, j, k]
    f1 = g[q[:, 0].astype(int), q[:, 1].astype(int), q[:, 2].astype(int)]
    t = (level - f0) / (f1 - f0)
    p = p0 + st[axis] * t[:, None]
    verts = p * np.asarray(spacing, float) + np.asarray(shift, float)
    # cells
    case = np.zeros((nx - 1, ny - 1, nz - 1), np.int64)
    for c in range(8):
        di, dj, dk = c & 1, (c >> 1) & 1, (c >> 2) & 1
        case |= above[di:nx - 1 + di, dj:ny - 1 + dj, dk:nz - 1 + dk].astype(np.int64) << c
    ci, cj, ck = np.nonzero(ntri[case] > 0)
    cs = case[ci, cj, ck]
    cell = ci + nx * (cj + ny * ck)
    faces, order = [], []
    for tt in range(MAXTRI):
        sel = ntri[cs] > tt
        if not sel.any():
            continue
        tri_v = []
        for r in range(3):
            e = tri[cs[sel], 3 * tt + r].astype(np.int64)
            ax = e >> 2
            qq = e & 3
            o1 = np.where(ax == 0, 1, 0)
            o2 = np.where(ax == 2, 1, 2)
            off = np.zeros((sel.sum(), 3), np.int64)
            off[np.arange(off.shape[0]), o1] = qq & 1
            off[np.arange(off.shape[0]), o2] = (qq >> 1) & 1
            si = ci[sel] + off[:, 0]
            sj = cj[sel] + off[:, 1]
            sk = ck[sel] + off[:, 2]
            tri_v.append(vid[3 * (si + nx * (sj + ny * sk)) + ax])
        faces.append(np.stack(tri_v, 1))
        order.append(np.stack([cell[sel], np.full(sel.sum(), tt)], 1))
    if not faces:
        return verts, np.zeros((0, 3), np.int64)
    faces = np.concatenate(faces)
    order = np.concatenate(order)
    idx = np.lexsort((order[:, 1], order[:, 0]))
    return verts, faces[idx]


def surface_raw(f3, level, h, origin, upsample=2):
    """Padded, zoomed marching cubes with the reference's spacing and shift."""
    g, sp = zoomed(f3, upsample)
    return marching_cubes(g, level, sp * h, np.asarray(origin, float) - 0.5 * h)


def taubin(verts, faces, iterations, lamb=0.5, mu=-0.53):
    """Taubin smoothing: v += w (mean of the unique neighbours - v), w = lamb, mu, ..."""
    v = np.array(verts, float)
    nv = v.shape[0]
    a = np.concatenate([faces[:, 0], faces[:, 1], faces[:, 2]])
    b = np.concatenate([faces[:, 1], faces[:, 2], faces[:, 0]])
    A = coo_matrix((np.ones(2 * a.size), (np.concatenate([a, b]), np.concatenate([b, a]))), shape=(nv, nv)).tocsr()
    A.data[:] = 1.0
    deg = np.asarray(A.sum(axis=1)).ravel()
    for it in range(iterations):
        w = lamb if it % 2 == 0 else mu
        mean = (A @ v) / np.maximum(deg, 1)[:, None]
        v = np.where(deg[:, None] > 0, v + w * (mean - v), v)
    return v


def components(faces, nv):
    """Per-face component label = smallest vertex index of its component."""
    a = np.concatenate([faces[:, 0], faces[:, 1]])
    b = np.concatenate([faces[:, 1], faces[:, 2]])
    G = coo_matrix((np.ones(a.size), (a, b)), shape=(nv, nv))
    _, lab = connected_components(G, directed=False)
    rep = np.full(lab.max() + 1, nv, np.int64)
    np.minimum.at(rep, lab, np.arange(nv))
    return rep[lab[faces[:, 0]]]


def volume(verts, faces):
    v0, v1, v2 = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
    return float(np.einsum("ij,ij->i", v0, np.cross(v1, v2)).sum() / 6.0)
