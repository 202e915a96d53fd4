"""FP64 CPU oracle of the voxeliser (geometry.voxel_fill, geometry.py:89-149 of anneal 0.3.0).

TEST INFRASTRUCTURE ONLY: the checker for the GPU voxeliser in tests/. The product never
imports it.

A numpy restatement of the reference's ray-parity method, step for step:

* sample coordinates (geometry.py:91-94): per axis, origin + h (i + (a + 1/2)/s) for element
  i and sub-sample a; x and y shifted by h 6.18e-6 and h 4.14e-6 so that no ray runs exactly
  along a mesh edge of an axis-aligned model;
* columns per triangle (geometry.py:99-105): the sample columns whose x lies in
  [min x, max x] of the triangle (searchsorted left / right), the same along y;
* crossings (geometry.py:124-131): the barycentric coordinates of the column in the
  triangle's xy projection, evaluated with the reference's operation order; a column crosses
  when the projected area is non-zero and all three coordinates are >= 0, at the height
  interpolated from the vertices;
* parity (geometry.py:139-146): every crossing becomes the key column + (z - zlo) / zr,
  zr = 1.001 (zhi - zlo) + 1e-9; a sample of height zs counts the keys in
  [column, column + clip((zs - zlo) / zr, 0, 0.999999)); odd means inside;
* fraction (geometry.py:147-149): the mean of the s^3 inside flags of an element, returned
  flat with x fastest.

The triangle loop is plain Python over numpy column blocks: meant for meshes of a few
thousand triangles on small grids. Pinned against the reference's own function by the
fixtures in tests/golden/voxel.npz (tests/golden/make_golden.py, --only voxel).
"""
import numpy as np


def sample_axes(n, h, origin, s, shift):
    """Sample coordinates along one axis (geometry.py:91-94)."""
    sub = (np.arange(s) + 0.5) / s
    c = (origin + h * (np.arange(n)[:, None] + sub[None, :])).ravel()
    return c + h * shift if shift else c


def crossings(tri, xs, ys):
    """(column, z) of every ray crossing: column = ix + len(xs) iy."""
    cols, zs = [], []
    nxs = xs.size
    for v in tri:
        lo, hi = v.min(axis=0), v.max(axis=0)
        ix = np.arange(np.searchsorted(xs, lo[0]), np.searchsorted(xs, hi[0], side="right"))
        iy = np.arange(np.searchsorted(ys, lo[1]), np.searchsorted(ys, hi[1], side="right"))
        if ix.size == 0 or iy.size == 0:
            continue
        IX, IY = np.meshgrid(ix, iy)
        IX, IY = IX.ravel(), IY.ravel()
        px, py = xs[IX], ys[IY]
        (x0, y0, z0), (x1, y1, z1), (x2, y2, z2) = v
        d = (y1 - y2) * (x0 - x2) + (x2 - x1) * (y0 - y2)
        if d == 0:
            continue
        l0 = ((y1 - y2) * (px - x2) + (x2 - x1) * (py - y2)) / d
        l1 = ((y2 - y0) * (px - x2) + (x0 - x2) * (py - y2)) / d
        l2 = 1 - l0 - l1
        hit = (l0 >= 0) & (l1 >= 0) & (l2 >= 0)
        z = l0 * z0 + l1 * z1 + l2 * z2
        cols.append((IX + nxs * IY)[hit])
        zs.append(z[hit])
    if not cols:
        return np.zeros(0, np.int64), np.zeros(0)
    return np.concatenate(cols), np.concatenate(zs)


def voxel_fill(tri, shape, h, origin, s=3):
    """Fill fractions (nx*ny*nz,) float64, x fastest, of the triangles tri (n, 3, 3)."""
    tri = np.asarray(tri, np.float64)
    nx, ny, nz = shape
    xs = sample_axes(nx, h, origin[0], s, 6.18e-6)
    ys = sample_axes(ny, h, origin[1], s, 4.14e-6)
    zs = sample_axes(nz, h, origin[2], s, 0.0)
    zlo, zhi = tri[:, :, 2].min(), tri[:, :, 2].max()
    zr = (zhi - zlo) * 1.001 + 1e-9
    col, z = crossings(tri, xs, ys)
    keys = np.sort(col.astype(np.float64) + (z - zlo) / zr)
    ncol = xs.size * ys.size
    c = np.arange(ncol, dtype=np.float64)
    zq = np.clip((zs - zlo) / zr, 0.0, 0.999999)
    below = np.searchsorted(keys, (c[:, None] + zq[None, :]).ravel()).reshape(ncol, zs.size)
    below -= np.searchsorted(keys, c)[:, None]
    inside = (below & 1).astype(bool).reshape(ny, s, nx, s, nz, s)
    frac = inside.mean(axis=(1, 3, 5))          # (ny, nx, nz)
    return np.ascontiguousarray(frac.transpose(2, 0, 1)).ravel()  # (nz, ny, nx): x fastest


def triangle_soup(n, lo, hi, seed):
    """n seeded random triangles with vertices uniform in the box [lo, hi]^3 (not closed: the
    parity is then meaningless, but every rounding path of the test is exercised)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=(n, 3, 3))
