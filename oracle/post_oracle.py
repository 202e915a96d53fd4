"""CPU oracle of the steps between the design and the surface (export.py:8-158 of anneal 0.3.0).

TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels of anl_post.cu in tests/. The
product never imports it.

* ``output_field`` -- export.py:8-14, elementwise;
* ``choose_level`` -- export.py:17-28: 40 bisection steps of count(f > t) against the
  design's volume, clamped to [0.3, 0.7];
* ``components`` -- scipy.ndimage.label of a mask with 6-connectivity (the reference's own
  call in keep_load_paths, export.py:44), relabelled by each component's smallest element
  index so that it compares with the GPU labels;
* ``distance`` -- scipy.ndimage.distance_transform_edt of the padded mask (export.py:155).

Pinned against the reference's own functions by tests/golden/post.npz.
"""
import numpy as np
from scipy import ndimage


def output_field(x, fill, active, solid_fill, void_fill, frozen):
    f = np.maximum(x * fill, np.where(active, solid_fill, 0.0))
    f = np.minimum(f, 1.0 - void_fill)
    f[frozen] = np.maximum(f[frozen], fill[frozen])
    return f


def choose_level(f, target, lo=0.05, hi=0.95, steps=40):
    for _ in range(steps):
        t = 0.5 * (lo + hi)
        if float(np.count_nonzero(f > t)) > target:
            lo = t
        else:
            hi = t
    return float(np.clip(0.5 * (lo + hi), 0.3, 0.7))


def components(mask_flat, shape):
    """Flat x-fastest labels: the smallest element index of the component, -1 off the mask."""
    nx, ny, nz = shape
    lab, n = ndimage.label(mask_flat.reshape(nz, ny, nx))
    lab = lab.ravel()
    out = np.full(lab.size, -1, np.int64)
    if n:
        first = np.full(n + 1, lab.size, np.int64)
        np.minimum.at(first, lab, np.arange(lab.size))
        out[lab > 0] = first[lab[lab > 0]]
    return out


def distance(mask_flat, shape):
    """Distance to the nearest non-mask element with the grid padded by an empty layer."""
    nx, ny, nz = shape
    b = np.pad(mask_flat.reshape(nz, ny, nx).astype(bool), 1)
    return ndimage.distance_transform_edt(b)[1:-1, 1:-1, 1:-1].ravel()
