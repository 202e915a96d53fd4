"""GPU voxeliser (anl_voxel_fill) against the reference's voxel_fill and the CPU oracle.

Bit-exact: the fill fractions must equal the reference's golden outputs (tests/golden/
voxel.npz) and the oracle's (oracle/voxel_oracle.py) on larger meshes and other sub-sample
counts; the sphere volume check of test_core.py:31-36 holds at several resolutions."""
import os

import numpy as np
import pytest
import torch

from anneal_gb300 import geometry as G
from anneal_gb300.fem import Grid
from oracle import voxel_oracle as VO

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "voxel.npz"))


def _grid_around(V, h):
    lo, hi = V.min(axis=0), V.max(axis=0)
    return Grid(tuple(int(v) for v in np.ceil((hi - lo + 2 * h) / h)), h, lo - h)


@pytest.mark.parametrize("name", [str(n) for n in Z["names"]])
def test_matches_reference_golden(name):
    shape = tuple(int(v) for v in Z[name + "_shape"])
    g = Grid(shape, float(Z[name + "_h"]), Z[name + "_origin"])
    f = G.voxel_fill(Z[name + "_tri"], g, s=int(Z[name + "_s"]))
    assert f.dtype == np.float64 and f.shape == (g.nelem,)
    assert np.array_equal(f, Z[name + "_fill"])


@pytest.mark.parametrize("sub,radius,h,s", [(5, 20.0, 0.5, 3), (3, 6.0, 0.35, 1), (3, 6.0, 0.7, 7),
                                            (4, 9.0, 0.6, 11)])
def test_matches_oracle(sub, radius, h, s):
    V, F = G.icosphere(sub, radius, (0.37, -1.1, 2.3))
    g = _grid_around(V, h)
    f = G.voxel_fill(V[F], g, s=s)
    ref = VO.voxel_fill(V[F], g.shape, g.h, g.origin, s)
    assert np.array_equal(f, ref)


def test_soup_and_rotated_boxes_match_oracle():
    rng = np.random.default_rng(17)
    tri = VO.triangle_soup(2000, -5.0, 5.0, 9)
    rot = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    V, F = G.box((6.0, 2.0, 3.5), (0.5, 0.2, -0.3), rot)
    tri = np.concatenate([tri, V[F]])
    g = Grid((40, 37, 29), 0.27, (-5.4, -5.1, -4.0))
    assert np.array_equal(G.voxel_fill(tri, g), VO.voxel_fill(tri, g.shape, g.h, g.origin, 3))


@pytest.mark.parametrize("sub,radius,h", [(4, 10.0, 0.75), (6, 60.0, 0.5)])
def test_sphere_volume(sub, radius, h):
    """test_core.py:31-36 (and a 244^3 grid of 14.5 M elements)."""
    V, F = G.icosphere(sub, radius)
    g = _grid_around(V, h)
    f = G.voxel_fill(V[F], g)
    mv = G.mesh_volume(V, F)
    assert abs(f.sum() * h ** 3 - mv) / mv < 0.005
    assert f.min() >= 0.0 and f.max() <= 1.0


def test_stats_determinism_and_errors():
    V, F = G.icosphere(4, 10.0)
    g = _grid_around(V, 0.75)
    vox = G.Voxeliser()
    t = torch.as_tensor(V[F], device="cuda")
    a = vox.fill_device(t, g.shape, g.h, g.origin, stats=True)
    pairs, hits = vox.pairs, vox.hits
    b = vox.fill_device(t, g.shape, g.h, g.origin)
    assert torch.equal(a, b)
    # every sample column through the sphere crosses it twice (in and out)
    assert 0 < hits <= pairs and hits % 2 == 0
    with pytest.raises(ValueError):
        vox.fill_device(t[:0], g.shape, g.h, g.origin)
    from anneal_gb300._native import NativeError
    with pytest.raises(NativeError):
        vox.fill_device(t, g.shape, g.h, g.origin, s=17)
    vox.close()


def test_large_case_matches_reference_digest():
    """128 x 64 x 64 grid, 20,480-triangle sphere: SHA-256 of the fill bytes equals the
    reference's (computed by tests/golden/make_golden.py)."""
    import hashlib
    V, F = G.icosphere(5, 0.45 * 64, (0.3 * 128, 32.0, 32.0))
    tri = np.ascontiguousarray(V[F])
    assert hashlib.sha256(tri.tobytes()).hexdigest() == str(Z["big_tri_sha256"]), "test mesh differs"
    f = G.voxel_fill(tri, Grid((128, 64, 64), 1.0, (0.0, 0.0, 0.0)))
    assert f.sum() == float(Z["big_fill_sum"])
    assert hashlib.sha256(f.tobytes()).hexdigest() == str(Z["big_fill_sha256"])
