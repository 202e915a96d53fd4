"""The voxeliser oracle (oracle/voxel_oracle.py) against the reference's own voxel_fill.

tests/golden/voxel.npz holds geometry.voxel_fill (geometry.py:89-149) outputs on closed
meshes, a box whose top face lies on a sample plane, a triangle soup and s = 2, 3, 5; the
oracle must reproduce them bit for bit. The sphere case is the reference's volume check
(test_core.py:31-36)."""
import os

import numpy as np
import pytest

from anneal_gb300 import geometry as G
from oracle import voxel_oracle as VO

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "voxel.npz"))


@pytest.mark.parametrize("name", [str(n) for n in Z["names"]])
def test_oracle_matches_reference(name):
    f = VO.voxel_fill(Z[name + "_tri"], tuple(int(v) for v in Z[name + "_shape"]), float(Z[name + "_h"]),
                      Z[name + "_origin"], int(Z[name + "_s"]))
    assert np.array_equal(f, Z[name + "_fill"])


def test_sphere_volume_kat():
    """test_core.py:31-36: |voxel volume - mesh volume| / mesh volume < 0.5 %."""
    V, F = G.icosphere(4, 10.0)
    h = 0.75
    fill = Z["sphere_fill"]
    assert np.allclose(Z["sphere_tri"], V[F])
    vol = fill.sum() * h ** 3
    mv = G.mesh_volume(V, F)
    assert abs(vol - mv) / mv < 0.005


def test_test_meshes_closed():
    from anneal_gb300.export import Mesh
    for V, F in (G.icosphere(3, 2.0), G.box((1.0, 2.0, 3.0), (0.5, 0.0, 0.0), np.eye(3)[[1, 2, 0]])):
        m = Mesh(V, F)
        assert m.is_watertight and m.volume > 0


def test_box_plane_fill_values():
    """An axis-aligned 3 x 3 x 1.5 box at h = 1: the elements fully inside have fill 1, the
    layer the top face cuts in half has 2/3 (the crossing is not below the sample at 1.5)."""
    f = Z["box_plane_fill"].reshape(4, 5, 5)  # (z, y, x)
    assert np.all(f[1, 1:4, 1:4] == 1.0)
    assert np.allclose(f[2, 1:4, 1:4], 2.0 / 3.0)
    assert f[0].sum() == 0.0 and f[3].sum() == 0.0


def test_triangles_of_accepts_mesh_forms():
    """voxel_fill takes what the reference passes (an object with .triangles) and the other
    common mesh forms; all give the same (n, 3, 3) FP64 array."""
    import types
    V, F = G.icosphere(1, 2.0)
    t = V[F]
    for m in (types.SimpleNamespace(triangles=t), types.SimpleNamespace(vertices=V, faces=F), t,
              t.astype(np.float32).astype(np.float64).tolist()):
        got = G.triangles_of(m)
        assert got.shape == t.shape and got.dtype == np.float64
    assert np.array_equal(G.triangles_of(types.SimpleNamespace(vertices=V, faces=F)), t)
    with pytest.raises(ValueError):
        G.triangles_of(np.zeros((4, 3)))
