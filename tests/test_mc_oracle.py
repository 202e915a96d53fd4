"""The marching-cubes case table and the CPU oracle of the export (no GPU needed).

skimage and trimesh are absent, so the triangulation cannot be pinned to the reference
vertex by vertex; the checks here are the invariants the reference's own tests assert on
its export (closed surface, outward normals: test_library_dfm.py:118-131, test_core.py:77-87)
plus the volume of a sphere."""
import numpy as np
import pytest

from oracle import mc_oracle as M


def _closed_and_outward(verts, faces):
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    n = verts.shape[0]
    fwd = e[:, 0] * n + e[:, 1]
    rev = e[:, 1] * n + e[:, 0]
    return np.unique(fwd).size == fwd.size and np.array_equal(np.sort(fwd), np.sort(rev))


def test_table_is_consistent():
    ntri, tri = M.case_table()
    assert ntri[0] == 0 and ntri[255] == 0
    assert ntri[1] == 1 and ntri.max() <= M.MAXTRI
    # complementary cases cut the same edges
    for c in range(256):
        a = set(tri[c, :3 * ntri[c]].tolist())
        b = set(tri[255 - c, :3 * ntri[255 - c]].tolist())
        assert a == b, c


def test_library_table_matches_oracle():
    from anneal_gb300 import export as X
    ntri, tri = X.case_table()
    ont, otri = M.case_table()
    assert np.array_equal(ntri, ont)
    for c in range(256):
        assert np.array_equal(tri[c, :3 * ntri[c]], otri[c, :3 * ont[c]]), c


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_random_field_is_closed_and_outward(seed):
    rng = np.random.default_rng(seed)
    f = rng.random((7, 6, 5))
    v, fc = M.surface_raw(f, 0.5, 1.0, (0, 0, 0), upsample=2)
    assert fc.shape[0] > 0
    assert _closed_and_outward(v, fc)
    assert M.volume(v, fc) > 0


def test_oracle_sphere_volume():
    n = 24
    c = (np.arange(n) + 0.5 - n / 2)
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    r = 8.0
    f = np.clip(r + 0.5 - np.sqrt(x ** 2 + y ** 2 + z ** 2), 0, 1)   # ~ fill fraction
    v, fc = M.surface_raw(f, 0.5, 1.0, (0, 0, 0), upsample=2)
    assert _closed_and_outward(v, fc)
    vol = M.volume(v, fc)
    assert abs(vol / (4 / 3 * np.pi * r ** 3) - 1) < 0.02
    # Euler characteristic of a sphere
    e = np.unique(np.sort(np.concatenate([fc[:, [0, 1]], fc[:, [1, 2]], fc[:, [2, 0]]]), axis=1), axis=0)
    assert v.shape[0] - e.shape[0] + fc.shape[0] == 2
