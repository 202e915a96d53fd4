"""GPU iso-surface export against the CPU oracle (oracle/mc_oracle.py), through the C ABI.

The extraction is compared exactly in topology (same faces, same vertex order) and to FP32
rounding in geometry; smoothing and components to the oracle's FP64 results."""
import numpy as np
import pytest
import torch

from oracle import mc_oracle as M

pytestmark = pytest.mark.gpu


def _extract(f3, level, h=1.0, origin=(0.0, 0.0, 0.0), upsample=2, smooth=0):
    from anneal_gb300 import export as X
    nx, ny, nz = f3.shape
    flat = torch.as_tensor(np.ascontiguousarray(f3.transpose(2, 1, 0)).ravel(), dtype=torch.float32, device="cuda")
    mc = X.MarchingCubes()
    mc.extract(flat, (nx, ny, nz), level, h, origin, upsample)
    if smooth:
        mc.smooth(smooth)
    lab = mc.components().long().cpu().numpy()
    v, f = mc.mesh_device()
    out = v.double().cpu().numpy(), f.long().cpu().numpy(), lab
    mc.close()
    return out


@pytest.mark.parametrize("shape,upsample,seed", [((7, 6, 5), 2, 0), ((13, 9, 11), 2, 1), ((10, 4, 6), 1, 2),
                                                 ((5, 5, 5), 3, 3)])
def test_extract_matches_oracle(shape, upsample, seed):
    rng = np.random.default_rng(seed)
    f3 = rng.random(shape)
    h, origin = 0.7, (1.0, -2.0, 0.5)
    v, f, _ = _extract(f3, 0.45, h, origin, upsample)
    ov, of = M.surface_raw(f3, 0.45, h, origin, upsample)
    assert np.array_equal(f, of)
    assert np.abs(v - ov).max() <= 2e-5 * max(1.0, np.abs(ov).max())


def test_sphere_is_closed_outward_and_right_sized():
    from anneal_gb300 import export as X
    n = 40
    c = np.arange(n) + 0.5 - n / 2
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    r = 14.0
    f3 = np.clip(r + 0.5 - np.sqrt(x ** 2 + y ** 2 + z ** 2), 0, 1)
    v, f, lab = _extract(f3, 0.5)
    m = X.Mesh(v, f)
    assert m.is_watertight
    assert abs(m.volume / (4 / 3 * np.pi * r ** 3) - 1) < 0.01
    assert np.unique(lab).size == 1


def test_taubin_matches_oracle():
    rng = np.random.default_rng(5)
    f3 = rng.random((9, 8, 7))
    v0, f0, _ = _extract(f3, 0.5, smooth=0)
    v, f, _ = _extract(f3, 0.5, smooth=10)
    assert np.array_equal(f, f0)
    want = M.taubin(v0, f0, 10, 0.5, -0.53)
    assert np.abs(v - want).max() <= 1e-4 * max(1.0, np.abs(want).max())


def test_components_match_oracle():
    rng = np.random.default_rng(7)
    f3 = (rng.random((16, 12, 10)) > 0.7).astype(float)   # many small blobs
    v, f, lab = _extract(f3, 0.5)
    want = M.components(f, v.shape[0])
    assert np.array_equal(lab, want)
    assert np.unique(lab).size > 3


def test_surface_drops_small_fragments_and_faces_outward():
    from anneal_gb300 import export as X
    from anneal_gb300.fem import Grid
    g = Grid((24, 16, 16), 1.0, (0.0, 0.0, 0.0))
    f3 = np.zeros(g.shape)
    f3[2:20, 3:13, 3:13] = 1.0      # main body
    f3[22, 14, 14] = 1.0           # one voxel, far under 1 % of the body
    msgs = []
    mesh = X.surface(g, g.to1d(f3), 0.5, upsample=2, smooth=10, log=msgs.append)
    assert any("removed 1 floating fragment" in s for s in msgs)
    m = X.Mesh(mesh.vertices, mesh.faces)
    assert m.is_watertight and m.volume > 0
    assert abs(m.volume / (18 * 10 * 10) - 1) < 0.15


def test_empty_field_raises():
    from anneal_gb300 import export as X
    from anneal_gb300.fem import Grid
    g = Grid((4, 4, 4), 1.0, (0, 0, 0))
    with pytest.raises(RuntimeError, match="empty at the chosen level"):
        X.surface(g, np.zeros(g.nelem), 0.5)
