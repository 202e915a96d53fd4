"""GPU steps between the design and the surface (anl_output_field, anl_choose_level,
anl_label_above, anl_edt) against the reference's outputs (tests/golden/post.npz) and the
CPU oracle (oracle/post_oracle.py, whose labelling and distance transform are scipy's)."""
import os
import types

import numpy as np
import pytest
import torch

from anneal_gb300 import export as X
from anneal_gb300.fem import Grid
from oracle import post_oracle as PO

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "post.npz"))
NAMES = [str(n) for n in Z["names"]]


def _prob(name):
    d = {k: Z[f"{name}_{k}"] for k in ("x", "fill", "active", "solid_fill", "void_fill", "frozen", "f",
                                       "sdf_fixed", "sdf_load")}
    g = Grid(tuple(int(v) for v in Z["shape"]), 1.0, (0.0, 0.0, 0.0))
    anchors = [types.SimpleNamespace(name="clamp", role="fixed", region=types.SimpleNamespace(sdf=lambda p, s=d["sdf_fixed"]: s)),
               types.SimpleNamespace(name="tip", role="load", region=types.SimpleNamespace(sdf=lambda p, s=d["sdf_load"]: s))]
    prob = types.SimpleNamespace(grid=g, fill=d["fill"], active=d["active"], solid_fill=d["solid_fill"],
                                 void_fill=d["void_fill"], frozen=d["frozen"], anchors=anchors)
    return prob, d


@pytest.mark.parametrize("name", NAMES)
def test_output_field_and_level_match_reference(name):
    prob, d = _prob(name)
    assert np.array_equal(X.output_field(prob, d["x"]), Z[f"{name}_output_field"])
    assert X.choose_level(prob, d["f"], d["x"]) == float(Z[f"{name}_level"])


@pytest.mark.parametrize("i", [0, 1])
def test_unclamped_level_matches_reference(i):
    prob = types.SimpleNamespace(fill=Z[f"level{i}_fill"])
    assert X.choose_level(prob, Z[f"level{i}_f"], Z[f"level{i}_x"]) == float(Z[f"level{i}_out"])


@pytest.mark.parametrize("steps", [0, 1, 7, 8, 9, 40, 53])
def test_bisection_any_step_count(steps):
    rng = np.random.default_rng(steps)
    f = rng.random(50000)
    target = 17000.5
    lo, hi = X.level_bisection(f, target, 0.05, 0.95, steps)
    rlo, rhi = 0.05, 0.95
    for _ in range(steps):
        t = 0.5 * (rlo + rhi)
        if float(np.count_nonzero(f > t)) > target:
            rlo = t
        else:
            rhi = t
    assert (lo, hi) == (rlo, rhi)


@pytest.mark.parametrize("name", NAMES)
def test_keep_load_paths_matches_reference(name):
    prob, d = _prob(name)
    logs = []
    f2, level = X.keep_load_paths(prob, d["f"], 0.5, log=logs.append, repair=bool(Z[f"{name}_repair"]))
    assert np.array_equal(f2, Z[f"{name}_kept_f"])
    assert level == float(Z[f"{name}_kept_level"])
    want = [str(s) for s in Z[f"{name}_log"] if str(s)]
    assert logs == want


@pytest.mark.parametrize("shape,p,seed", [((23, 17, 11), 0.55, 0), ((64, 40, 33), 0.6, 1), ((40, 40, 40), 0.7, 2),
                                          ((7, 1, 5), 0.5, 3)])
def test_labels_match_ndimage(shape, p, seed):
    rng = np.random.default_rng(seed)
    f = rng.random(int(np.prod(shape)))
    lab = X.label_above(f, shape, 1.0 - p).cpu().numpy()
    assert np.array_equal(lab, PO.components(f > 1.0 - p, shape))


def test_labels_large_grid_partition():
    """256 x 128 x 128 (4.2 M elements) at the percolation-critical density: same partition as
    ndimage.label, and labels stable over repeated runs."""
    shape = (256, 128, 128)
    rng = np.random.default_rng(5)
    f = rng.random(int(np.prod(shape)))
    a = X.label_above(f, shape, 1.0 - 0.3116)
    b = X.label_above(f, shape, 1.0 - 0.3116)
    assert torch.equal(a, b)
    assert np.array_equal(a.cpu().numpy(), PO.components(f > 1.0 - 0.3116, shape))


@pytest.mark.parametrize("shape,p,seed", [((23, 17, 11), 0.7, 0), ((50, 31, 40), 0.9, 1), ((9, 9, 9), 1.0, 2),
                                          ((64, 64, 32), 0.97, 3), ((1, 13, 6), 0.8, 4)])
def test_distance_transform_matches_scipy(shape, p, seed):
    rng = np.random.default_rng(seed)
    m = rng.random(int(np.prod(shape))) < p
    d = X.distance_transform(m, shape).cpu().numpy()
    assert np.array_equal(d, PO.distance(m, shape))


def test_distance_transform_solid_block():
    """A solid 60 x 40 x 30 block: the distance is the step count to the nearest face + 1."""
    shape = (60, 40, 30)
    d = X.distance_transform(np.ones(60 * 40 * 30, bool), shape).cpu().numpy().reshape(30, 40, 60)
    k, j, i = np.meshgrid(np.arange(30), np.arange(40), np.arange(60), indexing="ij")
    want = np.minimum.reduce([i + 1, 60 - i, j + 1, 40 - j, k + 1, 30 - k]).astype(float)
    assert np.array_equal(d, want)
