"""The post-processing oracle (oracle/post_oracle.py) against the reference's own
export.output_field and choose_level (tests/golden/post.npz, made by
tests/golden/make_golden.py --only post)."""
import os

import numpy as np
import pytest

from oracle import post_oracle as PO

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "post.npz"))
NAMES = [str(n) for n in Z["names"]]


@pytest.mark.parametrize("name", NAMES)
def test_output_field_and_level(name):
    d = {k: Z[f"{name}_{k}"] for k in ("x", "fill", "active", "solid_fill", "void_fill", "frozen", "f")}
    fo = PO.output_field(d["x"], d["fill"], d["active"], d["solid_fill"], d["void_fill"], d["frozen"])
    assert np.array_equal(fo, Z[f"{name}_output_field"])
    target = float((d["x"] * d["fill"]).sum())
    assert PO.choose_level(d["f"], target) == float(Z[f"{name}_level"])


@pytest.mark.parametrize("i", [0, 1])
def test_unclamped_level(i):
    target = float((Z[f"level{i}_x"] * Z[f"level{i}_fill"]).sum())
    assert PO.choose_level(Z[f"level{i}_f"], target) == float(Z[f"level{i}_out"])


def test_components_relabel():
    m = np.zeros(5 * 4 * 3, bool)
    m[[0, 1, 7, 59]] = True
    lab = PO.components(m, (5, 4, 3))
    assert lab[0] == 0 and lab[1] == 0 and lab[7] == 7 and lab[59] == 59 and lab[2] == -1
