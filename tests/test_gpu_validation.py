"""Closed-form checks of the GPU solver, compared with the values the reference's validation
gate computed (validate.py:38-129, recorded in tests/golden/validate.json by make_golden.py).

The physical set-ups are the gate's: a 10 x 2 x 4 bar in uniform tension (supported against
rigid motion only), the same bar with a partially filled top layer, cantilevers 2, 4 and 8
elements deep against Timoshenko's beam, bit-identical reruns and an optimised cantilever
against a uniform one at equal mass. The code here is this project's own; the reference's
own gate runs against the GPU solver through anneal_gb300.integrate.install."""
import hashlib
import json
import os
import re

import numpy as np
import pytest

from anneal_gb300 import fem as G
from anneal_gb300 import optimize as O

pytestmark = pytest.mark.gpu

E0, NU = 1000.0, 0.3
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "validate.json")


def _recorded():
    with open(GOLDEN) as fh:
        return json.load(fh)


class Bar:
    """A box of nx x ny x nz cubes of side h, loaded on its x = nx h face."""

    def __init__(self, nx, ny, nz, h=1.0):
        self.g = G.Grid((nx, ny, nz), h, (0.0, 0.0, 0.0))
        self.h = h
        n = np.arange(self.g.nnode)
        self.node_xyz = self.g.node_coords(n)
        self.i, self.j, self.k = self.g.elem_ijk(np.arange(self.g.nelem))

    def nodes(self, x=None, y=None, z=None):
        sel = np.ones(self.g.nnode, bool)
        for c, v in enumerate((x, y, z)):
            if v is not None:
                sel &= np.abs(self.node_xyz[:, c] - v) < 1e-9
        return np.flatnonzero(sel)

    def end_face_load(self, total, comp, weights):
        """`total` in direction `comp` over the +x faces of the last element column, each
        element's share in proportion to `weights`, a quarter to each face corner."""
        last = np.flatnonzero(self.i == self.g.nx - 1)
        w = np.asarray(weights, float)[last]
        en = self.g.element_nodes(last)
        plus_x = [a for a in range(8) if G.LOCAL[a, 0] == 1]
        F = np.zeros(3 * self.g.nnode)
        for a in plus_x:
            np.add.at(F, 3 * en[:, a] + comp, total * w / w.sum() / 4.0)
        return F

    def tip_mean(self, u, comp):
        tip = self.nodes(x=self.g.nx * self.h)
        return float(u[3 * tip + comp].mean())


def _solve(bar, fixed, E, F, rtol=1e-12):
    fem = G.FEM(bar.g, np.ones(bar.g.nelem, bool), fixed, NU)
    u = fem.expand(fem.solve(fem.assemble(E), [fem.reduce_load(F)], rtol=rtol)[0])
    fem.close()
    return u


def _tension_tip(nz, top_fill=None, F=100.0):
    bar = Bar(10, 2, nz)
    fill = np.ones(bar.g.nelem)
    if top_fill is not None:
        fill[bar.k == nz - 1] = top_fill
    # x fixed on the x = 0 face; y and z fixed at one corner, z at the corner across y:
    # rigid motions are stopped, the lateral contraction is free
    fixed = list(3 * bar.nodes(x=0.0))
    c0, c1 = bar.nodes(x=0.0, y=0.0, z=0.0)[0], bar.nodes(x=0.0, y=2.0, z=0.0)[0]
    fixed += [3 * c0 + 1, 3 * c0 + 2, 3 * c1 + 2]
    u = _solve(bar, fixed, E0 * fill, bar.end_face_load(F, 0, fill))
    return bar.tip_mean(u, 0)


def test_rigid_motions_store_no_energy():
    ke, _, _ = G.hex8_matrices(NU, 1.0)
    p = G.LOCAL.astype(float)
    translation = np.tile([1.0, 0.0, 0.0], 8)
    rotation = np.column_stack([-p[:, 1], p[:, 0], np.zeros(8)]).ravel()
    assert abs(translation @ ke @ translation) < 1e-10
    assert abs(rotation @ ke @ rotation) < 1e-10


def test_uniform_tension_is_FL_over_AE():
    ux = _tension_tip(4)
    exact = 100.0 * 10 / (2 * 4 * E0)
    assert abs(ux / exact - 1) < 1e-8
    assert abs(ux / _recorded()["_tension_ux"] - 1) < 1e-8


def test_partial_fill_layer_carries_its_share():
    """A 6.4-cell-deep bar: six full layers and one at fill 0.4 is exact; six full layers is 6.7 % off."""
    exact = 100.0 * 10 / (2 * 6.4 * E0)
    partial, binary = _tension_tip(7, top_fill=0.4), _tension_tip(6)
    assert abs(partial / exact - 1) < 1e-8
    assert abs(binary / exact - 1) > 0.05
    assert abs(partial / _recorded()["_partial_ux"] - 1) < 1e-8


@pytest.mark.parametrize("nd", [2, 4, 8])
def test_cantilever_against_timoshenko(nd):
    """Tip deflection over Timoshenko's (shear locking of the trilinear brick makes it stiffer),
    equal to the reference's ratio to the printed 0.1 %."""
    d = b = 4.0
    L, P = 40.0, 10.0
    bar = Bar(10 * nd, nd, nd, h=d / nd)
    clamp = bar.nodes(x=0.0)
    fixed = (3 * clamp[:, None] + np.arange(3)).ravel()
    u = _solve(bar, fixed, np.full(bar.g.nelem, E0), bar.end_face_load(-P, 2, np.ones(bar.g.nelem)))
    I = b * d ** 3 / 12
    Gs = E0 / (2 * (1 + NU))
    timo = P * L ** 3 / (3 * E0 * I) + P * L / (5 / 6 * Gs * b * d)
    ratio = -bar.tip_mean(u, 2) / timo
    printed = dict((int(a), float(r)) for a, r in
                   re.findall(r"(\d+) deep ([\d.]+)%", _recorded()["check_cantilever"]["detail"]))
    assert abs(100 * ratio - printed[nd]) <= 0.051
    assert {2: (0.84, 0.90), 4: (0.93, 0.98), 8: (0.97, 0.995)}[nd][0] <= ratio


def test_reruns_are_bit_identical():
    bar = Bar(20, 4, 4)
    clamp = bar.nodes(x=0.0)
    fixed = (3 * clamp[:, None] + np.arange(3)).ravel()
    F = bar.end_face_load(-1.0, 2, np.ones(bar.g.nelem))
    digests = set()
    for _ in range(2):
        fem = G.FEM(bar.g, np.ones(bar.g.nelem, bool), fixed, NU)
        u = fem.solve(fem.assemble(np.full(bar.g.nelem, E0)), [fem.reduce_load(F)])[0]
        digests.add(hashlib.sha256(u.tobytes()).hexdigest())
        fem.close()
    assert len(digests) == 1


def test_optimised_cantilever_beats_uniform():
    r = O.benchmark_cantilever()
    assert r["stiffer_pct"] > 20 and abs(r["vol_err"]) < 1e-3
    printed = float(re.search(r"([\d.]+)% stiffer", _recorded()["check_simp"]["detail"]).group(1))
    assert abs(r["stiffer_pct"] - printed) < 2.0
