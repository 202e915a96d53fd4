"""Generate the large-grid parity fixtures in this folder with the FP64 CPU oracle.

The reference's own ``FEM.__init__`` needs about 44 KB of host memory per element for its CSR
pattern and scatter maps (fem.py:133-196), so it cannot build the 192x96x96 and 256x128x128
grids on a machine with less than 80-190 GB of RAM. At those sizes the oracle is the project's
FP64 matrix-free restatement of fem.py / optimize.py (oracle/oracle.py, oracle/anneal_oracle.c),
which tests/test_oracle_golden.py pins to the reference's own outputs on the grids the
reference can build (including the 48x24x24 cantilever, 50 iterations).

Fixtures written:

* ``lbracket192_30it.npz`` -- the 192x96x96 L-bracket (void x>96 and z>48, two clamped round
  patches with frozen shells, a round top load patch), E0 1, nu 0.3, p 3 from the first
  iteration (warm start from a uniform design), no projection, r 2.0, vf 0.25, Emin 1e-9, OC
  move 0.2, 30 SIMP iterations, CG relative residual 1e-6.
* ``lbracket256_3it.npz`` -- the same problem scaled to 256x128x128 (12.8M DOF), the first 3
  SIMP iterations.
* ``sixcase160_3it.npz`` -- the same problem at 160x80x80 (3.17M DOF) with six load cases (unit
  force along +-x, +-y, +-z on the top patch, summed compliance), the first 3 SIMP iterations;
  ``h_compliance_cases`` holds every case's compliance per iteration.

Each holds the per-iteration compliance, volume fraction, change and CG iterations, and the
final physical density quantised to uint16 (x = q / 65535, within 7.7e-6 of the oracle's): on
the full grid for 192x96x96; for 256x128x128 at every 17th element (``x_q16_stride17``: element
17 m, which visits every x position) together with the sum of the exact density over every
x-row (``row_sums``, index j + ny k), so the file stays small while every element is covered.

Run from the repository root (8 cores: about 9, 2 and 3 minutes):

    python tests/golden/make_oracle_fixtures.py [--only 192|256|six160]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = {
    "192": dict(scale=1.0, iters=30, name="lbracket192_30it.npz", sample=False),
    "256": dict(scale=4.0 / 3.0, iters=3, name="lbracket256_3it.npz", sample=True),
    "six160": dict(scale=5.0 / 6.0, iters=3, name="sixcase160_3it.npz", sample=True, six=True),
}


def run_case(scale, iters, name, log=print, sample=False, six=False):
    from anneal_gb300 import problems as P
    from oracle import oracle as O
    O.build()
    make = P.six_case_bracket if six else P.lbracket
    w = make(scale=scale, vf=0.25, r_vox=2.0, emin=1e-9)
    t0 = time.time()
    run = O.SimpRun(w.shape, 1.0, w.fill, w.active, w.frozen, w.fixed, w.loads, w.weights, w.E0, w.nu, w.vf,
                    iters=iters, r_mm=w.r_vox, p_final=3.0, move=0.2, x0=np.full(w.nelem, w.vf), beta_max=0.0,
                    rtol=1e-6, emin=1e-9, log=log)
    for _ in range(iters):
        run.step()
    x = run.full_x()
    q = np.round(np.clip(x, 0.0, 1.0) * 65535.0).astype(np.uint16)
    h = run.hist
    fields = {"x_q16_stride17": q[::17], "row_sums": x.reshape(-1, w.shape[0]).sum(axis=1)} if sample \
        else {"x_q16": q}
    if six:
        fields["h_compliance_cases"] = np.array([r["compliance"] for r in run.hist])
    np.savez_compressed(os.path.join(HERE, name), shape=np.array(w.shape), iters=iters, rtol=1e-6,
                        h_compliance=np.array([r["compliance"][0] for r in h]),
                        h_volumeFraction=np.array([r["volumeFraction"] for r in h]),
                        h_change=np.array([r["change"] for r in h]),
                        h_cg=np.array([r["cgIters"][0] for r in h]),
                        threads=O.num_threads(), seconds=time.time() - t0, **fields)
    log(f"{name}: {iters} iterations in {time.time() - t0:.0f} s on {O.num_threads()} threads")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=sorted(CASES))
    args = ap.parse_args()
    for key, c in CASES.items():
        if args.only and key != args.only:
            continue
        run_case(c["scale"], c["iters"], c["name"], sample=c["sample"], six=c.get("six", False))


if __name__ == "__main__":
    main()
