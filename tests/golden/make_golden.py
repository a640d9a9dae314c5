"""Generate tests/golden/propagators_d4.npz from the reference's own gate fixtures.

Reads the 16x16 REAL/IMAG propagator tables of
Case_Studies/Extensible_Wrapper/Propagator_{0.005,0.01}_{left,bulk,right}_{REAL,IMAG}.nml
(d = 4 Liouvillian gates, read by TEBDSolve.f90:172-206 with list-directed
`read(11,*)`, i.e. column-major fill) and records, for a seeded random chi=6,
d=4 bond, the oracle's outputs for each gate.  Run here, where the reference
tree is mounted:  python tests/golden/make_golden.py /path/to/OpenTEBD-extended
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

NAMES = ["0.005_left", "0.005_bulk", "0.005_right", "0.01_left", "0.01_bulk", "0.01_right"]


def read_gate(ref, name):
    base = os.path.join(ref, "Case_Studies", "Extensible_Wrapper", "Propagator_%s_%%s.nml" % name)
    re_ = np.loadtxt(base % "REAL").T  # list-directed read fills columns first
    im_ = np.loadtxt(base % "IMAG").T
    return re_ + 1j * im_


def random_bond(chi, d, seed):
    rng = np.random.default_rng(seed)
    g = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
         for _ in range(2)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(3)]
    lam = [l / np.linalg.norm(l) for l in lam]
    return g, lam


def main(ref):
    chi, d = 6, 4
    out = {"chi": chi, "d": d, "names": np.array(NAMES)}
    g, lam = random_bond(chi, d, 2024)
    out["gamma1"], out["gamma2"] = g
    out["lam0"], out["lam1"], out["lam2"] = lam
    for nm in NAMES:
        U = read_gate(ref, nm)
        g1, g2, l1, te, s = O.two_site_op(g[0], g[1], lam[0], lam[1], lam[2], U)
        key = nm.replace(".", "p")
        out["gate_" + key] = U
        out["sigma_" + key] = s
        out["lambda_" + key] = l1
        out["truncerr_" + key] = te
    np.savez_compressed(os.path.join(HERE, "propagators_d4.npz"), **out)
    print("wrote", os.path.join(HERE, "propagators_d4.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the OpenTEBD-extended tree>")
    main(sys.argv[1])
