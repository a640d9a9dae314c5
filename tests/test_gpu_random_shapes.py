"""Seeded random shapes for the dense update: chi in 1..64, d in 2..5, Lambdas
with exact zeros anywhere and repeated values (ties), random unitary gates; plain
FP64 and the precision form against the oracle (hypothesis-style coverage with
fixed seeds, since the GPU image has no hypothesis)."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu

SIG_REL, SIG_ABS = 1e-12, 1e-13


def case(seed):
    rng = np.random.default_rng(1000 + seed)
    chi = int(rng.integers(1, 65))
    d = int(rng.integers(2, 6))
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(4)]
    lam = []
    for _ in range(5):
        l = np.sort(rng.random(chi))[::-1]
        if chi > 2 and rng.random() < 0.5:  # ties
            k = int(rng.integers(0, chi - 1))
            l[k + 1] = l[k]
        if chi > 1 and rng.random() < 0.5:  # exact zeros anywhere but the first
            l[rng.choice(np.arange(1, chi), size=int(rng.integers(1, max(2, chi // 3))), replace=False)] = 0.0
        lam.append(l / np.linalg.norm(l))
    z = (rng.standard_normal((d * d, d * d)) + 1j * rng.standard_normal((d * d, d * d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return chi, d, gam, lam, q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("seed", range(16))
@pytest.mark.parametrize("svd_mode", [0, 5])
def test_random_shape_matches_oracle(pkg, oracle, seed, svd_mode):
    chi, d, gam, lam, U = case(seed)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = np.asarray(c.singular_values(2))
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    ref = np.asarray(rs)[: len(s)]
    tol = SIG_REL * ref + SIG_ABS * max(ref[0], 1e-300)
    assert np.all(np.abs(s - ref) <= tol), (chi, d, float(np.max(np.abs(s - ref) - tol)))
    assert np.allclose(l1, rl1, atol=1e-11), (chi, d)
    assert abs(te - rte) < 1e-11
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-10), (chi, d)
