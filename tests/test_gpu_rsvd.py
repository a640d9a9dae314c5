"""The randomized SVD route (TEBD_SVD_RSVD) against the oracle.

A bond whose compacted Theta (n = d chi) is much larger than the kept rank
(chi + oversampling + 16 <= n) is decomposed from a sketch: FP64-class products on
the tensor cores, two FP64 SVDs of n x (chi + p), and a judge on every kept
triplet's residual.  Checked here:
* accepted bonds (judge tolerance 1e-5 of ||Theta|| on the residuals; these
  synthetic bonds have slowly decaying spectra, sigma_chi / sigma_0 ~ 0.1-0.25):
  the chi kept singular values within 1e-8 of s_max, Lambda within 1e-8,
  truncation error within 1e-8 relative -- the error goes as the square of the
  residual;
* a tolerance no sketch can meet sends every bond to the full SVD: then the
  results meet the FP64 bars (1e-12 relative on sigma, 1e-11 on Lambda);
* a batched sweep of saturated bonds (faster-decaying Lambdas) against the
  plain FP64 route: two-site density matrices within 1e-8.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _saturated(L, d, chi, seed, decay=16.0):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = []
    for _ in range(L + 1):
        l = np.exp(-np.arange(chi) / decay)
        lam.append(l / np.linalg.norm(l))
    return gam, lam


def _unitary(n, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("chi,d,p,q", [(48, 5, 64, 2), (48, 5, 128, 1), (64, 4, 48, 2), (40, 6, 64, 3)])
def test_rsvd_bond_matches_oracle(pkg, oracle, chi, d, p, q):
    gam, lam = _saturated(4, d, chi, chi + d)
    U = _unitary(d * d, 5)
    with pkg.Chain(4, d, chi, svd_mode=pkg.SVD_RSVD) as c:
        c.set_rsvd(oversample=p, power_iters=q)
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        l1 = c.get_lambda(3)
        st = c.stats()
    assert st["rsvd_updates"] == 1 and st["rsvd_fallbacks"] == 0, st
    _, _, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    assert len(s) == chi
    assert np.max(np.abs(s - rs[:chi])) <= 1e-8 * rs[0]
    assert np.max(np.abs(l1 - rl1)) < 1e-8
    assert abs(te - rte) < 1e-12 + 1e-8 * rte


def test_rsvd_unmeetable_tolerance_falls_back_to_full_svd(pkg, oracle):
    chi, d = 48, 5
    gam, lam = _saturated(4, d, chi, 3)
    U = _unitary(d * d, 4)
    with pkg.Chain(4, d, chi, svd_mode=pkg.SVD_RSVD) as c:
        c.set_rsvd(oversample=32, power_iters=0, tol=1e-300)
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        l1 = c.get_lambda(3)
        st = c.stats()
    assert st["rsvd_updates"] == 1 and st["rsvd_fallbacks"] == 1, st
    _, _, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    rs = rs[:len(s)]
    assert np.all(np.abs(s - rs) <= 1e-12 * rs + 1e-13 * rs[0])
    assert np.max(np.abs(l1 - rl1)) < 1e-11
    assert abs(te - rte) < 1e-11


def test_rsvd_sweep_matches_plain_fp64(pkg):
    from oracle import observables as obs

    H = pkg.hamiltonians
    L, d, chi = 12, 5, 48
    gam, lam = _saturated(L, d, chi, 9, decay=6.0)
    Hb = H.bose_hubbard(L, d, 1.0, 2.0)
    gate = H.matrix_exponential(Hb[1], 0.005)
    links = list(range(1, L, 2))
    res = {}
    for mode in (pkg.SVD_FP64, pkg.SVD_RSVD):
        with pkg.Chain(L, d, chi, svd_mode=mode) as c:
            c.set_state(gam, lam)
            te = c.apply_bonds(links, [gate] * len(links))
            g, l = c.get_state()
            res[mode] = (te, g, l, c.stats())
    te0, g0, l0, _ = res[pkg.SVD_FP64]
    te1, g1, l1, st = res[pkg.SVD_RSVD]
    assert st["rsvd_updates"] == len(links)
    assert np.max(np.abs(te1 - te0)) < 1e-10
    for k in links:
        a = obs.two_site_rho(l0[k - 1], g0[k - 1], l0[k], g0[k], l0[k + 1])
        b = obs.two_site_rho(l1[k - 1], g1[k - 1], l1[k], g1[k], l1[k + 1])
        assert np.max(np.abs(a - b)) < 1e-8, k


def test_rsvd_wide_sketch_chi1024(pkg):
    """The learned-rank configuration's largest bonds: d = 3, chi = 1024 (Theta
    3072 x 3072), a sketch of 1152 columns (p = 128, wider than 1024: the
    Cholesky's recursive blocking and the widest product tiles), on a state
    prepared by one double-float sweep; two-site density matrices (device
    observables) and Lambdas against plain FP64 within 1e-8."""
    H = pkg.hamiltonians
    L, d, chi = 4, 3, 1024
    gam, lam = _saturated(L, d, chi, 11, decay=128.0)
    gate = H.matrix_exponential(H.bose_hubbard(L, d, 1.0, 2.0)[1], 0.005)
    links = [1, 3]
    with pkg.Chain(L, d, chi, svd_mode=pkg.SVD_DF) as c:
        c.set_state(gam, lam)
        c.apply_bonds(links, [gate] * len(links))
        gam, lam = c.get_state()
    res = {}
    for mode in (pkg.SVD_FP64, pkg.SVD_RSVD):
        with pkg.Chain(L, d, chi, svd_mode=mode) as c:
            c.set_state(gam, lam)
            if mode == pkg.SVD_RSVD:
                c.set_theta_form(107)
                c.set_rsvd(oversample=128, power_iters=2)
            c.apply_bonds(links, [gate] * len(links))
            res[mode] = ([c.two_site_rho(k) for k in links], c.get_state()[1], c.stats())
    r0, l0, _ = res[pkg.SVD_FP64]
    r1, l1, st = res[pkg.SVD_RSVD]
    assert st["rsvd_updates"] == len(links) and st["rsvd_fallbacks"] == 0
    for a, b in zip(r0, r1):
        assert np.max(np.abs(a - b)) < 1e-8
    for k in links:
        assert np.max(np.abs(l0[k] - l1[k])) < 1e-8
