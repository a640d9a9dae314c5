"""The kept-rank form (tebd_set_rank_bound): after an update the fewest leading
singular values whose discarded weight stays within the bound are kept, the rest
of Lambda becomes exact zeros.  Checked against the oracle's full spectrum."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


def random_bond(chi, d, seed, width):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(4)]
    lam = []
    for _ in range(5):
        l = np.exp(-np.arange(chi) / width)
        lam.append(l / np.linalg.norm(l))
    return gam, lam


def expected_keep(s_all, chi, bound):
    """Fewest leading values with (weight beyond chi) + (dropped kept values) <= bound."""
    s = np.asarray(s_all)
    top = np.where(s[:chi] > 1e-15, s[:chi], 0.0)
    w = max(1.0 - np.sum(top ** 2), 0.0)
    keep = chi
    while keep > 1 and w + top[keep - 1] ** 2 <= bound:
        w += top[keep - 1] ** 2
        keep -= 1
    return keep


@pytest.mark.parametrize("svd_mode", [0, 4, 5])
@pytest.mark.parametrize("bound", [1e-6, 1e-4, 1e-3])
def test_rank_bound_dense_update(pkg, oracle, svd_mode, bound):
    chi, d = 96, 4  # n = 384: bidiagonal route in modes 0 and 5, QR + Jacobi in mode 4
    gam, lam = random_bond(chi, d, 5, 8.0)
    U = pkg.hamiltonians.matrix_exponential(pkg.hamiltonians.heisenberg(4, 1.0, 0.8, 0.6, spin=1.5)[1], 0.3)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    keep = expected_keep(rs, chi, bound)
    assert 1 < keep < chi
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        c.set_rank_bound(bound)
        te = c.two_site_op(2, U)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    assert np.all(l1[keep:] == 0.0) and np.all(l1[:keep] > 0.0)
    kw = np.sum(rs[:keep] ** 2)
    assert np.allclose(l1[:keep], rs[:keep] / np.sqrt(kw), atol=1e-11)
    assert abs(te - (1.0 - kw)) < 1e-11 and te <= bound * (1 + 1e-9) + 1e-15
    # the kept part of the bond is the rank-`keep` truncation of the oracle's update
    rl_k = np.where(np.arange(chi) < keep, rs[:chi] / np.sqrt(kw), 0.0)
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl_k, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-10)


def test_rank_bound_zero_is_the_reference_rule(pkg, oracle):
    chi, d = 32, 3
    gam, lam = random_bond(chi, d, 6, 6.0)
    U = pkg.hamiltonians.matrix_exponential(pkg.hamiltonians.heisenberg(4, 1.0, 1.0, 0.5, spin=1.0)[1], 0.2)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    with pkg.Chain(4, d, chi) as c:
        c.set_state(gam, lam)
        c.set_rank_bound(1e-3)
        c.set_rank_bound(0.0)
        te = c.two_site_op(2, U)
        l1 = c.get_lambda(3)
        with pytest.raises(pkg.TebdError):
            c.set_rank_bound(-1e-3)
        with pytest.raises(pkg.TebdError):
            c.set_rank_bound(1.0)
    assert np.allclose(l1, rl1, atol=1e-11) and abs(te - rte) < 1e-11


def test_rank_bound_nc_update(pkg, oracle):
    """NC: kept values beyond the rank get Lambda 0 and label 10000."""
    H = pkg.hamiltonians
    L, d, chi, N = 8, 3, 16, 8
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, np.linspace(1.0, 3.0, L)), 0.2, 2)
    for _ in range(3):
        oracle.trotter_step_nc(gam, lam, ll, lr, U, N, d - 1, 2)
    link = 4
    r = oracle.two_site_op_nc(gam[link - 1], gam[link], lam[link - 1], lam[link], lam[link + 1], U[link - 1],
                              ll[link - 1], ll[link], lr[link], lr[link + 1], N, d - 1)
    s_sorted = np.sort(r[6])[::-1]
    bound = 1e-4
    keep = expected_keep(s_sorted, chi, bound)
    assert 1 < keep < min(chi, np.sum(s_sorted > 1e-10))
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        c.set_rank_bound(bound)
        te = c.two_site_op(link, U[link - 1])
        l1 = c.get_lambda(link + 1)
        lab_l, lab_r = c.get_labels(link + 1)
    kw = np.sum(s_sorted[:keep] ** 2)
    assert np.all(l1[keep:] == 0.0) and np.all(lab_l[keep:] == 10000) and np.all(lab_r[keep:] == 10000)
    assert np.allclose(np.sort(l1[:keep])[::-1], s_sorted[:keep] / np.sqrt(kw), atol=1e-11)
    assert abs(te - (1.0 - kw)) < 1e-11
