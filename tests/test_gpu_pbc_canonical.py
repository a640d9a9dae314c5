"""Swapping, the periodic-boundary 2nd-order Trotter step and CanonicalFormAllNC
through the C ABI against the oracle (gauge-invariant comparisons)."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


def rel_close(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b))) <= tol * max(1.0, float(np.max(np.abs(b))))


def random_bond(chi, d, seed, L=4):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(L + 1)]
    lam = [l / np.linalg.norm(l) for l in lam]
    return gam, lam


@pytest.mark.parametrize("chi,d", [(6, 2), (12, 3)])
def test_swapping_matches_oracle(pkg, oracle, chi, d):
    """Unnormalised random bond: Swapping keeps the raw singular values, so the
    truncation error is |1 - sum of kept S^2| of the unnormalised Theta."""
    gam, lam = random_bond(chi, d, 40 + chi)
    with pkg.Chain(4, d, chi) as c:
        c.set_state(gam, lam)
        te = c.swapping(2)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    rg1, rg2, rl1, rte = oracle.swapping(gam[1], gam[2], lam[1], lam[2], lam[3])
    assert np.allclose(l1, rl1, atol=1e-11)
    assert abs(te - rte) <= 1e-11 * max(1.0, abs(rte))
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert rel_close(rho, rrho, 1e-11)


def test_swap_twice_is_identity(pkg):
    H = pkg.hamiltonians
    L, d, chi = 6, 2, 8
    rng = np.random.default_rng(3)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    U = H.construct_propagators(H.heisenberg(L, 1.0, 1.0, 0.3), 0.1, 2)
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        for _ in range(3):
            c.trotter_step(U, 2)
        g0, l0 = c.get_state()
        t1 = c.swapping(3)
        t2 = c.swapping(3)
        g1, l1 = c.get_state()
    assert t1 < 1e-12 and t2 < 1e-12
    for a, b in zip(l1, l0):
        assert np.allclose(a, b, atol=1e-12)
    assert abs(abs(obs.inner_product(g0, l0, g1, l1)) - 1.0) < 1e-12


@pytest.mark.parametrize("L", [6, 7])
def test_trotter_step_pbc_matches_oracle(pkg, oracle, L):
    H = pkg.hamiltonians
    d, chi, dt = 2, 8, 0.05
    rng = np.random.default_rng(L)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    Hb = H.heisenberg(L, 1.0, 1.0, 0.5)
    U = list(H.construct_propagators(Hb, dt, 2)) + [H.matrix_exponential(Hb[1], dt)]  # Udt(L): edge
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        te = [c.trotter_step_pbc(U) for _ in range(2)]
        g_gpu, l_gpu = c.get_state()
    rte = [oracle.trotter_step_pbc(gam, lam, U) for _ in range(2)]
    assert np.allclose(te, rte, atol=1e-10)
    for a, b in zip(l_gpu, lam):
        assert np.allclose(a, b, atol=1e-10)
    sz = np.diag([0.5, -0.5])
    assert np.allclose(obs.one_site_expval(g_gpu, l_gpu, sz), obs.one_site_expval(gam, lam, sz), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g_gpu, l_gpu)) - 1.0) < 1e-10


@pytest.mark.parametrize("L,chi", [(6, 8), (7, 8), (7, 4)])
def test_trotter_step_pbc_forest_ruth_matches_oracle(pkg, oracle, L, chi):
    """TrotterStep5thOrderPBC in both gate layouts (even L: 2L gates, odd L: 3L),
    exact (chi = 8) and truncated (chi = 4)."""
    H = pkg.hamiltonians
    d, dt = 2, 0.05
    rng = np.random.default_rng(100 + L)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    hb = H.heisenberg(L, 1.0, 1.0, 0.5)[0]
    U = H.construct_propagators([hb] * L, dt, 5, boundary="P")
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        te = [c.trotter_step_pbc(U, 5) for _ in range(2)]
        g_gpu, l_gpu = c.get_state()
        with pytest.raises(pkg.TebdError):
            c.trotter_step_pbc(U[: len(U) - 1], 5)
    rte = [oracle.trotter_step_pbc(gam, lam, U, 5) for _ in range(2)]
    assert np.allclose(te, rte, atol=1e-10)
    for a, b in zip(l_gpu, lam):
        assert np.allclose(a, b, atol=1e-10)
    sz = np.diag([0.5, -0.5])
    assert np.allclose(obs.one_site_expval(g_gpu, l_gpu, sz), obs.one_site_expval(gam, lam, sz), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g_gpu, l_gpu)) - 1.0) < 1e-10


def test_canonical_form_all_nc_matches_oracle(pkg, oracle):
    H = pkg.hamiltonians
    L, d, chi, N = 8, 3, 12, 8
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 1.0, 0.0), 0.05, 2)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        for _ in range(2):
            c.trotter_step(U, 2)
        gam, lam, ll, lr = c.get_state()
        c.canonical_form_all_nc()
        g2, l2, ll2, lr2 = c.get_state()
    eye = np.eye(d * d, dtype=complex)
    gam, lam, ll, lr = list(gam), list(lam), list(ll), list(lr)
    for link in list(range(1, L)) + list(range(L - 1, 0, -1)):
        r = oracle.two_site_op_nc(gam[link - 1], gam[link], lam[link - 1], lam[link], lam[link + 1], eye,
                                  ll[link - 1], ll[link], lr[link], lr[link + 1], N, d - 1)
        gam[link - 1], gam[link], lam[link], ll[link], lr[link] = r[0], r[1], r[2], r[3], r[4]
    for a, b in zip(l2, lam):
        assert np.allclose(a, b, atol=1e-10)
    num = np.diag(np.arange(d, dtype=float))
    assert np.allclose(obs.one_site_expval(g2, l2, num), obs.one_site_expval(gam, lam, num), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g2, l2)) - 1.0) < 1e-10


def _rho_normalised(l0, g1, l1, g2, l2):
    r = obs.two_site_rho(l0, g1, l1, g2, l2)
    return r / np.trace(r).real


@pytest.mark.parametrize("chi,d", [(6, 2), (16, 3)])
def test_canonical_form_matches_oracle(pkg, oracle, chi, d):
    """One bond of a random (non-canonical) chain: the new Lambda1 and the bond's
    normalised two-site density matrix (Gammas only up to the SVD gauge)."""
    gam, lam = random_bond(chi, d, 70 + chi)
    with pkg.Chain(4, d, chi) as c:
        c.set_state(gam, lam)
        c.canonical_form(2)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    rg1, rl1, rg2 = oracle.canonical_form(lam[1], gam[1], lam[2], gam[2], lam[3])
    assert np.allclose(l1, rl1, atol=1e-11)
    assert rel_close(_rho_normalised(lam[1], g1, l1, g2, lam[3]), _rho_normalised(lam[1], rg1, rl1, rg2, lam[3]),
                     1e-10)


def test_canonical_form_all_matches_oracle(pkg, oracle):
    rng = np.random.default_rng(9)
    L, d, chi = 6, 2, 6
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(L + 1)]
    lam[0] = np.eye(chi)[0]
    lam[L] = np.eye(chi)[0]
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        c.canonical_form_all()
        g_gpu, l_gpu = c.get_state()
    oracle.canonical_form_all(gam, lam)
    for a, b in zip(l_gpu, lam):
        assert np.allclose(a, b, atol=1e-10)
    sz = np.diag([0.5, -0.5])
    ea = obs.one_site_expval(g_gpu, l_gpu, sz) / obs.one_site_expval(g_gpu, l_gpu, np.eye(2))
    eb = obs.one_site_expval(gam, lam, sz) / obs.one_site_expval(gam, lam, np.eye(2))
    assert np.allclose(ea, eb, atol=1e-10)
