"""Edge cases of the update: empty and completely filled number-conserving chains
(one charge block of one state), a chain of two sites (one bond, no even sweep),
and a bond whose outer Lambdas keep a single Schmidt value."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("filling", ["empty", "full"])
def test_nc_chain_with_one_charge_state_stays_put(pkg, oracle, filling):
    H = pkg.hamiltonians
    L, d, chi = 6, 3, 4
    N = 0 if filling == "empty" else L * (d - 1)
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 2.0), 0.05, 2)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        te = [c.trotter_step(U, 2) for _ in range(2)]
        g1, l1, ll1, lr1 = c.get_state()
    rte = [oracle.trotter_step_nc(gam, lam, ll, lr, U, N, d - 1, 2) for _ in range(2)]
    assert np.allclose(te, rte, atol=1e-12) and max(te) < 1e-12
    for a, b, la, lb in zip(l1, lam, ll1, ll):
        assert np.allclose(a, b, atol=1e-12) and np.array_equal(la, lb)
        assert abs(a[0] - 1.0) < 1e-12 and np.all(a[1:] == 0.0)
    n = obs.one_site_expval(g1, l1, np.diag(np.arange(d, dtype=float)))
    assert np.allclose(n, 0.0 if filling == "empty" else d - 1, atol=1e-12)


@pytest.mark.parametrize("order", [2, 5])
def test_two_site_chain(pkg, oracle, order):
    """L = 2: one bond; the second order's even sweep and the Forest-Ruth even
    sweeps are empty."""
    H = pkg.hamiltonians
    L, d, chi = 2, 3, 3
    rng = np.random.default_rng(21)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    U = H.construct_propagators(H.heisenberg(L, 1.0, 0.7, 0.4, spin=1.0), 0.1, order)
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        te = [c.trotter_step(U, order) for _ in range(3)]
        g1, l1 = c.get_state()
    rte = [oracle.trotter_step(gam, lam, U, order) for _ in range(3)]
    assert np.allclose(te, rte, atol=1e-12)
    assert np.allclose(l1[1], lam[1], atol=1e-11)
    assert abs(abs(np.vdot(obs.state_vector(gam, lam), obs.state_vector(g1, l1))) - 1.0) < 1e-11


def test_bond_between_single_valued_lambdas(pkg, oracle):
    """Lambda0 and Lambda2 with one nonzero value: Theta compacts to d x d."""
    rng = np.random.default_rng(22)
    chi, d = 16, 4
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(4)]
    lam = [np.eye(chi)[0] for _ in range(5)]
    lam[2] = np.exp(-np.arange(chi) / 3.0)
    lam[2] /= np.linalg.norm(lam[2])
    U = pkg.hamiltonians.matrix_exponential(pkg.hamiltonians.heisenberg(4, 1.0, 1.0, 1.0, spin=1.5)[1], 0.4)
    with pkg.Chain(4, d, chi) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    assert np.allclose(l1, rl1, atol=1e-12) and abs(te - rte) < 1e-12
    assert np.count_nonzero(l1) <= d
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-12)
