"""GPU parity of the number-conserving update (TwoSiteOpNC / TrotterStepNC) against the oracle.

The reference keeps the labels (particle number left of each Schmidt index) as
part of the state, so besides the gauge-invariant checks (Lambdas, <n_i>, bond
energies, overlap) the labels are compared: exactly when the spectrum has no
cross-block degeneracy (random per-site U breaks the chain's reflection
symmetry), and as (lambda, label) multisets otherwise.
"""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


def nc_setup(pkg, L, d, chi, N, seed, dt, order=2, scalar_u=False):
    H = pkg.hamiltonians
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    rng = np.random.default_rng(seed)
    U = 2.0 if scalar_u else rng.uniform(1.0, 3.0, L)
    Hb = H.bose_hubbard(L, d, 1.0, U)
    Udt = H.construct_propagators(Hb, dt, order)
    return gam, lam, ll, lr, Hb, Udt


def state_close(pkg, gpu, ref, Hb, d, N, tol=1e-10, exact_labels=True):
    g1, l1, ll1, lr1 = gpu
    g2, l2, ll2, lr2 = ref
    for a, b in zip(l1, l2):
        assert np.allclose(np.sort(a), np.sort(b), atol=tol)
    for link, (a, b, la, lb) in enumerate(zip(l1, l2, ll1, ll2), start=1):
        if exact_labels:
            assert np.allclose(a, b, atol=tol), link
            assert np.array_equal(la, lb), (link, la, lb)
        else:
            ka = sorted(zip(np.round(a, 8), la))
            kb = sorted(zip(np.round(b, 8), lb))
            assert ka == kb, link
    for a, b in zip(lr1, lr2):
        assert np.array_equal(np.sort(a), np.sort(b))
    nop = np.diag(np.arange(d, dtype=float))
    n1 = obs.one_site_expval(g1, l1, nop)
    n2 = obs.one_site_expval(g2, l2, nop)
    assert np.allclose(n1, n2, atol=tol)
    # truncation to chi makes the canonical-form density slightly off N in both; the
    # GPU must reproduce the oracle's sum, and both stay close to N
    assert abs(n1.sum() - n2.sum()) < tol
    assert abs(n1.sum() - N) < 1e-4
    assert np.allclose(obs.bond_energy(g1, l1, Hb), obs.bond_energy(g2, l2, Hb), atol=tol)
    assert abs(abs(obs.inner_product(g2, l2, g1, l1)) - 1.0) < tol


@pytest.mark.parametrize("L,d,chi,N", [(6, 3, 9, 6), (8, 4, 16, 8)])
def test_nc_single_updates_match_oracle(pkg, oracle, L, d, chi, N):
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 3, 0.1)
    # a few oracle steps first so that every bond has several charge blocks
    for _ in range(3):
        oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, 2)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        for link in (1, L // 2, L - 1):
            te = c.two_site_op(link, Udt[link - 1])
            r = oracle.two_site_op_nc(gam[link - 1], gam[link], lam[link - 1], lam[link], lam[link + 1],
                                      Udt[link - 1], ll[link - 1], ll[link], lr[link], lr[link + 1], N, d - 1)
            gam[link - 1], gam[link], lam[link], ll[link], lr[link] = r[0], r[1], r[2], r[3], r[4]
            assert abs(te - r[5]) < 1e-11
            s = c.singular_values(link)
            assert s.shape == r[6].shape
            assert np.allclose(np.sort(s)[::-1], np.sort(r[6])[::-1], rtol=1e-10, atol=1e-13)
        state_close(pkg, c.get_state(), (gam, lam, ll, lr), Hb, d, N)


@pytest.mark.parametrize("order", [2, 5])
def test_nc_trotter_steps_match_oracle(pkg, oracle, order):
    L, d, chi, N = 8, 3, 12, 8
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 7, 0.05, order)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        for _ in range(4):
            te = c.trotter_step(Udt, order)
            rte = oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, order)
            assert abs(te - rte) < 1e-10
        state_close(pkg, c.get_state(), (gam, lam, ll, lr), Hb, d, N)


def test_nc_reflection_symmetric_chain(pkg, oracle):
    """Scalar U keeps the chain reflection symmetric: the centre bond has exactly
    degenerate blocks, so labels are compared as (lambda, label) multisets."""
    L, d, chi, N = 6, 3, 9, 6
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 0, 0.1, scalar_u=True)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        for _ in range(3):
            c.trotter_step(Udt, 2)
            oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, 2)
        state_close(pkg, c.get_state(), (gam, lam, ll, lr), Hb, d, N, exact_labels=False)


def test_nc_larger_bond_properties(pkg, oracle):
    """d=5, chi=48 (blocks of tens of rows, rectangular, both orientations):
    oracle parity plus conservation of N and label consistency."""
    L, d, chi, N = 10, 5, 48, 10
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 5, 0.2)
    for _ in range(4):
        oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, 2)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        te = c.trotter_step(Udt, 2)
        rte = oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, 2)
        assert abs(te - rte) < 1e-10
        g, l, lla, lra = c.get_state()
    state_close(pkg, (g, l, lla, lra), (gam, lam, ll, lr), Hb, d, N)
    for link in range(1, L + 2):
        used = lla[link - 1] < 1000
        assert np.all(lla[link - 1][used] + lra[link - 1][used] == N)
        assert np.all(l[link - 1][~used] == 0)


def test_nc_mode_errors(pkg):
    with pytest.raises(pkg.TebdError) as e:
        pkg.Chain(4, 3, 4, mode=pkg.MODE_NC, tot_num=1000)
    assert e.value.code == 1
    with pkg.Chain(4, 3, 4, mode=pkg.MODE_NC, tot_num=4) as c:
        with pytest.raises(pkg.TebdError) as e:
            pkg.TwoSiteOp(1, np.eye(9, dtype=complex), c)
        assert e.value.code == 6
