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


def _nc_bond_with_large_blocks(chi=96, d=3, N=20, seed=8):
    """A link-2 bond of an L=4 chain whose charge blocks are 64x32, 96x64, 64x96
    and 32x64: alpha labels {8,9,10}, beta labels {9..12}, gamma labels {7,8,9}."""
    rng = np.random.default_rng(seed)
    L = 4
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = []
    for _ in range(L + 1):
        l = np.exp(-np.arange(chi) / 24.0)
        lam.append(l / np.linalg.norm(l))
    ll = [np.full(chi, 10000, dtype=np.int32) for _ in range(L + 1)]
    lr = [np.full(chi, 10000, dtype=np.int32) for _ in range(L + 1)]
    ll[1] = np.repeat(np.array([8, 9, 10], dtype=np.int32), chi // 3)
    ll[2] = np.repeat(np.array([9, 10, 11, 12], dtype=np.int32), chi // 4)
    lr[3] = np.repeat(np.array([7, 8, 9], dtype=np.int32), chi // 3)
    for k in (1, 2):
        lr[k] = (N - ll[k]).astype(np.int32)
    ll[3] = (N - lr[3]).astype(np.int32)
    return gam, lam, ll, lr


@pytest.mark.parametrize("svd_mode", [0, 5])
def test_nc_large_blocks_take_the_bidiagonal_route(pkg, oracle, svd_mode):
    """Blocks with both sides >= 16 go through the bidiagonal route (all their
    triplets; here all four blocks), the update matches the oracle's per-block
    ZGESVD."""
    chi, d, N = 96, 3, 20
    gam, lam, ll, lr = _nc_bond_with_large_blocks(chi, d, N)
    Hb = pkg.hamiltonians.bose_hubbard(4, d, 1.0, 2.0)
    U = pkg.hamiltonians.matrix_exponential(Hb[1], 0.3)
    with pkg.Chain(4, d, chi, mode=pkg.MODE_NC, tot_num=N, svd_mode=svd_mode) as c:
        c.set_state(gam, lam, ll, lr)
        c.reset_stats()
        te = c.two_site_op(2, U)
        assert c.stats()["gebrd_launches"] >= 1
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
        la, lb = c.get_labels(3)
    r = oracle.two_site_op_nc(gam[1], gam[2], lam[1], lam[2], lam[3], U, ll[1], ll[2], lr[2], lr[3], N, d - 1)
    rg1, rg2, rl1, rll1, rlr1, rte, rs = r
    assert abs(te - rte) < 1e-11
    assert np.allclose(np.sort(l1), np.sort(rl1), atol=1e-11)
    assert sorted(zip(np.round(l1, 8), la)) == sorted(zip(np.round(rl1, 8), rll1))
    assert np.all(np.isfinite(g1)) and np.all(np.isfinite(g2))
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-11)
