"""GPU parity of the number-conserving routines with internal degrees of freedom
(TwoSiteOpNC / TrotterStepNC with intDegFree and Conserv%vi), SwappingNC and the
number-conserving periodic steps against the oracle."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu

CONSERV = np.array([0, 1, 1, 2])  # |0>, |a>, |b>, |ab>


def two_species_bond(ta=1.0, tb=0.6, U=1.0, V=0.3, x=0.2):
    ca = np.zeros((4, 4))
    cb = np.zeros((4, 4))
    ca[0, 1] = ca[2, 3] = 1.0
    cb[0, 2] = cb[1, 3] = 1.0
    na, nb = ca.T @ ca, cb.T @ cb
    e = np.eye(4)
    h = -ta * (np.kron(ca.T, ca) + np.kron(ca, ca.T)) - tb * (np.kron(cb.T, cb) + np.kron(cb, cb.T))
    h = h + U * (np.kron(na @ nb, e) + np.kron(e, na @ nb)) + V * np.kron(na, nb)
    return h + 1j * x * (np.kron(ca.T @ cb, cb.T @ ca) - np.kron(cb.T @ ca, ca.T @ cb))


def sector_state(H, L, chi, seed):
    rng = np.random.default_rng(seed)
    c0 = np.zeros((4, L), complex)
    nums = [(1, 1, 2, 0)[s % 4] for s in range(L)]
    for s, n in enumerate(nums):
        idx = [j for j in range(4) if CONSERV[j] == n]
        c0[idx, s] = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    c0 /= np.linalg.norm(c0, axis=0)
    N = int(sum(nums))
    gam, lam = H.product_state(c0, chi)
    ll, lr = H.product_state_labels(c0, chi, N, CONSERV)
    return gam, lam, ll, lr, N


@pytest.mark.parametrize("L,chi,order", [(6, 16, 2), (6, 16, 5), (8, 10, 2)])
def test_nc_intdegfree_trotter_matches_oracle(pkg, oracle, L, chi, order):
    H = pkg.hamiltonians
    d = 4
    gam, lam, ll, lr, N = sector_state(H, L, chi, 30 + L + order)
    hb = [two_species_bond(U=1.0 + 0.1 * s) for s in range(L - 1)]
    U = H.construct_propagators(hb, 0.05, order)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N, max_filling=2, conserv=CONSERV) as c:
        c.set_state(gam, lam, ll, lr)
        te = [c.trotter_step(U, order) for _ in range(3)]
        g1, l1, ll1, lr1 = c.get_state()
    rte = [oracle.trotter_step_nc(gam, lam, ll, lr, U, N, 2, order, conserv=CONSERV) for _ in range(3)]
    assert np.allclose(te, rte, atol=1e-10)
    for link, (a, b, la, lb) in enumerate(zip(l1, lam, ll1, ll), start=1):
        assert np.allclose(np.sort(a), np.sort(b), atol=1e-10), link
        assert sorted(zip(np.round(a, 8), la)) == sorted(zip(np.round(b, 8), lb)), link
    for la, ra in zip(ll1, lr1):
        used = la < 1000
        assert np.all(ra[used] == N - la[used]) and np.all(ra[~used] == 10000)
    nop = np.diag(CONSERV.astype(float))
    n1, n2 = obs.one_site_expval(g1, l1, nop), obs.one_site_expval(gam, lam, nop)
    assert np.allclose(n1, n2, atol=1e-10)
    assert abs(n1.sum() - N) < 1e-6
    assert np.allclose(obs.bond_energy(g1, l1, hb), obs.bond_energy(gam, lam, hb), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g1, l1)) - 1.0) < 1e-10


def test_nc_identity_conserv_is_the_plain_update(pkg):
    """Conserv(i) = i-1 runs the intDegFree kernels on the plain problem: same state."""
    H = pkg.hamiltonians
    L, d, chi, N = 8, 3, 12, 8
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, np.linspace(1.0, 3.0, L)), 0.05, 2)
    out = []
    for cons in (None, np.arange(d)):
        with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N, conserv=cons) as c:
            c.set_state(gam, lam, ll, lr)
            te = [c.trotter_step(U, 2) for _ in range(3)]
            out.append((te,) + tuple(c.get_state()))
    (t0, g0, l0, ll0, lr0), (t1, g1, l1, ll1, lr1) = out
    assert np.allclose(t0, t1, atol=1e-13)
    for a, b in zip(l0, l1):
        assert np.allclose(a, b, atol=1e-13)
    for a, b in zip(ll0 + lr0, ll1 + lr1):
        assert np.array_equal(a, b)
    assert abs(abs(obs.inner_product(g0, l0, g1, l1)) - 1.0) < 1e-12


def test_conserv_and_filling_errors(pkg):
    with pkg.Chain(4, 2, 4) as c:
        with pytest.raises(pkg.TebdError):
            c.set_conserv([0, 1])  # dense handle
    with pkg.Chain(4, 8, 4, mode=pkg.MODE_NC, tot_num=2, max_filling=2) as c:
        with pytest.raises(pkg.TebdError):
            c.set_conserv([0] * 8)  # 64 pairs share the total 0
        with pytest.raises(pkg.TebdError):
            c.set_conserv([0, 1, -1, 2, 0, 1, 1, 2])
        with pytest.raises(pkg.TebdError):
            c.set_conserv([0, 1, 3, 2, 0, 1, 1, 2])  # above max_filling
    # without intDegFree the physical index is the number: max_filling = d-1
    H = pkg.hamiltonians
    gam, lam, ll, lr = H.initial_set_nc(4, 2, 4, 2)
    for mf in (0, 2):
        with pkg.Chain(4, 2, 4, mode=pkg.MODE_NC, tot_num=2, max_filling=mf) as c:
            c.set_state(gam, lam, ll, lr)
            with pytest.raises(pkg.TebdError) as e:
                c.two_site_op(1, np.eye(4, dtype=complex))
            assert "max_filling" in str(e.value)


def _nc_evolved(pkg, L, d, chi, N, conserv=None, steps=2):
    """A number-conserving chain after a few open-boundary steps (oracle)."""
    from oracle import oracle
    H = pkg.hamiltonians
    if conserv is None:
        gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
        hb = H.bose_hubbard(L, d, 1.0, np.linspace(1.0, 3.0, L))
        mf = d - 1
    else:
        gam, lam, ll, lr, N = sector_state(H, L, chi, 5)
        hb = [two_species_bond(U=1.0 + 0.1 * s) for s in range(L - 1)]
        mf = 2
    U = H.construct_propagators(hb, 0.1, 2)
    for _ in range(steps):
        oracle.trotter_step_nc(gam, lam, ll, lr, U, N, mf, 2, conserv=conserv)
    return gam, lam, ll, lr, N, mf


@pytest.mark.parametrize("idf", [False, True])
def test_swapping_nc_matches_oracle(pkg, oracle, idf):
    L = 6
    d, chi = (4, 12) if idf else (3, 9)
    cons = CONSERV if idf else None
    gam, lam, ll, lr, N, mf = _nc_evolved(pkg, L, d, chi, L, cons)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N, max_filling=mf, conserv=cons) as c:
        c.set_state(gam, lam, ll, lr)
        te = c.swapping(3)
        g1, l1, ll1, lr1 = c.get_state()
    rg1, rg2, rl1, rll1, rlr1, rte = oracle.swapping_nc(gam[2], gam[3], lam[2], lam[3], lam[4], ll[2], ll[3],
                                                        lr[3], lr[4], N, mf, conserv=cons)
    assert abs(te - rte) < 1e-11
    assert np.allclose(np.sort(l1[3]), np.sort(rl1), atol=1e-11)
    assert sorted(zip(np.round(l1[3], 8), ll1[3])) == sorted(zip(np.round(rl1, 8), rll1))
    rho = obs.two_site_rho(lam[2], g1[2], l1[3], g1[3], lam[4])
    rrho = obs.two_site_rho(lam[2], rg1, rl1, rg2, lam[4])
    assert np.allclose(rho, rrho, atol=1e-11)


@pytest.mark.parametrize("L,order,idf", [(5, 2, False), (6, 5, False), (5, 5, True), (6, 2, True)])
def test_trotter_step_pbc_nc_matches_oracle(pkg, oracle, L, order, idf):
    """TrotterStep2ndOrderPBCNC / 5thOrderPBCNC, plain and with intDegFree."""
    H = pkg.hamiltonians
    d, chi = (4, 12) if idf else (3, 9)
    cons = CONSERV if idf else None
    gam, lam, ll, lr, N, mf = _nc_evolved(pkg, L, d, chi, L, cons, steps=1)
    hb = two_species_bond() if idf else H.bose_hubbard(L, d, 1.0, 2.0)[1]
    U = H.construct_propagators([hb] * L, 0.05, order, boundary="P")
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N, max_filling=mf, conserv=cons) as c:
        c.set_state(gam, lam, ll, lr)
        te = [c.trotter_step_pbc(U, order) for _ in range(2)]
        g1, l1, ll1, lr1 = c.get_state()
    rte = [oracle.trotter_step_pbc_nc(gam, lam, ll, lr, U, N, mf, order, conserv=cons) for _ in range(2)]
    assert np.allclose(te, rte, atol=1e-10)
    for link, (a, b, la, lb) in enumerate(zip(l1, lam, ll1, ll), start=1):
        assert np.allclose(np.sort(a), np.sort(b), atol=1e-10), link
        assert sorted(zip(np.round(a, 8), la)) == sorted(zip(np.round(b, 8), lb)), link
    nop = np.diag((CONSERV if idf else np.arange(d)).astype(float))
    assert np.allclose(obs.one_site_expval(g1, l1, nop), obs.one_site_expval(gam, lam, nop), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g1, l1)) - 1.0) < 1e-10
