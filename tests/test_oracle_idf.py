"""Known answers for the oracle's number-conserving routines: the intDegFree
branches of FormThetaNC, ThetaOperationNC, RenormThetaNC, SizeOfBlocks and
IndexLeft/Right, SwappingNC, and the number-conserving periodic steps."""
import numpy as np
import pytest

from oracle import observables as obs

# two species of hard-core particles: local states |0>, |a>, |b>, |ab>
CONSERV = np.array([0, 1, 1, 2])


def two_species_bond():
    ca = np.zeros((4, 4))
    cb = np.zeros((4, 4))
    ca[0, 1] = ca[2, 3] = 1.0
    cb[0, 2] = cb[1, 3] = 1.0
    na, nb = ca.T @ ca, cb.T @ cb
    e = np.eye(4)
    h = -(np.kron(ca.T, ca) + np.kron(ca, ca.T)) - 0.6 * (np.kron(cb.T, cb) + np.kron(cb, cb.T))
    h = h + np.kron(na @ nb, e) + np.kron(e, na @ nb) + 0.3 * np.kron(na, nb)
    # species exchange across the bond (complex, number conserving)
    h = h + 0.2j * (np.kron(ca.T @ cb, cb.T @ ca) - np.kron(cb.T @ ca, ca.T @ cb))
    return h


def sector_product_state(L, seed):
    """Sites with numbers 1, 1, 2, 0, ...: superpositions inside each sector."""
    rng = np.random.default_rng(seed)
    c0 = np.zeros((4, L), complex)
    for s in range(L):
        n = (1, 1, 2, 0)[s % 4]
        idx = [j for j in range(4) if CONSERV[j] == n]
        c0[idx, s] = rng.standard_normal(len(idx)) + 1j * rng.standard_normal(len(idx))
    return c0 / np.linalg.norm(c0, axis=0), int(sum((1, 1, 2, 0)[s % 4] for s in range(L)))


@pytest.fixture(scope="module")
def H(pkg):
    return pkg.hamiltonians


@pytest.mark.parametrize("order", [2, 5])
def test_nc_with_internal_states_follows_the_dense_update(oracle, H, order):
    """At exact chi the block-sparse update with Conserv = (0,1,1,2) and the dense
    update give the same state (a U(1)-symmetric gate on a state of definite
    number), and the labels stay consistent with the kept Schmidt vectors."""
    L, d, chi = 4, 4, 16
    c0, N = sector_product_state(L, 2)
    hb = two_species_bond()
    U = H.construct_propagators([hb] * (L - 1), 0.05, order)
    gd, ld = H.product_state(c0, chi)
    gn, ln = H.product_state(c0, chi)
    ll, lr = H.product_state_labels(c0, chi, N, CONSERV)
    for _ in range(6):
        oracle.trotter_step(gd, ld, U, order)
        te = oracle.trotter_step_nc(gn, ln, ll, lr, U, N, 2, order, conserv=CONSERV)
        assert te < 1e-12
    a, b = obs.state_vector(gd, ld), obs.state_vector(gn, ln)
    assert 1.0 - abs(np.vdot(a, b)) < 1e-12
    for link in range(1, L):
        used = ll[link] < 1000
        assert np.all(lr[link][used] == N - ll[link][used])
        assert np.all(ln[link][~used] == 0.0)
        assert abs(np.sum(ln[link] ** 2) - 1.0) < 1e-12


def test_identity_conserv_is_the_plain_update(oracle, H):
    """Conserv(i) = i-1 with maxFilling = d-1 makes every intDegFree branch the
    plain one term for term."""
    L, d, chi, N = 6, 3, 9, 6
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 2.0), 0.05, 2)
    g2 = [g.copy(order="F") for g in gam]
    l2, ll2, lr2 = [x.copy() for x in lam], [x.copy() for x in ll], [x.copy() for x in lr]
    for _ in range(3):
        oracle.trotter_step_nc(gam, lam, ll, lr, U, N, d - 1, 2)
        oracle.trotter_step_nc(g2, l2, ll2, lr2, U, N, d - 1, 2, conserv=np.arange(d))
    for a, b in zip(gam, g2):
        assert np.array_equal(a, b)
    for a, b in zip(lam + ll + lr, l2 + ll2 + lr2):
        assert np.array_equal(a, b)


def test_product_state_labels_take_the_first_component_with_conserv(H):
    """ProductStateLabels: Conserv of the first nonzero component with intDegFree,
    j-1 of the last one without."""
    c0 = np.zeros((4, 2), complex)
    c0[[1, 2], 0] = 1.0 / np.sqrt(2.0)
    c0[3, 1] = 1.0
    ll, lr = H.product_state_labels(c0, 4, 3, CONSERV)
    assert [int(x[0]) for x in ll] == [0, 1, 3] and [int(x[0]) for x in lr] == [3, 2, 0]
    ll, lr = H.product_state_labels(c0, 4, 5, None)
    assert [int(x[0]) for x in ll] == [0, 2, 5]


@pytest.mark.parametrize("L", [4, 5])
@pytest.mark.parametrize("order", [2, 5])
@pytest.mark.parametrize("idf", [False, True])
def test_nc_periodic_steps_follow_the_dense_ones(oracle, H, L, order, idf):
    """TrotterStep2ndOrderPBCNC / 5thOrderPBCNC (with SwappingNC) at exact chi give
    the state of the dense periodic steps, which the exact ring evolution pins."""
    if idf:
        d, chi, mf = 4, 16, 2
        c0, N = sector_product_state(L, 11)
        hb = two_species_bond()
        gam, lam = H.product_state(c0, chi)
        ll, lr = H.product_state_labels(c0, chi, N, CONSERV)
        cons = CONSERV
    else:
        d, N, mf = 3, L, 2
        chi = d ** (L // 2)
        hb = H.bose_hubbard(L, d, 1.0, 2.0)[1]
        gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
        cons = None
    U = H.construct_propagators([hb] * L, 0.05, order, boundary="P")
    gd = [g.copy(order="F") for g in gam]
    ld = [x.copy() for x in lam]
    for _ in range(3):
        te = oracle.trotter_step_pbc_nc(gam, lam, ll, lr, U, N, mf, order, conserv=cons)
        oracle.trotter_step_pbc(gd, ld, U, order)
        assert te < 1e-11
    assert 1.0 - abs(np.vdot(obs.state_vector(gd, ld), obs.state_vector(gam, lam))) < 1e-12
    for link in range(1, L):
        used = ll[link] < 1000
        assert np.all(lr[link][used] == N - ll[link][used])


def test_swapping_nc_is_the_dense_swap(oracle, H):
    """SwappingNC on a number-conserving bond: same Lambda (as a multiset) and
    two-site density as the dense Swapping of the same chain."""
    L, d, chi, N = 6, 3, 9, 6
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, np.linspace(1.0, 3.0, L)), 0.1, 2)
    for _ in range(2):
        oracle.trotter_step_nc(gam, lam, ll, lr, U, N, d - 1, 2)
    a = oracle.swapping_nc(gam[2], gam[3], lam[2], lam[3], lam[4], ll[2], ll[3], lr[3], lr[4], N, d - 1)
    b = oracle.swapping(gam[2], gam[3], lam[2], lam[3], lam[4])
    assert abs(a[5] - b[3]) < 1e-13
    assert np.allclose(np.sort(a[2]), np.sort(b[2]), atol=1e-13)
    ra = obs.two_site_rho(lam[2], a[0], a[2], a[1], lam[4])
    rb = obs.two_site_rho(lam[2], b[0], b[2], b[1], lam[4])
    assert np.allclose(ra, rb, atol=1e-13)
