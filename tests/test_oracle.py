"""CPU tests: the oracle against analytic known answers and the reference's fixtures.

The reference ships no tests or golden vectors and cannot be compiled here (no
Fortran compiler), so these known answers are what pins the oracle
(tests/golden/make_golden.py records the oracle's outputs on the reference's
own propagator fixtures so later changes cannot drift silently).
"""
import os

import numpy as np
import pytest

from oracle import observables as obs

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def H(pkg):
    return pkg.hamiltonians


def _random_unitary(n, rng):
    z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def test_product_gate_keeps_rank_one(oracle, H):
    rng = np.random.default_rng(1)
    d, chi = 3, 4
    c = rng.standard_normal((d, 2)) + 1j * rng.standard_normal((d, 2))
    c /= np.linalg.norm(c, axis=0)
    gam, lam = H.product_state(c, chi)
    U = np.kron(_random_unitary(d, rng), _random_unitary(d, rng))
    g1, g2, l1, te, s = oracle.two_site_op(gam[0], gam[1], lam[0], lam[1], lam[2], U)
    assert abs(s[0] - 1.0) < 1e-14 and np.all(s[1:] < 1e-14)
    assert np.allclose(l1, np.eye(chi)[0], atol=1e-14)
    assert te < 1e-14


def test_ghz_schmidt_values(oracle, H):
    """CNOT chain on |+>|0>...|0> gives the GHZ state: Lambda = (1/sqrt2, 1/sqrt2)
    on every link (the analytic Lambda of SpecialState, local_operations_module.f90:2097-2153)."""
    L, d, chi = 6, 2, 2
    c = np.zeros((2, L), complex)
    c[0, :] = 1.0
    c[:, 0] = [1 / np.sqrt(2), 1 / np.sqrt(2)]
    gam, lam = H.product_state(c, chi)
    cnot = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], complex)
    for link in range(1, L):
        g1, g2, l1, te, _ = oracle.two_site_op(gam[link - 1], gam[link], lam[link - 1], lam[link], lam[link + 1], cnot)
        gam[link - 1], gam[link], lam[link] = g1, g2, l1
    for link in range(2, L + 1):
        assert np.allclose(lam[link - 1], [2 ** -0.5, 2 ** -0.5], atol=1e-14)
    # the state is (|00..0> + |11..1>)/sqrt2
    sz = np.diag([0.5, -0.5])
    assert np.allclose(obs.one_site_expval(gam, lam, sz), 0.0, atol=1e-14)


def _xx_exact_sz(L, t):
    """Free-fermion Sz profile of the XX chain from the domain wall |up..up dn..dn>."""
    h = np.zeros((L, L))
    for i in range(L - 1):
        h[i, i + 1] = h[i + 1, i] = 0.5  # J/2 hopping, J = 1
    w, v = np.linalg.eigh(h)
    U = (v * np.exp(-1j * w * t)) @ v.T
    n0 = np.array([1.0] * (L // 2) + [0.0] * (L - L // 2))
    return (np.abs(U) ** 2) @ n0 - 0.5


@pytest.mark.parametrize("order,dt,tol", [(2, 0.02, 2e-4), (5, 0.05, 2e-5)])
def test_xx_domain_wall_free_fermions(oracle, H, order, dt, tol):
    """Known answer: XXDynamics' domain-wall quench (Heisenberg_Wrapper/XXDynamics.f90:113-120)
    against the exact free-fermion solution; 2nd order and Forest-Ruth sweeps."""
    L, chi, T = 10, 16, 1.0
    c = np.zeros((2, L), complex)
    c[0, : L // 2] = 1.0
    c[1, L // 2:] = 1.0
    gam, lam = H.product_state(c, chi)
    Hb = H.heisenberg(L, 1.0, 1.0, 0.0)
    U = H.construct_propagators(Hb, dt, order)
    steps = int(round(T / dt))
    for _ in range(steps):
        oracle.trotter_step(gam, lam, U, order)
    sz = obs.one_site_expval(gam, lam, np.diag([0.5, -0.5]))
    err = np.max(np.abs(sz - _xx_exact_sz(L, steps * dt)))
    assert err < tol, err
    assert all(abs(np.sum(l ** 2) - 1.0) < 1e-12 for l in lam[1:-1])


def test_identity_gate_is_state_preserving(oracle, H):
    """The identity-gate sweep of CanonicalFormAllNC (propagation_module.f90:1952-1983)
    must leave a canonical state unchanged."""
    rng = np.random.default_rng(3)
    L, d, chi = 6, 2, 8
    c = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c /= np.linalg.norm(c, axis=0)
    gam, lam = H.product_state(c, chi)
    Hb = H.heisenberg(L, 1.0, 0.7, 0.4)
    U = H.construct_propagators(Hb, 0.3, 2)
    for _ in range(4):
        oracle.trotter_step(gam, lam, U, 2)
    ref = ([g.copy(order="F") for g in gam], [l.copy() for l in lam])
    eye = np.eye(d * d, dtype=complex)
    for link in list(range(1, L)) + list(range(L - 1, 0, -1)):
        g1, g2, l1, te, _ = oracle.two_site_op(gam[link - 1], gam[link], lam[link - 1], lam[link], lam[link + 1], eye)
        gam[link - 1], gam[link], lam[link] = g1, g2, l1
        assert te < 1e-12
    for a, b in zip(lam, ref[1]):
        assert np.allclose(a, b, atol=1e-12)
    ov = obs.inner_product(ref[0], ref[1], gam, lam)
    assert abs(abs(ov) - 1.0) < 1e-12


def test_real_gate_equals_complex_gate(oracle, H):
    rng = np.random.default_rng(4)
    chi, d = 5, 3
    g = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi))) for _ in range(2)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(3)]
    R = rng.standard_normal((d * d, d * d))
    a = oracle.two_site_op(g[0], g[1], lam[0], lam[1], lam[2], R)
    b = oracle.two_site_op(g[0], g[1], lam[0], lam[1], lam[2], R.astype(complex))
    assert np.allclose(a[4], b[4], rtol=1e-13, atol=1e-15)
    assert np.allclose(a[2], b[2], rtol=1e-13, atol=1e-15)


def test_nc_update_matches_dense_update(oracle, H):
    """On a number-conserving state with a number-conserving gate, TwoSiteOpNC and
    TwoSiteOp are the same update: equal Schmidt spectra, densities and energies."""
    L, d, chi, N = 6, 3, 9, 6
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    gd = [g.copy(order="F") for g in gam]
    ld = [l.copy() for l in lam]
    Hb = H.bose_hubbard(L, d, 1.0, 2.0)
    U = H.construct_propagators(Hb, 0.05, 2)
    for _ in range(5):
        te_nc = oracle.trotter_step_nc(gam, lam, ll, lr, U, N, d - 1, 2)
        te_d = oracle.trotter_step(gd, ld, U, 2)
    for a, b in zip(lam, ld):
        assert np.allclose(np.sort(a), np.sort(b), atol=1e-9)
    nop = np.diag(np.arange(d, dtype=float))
    n_nc = obs.one_site_expval(gam, lam, nop)
    n_d = obs.one_site_expval(gd, ld, nop)
    assert np.allclose(n_nc, n_d, atol=1e-9)
    assert abs(n_nc.sum() - N) < 1e-9
    assert np.allclose(obs.bond_energy(gam, lam, Hb), obs.bond_energy(gd, ld, Hb), atol=1e-9)
    # labels: every used Schmidt index carries the particle number to its left
    for link in range(1, L + 2):
        used = lam[link - 1] > 0
        assert np.all(ll[link - 1][used] < 1000)
        assert np.all(ll[link - 1][used] + lr[link - 1][used] == N)


def test_golden_fixtures_reproduce(oracle):
    """The oracle still reproduces its recorded outputs on the reference's own
    d=4 propagator fixtures (Extensible_Wrapper/Propagator_*.nml)."""
    z = np.load(os.path.join(HERE, "golden", "propagators_d4.npz"))
    for nm in z["names"]:
        key = str(nm).replace(".", "p")
        _, _, l1, te, s = oracle.two_site_op(z["gamma1"], z["gamma2"], z["lam0"], z["lam1"], z["lam2"], z["gate_" + key])
        assert np.allclose(s, z["sigma_" + key], rtol=1e-12, atol=1e-15)
        assert np.allclose(l1, z["lambda_" + key], rtol=1e-12, atol=1e-15)
        assert abs(te - float(z["truncerr_" + key])) < 1e-13
    # the gates are the fixtures as the reference reads them (column-major fill)
    assert z["gate_0p01_bulk"].shape == (16, 16)
    assert abs(z["gate_0p01_bulk"][0, 0].real - 0.9999500493370335752) < 1e-16


def test_forest_ruth_theta(H):
    th = H.forest_ruth_theta()
    assert abs(th - 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))) < 1e-7  # single-precision exponent literal
    assert th != 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))
