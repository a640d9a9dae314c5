"""GPU parity of the dense two-site update (TwoSiteOp / TrotterStep) against the oracle.

Comparison rule (gauge-invariant quantities only; raw Gammas are not unique):
* singular values:  |s_gpu - s_ref| <= 1e-12 * s_ref + 1e-13 * s_max   (LAPACK's own
  accuracy is absolute, ~n*eps*s_max, so the relative 1e-12 bar applies down to
  s/s_max ~ 1e-1 and the absolute floor below it)
* Lambdas, truncation error, local observables, bond energies: 1e-11 absolute
* state overlap |<psi_ref|psi_gpu>|: 1 - 1e-11
"""
import os

import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
SIG_REL, SIG_ABS = 1e-12, 1e-13


def sigma_ok(s_gpu, s_ref):
    """The bidiagonal route reports only the chi values it keeps, the Jacobi routes
    all d*chi: compare the leading len(s_gpu) values."""
    s_gpu, s_ref = np.asarray(s_gpu), np.asarray(s_ref)
    assert 1 <= len(s_gpu) <= len(s_ref)
    s_ref = s_ref[:len(s_gpu)]
    tol = SIG_REL * s_ref + SIG_ABS * max(s_ref[0], 1e-300)
    return np.all(np.abs(s_gpu - s_ref) <= tol), np.max(np.abs(s_gpu - s_ref) - tol)


def random_bond(chi, d, seed, L=4):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(L + 1)]
    lam = [l / np.linalg.norm(l) for l in lam]
    return gam, lam


def random_unitary(n, rng):
    z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("svd_mode", [0, 2, 3, 4])
@pytest.mark.parametrize("chi,d", [(1, 2), (8, 2), (16, 3), (12, 5), (32, 4)])
def test_single_update_matches_oracle(pkg, oracle, chi, d, svd_mode):
    """Every SVD route: default per-bond choice (0), plain Jacobi (2), bidiagonalisation
    with bisection and inverse iteration (3), pivoted QR + Jacobi on R^H (4)."""
    gam, lam = random_bond(chi, d, 100 + chi + d)
    U = random_unitary(d * d, np.random.default_rng(chi * d))
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    ok, worst = sigma_ok(s, rs)
    assert ok, worst
    assert np.allclose(l1, rl1, atol=1e-11)
    assert abs(te - rte) < 1e-11
    # gauge-invariant: the updated two-site wavefunction (rho2) and its energy
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-11)


def test_real_gate_and_edges(pkg, oracle):
    chi, d, L = 6, 3, 5
    gam, lam = random_bond(chi, d, 5, L)
    R = np.random.default_rng(9).standard_normal((d * d, d * d))
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        for link in (1, L - 1):
            te = c.two_site_op(link, R)
            rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[link - 1], gam[link], lam[link - 1], lam[link],
                                                        lam[link + 1], R)
            gam[link - 1], gam[link], lam[link] = rg1, rg2, rl1
            ok, worst = sigma_ok(c.singular_values(link), rs)
            assert ok, worst
            assert abs(te - rte) < 1e-11
            assert np.allclose(c.get_lambda(link + 1), rl1, atol=1e-11)


@pytest.mark.parametrize("svd_mode", [0, 3])
def test_rank_deficient_product_state(pkg, oracle, svd_mode):
    """Product state, product gate: one singular value 1, all others exactly 0."""
    H = pkg.hamiltonians
    rng = np.random.default_rng(2)
    d, chi, L = 3, 8, 4
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    U = np.kron(random_unitary(d, rng), random_unitary(d, rng))
    with pkg.Chain(L, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        assert abs(s[0] - 1) < 1e-14 and np.all(s[1:] < 1e-14)
        assert te < 1e-14
        assert np.allclose(c.get_lambda(3), np.eye(chi)[0], atol=1e-14)


@pytest.mark.parametrize("svd_mode", [0, 3])
@pytest.mark.parametrize("chi,d,fracs", [(9, 3, (0.5, 0.3, 0.7)), (40, 2, (0.5, 0.3, 0.7)),
                                         (40, 2, (0.2, 0.3, 0.6))])
def test_exact_zero_lambdas_anywhere(pkg, oracle, chi, d, fracs, svd_mode):
    """Rows/columns of exactly-zero Lambdas are dropped from the SVD; zeros at
    interior positions and differing counts on the three links must give the
    reference's Lambdas and Gammas' physics.  The compacted Theta is wide in the
    first two cases (the bidiagonal mode works on Theta^H) and tall in the last."""
    gam, lam = random_bond(chi, d, 31 + chi)
    rng = np.random.default_rng(chi)
    for l, frac in zip(lam[1:4], fracs):
        l[rng.random(chi) < frac] = 0.0
        l[0] = max(l[0], 0.1)
        l /= np.linalg.norm(l)
    U = random_unitary(d * d, rng)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    ok, worst = sigma_ok(s, rs)
    assert ok, worst
    assert np.allclose(l1, rl1, atol=1e-11)
    assert abs(te - rte) < 1e-11
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-11)
    # dropped rows of Gamma1 / columns of Gamma2 are zero, as FormGamma1/2's guard makes them
    assert np.all(g1[lam[1] == 0] == 0)
    assert np.all(g2[:, :, lam[3] == 0] == 0)


def test_golden_reference_propagators(pkg):
    """The reference's own d=4 gate fixtures (Extensible_Wrapper/Propagator_*.nml),
    against the oracle outputs recorded in tests/golden/propagators_d4.npz."""
    z = np.load(os.path.join(HERE, "golden", "propagators_d4.npz"))
    chi, d = int(z["chi"]), int(z["d"])
    for nm in z["names"]:
        key = str(nm).replace(".", "p")
        with pkg.Chain(3, d, chi) as c:
            c.set_state([z["gamma1"], z["gamma2"], z["gamma2"]], [z["lam0"], z["lam1"], z["lam2"], z["lam2"]])
            te = c.two_site_op(1, z["gate_" + key])
            ok, worst = sigma_ok(c.singular_values(1), z["sigma_" + key])
            assert ok, (key, worst)
            assert np.allclose(c.get_lambda(2), z["lambda_" + key], atol=1e-11)
            assert abs(te - float(z["truncerr_" + key])) < 1e-11


@pytest.mark.parametrize("svd_mode", [0, 3, 5])
@pytest.mark.parametrize("order", [2, 5])
def test_trotter_steps_match_oracle(pkg, oracle, order, svd_mode):
    """Full sweeps (batched same-parity bonds on the GPU vs sequential bonds in the
    oracle) on a Heisenberg chain; compares every Lambda, <Sz>, bond energies and
    the overlap of the two states."""
    H = pkg.hamiltonians
    L, d, chi = 8, 2, 8
    rng = np.random.default_rng(11)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    Hb = H.heisenberg(L, 1.0, 1.0, 0.5)
    U = H.construct_propagators(Hb, 0.1, order)
    with pkg.Chain(L, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        for _ in range(3):
            te = c.trotter_step(U, order)
            rte = oracle.trotter_step(gam, lam, U, order)
            assert abs(te - rte) < 1e-10
        g_gpu, l_gpu = c.get_state()
    for a, b in zip(l_gpu, lam):
        assert np.allclose(a, b, atol=1e-10)
    sz = np.diag([0.5, -0.5])
    assert np.allclose(obs.one_site_expval(g_gpu, l_gpu, sz), obs.one_site_expval(gam, lam, sz), atol=1e-10)
    assert np.allclose(obs.bond_energy(g_gpu, l_gpu, Hb), obs.bond_energy(gam, lam, Hb), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g_gpu, l_gpu)) - 1.0) < 1e-10


@pytest.mark.parametrize("svd_mode,drop", [(0, None), (4, None), (0, "left"), (0, "right"), (5, None), (5, "left")])
def test_bose_hubbard_full_size_single_bond(pkg, oracle, svd_mode, drop):
    """Bond of the d=5, chi=128 Bose-Hubbard workload (n = 640) against LAPACK, plus
    size-independent properties: sum lambda^2 = 1, truncerr = 1 - sum of kept S^2,
    and left/right canonical conditions of the new Gammas.  The default route takes
    the bidiagonal path here (640 columns); mode 4 forces QR + Jacobi; mode 5 runs
    the bidiagonalisation's heavy passes in double-float.  Three exact
    zeros in the left (right) Lambda make the compacted Theta 625 x 640 (640 x 625):
    the wide one is bidiagonalised as Theta^H."""
    chi, d = 128, 5
    gam, lam = random_bond(chi, d, 77)
    for l in lam:
        l[:] = np.exp(-np.arange(chi) / 16.0)
        l /= np.linalg.norm(l)
    if drop is not None:
        l = lam[1] if drop == "left" else lam[3]
        l[[5, 40, 90]] = 0.0
        l /= np.linalg.norm(l)
    Hb = pkg.hamiltonians.bose_hubbard(4, d, 1.0, 2.0)
    U = pkg.hamiltonians.matrix_exponential(Hb[1], 0.005)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
        assert c.stats()["bidiag_updates"] == (1 if svd_mode in (0, 5) else 0)
    rg1, rg2, rl1, rte, rs = oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U)
    ok, worst = sigma_ok(s, rs)
    assert ok, worst
    assert len(s) >= chi
    assert np.allclose(l1, rl1, atol=1e-11)
    assert abs(te - rte) < 1e-11
    assert abs(np.sum(l1 ** 2) - 1) < 1e-12
    assert abs(te - abs(1 - np.sum(s[:chi] ** 2))) < 1e-12
    # left canonical: sum_{a,i} conj(G1(a,i,b)) l0(a)^2 G1(a,i,b') = delta  (kept b)
    A = (g1 * lam[1][:, None, None]).reshape(chi * d, chi)
    kept = l1 > 1e-8
    M = A.conj().T @ A
    assert np.allclose(M[np.ix_(kept, kept)], np.eye(kept.sum()), atol=1e-9)
    B = (g2 * lam[3][None, None, :]).reshape(chi, d * chi)
    N = B @ B.conj().T
    assert np.allclose(N[np.ix_(kept, kept)], np.eye(kept.sum()), atol=1e-9)


def test_error_paths(pkg):
    with pkg.Chain(4, 2, 4) as c:
        with pytest.raises(pkg.TebdError) as e:
            c.two_site_op(4, np.eye(4, dtype=complex))  # link must be <= L-1
        assert e.value.code == 1
        with pytest.raises(pkg.TebdError) as e:
            c.apply_bonds([1, 2], [np.eye(4), np.eye(4)])  # overlapping bonds
        assert e.value.code == 1
        with pytest.raises(pkg.TebdError) as e:
            pkg.TwoSiteOpNC(1, np.eye(4, dtype=complex), c)
        assert e.value.code == 6
        with pytest.raises(pkg.TebdError):
            c.trotter_step([np.eye(4)] * 2, 2)  # too few gates
        assert c.kernel_launches() == 0
