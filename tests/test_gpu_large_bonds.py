"""Single bond updates at the largest bond sizes of the configurations, against
LAPACK through the oracle:

* d = 4, chi = 256 (Theta 1024 x 1024), the Fermi-Hubbard shape;
* d = 3, chi = 1024 (Theta 3072 x 3072), the spin-1 shape at its maximum chi.

Inputs follow the single-update micro-benchmark: complex Gaussian Gammas,
geometric Lambdas lambda_k ~ exp(-k / w), a Haar-random d^2 x d^2 unitary gate.
Both run the bidiagonal route, in plain FP64 and in the double-float form.  The
3072 case is checked through size-independent properties (the oracle's full
update takes minutes there): singular values against a values-only LAPACK SVD of
the same Theta, truncation error, Eckart-Young optimality of the kept rank and
the canonical conditions."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu

SIG_REL, SIG_ABS = 1e-12, 1e-13
_REF = {}


def haar_unitary(n, rng):
    z = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def bond_case(chi, d, width, seed=1234):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(4)]
    lam = []
    for _ in range(5):
        l = np.exp(-np.arange(chi) / width)
        lam.append(l / np.linalg.norm(l))
    return gam, lam, haar_unitary(d * d, rng)


def reference(oracle, chi, d, width):
    key = (chi, d, width)
    if key not in _REF:
        gam, lam, U = bond_case(chi, d, width)
        _REF[key] = (gam, lam, U, oracle.two_site_op(gam[1], gam[2], lam[1], lam[2], lam[3], U))
    return _REF[key]


@pytest.mark.parametrize("svd_mode", [0, 5])
def test_fermi_hubbard_shape_bond_matches_lapack(pkg, oracle, svd_mode):
    """d = 4, chi = 256 against the oracle's update (ZGESVD 'A','A')."""
    chi, d, width = 256, 4, 32.0
    gam, lam, U, (rg1, rg2, rl1, rte, rs) = reference(oracle, chi, d, width)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = c.singular_values(2)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
        assert c.stats()["bidiag_updates"] == 1
    s = np.asarray(s)
    ref = np.asarray(rs)[: len(s)]
    assert len(s) >= chi
    tol = SIG_REL * ref + SIG_ABS * ref[0]
    assert np.all(np.abs(s - ref) <= tol), float(np.max(np.abs(s - ref) - tol))
    assert np.allclose(l1, rl1, atol=1e-11)
    assert abs(te - rte) < 1e-11
    assert abs(np.sum(l1 ** 2) - 1.0) < 1e-12
    # canonical conditions of the new Gammas on the kept Schmidt indices
    kept = l1 > 1e-8
    A = (g1 * lam[1][:, None, None]).reshape(chi * d, chi)
    assert np.allclose((A.conj().T @ A)[np.ix_(kept, kept)], np.eye(kept.sum()), atol=1e-9)
    B = (g2 * lam[3][None, None, :]).reshape(chi, d * chi)
    assert np.allclose((B @ B.conj().T)[np.ix_(kept, kept)], np.eye(kept.sum()), atol=1e-9)
    # the bond's two-site density matrix (gauge invariant)
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-11)


def theta_matrix(gam, lam, U, d, chi):
    """Normalised gate-applied Theta of bond 2 as a (d chi) x (d chi) matrix."""
    th = np.einsum("a,aig,g,gjb,b->aijb", lam[1], gam[1], lam[2], gam[2], lam[3], optimize=True)
    U4 = U.reshape(d, d, d, d)  # (k, l, i, j): row (k, l), column (i, j), right index fastest
    th = np.einsum("klij,aijb->aklb", U4, th, optimize=True)
    M = th.transpose(1, 0, 2, 3).reshape(d * chi, d * chi)  # rows (i, alpha), columns (j, beta)
    return M / np.linalg.norm(M)


@pytest.mark.parametrize("svd_mode", [0, 5])
def test_spin1_max_chi_bond_properties(pkg, svd_mode):
    """d = 3, chi = 1024 (Theta 3072 x 3072)."""
    chi, d, width = 1024, 3, 64.0
    gam, lam, U = bond_case(chi, d, width)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        te = c.two_site_op(2, U)
        s = np.asarray(c.singular_values(2))
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
        assert c.stats()["bidiag_updates"] == 1
    M = theta_matrix(gam, lam, U, d, chi)
    ref = np.linalg.svd(M, compute_uv=False)
    assert len(s) >= chi
    tol = SIG_REL * ref[: len(s)] + SIG_ABS * ref[0]
    assert np.all(np.abs(s - ref[: len(s)]) <= tol), float(np.max(np.abs(s - ref[: len(s)]) - tol))
    kept_w = np.sum(ref[:chi] ** 2)
    assert abs(te - abs(1.0 - kept_w)) < 1e-12
    assert np.allclose(l1, ref[:chi] / np.sqrt(kept_w), atol=1e-11)
    # Eckart-Young: the update's rank-chi reconstruction is the optimal one
    R = np.einsum("a,aig,g,gjb,b->iajb", lam[1], g1, l1, g2, lam[3], optimize=True).reshape(d * chi, d * chi)
    R *= np.sqrt(kept_w)
    assert abs(np.linalg.norm(M - R) ** 2 - np.sum(ref[chi:] ** 2)) < 1e-11
    kept = l1 > 1e-8
    A = (g1 * lam[1][:, None, None]).reshape(chi * d, chi)
    assert np.allclose((A.conj().T @ A)[np.ix_(kept, kept)], np.eye(kept.sum()), atol=1e-9)
    B = (g2 * lam[3][None, None, :]).reshape(chi, d * chi)
    assert np.allclose((B @ B.conj().T)[np.ix_(kept, kept)], np.eye(kept.sum()), atol=1e-9)
