"""GPU observables (observables_module.f90) against the oracle's restatements.

The observables are sums of products of the state's numbers, with no SVD, so the
bar is rounding: 1e-12 relative to the magnitude of the result (sums run in a
different order from the reference's loops).
"""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu
TOL = 1e-12


def open_chain(L, d, chi, seed, zero_frac=0.0):
    """Random Gammas, decaying interior Lambdas (optionally with exact zeros), edge
    Lambdas e_1 as the reference's open chains have them."""
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           / np.sqrt(chi * d) for _ in range(L)]
    lam = []
    for link in range(L + 1):
        if link in (0, L):
            l = np.zeros(chi)
            l[0] = 1.0
        else:
            l = np.sort(rng.random(chi))[::-1] * np.exp(-np.arange(chi) / 4.0)
            if zero_frac:
                l[rng.random(chi) < zero_frac] = 0.0
                l[0] = max(l[0], 0.1)
            l /= np.linalg.norm(l)
        lam.append(l)
    return gam, lam


def herm(n, rng):
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return a + a.conj().T


def close(a, b, tol=TOL):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(1.0, float(np.max(np.abs(b))))
    return float(np.max(np.abs(a - b))) <= tol * scale


@pytest.mark.parametrize("L,d,chi,zf", [(6, 3, 8, 0.0), (5, 2, 16, 0.3), (4, 5, 40, 0.2)])
def test_one_and_two_site_observables(pkg, L, d, chi, zf):
    gam, lam = open_chain(L, d, chi, 7 + chi, zf)
    rng = np.random.default_rng(chi)
    opc = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    opr = rng.standard_normal((d, d))
    Hs = [herm(d * d, rng) for _ in range(L - 1)]
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        rho1 = c.single_site_rho()
        ec = c.one_site_expval(opc)
        er = c.one_site_expval(opr)
        rho2 = [c.two_site_rho(l) for l in range(1, L)]
        en = c.local_energy(Hs)
        tot = c.total_energy(Hs)
        ent = c.chain_entropy()
        # the chain is unchanged by measuring it
        g2, l2 = c.get_state()
    for s in range(L):
        assert close(rho1[s], obs.single_site_rho(lam[s], gam[s], lam[s + 1])), s
    ref_c = np.array([np.einsum("ij,ji->", opc, obs.single_site_rho(lam[s], gam[s], lam[s + 1]))
                      for s in range(L)])
    assert close(ec, ref_c)
    assert close(er, obs.one_site_expval(gam, lam, opr))
    for l in range(1, L):
        assert close(rho2[l - 1], obs.two_site_rho(lam[l - 1], gam[l - 1], lam[l], gam[l], lam[l + 1])), l
    ref_en = obs.bond_energy(gam, lam, Hs)
    assert close(en, ref_en)
    assert abs(tot - ref_en.sum()) <= TOL * max(1.0, np.abs(ref_en).sum())
    assert close(ent, obs.chain_entropy(lam, d))
    for a, b in zip(g2, gam):
        assert np.array_equal(a, b)


def test_inner_product(pkg):
    L, d, chi = 7, 3, 12
    ga, la = open_chain(L, d, chi, 1)
    gb, lb = open_chain(L, d, chi, 2, 0.25)
    with pkg.Chain(L, d, chi) as a, pkg.Chain(L, d, chi) as b:
        a.set_state(ga, la)
        b.set_state(gb, lb)
        ab, aa, ba = a.inner_product(b), a.inner_product(a), pkg.InnerProduct(b, a)
    r_ab = obs.inner_product(ga, la, gb, lb)
    assert abs(ab - r_ab) <= TOL * max(1.0, abs(r_ab))
    assert abs(aa - obs.inner_product(ga, la, ga, la)) <= TOL * max(1.0, abs(aa))
    assert abs(ba - np.conj(r_ab)) <= TOL * max(1.0, abs(r_ab))


def test_observables_along_bose_hubbard_evolution(pkg):
    """Bose-Hubbard (d=5) from the perturbed Mott state: <n_i>, bond energies and the
    norm after a few Trotter steps; particle number and energy conserved."""
    H = pkg.hamiltonians
    L, d, chi = 12, 5, 24
    carray = np.zeros((d, L), complex)
    carray[1, :] = 1.0
    gam, lam = H.perturbed_product_state(carray, chi, 1e-3, 1)
    Hb = H.bose_hubbard(L, d, 1.0, 2.0, 0.0)
    U = H.construct_propagators(Hb, 0.01, 2)
    num = np.diag(np.arange(d, dtype=float))
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        e0 = c.total_energy(Hb)
        n0 = c.one_site_expval(num)
        for _ in range(5):
            c.trotter_step(U, 2)
        n_gpu = c.one_site_expval(num)
        en = c.local_energy(Hb)
        e1 = c.total_energy(Hb)
        nrm = c.inner_product(c)
        g, l = c.get_state()
    assert close(n_gpu, obs.one_site_expval(g, l, num))
    assert close(en, obs.bond_energy(g, l, Hb))
    assert abs(nrm - 1.0) < 1e-10
    assert abs(np.sum(n_gpu) - np.sum(n0)) < 1e-10  # the gates conserve the particle number
    assert abs(e1 - e0) < 1e-5                       # Trotter drift (oracle: 2.0e-6 after 5 steps)


def test_observables_in_number_conserving_mode(pkg):
    """The same entry points on an NC handle (labels do not enter the formulas)."""
    H = pkg.hamiltonians
    L, d, chi, N = 8, 4, 16, 8
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    Hb = H.bose_hubbard(L, d, 1.0, 1.5, 0.0)
    U = H.construct_propagators(Hb, 0.02, 2)
    num = np.diag(np.arange(d, dtype=float))
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        for _ in range(3):
            c.trotter_step(U, 2)
        n_gpu = c.one_site_expval(num)
        en = c.local_energy(Hb)
        st = c.get_state()
    g, l = st[0], st[1]
    assert close(n_gpu, obs.one_site_expval(g, l, num))
    assert close(en, obs.bond_energy(g, l, Hb))
    assert abs(np.sum(n_gpu) - N) < 1e-9


def test_observable_errors(pkg):
    with pkg.Chain(4, 2, 4) as a, pkg.Chain(4, 2, 8) as b:
        with pytest.raises(pkg.TebdError) as e:
            a.inner_product(b)
        assert e.value.code == 1
        with pytest.raises(pkg.TebdError) as e:
            a.two_site_rho(4)
        assert e.value.code == 1
        with pytest.raises(pkg.TebdError) as e:
            a.local_energy([np.eye(4)] * 2)  # needs L-1 = 3 bond operators
        assert e.value.code == 1
