"""Known answers for the oracle's Swapping and periodic-boundary Trotter step."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def H(pkg):
    return pkg.hamiltonians


def _canonical_chain(H, oracle, L=6, d=2, chi=8, seed=4):
    rng = np.random.default_rng(seed)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    U = H.construct_propagators(H.heisenberg(L, 1.0, 1.0, 0.3), 0.1, 2)
    for _ in range(3):
        oracle.trotter_step(gam, lam, U, 2)
    return gam, lam


def test_swapping_is_the_swap_gate_on_a_normalised_state(oracle, H):
    from oracle import observables as obs
    gam, lam = _canonical_chain(H, oracle)
    d = 2
    swap = np.zeros((d * d, d * d), complex)
    for i in range(d):
        for j in range(d):
            swap[i * d + j, j * d + i] = 1.0
    a = oracle.swapping(gam[2], gam[3], lam[2], lam[3], lam[4])
    b = oracle.two_site_op(gam[2], gam[3], lam[2], lam[3], lam[4], swap)
    assert np.allclose(a[2], b[2], atol=1e-13) and abs(a[3] - b[3]) < 1e-13
    ra = obs.two_site_rho(lam[2], a[0], a[2], a[1], lam[4])
    rb = obs.two_site_rho(lam[2], b[0], b[2], b[1], lam[4])
    assert np.allclose(ra, rb, atol=1e-13)


def test_swap_twice_restores_the_chain(oracle, H):
    from oracle import observables as obs
    gam, lam = _canonical_chain(H, oracle)
    ref = ([g.copy(order="F") for g in gam], [l.copy() for l in lam])
    for _ in range(2):
        g1, g2, l1, te = oracle.swapping(gam[1], gam[2], lam[1], lam[2], lam[3])
        gam[1], gam[2], lam[2] = g1, g2, l1
        assert te < 1e-12
    assert np.allclose(lam[2], ref[1][2], atol=1e-13)
    assert abs(abs(obs.inner_product(ref[0], ref[1], gam, lam)) - 1.0) < 1e-12


def test_pbc_step_on_a_product_gate_ring(oracle, H):
    """Product gates (no entanglement) on a ring: the PBC step applies each local
    factor once, so a product state stays a product state of the expected spinors."""
    L, d, chi = 5, 2, 4
    rng = np.random.default_rng(1)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    gam, lam = H.product_state(c0, chi)
    phase = np.diag(np.exp(1j * np.array([0.3, -0.3])))
    eye = np.eye(d)
    gates = [np.kron(phase, eye) for _ in range(L - 1)] + [np.kron(eye, eye)]
    te = oracle.trotter_step_pbc(gam, lam, gates)
    assert te < 1e-12
    for l in lam:
        assert abs(l[0] - 1.0) < 1e-12 and np.all(np.abs(l[1:]) < 1e-12)


def test_canonical_form_keeps_a_canonical_chain(oracle, H):
    from oracle import observables as obs
    gam, lam = _canonical_chain(H, oracle)
    g1, l1, g2 = oracle.canonical_form(lam[1], gam[1], lam[2], gam[2], lam[3])
    assert np.allclose(l1, lam[2], atol=1e-12)
    r0 = obs.two_site_rho(lam[1], gam[1], lam[2], gam[2], lam[3])
    r1 = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    assert np.allclose(r0, r1, atol=1e-12)


def test_canonical_form_all_makes_a_random_chain_canonical(oracle):
    rng = np.random.default_rng(7)
    L, d, chi = 5, 2, 4
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(L + 1)]
    lam[0] = np.eye(chi)[0]
    lam[L] = np.eye(chi)[0]
    oracle.canonical_form_all(gam, lam)
    for l in lam[1:L]:
        assert abs(np.sum(l ** 2) - 1.0) < 1e-12
    # left-canonical condition on the bulk sites: sum conj(G) l0^2 G = 1 on the kept indices
    for s in range(1, L - 1):
        A = (gam[s] * lam[s][:, None, None]).reshape(chi * d, chi)
        keep = lam[s + 1] > 1e-6
        Mx = A.conj().T @ A
        assert np.allclose(Mx[np.ix_(keep, keep)], np.eye(keep.sum()), atol=1e-8)


def _ring_hamiltonian(L, hb, d):
    """Dense H of a ring: hb on bonds (s, s+1) and on the edge (site 1 left, site L right)."""
    N = d ** L
    Hf = np.zeros((N, N), complex)
    for b in range(L - 1):
        Hf += np.kron(np.kron(np.eye(d ** b), hb), np.eye(d ** (L - b - 2)))
    h4 = hb.reshape(d, d, d, d)
    shape = (d,) * L
    for idx in range(N):
        digs = np.unravel_index(idx, shape)
        for i1 in range(d):
            for iL in range(d):
                v = h4[i1, iL, digs[0], digs[-1]]
                if v != 0:
                    Hf[np.ravel_multi_index((i1,) + digs[1:-1] + (iL,), shape), idx] += v
    return Hf


@pytest.mark.parametrize("L", [5, 6])
@pytest.mark.parametrize("order,dt,bound", [(2, 0.1, 2e-7), (5, 0.1, 2e-11), (5, 0.05, 1e-13)])
def test_pbc_steps_follow_the_exact_ring_evolution(oracle, H, L, order, dt, bound):
    """TrotterStep2ndOrderPBC / 5thOrderPBC with NEWConstructPropagators' periodic
    gates against exp(-iHt) of the ring (exact chi, no truncation): the infidelity
    after t = 0.4 falls like dt^4 (order 2) and dt^8 (Forest-Ruth), which a wrong
    gate index, fraction or sweep would break by orders of magnitude."""
    from oracle import observables as obs
    d, chi = 2, 2 ** (L // 2)
    hb = H.heisenberg(L, 1.0, 1.0, 0.7)[0]
    rng = np.random.default_rng(L)
    c0 = rng.standard_normal((d, L)) + 1j * rng.standard_normal((d, L))
    c0 /= np.linalg.norm(c0, axis=0)
    psi0 = c0[:, 0]
    for s in range(1, L):
        psi0 = np.kron(psi0, c0[:, s])
    steps = int(round(0.4 / dt))
    gam, lam = H.product_state(c0, chi)
    U = H.construct_propagators([hb] * L, dt, order, boundary="P")
    assert len(U) == (L if order == 2 else (3 * L if L % 2 else 2 * L))
    te = sum(oracle.trotter_step_pbc(gam, lam, U, order) for _ in range(steps))
    assert te < 1e-11
    w, v = np.linalg.eigh(_ring_hamiltonian(L, hb, d))
    exact = v @ (np.exp(-1j * w * dt * steps) * (v.conj().T @ psi0))
    assert 1.0 - abs(np.vdot(exact, obs.state_vector(gam, lam))) < bound


def test_fermi_hubbard_two_site_known_answer(H):
    """Two-site Hubbard at half filling: ground energy -sqrt(U^2/4 + 4 J^2) with the
    particle-hole symmetric interaction; the bond term conserves the number."""
    J, U = 1.0, 4.0
    h = H.fermi_hubbard(2, J, U)[0]
    assert np.allclose(h, h.conj().T)
    _, _, one, n, _, _ = H.fermi_ops()
    N = np.kron(n, one) + np.kron(one, n)
    assert np.allclose(h @ N, N @ h)
    sector = np.where(np.isclose(np.diag(N), 2.0))[0]
    e = np.linalg.eigvalsh(h[np.ix_(sector, sector)])
    assert abs(e[0] + np.sqrt(U * U / 4 + 4 * J * J)) < 1e-12
    # one particle: hopping only (the interaction terms cancel), -J and +J twice each
    s1 = np.where(np.isclose(np.diag(N), 1.0))[0]
    assert np.allclose(np.linalg.eigvalsh(h[np.ix_(s1, s1)]), [-J, -J, J, J])
