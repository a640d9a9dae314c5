"""The number-conserving Theta on the tensor cores (tebd_set_theta_form(107) on an
NC handle): each charge block's class sums as one grouped digit-plane product
written into the block, then the gate applied in place.

Against the oracle (FormThetaNC's per-entry class sums in FP64): the same bars as
the FP64 path -- truncation error within 1e-10 to 1e-11, Lambdas within 1e-10 to
1e-11, labels exact (or as (lambda, label) multisets where blocks are degenerate),
<n_i>, bond energies and the overlap within 1e-10 -- for single bonds with
random (not block-sparse) Gammas, Trotter steps in 2nd and 5th order, intDegFree,
SwappingNC, and a d=5, chi=64 chain compared with the plain FP64 route.
"""
import numpy as np
import pytest

from oracle import observables as obs

from test_gpu_nc import _nc_bond_with_large_blocks, nc_setup, state_close
from test_gpu_nc_idf import CONSERV, _nc_evolved, sector_state, two_species_bond

pytestmark = pytest.mark.gpu


def _tc_ran(c):
    st = c.stats()
    return st["tc_launches"] > 0 and st["tc_mma_flops"] > 0


@pytest.mark.parametrize("svd_mode", [0, 5])
def test_tc_theta_large_blocks_match_oracle(pkg, oracle, svd_mode):
    """Random Gammas with entries outside the allowed blocks: only the class
    betas may enter each block's sum."""
    chi, d, N = 96, 3, 20
    gam, lam, ll, lr = _nc_bond_with_large_blocks(chi, d, N)
    Hb = pkg.hamiltonians.bose_hubbard(4, d, 1.0, 2.0)
    U = pkg.hamiltonians.matrix_exponential(Hb[1], 0.3)
    with pkg.Chain(4, d, chi, mode=pkg.MODE_NC, tot_num=N, svd_mode=svd_mode) as c:
        c.set_theta_form(107)
        c.set_profiling(True)
        c.set_state(gam, lam, ll, lr)
        c.reset_stats()
        te = c.two_site_op(2, U)
        assert _tc_ran(c)
        g1, g2, l1 = c.get_gamma(2), c.get_gamma(3), c.get_lambda(3)
        la, _ = c.get_labels(3)
    r = oracle.two_site_op_nc(gam[1], gam[2], lam[1], lam[2], lam[3], U, ll[1], ll[2], lr[2], lr[3], N, d - 1)
    rg1, rg2, rl1, rll1, _, rte, _ = r
    assert abs(te - rte) < 1e-11
    assert np.allclose(np.sort(l1), np.sort(rl1), atol=1e-11)
    assert sorted(zip(np.round(l1, 8), la)) == sorted(zip(np.round(rl1, 8), rll1))
    rho = obs.two_site_rho(lam[1], g1, l1, g2, lam[3])
    rrho = obs.two_site_rho(lam[1], rg1, rl1, rg2, lam[3])
    assert np.allclose(rho, rrho, atol=1e-11)


@pytest.mark.parametrize("L,d,chi,N", [(6, 3, 9, 6), (8, 4, 16, 8)])
def test_tc_theta_single_updates_match_oracle(pkg, oracle, L, d, chi, N):
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 3, 0.1)
    for _ in range(3):
        oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, 2)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_theta_form(107)
        c.set_state(gam, lam, ll, lr)
        for link in (1, L // 2, L - 1):
            te = c.two_site_op(link, Udt[link - 1])
            r = oracle.two_site_op_nc(gam[link - 1], gam[link], lam[link - 1], lam[link], lam[link + 1],
                                      Udt[link - 1], ll[link - 1], ll[link], lr[link], lr[link + 1], N, d - 1)
            gam[link - 1], gam[link], lam[link], ll[link], lr[link] = r[0], r[1], r[2], r[3], r[4]
            assert abs(te - r[5]) < 1e-11
            s = c.singular_values(link)
            assert np.allclose(np.sort(s)[::-1], np.sort(r[6])[::-1], rtol=1e-10, atol=1e-13)
        state_close(pkg, c.get_state(), (gam, lam, ll, lr), Hb, d, N)


@pytest.mark.parametrize("order", [2, 5])
def test_tc_theta_trotter_steps_match_oracle(pkg, oracle, order):
    L, d, chi, N = 8, 3, 12, 8
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 7, 0.05, order)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_theta_form(107)
        c.set_state(gam, lam, ll, lr)
        for _ in range(4):
            te = c.trotter_step(Udt, order)
            rte = oracle.trotter_step_nc(gam, lam, ll, lr, Udt, N, d - 1, order)
            assert abs(te - rte) < 1e-10
        state_close(pkg, c.get_state(), (gam, lam, ll, lr), Hb, d, N)


def test_tc_theta_intdegfree_matches_oracle(pkg, oracle):
    H = pkg.hamiltonians
    L, d, chi, order = 6, 4, 16, 2
    gam, lam, ll, lr, N = sector_state(H, L, chi, 38)
    hb = [two_species_bond(U=1.0 + 0.1 * s) for s in range(L - 1)]
    U = H.construct_propagators(hb, 0.05, order)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N, max_filling=2, conserv=CONSERV) as c:
        c.set_theta_form(107)
        c.set_state(gam, lam, ll, lr)
        te = [c.trotter_step(U, order) for _ in range(3)]
        g1, l1, ll1, lr1 = c.get_state()
    rte = [oracle.trotter_step_nc(gam, lam, ll, lr, U, N, 2, order, conserv=CONSERV) for _ in range(3)]
    assert np.allclose(te, rte, atol=1e-10)
    for link, (a, b, la, lb) in enumerate(zip(l1, lam, ll1, ll), start=1):
        assert np.allclose(np.sort(a), np.sort(b), atol=1e-10), link
        assert sorted(zip(np.round(a, 8), la)) == sorted(zip(np.round(b, 8), lb)), link
    nop = np.diag(CONSERV.astype(float))
    assert np.allclose(obs.one_site_expval(g1, l1, nop), obs.one_site_expval(gam, lam, nop), atol=1e-10)
    assert np.allclose(obs.bond_energy(g1, l1, hb), obs.bond_energy(gam, lam, hb), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g1, l1)) - 1.0) < 1e-10


@pytest.mark.parametrize("idf", [False, True])
def test_tc_theta_swapping_matches_oracle(pkg, oracle, idf):
    L = 6
    d, chi = (4, 12) if idf else (3, 9)
    cons = CONSERV if idf else None
    gam, lam, ll, lr, N, mf = _nc_evolved(pkg, L, d, chi, L, cons)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N, max_filling=mf, conserv=cons) as c:
        c.set_theta_form(107)
        c.set_state(gam, lam, ll, lr)
        te = c.swapping(3)
        g1, l1, ll1, _ = c.get_state()
    rg1, rg2, rl1, rll1, _, rte = oracle.swapping_nc(gam[2], gam[3], lam[2], lam[3], lam[4], ll[2], ll[3],
                                                     lr[3], lr[4], N, mf, conserv=cons)
    assert abs(te - rte) < 1e-11
    assert np.allclose(np.sort(l1[3]), np.sort(rl1), atol=1e-11)
    assert sorted(zip(np.round(l1[3], 8), ll1[3])) == sorted(zip(np.round(rl1, 8), rll1))
    rho = obs.two_site_rho(lam[2], g1[2], l1[3], g1[3], lam[4])
    rrho = obs.two_site_rho(lam[2], rg1, rl1, rg2, lam[4])
    assert np.allclose(rho, rrho, atol=1e-11)


def test_tc_theta_chain_matches_fp64_route(pkg):
    """d=5, chi=64, L=16: eight 2nd-order steps from the Mott state (blocks of up to
    ~100 rows on several size buckets), tensor-core Theta against the FP64 Theta:
    labels exact, Lambdas and observables within 1e-10."""
    L, d, chi, N = 16, 5, 64, 16
    gam, lam, ll, lr, Hb, Udt = nc_setup(pkg, L, d, chi, N, 11, 0.05)
    out = []
    for form in (0, 107):
        with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
            c.set_theta_form(form)
            c.set_state(gam, lam, ll, lr)
            te = sum(c.trotter_step(Udt, 2) for _ in range(8))
            out.append((te, c.get_state(), c.local_energy(Hb)))
    (te0, s0, e0), (te1, s1, e1) = out
    assert max(int(np.sum(x > 0)) for x in s0[1]) > 8  # several charge blocks by now
    assert abs(te0 - te1) < 1e-10
    for a, b in zip(s0[1], s1[1]):
        assert np.max(np.abs(a - b)) < 1e-10
    for a, b in zip(s0[2] + s0[3], s1[2] + s1[3]):
        assert np.array_equal(a, b)
    assert np.max(np.abs(e0 - e1)) < 1e-10
    nop = np.diag(np.arange(d, dtype=float))
    assert np.allclose(obs.one_site_expval(*s0[:2], nop), obs.one_site_expval(*s1[:2], nop), atol=1e-10)


def test_tc_theta_form_rules(pkg):
    with pkg.Chain(4, 3, 4, mode=pkg.MODE_NC, tot_num=4) as c:
        with pytest.raises(pkg.TebdError) as e:
            c.set_theta_form(3)  # 3xTF32 (FP32 class) stays a dense-handle form
        assert e.value.code == 6  # TEBD_ERR_STATE
        for form in (0, 105, 107):
            c.set_theta_form(form)
