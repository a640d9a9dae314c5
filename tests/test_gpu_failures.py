"""Failure paths of the update, made on the host (no GPU fault involved).

The reference ignores ZGESVD's `info` (VidalCore_v_2.0/local_operations_module.f90:
335-336) and carries NaNs on silently.  The C ABI reports both failures instead,
and the bonds of the batch that met one keep their Gammas, Lambdas and labels:
* a NaN written into a Gamma from the host: TEBD_ERR_NONFINITE (dense, NC, and
  the allocation-free entry point);
* a Jacobi sweep cap of one on a bond routed to Jacobi: TEBD_ERR_SVD_NOCONV.
After the failure the handle stays usable: the same bond with a finite state, or
with the default sweep cap, updates normally.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TEBD_ERR_SVD_NOCONV, TEBD_ERR_NONFINITE = 4, 5


def _bond(chi, d, seed, L=4):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(L + 1)]
    return gam, [l / np.linalg.norm(l) for l in lam]


def _unitary(n, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _same(a, b):
    return all(np.array_equal(x, y, equal_nan=True) for x, y in zip(a, b))


@pytest.mark.parametrize("chi,d,svd_mode", [(8, 2, 0), (32, 3, 0), (32, 3, 3)])
def test_nan_gamma_gives_nonfinite_and_keeps_the_chain(pkg, chi, d, svd_mode):
    gam, lam = _bond(chi, d, 40 + chi)
    gam[1][1, 0, 2] = np.nan
    U = _unitary(d * d, 3)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:
        c.set_state(gam, lam)
        g0, l0 = c.get_state()
        with pytest.raises(pkg.TebdError) as e:
            c.two_site_op(2, U)
        assert e.value.code == TEBD_ERR_NONFINITE
        g1, l1 = c.get_state()
        assert _same(g0, g1) and _same(l0, l1)
        # the handle is still usable once the state is finite again
        gam[1][1, 0, 2] = 0.5
        c.set_state(gam, lam)
        c.two_site_op(2, U)
        assert np.all(np.isfinite(c.get_lambda(3)))


@pytest.mark.parametrize("svd_mode", [2, 4])
def test_sweep_cap_gives_noconv_and_keeps_the_chain(pkg, svd_mode):
    chi, d = 12, 3
    gam, lam = _bond(chi, d, 7)
    U = _unitary(d * d, 8)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode, max_sweeps=1) as c:
        c.set_state(gam, lam)
        g0, l0 = c.get_state()
        with pytest.raises(pkg.TebdError) as e:
            c.two_site_op(2, U)
        assert e.value.code == TEBD_ERR_SVD_NOCONV
        g1, l1 = c.get_state()
        assert _same(g0, g1) and _same(l0, l1)
    with pkg.Chain(4, d, chi, svd_mode=svd_mode) as c:  # default cap: converges
        c.set_state(gam, lam)
        c.two_site_op(2, U)
        assert c.sweeps(2) > 1


def test_nan_gamma_nc_keeps_gammas_lambdas_and_labels(pkg):
    H = pkg.hamiltonians
    L, d, chi, N = 8, 3, 16, 8
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    Udt = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 2.0), 0.05, 2)
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        for _ in range(3):  # entangle the Mott state a little
            c.trotter_step(Udt, 2)
        g, l, a, b = c.get_state()
        g[3][0, 1, 0] = np.nan
        c.set_state(g, l, a, b)
        before = c.get_state()
        with pytest.raises(pkg.TebdError) as e:
            c.two_site_op(4, Udt[3])
        assert e.value.code == TEBD_ERR_NONFINITE
        after = c.get_state()
        for x, y in zip(before, after):
            assert _same(x, y)


def test_nan_gamma_noalloc_keeps_the_chain(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    L, d, chi = 4, 3, 16
    gam, lam = _bond(chi, d, 9, L)
    gam[2][0, 0, 0] = np.nan
    g_dev = torch.from_numpy(np.stack([g.ravel(order="F") for g in gam])).cuda()
    l_dev = torch.from_numpy(np.stack(lam)).cuda()
    op_dev = torch.from_numpy(np.asfortranarray(_unitary(d * d, 2)).ravel(order="F")).cuda()
    g0, l0 = g_dev.clone(), l_dev.clone()
    te = ctypes.c_double(0.0)
    torch.cuda.synchronize()
    rc = lib.tebd_two_site_op_noalloc(L, d, chi, 2, g_dev.data_ptr(), l_dev.data_ptr(), op_dev.data_ptr(),
                                      ctypes.byref(te), None)
    assert rc == TEBD_ERR_NONFINITE
    assert torch.equal(torch.isnan(g0), torch.isnan(g_dev))
    assert torch.equal(torch.nan_to_num(g0), torch.nan_to_num(g_dev)) and torch.equal(l0, l_dev)
