"""The autotuner (tebd_autotune, csrc/tune.cu): it leaves the chain and the
statistics as they were, fills the device's table, and the tuned shapes give the
same update as the defaults (within rounding) and the oracle."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


def _saturated(pkg, L, d, chi, seed):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = []
    for _ in range(L + 1):
        l = np.exp(-np.arange(chi) / (chi / 6.0))
        lam.append(l / np.linalg.norm(l))
    return gam, lam


@pytest.mark.parametrize("mode", ["fp64", "df", "rsvd"])
def test_autotune_keeps_state_and_results(pkg, oracle, mode):
    H = pkg.hamiltonians
    L, d, chi = 12, 5, 48
    svd = {"fp64": pkg.SVD_FP64, "df": pkg.SVD_DF, "rsvd": pkg.SVD_RSVD}[mode]
    gam, lam = _saturated(pkg, L, d, chi, 3)
    gate = H.matrix_exponential(H.bose_hubbard(L, d, 1.0, 2.0)[1], 0.01)
    links = list(range(1, L, 2))
    pkg.clear_tuning(0)
    try:
        with pkg.Chain(L, d, chi, svd_mode=svd) as c:
            c.set_state(gam, lam)
            if mode == "rsvd":
                c.set_rsvd(oversample=32, power_iters=2)
            c.apply_bonds(links, [gate] * len(links))  # a state whose bonds the route can take
            g0, l0 = c.get_state()
            c.reset_stats()
            base, best = c.autotune(links, [gate] * len(links))
            assert 0 < best <= base
            assert c.stats()["updates"] == 0
            g1, l1 = c.get_state()
            for a, b in zip(g0 + l0, g1 + l1):
                assert np.array_equal(a, b)
            rows = pkg.get_tuning(0)
            assert rows, "no tuning entries"
            routes = {r["route"] for r in rows}
            assert ("randomized-route Cholesky" in routes) == (mode == "rsvd")
            assert ("randomized-route Cholesky blocking" in routes) == (mode == "rsvd")
            for r in rows:
                assert r["cluster"] in (0, 1, 2, 3, 4, 5, 6, 7, 8) and r["team"] in (0, 1, 2, 4, 8)
                assert r["panel"] in (0, 4, 8, 16) and r["chol_cluster"] in (0, 1, 2, 4, 8)
                assert r["chol_leaf"] in (0, 128, 192, 256, 384, 768)
                assert r["orth_cluster"] in (0, 1, 2, 4, 8)
                assert r["batch_us"] > 0
            c.apply_bonds(links, [gate] * len(links))  # tuned shapes
            gt, lt = c.get_state()
            st = c.stats()
            if mode == "rsvd":  # one batch on the route, with the sketch set above
                assert st["rsvd_batches"] == 1 and st["rsvd_updates"] > 0
                assert st["rsvd_oversample_sum"] == 32 and st["rsvd_power_sum"] == 2
            else:
                assert st["rsvd_batches"] == 0
        pkg.clear_tuning(0)
        assert pkg.get_tuning(0) == []
        with pkg.Chain(L, d, chi, svd_mode=svd) as c:  # default shapes, same start
            c.set_state(g0, l0)
            if mode == "rsvd":
                c.set_rsvd(oversample=32, power_iters=2)
            c.apply_bonds(links, [gate] * len(links))
            gd, ld = c.get_state()
        for k in links:
            assert np.allclose(lt[k], ld[k], atol=1e-12)
            a = obs.two_site_rho(lt[k - 1], gt[k - 1], lt[k], gt[k], lt[k + 1])
            b = obs.two_site_rho(ld[k - 1], gd[k - 1], ld[k], gd[k], ld[k + 1])
            assert np.max(np.abs(a - b)) < 1e-11
        # and the oracle on one bond
        k = links[len(links) // 2]
        r = oracle.two_site_op(g0[k - 1], g0[k], l0[k - 1], l0[k], l0[k + 1], gate)
        assert np.allclose(lt[k], r[2], atol=1e-10 if mode == "rsvd" else 1e-12)
    finally:
        pkg.clear_tuning(0)
