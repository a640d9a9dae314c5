"""State I/O in the reference's record formats through the C ABI: files written by
the library equal the oracle's restatement byte for byte, and reading them back
restores the chain (exactly for kind 'B', to 15 significant digits for 'S')."""
import numpy as np
import pytest

from oracle import io_formats as F

pytestmark = pytest.mark.gpu


def state(L, d, chi, seed):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] * 10.0 ** -rng.integers(0, 3) for _ in range(L + 1)]
    return gam, lam


@pytest.mark.parametrize("kind", ["S", "B"])
def test_record_and_read_back(pkg, tmp_path, kind):
    L, d, chi = 4, 3, 5
    gam, lam = state(L, d, chi, 3)
    lp, gp = tmp_path / "lambdas.dat", tmp_path / "gammas.dat"
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        c.record_lambdas(lp, kind)
        c.record_gammas(gp, kind)
    assert lp.read_text() == F.format_lambdas(lam, kind)
    assert gp.read_text() == F.format_gammas(gam, kind)
    with pkg.Chain(L, d, chi) as c:
        c.read_gamma_lambda(lp, gp, kind)
        g2, l2 = c.get_state()
    for a, b in zip(l2, lam):
        assert np.array_equal(a, b) if kind == "B" else np.allclose(a, b, rtol=5.1e-15, atol=0)
    for a, b in zip(g2, gam):
        if kind == "B":
            assert np.array_equal(a, b)
        else:
            assert np.allclose(a.real, b.real, rtol=5.1e-15, atol=0)
            assert np.allclose(a.imag, b.imag, rtol=5.1e-15, atol=0)


def test_read_smaller_chi_keeps_the_rest(pkg, tmp_path):
    """readGammaLambda(..., chiNow) fills the leading chiNow block of a larger
    allocation and leaves the other entries as they were."""
    L, d, chi, chi_now = 3, 2, 6, 4
    small_g, small_l = state(L, d, chi_now, 5)
    (tmp_path / "l.dat").write_text(F.format_lambdas(small_l, "B"))
    (tmp_path / "g.dat").write_text(F.format_gammas(small_g, "B"))
    big_g, big_l = state(L, d, chi, 6)
    with pkg.Chain(L, d, chi) as c:
        c.set_state(big_g, big_l)
        c.read_gamma_lambda(tmp_path / "l.dat", tmp_path / "g.dat", "B", chi_now)
        g2, l2 = c.get_state()
    for a, b, full in zip(l2, small_l, big_l):
        assert np.array_equal(a[:chi_now], b) and np.array_equal(a[chi_now:], full[chi_now:])
    for a, b, full in zip(g2, small_g, big_g):
        assert np.array_equal(a[:chi_now, :, :chi_now], b)
        assert np.array_equal(a[chi_now:], full[chi_now:]) and np.array_equal(a[:, :, chi_now:], full[:, :, chi_now:])


def test_labels_round_trip_nc(pkg, tmp_path):
    H = pkg.hamiltonians
    L, d, chi, N = 6, 3, 8, 6
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 1.0, 0.0), 0.05, 2)
    p = {k: tmp_path / (k + ".dat") for k in ("l", "g", "ll", "lr")}
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.set_state(gam, lam, ll, lr)
        c.trotter_step(U, 2)
        ref = c.get_state()
        c.record_lambdas(p["l"], "B")
        c.record_gammas(p["g"], "B")
        c.record_labels(p["ll"], p["lr"])
    assert p["ll"].read_text() == F.format_labels(ref[2])
    assert p["lr"].read_text() == F.format_labels(ref[3])
    with pkg.Chain(L, d, chi, mode=pkg.MODE_NC, tot_num=N) as c:
        c.read_gamma_lambda_labels(p["l"], p["g"], p["ll"], p["lr"], "B")
        got = c.get_state()
    for a, b in zip(got, ref):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_io_errors(pkg, tmp_path):
    with pkg.Chain(3, 2, 4) as c:
        with pytest.raises(pkg.TebdError):
            c.record_lambdas(tmp_path / "x.dat", "Q")
        with pytest.raises(pkg.TebdError):
            c.read_gamma_lambda(tmp_path / "missing_l.dat", tmp_path / "missing_g.dat")
        (tmp_path / "short.dat").write_text(F.format_lambdas([np.ones(4)] * 2, "S"))  # L+1 = 4 records needed
        (tmp_path / "g.dat").write_text("")
        with pytest.raises(pkg.TebdError):
            c.read_gamma_lambda(tmp_path / "short.dat", tmp_path / "g.dat")
        with pytest.raises(pkg.TebdError) as e:
            c.record_labels(tmp_path / "a.dat", tmp_path / "b.dat")  # dense handle
        assert e.value.code == 6
