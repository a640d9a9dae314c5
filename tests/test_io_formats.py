"""The oracle's restatement of the reference's record formats (io_module.f90)
against values worked out by hand from the Fortran edit descriptors."""
import numpy as np

from oracle import io_formats as F


def test_e30_15_fields():
    assert F.e30_15(1.0) == " " * 9 + "0.100000000000000E+01"
    assert F.e30_15(-2.5e-3) == " " * 8 + "-0.250000000000000E-02"
    assert F.e30_15(0.0) == " " * 9 + "0.000000000000000E+00"
    assert F.e30_15(1.2345678901234567e-120) == " " * 9 + "0.123456789012346-119"
    assert F.e30_15(9.999999999999999e99) == " " * 9 + "0.100000000000000+101"
    assert all(len(F.e30_15(x)) == 30 for x in (1e300, -1e-300, 123.456))


def test_b80_fields():
    assert F.b80(1.0) == ("1" * 10 + "0" * 52).rjust(80)
    assert F.b80(0.0) == "0".rjust(80)
    assert F.b80(-1.0) == ("10" + "1" * 10 + "0" * 52).rjust(80)  # sign bit set


def test_round_trips():
    rng = np.random.default_rng(0)
    L, chi, d = 3, 4, 2
    lam = [rng.standard_normal(chi) * 10.0 ** rng.integers(-150, 150, chi) for _ in range(L + 1)]
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    for a, b in zip(F.parse_lambdas(F.format_lambdas(lam, "B"), L, chi, "B"), lam):
        assert np.array_equal(a, b)
    for a, b in zip(F.parse_lambdas(F.format_lambdas(lam, "S"), L, chi, "S"), lam):
        assert np.allclose(a, b, rtol=5.1e-15, atol=0)  # 15 significant digits
    for a, b in zip(F.parse_gammas(F.format_gammas(gam, "B"), L, chi, d, "B"), gam):
        assert np.array_equal(a, b)
    text = F.format_gammas(gam, "S")
    assert len(text.splitlines()) == 2 * L * chi * chi
    assert all(len(line) == 30 * d for line in text.splitlines())
