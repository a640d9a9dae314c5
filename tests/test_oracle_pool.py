"""The parallel sweep driver (oracle/pool.py) against the oracle's own sequential
Trotter steps: same Gammas, Lambdas, labels and summed truncation error, for
dense and number-conserving chains, 2nd order and Forest-Ruth."""
import copy
import importlib.util
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle.pool import SweepPool, _trim, _untrim

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _hamiltonians():
    spec = importlib.util.spec_from_file_location(
        "hamiltonians", os.path.join(ROOT, "opentebd-extended_gb300", "hamiltonians.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_trim_roundtrip():
    g = np.zeros((6, 3, 6), complex, order="F")
    g[:2, :, :4] = 1.0 + 2.0j
    corner, chi = _trim(g)
    assert corner.shape == (2, 3, 4) and chi == 6
    assert np.array_equal(_untrim((corner, chi)), g)
    z = np.zeros((4, 2, 4), complex, order="F")
    assert np.array_equal(_untrim(_trim(z)), z)


@pytest.mark.parametrize("order", [2, 5])
def test_dense_sweeps_equal_sequential(order):
    H = _hamiltonians()
    L, d, chi = 8, 2, 8
    carray = np.zeros((d, L), complex)
    carray[0, 0::2] = 1.0
    carray[1, 1::2] = 1.0
    gam, lam = H.product_state(carray, chi)
    U = H.construct_propagators(H.heisenberg(L, 1.0, 1.0, 1.0), 0.1, order)
    g2, l2 = copy.deepcopy(gam), copy.deepcopy(lam)
    with SweepPool(2) as P:
        te = [P.trotter_step(gam, lam, U, order) for _ in range(3)]
    te2 = [O.trotter_step(g2, l2, U, order) for _ in range(3)]
    assert np.allclose(te, te2, rtol=1e-12, atol=1e-15)
    for a, b in zip(gam + lam, g2 + l2):
        assert np.array_equal(a, b)


def test_nc_sweeps_equal_sequential():
    H = _hamiltonians()
    L, d, chi, N = 8, 3, 12, 8
    gam, lam, ll, lr = H.initial_set_nc(L, d, chi, N)
    U = H.construct_propagators(H.bose_hubbard(L, d, 1.0, np.random.default_rng(7).uniform(1, 3, L)), 0.05, 2)
    g2, l2, ll2, lr2 = (copy.deepcopy(x) for x in (gam, lam, ll, lr))
    with SweepPool(2) as P:
        te = [P.trotter_step_nc(gam, lam, ll, lr, U, N, d - 1, 2) for _ in range(3)]
    te2 = [O.trotter_step_nc(g2, l2, ll2, lr2, U, N, d - 1, 2) for _ in range(3)]
    assert np.allclose(te, te2, rtol=1e-12, atol=1e-15)
    for a, b in zip(gam + lam + ll + lr, g2 + l2 + ll2 + lr2):
        assert np.array_equal(a, b)
