"""The CPU-runnable configuration end to end: spin-1/2 Heisenberg chain with
J = 1, Delta = 1, L = 32, d = 2, chi = 32, open boundaries, Neel product state,
2nd-order Trotter steps of dt = 0.01, 100 steps (4700 bond updates), on the GPU
through the C ABI and in the oracle, compared on the final state."""
import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


def test_heisenberg_neel_quench_100_steps(pkg, oracle):
    H = pkg.hamiltonians
    L, d, chi, dt, steps = 32, 2, 32, 0.01, 100
    carray = np.zeros((d, L), complex)
    carray[0, 0::2] = 1.0  # Neel: up on odd sites (1-based), down on even ones
    carray[1, 1::2] = 1.0
    gam, lam = H.product_state(carray, chi)
    Hb = H.heisenberg(L, 1.0, 1.0, 1.0)
    U = H.construct_propagators(Hb, dt, 2)
    with pkg.Chain(L, d, chi) as c:
        c.set_state(gam, lam)
        te = sum(c.trotter_step(U, 2) for _ in range(steps))
        g1, l1 = c.get_state()
        sz_gpu = c.one_site_expval(np.diag([0.5, -0.5]))
        e_gpu = c.local_energy(Hb)
        s_gpu = c.chain_entropy()
    rte = sum(oracle.trotter_step(gam, lam, U, 2) for _ in range(steps))
    assert abs(te - rte) < 1e-10
    for a, b in zip(l1, lam):
        assert np.allclose(a, b, atol=1e-10)
    sz = np.diag([0.5, -0.5])
    assert np.allclose(sz_gpu, obs.one_site_expval(gam, lam, sz), atol=1e-10)
    assert np.allclose(e_gpu, obs.bond_energy(gam, lam, Hb), atol=1e-10)
    assert np.allclose(s_gpu, obs.chain_entropy(lam, d), atol=1e-10)
    assert abs(abs(obs.inner_product(gam, lam, g1, l1)) - 1.0) < 1e-10
    # the quench moved the Neel pattern: the staggered magnetisation has decayed
    stag = np.mean(sz_gpu * (-1.0) ** np.arange(L))
    assert 0.0 < stag < 0.5 - 1e-3
