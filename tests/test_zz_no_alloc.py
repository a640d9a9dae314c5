"""tebd_two_site_op_noalloc: the update for callers that cannot allocate.

Some hosts cannot allocate device memory when they run the update: their device
memory comes from a fixed pool sized at start-up (a further cudaMalloc would fail
or break the pool's budget), or they keep the chain in their own device memory and
cannot own a library handle (creating one allocates the SVD workspaces of a whole
sweep), or they keep cudaMalloc/cudaFree -- which can stall or synchronise the
device -- out of a time-critical loop.  For them the library exposes one entry
point whose temporaries live in a static device array of fixed size
(d*chi <= 256).

This file checks it through the C ABI, for two calls in a row (the array keeps the
first call's contents, so the second call also checks that everything that must
start at zero is cleared):
* against the handle-based tebd_two_site_op on the same inputs (the existing
  entry point): Lambdas and truncation error within 1e-11, the two-site density
  matrix within 1e-11, normalised overlap within 1e-10;
* against the oracle's TwoSiteOp (new Lambda and truncation error within 1e-11);
* that device free memory is unchanged around a warmed-up call.
Shapes: an interior case, the d*chi = 256 limit at d = 2 and at d = 8 (whose gate
kernel needs more than the default 48 KB of shared memory), and chi = 1.
It is collected last so that a failure here stops a `-x` run only after every
other test has run.
"""
import ctypes

import numpy as np
import pytest

from oracle import observables as obs

pytestmark = pytest.mark.gpu


def _state(L, d, chi, seed):
    rng = np.random.default_rng(seed)
    gam = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
           for _ in range(L)]
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(L + 1)]
    if chi > 1:
        lam[2][chi // 2:] = 0.0  # exact zeros: the compacted path inside the update
    lam = [l / np.linalg.norm(l) for l in lam]
    return gam, lam


def _unitary(n, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _call(lib, L, d, chi, link, g_dev, l_dev, op_dev):
    te = ctypes.c_double(-1.0)
    rc = lib.tebd_two_site_op_noalloc(L, d, chi, link, g_dev.data_ptr(), l_dev.data_ptr(),
                                      op_dev.data_ptr(), ctypes.byref(te), None)
    return rc, te.value


@pytest.mark.parametrize("d,chi", [(4, 24), (2, 128), (8, 32), (4, 1)])
def test_noalloc_matches_handle_path_and_oracle_twice(pkg, oracle, d, chi):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    L = 5
    gam, lam = _state(L, d, chi, 5 + d + chi)
    gates = [_unitary(d * d, 11 + d), _unitary(d * d, 12 + d)]
    links = [2, 3]  # the second call overlaps the first bond's output site: order matters

    # caller-owned device chain (the test allocates; the entry point does not)
    g_dev = torch.from_numpy(np.stack([g.ravel(order="F") for g in gam])).cuda()
    l_dev = torch.from_numpy(np.stack(lam)).cuda()
    ref = pkg.Chain(L, d, chi)
    ref.set_state(gam, lam)
    for call, (link, U) in enumerate(zip(links, gates)):
        op_dev = torch.from_numpy(np.asfortranarray(U).ravel(order="F")).cuda()
        # the oracle's update of the same bond from the same (current) state
        g_in = [np.asfortranarray(g_dev[s].cpu().numpy().reshape((chi, d, chi), order="F")) for s in range(L)]
        l_in = [l_dev[s].cpu().numpy() for s in range(L + 1)]
        _, _, o_l1, o_te, _ = oracle.two_site_op(g_in[link - 1], g_in[link], l_in[link - 1], l_in[link],
                                                 l_in[link + 1], U)
        torch.cuda.synchronize()
        rc, te = _call(lib, L, d, chi, link, g_dev, l_dev, op_dev)
        assert rc == 0, (call, rc)
        te_ref = ref.two_site_op(link, U)
        g_out = [np.asfortranarray(g_dev[s].cpu().numpy().reshape((chi, d, chi), order="F")) for s in range(L)]
        l_out = [l_dev[s].cpu().numpy() for s in range(L + 1)]
        g_ref, l_ref = ref.get_state()
        # against the existing entry point
        assert abs(te - te_ref) < 1e-11, call
        for a, b in zip(l_out, l_ref):
            assert np.allclose(a, b, atol=1e-11), call
        rho = obs.two_site_rho(l_out[link - 1], g_out[link - 1], l_out[link], g_out[link], l_out[link + 1])
        rrho = obs.two_site_rho(l_ref[link - 1], g_ref[link - 1], l_ref[link], g_ref[link], l_ref[link + 1])
        assert np.allclose(rho, rrho, atol=1e-11), call
        ov = obs.inner_product(g_ref, l_ref, g_out, l_out)  # the random chain is not normalised
        nn = obs.inner_product(g_ref, l_ref, g_ref, l_ref) * obs.inner_product(g_out, l_out, g_out, l_out)
        assert abs(abs(ov) / np.sqrt(abs(nn)) - 1.0) < 1e-10, call
        # against the oracle
        assert abs(te - o_te) < 1e-11, call
        assert np.max(np.abs(l_out[link] - o_l1)) < 1e-11, call
    ref.close()


def test_noalloc_allocates_no_device_memory(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    L, d, chi = 4, 4, 32
    gam, lam = _state(L, d, chi, 3)
    g_dev = torch.from_numpy(np.stack([g.ravel(order="F") for g in gam])).cuda()
    l_dev = torch.from_numpy(np.stack(lam)).cuda()
    op_dev = torch.from_numpy(np.asfortranarray(_unitary(d * d, 4)).ravel(order="F")).cuda()
    torch.cuda.synchronize()
    assert _call(lib, L, d, chi, 2, g_dev, l_dev, op_dev)[0] == 0  # warm-up: module load, set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for link in (1, 2, 3, 2):
        assert _call(lib, L, d, chi, link, g_dev, l_dev, op_dev)[0] == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg):
    lib = pkg.load_library()
    te = ctypes.c_double(0.0)
    # d*chi = 5*64 = 320 > 256: refused before any device work
    assert lib.tebd_two_site_op_noalloc(4, 5, 64, 1, 1, 1, 1, ctypes.byref(te), None) == 1
    assert lib.tebd_two_site_op_noalloc(4, 2, 8, 0, 1, 1, 1, ctypes.byref(te), None) == 1
    assert lib.tebd_two_site_op_noalloc(4, 9, 8, 1, 1, 1, 1, ctypes.byref(te), None) == 1  # d > 8
