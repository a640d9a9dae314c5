"""tebd_two_site_op_noalloc: the update for callers that cannot allocate.

Some callers may not allocate device memory when they run the update (they are
inside a CUDA-graph capture, or their device memory comes from a fixed pool, or
their Fortran host keeps its own device-resident chain and no library handle).
For them the library exposes one entry point whose temporaries live in a static
device array of fixed size (d*chi <= 256).  This file checks it through the C ABI
against the handle-based tebd_two_site_op on the same inputs, for two calls in a
row (the array keeps the first call's contents, so the second call also checks
that everything that must start at zero is cleared).  It is collected last so
that a failure here stops a `-x` run only after every other test has run.
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
    lam[2][chi // 2:] = 0.0  # exact zeros: the compacted path inside the update
    lam = [l / np.linalg.norm(l) for l in lam]
    return gam, lam


def _unitary(n, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def test_noalloc_matches_handle_path_twice(pkg):
    torch = pytest.importorskip("torch")
    lib = pkg.load_library()
    L, d, chi = 5, 4, 24  # n = 96 <= 256
    gam, lam = _state(L, d, chi, 5)
    gates = [_unitary(d * d, 11), _unitary(d * d, 12)]
    links = [2, 3]  # second call overlaps the first bond's output site: order matters

    # caller-owned device chain (the test allocates; the entry point does not)
    g_dev = torch.from_numpy(np.stack([g.ravel(order="F") for g in gam])).cuda()
    l_dev = torch.from_numpy(np.stack(lam)).cuda()
    ref = pkg.Chain(L, d, chi)
    ref.set_state(gam, lam)
    for call, (link, U) in enumerate(zip(links, gates)):
        op_dev = torch.from_numpy(np.asfortranarray(U).ravel(order="F")).cuda()
        te = ctypes.c_double(-1.0)
        torch.cuda.synchronize()
        rc = lib.tebd_two_site_op_noalloc(L, d, chi, link, g_dev.data_ptr(), l_dev.data_ptr(),
                                          op_dev.data_ptr(), ctypes.byref(te), None)
        assert rc == 0, (call, rc)
        te_ref = ref.two_site_op(link, U)
        g_out = [np.asfortranarray(g_dev[s].cpu().numpy().reshape((chi, d, chi), order="F")) for s in range(L)]
        l_out = [l_dev[s].cpu().numpy() for s in range(L + 1)]
        g_ref, l_ref = ref.get_state()
        assert abs(te.value - te_ref) < 1e-11, call
        for a, b in zip(l_out, l_ref):
            assert np.allclose(a, b, atol=1e-11), call
        rho = obs.two_site_rho(l_out[link - 1], g_out[link - 1], l_out[link], g_out[link], l_out[link + 1])
        rrho = obs.two_site_rho(l_ref[link - 1], g_ref[link - 1], l_ref[link], g_ref[link], l_ref[link + 1])
        assert np.allclose(rho, rrho, atol=1e-11), call
        # the random chain is not normalised: compare the normalised overlap
        ov = obs.inner_product(g_ref, l_ref, g_out, l_out)
        nn = obs.inner_product(g_ref, l_ref, g_ref, l_ref) * obs.inner_product(g_out, l_out, g_out, l_out)
        assert abs(abs(ov) / np.sqrt(abs(nn)) - 1.0) < 1e-10, call
    ref.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg):
    lib = pkg.load_library()
    te = ctypes.c_double(0.0)
    # d*chi = 5*64 = 320 > 256: refused before any device work
    assert lib.tebd_two_site_op_noalloc(4, 5, 64, 1, 1, 1, 1, ctypes.byref(te), None) == 1
    assert lib.tebd_two_site_op_noalloc(4, 2, 8, 0, 1, 1, 1, ctypes.byref(te), None) == 1
