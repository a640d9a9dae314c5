"""The learned part of the learned-rank form: the model's hand-written kernels
against the CPU oracle, its training on spectra the method produces, and what it
gains the randomized route.

* forward and gradient (tebd_mlp_forward / tebd_mlp_loss_grad, FP32 on the GPU)
  against oracle/mlp_oracle.py (float64): outputs within 1e-4 relative, loss
  within 1e-5 relative, gradient within 1e-3 relative in norm and per element
  within 1e-3 of the largest gradient entry;
* training (tebd_mlp_train, Adam) on logged spectra lowers the loss tenfold and
  predicts held-out spectra (log10 of singular-value ratios) better than their
  mean;
* A/B: the same Trotter steps of a saturated Bose-Hubbard chain through the
  randomized route with a trained model choosing the sketch, against a
  conservative fixed sketch (p = 128, q = 3) and a cheap one (p = 16, q = 0): the
  model keeps the conservative sketch's agreement with plain FP64 (two-site
  density matrices within 1e-8) for fewer tensor-core flops, and sends no more
  bonds to the full SVD than the cheap sketch.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO
from oracle import observables as obs

pytestmark = pytest.mark.gpu


def _rand(seed, n):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, MO.N_IN)).astype(np.float32)
    t = rng.standard_normal((n, MO.N_OUT)).astype(np.float32)
    p = (0.2 * rng.standard_normal(MO.N_PARAMS)).astype(np.float32)
    return x, t, p


def test_mlp_forward_matches_cpu_oracle(pkg):
    x, _, p = _rand(1, 257)
    m = pkg.Mlp(seed=3)
    m.set_params(p)
    y = m.forward(x)
    yr, _ = MO.forward(p, x)
    assert np.max(np.abs(y - yr)) <= 1e-4 * max(1.0, np.max(np.abs(yr)))
    m.close()


def test_mlp_gradient_matches_cpu_oracle(pkg):
    x, t, p = _rand(2, 300)
    m = pkg.Mlp(seed=4)
    m.set_params(p)
    loss, g = m.loss_grad(x, t)
    lr, gr = MO.loss_grad(p, x, t)
    assert abs(loss - lr) <= 1e-5 * lr
    assert np.linalg.norm(g - gr) <= 1e-3 * np.linalg.norm(gr)
    assert np.max(np.abs(g - gr)) <= 1e-3 * np.max(np.abs(gr))
    m.close()


def _bh_chain(pkg, L, d, chi, seed):
    H = pkg.hamiltonians
    carray = np.zeros((d, L), complex)
    carray[1, :] = 1.0
    gam, lam = H.perturbed_product_state(carray, chi, 1e-3, seed)
    return gam, lam


def _logged(pkg, seeds, L=12, d=5, chi=24, dt=0.05, steps=25):
    from importlib import import_module

    learned = import_module(pkg.__name__ + ".learned")
    H = pkg.hamiltonians
    gates = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 2.0), dt, 2)
    xs, ts = [], []
    for s in seeds:
        gam, lam = _bh_chain(pkg, L, d, chi, s)
        x, t = learned.log_run(pkg, gam, lam, gates, steps)
        xs.append(x)
        ts.append(t)
    return np.concatenate(xs), np.concatenate(ts)


def test_mlp_training_on_logged_spectra(pkg):
    x, t = _logged(pkg, [11, 12])
    xv, tv = _logged(pkg, [13])
    assert len(x) > 100 and len(xv) > 20
    m = pkg.Mlp(seed=5)
    l0, _ = m.loss_grad(x, t)
    loss = m.train(x, t, epochs=300, batch=128, lr=2e-3)
    assert loss < 0.1 * l0, (loss, l0)
    err_model = np.mean((m.forward(xv) - tv) ** 2)
    err_mean = np.mean((t.mean(0) - tv) ** 2)
    assert err_model < err_mean, (err_model, err_mean)
    m.close()


def test_learned_model_gains_over_fixed_sketch(pkg):
    """The model against two fixed sketches on the same saturated steps: a
    conservative one (p = 128, q = 3) that every bond passes, and a cheap one
    (p = 16, q = 0).  With the model the route keeps the conservative sketch's
    accuracy (two-site density matrices within 1e-8 of plain FP64) for fewer
    tensor-core flops, and sends no more bonds to the full SVD than the cheap
    sketch does."""
    H = pkg.hamiltonians
    x, t = _logged(pkg, [21, 22], L=12, d=5, chi=48, steps=30)
    m = pkg.Mlp(seed=6)
    m.train(x, t, epochs=300, batch=128, lr=2e-3)
    L, d, chi, dt = 12, 5, 48, 0.05
    gates = H.construct_propagators(H.bose_hubbard(L, d, 1.0, 2.0), dt, 2)
    gam, lam = _bh_chain(pkg, L, d, chi, 23)
    with pkg.Chain(L, d, chi) as c:  # to saturation in plain FP64
        c.set_state(gam, lam)
        for _ in range(30):
            c.trotter_step(gates, 2)
        gam, lam = c.get_state()
    res = {}
    for name, mode, sketch, model in (("fp64", pkg.SVD_FP64, None, None),
                                      ("conservative", pkg.SVD_RSVD, (128, 3), None),
                                      ("cheap", pkg.SVD_RSVD, (16, 0), None),
                                      ("model", pkg.SVD_RSVD, None, m)):
        with pkg.Chain(L, d, chi, svd_mode=mode) as c:
            c.set_state(gam, lam)
            if sketch is not None:
                c.set_rsvd(oversample=sketch[0], power_iters=sketch[1])
            if model is not None:
                c.set_rsvd_model(model, 1e-10)
            for _ in range(3):
                c.trotter_step(gates, 2)
            g, l = c.get_state()
            res[name] = ((g, l), c.stats())
    (g0, l0), _ = res["fp64"]
    for name in ("conservative", "model"):
        (g1, l1), st = res[name]
        assert st["rsvd_updates"] > 0, name
        for k in range(1, L):
            a = obs.two_site_rho(l0[k - 1], g0[k - 1], l0[k], g0[k], l0[k + 1])
            b = obs.two_site_rho(l1[k - 1], g1[k - 1], l1[k], g1[k], l1[k + 1])
            assert np.max(np.abs(a - b)) < 1e-8, (name, k)
    cons, cheap, model = res["conservative"][1], res["cheap"][1], res["model"][1]
    assert model["rsvd_flops"] < cons["rsvd_flops"], (model["rsvd_flops"], cons["rsvd_flops"])
    assert model["rsvd_fallbacks"] <= cheap["rsvd_fallbacks"], (model, cheap)
    m.close()


def test_spin1_learned_form_matches_fp64(pkg):
    """The learned-rank configuration's shape at reduced size: spin-1 chain with
    random single-ion anisotropy (d = 3), a random MPS at chi = 8 growing to
    chi = 24 (saturated from the second sweep, so that the randomized route is
    taken), discarded weight <= 1e-10 per update; the learned form (randomized
    route sized by the committed model, Theta on the tensor cores) and the same
    route with a fixed sketch against plain FP64 with the same kept-rank rule:
    local observables within 1e-8."""
    import os

    H = pkg.hamiltonians
    L, d, chi0, chi = 16, 3, 8, 24
    rng = np.random.default_rng(4)
    g = [np.asfortranarray(rng.standard_normal((chi0, d, chi0)) + 1j * rng.standard_normal((chi0, d, chi0)))
         for _ in range(L)]
    lm = [np.full(chi0, 1.0 / np.sqrt(chi0)) for _ in range(L + 1)]
    lm[0] = np.eye(chi0)[0]
    lm[L] = np.eye(chi0)[0]
    with pkg.Chain(L, d, chi0) as c:
        c.set_state(g, lm)
        c.canonical_form_all()
        g, lm = c.get_state()
    gam = []
    for x in g:
        y = np.zeros((chi, d, chi), complex, order="F")
        y[:chi0, :, :chi0] = x
        gam.append(y)
    lam = []
    for x in lm:
        y = np.zeros(chi)
        y[:chi0] = x
        lam.append(y)
    Di = np.random.default_rng(4).uniform(-0.5, 0.5, L)
    Hb = H.spin1_xxz_anisotropy(L, 1.0, 1.0, Di)
    U = H.construct_propagators(Hb, 0.01, 2)
    sz = H.spin_ops(1.0)[2]
    params = np.load(os.path.join(os.path.dirname(pkg.__file__), "data", "rsvd_model.npz"))["params"]
    m = pkg.Mlp(seed=0)
    m.set_params(params)
    res = {}
    for name in ("fp64", "fixed", "learned"):
        with pkg.Chain(L, d, chi, svd_mode=pkg.SVD_FP64 if name == "fp64" else pkg.SVD_RSVD) as c:
            c.set_rank_bound(1e-10)
            if name != "fp64":
                c.set_theta_form(107)
            if name == "fixed":
                c.set_rsvd(oversample=24, power_iters=2)
            if name == "learned":
                c.set_rsvd_model(m, 1e-10)
            c.set_state(gam, lam)
            for _ in range(6):
                c.trotter_step(U, 2)
            res[name] = (c.one_site_expval(sz), c.local_energy(Hb), c.chain_entropy(), c.stats())
    m.close()
    f = res["fp64"]
    assert res["fixed"][3]["rsvd_updates"] > 0  # the route is taken on this chain
    for name in ("fixed", "learned"):
        for a, b in zip(f[:3], res[name][:3]):
            assert np.max(np.abs(a - b)) < 1e-8, name
