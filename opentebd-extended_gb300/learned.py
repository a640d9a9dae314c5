"""Training data and training of the randomized route's model (tebd_mlp_*).

The model (csrc/mlp.cu) reads a bond's Lambda before an update and the gate, and
predicts the normalised Theta's singular values after it at the relative ranks
RANKS x chi; the randomized route uses the prediction to size its sketch per batch
(or to send a bond straight to the full SVD).  It is trained on spectra the method
itself produces: runs of the library with the QR + Jacobi route (TEBD_SVD_QRJ,
which returns every singular value, the tail beyond chi included), one sample per
bond update, replaying the sweeps of 2nd-order Trotter steps with
tebd_apply_bonds so that each bond's Lambda is read just before its update.

    python -m <package>.learned out.npz      (needs a GPU: logs, trains, saves)

The feature and target definitions here are the ones the library computes on the
device (k_mlp_features, rsvd_model_choice in capi.cu) -- keep them equal.
"""
from __future__ import annotations

import sys
import time

import numpy as np

RANKS = (0.75, 1.0, 1.125, 1.25, 1.5, 1.75, 2.0, 2.5)
FLOOR = -16.0


def gate_terms(U, d):
    """log10 |U - I|_F, log10 |offdiag(U)|_F (floored at -16), d / 8."""
    U = np.asarray(U, dtype=complex)
    dev = np.sum(np.abs(U - np.eye(len(U))) ** 2)
    off = np.sum(np.abs(U - np.diag(np.diag(U))) ** 2)
    f = lambda v: max(FLOOR, 0.5 * np.log10(v)) if v > 0 else FLOOR  # noqa: E731
    return [f(dev), f(off), d / 8.0]


def features(lam_prev, U, d):
    """67 floats: log10(lambda_k / lambda_0) at k = floor(j chi / 64), then the gate terms."""
    lam_prev = np.asarray(lam_prev, dtype=float)
    chi = len(lam_prev)
    l0 = lam_prev[0]
    x = np.full(67, FLOOR)
    for j in range(64):
        k = (j * chi) // 64
        r = lam_prev[k] / l0 if l0 > 0 else 0.0
        x[j] = np.log10(r) if r > 1e-16 else FLOOR
    x[64:] = gate_terms(U, d)
    return x


def targets(sigma, chi):
    """8 floats: log10(sigma_k / sigma_0) at k = round(rho chi) (1-based), rho in RANKS."""
    s = np.sort(np.asarray(sigma, dtype=float))[::-1]
    t = np.full(len(RANKS), FLOOR)
    if len(s) == 0 or s[0] <= 0:
        return t
    for i, rho in enumerate(RANKS):
        k = int(round(rho * chi)) - 1
        if k < len(s) and s[k] > 0:
            t[i] = max(FLOOR, np.log10(s[k] / s[0]))
    return t


def log_run(pkg, gam, lam, gates, steps, device=0, min_rank_frac=0.75):
    """Samples (x, t) from `steps` 2nd-order Trotter steps from (gam, lam) with the
    QR + Jacobi route; gates[link-1] is Udt(link).  Keeps the updates whose new
    Lambda has at least min_rank_frac x chi nonzero values (the bonds the
    randomized route can take)."""
    L = len(gam)
    chi, d, _ = gam[0].shape
    xs, ts = [], []
    odd = list(range(1, L, 2))
    even = list(range(2, L, 2))
    with pkg.Chain(L, d, chi, device=device, svd_mode=pkg.SVD_QRJ) as c:
        c.set_state(gam, lam)
        for _ in range(steps):
            for links in (odd, even, odd):
                before = {k: c.get_lambda(k + 1) for k in links}
                c.apply_bonds(links, [gates[k - 1] for k in links])
                for k in links:
                    s = c.singular_values(k)
                    if np.sum(c.get_lambda(k + 1) > 0) < min_rank_frac * chi:
                        continue
                    xs.append(features(before[k], gates[k - 1], d))
                    ts.append(targets(s, chi))
    if not xs:
        return np.zeros((0, 67), np.float32), np.zeros((0, len(RANKS)), np.float32)
    return np.asarray(xs, np.float32), np.asarray(ts, np.float32)


def training_runs(pkg, scale=1.0):
    """The logged workloads: the Bose-Hubbard (d = 5), spin-1/2 XXZ (d = 2) and
    Fermi-Hubbard (d = 4) chains of the configured runs at reduced L and chi, from
    their initial states, at a few time steps; `scale` multiplies the step counts."""
    H = pkg.hamiltonians
    runs = []
    # Bose-Hubbard, unit filling + perturbation (the plain-FP64 configuration's shape)
    for chi, dt, seed in ((32, 0.05, 11), (48, 0.04, 12)):
        L, d = 16, 5
        carray = np.zeros((d, L), complex)
        carray[1, :] = 1.0
        gam, lam = H.perturbed_product_state(carray, chi, 1e-3, seed)
        runs.append(("bose_hubbard", gam, lam, H.construct_propagators(H.bose_hubbard(L, d, 1.0, 2.0), dt, 2),
                     int(40 * scale)))
    # spin-1/2 XXZ, Neel state
    L, d, chi = 24, 2, 32
    carray = np.zeros((d, L), complex)
    carray[0, 0::2] = 1.0
    carray[1, 1::2] = 1.0
    gam, lam = H.product_state(carray, chi)
    runs.append(("xxz", gam, lam, H.construct_propagators(H.heisenberg(L, 1.0, 1.0, 1.0), 0.05, 2), int(60 * scale)))
    # Fermi-Hubbard, random MPS made canonical on the device
    L, d, chi = 12, 4, 32
    rng = np.random.default_rng(2)
    g = [np.asfortranarray(rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi)))
         for _ in range(L)]
    lm = [np.full(chi, 1.0 / np.sqrt(chi)) for _ in range(L + 1)]
    lm[0] = np.eye(chi)[0]
    lm[L] = np.eye(chi)[0]
    with pkg.Chain(L, d, chi) as c:
        c.set_state(g, lm)
        c.canonical_form_all()
        g, lm = c.get_state()
    runs.append(("fermi_hubbard", g, lm, H.construct_propagators(H.fermi_hubbard(L, 1.0, 4.0), 0.02, 2),
                 int(20 * scale)))
    return runs


def build_dataset(pkg, scale=1.0, device=0):
    xs, ts, names = [], [], []
    for name, gam, lam, gates, steps in training_runs(pkg, scale):
        x, t = log_run(pkg, gam, lam, gates, steps, device)
        xs.append(x)
        ts.append(t)
        names.append((name, len(x)))
    return np.concatenate(xs), np.concatenate(ts), names


def train(pkg, x, t, seed=0, epochs=400, batch=256, lr=1e-3, device=0):
    """A model trained on (x, t) by the library's kernels; returns (model, loss)."""
    m = pkg.Mlp(device=device, seed=seed)
    loss = m.train(x, t, epochs=epochs, batch=batch, lr=lr)
    return m, loss


def main(out):
    import os

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import __graft_entry__ as ge

    pkg = ge.load_package()
    t0 = time.time()
    x, t, names = build_dataset(pkg)
    t1 = time.time()
    rng = np.random.default_rng(0)
    perm = rng.permutation(len(x))
    x, t = x[perm], t[perm]
    m, loss = train(pkg, x, t)
    t2 = time.time()
    np.savez_compressed(out, params=m.params(), samples=len(x), runs=np.array([n for n, _ in names]),
                        run_samples=np.array([k for _, k in names]), train_loss=loss,
                        log_seconds=t1 - t0, train_seconds=t2 - t1)
    print("samples", len(x), dict(names), "train loss %.4g" % loss, "log %.1fs train %.1fs" % (t1 - t0, t2 - t1))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "rsvd_model.npz")
