"""The decomposition behind the number-conserving Theta on the tensor cores
(nc.cu: k_nc_sizes / k_nc_oz_pack / k_tc_oz / k_nc_mix), checked on the CPU
against the oracle's FormThetaNC / ThetaOperationNC / RenormThetaNC / SVDNC.

Restated here in numpy: the charge blocks of a bond (minmaxNLR's clipped range,
IndexLeft / IndexRight order), each block's pre-gate Theta as ONE dense product
over its class of betas (left label q, right label totNum - q), the gate applied
to the <= d allowed entries of each (alpha, gamma) read back from the blocks,
and the blocks' singular values normalised by the norm of every entry written.
If an allowed entry with a nonzero class sum could lie outside every block, or a
block entry could need betas of another class, the flattened singular values
would differ from the oracle's, which sums per entry as the reference does.
Random Gammas (not block-sparse) and labels with unused (>= 1000) entries.
"""
import numpy as np
import pytest

from oracle import oracle as O

UNUSED = 10000


def _blocks(ll0, lr2, N, mf, nl):
    """minmaxNLR + SizeOfBlocks + IndexLeft/Right: (minNL, rows, cols) with rows[k]
    / cols[k] the (alpha, i) / (gamma, j) of block k in the reference's order."""
    chi, d = len(ll0), len(nl)
    mnl, mnr = int(ll0.min()), int(lr2.min())
    mxl = max(0 if x == UNUSED else int(x) for x in ll0) + mf
    mxr = max(0 if x == UNUSED else int(x) for x in lr2) + mf
    if mxl > N - mnr:
        mxl = N - mnr
    else:
        mnr = N - mxl
    if mxr > N - mnl:
        mxr = N - mnl
    else:
        mnl = N - mxr
    nb = mxl - mnl + 1
    rows = [[] for _ in range(nb)]
    cols = [[] for _ in range(nb)]
    for a in range(chi):
        for i in range(d):
            if ll0[a] < 1000 and mnl <= ll0[a] + nl[i] <= mxl:
                rows[ll0[a] + nl[i] - mnl].append((a, i))
    for g in range(chi):
        for j in range(d):
            if lr2[g] < 1000 and mnr <= lr2[g] + nl[j] <= mxr:
                cols[N - (lr2[g] + nl[j]) - mnl].append((g, j))
    return mnl, rows, cols


def _block_svd(g1, g2, l0, l1, l2, U, ll0, ll1, lr1, lr2, N, mf, nl):
    chi, d, _ = g1.shape
    A = l0[:, None, None] * g1 * l1[None, None, :]      # (alpha, i, beta)
    B = g2 * l2[None, None, :]                          # (beta, j, gamma)
    mnl, rows, cols = _blocks(ll0, lr2, N, mf, nl)
    blk = {}
    for k, (R, C) in enumerate(zip(rows, cols)):
        q = mnl + k
        betas = [b for b in range(chi) if ll1[b] == q and lr1[b] == N - q]
        Ak = np.array([[A[a, i, b] for b in betas] for a, i in R], complex).reshape(len(R), len(betas))
        Bk = np.array([[B[b, j, g] for g, j in C] for b in betas], complex).reshape(len(betas), len(C))
        blk[k] = Ak @ Bk
    pos_r = {e: (k, r) for k, R in enumerate(rows) for r, e in enumerate(R)}
    pos_c = {e: (k, c) for k, C in enumerate(cols) for c, e in enumerate(C)}
    out = {k: np.zeros_like(v) for k, v in blk.items()}
    norm2 = 0.0
    U4 = np.asarray(U).reshape(d * d, d * d)
    for a in range(chi):
        for g in range(chi):
            if ll0[a] >= 1000 or lr2[g] >= 1000:
                continue
            ntot = N - ll0[a] - lr2[g]
            pairs = [(i, l) for i in range(d) for l in range(d) if nl[i] + nl[l] == ntot and 0 <= nl[l] <= mf]
            th = []
            for i, l in pairs:
                q = ll0[a] + nl[i]
                v = 0.0
                if nl[i] <= mf and 0 <= q <= N and (a, i) in pos_r and (g, l) in pos_c:
                    (kr, r), (kc, c) = pos_r[(a, i)], pos_c[(g, l)]
                    assert kr == kc  # an allowed entry's row and column share a block
                    v = blk[kr][r, c]
                th.append(v)
            for k, jj in pairs:
                o = sum(U4[k * d + jj, i * d + l] * t for (i, l), t in zip(pairs, th))
                norm2 += abs(o) ** 2
                if (a, k) in pos_r and (g, jj) in pos_c:
                    (kr, r), (_, c) = pos_r[(a, k)], pos_c[(g, jj)]
                    out[kr][r, c] = o
    s = np.concatenate([np.linalg.svd(v, compute_uv=False) for v in out.values() if v.size] or [np.zeros(0)])
    return np.sort(s)[::-1] / np.sqrt(norm2)


def _bond(chi, d, N, seed, nl):
    """A random bond whose labels are consistent (LabelLeft + LabelRight = N on
    each used index) with a few unused indices on every link."""
    rng = np.random.default_rng(seed)
    g1 = rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi))
    g2 = rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi))
    lam = [np.sort(rng.random(chi))[::-1] for _ in range(3)]
    span = max(nl)
    c0 = N // 2 - span
    ll0 = rng.integers(c0 - 1, c0 + 2, chi).astype(np.int32)
    ll1 = rng.integers(c0, c0 + span + 3, chi).astype(np.int32)
    lr2 = (N - rng.integers(c0 + span - 1, c0 + 2 * span + 2, chi)).astype(np.int32)
    for lab, lam_ in ((ll0, lam[0]), (ll1, lam[1]), (lr2, lam[2])):
        dead = rng.random(chi) < 0.15
        lab[dead] = UNUSED
        lam_[dead] = 0.0
    lr1 = np.where(ll1 < 1000, N - ll1, UNUSED).astype(np.int32)
    return g1, g2, lam, ll0, ll1, lr1, lr2


def _unitary(n, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("chi,d,N,conserv,seed", [(10, 3, 12, None, 1), (14, 4, 16, None, 2),
                                                  (12, 4, 14, [0, 1, 1, 2], 3), (9, 5, 10, None, 4)])
def test_block_products_match_formthetanc(chi, d, N, conserv, seed):
    nl = list(conserv) if conserv is not None else list(range(d))
    mf = max(nl)
    g1, g2, (l0, l1, l2), ll0, ll1, lr1, lr2 = _bond(chi, d, N, seed, nl)
    U = _unitary(d * d, 100 + seed)
    s_blocks = _block_svd(g1, g2, l0, l1, l2, U, ll0, ll1, lr1, lr2, N, mf, nl)
    r = O.two_site_op_nc(np.asfortranarray(g1), np.asfortranarray(g2), l0, l1, l2, U, ll0, ll1, lr1, lr2, N, mf,
                         conserv=None if conserv is None else np.array(conserv))
    s_ref = np.sort(r[6])[::-1]
    assert s_ref.size > 4 and s_blocks.size == s_ref.size
    assert np.allclose(s_blocks, s_ref, rtol=1e-12, atol=1e-14)
