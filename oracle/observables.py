"""Gauge-invariant checks on Vidal states (test infrastructure only).

numpy restatements of the reference's observables (VidalCore_v_2.0/observables_module.f90):

* :func:`single_site_rho`  -- FormSingleSiteRho (:95-117)
* :func:`one_site_expval`  -- OneSiteExpVal via Tr(rho O) (:134-254)
* :func:`two_site_rho`     -- ThetaKernal + TwoSiteRho for neighbouring sites (:704-835)
* :func:`bond_energy`      -- the per-bond term of TotalEnergy (:1432-1466)
* :func:`inner_product`    -- InnerProduct (:1031-1089)
* :func:`chain_entropy`    -- entanglement entropy of each Lambda, base d (ChainEntropy, :1583)
* :func:`state_vector`     -- the dense state of a small chain (no reference routine;
  used for exact-evolution known answers)

Gamma arrays are (chi, d, chi) complex, Lambdas (chi,) real, all 0-based lists.
"""
from __future__ import annotations

import numpy as np


def single_site_rho(lam0, gamma, lam1):
    """rho(i,j) = sum_{a,b} l0(a)^2 l1(b)^2 G(a,i,b) conj(G(a,j,b))."""
    w = gamma * lam0[:, None, None] * lam1[None, None, :]
    return np.einsum("aib,ajb->ij", w, w.conj())


def one_site_expval(gammas, lambdas, op):
    """<O_s> = Tr(O rho_s) for every site, rho_s(i,j) = psi_i conj(psi_j)."""
    return np.array([np.einsum("ij,ji->", op, single_site_rho(lambdas[s], gammas[s], lambdas[s + 1])).real
                     for s in range(len(gammas))])


def theta(lam0, g1, lam1, g2, lam2):
    """Theta(a,i,j,b) = l0(a) G1(a,i,g) l1(g) G2(g,j,b) l2(b)."""
    return np.einsum("a,aig,g,gjb,b->aijb", lam0, g1, lam1, g2, lam2, optimize=True)


def two_site_rho(lam0, g1, lam1, g2, lam2):
    """rho2[(k,l),(i,j)] = sum_{a,b} Theta(a,k,l,b) conj(Theta(a,i,j,b)); rows/cols in the
    gates' (i-1)*d+j order."""
    t = theta(lam0, g1, lam1, g2, lam2)
    chi, d, _, _ = t.shape
    m = t.transpose(1, 2, 0, 3).reshape(d * d, chi * chi)
    return m @ m.conj().T


def bond_energy(gammas, lambdas, H):
    """<H(i)> for every bond i = 1..L-1 (list index i-1)."""
    out = []
    for i in range(len(gammas) - 1):
        rho = two_site_rho(lambdas[i], gammas[i], lambdas[i + 1], gammas[i + 1], lambdas[i + 2])
        out.append(np.einsum("ij,ji->", H[i], rho).real)
    return np.array(out)


def inner_product(gL, lL, gR, lR):
    """<psi_L|psi_R> as InnerProduct computes it: transfer matrices of A_s = Gamma_s
    Lambda_{s+1}, started from left index 1 of site 1 and closed on right index 1 of
    site L, without the edge Lambdas themselves (they are e_1 for open chains)."""
    chi = gL[0].shape[0]
    E = np.zeros((chi, chi), complex)
    E[0, 0] = 1.0
    e1 = np.zeros(chi)
    e1[0] = 1.0
    for s in range(len(gL)):
        last = s == len(gL) - 1
        aL = gL[s] * (e1 if last else lL[s + 1])[None, None, :]
        aR = gR[s] * (e1 if last else lR[s + 1])[None, None, :]
        E = np.einsum("ab,aic,bid->cd", E, aL.conj(), aR, optimize=True)
    return E[0, 0]


def chain_entropy(lambdas, d):
    """ChainEntropy(link) for every link: -sum_{lambda != 0} lambda^2 ln|lambda^2| / ln(d)
    (observables_module.f90:1583-1602; the reference divides by LOG(localSize))."""
    out = []
    for l in lambdas:
        p = l[l != 0] ** 2
        out.append(float(-(p * np.log(np.abs(p))).sum() / np.log(d)))
    return np.array(out)


def state_vector(gammas, lambdas):
    """Dense state of a small open chain in Vidal form (test helper): the sum over
    Schmidt indices of Lambda(1) Gamma(1) Lambda(2) ... Gamma(L) Lambda(L+1),
    closed on the first index of the edge Lambdas (e_1 there).  Local index of
    site 1 is the slowest; d**L entries."""
    chi = gammas[0].shape[0]
    r = np.asarray(lambdas[0], dtype=complex)[None, :]
    for s, g in enumerate(gammas):
        r = np.einsum("pa,aib,b->pib", r, g, lambdas[s + 1]).reshape(-1, chi)
    return r[:, 0].copy()
