"""Gauge-invariant checks on Vidal states (test infrastructure only).

numpy restatements of the reference's observables (VidalCore_v_2.0/observables_module.f90):

* :func:`single_site_rho`  -- FormSingleSiteRho (:95-117)
* :func:`one_site_expval`  -- OneSiteExpVal via Tr(rho O) (:134-254)
* :func:`two_site_rho`     -- ThetaKernal + TwoSiteRho for neighbouring sites (:704-835)
* :func:`bond_energy`      -- the per-bond term of TotalEnergy (:1432-1466)
* :func:`inner_product`    -- InnerProduct (:1031-1089)
* :func:`chain_entropy`    -- von Neumann entropy of each Lambda (ChainEntropy, :1583)

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
    """<psi_L|psi_R> by left-to-right transfer matrices of A_s = Gamma_s Lambda_{s+1}."""
    E = np.outer(lL[0], lR[0]).astype(complex)
    for s in range(len(gL)):
        aL = gL[s] * lL[s + 1][None, None, :]
        aR = gR[s] * lR[s + 1][None, None, :]
        E = np.einsum("ab,aic,bid->cd", E, aL.conj(), aR, optimize=True)
    return E.sum()


def chain_entropy(lambdas):
    out = []
    for l in lambdas:
        p = l[l > 0] ** 2
        out.append(float(-(p * np.log(p)).sum()))
    return np.array(out)
