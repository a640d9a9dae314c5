"""Host-side producers of the hot path's inputs: bond Hamiltonians, gates, initial states.

These are not on the GPU path (they build d^2 x d^2 matrices once per run), but
a user switching from the reference needs them to feed ``TrotterStep``.  Each
builder restates a reference routine (paths relative to the OpenTEBD-extended
tree); ``tensorProd(A, B)`` of TEBDtools_module.f90:230-246 is ``np.kron(A, B)``
(row (i-1)*dB+j, column (k-1)*dB+l), which is also the gates' index order.
"""
from __future__ import annotations

import numpy as np


# ---------------------------------------------------------------------------
# operators
# ---------------------------------------------------------------------------
def bose_ops(d):
    """CreateFieldOps (bose_hubbard_module.f90:50-111): a(j,j+1)=sqrt(j), one, t_op."""
    a = np.zeros((d, d))
    for j in range(1, d):
        a[j - 1, j] = np.sqrt(float(j))
    one = np.eye(d)
    t = np.kron(a.T, a)
    t = t + t.T
    return a, one, t


def spin_ops(spin):
    """CreateHeisenbergOps (heisenberg_module.f90:52-118) for spin S, d = 2S+1."""
    d = int(round(2 * spin + 1))
    sz = np.zeros((d, d))
    sx = np.zeros((d, d))
    sy = np.zeros((d, d), dtype=complex)
    for i in range(1, d + 1):
        m = spin - (i - 1)
        sz[i - 1, i - 1] = m
        if i != d:
            v = np.sqrt((spin + m) * (spin + 1.0 - m))
            sx[i - 1, i] = v
            sy[i - 1, i] = v
    sx = 0.5 * (sx + sx.T)
    sy = 1j * 0.5 * (sy.T - sy)
    return sx, sy, sz, np.eye(d)


# ---------------------------------------------------------------------------
# bond Hamiltonians H(i), i = 1..L-1 (index i-1 in the returned list)
# ---------------------------------------------------------------------------
def heisenberg(L, Jx, Jy, Jz, spin=0.5, mag_field=None):
    """HamiltonianHeisenberg (heisenberg_module.f90:143-174), open boundaries."""
    sx, sy, sz, one = spin_ops(spin)
    H = []
    for _ in range(L - 1):
        h = Jx * np.kron(sx, sx) + Jy * np.kron(sy, sy) + Jz * np.kron(sz, sz)
        if mag_field is not None:
            h = h + mag_field * 0.5 * (np.kron(sz, one) + np.kron(one, sz))  # HamiOneSite
        H.append(np.asarray(h, dtype=complex))
    if mag_field is not None:
        H[0] = H[0] + mag_field * 0.5 * np.kron(sz, one)       # HamiLeft
        H[-1] = H[-1] + mag_field * 0.5 * np.kron(one, sz)     # HamiRight
    return H


def spin1_xxz_anisotropy(L, J, delta, D):
    """Spin-1 XXZ chain plus single-ion anisotropy sum_i D_i Sz_i^2.

    The coupling part is HamiltonianHeisenberg with spin=1 (Jx=Jy=J, Jz=J*delta).
    The reference has no D*Sz^2 builder; the one-site term is split over the two
    bonds of a site as HamiOneSite/HamiLeft/HamiRight do
    (Hamiltonian_tools_module.f90:816-886): 1/2 to each bond, the edge halves
    added to the first and last bond."""
    sx, sy, sz, one = spin_ops(1.0)
    sz2 = sz @ sz
    H = []
    for i in range(L - 1):
        h = J * (np.kron(sx, sx) + np.kron(sy, sy).real) + J * delta * np.kron(sz, sz)
        h = h + 0.5 * D[i] * np.kron(sz2, one) + 0.5 * D[i + 1] * np.kron(one, sz2)
        H.append(np.asarray(h, dtype=complex))
    H[0] = H[0] + 0.5 * D[0] * np.kron(sz2, one)
    H[-1] = H[-1] + 0.5 * D[L - 1] * np.kron(one, sz2)
    return H


def bose_hubbard(L, d, J, U, mu=0.0, V=0.0):
    """HamiltonianBoseHubbardScalar (scalar U) or ...UVector (per-site U array):
    bose_hubbard_module.f90:131-201 and :203-273, open boundaries, no extPot.
    The UVector edge term uses U0(systemSize-1) for the last site, exactly as the
    reference writes it (:254-256)."""
    a, one, t = bose_ops(d)
    n = a.T @ a
    nn = n @ n
    Uv = np.full(L, float(U)) if np.isscalar(U) else np.asarray(U, dtype=float)
    H = []
    for i in range(L - 1):
        h = np.zeros((d * d, d * d))
        h = h + 0.25 * Uv[i] * np.kron(nn, one) - 0.25 * Uv[i] * np.kron(n, one)
        h = h + 0.25 * Uv[i + 1] * np.kron(one, nn) - 0.25 * Uv[i + 1] * np.kron(one, n)
        h = h - 0.5 * mu * np.kron(n, one)
        h = h - 0.5 * mu * np.kron(one, n)
        h = h - J * t
        h = h + V * np.kron(n, n)
        H.append(h)
    H[0] = H[0] + 0.25 * Uv[0] * np.kron(nn, one) - 0.25 * Uv[0] * np.kron(n, one)
    H[0] = H[0] - 0.5 * mu * np.kron(n, one)
    ulast = Uv[L - 2] if not np.isscalar(U) else Uv[L - 1]
    H[-1] = H[-1] + 0.25 * ulast * np.kron(one, nn) - 0.25 * ulast * np.kron(one, n)
    H[-1] = H[-1] - 0.5 * mu * np.kron(one, n)
    return [np.asarray(h, dtype=complex) for h in H]


# ---------------------------------------------------------------------------
# propagators
# ---------------------------------------------------------------------------
def fermi_ops():
    """Spin-1/2 fermion operators of CreateFermiSops (fermi_hubbard_module.f90:100-245)
    on the local Fock basis |n_up, n_down> in onsiteStateListIdof's order by total
    number: (0,0), (1,0), (0,1), (1,1).  a_k carries the Jordan-Wigner phase
    (-1)^(n of the components before k); returns a_up, a_down, one, ntot,
    fermiPhase and the two-site tunnelling operator ttot."""
    states = [(0, 0), (1, 0), (0, 1), (1, 1)]
    d = len(states)
    idx = {s: i for i, s in enumerate(states)}
    a = []
    for k in range(2):
        m = np.zeros((d, d))
        for j, sj in enumerate(states):
            if sj[k] == 0:
                continue
            nj = list(sj)
            nj[k] -= 1
            m[idx[tuple(nj)], j] = (-1.0) ** sum(sj[:k])
        a.append(m)
    one = np.eye(d)
    ntot = sum(x.T @ x for x in a)
    fphase = np.diag((-1.0) ** np.diag(ntot))
    ttot = sum(np.kron(x, one).T @ np.kron(fphase, x) + np.kron(fphase, x).T @ np.kron(x, one) for x in a)
    return a[0], a[1], one, ntot, fphase, ttot


def fermi_hubbard(L, J, U, mu=0.0):
    """HamiltonianHubbard (fermi_hubbard_module.f90:289-356), spin 1/2, open
    boundaries, no extPot/V0: -mu/2 (n x 1 + 1 x n) - J ttot + U/2 [(n_up - 1/2)
    (n_dn - 1/2) x 1 + 1 x (...)] per bond, the edge bonds carrying the missing
    halves of the first and last site."""
    au, ad, one, n, _, ttot = fermi_ops()
    hu = (au.T @ au - 0.5 * one) @ (ad.T @ ad - 0.5 * one)
    H = []
    for _ in range(L - 1):
        H.append(-0.5 * mu * (np.kron(n, one) + np.kron(one, n)) - J * ttot
                 + 0.5 * U * (np.kron(hu, one) + np.kron(one, hu)))
    H[0] = H[0] - 0.5 * mu * np.kron(n, one) + 0.5 * U * np.kron(hu, one)
    H[L - 2] = H[L - 2] - 0.5 * mu * np.kron(one, n) + 0.5 * U * np.kron(one, hu)
    return H


def matrix_exponential(H, t):
    """matrix_exponential_c (TEBDtools_module.f90:176-222): exp(-i t H) through the
    eigendecomposition of the Hermitian H (ZHEEV there, numpy eigh here)."""
    w, v = np.linalg.eigh(H)
    return (v * np.exp(-1j * t * w)) @ v.conj().T


def forest_ruth_theta():
    """FRtheta = 1/(2 - 2**(1.0/3.0)) with the single-precision exponent literal
    of TEBDtools_module.f90:1135."""
    return 1.0 / (2.0 - 2.0 ** float(np.float32(1.0) / np.float32(3.0)))


def construct_propagators(H, dt, order=2, boundary="O"):
    """NEWConstructPropagators (TEBDtools_module.f90:1079-1196).  Returns Udt as a
    list indexed like the reference's Udt(1..).  BoundaryCond='O': H holds the L-1
    bond terms; 'P': L terms, H(L) the edge bond (site 1 left, site L right)."""
    if boundary == "P":
        return _construct_propagators_pbc(H, dt, order)
    if boundary != "O":
        raise ValueError("boundary must be 'O' or 'P'")
    L1 = len(H)  # L - 1 bonds
    if order == 2:
        return [matrix_exponential(H[i], (0.5 if (i + 1) % 2 == 1 else 1.0) * dt) for i in range(L1)]
    if order != 5:
        raise ValueError("order must be 2 or 5")
    th = forest_ruth_theta()
    U = [None] * (2 * (L1 - 1) + 2)
    for i in range(1, L1 + 1):
        if i % 2 == 1:
            U[2 * (i - 1)] = matrix_exponential(H[i - 1], 0.5 * th * dt)
            U[2 * (i - 1) + 1] = matrix_exponential(H[i - 1], 0.5 * (1.0 - th) * dt)
        else:
            U[2 * (i - 1)] = matrix_exponential(H[i - 1], th * dt)
            U[2 * (i - 1) + 1] = matrix_exponential(H[i - 1], (1.0 - 2.0 * th) * dt)
    return U


def _construct_propagators_pbc(H, dt, order):
    """BoundaryCond='P' branches of NEWConstructPropagators (TEBDtools_module.f90:
    1100-1127 for order 2, 1149-1190 for order 5).  Even L: the edge term commutes
    with the even bonds, so both take full steps; odd L: the even bonds take half
    steps around the edge (order 2), or the nested Forest-Ruth fractions (order 5)."""
    L = len(H)
    ex = matrix_exponential
    if order == 2:
        even = 1.0 if L % 2 == 0 else 0.5
        U = [ex(H[i - 1], (0.5 if i % 2 == 1 else even) * dt) for i in range(1, L)]
        return U + [ex(H[L - 1], dt)]
    if order != 5:
        raise ValueError("order must be 2 or 5")
    th = forest_ruth_theta()
    if L % 2 == 0:
        U = [None] * (2 * L)
        for i in range(1, L):
            f = (0.5 * th, 0.5 * (1.0 - th)) if i % 2 == 1 else (th, 1.0 - 2.0 * th)
            U[2 * (i - 1)] = ex(H[i - 1], f[0] * dt)
            U[2 * (i - 1) + 1] = ex(H[i - 1], f[1] * dt)
        U[2 * (L - 1)] = ex(H[L - 1], th * dt)
        U[2 * (L - 1) + 1] = ex(H[L - 1], (1.0 - 2.0 * th) * dt)
        return U
    U = [None] * (3 * L)
    for i in range(1, L, 2):
        U[3 * (i - 1)] = ex(H[i - 1], 0.5 * th * dt)
        U[3 * (i - 1) + 1] = ex(H[i - 1], 0.5 * (1.0 - th) * dt)
    for i in range(2, L, 2):
        fr = (0.5 * th * th, 0.5 * (1.0 - th) * th, 0.5 * (1.0 - 2.0 * th) * th,
              0.5 * (1.0 - th) * (1.0 - 2.0 * th))
        for v in range(4):
            U[2 + 3 * (i - 2) + v] = ex(H[i - 1], fr[v] * dt)
    U[3 * (L - 1)] = ex(H[L - 1], th * th * dt)
    U[3 * (L - 1) + 1] = ex(H[L - 1], (1.0 - 2.0 * th) * th * dt)
    U[3 * (L - 1) + 2] = ex(H[L - 1], (1.0 - 2.0 * th) * (1.0 - 2.0 * th) * dt)
    return U


# ---------------------------------------------------------------------------
# initial states
# ---------------------------------------------------------------------------
def product_state(carray, chi):
    """ProductStateMPD (Hamiltonian_tools_module.f90:89-121): carray is (d, L)."""
    d, L = carray.shape
    gam = [np.zeros((chi, d, chi), dtype=complex, order="F") for _ in range(L)]
    lam = [np.zeros(chi) for _ in range(L + 1)]
    for i in range(L):
        gam[i][0, :, 0] = carray[:, i]
        lam[i][0] = 1.0
    lam[L][0] = 1.0
    return gam, lam


def product_state_labels(carray, chi, tot_num, conserv=None):
    """ProductStateLabels (Hamiltonian_tools_module.f90:124-178) for a product state
    of definite total number.  Plain form: the number of site i is j-1 of the LAST
    nonzero carray(j, i); with internal degrees of freedom (``conserv`` =
    Conserv%vi) it is Conserv(j) of the FIRST nonzero component, as there.
    Returns LabelLeft, LabelRight (10000 = unused)."""
    d, L = carray.shape
    ll = [np.full(chi, 10000, dtype=np.int32) for _ in range(L + 1)]
    lr = [np.full(chi, 10000, dtype=np.int32) for _ in range(L + 1)]
    ll[0][0] = 0
    for i in range(L):
        nz = [j for j in range(d) if abs(carray[j, i]) != 0.0]
        if not nz:
            raise ValueError("site %d has no nonzero component" % (i + 1))
        n = conserv[nz[0]] if conserv is not None else nz[-1]
        ll[i + 1][0] = ll[i][0] + n
    for i in range(L + 1):
        lr[i][0] = tot_num - ll[i][0]
    return ll, lr


def initial_set_nc(L, d, chi, tot_num):
    """InitialSetNC (Hamiltonian_tools_module.f90:369-523), intDegFree absent.
    Returns gammas, lambdas, LabelLeft, LabelRight (labels 10000 = unused)."""
    gam = [np.zeros((chi, d, chi), dtype=complex, order="F") for _ in range(L)]
    lam = [np.zeros(chi) for _ in range(L + 1)]
    ll = [np.full(chi, 10000, dtype=np.int32) for _ in range(L + 1)]
    lr = [np.full(chi, 10000, dtype=np.int32) for _ in range(L + 1)]
    if tot_num == 0:
        for i in range(L + 1):
            ll[i][0] = 0
            lr[i][0] = 0
            lam[i][0] = 1.0
        for i in range(L):
            gam[i][0, 0, 0] = 1.0
        return gam, lam, ll, lr
    if (L - tot_num % L) % 2 == 0 or tot_num % L == 0:
        hole = 0 if tot_num % L == 0 else (L - tot_num % L) // 2
    else:
        hole = (L - tot_num % L + 1) // 2
    tops = (tot_num - 1) % L + 1
    center = int(np.floor(tot_num / L - 1e-8)) + 1
    vals = [0] * (L + 2)  # 1-based link
    for i in range(1, hole + 2):
        vals[i] = 0 if i == 1 else vals[i - 1] + center - 1
    for i in range(hole + 2, hole + tops + 2):
        vals[i] = vals[i - 1] + center
    for i in range(hole + tops + 2, L + 2):
        vals[i] = vals[i - 1] + center - 1
    for i in range(1, L + 2):
        ll[i - 1][0] = vals[i]
        lr[i - 1][0] = tot_num - vals[i]
        lam[i - 1][0] = 1.0
    for i in range(1, hole + 1):
        gam[i - 1][0, center - 1, 0] = 1.0
    for i in range(hole + 1, hole + tops + 1):
        gam[i - 1][0, center, 0] = 1.0
    for i in range(hole + tops + 1, L + 1):
        gam[i - 1][0, center - 1, 0] = 1.0
    return gam, lam, ll, lr


def perturbed_product_state(carray, chi, amplitude, seed):
    """Product state plus a seeded complex Gaussian perturbation of `amplitude`
    on every Gamma entry; each site's physical vector is renormalised.  With
    Lambda = e_1 only Gamma(1,:,1) enters the state, so the result is a valid
    (canonical) product state; the other entries are overwritten by the first
    update of each bond."""
    d, L = carray.shape
    rng = np.random.default_rng(seed)
    gam, lam = product_state(carray, chi)
    for i in range(L):
        noise = rng.standard_normal((chi, d, chi)) + 1j * rng.standard_normal((chi, d, chi))
        g = gam[i] + amplitude * noise
        g[0, :, 0] /= np.linalg.norm(g[0, :, 0])
        gam[i] = np.asfortranarray(g)
    return gam, lam
