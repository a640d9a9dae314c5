"""Python side of the CPU oracle (test infrastructure only).

Loads ``oracle/build/libtebd_oracle.so`` (built from ``tebd_oracle.c`` by
:func:`build`) and hands it the host LAPACK ``zgesvd`` taken from
``scipy.linalg.cython_lapack``.  Only tests, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py`` may use this module; the product path never does.

Every function mirrors one reference routine (paths relative to the
OpenTEBD-extended tree):

* :func:`two_site_op`     -- ``TwoSiteOp_c``/``TwoSiteOp_r``
  (VidalCore_v_2.0/local_operations_module.f90:430-494)
* :func:`two_site_op_nc`  -- ``TwoSiteOpNC_c``/``_r``, with or without internal
  degrees of freedom (local_operations_module.f90:748-1964; ``conserv`` stands
  for the optional ``intDegFree`` argument plus the global ``Conserv%vi``)
* :func:`trotter_step`, :func:`trotter_step_nc` -- ``TrotterStep2ndOrder`` /
  ``TrotterStep5thOrder`` and NC twins (propagation_module.f90:82-252, 956-1018)
* :func:`trotter_step_pbc` -- ``TrotterStep2ndOrderPBC`` / ``TrotterStep5thOrderPBC``
  (propagation_module.f90:116-198, 254-614)

Parity unpinned: the reference is Fortran, no Fortran compiler is available
where this oracle is built, and the reference holds no tests or golden vectors.
The oracle is pinned by analytic known answers instead (tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "build")
LIB_PATH = os.path.join(BUILD_DIR, "libtebd_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the C restatement with gcc (portable flags: no -march=native)."""
    src = os.path.join(HERE, "tebd_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _capsule_pointer(capsule) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def lib():
    """Load (building if needed) the oracle library with LAPACK attached."""
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = ctypes.CDLL(LIB_PATH)
    from scipy.linalg import cython_lapack

    L.oracle_set_zgesvd.argtypes = [ctypes.c_void_p]
    L.oracle_set_zgesvd(_capsule_pointer(cython_lapack.__pyx_capi__["zgesvd"]))
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    L.oracle_two_site_op.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp]
    L.oracle_two_site_op_nc.argtypes = [ctypes.c_int] * 4 + [dp] * 7 + [ip] * 4 + [dp, dp, ip]
    L.oracle_trotter_step.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(dp)] * 3 + [dp]
    L.oracle_swapping.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp]
    L.oracle_canonical_form.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp]
    L.oracle_trotter_step_pbc.argtypes = [ctypes.c_int] * 3 + [ctypes.POINTER(dp)] * 3 + [dp]
    L.oracle_trotter_step_pbc5.argtypes = [ctypes.c_int] * 3 + [ctypes.POINTER(dp)] * 3 + [dp]
    L.oracle_set_conserv.argtypes = [ctypes.c_int, ip]
    L.oracle_swapping_nc.argtypes = [ctypes.c_int] * 4 + [dp] * 5 + [ip] * 4 + [dp]
    L.oracle_trotter_step_pbc_nc.argtypes = (
        [ctypes.c_int] * 6 + [ctypes.POINTER(dp)] * 2 + [ctypes.POINTER(ip)] * 2 + [ctypes.POINTER(dp), dp]
    )
    L.oracle_trotter_step_nc.argtypes = (
        [ctypes.c_int] * 6 + [ctypes.POINTER(dp)] * 2 + [ctypes.POINTER(ip)] * 2 + [ctypes.POINTER(dp), dp]
    )
    _lib = L
    return L


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _fcomplex(a, shape):
    a = np.asarray(a, dtype=np.complex128)
    assert a.shape == shape, (a.shape, shape)
    return np.asfortranarray(a)


def _check(st, what):
    if st != 0:
        raise RuntimeError("%s failed with oracle status %d" % (what, st))


def two_site_op(gamma1, gamma2, lam0, lam1, lam2, op2):
    """One dense bond update.  Arrays are numpy (chi,d,chi) complex / (chi,) real,
    ``op2`` is (d^2, d^2) real or complex.  Returns
    ``(gamma1', gamma2', lam1', truncerr, s_all)`` without touching the inputs."""
    chi, d, _ = gamma1.shape
    g1 = _fcomplex(gamma1, (chi, d, chi)).copy(order="F")
    g2 = _fcomplex(gamma2, (chi, d, chi)).copy(order="F")
    l0 = np.ascontiguousarray(lam0, dtype=np.float64)
    l1 = np.array(lam1, dtype=np.float64)
    l2 = np.ascontiguousarray(lam2, dtype=np.float64)
    op2 = np.asarray(op2)
    op_c = op_r = None
    if np.iscomplexobj(op2):
        op_c = np.asfortranarray(op2, dtype=np.complex128)
    else:
        op_r = np.asfortranarray(op2, dtype=np.float64)
    te = np.zeros(1)
    s = np.zeros(chi * d)
    st = lib().oracle_two_site_op(chi, d, _dptr(g1), _dptr(g2), _dptr(l0), _dptr(l1), _dptr(l2),
                                  _dptr(op_c), _dptr(op_r), _dptr(te), _dptr(s))
    _check(st, "oracle_two_site_op")
    return g1, g2, l1, float(te[0]), s


def _set_conserv(d, conserv):
    """Select the intDegFree branches with local numbers ``conserv`` (Conserv%vi),
    or the plain ones (local number i-1) for None."""
    if conserv is None:
        _check(lib().oracle_set_conserv(d, None), "oracle_set_conserv")
        return
    c = np.ascontiguousarray(conserv, dtype=np.int32)
    assert c.shape == (d,)
    _check(lib().oracle_set_conserv(d, _iptr(c)), "oracle_set_conserv")


def two_site_op_nc(gamma1, gamma2, lam0, lam1, lam2, op2, ll0, ll1, lr1, lr2, tot_num, max_filling,
                   conserv=None):
    """One number-conserving bond update; ``conserv`` (d local particle numbers)
    selects the intDegFree form.  Returns
    ``(gamma1', gamma2', lam1', ll1', lr1', truncerr, ssflat)``."""
    chi, d, _ = gamma1.shape
    _set_conserv(d, conserv)
    g1 = _fcomplex(gamma1, (chi, d, chi)).copy(order="F")
    g2 = _fcomplex(gamma2, (chi, d, chi)).copy(order="F")
    l0 = np.ascontiguousarray(lam0, dtype=np.float64)
    l1 = np.array(lam1, dtype=np.float64)
    l2 = np.ascontiguousarray(lam2, dtype=np.float64)
    a_ll0 = np.ascontiguousarray(ll0, dtype=np.int32)
    a_ll1 = np.array(ll1, dtype=np.int32)
    a_lr1 = np.array(lr1, dtype=np.int32)
    a_lr2 = np.ascontiguousarray(lr2, dtype=np.int32)
    op2 = np.asarray(op2)
    op_c = op_r = None
    if np.iscomplexobj(op2):
        op_c = np.asfortranarray(op2, dtype=np.complex128)
    else:
        op_r = np.asfortranarray(op2, dtype=np.float64)
    te = np.zeros(1)
    s = np.zeros(chi * d)
    sz = np.zeros(1, dtype=np.int32)
    st = lib().oracle_two_site_op_nc(chi, d, tot_num, max_filling, _dptr(g1), _dptr(g2), _dptr(l0),
                                     _dptr(l1), _dptr(l2), _dptr(op_c), _dptr(op_r), _iptr(a_ll0),
                                     _iptr(a_ll1), _iptr(a_lr1), _iptr(a_lr2), _dptr(te), _dptr(s),
                                     _iptr(sz))
    _check(st, "oracle_two_site_op_nc")
    return g1, g2, l1, a_ll1, a_lr1, float(te[0]), s[: int(sz[0])].copy()


def _ptr_array(arrs, ctype):
    P = ctypes.POINTER(ctype)
    return (P * len(arrs))(*[a.ctypes.data_as(P) for a in arrs])


def trotter_step(gammas, lambdas, gates, order=2):
    """One open-boundary Trotter step on lists of numpy arrays, updated in place.
    ``gammas[s]`` (chi,d,chi) Fortran-ordered complex, ``lambdas[l]`` (chi,),
    ``gates[g]`` (d^2,d^2) complex.  Returns the summed truncation error."""
    L = len(gammas)
    chi, d, _ = gammas[0].shape
    for g in gammas:
        assert g.flags.f_contiguous and g.dtype == np.complex128
    gts = [np.asfortranarray(g, dtype=np.complex128) for g in gates]
    te = np.zeros(1)
    st = lib().oracle_trotter_step(L, chi, d, order, _ptr_array(gammas, ctypes.c_double),
                                   _ptr_array(lambdas, ctypes.c_double),
                                   _ptr_array(gts, ctypes.c_double), _dptr(te))
    _check(st, "oracle_trotter_step")
    return float(te[0])


def swapping(gamma1, gamma2, lam0, lam1, lam2):
    """Swapping on one bond (unnormalised Theta with its physical indices exchanged).
    Returns ``(gamma1', gamma2', lam1', truncerr)`` without touching the inputs."""
    chi, d, _ = gamma1.shape
    g1 = _fcomplex(gamma1, (chi, d, chi)).copy(order="F")
    g2 = _fcomplex(gamma2, (chi, d, chi)).copy(order="F")
    l0 = np.ascontiguousarray(lam0, dtype=np.float64)
    l1 = np.array(lam1, dtype=np.float64)
    l2 = np.ascontiguousarray(lam2, dtype=np.float64)
    te = np.zeros(1)
    st = lib().oracle_swapping(chi, d, _dptr(g1), _dptr(g2), _dptr(l0), _dptr(l1), _dptr(l2), _dptr(te))
    _check(st, "oracle_swapping")
    return g1, g2, l1, float(te[0])


def canonical_form(lam0, gamma1, lam1, gamma2, lam2):
    """CanonicalForm on one bond; returns ``(gamma1', lam1', gamma2')`` (inputs untouched)."""
    chi, d, _ = gamma1.shape
    g1 = _fcomplex(gamma1, (chi, d, chi)).copy(order="F")
    g2 = _fcomplex(gamma2, (chi, d, chi)).copy(order="F")
    l0 = np.ascontiguousarray(lam0, dtype=np.float64)
    l1 = np.array(lam1, dtype=np.float64)
    l2 = np.ascontiguousarray(lam2, dtype=np.float64)
    st = lib().oracle_canonical_form(chi, d, _dptr(l0), _dptr(g1), _dptr(l1), _dptr(g2), _dptr(l2))
    _check(st, "oracle_canonical_form")
    return g1, l1, g2


def canonical_form_all(gammas, lambdas):
    """CanonicalFormAll in place: CanonicalForm on links 1..L-1, then L-1..1."""
    L = len(gammas)
    for k in list(range(1, L)) + list(range(L - 1, 0, -1)):
        gammas[k - 1], lambdas[k], gammas[k] = canonical_form(lambdas[k - 1], gammas[k - 1], lambdas[k],
                                                               gammas[k], lambdas[k + 1])


def trotter_step_pbc(gammas, lambdas, gates, order=2):
    """TrotterStep2ndOrderPBC / TrotterStep5thOrderPBC in place; gates[g-1] = Udt(g)
    in NEWConstructPropagators' periodic layout (L gates for order 2, Udt(L) the
    edge bond; 3L for order 5 and odd L, 2L for even L)."""
    L = len(gammas)
    chi, d, _ = gammas[0].shape
    need = L if order == 2 else (3 * L if L % 2 == 1 else 2 * L)
    if order not in (2, 5) or len(gates) < need:
        raise ValueError("periodic step: order 2 or 5 with %d gates" % need)
    gts = [np.asfortranarray(g, dtype=np.complex128) for g in gates]
    te = np.zeros(1)
    fn = lib().oracle_trotter_step_pbc if order == 2 else lib().oracle_trotter_step_pbc5
    st = fn(L, chi, d, _ptr_array(gammas, ctypes.c_double), _ptr_array(lambdas, ctypes.c_double),
            _ptr_array(gts, ctypes.c_double), _dptr(te))
    _check(st, "oracle_trotter_step_pbc")
    return float(te[0])


def swapping_nc(gamma1, gamma2, lam0, lam1, lam2, ll0, ll1, lr1, lr2, tot_num, max_filling, conserv=None):
    """SwappingNC on one bond.  Returns ``(gamma1', gamma2', lam1', ll1', lr1', truncerr)``."""
    chi, d, _ = gamma1.shape
    _set_conserv(d, conserv)
    g1 = _fcomplex(gamma1, (chi, d, chi)).copy(order="F")
    g2 = _fcomplex(gamma2, (chi, d, chi)).copy(order="F")
    l0 = np.ascontiguousarray(lam0, dtype=np.float64)
    l1 = np.array(lam1, dtype=np.float64)
    l2 = np.ascontiguousarray(lam2, dtype=np.float64)
    a_ll0 = np.ascontiguousarray(ll0, dtype=np.int32)
    a_ll1 = np.array(ll1, dtype=np.int32)
    a_lr1 = np.array(lr1, dtype=np.int32)
    a_lr2 = np.ascontiguousarray(lr2, dtype=np.int32)
    te = np.zeros(1)
    st = lib().oracle_swapping_nc(chi, d, tot_num, max_filling, _dptr(g1), _dptr(g2), _dptr(l0), _dptr(l1),
                                  _dptr(l2), _iptr(a_ll0), _iptr(a_ll1), _iptr(a_lr1), _iptr(a_lr2), _dptr(te))
    _check(st, "oracle_swapping_nc")
    return g1, g2, l1, a_ll1, a_lr1, float(te[0])


def trotter_step_pbc_nc(gammas, lambdas, label_left, label_right, gates, tot_num, max_filling, order=2,
                        conserv=None):
    """TrotterStep2ndOrderPBCNC / 5thOrderPBCNC in place (gate layout as
    :func:`trotter_step_pbc`)."""
    L = len(gammas)
    chi, d, _ = gammas[0].shape
    need = L if order == 2 else (3 * L if L % 2 == 1 else 2 * L)
    if order not in (2, 5) or len(gates) < need:
        raise ValueError("periodic step: order 2 or 5 with %d gates" % need)
    _set_conserv(d, conserv)
    gts = [np.asfortranarray(g, dtype=np.complex128) for g in gates]
    te = np.zeros(1)
    st = lib().oracle_trotter_step_pbc_nc(L, chi, d, tot_num, max_filling, order,
                                          _ptr_array(gammas, ctypes.c_double),
                                          _ptr_array(lambdas, ctypes.c_double),
                                          _ptr_array(label_left, ctypes.c_int),
                                          _ptr_array(label_right, ctypes.c_int),
                                          _ptr_array(gts, ctypes.c_double), _dptr(te))
    _check(st, "oracle_trotter_step_pbc_nc")
    return float(te[0])


def trotter_step_nc(gammas, lambdas, label_left, label_right, gates, tot_num, max_filling, order=2,
                    conserv=None):
    """Number-conserving Trotter step; all lists updated in place.  ``conserv``
    selects the intDegFree form."""
    L = len(gammas)
    chi, d, _ = gammas[0].shape
    _set_conserv(d, conserv)
    gts = [np.asfortranarray(g, dtype=np.complex128) for g in gates]
    te = np.zeros(1)
    st = lib().oracle_trotter_step_nc(L, chi, d, tot_num, max_filling, order,
                                      _ptr_array(gammas, ctypes.c_double),
                                      _ptr_array(lambdas, ctypes.c_double),
                                      _ptr_array(label_left, ctypes.c_int),
                                      _ptr_array(label_right, ctypes.c_int),
                                      _ptr_array(gts, ctypes.c_double), _dptr(te))
    _check(st, "oracle_trotter_step_nc")
    return float(te[0])


if __name__ == "__main__":  # pragma: no cover - manual build entry
    print(build(force="--force" in sys.argv))
