"""Host-side mirror of the reference's TEBD interface over the sm_103a C ABI.

The Fortran reference exposes (paths relative to the OpenTEBD-extended tree):

* ``TwoSiteOp(link, Op2, Gammas, Lambdas, truncerr)``
  (VidalCore_v_2.0/local_operations_module.f90:46-48, 430-494)
* ``TwoSiteOpNC(link, Op2, Gammas, Lambdas, LabelLeft, LabelRight, truncerr)``
  (local_operations_module.f90:54-56, 1723-1964)
* ``TrotterStep(Udt, Gammas, Lambdas, totalTruncerr)`` and ``TrotterStepNC``
  (VidalCore_v_2.0/propagation_module.f90:42-114, 200-252, 890-1018)

Here the chain lives in device memory owned by a :class:`Chain` (the handle of
``include/tebd_capi.h``); Gammas/Lambdas/labels move only on ``set_*``/``get_*``.
The module-level functions :func:`TwoSiteOp`, :func:`TwoSiteOpNC` and
:func:`TrotterStep` keep the reference's argument meaning (1-based links, gates
as (d^2, d^2) matrices with the right site's index fastest) and return the
truncation error the Fortran routines write to ``truncerr``.

There is no CPU fallback: if ``lib/libtebd_gb300.so`` is missing or no sm_103
device is present, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libtebd_gb300.so")

TEBD_OK = 0
TEBD_ERR_ARG = 1
TEBD_ERR_CUDA = 2
TEBD_ERR_OOM = 3
TEBD_ERR_SVD_NOCONV = 4
TEBD_ERR_NONFINITE = 5
TEBD_ERR_STATE = 6
TEBD_ERR_NC_BLOCKS = 7
MODE_DENSE = 0
MODE_NC = 1
SVD_FP64 = 0
SVD_JACOBI = 2
SVD_BIDIAG = 3
SVD_QRJ = 4
SVD_DF = 5
SVD_RSVD = 6
OPTS_VERSION = 1

ERROR_NAMES = {
    TEBD_ERR_ARG: "TEBD_ERR_ARG",
    TEBD_ERR_CUDA: "TEBD_ERR_CUDA",
    TEBD_ERR_OOM: "TEBD_ERR_OOM",
    TEBD_ERR_SVD_NOCONV: "TEBD_ERR_SVD_NOCONV",
    TEBD_ERR_NONFINITE: "TEBD_ERR_NONFINITE",
    TEBD_ERR_STATE: "TEBD_ERR_STATE",
    TEBD_ERR_NC_BLOCKS: "TEBD_ERR_NC_BLOCKS",
}

# every symbol include/tebd_capi.h declares
EXPORTED_SYMBOLS = (
    "tebd_default_opts", "tebd_create", "tebd_destroy", "tebd_set_gamma", "tebd_get_gamma",
    "tebd_set_lambda", "tebd_get_lambda", "tebd_set_labels", "tebd_get_labels",
    "tebd_two_site_op", "tebd_two_site_op_r", "tebd_two_site_op_nc", "tebd_two_site_op_nc_r",
    "tebd_apply_bonds", "tebd_trotter_step", "tebd_get_singular_values", "tebd_get_sweeps",
    "tebd_sync", "tebd_last_error", "tebd_kernel_launches", "tebd_set_profiling", "tebd_get_stats",
    "tebd_reset_stats", "tebd_measure_fp64_peak", "tebd_get_stream", "tebd_two_site_op_noalloc",
    "tebd_single_site_rho", "tebd_one_site_expval", "tebd_one_site_expval_r", "tebd_two_site_rho",
    "tebd_local_energy", "tebd_total_energy", "tebd_inner_product", "tebd_chain_entropy",
    "tebd_record_lambdas", "tebd_record_gammas", "tebd_record_labels", "tebd_read_gamma_lambda",
    "tebd_read_gamma_lambda_labels", "tebd_swapping", "tebd_trotter_step_pbc", "tebd_canonical_form_all_nc",
    "tebd_canonical_form", "tebd_canonical_form_all", "tebd_set_conserv", "tebd_set_rank_bound",
    "tebd_zgemm_tc", "tebd_set_theta_form", "tebd_set_rsvd",
    "tebd_mlp_create", "tebd_mlp_destroy", "tebd_mlp_param_count", "tebd_mlp_last_error", "tebd_mlp_get_params",
    "tebd_mlp_set_params", "tebd_mlp_forward", "tebd_mlp_loss_grad", "tebd_mlp_train", "tebd_set_rsvd_model",
    "tebd_autotune", "tebd_get_tuning", "tebd_clear_tuning",
)


class TebdError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "?"), code, msg))
        self.code = code


class Opts(ctypes.Structure):
    _fields_ = [
        ("version", ctypes.c_int),
        ("device", ctypes.c_int),
        ("tot_num", ctypes.c_int),
        ("max_filling", ctypes.c_int),
        ("svd_mode", ctypes.c_int),
        ("max_sweeps", ctypes.c_int),
        ("max_batch", ctypes.c_int),
        ("reserved", ctypes.c_int),
        ("jacobi_tol", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("updates", ctypes.c_longlong),
        ("kernel_launches", ctypes.c_longlong),
        ("jacobi_launches", ctypes.c_longlong),
        ("jacobi_sweeps", ctypes.c_longlong),
        ("jacobi_pairs", ctypes.c_longlong),
        ("jacobi_rotations", ctypes.c_longlong),
        ("jacobi_flops", ctypes.c_double),
        ("jacobi_bytes", ctypes.c_double),
        ("jacobi_ms", ctypes.c_double),
        ("batch_ms", ctypes.c_double),
        ("compact_rows", ctypes.c_longlong),
        ("compact_cols", ctypes.c_longlong),
        ("qr_flops", ctypes.c_double),
        ("qr_ms", ctypes.c_double),
        ("rank_sum", ctypes.c_longlong),
        ("bidiag_ms", ctypes.c_double),
        ("bidiag_updates", ctypes.c_longlong),
        ("gebrd_flops", ctypes.c_double),
        ("gebrd_ms", ctypes.c_double),
        ("gebrd_launches", ctypes.c_longlong),
        ("rsvd_updates", ctypes.c_longlong),
        ("rsvd_fallbacks", ctypes.c_longlong),
        ("rsvd_flops", ctypes.c_double),
        ("rsvd_worst_residual", ctypes.c_double),
        ("rsvd_skipped", ctypes.c_longlong),
        ("tc_ms", ctypes.c_double),
        ("tc_launches", ctypes.c_longlong),
        ("tc_mma_flops", ctypes.c_double),
        ("rsvd_batches", ctypes.c_longlong),
        ("rsvd_oversample_sum", ctypes.c_longlong),
        ("rsvd_power_sum", ctypes.c_longlong),
        ("rsvd_retries", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "libtebd_gb300.so not found at %s: build it with "
            "`python opentebd-extended_gb300/build.py` (there is no CPU fallback)" % path)
    L = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    L.tebd_default_opts.argtypes = [ctypes.POINTER(Opts)]
    L.tebd_default_opts.restype = None
    L.tebd_create.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(Opts), ctypes.POINTER(vp)]
    L.tebd_destroy.argtypes = [vp]
    for nm in ("tebd_set_gamma", "tebd_get_gamma", "tebd_set_lambda", "tebd_get_lambda"):
        getattr(L, nm).argtypes = [vp, ctypes.c_int, dp]
    L.tebd_set_labels.argtypes = [vp, ctypes.c_int, ip, ip]
    L.tebd_get_labels.argtypes = [vp, ctypes.c_int, ip, ip]
    for nm in ("tebd_two_site_op", "tebd_two_site_op_r", "tebd_two_site_op_nc", "tebd_two_site_op_nc_r"):
        getattr(L, nm).argtypes = [vp, ctypes.c_int, dp, dp]
    L.tebd_apply_bonds.argtypes = [vp, ctypes.c_int, ip, ctypes.POINTER(dp), dp]
    L.tebd_trotter_step.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(dp), dp]
    L.tebd_get_singular_values.argtypes = [vp, ctypes.c_int, dp, ip]
    L.tebd_get_sweeps.argtypes = [vp, ctypes.c_int, ip]
    L.tebd_sync.argtypes = [vp]
    L.tebd_last_error.argtypes = [vp]
    L.tebd_last_error.restype = ctypes.c_char_p
    L.tebd_kernel_launches.argtypes = [vp]
    L.tebd_kernel_launches.restype = ctypes.c_longlong
    L.tebd_set_profiling.argtypes = [vp, ctypes.c_int]
    L.tebd_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.tebd_reset_stats.argtypes = [vp]
    L.tebd_measure_fp64_peak.argtypes = [ctypes.c_int, dp]
    L.tebd_autotune.argtypes = [vp, ctypes.c_int, ip, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), dp, dp]
    L.tebd_get_tuning.argtypes = [ctypes.c_int, ip, ctypes.c_int, ip]
    L.tebd_clear_tuning.argtypes = [ctypes.c_int]
    L.tebd_get_stream.argtypes = [vp]
    L.tebd_get_stream.restype = ctypes.c_void_p
    L.tebd_two_site_op_noalloc.argtypes = [ctypes.c_int] * 4 + [vp, vp, vp, dp, vp]
    ll = ctypes.c_longlong
    L.tebd_zgemm_tc.argtypes = [ctypes.c_int] * 4 + [vp, ll, ctypes.c_int] * 3 + [ctypes.c_int, vp]
    L.tebd_single_site_rho.argtypes = [vp, dp]
    L.tebd_one_site_expval.argtypes = [vp, dp, dp]
    L.tebd_one_site_expval_r.argtypes = [vp, dp, dp]
    L.tebd_two_site_rho.argtypes = [vp, ctypes.c_int, dp]
    L.tebd_local_energy.argtypes = [vp, ctypes.c_int, ctypes.POINTER(dp), dp]
    L.tebd_total_energy.argtypes = [vp, ctypes.c_int, ctypes.POINTER(dp), dp]
    L.tebd_inner_product.argtypes = [vp, vp, dp]
    L.tebd_chain_entropy.argtypes = [vp, dp]
    L.tebd_swapping.argtypes = [vp, ctypes.c_int, dp]
    L.tebd_trotter_step_pbc.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(dp), dp]
    L.tebd_canonical_form_all_nc.argtypes = [vp]
    L.tebd_set_conserv.argtypes = [vp, ip]
    L.tebd_set_rank_bound.argtypes = [vp, ctypes.c_double]
    L.tebd_set_theta_form.argtypes = [vp, ctypes.c_int]
    L.tebd_set_rsvd.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    fp = ctypes.POINTER(ctypes.c_float)
    L.tebd_mlp_create.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(vp)]
    L.tebd_mlp_destroy.argtypes = [vp]
    L.tebd_mlp_param_count.argtypes = []
    L.tebd_mlp_last_error.argtypes = [vp]
    L.tebd_mlp_last_error.restype = ctypes.c_char_p
    L.tebd_mlp_get_params.argtypes = [vp, fp]
    L.tebd_mlp_set_params.argtypes = [vp, fp]
    L.tebd_mlp_forward.argtypes = [vp, ctypes.c_int, fp, fp]
    L.tebd_mlp_loss_grad.argtypes = [vp, ctypes.c_int, fp, fp, dp, fp]
    L.tebd_mlp_train.argtypes = [vp, ctypes.c_int, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_float, dp]
    L.tebd_set_rsvd_model.argtypes = [vp, vp, ctypes.c_double]
    L.tebd_canonical_form.argtypes = [vp, ctypes.c_int]
    L.tebd_canonical_form_all.argtypes = [vp]
    cp = ctypes.c_char_p
    L.tebd_record_lambdas.argtypes = [vp, cp, ctypes.c_char, ctypes.c_int]
    L.tebd_record_gammas.argtypes = [vp, cp, ctypes.c_char, ctypes.c_int]
    L.tebd_record_labels.argtypes = [vp, cp, cp]
    L.tebd_read_gamma_lambda.argtypes = [vp, cp, cp, ctypes.c_char, ctypes.c_int]
    L.tebd_read_gamma_lambda_labels.argtypes = [vp, cp, cp, cp, cp, ctypes.c_char, ctypes.c_int]
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _as_gate(op2, d):
    """(d^2, d^2) gate -> Fortran-ordered complex128 array (the C ABI's layout)."""
    g = np.asfortranarray(np.asarray(op2, dtype=np.complex128))
    if g.shape != (d * d, d * d):
        raise ValueError("gate must be (d^2, d^2) = (%d, %d), got %s" % (d * d, d * d, g.shape))
    return g


class Chain:
    """Device-resident Vidal chain: L Gammas (chi, d, chi), L+1 Lambdas (chi,),
    and in number-conserving mode LabelLeft/LabelRight (L+1, chi)."""

    def __init__(self, L, d, chi, mode=MODE_DENSE, tot_num=0, max_filling=None,
                 svd_mode=SVD_FP64, max_sweeps=0, max_batch=0, jacobi_tol=0.0, device=0,
                 conserv=None):
        self._lib = load_library()
        o = Opts()
        self._lib.tebd_default_opts(ctypes.byref(o))
        o.device = device
        o.tot_num = tot_num
        o.max_filling = (d - 1) if max_filling is None else max_filling
        o.svd_mode = svd_mode
        o.max_sweeps = max_sweeps
        o.max_batch = max_batch
        o.jacobi_tol = jacobi_tol
        h = ctypes.c_void_p()
        rc = self._lib.tebd_create(L, d, chi, mode, ctypes.byref(o), ctypes.byref(h))
        if rc != TEBD_OK:
            raise TebdError(rc, self._lib.tebd_last_error(None).decode())
        self.h = h
        self.L, self.d, self.chi, self.mode = L, d, chi, mode
        self.tot_num, self.max_filling = o.tot_num, o.max_filling
        self.conserv = None
        if conserv is not None:
            self.set_conserv(conserv)

    def set_rank_bound(self, bound):
        """Kept-rank form: keep the fewest singular values whose discarded weight is
        at most ``bound`` per update (0 = the reference's rule, chi values)."""
        self._check(self._lib.tebd_set_rank_bound(self.h, float(bound)))

    def set_theta_form(self, form):
        """Theta formation: 0 CUDA cores (default), 3 = 3xTF32 on the tensor cores
        (dense chains), 100 + S = S bf16 digit planes on the tensor cores (S = 7:
        FP64 class; on number-conserving chains one product per charge block)."""
        self._check(self._lib.tebd_set_theta_form(self.h, int(form)))

    def set_rsvd(self, oversample=64, power_iters=2, tol=1e-5, slices=7):
        """Randomized route of TEBD_SVD_RSVD: sketch width kept rank + oversample,
        power iterations, judge tolerance (largest triplet residual / ||Theta||)
        and the digit planes of its tensor-core products."""
        self._check(self._lib.tebd_set_rsvd(self.h, int(oversample), int(power_iters), float(tol), int(slices)))

    def set_rsvd_model(self, model, target=1e-6):
        """Attach a trained Mlp (None detaches): per batch it sets the randomized
        route's oversampling and power count, or sends bonds to the full SVD."""
        self._check(self._lib.tebd_set_rsvd_model(self.h, model.h if model is not None else None, float(target)))
        self._model = model  # keep it alive while attached

    def set_conserv(self, conserv):
        """Internal degrees of freedom for the NC routines: ``conserv`` = Conserv%vi
        (d particle numbers) stands for the reference's OPTIONAL intDegFree argument
        plus its Conserv global; None restores the plain form (number i-1)."""
        if conserv is None:
            self._check(self._lib.tebd_set_conserv(self.h, None))
            self.conserv = None
            return
        c = np.ascontiguousarray(conserv, dtype=np.int32)
        if c.shape != (self.d,):
            raise ValueError("conserv needs d = %d entries" % self.d)
        self._check(self._lib.tebd_set_conserv(self.h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        self.conserv = c.copy()

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self._lib.tebd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != TEBD_OK:
            raise TebdError(rc, self._lib.tebd_last_error(self.h).decode())

    # -- state transfer -------------------------------------------------------
    def set_gamma(self, site, gamma):
        g = np.asfortranarray(np.asarray(gamma, dtype=np.complex128))
        assert g.shape == (self.chi, self.d, self.chi), g.shape
        self._check(self._lib.tebd_set_gamma(self.h, site, _dp(g)))

    def get_gamma(self, site):
        g = np.zeros((self.chi, self.d, self.chi), dtype=np.complex128, order="F")
        self._check(self._lib.tebd_get_gamma(self.h, site, _dp(g)))
        return g

    def get_gamma_into(self, site, out):
        """Download Gamma(site) into a caller-owned Fortran-ordered complex128 array."""
        assert out.dtype == np.complex128 and out.flags.f_contiguous and out.shape == (self.chi, self.d, self.chi)
        self._check(self._lib.tebd_get_gamma(self.h, site, _dp(out)))

    def get_lambda_into(self, link, out):
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.shape == (self.chi,)
        self._check(self._lib.tebd_get_lambda(self.h, link, _dp(out)))

    def set_lambda(self, link, lam):
        v = np.ascontiguousarray(lam, dtype=np.float64)
        assert v.shape == (self.chi,)
        self._check(self._lib.tebd_set_lambda(self.h, link, _dp(v)))

    def get_lambda(self, link):
        v = np.zeros(self.chi)
        self._check(self._lib.tebd_get_lambda(self.h, link, _dp(v)))
        return v

    def set_labels(self, link, left=None, right=None):
        a = None if left is None else np.ascontiguousarray(left, dtype=np.int32)
        b = None if right is None else np.ascontiguousarray(right, dtype=np.int32)
        self._check(self._lib.tebd_set_labels(self.h, link, None if a is None else _ip(a),
                                              None if b is None else _ip(b)))

    def get_labels(self, link):
        a = np.zeros(self.chi, dtype=np.int32)
        b = np.zeros(self.chi, dtype=np.int32)
        self._check(self._lib.tebd_get_labels(self.h, link, _ip(a), _ip(b)))
        return a, b

    def set_state(self, gammas, lambdas, label_left=None, label_right=None):
        for s, g in enumerate(gammas, start=1):
            self.set_gamma(s, g)
        for l, v in enumerate(lambdas, start=1):
            self.set_lambda(l, v)
        if label_left is not None:
            for l in range(1, self.L + 2):
                self.set_labels(l, label_left[l - 1], label_right[l - 1])

    def get_state(self):
        gam = [self.get_gamma(s) for s in range(1, self.L + 1)]
        lam = [self.get_lambda(l) for l in range(1, self.L + 2)]
        if self.mode == MODE_NC:
            ll, lr = zip(*[self.get_labels(l) for l in range(1, self.L + 2)])
            return gam, lam, list(ll), list(lr)
        return gam, lam

    # -- the hot path -----------------------------------------------------------
    def two_site_op(self, link, op2):
        """TwoSiteOp / TwoSiteOpNC on bond `link` (1-based); returns truncerr."""
        op2 = np.asarray(op2)
        te = np.zeros(1)
        if np.iscomplexobj(op2):
            g = _as_gate(op2, self.d)
            fn = self._lib.tebd_two_site_op_nc if self.mode == MODE_NC else self._lib.tebd_two_site_op
        else:
            g = np.asfortranarray(op2, dtype=np.float64)
            if g.shape != (self.d ** 2, self.d ** 2):
                raise ValueError("gate must be (d^2, d^2)")
            fn = self._lib.tebd_two_site_op_nc_r if self.mode == MODE_NC else self._lib.tebd_two_site_op_r
        self._check(fn(self.h, link, _dp(g), _dp(te)))
        return float(te[0])

    def apply_bonds(self, links, gates):
        """Batched update of non-overlapping bonds; returns the truncation errors."""
        gs = [_as_gate(g, self.d) for g in gates]
        arr = (ctypes.POINTER(ctypes.c_double) * len(gs))(*[_dp(g) for g in gs])
        lk = np.ascontiguousarray(links, dtype=np.int32)
        te = np.zeros(len(gs))
        self._check(self._lib.tebd_apply_bonds(self.h, len(gs), _ip(lk), arr, _dp(te)))
        return te

    def autotune(self, links, gates):
        """Tune the SVD routes' launch shapes on this batch (tebd_autotune); the
        chain is left as it was.  Returns (default ms, tuned ms) of the batch."""
        gs = [_as_gate(g, self.d) for g in gates]
        arr = (ctypes.POINTER(ctypes.c_double) * len(gs))(*[_dp(g) for g in gs])
        lk = np.ascontiguousarray(links, dtype=np.int32)
        base, best = np.zeros(1), np.zeros(1)
        self._check(self._lib.tebd_autotune(self.h, len(gs), _ip(lk), arr, _dp(base), _dp(best)))
        return float(base[0]), float(best[0])

    def trotter_step(self, Udt, order=2):
        """TrotterStep(Udt, ...) with open boundaries; Udt[g-1] is the reference's Udt(g)."""
        gs = [_as_gate(g, self.d) for g in Udt]
        arr = (ctypes.POINTER(ctypes.c_double) * len(gs))(*[_dp(g) for g in gs])
        te = np.zeros(1)
        self._check(self._lib.tebd_trotter_step(self.h, order, len(gs), arr, _dp(te)))
        return float(te[0])

    def swapping(self, link):
        """Swapping(link): exchange the physical indices of sites link, link+1; truncerr."""
        te = np.zeros(1)
        self._check(self._lib.tebd_swapping(self.h, link, _dp(te)))
        return float(te[0])

    def trotter_step_pbc(self, Udt, order=2):
        """TrotterStep2ndOrderPBC / TrotterStep5thOrderPBC (BoundaryCond='P'); Udt in
        NEWConstructPropagators' periodic layout: L gates for order 2 (Udt(L) the
        edge bond), 3L (odd L) or 2L (even L) for order 5."""
        gs = [_as_gate(g, self.d) for g in Udt]
        arr = (ctypes.POINTER(ctypes.c_double) * len(gs))(*[_dp(g) for g in gs])
        te = np.zeros(1)
        self._check(self._lib.tebd_trotter_step_pbc(self.h, order, len(gs), arr, _dp(te)))
        return float(te[0])

    def canonical_form(self, link):
        """CanonicalForm on bond `link` (dense mode)."""
        self._check(self._lib.tebd_canonical_form(self.h, link))

    def canonical_form_all(self):
        """CanonicalFormAll: CanonicalForm on links 1..L-1 then L-1..1 (dense mode)."""
        self._check(self._lib.tebd_canonical_form_all(self.h))

    def canonical_form_all_nc(self):
        """CanonicalFormAllNC: identity TwoSiteOpNC sweeps forward and back."""
        self._check(self._lib.tebd_canonical_form_all_nc(self.h))

    def singular_values(self, link):
        s = np.zeros(self.d * self.chi)
        c = np.zeros(1, dtype=np.int32)
        self._check(self._lib.tebd_get_singular_values(self.h, link, _dp(s), _ip(c)))
        return s[: int(c[0])].copy()

    def sweeps(self, link):
        c = np.zeros(1, dtype=np.int32)
        self._check(self._lib.tebd_get_sweeps(self.h, link, _ip(c)))
        return int(c[0])

    def sync(self):
        self._check(self._lib.tebd_sync(self.h))

    def kernel_launches(self):
        return int(self._lib.tebd_kernel_launches(self.h))

    def set_profiling(self, on=True):
        self._check(self._lib.tebd_set_profiling(self.h, 1 if on else 0))

    def stats(self):
        st = Stats()
        self._check(self._lib.tebd_get_stats(self.h, ctypes.byref(st)))
        return st.as_dict()

    def reset_stats(self):
        self._check(self._lib.tebd_reset_stats(self.h))

    # -- observables on the device (observables_module.f90) ----------------------
    def single_site_rho(self):
        """SingleSiteDensityMatrix: (L, d, d) complex, rho[s-1] for site s."""
        r = np.zeros((self.L, self.d, self.d), dtype=np.complex128)
        buf = np.zeros(self.L * self.d * self.d, dtype=np.complex128)
        self._check(self._lib.tebd_single_site_rho(self.h, _dp(buf)))
        for s in range(self.L):
            r[s] = buf[s * self.d ** 2:(s + 1) * self.d ** 2].reshape(self.d, self.d, order="F")
        return r

    def one_site_expval(self, op):
        """OneSiteExpVal: Tr(Op rho_s) for s = 1..L (complex Op -> complex, real Op -> real)."""
        op = np.asarray(op)
        if np.iscomplexobj(op):
            o = np.asfortranarray(op, dtype=np.complex128)
            out = np.zeros(self.L, dtype=np.complex128)
            self._check(self._lib.tebd_one_site_expval(self.h, _dp(o), _dp(out)))
        else:
            o = np.asfortranarray(op, dtype=np.float64)
            out = np.zeros(self.L)
            self._check(self._lib.tebd_one_site_expval_r(self.h, _dp(o), _dp(out)))
        return out

    def two_site_rho(self, link):
        """TwoSiteRho on sites link, link+1: (d^2, d^2), rows (i-1)*d+j as the gates."""
        r = np.zeros((self.d ** 2, self.d ** 2), dtype=np.complex128, order="F")
        self._check(self._lib.tebd_two_site_rho(self.h, link, _dp(r)))
        return r

    def _bond_ops(self, H):
        hs = [np.asfortranarray(h, dtype=np.complex128) for h in H]
        arr = (ctypes.POINTER(ctypes.c_double) * len(hs))(*[_dp(h) for h in hs])
        return hs, arr

    def local_energy(self, H):
        """LocalEnergy: Re Tr(H(l) rho2(l)) for bonds l = 1..L-1 (H[l-1] is H(l))."""
        hs, arr = self._bond_ops(H)
        out = np.zeros(self.L - 1)
        self._check(self._lib.tebd_local_energy(self.h, len(hs), arr, _dp(out)))
        return out

    def total_energy(self, H):
        """TotalEnergy (open boundary)."""
        hs, arr = self._bond_ops(H)
        out = np.zeros(1)
        self._check(self._lib.tebd_total_energy(self.h, len(hs), arr, _dp(out)))
        return float(out[0])

    def inner_product(self, other):
        """InnerProduct(self, other) = <self|other>."""
        out = np.zeros(1, dtype=np.complex128)
        self._check(self._lib.tebd_inner_product(self.h, other.h, _dp(out)))
        return complex(out[0])

    # -- state I/O in the reference's record formats (io_module.f90) ------------
    def record_lambdas(self, path, kind="S", append=False):
        """RecordLambdas: kind 'S' (E30.15) or 'B' (B80, exact)."""
        self._check(self._lib.tebd_record_lambdas(self.h, os.fsencode(path), kind.encode(), int(append)))

    def record_gammas(self, path, kind="S", append=False):
        """RecordGammas: real parts, then imaginary parts, one record per (site, alpha, beta)."""
        self._check(self._lib.tebd_record_gammas(self.h, os.fsencode(path), kind.encode(), int(append)))

    def record_labels(self, path_left=None, path_right=None):
        """RecordLabel of LabelLeft and LabelRight (NC mode)."""
        self._check(self._lib.tebd_record_labels(self.h, None if path_left is None else os.fsencode(path_left),
                                                 None if path_right is None else os.fsencode(path_right)))

    def read_gamma_lambda(self, lambda_path, gamma_path, kind="S", chi_now=None):
        """readGammaLambda into this chain (records of chi_now values; default chi)."""
        self._check(self._lib.tebd_read_gamma_lambda(self.h, os.fsencode(lambda_path), os.fsencode(gamma_path),
                                                     kind.encode(), chi_now or self.chi))

    def read_gamma_lambda_labels(self, lambda_path, gamma_path, left_path, right_path, kind="S", chi_now=None):
        """readGammaLambdaLabels into this chain (NC mode)."""
        self._check(self._lib.tebd_read_gamma_lambda_labels(
            self.h, os.fsencode(lambda_path), os.fsencode(gamma_path), os.fsencode(left_path),
            os.fsencode(right_path), kind.encode(), chi_now or self.chi))

    def chain_entropy(self):
        """ChainEntropy(link) for links 1..L+1 (entropy in base d, as the reference)."""
        out = np.zeros(self.L + 1)
        self._check(self._lib.tebd_chain_entropy(self.h, _dp(out)))
        return out

    def stream(self):
        """The handle's cudaStream_t as an integer."""
        return int(self._lib.tebd_get_stream(self.h) or 0)


def measure_fp64_peak(device=0):
    """FP64 FMA throughput of the device in TFLOP/s (DFMA loop in the library)."""
    lib = load_library()
    v = np.zeros(1)
    rc = lib.tebd_measure_fp64_peak(device, _dp(v))
    if rc != TEBD_OK:
        raise TebdError(rc, "tebd_measure_fp64_peak failed")
    return float(v[0])


TUNE_ROUTES = {0: "fp64 bidiagonal", 1: "double-float bidiagonal", 2: "randomized-route Cholesky",
               3: "randomized-route Cholesky blocking"}


def get_tuning(device=0):
    """The device's autotuner table as dicts (tebd_get_tuning); 0 = the default shape."""
    lib = load_library()
    cnt = np.zeros(1, dtype=np.int32)
    rc = lib.tebd_get_tuning(device, None, 0, _ip(cnt))
    if rc != TEBD_OK:
        raise TebdError(rc, "tebd_get_tuning failed")
    n = int(cnt[0])
    buf = np.zeros(10 * max(n, 1), dtype=np.int32)
    rc = lib.tebd_get_tuning(device, _ip(buf), n, _ip(cnt))
    if rc != TEBD_OK:
        raise TebdError(rc, "tebd_get_tuning failed")
    keys = ("route", "n_bucket", "bonds_bucket", "cluster", "team", "chol_cluster", "panel", "chol_leaf",
            "orth_cluster", "batch_us")
    rows = [dict(zip(keys, (int(v) for v in buf[10 * i:10 * i + 10]))) for i in range(n)]
    for r in rows:
        r["route"] = TUNE_ROUTES.get(r["route"], r["route"])
    return rows


def clear_tuning(device=0):
    """Empty the device's autotuner table (tebd_clear_tuning)."""
    rc = load_library().tebd_clear_tuning(device)
    if rc != TEBD_OK:
        raise TebdError(rc, "tebd_clear_tuning failed")


# -- reference-named entry points ---------------------------------------------
def TwoSiteOp(link, Op2, chain: Chain) -> float:
    """local_operations_module.f90 TwoSiteOp(link, Op2, Gammas, Lambdas, truncerr)."""
    if chain.mode != MODE_DENSE:
        raise TebdError(TEBD_ERR_STATE, "TwoSiteOp needs a dense chain")
    return chain.two_site_op(link, Op2)


def TwoSiteOpNC(link, Op2, chain: Chain) -> float:
    """local_operations_module.f90 TwoSiteOpNC(link, Op2, Gammas, Lambdas, LabelLeft, LabelRight, truncerr)."""
    if chain.mode != MODE_NC:
        raise TebdError(TEBD_ERR_STATE, "TwoSiteOpNC needs a number-conserving chain")
    return chain.two_site_op(link, Op2)


def TrotterStep(Udt, chain: Chain, order=2) -> float:
    """propagation_module.f90 TrotterStep / TrotterStepNC (BoundaryCond='O')."""
    return chain.trotter_step(Udt, order)


def OneSiteExpVal(Op, chain: Chain):
    """OneSiteExpVal(expList, Op, Gammas, Lambdas) on the GPU: returns expList."""
    return chain.one_site_expval(Op)


def TotalEnergy(H, chain: Chain) -> float:
    """TotalEnergy(energy, H, Gammas, Lambdas), open boundary: returns energy."""
    return chain.total_energy(H)


def LocalEnergy(H, chain: Chain):
    """LocalEnergy(energy, H, Gammas, Lambdas), open boundary: returns energy(1:L-1)."""
    return chain.local_energy(H)


def InnerProduct(chain_left: Chain, chain_right: Chain) -> complex:
    """InnerProduct(GammasL, LambdasL, GammasR, LambdasR)."""
    return chain_left.inner_product(chain_right)


def ChainEntropy(link, chain: Chain) -> float:
    """ChainEntropy(link, Lambdas)."""
    return float(chain.chain_entropy()[link - 1])


class Mlp:
    """The learned model of the randomized route (tebd_mlp_*): 67 -> 128 -> 128 -> 8,
    FP32, trained on the GPU by the library's kernels.  x: (n, 67), targets (n, 8)."""

    N_IN, N_OUT = 67, 8

    def __init__(self, device=0, seed=0):
        self._lib = load_library()
        h = ctypes.c_void_p()
        rc = self._lib.tebd_mlp_create(device, seed, ctypes.byref(h))
        if rc != TEBD_OK:
            raise TebdError(rc, "tebd_mlp_create failed")
        self.h = h
        self.n_params = self._lib.tebd_mlp_param_count()

    def _check(self, rc):
        if rc != TEBD_OK:
            raise TebdError(rc, self._lib.tebd_mlp_last_error(self.h).decode())

    @staticmethod
    def _f(a, cols):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.ndim != 2 or a.shape[1] != cols:
            raise ValueError("expected (n, %d) array" % cols)
        return a

    def params(self):
        p = np.zeros(self.n_params, np.float32)
        self._check(self._lib.tebd_mlp_get_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        self._check(self._lib.tebd_mlp_set_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def forward(self, x):
        x = self._f(x, self.N_IN)
        y = np.zeros((len(x), self.N_OUT), np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self._lib.tebd_mlp_forward(self.h, len(x), x.ctypes.data_as(fp), y.ctypes.data_as(fp)))
        return y

    def loss_grad(self, x, t):
        x, t = self._f(x, self.N_IN), self._f(t, self.N_OUT)
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_double(0.0)
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self._lib.tebd_mlp_loss_grad(self.h, len(x), x.ctypes.data_as(fp), t.ctypes.data_as(fp),
                                                 ctypes.byref(loss), g.ctypes.data_as(fp)))
        return loss.value, g

    def train(self, x, t, epochs=200, batch=256, lr=1e-3):
        x, t = self._f(x, self.N_IN), self._f(t, self.N_OUT)
        loss = ctypes.c_double(0.0)
        fp = ctypes.POINTER(ctypes.c_float)
        self._check(self._lib.tebd_mlp_train(self.h, len(x), x.ctypes.data_as(fp), t.ctypes.data_as(fp), epochs,
                                             batch, float(lr), ctypes.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            self._lib.tebd_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
