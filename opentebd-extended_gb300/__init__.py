"""GB300 (sm_103a) Vidal two-site TEBD update behind the reference's interface.

The directory name is not a Python identifier; load it with
``__graft_entry__.load_package()`` (registered as ``opentebd_extended_gb300``).
"""
from . import hamiltonians  # noqa: F401
from .tebd import (  # noqa: F401
    Chain, Mlp, TebdError, TrotterStep, TwoSiteOp, TwoSiteOpNC, load_library,
    OneSiteExpVal, TotalEnergy, LocalEnergy, InnerProduct, ChainEntropy,
    MODE_DENSE, MODE_NC, SVD_FP64, SVD_JACOBI, SVD_BIDIAG, SVD_QRJ, SVD_DF, SVD_RSVD, EXPORTED_SYMBOLS, measure_fp64_peak,
    get_tuning, clear_tuning,
)
