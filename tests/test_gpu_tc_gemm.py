"""The split-precision complex product on the tensor cores (tcgen05, TMA, TMEM).

tebd_zgemm_tc computes C_p = A_p B_p for a batch of complex matrices through the
real embedding of the complex product, with TF32 operand planes.  Checked against
numpy's complex128 product on the same inputs, with the error of each element
measured relative to (|A| |B|)_ij -- the scale of the rounding error of any
product of those operands:
* 3xTF32 (hi*hi + hi*lo + lo*hi, FP32 accumulation): every element within
  3e-5, Frobenius-relative within 2e-6 (FP32 accumulation over 2k real terms);
* 1xTF32 (10-bit significands): every element within 4e-3, Frobenius-relative
  within 1e-3.
Shapes cover one element, ragged sizes (not multiples of the 128 x 128 tile or
the 32-wide K block), a batch, and a saturated-bond size (640 x 640 x 128).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {3: (3e-5, 2e-6), 1: (4e-3, 1e-3)}


def _cplx(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _run(pkg, torch, A, B, form, ldc_extra=0, C0=None):
    """A: (nprob, k, lda) and B: (nprob, n, ldb) complex arrays holding column-major
    matrices (element (i, l) of A_p at A[p, l, i])."""
    lib = pkg.load_library()
    nprob, k, lda = A.shape
    _, n, ldb = B.shape
    m = lda
    ldc = m + ldc_extra
    Ad = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    C = np.zeros((nprob, n, ldc), complex) if C0 is None else C0.copy()
    Cd = torch.from_numpy(C).cuda()
    torch.cuda.synchronize()
    rc = lib.tebd_zgemm_tc(nprob, m, n, k, Ad.data_ptr(), k * lda, lda, Bd.data_ptr(), n * ldb, ldb,
                           Cd.data_ptr(), n * ldc, ldc, form, None)
    assert rc == 0, rc
    return Cd.cpu().numpy()


@pytest.mark.parametrize("form", [3, 1])
@pytest.mark.parametrize("nprob,m,n,k", [(1, 1, 1, 1), (2, 128, 64, 32), (3, 200, 130, 77), (1, 640, 640, 128)])
def test_zgemm_tc_matches_complex128(pkg, form, nprob, m, n, k):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m + 7 * n + 13 * k + form)
    A = _cplx(rng, (nprob, k, m))
    B = _cplx(rng, (nprob, n, k))
    C = _run(pkg, torch, A, B, form)
    el_tol, fro_tol = TOL[form]
    for p in range(nprob):
        Ap, Bp = A[p].T, B[p].T  # m x k, k x n
        ref = Ap @ Bp
        scale = np.abs(Ap) @ np.abs(Bp)
        err = np.abs(C[p].T - ref)
        assert np.max(err / scale) < el_tol, np.max(err / scale)
        assert np.linalg.norm(err) / np.linalg.norm(scale) < fro_tol


def test_zgemm_tc_leaves_padding_of_c_untouched(pkg):
    """ldc > m: the rows between m and ldc belong to the caller and keep their values."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    A = _cplx(rng, (1, 40, 70))
    B = _cplx(rng, (1, 50, 40))
    C0 = np.full((1, 50, 75), 7.0 + 3.0j)
    C = _run(pkg, torch, A, B, 3, ldc_extra=5, C0=C0)
    assert np.all(C[0, :, 70:] == 7.0 + 3.0j)
    ref = A[0].T @ B[0].T
    assert np.max(np.abs(C[0, :, :70].T - ref)) < 1e-4


@pytest.mark.parametrize("slices", [7, 5, 3])
@pytest.mark.parametrize("nprob,m,n,k", [(1, 1, 1, 1), (2, 130, 70, 33), (1, 640, 160, 640), (1, 300, 40, 700)])
def test_zgemm_ozaki_error_bound(pkg, slices, nprob, m, n, k):
    """Error-free splitting into `slices` bf16 digit planes: every element within
    2^(-7 slices + 2) x (row max of A) x (column max of B) x 2k of the complex128
    product (k = 700 needs two exact 512-term chunks of the real embedding)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m + n + k + slices)
    A = _cplx(rng, (nprob, k, m)) * np.exp(rng.uniform(-3, 3, (nprob, 1, m)))  # rows of different scales
    B = _cplx(rng, (nprob, n, k)) * np.exp(rng.uniform(-3, 3, (nprob, n, 1)))
    C = _run(pkg, torch, A, B, 100 + slices)
    for p in range(nprob):
        Ap, Bp = A[p].T, B[p].T
        ref = Ap @ Bp
        rmax = np.max(np.maximum(np.abs(Ap.real), np.abs(Ap.imag)), axis=1)
        cmax = np.max(np.maximum(np.abs(Bp.real), np.abs(Bp.imag)), axis=0)
        bound = 2.0 ** (-7 * slices + 2) * np.outer(rmax, cmax) * 2 * k
        err = np.abs(C[p].T - ref)
        assert np.all(err <= bound + 1e-300), np.max(err / bound)


def test_zgemm_ozaki7_matches_fp64_to_rounding(pkg):
    """With 7 slices the product is FP64 class: within 4e-15 of complex128 relative
    to (|A| |B|)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    A = _cplx(rng, (1, 640, 640))
    B = _cplx(rng, (1, 128, 640))
    C = _run(pkg, torch, A, B, 107)
    ref = A[0].T @ B[0].T
    scale = np.abs(A[0].T) @ np.abs(B[0].T)
    assert np.max(np.abs(C[0].T - ref) / scale) < 4e-15
