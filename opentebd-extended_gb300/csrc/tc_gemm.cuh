// tc_gemm.cuh -- split-precision complex products on the sm_103a tensor cores.
//
// A complex product C (m x n) = A (m x k) * B (k x n) is computed as one real
// product on the 5th-generation tensor cores (tcgen05.mma, TMEM accumulator,
// operands staged by TMA):
//   A_r (m x 2k), row i = (re a_i0, im a_i0, re a_i1, im a_i1, ...)
//   B_r (2n x 2k), row 2j   = (re b_0j, -im b_0j, re b_1j, -im b_1j, ...)
//                  row 2j+1 = (im b_0j,  re b_0j, im b_1j,  re b_1j, ...)
//   C_r = A_r B_r^T (m x 2n): column 2j = Re c_ij, column 2j+1 = Im c_ij.
// Each real operand is held as TF32 planes in K-major order (row-major, the K
// index contiguous), padded to 128 rows and 32 columns:
//   3xTF32 -- hi = tf32(x), lo = tf32(x - hi); the product accumulates
//             hi*hi + hi*lo + lo*hi in FP32 (the lo*lo term, ~2^-22 relative,
//             is dropped): about FP32 accuracy from three TF32 passes;
//   1xTF32 -- hi only (10-bit significands), for sketches where a subspace, not
//             the digits, is wanted.
// Planes of one operand are stored [plane][problem][row][k], so one 3-D tensor
// map (x = k, y = row, z = plane * nprob + problem) covers a whole batch.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "tebd_internal.cuh"

namespace tebd {

constexpr int kTcBM = 128;  // output rows per CTA (the MMA's M)
constexpr int kTcBN = 128;  // real output columns per CTA (the MMA's N)
constexpr int kTcBK = 32;   // K per stage: 32 FP32 = one 128-byte swizzle row

enum TcForm { kTc1xTF32 = 1, kTc3xTF32 = 3 };

// One batch of real products C_r = A_r B_r^T on the tensor cores.  The planes
// must have been packed (tc_pack_*) with rows padded to kTcBM and k to kTcBK.
struct TcBatch {
  const float *a_planes;  // [na][nprob][m_pad][k_pad]
  const float *b_planes;  // [nb][nprob][n_pad][k_pad] (n_pad = padded 2n)
  int nprob, m_pad, n_pad, k_pad;
  int form;               // kTc1xTF32 or kTc3xTF32
  // epilogue: complex FP64 output, problem p at out + p * out_stride,
  // element (i, j) at out[i * rs + j * cs] (complex units) for i < m[p], j < n[p]
  double2 *out;
  long long out_stride;
  long long rs, cs;
  const int *m_d, *n_d;   // per-problem sizes at m_d[p * dim_stride] (complex units), or null
  int dim_stride;
  int m, n;               // sizes used when m_d / n_d are null
  int accumulate;         // 1: out += C, 0: out = C
  double alpha;           // scale applied to C
  const unsigned char *optr;  // optional: output base of problem p read at optr + p * optr_stride
  int optr_stride;            // (cs == 0 then means: column stride = the problem's m)
};

// Launch one batch on `st`.  err_d: device int set non-zero if a pipeline wait
// ran out of time (the kernel then returns without writing).
cudaError_t tc_gemm_launch(const TcBatch &b, int *err_d, cudaStream_t st);

// Pack a complex column-major matrix (element (i, k) at src[i + ld * k], problem p
// at src + p * pstride) into A planes: row i, columns 2k, 2k+1.  conj != 0 packs
// conj(src) and trans != 0 packs the transpose (element (i, k) read at
// src[k + ld * i]), so A^H is trans = conj = 1.
cudaError_t tc_pack_a(const double2 *src, long long pstride, int ld, int rows, int cols, int trans,
                      int conj, int nprob, int m_pad, int k_pad, int form, float *planes,
                      cudaStream_t st);
// Pack the complex K x N matrix B (element (k, j) at src[k + ld * j], or
// src[j + ld * k] when trans != 0, conj as above) into B_r planes (2n rows).
cudaError_t tc_pack_b(const double2 *src, long long pstride, int ld, int krows, int ncols, int trans,
                      int conj, int nprob, int n_pad, int k_pad, int form, float *planes,
                      cudaStream_t st);

inline int tc_pad(int x, int q) { return (x + q - 1) / q * q; }
inline int tc_planes(int form) { return form == kTc3xTF32 ? 2 : 1; }

// ---------------------------------------------------------------------------
// FP64-class products: error-free splitting into bf16 integer digits (the
// Ozaki scheme; K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication", Numer. Algorithms 59, 2012).
//
// Every real row r of A_r (and of B_r) gets the power of two 2^e_r above its
// largest magnitude and S digit planes: x = 2^e_r sum_s D_s 2^(-7(s+1)) + rest,
// with D_0 in [-128, 128], D_s in [-64, 64] (s > 0), integers held exactly in
// bf16, |rest| <= 2^(e_r - 7S - 1).  The real product is
//   c_rc = 2^(e_r + f_c) sum_g 2^(-7(g+2)) sum_{s+t=g} (D^A_s D^B_t^T)_rc,
// keeping the groups g = 0..S-1.  One group's sum over a K chunk of 512 real
// terms stays below 2^24 for g <= 5 (each digit product is at most 2^14), so the
// tensor cores' FP32 accumulation of it is exact; the chunks and groups are
// combined in FP64.  Accuracy: about 2^(-7S) relative to (row max x column max)
// per term -- S = 7 is FP64 class (~1e-15), S = 5 ~ 1e-11.
// ---------------------------------------------------------------------------
constexpr int kOzBN = 128;     // real output columns per CTA
constexpr int kOzBK = 32;      // bf16 per 64-byte row (K block)
constexpr int kOzMaxS = 7;

struct OzBatch {
  const unsigned short *a_dig;  // bf16 digits [S][nprob][m_pad][k_pad]
  const unsigned short *b_dig;  // bf16 digits [S][nprob][n_pad][k_pad] (n_pad real rows)
  const int *a_exp;             // [nprob][m_pad] row exponents
  const int *b_exp;             // [nprob][n_pad / 2] exponents of the complex columns
  int nprob, m_pad, n_pad, k_pad, slices;
  double2 *out;                 // as TcBatch
  long long out_stride, rs, cs;
  const int *m_d, *n_d;         // per-problem sizes at m_d[p * dim_stride] (complex units), or null
  int dim_stride;
  int m, n;
  int accumulate;
  double alpha;
  const unsigned char *optr;    // optional: output base of problem p read at optr + p * optr_stride
  int optr_stride;
};

cudaError_t oz_gemm_launch(const OzBatch &b, int *err_d, cudaStream_t st);

// Digits and exponents of the A operand (same source conventions as tc_pack_a);
// exps must hold nprob * m_pad ints.
cudaError_t oz_pack_a(const double2 *src, long long pstride, int ld, int rows, int cols, int trans,
                      int conj, int nprob, int m_pad, int k_pad, int slices, unsigned short *dig,
                      int *exps, cudaStream_t st);
// Digits and exponents of the B operand (as tc_pack_b); exps: nprob * n_pad / 2 ints.
cudaError_t oz_pack_b(const double2 *src, long long pstride, int ld, int krows, int ncols, int trans,
                      int conj, int nprob, int n_pad, int k_pad, int slices, unsigned short *dig,
                      int *exps, cudaStream_t st);

// ---------------------------------------------------------------------------
// One batched complex product C_p (m x n) = op(A_p) (m x k) op(B_p) (k x n) in
// any of the forms: 1 / 3 (1xTF32, 3xTF32) or 100 + S (S bf16 digit planes).
// op(A): element (i, l) at a[i + lda l] (a_trans = 0) or a[l + lda i] (a_trans = 1),
// conjugated when a_conj; op(B): (l, j) at b[l + ldb j] or b[j + ldb l].  The
// sizes are the batch maxima: each operand is read up to them (the caller
// zero-fills beyond a problem's own extent), the output is written only inside
// the problem's own m_d / n_d.
// ---------------------------------------------------------------------------
struct ZProd {
  const double2 *a;
  long long a_stride;
  int lda, a_trans, a_conj;
  const double2 *b;
  long long b_stride;
  int ldb, b_trans, b_conj;
  int nprob, m, n, k;
  int form;
  double2 *out;
  long long out_stride, rs, cs;
  const int *m_d, *n_d;
  int dim_stride;
  int accumulate;
  double alpha;
  const unsigned char *optr;
  int optr_stride;
  // digit-plane forms: A already packed (oz_pack_a with at least the form's planes,
  // m_pad = tc_pad(m, 128), k_pad = tc_pad(2 k, 32)) -- A is then not read
  const unsigned short *a_dig;
  const int *a_exp;
  // optional events recorded around the product kernel alone (profiling)
  cudaEvent_t ev0, ev1;
};
inline bool zprod_oz(int form) { return form > 100 && form <= 100 + kOzMaxS; }
size_t zprod_ws_bytes(const ZProd &z);
// tensor-core multiply-adds the product kernel issues, as flops (2 per
// multiply-add): planes pairs x 2 x m_pad x n_pad x k_pad x `active` problems
double zprod_mma_flops(const ZProd &z, int active);
// ws: zprod_ws_bytes(z) bytes of device memory (256-byte aligned).
cudaError_t zprod_run(const ZProd &z, void *ws, int *err_d, cudaStream_t st);

}  // namespace tebd
