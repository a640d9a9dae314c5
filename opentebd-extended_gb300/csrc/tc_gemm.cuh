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
  const int *m_d, *n_d;   // device arrays of per-problem sizes (complex units), or null
  int m, n;               // sizes used when m_d / n_d are null
  int accumulate;         // 1: out += C, 0: out = C
  double alpha;           // scale applied to C
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

}  // namespace tebd
