// jacobi.cu -- batched one-sided (Hestenes) Jacobi SVD, complex, FP64 or FP32.
//
// Replaces the ZGESVD('A','A') call of SVDTruncation
// (VidalCore_v_2.0/local_operations_module.f90:322-345) and of SVDNC (:1470-1492).
//
// Algorithm.  The columns of X (m x n) are orthogonalised pairwise by complex
// Jacobi rotations; the same rotations are accumulated into V, so that at
// convergence X = U*Sigma and Theta = U*Sigma*V^H.  One-sided Jacobi keeps
// the singular values accurate relative to their own size (better than the
// bidiagonal route of ZGESVD), so it is used as the FP64 reference-parity SVD.
//
// Parallel schedule.  A sweep visits every column pair once in npad-1 rounds
// of npad/2 disjoint pairs (round-robin "circle" tournament, npad = n rounded
// up to even).  One kernel launch per round: every warp of the grid owns one
// pair of one problem, so all pairs of all batched problems rotate concurrently
// and the launch boundary is the only synchronisation.  Matrices stay in HBM
// and are streamed through L2 (cfg: n <= 3072).
//
// Convergence.  A pair is rotated when |a^H b| > tol*|a||b|; a sweep without a
// rotation ends the problem.  A problem that exceeds the sweep cap reports
// TEBD_ERR_SVD_NOCONV.  Every wait is a host-side loop over bounded launches:
// no kernel spins.
#include <math.h>

#include "tebd_internal.cuh"

namespace tebd {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
struct JacobiBig;
template <>
struct JacobiBig<double> {
  static __device__ __forceinline__ double v() { return 1e150; }
};
template <>
struct JacobiBig<float> {
  static __device__ __forceinline__ float v() { return 1e18f; }
};

// Rotate columns (A, B) of X and (VA, VB) of V by the unitary 2x2 that makes
// them orthogonal.  Gram [[al, g e^{i phi}], [g e^{-i phi}, be]]:
//   zeta = (be - al) / (2 g),  t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)),
//   c = 1/sqrt(1+t^2), s = c t,
//   a' = c a - s e^{-i phi} b,   b' = s e^{i phi} a + c b.
template <typename T>
__device__ __forceinline__ bool jacobi_pair(typename cplx<T>::type *__restrict__ A,
                                            typename cplx<T>::type *__restrict__ B,
                                            typename cplx<T>::type *__restrict__ VA,
                                            typename cplx<T>::type *__restrict__ VB, int m,
                                            int nv, int lane, T tol) {
  using C2 = typename cplx<T>::type;
  T al = 0, be = 0, gr = 0, gi = 0;
  for (int r = lane; r < m; r += 32) {
    const C2 a = A[r], b = B[r];
    al = fma(a.x, a.x, fma(a.y, a.y, al));
    be = fma(b.x, b.x, fma(b.y, b.y, be));
    gr = fma(a.x, b.x, fma(a.y, b.y, gr));
    gi = fma(a.x, b.y, fma(-a.y, b.x, gi));
  }
  al = warp_sum(al);
  be = warp_sum(be);
  gr = warp_sum(gr);
  gi = warp_sum(gi);
  const T g = sqrt(gr * gr + gi * gi);
  if (!(g > tol * sqrt(al) * sqrt(be))) return false;
  const T zeta = (be - al) / (T(2) * g);
  T t;
  if (fabs(zeta) > JacobiBig<T>::v())
    t = T(0.5) / zeta;
  else
    t = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  const T c = T(1) / sqrt(T(1) + t * t);
  const T s = c * t;
  const T sr = s * (gr / g), si = s * (gi / g);
  for (int r = lane; r < m; r += 32) {
    const C2 a = A[r], b = B[r];
    C2 na, nb;
    na.x = fma(c, a.x, fma(-sr, b.x, -si * b.y));
    na.y = fma(c, a.y, fma(-sr, b.y, si * b.x));
    nb.x = fma(sr, a.x, fma(-si, a.y, c * b.x));
    nb.y = fma(sr, a.y, fma(si, a.x, c * b.y));
    A[r] = na;
    B[r] = nb;
  }
  for (int r = lane; r < nv; r += 32) {
    const C2 a = VA[r], b = VB[r];
    C2 na, nb;
    na.x = fma(c, a.x, fma(-sr, b.x, -si * b.y));
    na.y = fma(c, a.y, fma(-sr, b.y, si * b.x));
    nb.x = fma(sr, a.x, fma(-si, a.y, c * b.x));
    nb.y = fma(sr, a.y, fma(si, a.x, c * b.y));
    VA[r] = na;
    VB[r] = nb;
  }
  return true;
}

constexpr int kJacobiWarps = 8;  // warps (column pairs) per CTA

template <typename T>
__global__ void __launch_bounds__(kJacobiWarps * 32)
    k_jacobi_round(const JacobiProblem<T> *__restrict__ probs, const int *__restrict__ done,
                   int *__restrict__ rot, int round, T tol) {
  const int p = blockIdx.y;
  if (done[p]) return;
  const JacobiProblem<T> P = probs[p];
  const int npad = P.n + (P.n & 1);
  const int R = npad - 1;
  if (round >= R) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kJacobiWarps + warp;
  if (k >= npad / 2) return;
  int i, j;
  if (k == 0) {
    i = R;
    j = round;
  } else {
    i = (round + k) % R;
    j = (round - k + R) % R;
  }
  if (i >= P.n || j >= P.n) return;  // the phantom column of an odd n
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
  const bool r = jacobi_pair<T>(P.X + (size_t)P.ldx * i, P.X + (size_t)P.ldx * j,
                                P.V + (size_t)P.ldv * i, P.V + (size_t)P.ldv * j, P.m, P.n, lane,
                                tol);
  if (r && lane == 0) rot[p] = 1;
}

__global__ void k_jacobi_init(int nprob, int *rot, int *done, int *sweeps) {
  for (int p = threadIdx.x; p < nprob; p += blockDim.x) {
    rot[p] = 0;
    done[p] = 0;
    sweeps[p] = 0;
  }
}

__global__ void k_jacobi_sweep_end(int nprob, int *rot, int *done, int *sweeps, int *pending) {
  if (threadIdx.x != 0) return;
  int cnt = 0;
  for (int p = 0; p < nprob; ++p) {
    if (!done[p]) {
      sweeps[p] += 1;
      if (rot[p] == 0) done[p] = 1;
      rot[p] = 0;
    }
    cnt += !done[p];
  }
  pending[0] = cnt;
}

template <typename T>
static int jacobi_sweeps(tebd_handle *h, const JacobiProblem<T> *probs_d, int nprob, int nmax,
                         T tol, int max_sweeps, int *sweeps_used) {
  cudaStream_t st = h->stream;
  const int npad = nmax + (nmax & 1);
  const int rounds = npad - 1;
  const unsigned gx = (unsigned)((npad / 2 + kJacobiWarps - 1) / kJacobiWarps);
  int *pending_h = reinterpret_cast<int *>(h->pinned);
  for (int sw = 0; sw < max_sweeps; ++sw) {
    for (int r = 0; r < rounds; ++r) {
      k_jacobi_round<T><<<dim3(gx, nprob), kJacobiWarps * 32, 0, st>>>(probs_d, h->js.done,
                                                                       h->js.rot, r, tol);
      TEBD_LAUNCHED(h);
    }
    k_jacobi_sweep_end<<<1, 32, 0, st>>>(nprob, h->js.rot, h->js.done, h->js.sweeps,
                                          h->js.pending);
    TEBD_LAUNCHED(h);
    int rc = check_cuda(h, cudaMemcpyAsync(pending_h, h->js.pending, sizeof(int),
                                           cudaMemcpyDeviceToHost, st),
                        "jacobi pending copy");
    if (rc) return rc;
    rc = check_cuda(h, cudaStreamSynchronize(st), "jacobi sweep");
    if (rc) return rc;
    *sweeps_used = sw + 1;
    if (*pending_h == 0) return TEBD_OK;
  }
  return set_error(h, TEBD_ERR_SVD_NOCONV, "Jacobi SVD did not converge within the sweep cap");
}

int run_jacobi(tebd_handle *h, int nb, int /*svd_mode*/) {
  const int n = h->n;
  k_jacobi_init<<<1, 64, 0, h->stream>>>(nb, h->js.rot, h->js.done, h->js.sweeps);
  TEBD_LAUNCHED(h);
  const double tol = h->opts.jacobi_tol > 0 ? h->opts.jacobi_tol : (double)n * 2.220446049250313e-16;
  const int cap = h->opts.max_sweeps > 0 ? h->opts.max_sweeps : 60;
  int used = 0;
  return jacobi_sweeps<double>(h, reinterpret_cast<const JacobiProblem<double> *>(h->jprob_d), nb, n,
                               tol, cap, &used);
}

// Generic entry used by the NC path: caller-provided problem table.
int run_jacobi_problems(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob, int nmax) {
  k_jacobi_init<<<1, 64, 0, h->stream>>>(nprob, h->js.rot, h->js.done, h->js.sweeps);
  TEBD_LAUNCHED(h);
  const double tol =
      h->opts.jacobi_tol > 0 ? h->opts.jacobi_tol : (double)(nmax > 8 ? nmax : 8) * 2.220446049250313e-16;
  const int cap = h->opts.max_sweeps > 0 ? h->opts.max_sweeps : 60;
  int used = 0;
  return jacobi_sweeps<double>(h, probs_d, nprob, nmax, tol, cap, &used);
}

}  // namespace tebd
