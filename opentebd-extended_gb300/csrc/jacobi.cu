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
#include <cooperative_groups.h>
#include <math.h>

#include <vector>

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
                                            int nv, int lane, T tol, double floor) {
  using C2 = typename cplx<T>::type;
  T al = 0, be = 0, gr = 0, gi = 0;
  for (int r = lane; r < m; r += 32) {
    const C2 a = __ldcg(A + r), b = __ldcg(B + r);
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
  if (!(g > tol * sqrt(al) * sqrt(be)) || (double)al <= floor || (double)be <= floor) return false;
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
    const C2 a = __ldcg(A + r), b = __ldcg(B + r);
    C2 na, nb;
    na.x = fma(c, a.x, fma(-sr, b.x, -si * b.y));
    na.y = fma(c, a.y, fma(-sr, b.y, si * b.x));
    nb.x = fma(sr, a.x, fma(-si, a.y, c * b.x));
    nb.y = fma(sr, a.y, fma(si, a.x, c * b.y));
    A[r] = na;
    B[r] = nb;
  }
  for (int r = lane; r < nv; r += 32) {
    const C2 a = __ldcg(VA + r), b = __ldcg(VB + r);
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
  if (done[p]) return;  // uniform per CTA
  const JacobiProblem<T> P = probs[p];
  const int npad = P.n + (P.n & 1);
  const int R = npad - 1;
  if (round >= R) return;  // uniform per CTA
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kJacobiWarps + warp;
  int i = -1, j = -1;
  if (k < npad / 2) {
    if (k == 0) {
      i = R;
      j = round;
    } else {
      i = (round + k) % R;
      j = (round - k + R) % R;
    }
    if (i > j) {
      const int t = i;
      i = j;
      j = t;
    }
  }
  bool rotated = false;
  if (i >= 0 && j < P.n)  // j == P.n is the phantom column of an odd n
    rotated = jacobi_pair<T>(P.X + (size_t)P.ldx * i, P.X + (size_t)P.ldx * j,
                             P.V + (size_t)P.ldv * i, P.V + (size_t)P.ldv * j, P.m, P.n, lane, tol,
                             P.floor);
  const int c = __syncthreads_count(rotated && lane == 0);
  if (threadIdx.x == 0 && c) atomicAdd(&rot[p], c);
}

__global__ void k_jacobi_init(int nprob, int *rot, int *done, int *sweeps) {
  for (int p = threadIdx.x; p < nprob; p += blockDim.x) {
    rot[p] = 0;
    done[p] = 0;
    sweeps[p] = 0;
  }
}

// End of a sweep: converge problems without rotations, accumulate the work
// counters (pairs visited, rows streamed) used for roofline reporting.
template <typename T>
__global__ void k_jacobi_sweep_end(const JacobiProblem<T> *__restrict__ probs, int nprob, int *rot,
                                   int *done, int *sweeps, int *pending,
                                   unsigned long long *counters) {
  if (threadIdx.x != 0) return;
  int cnt = 0;
  unsigned long long nrot = 0, npairs = 0, rows = 0, rrows = 0;
  for (int p = 0; p < nprob; ++p) {
    if (!done[p]) {
      const unsigned long long n = (unsigned long long)probs[p].n;
      const unsigned long long pairs = n * (n - 1) / 2;
      sweeps[p] += 1;
      npairs += pairs;
      rows += pairs * (unsigned long long)probs[p].m;
      nrot += (unsigned long long)rot[p];
      rrows += (unsigned long long)rot[p] * (unsigned long long)(probs[p].m + probs[p].n);
      if (rot[p] == 0) done[p] = 1;
      rot[p] = 0;
    }
    cnt += !done[p];
  }
  counters[0] += nrot;
  counters[1] += npairs;
  counters[2] += rows;
  counters[3] += rrows;
  pending[0] = cnt;
}

// ---------------------------------------------------------------------------
// Persistent variant: one thread-block cluster per problem runs every round of
// every sweep in a single launch.  The rounds of a sweep are separated by
// cluster barriers (barrier.cluster arrive.release / wait.acquire), which order
// the global-memory column updates between the CTAs of the cluster; no launch
// per round.  The rotation count of a sweep is summed in a per-problem counter
// (two, alternating by sweep parity) that every CTA reads after the sweep's
// last barrier, so all CTAs of a cluster take the same exit decision.  The loop
// is bounded by the sweep cap; nothing spins.
// ---------------------------------------------------------------------------
constexpr int kPW = 16;  // warps per CTA of the persistent kernel

template <typename T>
__global__ void __launch_bounds__(kPW * 32)
    k_jacobi_persistent(const JacobiProblem<T> *__restrict__ probs, int *__restrict__ rotc,
                        int *__restrict__ done, int *__restrict__ sweeps,
                        unsigned long long *__restrict__ counters, T tol, int max_sweeps) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int p = blockIdx.y;
  const int crank = (int)cluster.block_rank();
  const int C = (int)cluster.num_blocks();
  const JacobiProblem<T> P = probs[p];
  const int npad = P.n + (P.n & 1), R = npad - 1, half = npad / 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = crank * kPW + warp, nw = C * kPW;
  int sw = 0, converged = (P.n < 2);
  unsigned long long nrot = 0, npairs = 0, rows = 0, rrows = 0;
  for (; sw < max_sweeps && !converged; ++sw) {
    int *cnt = rotc + 2 * p + (sw & 1);
    int local = 0;
    for (int r = 0; r < R; ++r) {
      for (int k = gw; k < half; k += nw) {
        int i, j;
        if (k == 0) {
          i = R;
          j = r;
        } else {
          i = (r + k) % R;
          j = (r - k + R) % R;
        }
        if (i > j) {
          const int t = i;
          i = j;
          j = t;
        }
        if (j < P.n &&
            jacobi_pair<T>(P.X + (size_t)P.ldx * i, P.X + (size_t)P.ldx * j, P.V + (size_t)P.ldv * i,
                           P.V + (size_t)P.ldv * j, P.m, P.n, lane, tol, P.floor))
          local += (lane == 0);
      }
      cluster.sync();
      // the other parity's counter was last read before this sweep's first barrier
      if (r == 0 && crank == 0 && threadIdx.x == 0) rotc[2 * p + ((sw + 1) & 1)] = 0;
    }
    if (local) atomicAdd(cnt, local);
    cluster.sync();
    const int total = __ldcg(cnt);
    if (crank == 0 && threadIdx.x == 0) {
      const unsigned long long pairs = (unsigned long long)P.n * (unsigned long long)(P.n - 1) / 2;
      npairs += pairs;
      rows += pairs * (unsigned long long)P.m;
      nrot += (unsigned long long)total;
      rrows += (unsigned long long)total * (unsigned long long)(P.m + P.n);
    }
    converged = (total == 0);
  }
  if (crank == 0 && threadIdx.x == 0) {
    sweeps[p] = sw;
    done[p] = converged;
    atomicAdd(&counters[0], nrot);
    atomicAdd(&counters[1], npairs);
    atomicAdd(&counters[2], rows);
    atomicAdd(&counters[3], rrows);
  }
}

// Cluster size: enough warps for the pairs of one round, at most 8 CTAs.
static int persistent_cluster_size(int nmax) {
  const int half = (nmax + (nmax & 1)) / 2;
  int c = (half + kPW - 1) / kPW;
  return c < 1 ? 1 : (c > 8 ? 8 : c);
}

template <typename T>
static int jacobi_persistent(tebd_handle *h, const JacobiProblem<T> *probs_d, int nprob, int nmax,
                             T tol, int max_sweeps) {
  cudaStream_t st = h->stream;
  int rc = check_cuda(h, cudaMemsetAsync(h->js.rot, 0, sizeof(int) * 2 * nprob, st), "reset counters");
  if (rc) return rc;
  const int C = persistent_cluster_size(nmax);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C, nprob, 1);
  cfg.blockDim = dim3(kPW * 32, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (h->profiling) cudaEventRecord(h->ev[0], st);
  rc = check_cuda(h, cudaLaunchKernelEx(&cfg, k_jacobi_persistent<T>, probs_d, h->js.rot, h->js.done,
                                        h->js.sweeps, h->js.counters, tol, max_sweeps),
                  "jacobi persistent launch");
  if (rc) return rc;
  TEBD_LAUNCHED(h);
  h->stats.jacobi_launches += 1;
  if (h->profiling) cudaEventRecord(h->ev[1], st);
  // convergence flags of the batch
  std::vector<int> dn(nprob);
  rc = check_cuda(h, cudaMemcpyAsync(dn.data(), h->js.done, sizeof(int) * nprob,
                                     cudaMemcpyDeviceToHost, st), "read convergence");
  if (rc) return rc;
  rc = check_cuda(h, cudaStreamSynchronize(st), "jacobi persistent");
  if (rc) return rc;
  if (h->profiling) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess) h->stats.jacobi_ms += ms;
  }
  for (int p = 0; p < nprob; ++p)
    if (!dn[p])
      return set_error(h, TEBD_ERR_SVD_NOCONV, "Jacobi SVD did not converge within the sweep cap");
  return TEBD_OK;
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
    if (h->profiling) cudaEventRecord(h->ev[0], st);
    for (int r = 0; r < rounds; ++r) {
      k_jacobi_round<T><<<dim3(gx, nprob), kJacobiWarps * 32, 0, st>>>(probs_d, h->js.done,
                                                                       h->js.rot, r, tol);
      TEBD_LAUNCHED(h);
    }
    h->stats.jacobi_launches += rounds;
    if (h->profiling) cudaEventRecord(h->ev[1], st);
    k_jacobi_sweep_end<T><<<1, 32, 0, st>>>(probs_d, nprob, h->js.rot, h->js.done, h->js.sweeps,
                                             h->js.pending, h->js.counters);
    TEBD_LAUNCHED(h);
    int rc = check_cuda(h, cudaMemcpyAsync(pending_h, h->js.pending, sizeof(int),
                                           cudaMemcpyDeviceToHost, st),
                        "jacobi pending copy");
    if (rc) return rc;
    rc = check_cuda(h, cudaStreamSynchronize(st), "jacobi sweep");
    if (rc) return rc;
    if (h->profiling) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess) h->stats.jacobi_ms += ms;
    }
    *sweeps_used = sw + 1;
    if (*pending_h == 0) return TEBD_OK;
  }
  return set_error(h, TEBD_ERR_SVD_NOCONV, "Jacobi SVD did not converge within the sweep cap");
}

// Dense batch: nmax = largest compacted column count of the batch (the rounds
// of smaller problems past their own n-1 return at once).
int run_jacobi(tebd_handle *h, int nb, int /*svd_mode*/, int nmax) {
  const int n = nmax;
  k_jacobi_init<<<1, 64, 0, h->stream>>>(nb, h->js.rot, h->js.done, h->js.sweeps);
  TEBD_LAUNCHED(h);
  const double tol =
      h->opts.jacobi_tol > 0 ? h->opts.jacobi_tol : (double)(n > 16 ? n : 16) * 2.220446049250313e-16;
  const int cap = h->opts.max_sweeps > 0 ? h->opts.max_sweeps : 60;
  return jacobi_persistent<double>(h, reinterpret_cast<const JacobiProblem<double> *>(h->jprob_d), nb,
                                   n, tol, cap);
}

// Generic entry used by the NC path: caller-provided problem table.
int run_jacobi_problems(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob, int nmax) {
  k_jacobi_init<<<1, 64, 0, h->stream>>>(nprob, h->js.rot, h->js.done, h->js.sweeps);
  TEBD_LAUNCHED(h);
  const double tol =
      h->opts.jacobi_tol > 0 ? h->opts.jacobi_tol : (double)(nmax > 8 ? nmax : 8) * 2.220446049250313e-16;
  const int cap = h->opts.max_sweeps > 0 ? h->opts.max_sweeps : 60;
  return jacobi_persistent<double>(h, probs_d, nprob, nmax, tol, cap);
}

// Read the device work counters into the handle's stats (called after a batch).
int jacobi_collect(tebd_handle *h) {
  unsigned long long c[4];
  int rc = check_cuda(h, cudaMemcpyAsync(c, h->js.counters, sizeof(c), cudaMemcpyDeviceToHost,
                                         h->stream), "read jacobi counters");
  if (rc) return rc;
  rc = check_cuda(h, cudaMemsetAsync(h->js.counters, 0, sizeof(c), h->stream), "reset counters");
  if (rc) return rc;
  rc = check_cuda(h, cudaStreamSynchronize(h->stream), "read jacobi counters");
  if (rc) return rc;
  h->stats.jacobi_rotations += (long long)c[0];
  h->stats.jacobi_pairs += (long long)c[1];
  // FP64 flops: 16 per row for the three dot products of every visited pair,
  // 20 per row of X and of V for every rotated pair (2 columns x 2 components x 5).
  h->stats.jacobi_flops += 16.0 * (double)c[2] + 20.0 * (double)c[3];
  // bytes: dot pass reads 2 columns; a rotation re-reads and writes the 2 columns
  // of X and of V (16 B per complex element).
  h->stats.jacobi_bytes += 32.0 * (double)c[2] + 64.0 * (double)c[3];
  return TEBD_OK;
}

// FP64 FMA throughput probe: independent fma chains, no memory traffic.
__global__ void k_fp64_peak(double *out, double a, double b, int iters) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int measure_fp64_peak(int device, double *tflops) {
  if (cudaSetDevice(device) != cudaSuccess) return TEBD_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return TEBD_ERR_CUDA;
  const int blocks = prop.multiProcessorCount * 8, threads = 256, iters = 4096;
  double *buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return TEBD_ERR_OOM;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(a);
    k_fp64_peak<<<blocks, threads>>>(buf, 0.999, 1e-3, iters);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  if (e != cudaSuccess) return TEBD_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return TEBD_OK;
}

}  // namespace tebd

namespace tebd {

// Handle-free Jacobi launches for the allocation-free entry point (noalloc.cu).
void raw_jacobi_init(cudaStream_t st, int *rot, int *done, int *sweeps) {
  k_jacobi_init<<<1, 64, 0, st>>>(1, rot, done, sweeps);
}

void raw_jacobi_sweep(cudaStream_t st, const JacobiProblem<double> *probs_d, int *rot, int *done,
                      int *sweeps, int *pending, unsigned long long *counters, int nmax,
                      double tol) {
  const int npad = nmax + (nmax & 1);
  const unsigned gx = (unsigned)((npad / 2 + kJacobiWarps - 1) / kJacobiWarps);
  for (int r = 0; r < npad - 1; ++r)
    k_jacobi_round<double><<<dim3(gx, 1), kJacobiWarps * 32, 0, st>>>(probs_d, done, rot, r, tol);
  k_jacobi_sweep_end<double><<<1, 32, 0, st>>>(probs_d, 1, rot, done, sweeps, pending, counters);
}

}  // namespace tebd

namespace tebd {

// Non-template entry for the QR-preconditioned path (qrj.cu).
int jacobi_persistent_double(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob,
                             int nmax, double tol, int max_sweeps) {
  return jacobi_persistent<double>(h, probs_d, nprob, nmax, tol, max_sweeps);
}

}  // namespace tebd
