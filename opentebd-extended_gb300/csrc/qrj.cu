// qrj.cu -- SVD of the compacted Theta by rank-revealing QR + one-sided Jacobi.
//
// Replaces SVDTruncation's ZGESVD('A','A') (local_operations_module.f90:322-345)
// for the dense update.  The algorithm is the preconditioned Jacobi SVD of
// Drmac and Veselic (the method behind LAPACK's xGEJSV):
//   1. Householder QR with column pivoting, Theta P = Q R (ZGEQP3 semantics:
//      largest remaining column first, ZLARFG reflectors, column-norm
//      downdating with recomputation on cancellation), stopped at the numerical
//      rank k: the first step whose largest remaining column norm is below
//      2^-60 ||Theta||_F.  The neglected block has norm <= sqrt(n) 2^-60 ||Theta||,
//      three decades under the reference's 1e-15 Lambda guard.
//   2. One-sided Jacobi on A = R^H (n x k): A Z = W Sigma, converging in a few
//      sweeps because pivoted QR has already graded the columns.
//   3. Theta = (Q Z) Sigma (P W)^H:  U = Q [Z; 0] (reflectors applied in reverse),
//      V = P W (rows of W permuted back to Theta's column order).
// Every step is FP64.  The work is O(m n k) for the QR and O(n k^2) per Jacobi
// sweep instead of O(n^3) per sweep, and k is the Schmidt rank of the bond,
// which is far below d*chi until the chain saturates.
//
// Kernel shapes: one thread-block cluster per bond for the QR (cluster barriers
// between the pivot choice, the reflector and the trailing update of each step;
// the loop is bounded by min(m, n)), then per-column warps for the remaining passes.
#include <cooperative_groups.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "tebd_internal.cuh"

namespace tebd {

int jacobi_persistent_double(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob,
                             int nmax, double tol, int max_sweeps);

namespace {
constexpr int kQW = 16;  // warps per CTA of the QR kernel

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }
}  // namespace

// ---------------------------------------------------------------------------
// 1. column-pivoted Householder QR, in place on the slot's X (m x n, ld m)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kQW * 32) k_qrp(Slot *slots, const double *nrm, const int *path) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int s = blockIdx.y;
  if (path[s] != kPathQRJ) return;  // uniform per cluster
  const Slot S = slots[s];
  const Compact cp = *S.cp;
  const int m = cp.m, n = cp.n, kmax = min(m, n);
  double2 *X = S.X;
  double *vn1 = S.vn, *vn2 = S.vn + n;
  const int crank = (int)cluster.block_rank(), C = (int)cluster.num_blocks();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = crank * kQW + warp, nw = C * kQW;
  const double tol = kNegligibleColumn * nrm[s];
  const double tol3z = sqrt(2.220446049250313e-16);
  __shared__ int s_piv;
  __shared__ double s_max;
  // column norms and the identity permutation
  for (int c = gw; c < n; c += nw) {
    double acc = 0.0;
    for (int r = lane; r < m; r += 32) {
      const double2 v = __ldcg(X + r + (size_t)m * c);
      acc = fma(v.x, v.x, fma(v.y, v.y, acc));
    }
    acc = sqrt(wsum(acc));
    if (lane == 0) {
      vn1[c] = acc;
      vn2[c] = acc;
      S.jpvt[c] = c;
    }
  }
  cluster.sync();
  int k = kmax;
  for (int j = 0; j < kmax; ++j) {
    // A. pivot: first column of largest remaining norm (every CTA computes the same)
    if (warp == 0) {
      double best = -1.0;
      int bi = n;
      for (int c = j + lane; c < n; c += 32) {
        const double v = __ldcg(vn1 + c);
        if (v > best || (v == best && c < bi)) {
          best = v;
          bi = c;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        s_piv = bi;
        s_max = best;
      }
    }
    __syncthreads();
    const int pv = s_piv;
    const double mx = s_max;
    cluster.sync();  // everyone has read vn1 before the swap below
    if (!(mx > tol)) {
      k = j;
      break;
    }
    // B. swap columns j <-> pv and build the reflector of column j (one warp)
    if (crank == 0 && warp == 0) {
      if (pv != j) {
        for (int r = lane; r < m; r += 32) {
          const double2 a = __ldcg(X + r + (size_t)m * j), b = __ldcg(X + r + (size_t)m * pv);
          X[r + (size_t)m * j] = b;
          X[r + (size_t)m * pv] = a;
        }
        if (lane == 0) {
          const int t = __ldcg(S.jpvt + j);
          S.jpvt[j] = __ldcg(S.jpvt + pv);
          S.jpvt[pv] = t;
          double tv = __ldcg(vn1 + j);
          vn1[j] = __ldcg(vn1 + pv);
          vn1[pv] = tv;
          tv = __ldcg(vn2 + j);
          vn2[j] = __ldcg(vn2 + pv);
          vn2[pv] = tv;
        }
        __syncwarp();
      }
      // ZLARFG on (alpha = X[j,j], x = X[j+1:, j])
      double acc = 0.0;
      for (int r = j + 1 + lane; r < m; r += 32) {
        const double2 v = __ldcg(X + r + (size_t)m * j);
        acc = fma(v.x, v.x, fma(v.y, v.y, acc));
      }
      const double xnorm = sqrt(wsum(acc));
      const double2 alpha = __ldcg(X + j + (size_t)m * j);
      double2 tau = make_double2(0.0, 0.0);
      if (!(xnorm == 0.0 && alpha.y == 0.0)) {
        const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm), alpha.x);
        tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
        // scale = 1 / (alpha - beta)
        const double dr = alpha.x - beta, di = alpha.y;
        const double den = dr * dr + di * di;
        const double2 sc = make_double2(dr / den, -di / den);
        for (int r = j + 1 + lane; r < m; r += 32) {
          const double2 v = __ldcg(X + r + (size_t)m * j);
          X[r + (size_t)m * j] = make_double2(v.x * sc.x - v.y * sc.y, v.x * sc.y + v.y * sc.x);
        }
        if (lane == 0) X[j + (size_t)m * j] = make_double2(beta, 0.0);
      }
      if (lane == 0) S.tau[j] = tau;
    }
    cluster.sync();
    // C. apply H^H = I - conj(tau) v v^H to columns j+1..n-1, then downdate norms
    const double2 tau = __ldcg(&S.tau[j]);
    for (int c = j + 1 + gw; c < n; c += nw) {
      double wr = 0.0, wi = 0.0;  // w = v^H x, v_j = 1
      for (int r = j + lane; r < m; r += 32) {
        const double2 x = __ldcg(X + r + (size_t)m * c);
        const double2 v = r == j ? make_double2(1.0, 0.0) : __ldcg(X + r + (size_t)m * j);
        wr = fma(v.x, x.x, fma(v.y, x.y, wr));
        wi = fma(v.x, x.y, fma(-v.y, x.x, wi));
      }
      wr = wsum(wr);
      wi = wsum(wi);
      // f = conj(tau) * w
      const double fr = tau.x * wr + tau.y * wi, fi = tau.x * wi - tau.y * wr;
      for (int r = j + lane; r < m; r += 32) {
        const double2 v = r == j ? make_double2(1.0, 0.0) : __ldcg(X + r + (size_t)m * j);
        double2 x = __ldcg(X + r + (size_t)m * c);
        x.x -= v.x * fr - v.y * fi;
        x.y -= v.x * fi + v.y * fr;
        X[r + (size_t)m * c] = x;
      }
      __syncwarp();
      const double v1 = __ldcg(vn1 + c), v2 = __ldcg(vn2 + c);
      if (v1 != 0.0) {  // ZLAQP2 norm downdate
        const double2 xj = __ldcg(X + j + (size_t)m * c);
        double temp = sqrt(xj.x * xj.x + xj.y * xj.y) / v1;
        temp = 1.0 - temp * temp;
        temp = temp > 0.0 ? temp : 0.0;
        const double r2 = v1 / v2;
        const double temp2 = temp * r2 * r2;
        double nv;
        if (temp2 <= tol3z) {
          double acc = 0.0;
          for (int r = j + 1 + lane; r < m; r += 32) {
            const double2 v = __ldcg(X + r + (size_t)m * c);
            acc = fma(v.x, v.x, fma(v.y, v.y, acc));
          }
          nv = sqrt(wsum(acc));
          if (lane == 0) vn2[c] = nv;
        } else {
          nv = v1 * sqrt(temp);
        }
        __syncwarp();
        if (lane == 0) vn1[c] = nv;
      }
    }
    cluster.sync();
  }
  if (crank == 0 && threadIdx.x == 0) S.cp->k = k;
}

// ---------------------------------------------------------------------------
// 2. A = R^H (n x k, ld n) and Z = I (k x k, ld k); Jacobi problem of the slot
// ---------------------------------------------------------------------------
__global__ void k_qrj_build(Slot *slots, JacobiProblem<double> *jp, const double *nrm,
                            const int *path) {
  const int s = blockIdx.y;
  if (path[s] != kPathQRJ) {  // the bidiagonal route: no Jacobi problem for this slot
    if (blockIdx.x == 0 && threadIdx.x == 0) jp[s].n = 0;
    return;
  }
  const Slot S = slots[s];
  const Compact cp = *S.cp;
  const int m = cp.m, n = cp.n, k = cp.k;
  double2 *A = S.aux, *Z = S.aux + (size_t)n * n;
  const size_t tot = (size_t)n * k + (size_t)k * k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < (size_t)n * k) {
      const int c = (int)(e % n), r = (int)(e / n);  // A[c, r] = conj(R[r, c])
      double2 v = make_double2(0.0, 0.0);
      if (r <= c) {
        const double2 x = S.X[r + (size_t)m * c];
        v = make_double2(x.x, -x.y);
      }
      A[e] = v;
    } else {
      const size_t f = e - (size_t)n * k;
      Z[f] = make_double2((f % k) == (f / k) ? 1.0 : 0.0, 0.0);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    JacobiProblem<double> P;
    P.X = A;
    P.V = Z;
    P.m = n;
    P.n = k;
    P.ldx = n > 0 ? n : 1;
    P.ldv = k > 0 ? k : 1;
    const double f = kNegligibleColumn * nrm[s];
    P.floor = f * f;
    jp[s] = P;
  }
}

// ---------------------------------------------------------------------------
// 3a. Y = Q [Z; 0] (m x k, ld m), one warp per column; sigma_i = |A(:,i)|
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_qrj_apply_q(Slot *slots, const int *path) {
  const int s = blockIdx.y;
  if (path[s] != kPathQRJ) return;
  const Slot S = slots[s];
  const Compact cp = *S.cp;
  const int m = cp.m, n = cp.n, k = cp.k;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + warp;
  if (i >= k) return;
  const double2 *A = S.aux, *Z = S.aux + (size_t)n * n;
  double2 *Y = S.aux + 2 * (size_t)n * n;
  double acc = 0.0;
  for (int r = lane; r < n; r += 32) {
    const double2 v = A[r + (size_t)n * i];
    acc = fma(v.x, v.x, fma(v.y, v.y, acc));
  }
  acc = sqrt(wsum(acc));
  if (lane == 0) S.vn[i] = acc;  // sigma_i (vn is free after the QR)
  for (int r = lane; r < m; r += 32)
    Y[r + (size_t)m * i] = r < k ? Z[r + (size_t)k * i] : make_double2(0.0, 0.0);
  __syncwarp();
  for (int j = k - 1; j >= 0; --j) {  // Q Y = H_0 (H_1 (... H_{k-1} Y))
    const double2 tau = S.tau[j];
    double wr = 0.0, wi = 0.0;
    for (int r = j + lane; r < m; r += 32) {
      const double2 y = Y[r + (size_t)m * i];
      const double2 v = r == j ? make_double2(1.0, 0.0) : S.X[r + (size_t)m * j];
      wr = fma(v.x, y.x, fma(v.y, y.y, wr));
      wi = fma(v.x, y.y, fma(-v.y, y.x, wi));
    }
    wr = wsum(wr);
    wi = wsum(wi);
    const double fr = tau.x * wr - tau.y * wi, fi = tau.x * wi + tau.y * wr;  // tau * w
    for (int r = j + lane; r < m; r += 32) {
      const double2 v = r == j ? make_double2(1.0, 0.0) : S.X[r + (size_t)m * j];
      double2 y = Y[r + (size_t)m * i];
      y.x -= v.x * fr - v.y * fi;
      y.y -= v.x * fi + v.y * fr;
      Y[r + (size_t)m * i] = y;
    }
    __syncwarp();
  }
}

// 3b. X(:, i) = Y(:, i) sigma_i  (= U Sigma, what the sort/restore kernels read)
//     V(jpvt(c), i) = A(c, i) / sigma_i (= P W)
__global__ void k_qrj_store(Slot *slots, const int *path) {
  const int s = blockIdx.y;
  if (path[s] != kPathQRJ) return;
  const Slot S = slots[s];
  const Compact cp = *S.cp;
  const int m = cp.m, n = cp.n, k = cp.k;
  const double2 *A = S.aux, *Y = S.aux + 2 * (size_t)n * n;
  const size_t tot = (size_t)m * k + (size_t)n * k;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    if (e < (size_t)m * k) {
      const int i = (int)(e / m);
      const double sg = S.vn[i];
      const double2 y = Y[e];
      S.X[e] = make_double2(y.x * sg, y.y * sg);
    } else {
      const size_t f = e - (size_t)m * k;
      const int c = (int)(f % n), i = (int)(f / n);
      const double sg = S.vn[i];
      const double2 a = A[f];
      S.V[(size_t)S.jpvt[c] + (size_t)n * i] =
          sg > 0.0 ? make_double2(a.x / sg, a.y / sg) : make_double2(0.0, 0.0);
    }
  }
}

// ---------------------------------------------------------------------------
// host orchestration (dense batch, after launch_dense_prepare)
// ---------------------------------------------------------------------------
static int qr_cluster_size(int nmax) {
  int c = (nmax + kQW * 8 - 1) / (kQW * 8);  // ~8 columns per warp per step
  return c < 1 ? 1 : (c > 8 ? 8 : c);
}

int run_qrj(tebd_handle *h, int nb, int nmax) {
  cudaStream_t st = h->stream;
  int rc;
  // 1. QR with column pivoting
  {
    const int C = qr_cluster_size(nmax);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C, nb, 1);
    cfg.blockDim = dim3(kQW * 32, 1, 1);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (h->profiling) cudaEventRecord(h->ev[0], st);
    rc = check_cuda(h, cudaLaunchKernelEx(&cfg, k_qrp, h->slots_d, (const double *)h->nrm,
                                          (const int *)h->path_d), "QR launch");
    if (rc) return rc;
    TEBD_LAUNCHED(h);
    if (h->profiling) cudaEventRecord(h->ev[1], st);
  }
  // ranks of the batch
  std::vector<Compact> cp(nb);
  rc = check_cuda(h, cudaMemcpyAsync(cp.data(), h->cp_d, sizeof(Compact) * nb, cudaMemcpyDeviceToHost, st),
                  "read ranks");
  if (rc) return rc;
  rc = check_cuda(h, cudaStreamSynchronize(st), "QR");
  if (rc) return rc;
  if (h->profiling) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess) h->stats.qr_ms += ms;
  }
  int kmax = 0;
  size_t maxnk = 1, maxmk = 1;
  for (int s = 0; s < nb; ++s) {
    if (h->path_h[s] != kPathQRJ) continue;
    const double m = cp[s].m, n = cp[s].n, k = cp[s].k;
    kmax = std::max(kmax, cp[s].k);
    maxnk = std::max(maxnk, (size_t)(n * k + k * k));
    maxmk = std::max(maxmk, (size_t)(m * k + n * k));
    // 16 flop per element of each reflector application: w = v^H x and x -= f v
    h->stats.qr_flops += 16.0 * (k * m * n - (m + n) * k * (k - 1) / 2.0 + k * (k - 1) * (2 * k - 1) / 6.0);
    h->stats.qr_flops += 16.0 * m * k * k;  // U = Q [Z; 0] (upper bound)
    h->stats.rank_sum += cp[s].k;
  }
  // 2. Jacobi on R^H
  JacobiProblem<double> *jp = reinterpret_cast<JacobiProblem<double> *>(h->jprob_d);
  unsigned gx = cdiv(maxnk, 256);
  if (gx > 512) gx = 512;
  k_qrj_build<<<dim3(gx, nb), 256, 0, st>>>(h->slots_d, jp, h->nrm, h->path_d);
  TEBD_LAUNCHED(h);
  const double tol = h->opts.jacobi_tol > 0 ? h->opts.jacobi_tol
                                            : (double)(kmax > 16 ? kmax : 16) * 2.220446049250313e-16;
  const int cap = h->opts.max_sweeps > 0 ? h->opts.max_sweeps : 60;
  if ((rc = jacobi_persistent_double(h, jp, nb, kmax, tol, cap))) return rc;
  // 3. U and V
  k_qrj_apply_q<<<dim3(cdiv(kmax > 0 ? kmax : 1, 8), nb), 256, 0, st>>>(h->slots_d, h->path_d);
  TEBD_LAUNCHED(h);
  gx = cdiv(maxmk, 256);
  if (gx > 512) gx = 512;
  k_qrj_store<<<dim3(gx, nb), 256, 0, st>>>(h->slots_d, h->path_d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "QRJ launch");
}

}  // namespace tebd
