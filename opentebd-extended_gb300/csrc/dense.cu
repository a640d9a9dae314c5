// dense.cu -- HBM/L2 passes and the Theta contraction of the dense two-site update.
//
// Replaces, for a batch of same-parity bonds at once (one grid z/y index per bond):
//   FormTheta      local_operations_module.f90:184-211   -> k_theta_form
//   ThetaOperation local_operations_module.f90:213-280   -> k_gate_apply
//   ReshapeTheta   local_operations_module.f90:283-320   -> k_theta_form's permuted store
//                                                            + k_norm_partial/k_norm_final
//   FormLambda1    local_operations_module.f90:347-379   -> k_sigma_sort + k_lambda
//   FormGamma1     local_operations_module.f90:381-404   -> k_restore_gamma1
//   FormGamma2     local_operations_module.f90:406-428   -> k_restore_gamma2
//
// Theta is built directly in the reshaped (d chi) x (d chi) layout of ReshapeTheta:
// row (i-1)chi+alpha, column (j-1)chi+beta (1-based), column-major, ld = n = d*chi.
// The 1/||Theta|| scaling of ReshapeTheta is not applied to the matrix: the SVD
// factors do not depend on it, and the singular values are divided by the norm.
#include <math.h>

#include "tebd_internal.cuh"

namespace tebd {

// ---------------------------------------------------------------------------
// Theta = diag(l0) G1 diag(l1) G2 diag(l2) as a complex FP64 GEMM.
// A[r, g] = l0[r%chi] G1[r + n g]          (n x chi, the Gamma1 array as-is)
// B[g, c] = l1[g] G2[g + chi c] l2[c/d]    (chi x n, the Gamma2 array as-is)
// C[r, c] is stored at X[r + n*((c%d)*chi + c/d)] (ReshapeTheta's column order).
// Tile 64x64 outputs, k-step 8, 256 threads, 4x4 complex outputs per thread.
// ---------------------------------------------------------------------------
constexpr int TT_M = 64, TT_N = 64, TT_K = 8;

__global__ void __launch_bounds__(256) k_theta_form(const double2 *__restrict__ gam,
                                                    const double *__restrict__ lam,
                                                    const int *__restrict__ links, Slot *slots,
                                                    int chi, int d) {
  const int n = chi * d;
  const int s = blockIdx.z;
  const int link = links[s];  // 1-based
  const size_t csz = (size_t)chi * d * chi;
  const double2 *G1 = gam + (size_t)(link - 1) * csz;
  const double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l1 = lam + (size_t)link * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  double2 *X = slots[s].X;

  __shared__ double2 As[TT_K][TT_M + 1];
  __shared__ double2 Bs[TT_K][TT_N + 1];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;  // 16 x 16 thread grid, 4x4 outputs each
  const int r0 = blockIdx.x * TT_M, c0 = blockIdx.y * TT_N;
  double2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);

  for (int k0 = 0; k0 < chi; k0 += TT_K) {
    // A tile: 64 rows x 8 k  (512 elements, 2 per thread), coalesced along rows
    for (int e = tid; e < TT_M * TT_K; e += 256) {
      const int rr = e % TT_M, kk = e / TT_M;
      const int r = r0 + rr, g = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (r < n && g < chi) v = cscale(G1[r + (size_t)n * g], l0[r % chi]);
      As[kk][rr] = v;
    }
    // B tile: 8 k x 64 cols, coalesced along k (the Gamma2 leading dimension)
    for (int e = tid; e < TT_K * TT_N; e += 256) {
      const int kk = e % TT_K, cc = e / TT_K;
      const int g = k0 + kk, c = c0 + cc;
      double2 v = make_double2(0.0, 0.0);
      if (g < chi && c < n) v = cscale(G2[g + (size_t)chi * c], l1[g] * l2[c / d]);
      Bs[kk][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TT_K; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][tr + 16 * q];
        b[q] = Bs[kk][tc + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          acc[p][q].x = fma(a[p].x, b[q].x, acc[p][q].x);
          acc[p][q].x = fma(-a[p].y, b[q].y, acc[p][q].x);
          acc[p][q].y = fma(a[p].x, b[q].y, acc[p][q].y);
          acc[p][q].y = fma(a[p].y, b[q].x, acc[p][q].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int r = r0 + tr + 16 * p;
    if (r >= n) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + tc + 16 * q;
      if (c >= n) continue;
      const int lphys = c % d, beta = c / d;
      X[r + (size_t)n * ((size_t)lphys * chi + beta)] = acc[p][q];
    }
  }
}

// ---------------------------------------------------------------------------
// ThetaOperation: for every (alpha, beta) the d^2-vector Theta(alpha,:,:,beta)
// is multiplied by Op2 (row (i-1)d+j, column (k-1)d+l).  In place.
// ---------------------------------------------------------------------------
constexpr int kMaxD = 8;

__global__ void __launch_bounds__(128) k_gate_apply(Slot *slots, int chi, int d) {
  extern __shared__ double2 gsm[];  // d^4
  const int s = blockIdx.y;
  const int n = chi * d, d2 = d * d;
  const double2 *G = slots[s].gate;
  for (int e = threadIdx.x; e < d2 * d2; e += blockDim.x) gsm[e] = G[e];
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= chi * chi) return;
  const int alpha = t % chi, beta = t / chi;
  double2 *X = slots[s].X;
  double2 v[kMaxD * kMaxD];
  for (int k = 0; k < d; ++k)
    for (int l = 0; l < d; ++l)
      v[k * d + l] = X[(size_t)(k * chi + alpha) + (size_t)n * (l * chi + beta)];
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) {
      const int row = i * d + j;
      double2 acc = make_double2(0.0, 0.0);
      for (int kl = 0; kl < d2; ++kl) {
        const double2 g = gsm[row + d2 * kl];
        acc.x = fma(g.x, v[kl].x, acc.x);
        acc.x = fma(-g.y, v[kl].y, acc.x);
        acc.y = fma(g.x, v[kl].y, acc.y);
        acc.y = fma(g.y, v[kl].x, acc.y);
      }
      X[(size_t)(i * chi + alpha) + (size_t)n * (j * chi + beta)] = acc;
    }
}

// ---------------------------------------------------------------------------
// Frobenius norm of Theta, deterministic two-level reduction (fixed order).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_norm_partial(Slot *slots, int n, double *part) {
  const int s = blockIdx.y;
  const size_t total = (size_t)n * n;
  const size_t chunk = (total + kNormParts - 1) / kNormParts;
  const size_t beg = blockIdx.x * chunk;
  const size_t end = beg + chunk < total ? beg + chunk : total;
  const double2 *X = slots[s].X;
  double acc = 0.0;
  for (size_t e = beg + threadIdx.x; e < end; e += blockDim.x) {
    const double2 v = X[e];
    acc = fma(v.x, v.x, fma(v.y, v.y, acc));
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[s * kNormParts + blockIdx.x] = red[0];
}

__global__ void k_norm_final(const double *part, double *nrm, int nb, int *status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nb) return;
  double acc = 0.0;
  for (int j = 0; j < kNormParts; ++j) acc += part[s * kNormParts + j];
  const double v = sqrt(acc);
  nrm[s] = v;
  if (!isfinite(v)) atomicOr(&status[0], 1);
}

// V = identity (n x n) for every slot
__global__ void k_eye(Slot *slots, int n) {
  const int s = blockIdx.y;
  double2 *V = slots[s].V;
  const size_t total = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e % n, c = e / n;
    V[e] = make_double2(r == c ? 1.0 : 0.0, 0.0);
  }
}

// ---------------------------------------------------------------------------
// After the SVD: column norms of X = U Sigma, descending order (rank sort,
// ties broken by column index), normalised singular values S = sigma/||Theta||.
// One CTA per slot, one warp per column for the norms.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_sigma_sort(Slot *slots, const double *nrm, int n,
                                                     int *status) {
  extern __shared__ double sig[];  // n
  const int s = blockIdx.x;
  const double2 *X = slots[s].X;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = warp; c < n; c += nw) {
    double acc = 0.0;
    for (int r = lane; r < n; r += 32) {
      const double2 v = X[r + (size_t)n * c];
      acc = fma(v.x, v.x, fma(v.y, v.y, acc));
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) sig[c] = sqrt(acc);
  }
  __syncthreads();
  const double inv = 1.0 / nrm[s];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double v = sig[k];
    if (!isfinite(v)) atomicOr(&status[0], 1);
    int rank = 0;
    for (int m = 0; m < n; ++m) {
      const double w = sig[m];
      rank += (w > v) || (w == v && m < k);
    }
    slots[s].perm[rank] = k;
    slots[s].S[rank] = v * inv;
  }
}

// FormLambda1 (:347-379): sequential in the reference's order, one thread per slot.
__global__ void k_lambda(Slot *slots, const int *links, double *lam, double *truncerr, int chi,
                         int nb) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nb) return;
  const double *S = slots[s].S;
  double norm = 0.0;
  for (int a = 0; a < chi; ++a)
    if (fabs(S[a]) > kGuardDense) norm = norm + S[a] * S[a];
  truncerr[s] = fabs(1.0 - norm);
  double *l1 = lam + (size_t)links[s] * chi;
  const double rs = sqrt(norm);
  for (int a = 0; a < chi; ++a) l1[a] = (fabs(S[a]) > kGuardDense) ? S[a] / rs : 0.0;
}

// Keep the last spectrum and sweep count of every link for tebd_get_singular_values.
__global__ void k_store_spectrum(Slot *slots, const int *links, const int *sweeps, double *sig_link,
                                 int *sig_count, int *sweeps_link, int n) {
  const int s = blockIdx.x;
  const int link = links[s];
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    sig_link[(size_t)(link - 1) * n + k] = slots[s].S[k];
  if (threadIdx.x == 0) {
    sig_count[link - 1] = n;
    sweeps_link[link - 1] = sweeps[s];
  }
}

// FormGamma1 (:381-404): Gamma1(alpha,i,beta) = U((i-1)chi+alpha, beta) / Lambda0(alpha)
// with U(:,beta) = X(:,perm(beta)) / sigma(perm(beta)).  Same linear index on both sides.
__global__ void k_restore_gamma1(double2 *gam, const double *lam, const int *links, Slot *slots,
                                 const double *nrm, int chi, int d) {
  const int s = blockIdx.y;
  const int n = chi * d;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * chi) return;
  const int link = links[s];
  const int r = (int)(t % n), beta = (int)(t / n);
  const int alpha = r % chi;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const int col = slots[s].perm[beta];
  const double sigma = slots[s].S[beta] * nrm[s];
  double2 out = make_double2(0.0, 0.0);
  if (fabs(l0[alpha]) > kGuardDense && sigma > 0.0) {
    const double2 x = slots[s].X[r + (size_t)n * col];
    const double sc = 1.0 / (sigma * l0[alpha]);
    out = make_double2(x.x * sc, x.y * sc);
  }
  gam[(size_t)(link - 1) * chi * d * chi + t] = out;
}

// FormGamma2 (:406-428): Gamma2(alpha,i,beta) = VT(alpha,(i-1)chi+beta) / Lambda2(beta),
// VT = V^H, i.e. conj(V((i-1)chi+beta, perm(alpha))).  32x32 tile transpose through smem.
__global__ void __launch_bounds__(256) k_restore_gamma2(double2 *gam, const double *lam,
                                                        const int *links, Slot *slots, int chi,
                                                        int d) {
  __shared__ double2 tile[32][33];
  const int s = blockIdx.z;
  const int n = chi * d;
  const int link = links[s];
  const int a0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const double2 *V = slots[s].V;
  const int *perm = slots[s].perm;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int yy = ty; yy < 32; yy += 8) {
    const int alpha = a0 + yy, c = c0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (alpha < chi && c < n) v = V[c + (size_t)n * perm[alpha]];
    tile[yy][tx] = v;
  }
  __syncthreads();
  const double *l2 = lam + (size_t)(link + 1) * chi;
  double2 *G2 = gam + (size_t)link * chi * d * chi;
  for (int yy = ty; yy < 32; yy += 8) {
    const int c = c0 + yy, alpha = a0 + tx;
    if (alpha >= chi || c >= n) continue;
    const int i = c / chi, beta = c % chi;
    const double2 v = tile[tx][yy];
    double2 out = make_double2(0.0, 0.0);
    if (fabs(l2[beta]) > kGuardDense) {
      const double inv = 1.0 / l2[beta];
      out = make_double2(v.x * inv, -v.y * inv);
    }
    G2[alpha + (size_t)chi * i + (size_t)n * beta] = out;
  }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

int launch_dense_prepare(tebd_handle *h, int nb, bool /*real_gate: converted on the host*/) {
  const int chi = h->chi, d = h->d, n = h->n;
  cudaStream_t st = h->stream;
  k_theta_form<<<dim3(cdiv(n, TT_M), cdiv(n, TT_N), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                       h->slots_d, chi, d);
  TEBD_LAUNCHED(h);
  const size_t gsm = sizeof(double2) * (size_t)d * d * d * d;
  k_gate_apply<<<dim3(cdiv((size_t)chi * chi, 128), nb), 128, gsm, st>>>(h->slots_d, chi, d);
  TEBD_LAUNCHED(h);
  k_norm_partial<<<dim3(kNormParts, nb), 256, 0, st>>>(h->slots_d, n, h->nrm_part);
  TEBD_LAUNCHED(h);
  k_norm_final<<<cdiv(nb, 128), 128, 0, st>>>(h->nrm_part, h->nrm, nb, h->status_d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "dense prepare launch");
}

int launch_eye(tebd_handle *h, int nb) {
  const size_t total = (size_t)h->n * h->n;
  unsigned gx = cdiv(total, 256);
  if (gx > 1024) gx = 1024;
  k_eye<<<dim3(gx, nb), 256, 0, h->stream>>>(h->slots_d, h->n);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "eye launch");
}

int launch_dense_finish(tebd_handle *h, int nb) {
  const int chi = h->chi, d = h->d, n = h->n;
  cudaStream_t st = h->stream;
  k_sigma_sort<<<nb, 1024, sizeof(double) * n, st>>>(h->slots_d, h->nrm, n, h->status_d);
  TEBD_LAUNCHED(h);
  k_lambda<<<cdiv(nb, 64), 64, 0, st>>>(h->slots_d, h->links_d, h->lam, h->truncerr_d, chi, nb);
  TEBD_LAUNCHED(h);
  k_store_spectrum<<<nb, 256, 0, st>>>(h->slots_d, h->links_d, h->js.sweeps, h->sig_link_d,
                                       h->sig_count_d, h->sweeps_link_d, n);
  TEBD_LAUNCHED(h);
  k_restore_gamma1<<<dim3(cdiv((size_t)n * chi, 256), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                       h->slots_d, h->nrm, chi, d);
  TEBD_LAUNCHED(h);
  k_restore_gamma2<<<dim3(cdiv(chi, 32), cdiv(n, 32), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                        h->slots_d, chi, d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "dense finish launch");
}

}  // namespace tebd
