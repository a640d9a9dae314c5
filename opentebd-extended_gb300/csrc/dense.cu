// dense.cu -- HBM/L2 passes and the Theta contraction of the dense two-site update.
//
// Replaces, for a batch of same-parity bonds at once (one grid y/z index per bond):
//   FormTheta      local_operations_module.f90:184-211   -> k_theta_form
//   ThetaOperation local_operations_module.f90:213-280   -> k_gate_apply
//   ReshapeTheta   local_operations_module.f90:283-320   -> k_theta_form's permuted store
//                                                            + k_norm_partial/k_norm_final
//   FormLambda1    local_operations_module.f90:347-379   -> k_sigma_sort + k_lambda
//   FormGamma1     local_operations_module.f90:381-404   -> k_restore_gamma1
//   FormGamma2     local_operations_module.f90:406-428   -> k_restore_gamma2
//
// Theta is built directly in ReshapeTheta's matrix layout (row (i-1)chi+alpha,
// column (j-1)chi+beta), restricted to the kept indices of the Compact record:
// row i*r0 + a', column j*r2 + b', column-major with ld = m = d*r0.  Rows and
// columns of exact-zero Lambdas are identically zero in the reference's Theta,
// so the singular values are the same; the dropped ones are exact zeros.
// The 1/||Theta|| scaling of ReshapeTheta is not applied to the matrix: the SVD
// factors do not depend on it and the singular values are divided by the norm.
#include <math.h>

#include "df.cuh"
#include "tebd_internal.cuh"

namespace tebd {

// ---------------------------------------------------------------------------
// Compaction record and index maps (one CTA per slot, warp-ballot prefix scans).
// Also fills the slot's FP64 Jacobi problem (m, n, ld).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(96) k_compact(const double *__restrict__ lam, const int *links,
                                                Slot *slots, JacobiProblem<double> *jp, int chi,
                                                int d) {
  const int s = blockIdx.x;
  const int link = links[s];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double *l = lam + (size_t)(link - 1 + w) * chi;  // w=0: Lambda0, 1: Lambda1, 2: Lambda2
  int *idx = w == 0 ? slots[s].idx0 : (w == 1 ? slots[s].idx1 : slots[s].idx2);
  int *inv = w == 0 ? slots[s].inv0 : (w == 2 ? slots[s].inv2 : nullptr);
  int count = 0;
  for (int base = 0; base < chi; base += 32) {
    const int a = base + lane;
    const bool keep = a < chi && l[a] != 0.0;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int pos = count + __popc(m & ((1u << lane) - 1u));
    if (keep) idx[pos] = a;
    if (inv && a < chi) inv[a] = keep ? pos : -1;
    count += __popc(m);
  }
  __shared__ int cnt[3];
  if (lane == 0) cnt[w] = count;
  __syncthreads();
  if (threadIdx.x == 0) {
    Compact c;
    c.r0 = cnt[0];
    c.r1 = cnt[1];
    c.r2 = cnt[2];
    c.m = d * cnt[0];
    c.n = d * cnt[2];
    c.k = c.n;
    const double *l1 = lam + (size_t)link * chi;
    double lo = 0.0, hi = 0.0;
    for (int a = 0; a < chi; ++a)
      if (l1[a] != 0.0) {
        const double v = fabs(l1[a]);
        lo = (lo == 0.0 || v < lo) ? v : lo;
        hi = v > hi ? v : hi;
      }
    c.span = hi > 0.0 ? (float)(lo / hi) : 0.f;
    *slots[s].cp = c;
    jp[s].m = c.m;
    jp[s].n = c.n;
    jp[s].ldx = c.m > 0 ? c.m : 1;
    jp[s].ldv = c.n > 0 ? c.n : 1;
  }
}

// ---------------------------------------------------------------------------
// Theta = diag(l0) G1 diag(l1) G2 diag(l2) on the kept indices, complex FP64 GEMM.
// A[r', g'] = l0[a] G1[a + chi*i + chi*d*g]   r' = i*r0 + a', a = idx0[a'], g = idx1[g']
// B[g', c'] = l1[g] G2[g + chi*l + chi*d*b] l2[b]   c' = l + d*b', b = idx2[b']
// C[r', c'] is stored at X[r' + m*(l*r2 + b')].
// Tile 64x64 outputs, k-step 8, 256 threads, 4x4 complex outputs per thread.
// ---------------------------------------------------------------------------
constexpr int TT_M = 64, TT_N = 64, TT_K = 8;

__global__ void __launch_bounds__(256) k_theta_form(const double2 *__restrict__ gam,
                                                    const double *__restrict__ lam,
                                                    const int *__restrict__ links, Slot *slots,
                                                    int chi, int d) {
  const int s = blockIdx.z;
  const Compact cp = *slots[s].cp;
  const int r0b = blockIdx.x * TT_M, c0b = blockIdx.y * TT_N;
  if (r0b >= cp.m || c0b >= cp.n) return;  // uniform per CTA
  const int link = links[s];
  const size_t csz = (size_t)chi * d * chi;
  const double2 *G1 = gam + (size_t)(link - 1) * csz;
  const double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l1 = lam + (size_t)link * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  const int *idx0 = slots[s].idx0, *idx1 = slots[s].idx1, *idx2 = slots[s].idx2;
  double2 *X = slots[s].X;
  const int m = cp.m, n = cp.n, r0 = cp.r0, r1 = cp.r1, r2 = cp.r2;

  __shared__ double2 As[TT_K][TT_M + 1];
  __shared__ double2 Bs[TT_K][TT_N + 1];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;
  double2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);

  for (int k0 = 0; k0 < r1; k0 += TT_K) {
    for (int e = tid; e < TT_M * TT_K; e += 256) {
      const int rr = e % TT_M, kk = e / TT_M;
      const int r = r0b + rr, gk = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (r < m && gk < r1) {
        const int i = r / r0, a = idx0[r - i * r0], g = idx1[gk];
        v = cscale(G1[a + (size_t)chi * i + csz / chi * g], l0[a]);
      }
      As[kk][rr] = v;
    }
    for (int e = tid; e < TT_K * TT_N; e += 256) {
      const int kk = e % TT_K, cc = e / TT_K;
      const int gk = k0 + kk, c = c0b + cc;
      double2 v = make_double2(0.0, 0.0);
      if (gk < r1 && c < n) {
        const int lphys = c % d, b = idx2[c / d], g = idx1[gk];
        v = cscale(G2[g + (size_t)chi * lphys + (size_t)chi * d * b], l1[g] * l2[b]);
      }
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
    const int r = r0b + tr + 16 * p;
    if (r >= m) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0b + tc + 16 * q;
      if (c >= n) continue;
      const int lphys = c % d, bp = c / d;
      X[r + (size_t)m * ((size_t)lphys * r2 + bp)] = acc[p][q];
    }
  }
}

// Precision form (TEBD_SVD_DF): the same contraction accumulated in double-float
// on the FP32 pipe, tiles staged as double-float, the result stored in FP64.
__global__ void __launch_bounds__(256) k_theta_form_df(const double2 *__restrict__ gam,
                                                    const double *__restrict__ lam,
                                                    const int *__restrict__ links, Slot *slots,
                                                    int chi, int d) {
  const int s = blockIdx.z;
  const Compact cp = *slots[s].cp;
  const int r0b = blockIdx.x * TT_M, c0b = blockIdx.y * TT_N;
  if (r0b >= cp.m || c0b >= cp.n) return;  // uniform per CTA
  const int link = links[s];
  const size_t csz = (size_t)chi * d * chi;
  const double2 *G1 = gam + (size_t)(link - 1) * csz;
  const double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l1 = lam + (size_t)link * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  const int *idx0 = slots[s].idx0, *idx1 = slots[s].idx1, *idx2 = slots[s].idx2;
  double2 *X = slots[s].X;
  const int m = cp.m, n = cp.n, r0 = cp.r0, r1 = cp.r1, r2 = cp.r2;

  __shared__ float4 As[TT_K][TT_M + 1];
  __shared__ float4 Bs[TT_K][TT_N + 1];
  const int tid = threadIdx.x;
  const int tr = tid % 16, tc = tid / 16;
  float4 acc[4][4];  // double-float (re_hi, re_lo, im_hi, im_lo)
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_float4(0.f, 0.f, 0.f, 0.f);

  for (int k0 = 0; k0 < r1; k0 += TT_K) {
    for (int e = tid; e < TT_M * TT_K; e += 256) {
      const int rr = e % TT_M, kk = e / TT_M;
      const int r = r0b + rr, gk = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (r < m && gk < r1) {
        const int i = r / r0, a = idx0[r - i * r0], g = idx1[gk];
        v = cscale(G1[a + (size_t)chi * i + csz / chi * g], l0[a]);
      }
      As[kk][rr] = dfs(v);
    }
    for (int e = tid; e < TT_K * TT_N; e += 256) {
      const int kk = e % TT_K, cc = e / TT_K;
      const int gk = k0 + kk, c = c0b + cc;
      double2 v = make_double2(0.0, 0.0);
      if (gk < r1 && c < n) {
        const int lphys = c % d, b = idx2[c / d], g = idx1[gk];
        v = cscale(G2[g + (size_t)chi * lphys + (size_t)chi * d * b], l1[g] * l2[b]);
      }
      Bs[kk][cc] = dfs(v);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TT_K; ++kk) {
      float4 a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][tr + 16 * q];
        b[q] = Bs[kk][tc + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) df_cmac(acc[p][q].x, acc[p][q].y, acc[p][q].z, acc[p][q].w, a[p], b[q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int r = r0b + tr + 16 * p;
    if (r >= m) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0b + tc + 16 * q;
      if (c >= n) continue;
      const int lphys = c % d, bp = c / d;
      X[r + (size_t)m * ((size_t)lphys * r2 + bp)] = dfd(acc[p][q]);
    }
  }
}

// ---------------------------------------------------------------------------
// ThetaOperation: for every kept (alpha, beta) the d^2-vector Theta(alpha,:,:,beta)
// is multiplied by Op2 (row (i-1)d+j, column (k-1)d+l).  In place.
// ---------------------------------------------------------------------------
constexpr int kMaxD = 8;
constexpr int kGatePairs = 32;  // (alpha, beta) vectors staged per block

// Dynamic shared memory of k_gate_apply: the d^4 gate and kGatePairs d^2-vectors
// (98 304 B at d = 8, above the 48 KB default: set_gate_smem opts in).
inline size_t gate_smem_bytes(int d) {
  return sizeof(double2) * ((size_t)d * d * d * d + (size_t)kGatePairs * d * d);
}

// One block updates kGatePairs kept (alpha, beta) pairs: their d^2-vectors are
// read into shared memory (consecutive threads take consecutive alpha, so the
// reads are coalesced), the block synchronises, and every output element
// (pair, row) is a d^2-term dot product with one gate row.  Pairs of different
// blocks are disjoint, so the update is in place.
// kDF (the precision and learned-rank forms): the gate's d^2 complex
// multiply-adds per entry in double-float on the FP32 pipe (48-bit significands;
// the FP64 pipe made this kernel FP64-bound at chi = 512), the result rounded
// back to FP64.
template <bool kDF>
__global__ void __launch_bounds__(128) k_gate_apply(Slot *slots, int chi, int d) {
  extern __shared__ double2 gsm[];  // d^4 gate | kGatePairs * d^2 vectors
  const int s = blockIdx.y;
  const Compact cp = *slots[s].cp;
  const int npairs = cp.r0 * cp.r2;
  const int p0 = blockIdx.x * kGatePairs;
  if (p0 >= npairs) return;  // uniform over the block
  const int d2 = d * d;
  const double2 *G = slots[s].gate;
  double2 *vsm = gsm + d2 * d2;
  const int m = cp.m, r0 = cp.r0, r2 = cp.r2;
  const int np = min(kGatePairs, npairs - p0);
  double2 *X = slots[s].X;
  float4 *gdf = reinterpret_cast<float4 *>(gsm), *vdf = reinterpret_cast<float4 *>(vsm);  // kDF views
  for (int e = threadIdx.x; e < d2 * d2; e += blockDim.x) {
    if (kDF)
      gdf[e] = dfs(G[e]);
    else
      gsm[e] = G[e];
  }
  for (int e = threadIdx.x; e < kGatePairs * d2; e += blockDim.x) {
    const int p = e % kGatePairs, kl = e / kGatePairs;
    if (p >= np) continue;
    const int t = p0 + p, a = t % r0, b = t / r0, k = kl / d, l = kl % d;
    const double2 x = X[(size_t)(k * r0 + a) + (size_t)m * (l * r2 + b)];
    if (kDF)
      vdf[e] = dfs(x);
    else
      vsm[e] = x;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kGatePairs * d2; e += blockDim.x) {
    const int p = e % kGatePairs, row = e / kGatePairs;
    if (p >= np) continue;
    const int t = p0 + p, a = t % r0, b = t / r0, i = row / d, j = row % d;
    double2 acc = make_double2(0.0, 0.0);
    if (kDF) {
      float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
      for (int kl = 0; kl < d2; ++kl) df_cmac(rh, rl, ih, il, gdf[row + d2 * kl], vdf[kl * kGatePairs + p]);
      acc = dfd(make_float4(rh, rl, ih, il));
    } else {
      for (int kl = 0; kl < d2; ++kl) {
        const double2 g = gsm[row + d2 * kl];
        const double2 v = vsm[kl * kGatePairs + p];
        acc.x = fma(g.x, v.x, acc.x);
        acc.x = fma(-g.y, v.y, acc.x);
        acc.y = fma(g.x, v.y, acc.y);
        acc.y = fma(g.y, v.x, acc.y);
      }
    }
    X[(size_t)(i * r0 + a) + (size_t)m * (j * r2 + b)] = acc;
  }
}

// Opt k_gate_apply into the shared memory it needs on the current device (a
// per-function attribute; cheap, made before every launch).
static cudaError_t set_gate_smem(int d, bool df = false) {
  return cudaFuncSetAttribute(df ? k_gate_apply<true> : k_gate_apply<false>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gate_smem_bytes(d));
}

// ---------------------------------------------------------------------------
// Frobenius norm of Theta, deterministic two-level reduction (fixed order).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_norm_partial(Slot *slots, double *part) {
  const int s = blockIdx.y;
  const Compact cp = *slots[s].cp;
  const size_t total = (size_t)cp.m * cp.n;
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

__global__ void k_norm_final(const double *part, double *nrm, JacobiProblem<double> *jp, int nb,
                             int *status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nb) return;
  double acc = 0.0;
  for (int j = 0; j < kNormParts; ++j) acc += part[s * kNormParts + j];
  const double v = sqrt(acc);
  nrm[s] = v;
  const double f = kNegligibleColumn * v;
  jp[s].floor = f * f;
  if (!isfinite(v) || v == 0.0) atomicOr(&status[0], 1);
}

// V = identity (n x n, ld n) for every slot
__global__ void k_eye(Slot *slots) {
  const int s = blockIdx.y;
  const int n = slots[s].cp->n;
  double2 *V = slots[s].V;
  const size_t total = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e % n, c = e / n;
    V[e] = make_double2(r == c ? 1.0 : 0.0, 0.0);
  }
}

// ---------------------------------------------------------------------------
// After the SVD: column norms of X = U Sigma, descending order (rank sort, ties
// broken by column index), normalised singular values S = sigma/||Theta||; the
// n_full - n dropped values are exact zeros.  One CTA per slot.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_sigma_sort(Slot *slots, const double *nrm, int n_full,
                                                     int *status) {
  extern __shared__ double sig[];  // n
  const int s = blockIdx.x;
  const Compact cp = *slots[s].cp;
  const int m = cp.m, n = cp.k;  // X holds k columns sigma_c u_c (k = n for plain Jacobi)
  const double2 *X = slots[s].X;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = warp; c < n; c += nw) {
    double acc = 0.0;
    for (int r = lane; r < m; r += 32) {
      const double2 v = X[r + (size_t)m * c];
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
    for (int q = 0; q < n; ++q) {
      const double w = sig[q];
      rank += (w > v) || (w == v && q < k);
    }
    slots[s].perm[rank] = k;
    slots[s].S[rank] = v * inv;
  }
  for (int k = n + threadIdx.x; k < n_full; k += blockDim.x) {
    slots[s].perm[k] = -1;
    slots[s].S[k] = 0.0;
  }
}

// FormLambda1 (:347-379): sequential in the reference's order, one thread per slot.
// Kept-rank form (rank_bound > 0, no reference counterpart): keep the fewest
// leading values whose discarded weight -- the weight beyond chi, 1 - sum of the
// chi values, plus the dropped kept values summed from the smallest up -- stays
// within rank_bound; the rest of Lambda1 is set to exactly zero, so that the
// neighbouring updates compact those Schmidt indices away.
__global__ void k_lambda(Slot *slots, const int *links, double *lam, double *truncerr, int chi,
                         int nb, double rank_bound, const int *status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nb || (status[0] & 1)) return;  // non-finite batch: the chain is left as it was
  const double *S = slots[s].S;
  int keep = chi;
  if (rank_bound > 0.0) {
    double all = 0.0;
    for (int a = 0; a < chi; ++a)
      if (fabs(S[a]) > kGuardDense) all = all + S[a] * S[a];
    double w = fmax(1.0 - all, 0.0);  // weight beyond chi
    keep = chi;
    while (keep > 1) {
      const double v = fabs(S[keep - 1]) > kGuardDense ? S[keep - 1] * S[keep - 1] : 0.0;
      if (w + v > rank_bound) break;
      w += v;
      --keep;
    }
  }
  double norm = 0.0;
  for (int a = 0; a < keep; ++a)
    if (fabs(S[a]) > kGuardDense) norm = norm + S[a] * S[a];
  truncerr[s] = fabs(1.0 - norm);
  double *l1 = lam + (size_t)links[s] * chi;
  const double rs = sqrt(norm);
  for (int a = 0; a < chi; ++a) l1[a] = (a < keep && fabs(S[a]) > kGuardDense) ? S[a] / rs : 0.0;
}

// Keep the last spectrum and sweep count of every link for tebd_get_singular_values.
__global__ void k_store_spectrum(Slot *slots, const int *links, const int *sweeps, double *sig_link,
                                 int *sig_count, int *sweeps_link, int n, const int *path) {
  const int s = blockIdx.x;
  const int link = links[s];
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    sig_link[(size_t)(link - 1) * n + k] = slots[s].S[k];
  if (threadIdx.x == 0) {
    // the bidiagonal route computes only the kept values; the Jacobi routes all of them
    sig_count[link - 1] = path[s] != kPathQRJ ? slots[s].cp->k : n;
    sweeps_link[link - 1] = sweeps[s];
  }
}

// FormGamma1 (:381-404): Gamma1(alpha,i,beta) = U((i-1)chi+alpha, beta) / Lambda0(alpha)
// with U(:,beta) = X(:,perm(beta)) / sigma(perm(beta)); zero where the guard fails,
// where alpha was compacted away, and for columns beyond the rank.
__global__ void k_restore_gamma1(double2 *gam, const double *lam, const int *links, Slot *slots,
                                 const double *nrm, int chi, int d, const int *status) {
  if (status[0] & 1) return;  // non-finite batch: the chain is left as it was
  const int s = blockIdx.y;
  const int nf = chi * d;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)nf * chi) return;
  const Compact cp = *slots[s].cp;
  const int link = links[s];
  const int r = (int)(t % nf), beta = (int)(t / nf);
  const int i = r / chi, alpha = r % chi;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  double2 out = make_double2(0.0, 0.0);
  const int ap = slots[s].inv0[alpha];
  if (beta < cp.k && ap >= 0 && fabs(l0[alpha]) > kGuardDense) {
    const double sigma = slots[s].S[beta] * nrm[s];
    if (sigma > 0.0) {
      const int col = slots[s].perm[beta];
      const double2 x = slots[s].X[(size_t)(i * cp.r0 + ap) + (size_t)cp.m * col];
      const double sc = 1.0 / (sigma * l0[alpha]);
      out = make_double2(x.x * sc, x.y * sc);
    }
  }
  gam[(size_t)(link - 1) * chi * d * chi + t] = out;
}

// FormGamma2 (:406-428): Gamma2(alpha,i,beta) = VT(alpha,(i-1)chi+beta) / Lambda2(beta),
// VT = V^H, i.e. conj(V(i*r2 + b', perm(alpha))).  32x32 tile transpose through smem.
__global__ void __launch_bounds__(256) k_restore_gamma2(double2 *gam, const double *lam,
                                                        const int *links, Slot *slots, int chi,
                                                        int d, const int *status) {
  if (status[0] & 1) return;  // non-finite batch: the chain is left as it was
  __shared__ double2 tile[32][33];
  const int s = blockIdx.z;
  const int nf = chi * d;
  const Compact cp = *slots[s].cp;
  const int link = links[s];
  const int a0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const double2 *V = slots[s].V;
  const int *perm = slots[s].perm, *inv2 = slots[s].inv2;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int yy = ty; yy < 32; yy += 8) {
    const int alpha = a0 + yy, c = c0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (alpha < chi && alpha < cp.k && c < nf) {
      const int bp = inv2[c % chi];
      if (bp >= 0) v = V[(size_t)((c / chi) * cp.r2 + bp) + (size_t)cp.n * perm[alpha]];
    }
    tile[yy][tx] = v;
  }
  __syncthreads();
  const double *l2 = lam + (size_t)(link + 1) * chi;
  double2 *G2 = gam + (size_t)link * chi * d * chi;
  for (int yy = ty; yy < 32; yy += 8) {
    const int c = c0 + yy, alpha = a0 + tx;
    if (alpha >= chi || c >= nf) continue;
    const int i = c / chi, beta = c % chi;
    const double2 v = tile[tx][yy];
    double2 out = make_double2(0.0, 0.0);
    if (fabs(l2[beta]) > kGuardDense) {
      const double inv = 1.0 / l2[beta];
      out = make_double2(v.x * inv, -v.y * inv);
    }
    G2[alpha + (size_t)chi * i + (size_t)nf * beta] = out;
  }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

int launch_dense_prepare(tebd_handle *h, int nb, bool /*real_gate: converted on the host*/) {
  const int chi = h->chi, d = h->d, n = h->n;
  cudaStream_t st = h->stream;
  JacobiProblem<double> *jp = reinterpret_cast<JacobiProblem<double> *>(h->jprob_d);
  k_compact<<<nb, 96, 0, st>>>(h->lam, h->links_d, h->slots_d, jp, chi, d);
  TEBD_LAUNCHED(h);
  int tc = -1;  // tensor-core Theta (theta_tc.cu); -1: formed on the CUDA cores below
  if (h->theta_form != 0 && h->mode == TEBD_MODE_DENSE && (tc = launch_theta_tc(h, nb)) > 0) return tc;
  if (tc == 0) {
  } else if (h->opts.svd_mode == TEBD_SVD_DF || h->opts.svd_mode == TEBD_SVD_RSVD)
    k_theta_form_df<<<dim3(cdiv(n, TT_M), cdiv(n, TT_N), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                            h->slots_d, chi, d);
  else
    k_theta_form<<<dim3(cdiv(n, TT_M), cdiv(n, TT_N), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                         h->slots_d, chi, d);
  TEBD_LAUNCHED(h);
  const bool gdf = h->opts.svd_mode == TEBD_SVD_DF || h->opts.svd_mode == TEBD_SVD_RSVD;
  int rc = check_cuda(h, set_gate_smem(d, gdf), "gate shared memory");
  if (rc) return rc;
  (gdf ? k_gate_apply<true> : k_gate_apply<false>)<<<dim3(cdiv((size_t)chi * chi, kGatePairs), nb), 128,
                                                     gate_smem_bytes(d), st>>>(h->slots_d, chi, d);
  TEBD_LAUNCHED(h);
  k_norm_partial<<<dim3(kNormParts, nb), 256, 0, st>>>(h->slots_d, h->nrm_part);
  TEBD_LAUNCHED(h);
  k_norm_final<<<cdiv(nb, 128), 128, 0, st>>>(h->nrm_part, h->nrm, jp, nb, h->status_d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "dense prepare launch");
}

// Swapping decomposes Theta without ReshapeTheta's normalisation: once the SVD
// (which used the true norm for its negligible-column floor) is done, the norm
// seen by the sort, FormLambda1 and the restores is set to 1.
__global__ void k_unit_norm(double *nrm, int nb) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nb) nrm[s] = 1.0;
}

int launch_unit_norm(tebd_handle *h, int nb) {
  k_unit_norm<<<cdiv(nb, 128), 128, 0, h->stream>>>(h->nrm, nb);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "unit norm launch");
}

int launch_eye(tebd_handle *h, int nb) {
  const size_t total = (size_t)h->n * h->n;
  unsigned gx = cdiv(total, 256);
  if (gx > 1024) gx = 1024;
  k_eye<<<dim3(gx, nb), 256, 0, h->stream>>>(h->slots_d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "eye launch");
}

int launch_dense_finish(tebd_handle *h, int nb) {
  const int chi = h->chi, d = h->d, n = h->n;
  cudaStream_t st = h->stream;
  k_sigma_sort<<<nb, 1024, sizeof(double) * n, st>>>(h->slots_d, h->nrm, n, h->status_d);
  TEBD_LAUNCHED(h);
  k_lambda<<<cdiv(nb, 64), 64, 0, st>>>(h->slots_d, h->links_d, h->lam, h->truncerr_d, chi, nb,
                                        h->unnormalized ? 0.0 : h->rank_bound, h->status_d);
  TEBD_LAUNCHED(h);
  k_store_spectrum<<<nb, 256, 0, st>>>(h->slots_d, h->links_d, h->js.sweeps, h->sig_link_d,
                                       h->sig_count_d, h->sweeps_link_d, n, h->path_d);
  TEBD_LAUNCHED(h);
  k_restore_gamma1<<<dim3(cdiv((size_t)n * chi, 256), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                       h->slots_d, h->nrm, chi, d,
                                                                       h->status_d);
  TEBD_LAUNCHED(h);
  k_restore_gamma2<<<dim3(cdiv(chi, 32), cdiv(n, 32), nb), 256, 0, st>>>(h->gam, h->lam, h->links_d,
                                                                        h->slots_d, chi, d, h->status_d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "dense finish launch");
}

}  // namespace tebd

namespace tebd {

// Largest compacted column count of the batch (sizes the Jacobi rounds).
int dense_compact_sizes(tebd_handle *h, int nb, int *nmax, std::vector<Compact> *out) {
  std::vector<Compact> cp(nb);
  int rc = check_cuda(h, cudaMemcpyAsync(cp.data(), h->cp_d, sizeof(Compact) * nb,
                                         cudaMemcpyDeviceToHost, h->stream),
                      "read compaction");
  if (rc) return rc;
  rc = check_cuda(h, cudaStreamSynchronize(h->stream), "read compaction");
  if (rc) return rc;
  int mx = 0;
  for (int s = 0; s < nb; ++s) {
    if (cp[s].n > mx) mx = cp[s].n;
    h->stats.compact_rows += cp[s].m;
    h->stats.compact_cols += cp[s].n;
  }
  *nmax = mx;
  if (out) *out = cp;
  return TEBD_OK;
}

}  // namespace tebd

namespace tebd {

// Handle-free launch sequences for one bond (slot 0), used by the
// allocation-free entry point in noalloc.cu.  Same kernels, same order as
// launch_dense_prepare / launch_eye / launch_dense_finish.
cudaError_t raw_dense_prepare(cudaStream_t st, double2 *gam, const double *lam, const int *links_d,
                              Slot *slots_d, JacobiProblem<double> *jp, double *nrm_part, double *nrm,
                              int *status, int chi, int d) {
  const int n = chi * d;
  k_compact<<<1, 96, 0, st>>>(lam, links_d, slots_d, jp, chi, d);
  k_theta_form<<<dim3(cdiv(n, TT_M), cdiv(n, TT_N), 1), 256, 0, st>>>(gam, lam, links_d, slots_d,
                                                                      chi, d);
  cudaError_t e = set_gate_smem(d);
  if (e != cudaSuccess) return e;
  k_gate_apply<false><<<dim3(cdiv((size_t)chi * chi, kGatePairs), 1), 128, gate_smem_bytes(d), st>>>(
      slots_d, chi, d);
  k_norm_partial<<<dim3(kNormParts, 1), 256, 0, st>>>(slots_d, nrm_part);
  k_norm_final<<<1, 32, 0, st>>>(nrm_part, nrm, jp, 1, status);
  const size_t total = (size_t)n * n;
  unsigned gx = cdiv(total, 256);
  if (gx > 1024) gx = 1024;
  k_eye<<<dim3(gx, 1), 256, 0, st>>>(slots_d);
  return cudaPeekAtLastError();
}

cudaError_t raw_dense_finish(cudaStream_t st, double2 *gam, double *lam, const int *links_d,
                             Slot *slots_d, const double *nrm, double *truncerr, int *status, int chi,
                             int d) {
  const int n = chi * d;
  k_sigma_sort<<<1, 1024, sizeof(double) * n, st>>>(slots_d, nrm, n, status);
  k_lambda<<<1, 32, 0, st>>>(slots_d, links_d, lam, truncerr, chi, 1, 0.0, status);
  k_restore_gamma1<<<dim3(cdiv((size_t)n * chi, 256), 1), 256, 0, st>>>(gam, lam, links_d, slots_d,
                                                                       nrm, chi, d, status);
  k_restore_gamma2<<<dim3(cdiv(chi, 32), cdiv(n, 32), 1), 256, 0, st>>>(gam, lam, links_d, slots_d,
                                                                       chi, d, status);
  return cudaPeekAtLastError();
}

}  // namespace tebd
