// canon.cu -- CanonicalForm and CanonicalFormAll of the dense chain
// (VidalCore_v_2.0/local_operations_module.f90:496-610, propagation_module.f90:617-634),
// the re-orthogonalisation of the Schmidt bases the reference's imaginary-time
// evolution (ImagTimeProp) runs after its steps.  For one bond (Lambda0, Gamma1, Lambda1, Gamma2,
// Lambda2), chi x chi matrices throughout:
//   M1 = sum_{i,g} conj(G1(g,i,:))^T l0(g)^2 G1(g,i,:)      = U1 S1 U1^H
//   G1t(:,i,b) = G1(:,i,:) U1(:,b) / sqrt(S1(b))   (0 where S1(b) <= 1e-8)
//   X = diag(sqrt(S1)) U1^H
//   M2 = sum_{i,g} G2(:,i,g) l2(g)^2 conj(G2(:,i,g))^T      = U2 S2 U2^H
//   G2t(a,i,:) = (U2^H G2(:,i,:))(a,:) / sqrt(S2(a))  (0 where S2(a) <= 1e-8)
//   Y = diag(l1) U2 diag(sqrt(S2));  X Y = U S V^H
//   Lambda1 = S / sqrt(sum S^2),  G1 = G1t U,  G2 = V^H G2t
// The three SVDs (ZGESVD in the reference) are one-sided Jacobi solves on the
// library's persistent kernel, sorted to descending singular values; U = X/sigma.
// Singular vectors are unique up to phases (and rotations inside degenerate
// subspaces), so Gammas agree with the reference up to that gauge; Lambdas and
// the state agree to rounding.
#include <math.h>

#include <algorithm>
#include <vector>

#include "tebd_internal.cuh"

namespace tebd {

namespace {

inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// operand of the small GEMM: element (r, c) of op(P) with
//   op = P (trans = 0) or P^T / P^H (trans = 1, conj chooses), scaled by s[q]
//   where q is r (sside = 1) or c (sside = 2), reduced as q mod smod (smod > 0)
//   or q / sdiv, and squared when ssqr = 1
struct Opnd {
  const double2 *p;
  int ld;
  int trans, conj;
  const double *s;
  int sside, sdiv, smod;
  int ssqr;
};

__device__ __forceinline__ double2 opnd_at(const Opnd &o, int r, int c) {
  double2 v = o.trans ? o.p[c + (size_t)o.ld * r] : o.p[r + (size_t)o.ld * c];
  if (o.conj) v.y = -v.y;
  if (o.sside) {
    const int q = o.sside == 1 ? r : c;
    double w = o.s[o.smod > 0 ? q % o.smod : q / o.sdiv];
    if (o.ssqr) w *= w;
    v.x *= w;
    v.y *= w;
  }
  return v;
}

// C (M x N, ld ldc) = op(A) (M x K) op(B) (K x N); 32 x 32 tiles, 256 threads
__global__ void __launch_bounds__(256) k_cf_gemm(int M, int N, int K, Opnd A, Opnd B, double2 *C, int ldc) {
  __shared__ double2 As[16][33], Bs[16][33];
  const int m0 = blockIdx.x * 32, n0 = blockIdx.y * 32, t = threadIdx.x;
  const int tx = t & 15, ty = t >> 4;  // outputs (ty + 16u, tx + 16v), u, v in {0, 1}
  double2 acc[2][2] = {{make_double2(0, 0), make_double2(0, 0)}, {make_double2(0, 0), make_double2(0, 0)}};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = t; e < 16 * 32; e += 256) {
      const int mm = e % 32, kk = e / 32;
      As[kk][mm] = (m0 + mm < M && k0 + kk < K) ? opnd_at(A, m0 + mm, k0 + kk) : make_double2(0, 0);
      Bs[kk][mm] = (n0 + mm < N && k0 + kk < K) ? opnd_at(B, k0 + kk, n0 + mm) : make_double2(0, 0);
    }
    __syncthreads();
    for (int kk = 0; kk < 16; ++kk)
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const double2 a = As[kk][ty + 16 * u], b = Bs[kk][tx + 16 * v];
          acc[u][v].x = fma(a.x, b.x, fma(-a.y, b.y, acc[u][v].x));
          acc[u][v].y = fma(a.x, b.y, fma(a.y, b.x, acc[u][v].y));
        }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int r = m0 + ty + 16 * u, c = n0 + tx + 16 * v;
      if (r < M && c < N) C[r + (size_t)ldc * c] = acc[u][v];
    }
}

// X <- M (copy), V <- I, for the Jacobi solve of one n x n problem
__global__ void k_cf_svd_setup(const double2 *M, double2 *X, double2 *V, int n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n;
       e += (size_t)gridDim.x * blockDim.x) {
    X[e] = M[e];
    V[e] = make_double2((e % n) == (e / n) ? 1.0 : 0.0, 0.0);
  }
}

// after the Jacobi solve (X = U Sigma, V): sigma_k = |X(:,k)|, descending order
// (ties in column order); U(:,r) = X(:,k)/sigma_k (0 for sigma_k = 0), Vs(:,r) = V(:,k)
__global__ void __launch_bounds__(1024) k_cf_svd_finish(const double2 *X, const double2 *V, double2 *U,
                                                        double2 *Vs, double *S, int n) {
  extern __shared__ double sg[];
  int *rank = reinterpret_cast<int *>(sg + n);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = warp; c < n; c += nw) {
    double a = 0.0;
    for (int r = lane; r < n; r += 32) {
      const double2 v = X[r + (size_t)n * c];
      a = fma(v.x, v.x, fma(v.y, v.y, a));
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) sg[c] = sqrt(a);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    int r = 0;
    for (int q = 0; q < n; ++q) r += (sg[q] > sg[k]) || (sg[q] == sg[k] && q < k);
    rank[k] = r;
    S[r] = sg[k];
  }
  __syncthreads();
  for (size_t e = threadIdx.x; e < (size_t)n * n; e += blockDim.x) {
    const int r = (int)(e % n), k = (int)(e / n), dst = rank[k];
    const double inv = sg[k] > 0.0 ? 1.0 / sg[k] : 0.0;
    const double2 x = X[e];
    U[r + (size_t)n * dst] = make_double2(x.x * inv, x.y * inv);
    Vs[r + (size_t)n * dst] = V[e];
  }
}

// G1t(:, b) *= 1/sqrt(S1(b)) or 0 (columns of a (chi d) x chi matrix); X = diag(sqrt S1) U1^H
__global__ void k_cf_left(double2 *G1t, const double *S1, const double2 *U1, double2 *Xm, int chi, int d) {
  const size_t rows = (size_t)chi * d;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < rows * chi; e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / rows);
    const double s = S1[b];
    const double w = s > (double)1e-8f ? 1.0 / sqrt(s) : 0.0;
    G1t[e].x *= w;
    G1t[e].y *= w;
  }
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)chi * chi; e += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(e % chi), b = (int)(e / chi);
    const double2 u = U1[b + (size_t)chi * a];  // X(a,b) = sqrt(S1(a)) conj(U1(b,a))
    const double w = sqrt(S1[a]);
    Xm[e] = make_double2(w * u.x, -w * u.y);
  }
}

// G2t(a, :) *= 1/sqrt(S2(a)) or 0 (rows of a chi x (d chi) matrix); Y = diag(l1) U2 diag(sqrt S2)
__global__ void k_cf_right(double2 *G2t, const double *S2, const double2 *U2, const double *l1, double2 *Ym,
                           int chi, int d) {
  const size_t cols = (size_t)d * chi;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < cols * chi; e += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(e % chi);
    const double s = S2[a];
    const double w = s > (double)1e-8f ? 1.0 / sqrt(s) : 0.0;
    G2t[e].x *= w;
    G2t[e].y *= w;
  }
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)chi * chi; e += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(e % chi), b = (int)(e / chi);
    const double w = l1[a] * sqrt(S2[b]);
    const double2 u = U2[e];
    Ym[e] = make_double2(w * u.x, w * u.y);
  }
}

// Lambda1 = S / sqrt(sum S^2) (one warp, fixed order per lane then lanes in order)
__global__ void k_cf_lambda(const double *S, double *l1, int chi) {
  const int lane = threadIdx.x;
  double a = 0.0;
  for (int k = lane; k < chi; k += 32) a = fma(S[k], S[k], a);
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  const double inv = a > 0.0 ? 1.0 / sqrt(a) : 0.0;
  for (int k = lane; k < chi; k += 32) l1[k] = S[k] * inv;
}

}  // namespace

// workspace (complex unless noted): M1, M2, X, Y, M (chi^2 each), Jacobi X, V
// (chi^2 each), U1, U2, U, Vs (chi^2 each), G1t, G2t (chi d chi each), then
// doubles S1, S2, S (chi each); one Jacobi problem descriptor
struct CfWs {
  double2 *M1, *M2, *Xm, *Ym, *Mm, *JX, *JV, *U1, *U2, *U, *Vs, *G1t, *G2t;
  double *S1, *S2, *S;
  JacobiProblem<double> *prob;
};

static size_t cf_bytes(int chi, int d) {
  const size_t cc = (size_t)chi * chi, g = cc * d;
  return sizeof(double2) * (11 * cc + 2 * g) + sizeof(double) * 3 * chi + sizeof(JacobiProblem<double>) + 512;
}

static CfWs cf_carve(void *base, int chi, int d) {
  const size_t cc = (size_t)chi * chi, g = cc * d;
  double2 *p = reinterpret_cast<double2 *>(base);
  CfWs w;
  w.M1 = p;
  w.M2 = p + cc;
  w.Xm = p + 2 * cc;
  w.Ym = p + 3 * cc;
  w.Mm = p + 4 * cc;
  w.JX = p + 5 * cc;
  w.JV = p + 6 * cc;
  w.U1 = p + 7 * cc;
  w.U2 = p + 8 * cc;
  w.U = p + 9 * cc;
  w.Vs = p + 10 * cc;
  w.G1t = p + 11 * cc;
  w.G2t = w.G1t + g;
  double *q = reinterpret_cast<double *>(w.G2t + g);
  w.S1 = q;
  w.S2 = q + chi;
  w.S = q + 2 * chi;
  const size_t off = ((reinterpret_cast<size_t>(q + 3 * chi) + 255) & ~(size_t)255);
  w.prob = reinterpret_cast<JacobiProblem<double> *>(off);
  return w;
}

// SVD of the chi x chi matrix Min: U (sorted columns), S (descending), Vs
static int cf_svd(tebd_handle *h, const CfWs &w, const double2 *Min, double2 *U, double *S) {
  const int chi = h->chi;
  cudaStream_t st = h->stream;
  k_cf_svd_setup<<<cdiv((size_t)chi * chi, 256) < 256 ? cdiv((size_t)chi * chi, 256) : 256, 256, 0, st>>>(
      Min, w.JX, w.JV, chi);
  TEBD_LAUNCHED(h);
  int rc = run_jacobi_problems(h, w.prob, 1, chi);
  if (rc) return rc;
  const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)chi;
  k_cf_svd_finish<<<1, 1024, smem, st>>>(w.JX, w.JV, U, w.Vs, S, chi);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "canonical form svd");
}

static void gemm(tebd_handle *h, int M, int N, int K, Opnd A, Opnd B, double2 *C, int ldc) {
  k_cf_gemm<<<dim3(cdiv(M, 32), cdiv(N, 32)), 256, 0, h->stream>>>(M, N, K, A, B, C, ldc);
  TEBD_LAUNCHED(h);
}

static int canonical_form(tebd_handle *h, const CfWs &w, int link) {
  const int chi = h->chi, d = h->d, cd = chi * d;
  const size_t csz = (size_t)chi * d * chi;
  double2 *G1 = h->gam + (size_t)(link - 1) * csz, *G2 = h->gam + (size_t)link * csz;
  const double *l0 = h->lam + (size_t)(link - 1) * chi, *l2 = h->lam + (size_t)(link + 1) * chi;
  double *l1 = h->lam + (size_t)link * chi;
  cudaStream_t st = h->stream;
  const unsigned ge = 256;
  int rc;
  // M1(a,b) = sum_r conj(G1(r,a)) l0(r mod chi)^2 G1(r,b), G1 as (chi d) x chi, r = g + chi i
  gemm(h, chi, chi, cd, Opnd{G1, cd, 1, 1, l0, 2, 1, chi, 1}, Opnd{G1, cd, 0, 0, nullptr, 0, 1, 0, 0}, w.M1, chi);
  if ((rc = cf_svd(h, w, w.M1, w.U1, w.S1))) return rc;
  // G1t = G1 U1, then column scales and X
  gemm(h, cd, chi, chi, Opnd{G1, cd, 0, 0, nullptr, 0, 1, 0, 0}, Opnd{w.U1, chi, 0, 0, nullptr, 0, 1, 0, 0}, w.G1t,
       cd);
  k_cf_left<<<ge, 256, 0, st>>>(w.G1t, w.S1, w.U1, w.Xm, chi, d);
  TEBD_LAUNCHED(h);
  // M2(a,b) = sum_c G2(a,c) l2(c/d)^2 conj(G2(b,c)), G2 as chi x (d chi), c = i + d g
  gemm(h, chi, chi, cd, Opnd{G2, chi, 0, 0, l2, 2, d, 0, 1}, Opnd{G2, chi, 1, 1, nullptr, 0, 1, 0, 0}, w.M2, chi);
  if ((rc = cf_svd(h, w, w.M2, w.U2, w.S2))) return rc;
  // G2t = U2^H G2, then row scales and Y
  gemm(h, chi, cd, chi, Opnd{w.U2, chi, 1, 1, nullptr, 0, 1, 0, 0}, Opnd{G2, chi, 0, 0, nullptr, 0, 1, 0, 0}, w.G2t,
       chi);
  k_cf_right<<<ge, 256, 0, st>>>(w.G2t, w.S2, w.U2, l1, w.Ym, chi, d);
  TEBD_LAUNCHED(h);
  // M = X Y = U S V^H
  gemm(h, chi, chi, chi, Opnd{w.Xm, chi, 0, 0, nullptr, 0, 1, 0, 0}, Opnd{w.Ym, chi, 0, 0, nullptr, 0, 1, 0, 0},
       w.Mm, chi);
  if ((rc = cf_svd(h, w, w.Mm, w.U, w.S))) return rc;
  k_cf_lambda<<<1, 32, 0, st>>>(w.S, l1, chi);
  TEBD_LAUNCHED(h);
  // Gamma1 = G1t U, Gamma2 = V^H G2t
  gemm(h, cd, chi, chi, Opnd{w.G1t, cd, 0, 0, nullptr, 0, 1, 0, 0}, Opnd{w.U, chi, 0, 0, nullptr, 0, 1, 0, 0}, G1,
       cd);
  gemm(h, chi, cd, chi, Opnd{w.Vs, chi, 1, 1, nullptr, 0, 1, 0, 0}, Opnd{w.G2t, chi, 0, 0, nullptr, 0, 1, 0, 0},
       G2, chi);
  return check_cuda(h, cudaGetLastError(), "canonical form");
}

static int cf_prepare(tebd_handle *h, CfWs *w) {
  int rc = check_cuda(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (rc) return rc;
  const size_t need = cf_bytes(h->chi, h->d);
  if (h->obs_bytes < need) {
    cudaFree(h->obs_buf);
    h->obs_buf = nullptr;
    h->obs_bytes = 0;
    if ((rc = check_cuda(h, cudaMalloc(&h->obs_buf, need), "alloc canonical-form workspace"))) return rc;
    h->obs_bytes = need;
  }
  *w = cf_carve(h->obs_buf, h->chi, h->d);
  const int chi = h->chi;
  JacobiProblem<double> p = {w->JX, w->JV, chi, chi, chi, chi, 0.0};
  return check_cuda(h, cudaMemcpyAsync(w->prob, &p, sizeof p, cudaMemcpyHostToDevice, h->stream),
                    "upload canonical-form problem");
}

}  // namespace tebd

using namespace tebd;

extern "C" int tebd_canonical_form(tebd_handle *h, int link) {
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_DENSE) return set_error(h, TEBD_ERR_STATE, "CanonicalForm needs a TEBD_MODE_DENSE handle");
  if (link < 1 || link > h->L - 1) return set_error(h, TEBD_ERR_ARG, "tebd_canonical_form: link out of range");
  CfWs w;
  int rc;
  if ((rc = cf_prepare(h, &w))) return rc;
  if ((rc = canonical_form(h, w, link))) return rc;
  return check_cuda(h, cudaStreamSynchronize(h->stream), "canonical form");
}

extern "C" int tebd_canonical_form_all(tebd_handle *h) {
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_DENSE)
    return set_error(h, TEBD_ERR_STATE, "CanonicalFormAll needs a TEBD_MODE_DENSE handle");
  CfWs w;
  int rc;
  if ((rc = cf_prepare(h, &w))) return rc;
  for (int k = 1; k <= h->L - 1; ++k)
    if ((rc = canonical_form(h, w, k))) return rc;
  for (int k = h->L - 1; k >= 1; --k)
    if ((rc = canonical_form(h, w, k))) return rc;
  return check_cuda(h, cudaStreamSynchronize(h->stream), "canonical form all");
}
