// rsvd.cu -- the randomized SVD route of the learned-rank form (TEBD_SVD_RSVD):
// ZGESVD of SVDTruncation (VidalCore_v_2.0/local_operations_module.f90:322-345)
// replaced, for bonds whose compacted Theta is much larger than the rank kept,
// by a sketch of its leading singular subspace, with the full SVD as the fallback
// and the judge.
//
// Per bond (X = the gated, unnormalised Theta, m x n; r triplets wanted, sketch
// width s = r + p).  Every product below runs on the tensor cores as an
// error-free digit-plane product (tc_ozaki.cu) with 7 planes (FP64 class; the
// range finder's plane count is settable, tebd_set_rsvd).  The only FP64 CUDA-core work is
// O(s^3): the Cholesky factors of s x s Grams and one s x s SVD.
//   1. Xp = X zero-padded to the batch's m_max x n_max (kept: the fallback
//      restarts from it);
//   2. Q = orth(Xp Om) (Om: n x s complex Gaussian, fixed per handle), then q
//      times P = orth(Xp^H Q), Q = orth(Xp P); finally P = orth(Xp^H Q) --
//      span(P) approximates the top-s right singular subspace with error
//      ~ (sigma_{s+1}/sigma_i)^(2q+2);
//      orth(A) is CholQR: G = A^H A, G = R^H R (FP64, pivots below the Gram's
//      rounding level dropped), A <- A R^-1 -- once for the intermediate bases,
//      twice (CholQR2) for the final P;
//   3. C = Xp P (m x s), M = C^H C (s x s) and its SVD M = W Lambda W^H (the
//      bidiagonal route, FP64): the Rayleigh-Ritz triplets of Theta in span(P)
//      are (C w_i / |C w_i|, |C w_i|, P w_i);
//   4. the slot's X = C W (= U Sigma, m x r) and V = P W (n x r): the layout the
//      bidiagonal route leaves, so FormLambda1/FormGamma1/2 run unchanged;
//   5. the judge: for each kept triplet the residual of the other side,
//      rho_i = |Xp^H u_i - sigma_i v_i| (one more product, Xp^H (U Sigma)); a bond
//      whose largest rho_i exceeds tol * ||Theta|| is re-run from Xp with the
//      full SVD.  An accepted triplet's singular value is within ~rho^2/gap and
//      its vectors within ~rho/gap of the exact ones.
// The sketch width and power count come from tebd_set_rsvd or, per batch, from
// the learned model (mlp.cu).
#include <math.h>
#include <stddef.h>

#include <algorithm>
#include <functional>

#include <cooperative_groups.h>

#include "df.cuh"
#include "tc_gemm.cuh"

namespace tebd {

namespace {

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

// per-slot carve of the randomized-SVD workspace (bytes), for n_full x n_full
// Theta, sketch capacity sc and chi kept triplets at most
struct RsCarve {
  size_t xp, a, b, z, c, g, ri, w, rr, aux, tau, taup, bdws, th, per;
};
RsCarve rs_carve(int n, int sc, int chi) {
  RsCarve c;
  size_t aux_el = 0, bd_d = 0;
  bidiag_block_ws(sc, sc, std::min(chi, sc), &aux_el, &bd_d);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += al(bytes);
    return at;
  };
  c.xp = take(sizeof(double2) * (size_t)n * n);
  c.a = take(sizeof(double2) * (size_t)n * sc);
  c.b = take(sizeof(double2) * (size_t)n * sc);
  c.z = take(sizeof(double2) * (size_t)n * sc);
  c.c = take(sizeof(double2) * (size_t)n * sc);
  c.g = take(sizeof(double2) * (size_t)sc * sc);
  c.ri = take(sizeof(double2) * (size_t)sc * sc);
  c.w = take(sizeof(double2) * (size_t)sc * sc);
  c.rr = take(sizeof(double2) * (size_t)n * chi);
  c.aux = take(sizeof(double2) * aux_el);
  c.tau = take(sizeof(double2) * sc);
  c.taup = take(sizeof(double2) * sc);
  c.bdws = take(sizeof(double) * bd_d);
  c.th = take(sizeof(double));  // the Cholesky's pivot threshold
  c.per = o;
  return c;
}

// counter-based normal deviates for Om (Box-Muller on a 64-bit mix of the index)
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

__global__ void k_rs_omega(double2 *om, int n, int s, unsigned long long seed) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * s;
       e += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long a = mix64(seed ^ (2 * e + 1)), b = mix64(seed ^ (2 * e + 2) ^ 0x9e3779b97f4a7c15ULL);
    const double u1 = ((double)(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
    const double rad = sqrt(-2.0 * log(u1));
    om[e] = make_double2(rad * cos(6.283185307179586 * u2), rad * sin(6.283185307179586 * u2));
  }
}

// dims[s] = {m, n, s_active, r}: the bond's compacted sizes, the sketch width
// (0: not on this route) and the triplets wanted
struct RsDims {
  int m, n, s, r;
};

// 1. Xp (m_max x n_max, ld m_max) = X (m x n, ld m) zero-padded
__global__ void k_rs_pad(const Slot *slots, const RsDims *dims, double2 *ws, size_t per, int m_max, int n_max) {
  const int p = blockIdx.y;
  if (dims[p].s == 0) return;
  const Compact cp = *slots[p].cp;
  const double2 *X = slots[p].X;
  double2 *Xp = reinterpret_cast<double2 *>(reinterpret_cast<char *>(ws) + p * per);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)m_max * n_max;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % m_max), j = (int)(e / m_max);
    Xp[e] = (i < cp.m && j < cp.n) ? X[i + (size_t)cp.m * j] : make_double2(0.0, 0.0);
  }
}

// CholQR step on a Gram: G (s x s, Hermitian, both triangles) = R^H R with R
// upper triangular (right-looking Cholesky in place on the upper triangle), then
// Ri = R^-1 (upper).  A pivot at or below the bond's threshold (k_rs_thresh:
// `floor` times the largest diagonal entry of the whole Gram, its own rounding
// level: the products carry 7 S bits) marks a direction the sketch does not span
// to that accuracy: its row of R and column of R^-1 are zero, so A R^-1 has a zero
// column there.  The kernel works on one diagonal block (s x s inside a matrix
// of leading dimension ld, at byte offsets og / ori of the bond's workspace): the
// whole Gram, or a leaf of the recursive blocking in run_rsvd, whose off-diagonal
// blocks are digit-plane products on the tensor cores.  The O(s^3) work runs in
// double-float on the FP32 pipe (pairs of floats, 48-bit significands: the FP64
// pipe gives one SM ~7 GFLOP/s, too little for s^3 / 2 complex multiply-adds per
// call); only the s pivots and their reciprocals are FP64.  G and Ri hold float4
// (re_hi, re_lo, im_hi, im_lo) while the kernel runs -- the same 16 bytes as a
// double2 -- and Ri is converted back to FP64 at the end (R stays double-float).

__device__ __forceinline__ float4 df_scale(float4 v, float sh, float sl) {  // v * (sh + sl)
  float4 r;
  float p = __fmul_rn(v.x, sh), e = fmaf(v.x, sh, -p);
  e = fmaf(v.x, sl, e);
  e = fmaf(v.y, sh, e);
  r.x = __fadd_rn(p, e);
  r.y = __fadd_rn(e, -__fadd_rn(r.x, -p));
  p = __fmul_rn(v.z, sh);
  e = fmaf(v.z, sh, -p);
  e = fmaf(v.z, sl, e);
  e = fmaf(v.w, sh, e);
  r.z = __fadd_rn(p, e);
  r.w = __fadd_rn(e, -__fadd_rn(r.z, -p));
  return r;
}

__device__ __forceinline__ void df_split(double x, float &h, float &l) {
  h = (float)x;
  l = (float)(x - (double)h);
}

// per bond: the Cholesky's pivot threshold, floor x the largest diagonal entry of
// the Gram (s x s, ld s, FP64) at byte offset og, to byte offset oth
__global__ void k_rs_thresh(const RsDims *dims, char *ws, size_t per, size_t og, int s, double floor, size_t oth) {
  const int p = blockIdx.x;
  if (dims[p].s == 0) return;
  const double2 *G = reinterpret_cast<const double2 *>(ws + p * per + og);
  __shared__ double red[256];
  double mx = 0.0;
  for (int j = threadIdx.x; j < s; j += blockDim.x) mx = fmax(mx, G[j + (size_t)s * j].x);
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *reinterpret_cast<double *>(ws + p * per + oth) = red[0] * floor;
}

// Blocked form (panels of PB rows of R, PB = 16 up to s = 512, else 8): the panel
// rows are factored in shared memory and the trailing triangle takes one rank-PB
// update per panel; the inverse runs block rows from the bottom, each a product
// with the rows already inverted (one pass) and a triangular solve inside the
// block.  Dynamic shared memory: PB x s float4.
//
// A cluster of C CTAs (grid x = C, y = bond) shares one bond.  Every CTA factors
// each panel itself (the same rows and the same code give the same R rows), then
// updates the trailing columns l = rank (mod C); one cluster barrier per panel
// orders those updates before the next panel's rows are read, and rank 0 writes
// the factored rows back to G one panel later (once every CTA has read them).
// The inverse's columns are independent: each CTA solves its own, c = rank
// (mod C).  Reads of G that another CTA may have written go to L2 (ld.global.cg).
__global__ void __launch_bounds__(512) k_rs_chol(const RsDims *dims, char *ws, size_t per, size_t og, size_t ori,
                                                 int s, int ld, size_t oth, int PB) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
  const int p = blockIdx.y;
  if (dims[p].s == 0) return;  // uniform over the cluster: all its CTAs serve bond p
  extern __shared__ float4 P[];  // PB x s: panel rows, P[t * s + c]
  double2 *Gd = reinterpret_cast<double2 *>(ws + p * per + og);
  float4 *G = reinterpret_cast<float4 *>(Gd);
  float4 *Ri = reinterpret_cast<float4 *>(ws + p * per + ori);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
  auto own = [&](int x) { return x + ((rank - x) % C + C) % C; };  // first column >= x of this CTA
  __shared__ float ph[16], pl[16];  // reciprocal pivots of the panel, double-float
  const double thresh = *reinterpret_cast<const double *>(ws + p * per + oth);
  for (int c = own(0); c < s; c += C)
    for (int r = tid; r < s; r += nt) G[r + (size_t)ld * c] = dfs(__ldcg(&Gd[r + (size_t)ld * c]));  // in place
  cluster.sync();
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  auto write_back = [&](int j0, int jb) {  // rank 0: the factored rows j0.. of the panel in P
    for (int e = tid; e < jb * (s - j0); e += nt) {
      const int t = e % jb, c = j0 + e / jb;
      G[(j0 + t) + (size_t)ld * c] = c >= j0 + t ? P[t * s + c] : zero;
    }
  };
  int prev = -1;
  for (int j0 = 0; j0 < s; j0 += PB) {
    const int jb = min(PB, s - j0);
    if (rank == 0 && prev >= 0) write_back(prev, min(PB, s - prev));
    __syncthreads();
    // 1. panel rows j0..j0+jb-1, columns j0..s-1
    for (int e = tid; e < jb * (s - j0); e += nt) {
      const int t = e % jb, c = j0 + e / jb;
      P[t * s + c] = __ldcg(&G[(j0 + t) + (size_t)ld * c]);
    }
    __syncthreads();
    // 2. factor the panel in shared memory
    for (int t = 0; t < jb; ++t) {
      const int j = j0 + t;
      if (tid == 0) {
        const float4 g = P[t * s + j];
        const double d = (double)g.x + (double)g.y;
        const double pv = (d > thresh && d > 0.0) ? sqrt(d) : 0.0;
        float h, l;
        df_split(pv, h, l);
        P[t * s + j] = make_float4(h, l, 0.f, 0.f);
        df_split(pv > 0.0 ? 1.0 / pv : 0.0, h, l);
        ph[t] = h;
        pl[t] = l;
      }
      __syncthreads();
      for (int c = j + 1 + tid; c < s; c += nt) P[t * s + c] = df_scale(P[t * s + c], ph[t], pl[t]);
      __syncthreads();
      for (int e = tid; e < (jb - t - 1) * (s - j - 1); e += nt) {  // rows below t inside the panel
        const int u = t + 1 + e % (jb - t - 1), c = j + 1 + e / (jb - t - 1);
        if (c < j0 + u) continue;  // only the upper triangle
        const float4 a = P[t * s + j0 + u], b = P[t * s + c];
        float4 g = P[u * s + c];
        df_cmac_ca(g.x, g.y, g.z, g.w, make_float4(-a.x, -a.y, -a.z, -a.w), b);
        P[u * s + c] = g;
      }
      __syncthreads();
    }
    // 3. trailing triangle, this CTA's columns: G_kl -= sum_t conj(R_tk) R_tl, j0+jb <= k <= l;
    //    four rows per lane in flight (the loads are independent)
    for (int l = own(j0 + jb) + C * warp; l < s; l += C * nw) {
      float4 *col = G + (size_t)ld * l;  // written only by this CTA
      for (int k0 = j0 + jb + lane; k0 <= l; k0 += 128) {
        float4 g[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (k0 + 32 * u <= l) g[u] = col[k0 + 32 * u];
        for (int t = 0; t < jb; ++t) {
          const float4 b = P[t * s + l];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (k0 + 32 * u <= l) {
              const float4 a = P[t * s + k0 + 32 * u];
              df_cmac_ca(g[u].x, g[u].y, g[u].z, g[u].w, make_float4(-a.x, -a.y, -a.z, -a.w), b);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (k0 + 32 * u <= l) col[k0 + 32 * u] = g[u];
      }
    }
    prev = j0;
    cluster.sync();
  }
  if (rank == 0) write_back(prev, min(PB, s - prev));
  cluster.sync();
  // Ri = R^-1 (upper), block rows B = [b0, b0+jb) from the bottom, this CTA's columns:
  //   T(B, c) = sum_{l >= b0+jb} R(B, l) Ri(l, c)      (one pass over the rows done)
  //   Ri(B, c) = R(B, B)^-1 (delta(B, c) - T(B, c))    (triangular solve in the block)
  for (int c = own(0); c < s; c += C)
    for (int r = tid; r < s; r += nt) Ri[r + (size_t)ld * c] = zero;
  __syncthreads();
  const int nblk = (s + PB - 1) / PB;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int b0 = bi * PB, jb = min(PB, s - b0);
    for (int e = tid; e < jb * (s - b0); e += nt) {  // R(B, b0..s-1)
      const int t = e % jb, c = b0 + e / jb;
      P[t * s + c] = __ldcg(&G[(b0 + t) + (size_t)ld * c]);
    }
    __syncthreads();
    // T into Ri(B, c), one warp per column c, lanes over l: each Ri(l, c) is
    // loaded once for all jb rows of the block (two loads in flight per lane)
    for (int c = own(b0 + jb) + C * warp; c < s; c += C * nw) {
      const float4 *x = Ri + (size_t)ld * c;
      float acc[16][4];
#pragma unroll
      for (int t = 0; t < 16; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
      for (int l0 = b0 + jb + lane; l0 <= c; l0 += 64) {
        const bool two = l0 + 32 <= c;
        const float4 x0 = x[l0], x1 = two ? x[l0 + 32] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int t = 0; t < 16; ++t)
          if (t < jb) {
            df_cmac(acc[t][0], acc[t][1], acc[t][2], acc[t][3], P[t * s + l0], x0);
            if (two) df_cmac(acc[t][0], acc[t][1], acc[t][2], acc[t][3], P[t * s + l0 + 32], x1);
          }
      }
#pragma unroll
      for (int t = 0; t < 16; ++t)
        if (t < jb) {
          float rh = acc[t][0], rl = acc[t][1], jh = acc[t][2], jl = acc[t][3];
          for (int o = 16; o > 0; o >>= 1) {
            const float a = __shfl_xor_sync(0xffffffffu, rh, o), b = __shfl_xor_sync(0xffffffffu, rl, o);
            const float c2 = __shfl_xor_sync(0xffffffffu, jh, o), d2 = __shfl_xor_sync(0xffffffffu, jl, o);
            df_mac(rh, rl, a, b, 1.f, 0.f);
            df_mac(jh, jl, c2, d2, 1.f, 0.f);
          }
          if (lane == 0) Ri[(b0 + t) + (size_t)ld * c] = make_float4(rh, rl, jh, jl);
        }
    }
    __syncthreads();
    // triangular solve in the block, one thread per column c >= b0
    for (int c = own(b0) + C * tid; c < s; c += C * nt) {
      float4 xs[16];
      for (int t = jb - 1; t >= 0; --t) {
        float4 acc = (b0 + t == c) ? make_float4(1.f, 0.f, 0.f, 0.f) : zero;
        if (c >= b0 + jb) {
          const float4 q = Ri[(b0 + t) + (size_t)ld * c];
          acc = make_float4(-q.x, -q.y, -q.z, -q.w);
        }
        for (int u = t + 1; u < jb; ++u) {
          const float4 r = P[t * s + b0 + u];
          df_cmac(acc.x, acc.y, acc.z, acc.w, make_float4(-r.x, -r.y, -r.z, -r.w), xs[u]);
        }
        const float4 rd = P[t * s + b0 + t];
        const double d = (double)rd.x + (double)rd.y;
        float h, l;
        df_split(d > 0.0 ? 1.0 / d : 0.0, h, l);
        xs[t] = (b0 + t <= c) ? df_scale(acc, h, l) : zero;
      }
      for (int t = 0; t < jb; ++t) Ri[(b0 + t) + (size_t)ld * c] = xs[t];
    }
    __syncthreads();
  }
  double2 *Rd = reinterpret_cast<double2 *>(Ri);
  for (int c = own(0); c < s; c += C)
    for (int r = tid; r < s; r += nt) Rd[r + (size_t)ld * c] = dfd(Ri[r + (size_t)ld * c]);  // back to FP64, in place
}

// the slot's X (m x r, ld m) = the first m rows of U Sigma (ld m_max); k = r
__global__ void k_rs_store(Slot *slots, const RsDims *dims, const char *ws, size_t off, size_t per, int m_max,
                           int r) {
  const int p = blockIdx.y;
  if (dims[p].s == 0) return;
  Slot S = slots[p];
  const int m = S.cp->m;
  const double2 *U = reinterpret_cast<const double2 *>(ws + p * per + off);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)m * r;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % m), c = (int)(e / m);
    S.X[e] = U[i + (size_t)m_max * c];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) S.cp->k = r;
}

// judge: R = Xp^H (U Sigma) (n_max x r, ld n_max); rho_i = |R_i - sigma_i^2 v_i| / sigma_i
// with sigma_i = |column i of U Sigma|; bad[p] = 1 if max rho_i > tol ||Theta||.
// One CTA per bond, one warp per column.
__global__ void k_rs_judge(const Slot *slots, const RsDims *dims, const char *ws, size_t off_u, size_t off_r,
                           size_t per, int m_max, int n_max, const double *nrm, double tol, int *bad,
                           double *worst) {
  const int p = blockIdx.x;
  if (dims[p].s == 0) return;
  const int r = dims[p].r, n = slots[p].cp->n;
  const double2 *U = reinterpret_cast<const double2 *>(ws + p * per + off_u);
  const double2 *R = reinterpret_cast<const double2 *>(ws + p * per + off_r);
  const double2 *V = slots[p].V;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __shared__ double wmax[32];
  double mx = 0.0;
  for (int c = warp; c < r; c += nw) {
    double a = 0.0;
    for (int i = lane; i < m_max; i += 32) {
      const double2 u = U[i + (size_t)m_max * c];
      a = fma(u.x, u.x, fma(u.y, u.y, a));
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    const double s2 = a;  // sigma^2
    double e = 0.0;
    for (int i = lane; i < n; i += 32) {
      const double2 q = R[i + (size_t)n_max * c], v = V[i + (size_t)n * c];
      const double dx = q.x - s2 * v.x, dy = q.y - s2 * v.y;
      e = fma(dx, dx, fma(dy, dy, e));
    }
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    mx = fmax(mx, s2 > 0.0 ? sqrt(e / s2) : 0.0);
  }
  if (lane == 0) wmax[warp] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double w = 0.0;
    for (int i = 0; i < nw; ++i) w = fmax(w, wmax[i]);
    const double rel = w / nrm[p];
    worst[p] = rel;
    bad[p] = !(rel <= tol);  // NaN counts as bad
  }
}

// fallback: the slot's X (m x n, ld m) = Xp again
__global__ void k_rs_restore(Slot *slots, const int *again, const char *ws, size_t per, int m_max) {
  const int p = blockIdx.y;
  if (!again[p]) return;
  const Slot S = slots[p];
  const int m = S.cp->m, n = S.cp->n;
  const double2 *Xp = reinterpret_cast<const double2 *>(ws + p * per);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)m * n;
       e += (size_t)gridDim.x * blockDim.x)
    S.X[e] = Xp[(e % m) + (size_t)m_max * (e / m)];
}

}  // namespace

struct RsState {
  int n_full, sc, chi, nslots;
  RsCarve carve;
  void *ws;          // nslots * carve.per
  double2 *om;       // n_full x sc
  Slot *in_slots_d;  // the s x s problems of the bidiagonal route
  Compact *in_cp_d;
  int *in_path_d;
  RsDims *dims_d;
  int *bad_d;
  double *worst_d;
  std::vector<int> in_path_h;
  // digits of Xp (as the A operand) and of Xp^H, 7 planes, packed once per batch
  unsigned short *xd0, *xd1;
  int *xe0, *xe1;
};

void rsvd_free(tebd_handle *h) {
  RsState *r = static_cast<RsState *>(h->rs);
  if (!r) return;
  cudaFree(r->ws);
  cudaFree(r->om);
  cudaFree(r->in_slots_d);
  cudaFree(r->in_cp_d);
  cudaFree(r->in_path_d);
  cudaFree(r->dims_d);
  cudaFree(r->bad_d);
  cudaFree(r->worst_d);
  cudaFree(r->xd0);
  cudaFree(r->xd1);
  cudaFree(r->xe0);
  cudaFree(r->xe1);
  delete r;
  h->rs = nullptr;
}

// 7 digit planes of an n x n operand for every slot
static size_t rs_digit_bytes(int n, int ns) {
  return sizeof(unsigned short) * kOzMaxS * (size_t)ns * tc_pad(n, kTcBM) * tc_pad(2 * n, kOzBK);
}

static int rsvd_alloc(tebd_handle *h, int sc) {
  RsState *r = static_cast<RsState *>(h->rs);
  if (r && r->sc >= sc) return TEBD_OK;
  if (r) {
    int rc = check_cuda(h, cudaStreamSynchronize(h->stream), "randomized SVD workspace");
    if (rc) return rc;
    rsvd_free(h);
  }
  r = new (std::nothrow) RsState();
  if (!r) return set_error(h, TEBD_ERR_OOM, "randomized SVD state");
  h->rs = r;
  r->n_full = h->n;
  r->sc = sc;
  r->chi = h->chi;
  r->nslots = h->nslots;
  r->carve = rs_carve(h->n, sc, h->chi);
  int rc;
  const int ns = h->nslots;
  if ((rc = check_cuda(h, cudaMalloc(&r->ws, r->carve.per * ns), "alloc randomized SVD workspace")) ||
      (rc = check_cuda(h, cudaMalloc(&r->om, sizeof(double2) * (size_t)h->n * sc), "alloc sketch")) ||
      (rc = check_cuda(h, cudaMalloc(&r->in_slots_d, sizeof(Slot) * ns), "alloc rsvd slots")) ||
      (rc = check_cuda(h, cudaMalloc(&r->in_cp_d, sizeof(Compact) * ns), "alloc rsvd slots")) ||
      (rc = check_cuda(h, cudaMalloc(&r->in_path_d, sizeof(int) * ns), "alloc rsvd slots")) ||
      (rc = check_cuda(h, cudaMalloc(&r->dims_d, sizeof(RsDims) * ns), "alloc rsvd slots")) ||
      (rc = check_cuda(h, cudaMalloc(&r->bad_d, sizeof(int) * ns), "alloc rsvd flags")) ||
      (rc = check_cuda(h, cudaMalloc(&r->worst_d, sizeof(double) * ns), "alloc rsvd flags")) ||
      (rc = check_cuda(h, cudaMalloc(&r->xd0, rs_digit_bytes(h->n, ns)), "alloc rsvd digits")) ||
      (rc = check_cuda(h, cudaMalloc(&r->xd1, rs_digit_bytes(h->n, ns)), "alloc rsvd digits")) ||
      (rc = check_cuda(h, cudaMalloc(&r->xe0, sizeof(int) * ns * (size_t)tc_pad(h->n, kTcBM)), "alloc rsvd digits")) ||
      (rc = check_cuda(h, cudaMalloc(&r->xe1, sizeof(int) * ns * (size_t)tc_pad(h->n, kTcBM)), "alloc rsvd digits"))) {
    rsvd_free(h);
    return rc;
  }
  k_rs_omega<<<256, 256, 0, h->stream>>>(r->om, h->n, sc, 0x5eed5eedULL);
  TEBD_LAUNCHED(h);
  r->in_path_h.assign(ns, kPathQRJ);
  return check_cuda(h, cudaGetLastError(), "sketch generation");
}

// One bidiagonal-route batch on the s x s Grams: problem p's matrix at byte
// offset `off` of its workspace (ld s), its right vectors to offset `voff`
// (ld s); kk triplets.
static int rs_gram_svd(tebd_handle *h, RsState *R, const std::vector<int> &on, int nb, int s, size_t off,
                       size_t voff, int kk) {
  std::vector<Slot> sl(nb);
  std::vector<Compact> cp(nb);
  char *base = static_cast<char *>(R->ws);
  for (int p = 0; p < nb; ++p) {
    Slot &S = sl[p];
    memset(&S, 0, sizeof(S));
    char *w = base + p * R->carve.per;
    S.X = reinterpret_cast<double2 *>(w + off);
    S.V = reinterpret_cast<double2 *>(w + voff);
    S.aux = reinterpret_cast<double2 *>(w + R->carve.aux);
    S.tau = reinterpret_cast<double2 *>(w + R->carve.tau);
    S.taup = reinterpret_cast<double2 *>(w + R->carve.taup);
    S.bdws = reinterpret_cast<double *>(w + R->carve.bdws);
    S.cp = R->in_cp_d + p;
    cp[p] = {0, 0, 0, s, s, s};
    R->in_path_h[p] = on[p] ? kPathBidiag : kPathQRJ;
    if (on[p]) h->stats.gebrd_flops += 16.0 * s * (double)s * s - 16.0 / 3.0 * (double)s * s * s;
  }
  int rc;
  if ((rc = check_cuda(h, cudaMemcpyAsync(R->in_slots_d, sl.data(), sizeof(Slot) * nb, cudaMemcpyHostToDevice,
                                          h->stream), "upload rsvd slots")) ||
      (rc = check_cuda(h, cudaMemcpyAsync(R->in_cp_d, cp.data(), sizeof(Compact) * nb, cudaMemcpyHostToDevice,
                                          h->stream), "upload rsvd slots")) ||
      (rc = check_cuda(h, cudaMemcpyAsync(R->in_path_d, R->in_path_h.data(), sizeof(int) * nb,
                                          cudaMemcpyHostToDevice, h->stream), "upload rsvd routes")) ||
      (rc = check_cuda(h, cudaStreamSynchronize(h->stream), "upload rsvd slots")))  // host vectors go away
    return rc;
  BidiagBatch b;
  b.slots_d = R->in_slots_d;
  b.path_d = R->in_path_d;
  b.path_h = R->in_path_h.data();
  b.nb = nb;
  b.nmax = s;
  b.kk = kk;
  b.dfp = true;  // double-float passes: the s x s Gram's eigenvectors need no more
  b.right_only = 1;  // M = W Lambda W^H: only W is used
  b.phase = 0;
  b.cap = 0;
  return run_bidiag_batch(h, b);
}

// The randomized route for the bonds with route[p] == kPathRsvd (set by the
// caller from the compaction record); on return route[p] is kPathRsvd for the
// accepted bonds and the full route (kPathBidiag / kPathBidiagT) for the bonds
// the judge sent back, whose Theta is back in the slot's X.
int run_rsvd(tebd_handle *h, int nb, const std::vector<Compact> &cps, std::vector<int> &route,
             const std::vector<int> &rank, int sketch, int power) {
  int m_max = 0, n_max = 0, r_max = 0, s = 0;
  std::vector<RsDims> dims(nb, RsDims{0, 0, 0, 0});
  std::vector<int> on(nb, 0);
  for (int p = 0; p < nb; ++p) {
    if (route[p] != kPathRsvd) continue;
    on[p] = 1;
    m_max = std::max(m_max, cps[p].m);
    n_max = std::max(n_max, cps[p].n);
    r_max = std::max(r_max, rank[p]);
    s = std::max(s, std::min(sketch, std::min(cps[p].m, cps[p].n)));
  }
  if (!s) return TEBD_OK;
  s = std::max(s, r_max);
  const int nact = (int)std::count(on.begin(), on.end(), 1);  // bonds on the route
  int rc = rsvd_alloc(h, std::max(s, h->rs_sketch_cap));
  if (rc) return rc;
  h->rs_sketch_cap = std::max(h->rs_sketch_cap, s);
  RsState *R = static_cast<RsState *>(h->rs);
  for (int p = 0; p < nb; ++p)  // one rank for the batch: the s x s SVD computes r_max triplets
    if (on[p]) dims[p] = {cps[p].m, cps[p].n, s, r_max};
  cudaStream_t st = h->stream;
  if ((rc = check_cuda(h, cudaMemcpyAsync(R->dims_d, dims.data(), sizeof(RsDims) * nb, cudaMemcpyHostToDevice, st),
                       "upload rsvd sizes")) ||
      (rc = check_cuda(h, cudaStreamSynchronize(st), "upload rsvd sizes")))
    return rc;
  const size_t per = R->carve.per;
  char *ws = static_cast<char *>(R->ws);
  const RsCarve &c = R->carve;
  const long long pstr = (long long)(per / sizeof(double2));
  const int dstride = (int)(sizeof(RsDims) / sizeof(int));
  const int sk = h->rs_slices, fin = kOzMaxS;
  // out (rows x cols, ld rows, workspace offset oo) = op(A) op(B); A and B are
  // workspace offsets unless a base pointer is given
  auto prod = [&](size_t ao, int lda, int at, const double2 *abase, long long astr, size_t bo, int ldb,
                  const double2 *bbase, long long bstr, int rows, int cols, int k, size_t oo, int slices) -> int {
    ZProd z = {};
    z.a = abase ? abase : reinterpret_cast<const double2 *>(ws + ao);
    z.a_stride = astr;
    z.lda = lda;
    z.a_trans = at;
    z.a_conj = at;
    z.b = bbase ? bbase : reinterpret_cast<const double2 *>(ws + bo);
    z.b_stride = bstr;
    z.ldb = ldb;
    z.nprob = nb;
    z.m = rows;
    z.n = cols;
    z.k = k;
    z.form = 100 + slices;
    z.out = reinterpret_cast<double2 *>(ws + oo);
    z.out_stride = pstr;
    z.rs = 1;
    z.cs = rows;
    z.n_d = &R->dims_d[0].s;  // 0 off the route: those tiles exit at once
    z.dim_stride = dstride;
    z.alpha = 1.0;
    if (!abase && ao == c.xp) {  // Xp or Xp^H: digits packed once for the batch
      z.a_dig = at ? R->xd1 : R->xd0;
      z.a_exp = at ? R->xe1 : R->xe0;
    }
    int e = tc_reserve(h, zprod_ws_bytes(z));
    if (e) return e;
    tc_events(h, zprod_mma_flops(z, nact), &z.ev0, &z.ev1);
    e = check_cuda(h, zprod_run(z, h->tc_ws, h->tc_err, st), "randomized SVD product");
    h->launches += 5;
    h->stats.rsvd_flops += 8.0 * rows * (double)cols * k * nact;
    return e;
  };
  // one diagonal block of n x n (leading dimension ld) of every bond's Gram at
  // byte offset og, its inverse factor to ori: k_rs_chol on a cluster per bond
  auto leaf = [&](size_t og, size_t ori, int ss, int ld) -> int {
    const int nbk = nb;
    int PB = ss <= 512 ? 16 : 8;
    const TuneParams tp = tune_lookup(h, 2, ss, nact);
    if (tp.panel > 0) {  // the autotuner's panel height, when its staging fits
      if ((tp.panel == 4 || tp.panel == 8 || tp.panel == 16) && sizeof(float4) * (size_t)tp.panel * ss <= 200 * 1024)
        PB = tp.panel;
      else
        tune_reject(h);
    }
    const size_t smem = sizeof(float4) * (size_t)PB * ss;
    int e2 = check_cuda(h, cudaFuncSetAttribute(k_rs_chol, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "Cholesky shared memory");
    if (e2) return e2;
    // cluster size: the SMs shared out among the bonds on the route (at most 8),
    // or the autotuner's size when the launch can co-schedule it
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(512, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    auto fits = [&](int cs) {
      cfg.gridDim = dim3(cs, nbk, 1);
      attr[0].val.clusterDim.x = cs;
      int ncl = 0;
      const bool ok = cudaOccupancyMaxActiveClusters(&ncl, (const void *)k_rs_chol, &cfg) == cudaSuccess && ncl >= 1;
      if (!ok) cudaGetLastError();
      return ok;
    };
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int CS = std::max(1, std::min(8, sms / std::max(1, nact)));
    while (CS > 1 && !fits(CS)) --CS;
    if (tp.chol_cluster > 0) {
      if (tp.chol_cluster <= 8 && fits(tp.chol_cluster))
        CS = tp.chol_cluster;
      else
        tune_reject(h);
    }
    cfg.gridDim = dim3(CS, nbk, 1);
    attr[0].val.clusterDim.x = CS;
    e2 = check_cuda(h, cudaLaunchKernelEx(&cfg, k_rs_chol, (const RsDims *)R->dims_d, ws, per, og, ori, ss, ld,
                                          c.th, PB),
                    "Cholesky launch");
    TEBD_LAUNCHED(h);
    return e2;
  };
  // a product on blocks of the workspace: out (rows x cols, leading dimension
  // ldo, byte offset oo) = alpha op(A) B (+ out when acc), op(A) = A or A^H
  auto bprod = [&](size_t ao, int lda, int at, size_t bo, int ldb, int rows, int cols, int k, size_t oo, int ldo,
                   double alpha, int acc, int slices) -> int {
    ZProd z = {};
    z.a = reinterpret_cast<const double2 *>(ws + ao);
    z.a_stride = pstr;
    z.lda = lda;
    z.a_trans = at;
    z.a_conj = at;
    z.b = reinterpret_cast<const double2 *>(ws + bo);
    z.b_stride = pstr;
    z.ldb = ldb;
    z.nprob = nb;
    z.m = rows;
    z.n = cols;
    z.k = k;
    z.form = 100 + slices;
    z.out = reinterpret_cast<double2 *>(ws + oo);
    z.out_stride = pstr;
    z.rs = 1;
    z.cs = ldo;
    z.n_d = &R->dims_d[0].s;  // 0 off the route: those tiles exit at once
    z.dim_stride = dstride;
    z.alpha = alpha;
    z.accumulate = acc;
    int e = tc_reserve(h, zprod_ws_bytes(z));
    if (e) return e;
    tc_events(h, zprod_mma_flops(z, nact), &z.ev0, &z.ev1);
    e = check_cuda(h, zprod_run(z, h->tc_ws, h->tc_err, st), "Cholesky block product");
    h->launches += 5;
    h->stats.rsvd_flops += 8.0 * rows * (double)cols * k * nact;
    return e;
  };
  // Cholesky + inverse of the s x s Gram at c.g into c.ri, recursively by halves
  // above chol_leaf: with G = [G11 G12; G12^H G22] (n1 + n2),
  //   R11 = chol(G11), R12 = R11^-H G12 (in place of G12), G22 -= R12^H R12,
  //   R22 = chol(G22), Ri12 = -Ri11 (R12 Ri22) (R12 Ri22 through c.w),
  // the off-diagonal work as digit-plane products on the tensor cores, the
  // diagonal leaves in k_rs_chol.  Every pivot is judged against the whole
  // Gram's threshold.
  int chol_leaf = 384;  // the default; the autotuner may set it per sketch width
  std::function<int(size_t, size_t, int, int)> crec = [&](size_t gb, size_t rb, int n, int sl) -> int {
    if (n <= chol_leaf) return leaf(gb, rb, n, s);
    const int n1 = (n / 2 + 31) / 32 * 32, n2 = n - n1;
    const size_t col = sizeof(double2) * (size_t)s;  // bytes per column (ld s)
    const size_t g12 = gb + col * n1, g22 = gb + col * n1 + sizeof(double2) * n1;
    const size_t r12 = rb + col * n1, r22 = rb + col * n1 + sizeof(double2) * n1;
    int e;
    if ((e = crec(gb, rb, n1, sl)) || (e = bprod(rb, s, 1, g12, s, n1, n2, n1, g12, s, 1.0, 0, sl)) ||
        (e = bprod(g12, s, 1, g12, s, n2, n2, n1, g22, s, -1.0, 1, sl)) || (e = crec(g22, r22, n2, sl)) ||
        (e = bprod(g12, s, 0, r22, s, n1, n2, n2, c.w, n1, 1.0, 0, sl)) ||
        (e = bprod(rb, s, 0, c.w, n1, n1, n2, n1, r12, s, -1.0, 0, sl)))
      return e;
    return TEBD_OK;
  };
  auto rs_chol = [&](int ss, double fl, int sl) -> int {
    const TuneParams tb = tune_lookup(h, 3, ss, nact);
    chol_leaf = 384;
    if (tb.chol_leaf > 0) {
      if (tb.chol_leaf >= 64 && tb.chol_leaf <= kRsvdMaxSketch)
        chol_leaf = tb.chol_leaf;
      else
        tune_reject(h);
    }
    k_rs_thresh<<<nb, 256, 0, st>>>(R->dims_d, ws, per, c.g, ss, fl, c.th);
    TEBD_LAUNCHED(h);
    int e = check_cuda(h, cudaMemset2DAsync(ws + c.ri, per, 0, sizeof(double2) * (size_t)ss * ss, nb, st),
                       "Cholesky inverse reset");
    return e ? e : crec(c.g, c.ri, ss, sl);
  };
  // CholQR of the rows x s block at `buf` (ld rows), through `tmp`: one pass for
  // the range finder's intermediate bases (only their span matters), two (CholQR2,
  // the second with 7 planes) for the final basis P; the result is left in `buf`.
  // The sketch's width s is at most kRsvdMaxSketch (the Cholesky stages panels of
  // 8 rows of R, 8 x 1536 x 16 B = 192 KB of shared memory at the largest).
  auto cholqr2 = [&](size_t buf, size_t tmp, int rows, bool twice) -> int {
    int e;
    if ((e = prod(buf, rows, 1, nullptr, pstr, buf, rows, nullptr, pstr, s, s, rows, c.g, sk))) return e;
    if ((e = rs_chol(s, ldexp(1.0, -7 * sk + 9), sk))) return e;
    if ((e = prod(buf, rows, 0, nullptr, pstr, c.ri, s, nullptr, pstr, rows, s, s, tmp, sk))) return e;
    if (!twice)  // one pass: back into buf
      return check_cuda(h, cudaMemcpy2DAsync(ws + buf, per, ws + tmp, per, sizeof(double2) * (size_t)rows * s, nb,
                                             cudaMemcpyDeviceToDevice, st),
                        "CholQR copy");
    if ((e = prod(tmp, rows, 1, nullptr, pstr, tmp, rows, nullptr, pstr, s, s, rows, c.g, fin))) return e;
    if ((e = rs_chol(s, ldexp(1.0, -7 * fin + 9), fin))) return e;
    return prod(tmp, rows, 0, nullptr, pstr, c.ri, s, nullptr, pstr, rows, s, s, buf, fin);
  };
  // 1. padded copy
  k_rs_pad<<<dim3(256, nb), 256, 0, st>>>(h->slots_d, R->dims_d, reinterpret_cast<double2 *>(ws), per, m_max,
                                           n_max);
  TEBD_LAUNCHED(h);
  {
    const double2 *xp0 = reinterpret_cast<const double2 *>(ws + c.xp);
    if ((rc = check_cuda(h, oz_pack_a(xp0, pstr, m_max, m_max, n_max, 0, 0, nb, tc_pad(m_max, kTcBM),
                                      tc_pad(2 * n_max, kOzBK), fin, R->xd0, R->xe0, st),
                         "pack Xp")) ||
        (rc = check_cuda(h, oz_pack_a(xp0, pstr, m_max, n_max, m_max, 1, 1, nb, tc_pad(n_max, kTcBM),
                                      tc_pad(2 * m_max, kOzBK), fin, R->xd1, R->xe1, st),
                         "pack Xp^H")))
      return rc;
    h->launches += 4;
  }
  // 2. range finder
  if ((rc = prod(c.xp, m_max, 0, nullptr, pstr, 0, R->n_full, R->om, 0, m_max, s, n_max, c.a, sk)) ||
      (rc = cholqr2(c.a, c.b, m_max, false)))
    return rc;
  for (int it = 0; it < power; ++it)
    if ((rc = prod(c.xp, m_max, 1, nullptr, pstr, c.a, m_max, nullptr, pstr, n_max, s, m_max, c.z, sk)) ||
        (rc = cholqr2(c.z, c.b, n_max, false)) ||
        (rc = prod(c.xp, m_max, 0, nullptr, pstr, c.z, n_max, nullptr, pstr, m_max, s, n_max, c.a, sk)) ||
        (rc = cholqr2(c.a, c.b, m_max, false)))
      return rc;
  if ((rc = prod(c.xp, m_max, 1, nullptr, pstr, c.a, m_max, nullptr, pstr, n_max, s, m_max, c.z, sk)) ||
      (rc = cholqr2(c.z, c.b, n_max, true)))
    return rc;
  // 3. Rayleigh-Ritz: C = Xp P, M = C^H C, M = W Lambda W^H
  if ((rc = prod(c.xp, m_max, 0, nullptr, pstr, c.z, n_max, nullptr, pstr, m_max, s, n_max, c.c, fin)) ||
      (rc = prod(c.c, m_max, 1, nullptr, pstr, c.c, m_max, nullptr, pstr, s, s, m_max, c.g, fin)) ||
      (rc = rs_gram_svd(h, R, on, nb, s, c.g, c.w, r_max)))
    return rc;
  // 4. V = P W -> the slot's V (ld n); U Sigma = C W -> the slot's X (ld m); k = r
  {
    ZProd z = {};
    z.a = reinterpret_cast<const double2 *>(ws + c.z);
    z.a_stride = pstr;
    z.lda = n_max;
    z.b = reinterpret_cast<const double2 *>(ws + c.w);
    z.b_stride = pstr;
    z.ldb = s;
    z.nprob = nb;
    z.m = n_max;
    z.n = r_max;
    z.k = s;
    z.form = 100 + fin;
    z.rs = 1;
    z.cs = 0;  // ld = the bond's n (its m_d entry below)
    z.m_d = &R->dims_d[0].n;
    z.n_d = &R->dims_d[0].r;
    z.dim_stride = dstride;
    z.alpha = 1.0;
    z.optr = reinterpret_cast<const unsigned char *>(h->slots_d) + offsetof(Slot, V);
    z.optr_stride = (int)sizeof(Slot);
    if ((rc = tc_reserve(h, zprod_ws_bytes(z)))) return rc;
    tc_events(h, zprod_mma_flops(z, nact), &z.ev0, &z.ev1);
    if ((rc = check_cuda(h, zprod_run(z, h->tc_ws, h->tc_err, st), "randomized SVD V"))) return rc;
    h->launches += 5;
  }
  if ((rc = prod(c.c, m_max, 0, nullptr, pstr, c.w, s, nullptr, pstr, m_max, r_max, s, c.a, fin))) return rc;
  k_rs_store<<<dim3(256, nb), 256, 0, st>>>(h->slots_d, R->dims_d, ws, c.a, per, m_max, r_max);
  TEBD_LAUNCHED(h);
  // 5. judge: R = Xp^H (U Sigma), residuals of the kept triplets
  if ((rc = prod(c.xp, m_max, 1, nullptr, pstr, c.a, m_max, nullptr, pstr, n_max, r_max, m_max, c.rr, fin)))
    return rc;
  k_rs_judge<<<nb, 256, 0, st>>>(h->slots_d, R->dims_d, ws, c.a, c.rr, per, m_max, n_max, h->nrm, h->rs_tol,
                                 R->bad_d, R->worst_d);
  TEBD_LAUNCHED(h);
  std::vector<int> bad(nb, 0);
  std::vector<double> worst(nb, 0.0);
  if ((rc = check_cuda(h, cudaMemcpyAsync(bad.data(), R->bad_d, sizeof(int) * nb, cudaMemcpyDeviceToHost, st),
                       "read rsvd judge")) ||
      (rc = check_cuda(h, cudaMemcpyAsync(worst.data(), R->worst_d, sizeof(double) * nb, cudaMemcpyDeviceToHost, st),
                       "read rsvd judge")) ||
      (rc = check_cuda(h, cudaStreamSynchronize(st), "randomized SVD")) || (rc = tc_check(h)))
    return rc;
  int nagain = 0;
  for (int p = 0; p < nb; ++p) {
    if (!on[p]) {
      bad[p] = 0;
      continue;
    }
    h->stats.rsvd_updates++;
    h->stats.rsvd_worst_residual = std::max(h->stats.rsvd_worst_residual, worst[p]);
    if (bad[p]) {
      ++nagain;
      h->stats.rsvd_fallbacks++;
      route[p] = cps[p].m >= cps[p].n ? kPathBidiag : kPathBidiagT;
    }
  }
  if (nagain) {
    if ((rc = check_cuda(h, cudaMemcpyAsync(R->bad_d, bad.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st),
                         "upload rsvd fallback")))
      return rc;
    k_rs_restore<<<dim3(256, nb), 256, 0, st>>>(h->slots_d, R->bad_d, ws, per, m_max);
    TEBD_LAUNCHED(h);
    if ((rc = check_cuda(h, cudaStreamSynchronize(st), "randomized SVD fallback"))) return rc;
  }
  return check_cuda(h, cudaGetLastError(), "randomized SVD");
}

}  // namespace tebd

using namespace tebd;

extern "C" int tebd_set_rsvd(tebd_handle *h, int oversample, int power_iters, double tol, int slices) {
  if (!h) return TEBD_ERR_ARG;
  if (oversample < 0 || power_iters < 0 || power_iters > 4 || !(tol > 0.0 && tol < 1.0) || slices < 3 ||
      slices > kOzMaxS)
    return set_error(h, TEBD_ERR_ARG, "rsvd: oversample >= 0, 0 <= power_iters <= 4, 0 < tol < 1, 3 <= slices <= 7");
  h->rs_oversample = oversample;
  h->rs_power = power_iters;
  h->rs_tol = tol;
  h->rs_slices = slices;
  return TEBD_OK;
}
