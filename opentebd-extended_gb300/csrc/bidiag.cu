// bidiag.cu -- SVD of a large compacted Theta through Householder bidiagonalisation,
// computing only the chi singular triplets the update keeps.
//
// Replaces SVDTruncation's ZGESVD('A','A') (local_operations_module.f90:322-345)
// for bonds whose compacted Theta is m x n with m >= n >= max(256, 2 chi') (the
// saturated regime, where the rank k approaches n and the Jacobi route's
// O(n k^2)-per-sweep cost dominates).  FormLambda1/FormGamma1/FormGamma2 read
// only the first chi singular values and vectors, so only those are computed:
//   1. ZGEBD2 semantics: Q^H Theta P = B, B real upper bidiagonal (ZLARFG makes
//      beta real), left reflectors H(i) = I - tauq v v^H below the diagonal,
//      right reflectors G(i) = I - taup u u^H (u also copied column-wise to aux).
//   2. Singular values of B: bisection with Sturm counts on the Golub-Kahan
//      tridiagonal (zero diagonal, off-diagonals d0,e0,d1,...,d_{n-1}; its
//      eigenvalues are +-sigma), one thread per kept value, stopped at relative
//      width 2 eps.
//   3. Singular vectors of B: inverse iteration on the Golub-Kahan matrix shifted
//      by sigma_i (tridiagonal LU with partial pivoting, 3 solves from a fixed
//      pseudo-random start), eigenvector z = (v0,u0,v1,u1,...)/sqrt2; then the
//      u's and the v's are each re-orthogonalised (classical Gram-Schmidt applied
//      twice) in descending sigma order, which restores orthogonality inside
//      clusters of nearby values.
//   4. U = Q [Ub; 0], V = P Vb by applying the reflectors in reverse, one warp per
//      kept column; X(:,i) = U(:,i) sigma_i, V(:,i), the same layout the sort and
//      restore kernels read from the Jacobi routes.
// All arithmetic is FP64.  Cost: 32/3 n^3 (bidiagonalisation) + 16 (m+n) n chi'
// (back-transformation) instead of the Jacobi route's many O(n k^2) sweeps.
#include <cooperative_groups.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "df.cuh"
#include "tebd_internal.cuh"

namespace tebd {

namespace {
constexpr int kBW = 16;   // warps per CTA of the bidiagonalisation kernel

__device__ __forceinline__ double bsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

__device__ __forceinline__ bool on_route(int p) { return p == kPathBidiag || p == kPathBidiagT; }

// The matrix that is bidiagonalised, M x N with M >= N, in place in S.X (ld M):
// Theta itself (m x n) or, on the transposed route, Theta^H (n x m).
__device__ __forceinline__ void bd_dims(const Compact &cp, int p, int &M, int &N) {
  M = p == kPathBidiagT ? cp.n : cp.m;
  N = p == kPathBidiagT ? cp.m : cp.n;
}

// bdws layout of one bond (doubles): d (n), e (n), sigma (kk), then from an even
// offset the inverse-iteration scratch U0, U1, U2, PV, Y (2n x K each), the
// eigenvectors Z (2n x K) and the left vectors Yu (m x K complex, 16-byte aligned)
__host__ __device__ __forceinline__ size_t bd_scratch(int n, int kk) {
  return ((size_t)2 * n + kk + 1) & ~(size_t)1;
}

}  // namespace

// ---------------------------------------------------------------------------
// 1. Householder bidiagonalisation of the M x N matrix in S.X (ld M), M >= N,
//    in panels of kPanel columns (the delayed-update scheme of LAPACK's ZGEBRD /
//    ZLABRD).  Inside a panel the trailing matrix keeps its panel-start values A0
//    and the current matrix is A0 - V Y^H - Xp U^H, with v_k, u_k the panel's
//    left/right reflectors, y_k = tauq_k A^H v_k and x_k = taup_k A u_k.  Each
//    column costs two read-only passes over A0 (z = A0^H v, w = A0 u) plus
//    rank-2j corrections; at the panel end A0 <- A0 - V Y^H - Xp U^H.
//    One cluster per bond, four cluster barriers per column:
//      S1  column i corrected and its norm partials posted
//      S2  z = A0^H v and the small dots V^H v, Xp^H v posted
//      S3  y_i and row i corrected, row-norm partials posted, v_i stored
//      S4  w = A0 u by column chunks, Y^H u and U^H u posted, u_i stored
//    Every CTA recomputes the reflector scalars from the posted partial norms
//    (same values, same order), so no barrier waits on a single CTA's scalar work.
//    Output (as ZGEBD2): d, e in bdws; tauq in S.tau, v_i below the diagonal of
//    column i; taup in S.taup, u_i in column i of Pv with u_i(i+1) = 1.
// ---------------------------------------------------------------------------
constexpr int kDfLoads = 8;  // loads in flight per lane in the double-float passes
constexpr int kPanel = 8;   // columns per panel (narrow: the per-column corrections grow with it)
constexpr int kChunk = 32;  // columns per task of the w = A0 u pass
constexpr int kTile = 64;   // trailing-update tile (rows and columns)
constexpr int kKc = 16;     // trailing-update k chunk staged in shared memory
constexpr int kS = kTile + 8;  // staging stride (doubles): a fragment load is two wavefronts
constexpr size_t kStageDoubles = 4 * (size_t)kKc * kS;

// D += A B on the FP64 tensor pipe: mma m8n8k4, one A element (row lane/4, col lane%4),
// one B element (row lane%4, col lane/4), two D elements (row lane/4, cols 2(lane%4)+{0,1})
__device__ __forceinline__ void dmma(double &d0, double &d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

struct BdAux {
  double2 *Pv, *Yb, *Xb, *zb, *s1, *s2, *t1, *t2, *part;
  double *nrmL, *nrmR;
};

__host__ __device__ __forceinline__ size_t bd_aux_elems(int M, int N) {
  const int P = N < kPanel ? N : kPanel;
  return (size_t)N * N + (size_t)(N + M) * P + N + 4 * (size_t)P +
         (size_t)((N + kChunk - 1) / kChunk) * M + 16;
}

__device__ __forceinline__ BdAux bd_aux(double2 *aux, int M, int N) {
  const int P = min(kPanel, N);
  BdAux a;
  size_t o = 0;
  a.Pv = aux;
  o += (size_t)N * N;
  a.Yb = aux + o;  // N x P, ld N
  o += (size_t)N * P;
  a.Xb = aux + o;  // M x P, ld M
  o += (size_t)M * P;
  a.zb = aux + o;
  o += N;
  a.s1 = aux + o;
  a.s2 = a.s1 + P;
  a.t1 = a.s2 + P;
  a.t2 = a.t1 + P;
  o += 4 * (size_t)P;
  a.part = aux + o;  // ceil(N / kChunk) x M
  o += (size_t)((N + kChunk - 1) / kChunk) * M;
  a.nrmL = reinterpret_cast<double *>(aux + o);  // 8 per-CTA partial norms each
  a.nrmR = a.nrmL + 8;
  return a;
}

__device__ __forceinline__ double2 ldc(const double2 *p) { return __ldcg(p); }

// acc += conj(a) b
__device__ __forceinline__ void mac_ca(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
}
// acc += a b
__device__ __forceinline__ void mac(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
// acc -= a b
__device__ __forceinline__ void msub(double2 &acc, double2 a, double2 b) {
  acc.x = fma(-a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(-a.x, b.y, fma(-a.y, b.x, acc.y));
}
// acc -= a conj(b)
__device__ __forceinline__ void msub_cb(double2 &acc, double2 a, double2 b) {
  acc.x = fma(-a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
}

// ZLARFG's scalars from alpha and ||x||^2: beta (real), tau, and 1/(alpha - beta),
// the factor that turns x into the reflector's tail.
__device__ void larfg_scalars(double2 alpha, double xn2, double &beta, double2 &tau, double2 &sc) {
  if (xn2 == 0.0 && alpha.y == 0.0) {  // H = I, x left as it is
    beta = alpha.x;
    tau = make_double2(0.0, 0.0);
    sc = make_double2(1.0, 0.0);
    return;
  }
  beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2), alpha.x);
  tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
  const double dr = alpha.x - beta, di = alpha.y, den = dr * dr + di * di;
  sc = make_double2(dr / den, -di / den);
}

// CTA-wide sum, valid in every thread
__device__ double block_sum(double v, double *red) {
  v = bsum(v);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

__global__ void __launch_bounds__(kBW * 32) k_gebrd(Slot *slots, const int *path) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;  // uniform per cluster
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  double2 *A = S.X;
  double *dd = S.bdws, *ee = S.bdws + N;
  const BdAux ax = bd_aux(S.aux, M, N);
  const int C = (int)cluster.num_blocks(), crank = (int)cluster.block_rank();
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int gt = crank * nthr + tid, gthr = C * nthr;
  const int warp = tid >> 5, lane = tid & 31;
  const int gw = crank * (nthr >> 5) + warp, nw = C * (nthr >> 5);
  extern __shared__ double2 sh[];
  double2 *vec = sh;                    // max(M, N): v or u of the current column
  double2 *sm = sh + max(M, N);         // 4 kPanel small per-column vectors
  double *stg = reinterpret_cast<double *>(sm + 4 * kPanel);  // trailing-update staging
  __shared__ double red[32];
#define AE(r, c) A[(size_t)(r) + (size_t)M * (c)]
#define YB(c, k) ax.Yb[(size_t)(c) + (size_t)N * (k)]
#define XB(r, k) ax.Xb[(size_t)(r) + (size_t)M * (k)]
#define PV(c, k) ax.Pv[(size_t)(c) + (size_t)N * (k)]
  {  // norm partials of column 0 below the diagonal
    double acc = 0.0;
    for (int r = 1 + gt; r < M; r += gthr) {
      const double2 a = ldc(&AE(r, 0));
      acc = fma(a.x, a.x, fma(a.y, a.y, acc));
    }
    acc = block_sum(acc, red);
    if (tid == 0) ax.nrmL[crank] = acc;
  }
  cluster.sync();
  for (int p = 0; p < N; p += kPanel) {
    const int jb = min(kPanel, N - p);
    for (int j = 0; j < jb; ++j) {
      const int i = p + j;
      // ---- left reflector of column i (every CTA, identical inputs) ----
      double beta;
      double2 tau, sc;
      {
        double xn2 = 0.0;
        for (int q = 0; q < C; ++q) xn2 += __ldcg(&ax.nrmL[q]);
        larfg_scalars(ldc(&AE(i, i)), xn2, beta, tau, sc);
      }
      if (crank == 0 && tid == 0) {
        dd[i] = beta;
        S.tau[i] = tau;
      }
      if (i == N - 1) {  // last column: left reflector only
        for (int r = i + 1 + gt; r < M; r += gthr) AE(r, i) = cmul(ldc(&AE(r, i)), sc);
        break;
      }
      // ---- S2: z = A0(i:M, i+1:N)^H v, s1 = V^H v, s2 = Xp^H v ----
      for (int r = i + tid; r < M; r += nthr)
        vec[r - i] = r == i ? make_double2(1.0, 0.0) : cmul(ldc(&AE(r, i)), sc);
      __syncthreads();
      {
        const int ncol = N - i - 1, items = ncol + 2 * j;
        for (int it = gw; it < items; it += nw) {
          const double2 *col = it < ncol       ? &AE(0, i + 1 + it)
                               : it < ncol + j ? &AE(0, p + (it - ncol))
                                               : &XB(0, it - ncol - j);
          double2 acc = make_double2(0.0, 0.0);  // sum_r conj(col(r)) v(r)
          int r = i + lane;
          for (; r + 224 < M; r += 256) {
            double2 c[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) c[q] = ldc(col + r + 32 * q);
#pragma unroll
            for (int q = 0; q < 8; ++q) mac_ca(acc, c[q], vec[r + 32 * q - i]);
          }
          for (; r < M; r += 32) mac_ca(acc, ldc(col + r), vec[r - i]);
          acc.x = bsum(acc.x);
          acc.y = bsum(acc.y);
          if (lane == 0) {
            if (it < ncol)
              ax.zb[i + 1 + it] = acc;
            else if (it < ncol + j)
              ax.s1[it - ncol] = acc;
            else
              ax.s2[it - ncol - j] = acc;
          }
        }
      }
      cluster.sync();
      // ---- S3: y_i = tauq (z - Y s1 - U s2); row i of the current matrix ----
      if (tid < j) {
        sm[tid] = ldc(&ax.s1[tid]);
        sm[kPanel + tid] = ldc(&ax.s2[tid]);
        sm[2 * kPanel + tid] = ldc(&AE(i, p + tid));  // v_k(i)
        sm[3 * kPanel + tid] = ldc(&XB(i, tid));      // x_k(i)
      }
      __syncthreads();
      {
        double acc = 0.0;
        for (int c = i + 1 + gt; c < N; c += gthr) {
          double2 y = ldc(&ax.zb[c]);
          double2 rr = ldc(&AE(i, c));
          for (int k = 0; k < j; ++k) {
            const double2 yk = ldc(&YB(c, k)), uk = ldc(&PV(c, p + k));
            msub(y, yk, sm[k]);
            msub(y, uk, sm[kPanel + k]);
            msub_cb(rr, sm[2 * kPanel + k], yk);
            msub_cb(rr, sm[3 * kPanel + k], uk);
          }
          y = cmul(tau, y);
          YB(c, j) = y;
          rr.x -= y.x;  // v_i(i) = 1: rr -= conj(y)
          rr.y += y.y;
          AE(i, c) = rr;
          if (c >= i + 2) acc = fma(rr.x, rr.x, fma(rr.y, rr.y, acc));
        }
        acc = block_sum(acc, red);
        if (tid == 0) ax.nrmR[crank] = acc;
      }
      for (int r = i + 1 + gt; r < M; r += gthr) AE(r, i) = cmul(ldc(&AE(r, i)), sc);  // v_i
      cluster.sync();
      // ---- right reflector of row i (every CTA) ----
      double beta2;
      double2 tau2, sc2;
      {
        double xn2 = 0.0;
        for (int q = 0; q < C; ++q) xn2 += __ldcg(&ax.nrmR[q]);
        larfg_scalars(cconj(ldc(&AE(i, i + 1))), xn2, beta2, tau2, sc2);
      }
      if (crank == 0 && tid == 0) {
        ee[i] = beta2;
        S.taup[i] = tau2;
      }
      // ---- S4: w = A0(i+1:M, i+1:N) u by column chunks, t1 = Y^H u, t2 = U^H u ----
      for (int c = i + 1 + tid; c < N; c += nthr)
        vec[c - i - 1] = c == i + 1 ? make_double2(1.0, 0.0) : cmul(cconj(ldc(&AE(i, c))), sc2);
      __syncthreads();
      {
        const int rows = M - i - 1, cols = N - i - 1;
        const int nrb = (rows + 31) / 32, ncc = (cols + kChunk - 1) / kChunk;
        const int tasks = nrb * ncc, items = tasks + 2 * j + 1;
        for (int it = gw; it < items; it += nw) {
          if (it < tasks) {
            const int rb = it % nrb, cc = it / nrb;
            const int r = i + 1 + rb * 32 + lane;
            const int c0 = i + 1 + cc * kChunk, c1 = min(N, c0 + kChunk);
            if (r < M) {
              double2 acc = make_double2(0.0, 0.0);
              const double2 *rp = &AE(r, 0);
              int c = c0;
              for (; c + 7 < c1; c += 8) {
                double2 a[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) a[q] = ldc(rp + (size_t)M * (c + q));
#pragma unroll
                for (int q = 0; q < 8; ++q) mac(acc, a[q], vec[c + q - i - 1]);
              }
              for (; c < c1; ++c) mac(acc, ldc(rp + (size_t)M * c), vec[c - i - 1]);
              ax.part[(size_t)cc * M + r] = acc;
            }
          } else {
            const int k = it - tasks;  // 0..j: t1 over y_k; j+1..2j: t2 over u_(k-j-1)
            const double2 *cp = k <= j ? &YB(0, k) : &PV(0, p + k - j - 1);
            double2 acc = make_double2(0.0, 0.0);
            for (int c = i + 1 + lane; c < N; c += 32) mac_ca(acc, ldc(cp + c), vec[c - i - 1]);
            acc.x = bsum(acc.x);
            acc.y = bsum(acc.y);
            if (lane == 0) {
              if (k <= j)
                ax.t1[k] = acc;
              else
                ax.t2[k - j - 1] = acc;
            }
          }
        }
        for (int c = i + 1 + gt; c < N; c += gthr) PV(c, i) = vec[c - i - 1];  // u_i
      }
      cluster.sync();
      // ---- x_i = taup (w - V t1 - Xp t2); then column i+1 of the current matrix ----
      const bool next_in_panel = j + 1 < jb;
      if (tid <= j) {
        sm[tid] = ldc(&ax.t1[tid]);
        if (tid < j) sm[kPanel + tid] = ldc(&ax.t2[tid]);
        if (next_in_panel) {
          sm[2 * kPanel + tid] = ldc(&YB(i + 1, tid));      // y_k(i+1)
          sm[3 * kPanel + tid] = ldc(&PV(i + 1, p + tid));  // u_k(i+1)
        }
      }
      __syncthreads();
      {
        const int ncc = (N - i - 1 + kChunk - 1) / kChunk;
        double acc = 0.0;
        for (int r = i + 1 + gt; r < M; r += gthr) {
          double2 w = make_double2(0.0, 0.0);
          for (int q = 0; q < ncc; ++q) {  // fixed order
            const double2 t = ldc(&ax.part[(size_t)q * M + r]);
            w.x += t.x;
            w.y += t.y;
          }
          for (int k = 0; k <= j; ++k) msub(w, ldc(&AE(r, p + k)), sm[k]);
          for (int k = 0; k < j; ++k) msub(w, ldc(&XB(r, k)), sm[kPanel + k]);
          const double2 x = cmul(tau2, w);
          XB(r, j) = x;
          if (next_in_panel) {
            double2 a = ldc(&AE(r, i + 1));
            for (int k = 0; k <= j; ++k) {
              msub_cb(a, ldc(&AE(r, p + k)), sm[2 * kPanel + k]);
              msub_cb(a, k < j ? ldc(&XB(r, k)) : x, sm[3 * kPanel + k]);
            }
            AE(r, i + 1) = a;
            if (r >= i + 2) acc = fma(a.x, a.x, fma(a.y, a.y, acc));
          }
        }
        if (next_in_panel) {
          acc = block_sum(acc, red);
          if (tid == 0) ax.nrmL[crank] = acc;
        }
      }
      cluster.sync();
    }
    const int q = p + jb;
    if (q >= N) break;
    // ---- panel end: A0(q:M, q:N) -= V Y^H + Xp U^H (inner dimension 2 jb) ----
    // 64 x 64 tiles over the cluster's CTAs; each warp owns a 16 x 16 block and
    // accumulates its real and imaginary parts with four real DMMAs per k-step:
    //   Re -= Lr Rr^T + Li Ri^T,  Im -= Li Rr^T - Lr Ri^T   (L = [V Xp], R = [Y U])
    {
      const int K2 = 2 * jb;
      const int ntr = (M - q + kTile - 1) / kTile, ntc = (N - q + kTile - 1) / kTile;
      double *Lr = stg, *Li = stg + kKc * kS, *Rr = stg + 2 * kKc * kS, *Ri = stg + 3 * kKc * kS;
      const int wr = (warp & 3) * 16, wc = (warp >> 2) * 16;
      const int fr = lane >> 2, fk = lane & 3;
      for (int t = crank; t < ntr * ntc; t += C) {
        const int r0 = q + (t % ntr) * kTile, c0 = q + (t / ntr) * kTile;
        double cr[2][2][2], ci[2][2][2];
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
          for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int e = 0; e < 2; ++e) cr[x][y][e] = ci[x][y][e] = 0.0;
        for (int kc = 0; kc < K2; kc += kKc) {
          __syncthreads();
          for (int e = tid; e < kKc * kTile; e += nthr) {
            const int rr = e % kTile, kk = e / kTile, k = kc + kk;
            const int r = r0 + rr, c = c0 + rr;
            double2 l = make_double2(0.0, 0.0), g = make_double2(0.0, 0.0);
            if (k < K2) {
              if (r < M) l = k < jb ? ldc(&AE(r, p + k)) : ldc(&XB(r, k - jb));
              if (c < N) g = k < jb ? ldc(&YB(c, k)) : ldc(&PV(c, p + k - jb));
            }
            Lr[kk * kS + rr] = l.x;
            Li[kk * kS + rr] = l.y;
            Rr[kk * kS + rr] = g.x;
            Ri[kk * kS + rr] = g.y;
          }
          __syncthreads();
#pragma unroll
          for (int ks = 0; ks < kKc; ks += 4) {
            const int ko = (ks + fk) * kS;
            double ar[2], ai[2], br[2], bi[2];
#pragma unroll
            for (int b = 0; b < 2; ++b) {
              ar[b] = Lr[ko + wr + 8 * b + fr];
              ai[b] = Li[ko + wr + 8 * b + fr];
              br[b] = Rr[ko + wc + 8 * b + fr];
              bi[b] = Ri[ko + wc + 8 * b + fr];
            }
#pragma unroll
            for (int x = 0; x < 2; ++x)
#pragma unroll
              for (int y = 0; y < 2; ++y) {
                dmma(cr[x][y][0], cr[x][y][1], -ar[x], br[y]);
                dmma(cr[x][y][0], cr[x][y][1], -ai[x], bi[y]);
                dmma(ci[x][y][0], ci[x][y][1], -ai[x], br[y]);
                dmma(ci[x][y][0], ci[x][y][1], ar[x], bi[y]);
              }
          }
        }
#pragma unroll
        for (int x = 0; x < 2; ++x) {
          const int r = r0 + wr + 8 * x + fr;
          if (r >= M) continue;
#pragma unroll
          for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const int c = c0 + wc + 8 * y + 2 * fk + e;
              if (c >= N) continue;
              double2 v = ldc(&AE(r, c));
              v.x += cr[x][y][e];
              v.y += ci[x][y][e];
              AE(r, c) = v;
            }
        }
      }
    }
    cluster.sync();
    {  // norm partials of column q below the diagonal
      double acc = 0.0;
      for (int r = q + 1 + gt; r < M; r += gthr) {
        const double2 a = ldc(&AE(r, q));
        acc = fma(a.x, a.x, fma(a.y, a.y, acc));
      }
      acc = block_sum(acc, red);
      if (tid == 0) ax.nrmL[crank] = acc;
    }
    cluster.sync();
  }
#undef AE
#undef YB
#undef XB
#undef PV
}

// warp sum of a double-float, as a double (each lane's pair is exact in FP64)
__device__ __forceinline__ double df_warp_sum(float h, float l) { return bsum((double)h + (double)l); }

__global__ void __launch_bounds__(kBW * 32) k_gebrd_df(Slot *slots, const int *path) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;  // uniform per cluster
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  float4 *A = reinterpret_cast<float4 *>(S.X);  // (re_hi, re_lo, im_hi, im_lo)
  double *dd = S.bdws, *ee = S.bdws + N;
  const BdAux ax = bd_aux(S.aux, M, N);
  const int C = (int)cluster.num_blocks(), crank = (int)cluster.block_rank();
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int gt = crank * nthr + tid, gthr = C * nthr;
  const int warp = tid >> 5, lane = tid & 31;
  const int gw = crank * (nthr >> 5) + warp, nw = C * (nthr >> 5);
  extern __shared__ double2 sh[];
  float4 *vec = reinterpret_cast<float4 *>(sh);  // max(M, N): v or u of the current column
  double2 *sm = sh + max(M, N);         // 4 kPanel small per-column vectors
  double *stg = reinterpret_cast<double *>(sm + 4 * kPanel);  // trailing-update staging
  __shared__ double red[32];
#define AE(r, c) A[(size_t)(r) + (size_t)M * (c)]
#define YB(c, k) ax.Yb[(size_t)(c) + (size_t)N * (k)]
#define XB(r, k) ax.Xb[(size_t)(r) + (size_t)M * (k)]
#define PV(c, k) ax.Pv[(size_t)(c) + (size_t)N * (k)]
  {  // norm partials of column 0 below the diagonal
    double acc = 0.0;
    for (int r = 1 + gt; r < M; r += gthr) {
      const double2 a = dfl(&AE(r, 0));
      acc = fma(a.x, a.x, fma(a.y, a.y, acc));
    }
    acc = block_sum(acc, red);
    if (tid == 0) ax.nrmL[crank] = acc;
  }
  cluster.sync();
  for (int p = 0; p < N; p += kPanel) {
    const int jb = min(kPanel, N - p);
    for (int j = 0; j < jb; ++j) {
      const int i = p + j;
      // ---- left reflector of column i (every CTA, identical inputs) ----
      double beta;
      double2 tau, sc;
      {
        double xn2 = 0.0;
        for (int q = 0; q < C; ++q) xn2 += __ldcg(&ax.nrmL[q]);
        larfg_scalars(dfl(&AE(i, i)), xn2, beta, tau, sc);
      }
      if (crank == 0 && tid == 0) {
        dd[i] = beta;
        S.tau[i] = tau;
      }
      if (i == N - 1) {  // last column: left reflector only
        for (int r = i + 1 + gt; r < M; r += gthr) AE(r, i) = dfs(cmul(dfl(&AE(r, i)), sc));
        break;
      }
      // ---- S2: z = A0(i:M, i+1:N)^H v, s1 = V^H v, s2 = Xp^H v ----
      for (int r = i + tid; r < M; r += nthr)
        vec[r - i] = dfs(r == i ? make_double2(1.0, 0.0) : cmul(dfl(&AE(r, i)), sc));
      __syncthreads();
      {
        const int ncol = N - i - 1, items = ncol + 2 * j;
        for (int it = gw; it < items; it += nw) {
          double2 acc = make_double2(0.0, 0.0);  // sum_r conj(col(r)) v(r)
          if (it < ncol + j) {  // columns of A0 / of V: double-float on the FP32 pipe
            const float4 *col = &AE(0, it < ncol ? i + 1 + it : p + (it - ncol));
            float ar = 0.f, arl = 0.f, ai = 0.f, ail = 0.f;
            int r = i + lane;
            for (; r + 32 * (kDfLoads - 1) < M; r += 32 * kDfLoads) {
              float4 c[kDfLoads];
#pragma unroll
              for (int q = 0; q < kDfLoads; ++q) c[q] = __ldcg(col + r + 32 * q);
#pragma unroll
              for (int q = 0; q < kDfLoads; ++q) df_cmac_ca(ar, arl, ai, ail, c[q], vec[r + 32 * q - i]);
            }
            for (; r < M; r += 32) df_cmac_ca(ar, arl, ai, ail, __ldcg(col + r), vec[r - i]);
            acc = make_double2(df_warp_sum(ar, arl), df_warp_sum(ai, ail));
          } else {  // x_k columns (FP64)
            const double2 *col = &XB(0, it - ncol - j);
            for (int r = i + lane; r < M; r += 32) mac_ca(acc, ldc(col + r), dfd(vec[r - i]));
            acc.x = bsum(acc.x);
            acc.y = bsum(acc.y);
          }
          if (lane == 0) {
            if (it < ncol)
              ax.zb[i + 1 + it] = acc;
            else if (it < ncol + j)
              ax.s1[it - ncol] = acc;
            else
              ax.s2[it - ncol - j] = acc;
          }
        }
      }
      cluster.sync();
      // ---- S3: y_i = tauq (z - Y s1 - U s2); row i of the current matrix ----
      if (tid < j) {
        sm[tid] = ldc(&ax.s1[tid]);
        sm[kPanel + tid] = ldc(&ax.s2[tid]);
        sm[2 * kPanel + tid] = dfl(&AE(i, p + tid));  // v_k(i)
        sm[3 * kPanel + tid] = ldc(&XB(i, tid));      // x_k(i)
      }
      __syncthreads();
      {
        double acc = 0.0;
        for (int c = i + 1 + gt; c < N; c += gthr) {
          double2 y = ldc(&ax.zb[c]);
          double2 rr = dfl(&AE(i, c));
          for (int k = 0; k < j; ++k) {
            const double2 yk = ldc(&YB(c, k)), uk = ldc(&PV(c, p + k));
            msub(y, yk, sm[k]);
            msub(y, uk, sm[kPanel + k]);
            msub_cb(rr, sm[2 * kPanel + k], yk);
            msub_cb(rr, sm[3 * kPanel + k], uk);
          }
          y = cmul(tau, y);
          YB(c, j) = y;
          rr.x -= y.x;  // v_i(i) = 1: rr -= conj(y)
          rr.y += y.y;
          AE(i, c) = dfs(rr);
          if (c >= i + 2) acc = fma(rr.x, rr.x, fma(rr.y, rr.y, acc));
        }
        acc = block_sum(acc, red);
        if (tid == 0) ax.nrmR[crank] = acc;
      }
      for (int r = i + 1 + gt; r < M; r += gthr) AE(r, i) = dfs(cmul(dfl(&AE(r, i)), sc));  // v_i
      cluster.sync();
      // ---- right reflector of row i (every CTA) ----
      double beta2;
      double2 tau2, sc2;
      {
        double xn2 = 0.0;
        for (int q = 0; q < C; ++q) xn2 += __ldcg(&ax.nrmR[q]);
        larfg_scalars(cconj(dfl(&AE(i, i + 1))), xn2, beta2, tau2, sc2);
      }
      if (crank == 0 && tid == 0) {
        ee[i] = beta2;
        S.taup[i] = tau2;
      }
      // ---- S4: w = A0(i+1:M, i+1:N) u by column chunks, t1 = Y^H u, t2 = U^H u ----
      for (int c = i + 1 + tid; c < N; c += nthr)
        vec[c - i - 1] = dfs(c == i + 1 ? make_double2(1.0, 0.0) : cmul(cconj(dfl(&AE(i, c))), sc2));
      __syncthreads();
      {
        const int rows = M - i - 1, cols = N - i - 1;
        const int nrb = (rows + 31) / 32, ncc = (cols + kChunk - 1) / kChunk;
        const int tasks = nrb * ncc, items = tasks + 2 * j + 1;
        for (int it = gw; it < items; it += nw) {
          if (it < tasks) {
            const int rb = it % nrb, cc = it / nrb;
            const int r = i + 1 + rb * 32 + lane;
            const int c0 = i + 1 + cc * kChunk, c1 = min(N, c0 + kChunk);
            if (r < M) {
              float ar = 0.f, arl = 0.f, ai = 0.f, ail = 0.f;
              const float4 *rp = &AE(r, 0);
              int c = c0;
              for (; c + kDfLoads - 1 < c1; c += kDfLoads) {
                float4 a[kDfLoads];
#pragma unroll
                for (int q = 0; q < kDfLoads; ++q) a[q] = __ldcg(rp + (size_t)M * (c + q));
#pragma unroll
                for (int q = 0; q < kDfLoads; ++q) df_cmac(ar, arl, ai, ail, a[q], vec[c + q - i - 1]);
              }
              for (; c < c1; ++c) df_cmac(ar, arl, ai, ail, __ldcg(rp + (size_t)M * c), vec[c - i - 1]);
              ax.part[(size_t)cc * M + r] = make_double2((double)ar + (double)arl, (double)ai + (double)ail);
            }
          } else {
            const int k = it - tasks;  // 0..j: t1 over y_k; j+1..2j: t2 over u_(k-j-1)
            const double2 *cp = k <= j ? &YB(0, k) : &PV(0, p + k - j - 1);
            double2 acc = make_double2(0.0, 0.0);
            for (int c = i + 1 + lane; c < N; c += 32) mac_ca(acc, ldc(cp + c), dfd(vec[c - i - 1]));
            acc.x = bsum(acc.x);
            acc.y = bsum(acc.y);
            if (lane == 0) {
              if (k <= j)
                ax.t1[k] = acc;
              else
                ax.t2[k - j - 1] = acc;
            }
          }
        }
        for (int c = i + 1 + gt; c < N; c += gthr) PV(c, i) = dfd(vec[c - i - 1]);  // u_i
      }
      cluster.sync();
      // ---- x_i = taup (w - V t1 - Xp t2); then column i+1 of the current matrix ----
      const bool next_in_panel = j + 1 < jb;
      if (tid <= j) {
        sm[tid] = ldc(&ax.t1[tid]);
        if (tid < j) sm[kPanel + tid] = ldc(&ax.t2[tid]);
        if (next_in_panel) {
          sm[2 * kPanel + tid] = ldc(&YB(i + 1, tid));      // y_k(i+1)
          sm[3 * kPanel + tid] = ldc(&PV(i + 1, p + tid));  // u_k(i+1)
        }
      }
      __syncthreads();
      {
        const int ncc = (N - i - 1 + kChunk - 1) / kChunk;
        double acc = 0.0;
        for (int r = i + 1 + gt; r < M; r += gthr) {
          double2 w = make_double2(0.0, 0.0);
          for (int q = 0; q < ncc; ++q) {  // fixed order
            const double2 t = ldc(&ax.part[(size_t)q * M + r]);
            w.x += t.x;
            w.y += t.y;
          }
          for (int k = 0; k <= j; ++k) msub(w, dfl(&AE(r, p + k)), sm[k]);
          for (int k = 0; k < j; ++k) msub(w, ldc(&XB(r, k)), sm[kPanel + k]);
          const double2 x = cmul(tau2, w);
          XB(r, j) = x;
          if (next_in_panel) {
            double2 a = dfl(&AE(r, i + 1));
            for (int k = 0; k <= j; ++k) {
              msub_cb(a, dfl(&AE(r, p + k)), sm[2 * kPanel + k]);
              msub_cb(a, k < j ? ldc(&XB(r, k)) : x, sm[3 * kPanel + k]);
            }
            AE(r, i + 1) = dfs(a);
            if (r >= i + 2) acc = fma(a.x, a.x, fma(a.y, a.y, acc));
          }
        }
        if (next_in_panel) {
          acc = block_sum(acc, red);
          if (tid == 0) ax.nrmL[crank] = acc;
        }
      }
      cluster.sync();
    }
    const int q = p + jb;
    if (q >= N) break;
    // ---- panel end: A0(q:M, q:N) -= V Y^H + Xp U^H (inner dimension 2 jb) ----
    // 64 x 64 tiles over the cluster's CTAs, double-float on the FP32 pipe: each
    // thread starts from its 8 elements of A0 and subtracts the 2 jb products
    {
      const int K2 = 2 * jb;
      const int ntr = (M - q + kTile - 1) / kTile, ntc = (N - q + kTile - 1) / kTile;
      float4 *Ls = reinterpret_cast<float4 *>(stg), *Rs = Ls + kKc * kTile;
      const int tx = tid & 15, ty = tid >> 4;  // rows ty, ty + 32; columns tx + 16 b
      for (int t = crank; t < ntr * ntc; t += C) {
        const int r0 = q + (t % ntr) * kTile, c0 = q + (t / ntr) * kTile;
        float4 acc[2][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = r0 + ty + 32 * a, c = c0 + tx + 16 * b;
            acc[a][b] = (r < M && c < N) ? __ldcg(&AE(r, c)) : make_float4(0.f, 0.f, 0.f, 0.f);
          }
        for (int kc = 0; kc < K2; kc += kKc) {
          __syncthreads();
          for (int e = tid; e < kKc * kTile; e += nthr) {
            const int rr = e % kTile, kk = e / kTile, k = kc + kk;
            const int r = r0 + rr, c = c0 + rr;
            float4 l = make_float4(0.f, 0.f, 0.f, 0.f), g = l;
            if (k < K2) {
              if (r < M) l = k < jb ? __ldcg(&AE(r, p + k)) : dfs(ldc(&XB(r, k - jb)));
              if (c < N) g = dfs(k < jb ? ldc(&YB(c, k)) : ldc(&PV(c, p + k - jb)));
            }
            Ls[kk * kTile + rr] = l;
            Rs[kk * kTile + rr] = g;
          }
          __syncthreads();
          for (int kk = 0; kk < kKc; ++kk) {
            const float4 l0 = Ls[kk * kTile + ty], l1 = Ls[kk * kTile + ty + 32];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              const float4 g = Rs[kk * kTile + tx + 16 * b];
              df_cmsub_cb(acc[0][b], l0, g);  // acc -= l conj(g)
              df_cmsub_cb(acc[1][b], l1, g);
            }
          }
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = r0 + ty + 32 * a, c = c0 + tx + 16 * b;
            if (r < M && c < N) AE(r, c) = df_norm4(acc[a][b]);
          }
      }
    }
    cluster.sync();
    {  // norm partials of column q below the diagonal
      double acc = 0.0;
      for (int r = q + 1 + gt; r < M; r += gthr) {
        const double2 a = dfl(&AE(r, q));
        acc = fma(a.x, a.x, fma(a.y, a.y, acc));
      }
      acc = block_sum(acc, red);
      if (tid == 0) ax.nrmL[crank] = acc;
    }
    cluster.sync();
  }
#undef AE
#undef YB
#undef XB
#undef PV
}

// ---------------------------------------------------------------------------
// 2. bisection: sigma_i of B for i < kk (one team of kTeam lanes each), Golub-Kahan Sturm counts
// ---------------------------------------------------------------------------
// Sturm count of the Golub-Kahan matrix: eigenvalues below x; sq = squared
// off-diagonals (2n-1 of them).  Two independent recurrences interleave.
__device__ __forceinline__ void gk_count2(const double *sq, int n1, double x0, double x1, double pivmin,
                                          int &c0, int &c1) {
  double q0 = -x0, q1 = -x1;
  c0 = q0 < 0.0;
  c1 = q1 < 0.0;
  for (int j = 0; j < n1; ++j) {
    const double o2 = sq[j];
    if (fabs(q0) < pivmin) q0 = -pivmin;
    if (fabs(q1) < pivmin) q1 = -pivmin;
    q0 = -x0 - o2 / q0;
    q1 = -x1 - o2 / q1;
    c0 += q0 < 0.0;
    c1 += q1 < 0.0;
  }
}

__device__ __forceinline__ int gk_count(const double *sq, int n1, double x, double pivmin) {
  double q = -x;
  int c = q < 0.0;
  for (int j = 0; j < n1; ++j) {
    if (fabs(q) < pivmin) q = -pivmin;
    q = -x - sq[j] / q;
    c += q < 0.0;
  }
  return c;
}

// the same count in FP32 on off-diagonals scaled by 1/hi (values in [0, 1])
__device__ __forceinline__ int gk_count_f32(const float *sqf, int n1, float x) {
  float q = -x;
  int c = q < 0.0f;
  for (int j = 0; j < n1; ++j) {
    if (fabsf(q) < 1e-30f) q = -1e-30f;
    q = -x - __fdividef(sqf[j], q);
    c += q < 0.0f;
  }
  return c;
}

// The count in double-float on off-diagonals scaled by 1/hi (FP32 pipe): each step
// q = -x - o^2/q with Dekker's double-length division (quotient of the leading
// parts, remainder from an exact product, one correction).  Sign decisions are
// good to ~2^-44 ||T||; the FP64 stage checks the bracket it produces.
__device__ __forceinline__ int gk_count_df(const float2 *sqd, int n1, float xh, float xl) {
  float qh = -xh, ql = -xl;
  int c = qh < 0.0f;
  for (int j = 0; j < n1; ++j) {
    if (fabsf(qh) < 1e-30f) {
      qh = -1e-30f;
      ql = 0.0f;
    }
    const float2 a = sqd[j];
    const float q1 = __fdiv_rn(a.x, qh);
    const float ph = __fmul_rn(q1, qh);
    const float pe = fmaf(q1, qh, -ph);
    // remainder a - q1 q (exact leading difference, then the small terms)
    const float rh = __fadd_rn(a.x, -ph);
    const float rr = __fadd_rn(__fadd_rn(rh, -pe), __fadd_rn(a.y, -__fmul_rn(q1, ql)));
    const float q2 = __fdiv_rn(rr, qh);
    // t = q1 + q2 (fast two-sum), then q = -x - t
    const float th = __fadd_rn(q1, q2);
    const float tl = __fadd_rn(q2, -__fadd_rn(th, -q1));
    const float sh = __fadd_rn(-xh, -th);
    const float bp = __fadd_rn(sh, xh);
    const float err = __fadd_rn(__fadd_rn(-xh, -__fadd_rn(sh, -bp)), __fadd_rn(-th, -bp));
    const float sl = __fadd_rn(err, __fadd_rn(-xl, -tl));
    qh = __fadd_rn(sh, sl);
    ql = __fadd_rn(sl, -__fadd_rn(qh, -sh));
    c += qh < 0.0f;
  }
  return c;
}

// sigma_i of B for i < min(kk, n), descending.  One thread per value, one warp
// per block so that the FP64 work spreads over the SMs:
//   1. FP32 bisection on the scaled problem to width 2^-22 ||T||; FP32 Sturm counts
//      are exact for a T perturbed by a few float ulps, so the bracket widened by
//      2^-18 ||T|| holds sigma_i; two FP64 counts check it (reset to [0, ||T||]
//      otherwise).
//   2. Double-float bisection (FP32 pipe) to width 2^-42 ||T||; the bracket widened
//      by 2^-40 ||T|| is checked with two FP64 counts (reset to [0, ||T||]
//      otherwise).
//   3. FP64 bisection to width 2 eps sigma + eps ||T||: the absolute accuracy
//      LAPACK's bidiagonal SVD reaches on Theta as a whole.
//   Each value is found by a team of kTeam lanes that evaluate kTeam points of
//   the bracket at once (multisection): the counts are monotone in x, so the
//   leading run of "count <= target" in the team's ballot picks one of kTeam + 1
//   subintervals (8 lanes: about 3.2 bits per step instead of bisection's 1).
//   With few values in the batch (a dense sweep: 32 bonds x chi) the kernel is
//   bound by the latency of the sequential Sturm recurrences and the extra lanes
//   are free; with many (number-conserving blocks: every value of every block)
//   the counts fill the GPU on their own and teams of 1 lane (bisection) do the
//   least work.  The host picks kTeam per launch.
constexpr int kSigmaThreads = 32;
template <int kTeam>
__global__ void __launch_bounds__(kSigmaThreads) k_bd_sigma(Slot *slots, const int *path, int kk) {
  constexpr int kSigmaValues = kSigmaThreads / kTeam;  // values per block
  // step caps (safety only; the width tests end the loops): log2(kTeam + 1) bits
  // per step for the 22 bits of the FP32 stage and the ~26 of the double-float one
  constexpr int kIt32 = kTeam == 1 ? 26 : kTeam == 2 ? 17 : kTeam == 4 ? 12 : 10;
  constexpr int kItDf = kTeam == 1 ? 34 : kTeam == 2 ? 22 : kTeam == 4 ? 16 : 12;
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int K = min(kk, n);
  if ((int)(blockIdx.x * kSigmaValues) >= K) return;  // uniform per block
  const int n1 = 2 * n - 1;
  extern __shared__ double sq[];  // n1 squared off-diagonals, n1 scaled double-float, n1 scaled FP32
  float2 *sqd = reinterpret_cast<float2 *>(sq + n1);
  float *sqf = reinterpret_cast<float *>(sqd + n1);
  const double *dd = S.bdws, *ee = S.bdws + n;
  double hl = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    hl = fmax(hl, fabs(dd[j]) + (j < n - 1 ? fabs(ee[j]) : 0.0) + (j > 0 ? fabs(ee[j - 1]) : 0.0));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) hl = fmax(hl, __shfl_xor_sync(0xffffffffu, hl, o));
  const double hi = hl * (1.0 + 1e-12) + 1e-300;  // Gershgorin bound of the Golub-Kahan matrix
  const double inv_hi = 1.0 / hi;
  for (int j = threadIdx.x; j < n1; j += blockDim.x) {
    const double o = (j & 1) ? ee[j >> 1] : dd[j >> 1];
    sq[j] = o * o;
    const double os = (o * inv_hi) * (o * inv_hi);
    const float oh = (float)os;
    sqd[j] = make_float2(oh, (float)(os - (double)oh));
    sqf[j] = oh;
  }
  __syncthreads();
  const int team = threadIdx.x / kTeam, t = threadIdx.x % kTeam;
  const unsigned tmask = (kTeam == 32 ? 0xffffffffu : ((1u << kTeam) - 1u)) << (kTeam * team);
  const int i = blockIdx.x * kSigmaValues + team;
  if (i >= K) return;  // the whole team leaves together
  const int target = 2 * n - 1 - i;  // count(< x) <= target  <=>  x <= sigma_i
  const double pivmin = 1e-290 * fmax(1.0, hi * hi);
  // leading run of true votes of the team (bit t: point t has count <= target)
  auto lead = [&](bool ok) -> int {
    const unsigned b = (__ballot_sync(tmask, ok) >> (kTeam * team)) & ((1u << kTeam) - 1u);
    return __ffs(~b) - 1;
  };
  // 1. FP32 bracket of width 2^-22 on the scaled problem
  float lf = 0.0f, hf = 1.0f;
  for (int it = 0; it < kIt32 && hf - lf > 2.384185791015625e-07f; ++it) {
    const float w = (hf - lf) * (1.0f / (kTeam + 1));
    const int k = lead(gk_count_f32(sqf, n1, lf + w * (float)(t + 1)) <= target);
    const float nl = k > 0 ? lf + w * (float)k : lf;
    hf = k < kTeam ? lf + w * (float)(k + 1) : hf;
    lf = nl;
  }
  // 2. double-float stage to 2^-42 from the FP32 bracket widened by 2^-18
  double ls = fmax(0.0, (double)lf - 3.814697265625e-06), hs = fmin(1.0, (double)hf + 3.814697265625e-06);
  for (int it = 0; it < kItDf && hs - ls > 2.2737367544323206e-13; ++it) {
    const double w = (hs - ls) * (1.0 / (kTeam + 1));
    const double x = ls + w * (double)(t + 1);
    const float xh = (float)x;
    const int k = lead(gk_count_df(sqd, n1, xh, (float)(x - (double)xh)) <= target);
    const double nl = k > 0 ? ls + w * (double)k : ls;
    hs = k < kTeam ? ls + w * (double)(k + 1) : hs;
    ls = nl;
  }
  double lo = fmax(0.0, ls - 9.094947017729282e-13) * hi;  // widened by 2^-40
  double h = fmin(1.0, hs + 9.094947017729282e-13) * hi;
  {
    int c0, c1;
    gk_count2(sq, n1, lo, h, pivmin, c0, c1);
    if (!(c0 <= target && c1 > target)) {
      lo = 0.0;
      h = hi;
    }
  }
  // 3. FP64 multisection to 2 eps sigma + eps ||T||
  for (int it = 0; it < 60; ++it) {
    if (h - lo <= 4.440892098500626e-16 * h + 2.220446049250313e-16 * hi || h < 1e-30 * hi) break;
    const double w = (h - lo) * (1.0 / (kTeam + 1));
    const int k = lead(gk_count(sq, n1, lo + w * (double)(t + 1), pivmin) <= target);
    const double nl = k > 0 ? lo + w * (double)k : lo;
    h = k < kTeam ? lo + w * (double)(k + 1) : h;
    lo = nl;
  }
  const double sg = 0.5 * (lo + h);
  if (t == 0) S.bdws[2 * n + i] = sg < 1e-30 * hi ? 0.0 : sg;
}

// ---------------------------------------------------------------------------
// 3a. inverse iteration on (T_GK - sigma_i I), one thread per value.
// Scratch per value (transposed so that threads of a warp touch adjacent words):
//   U0 (reciprocal pivots), U1, U2 (upper factor of the pivoted LU), PV (multipliers),
//   Y (swap flags), then the vector Z itself.
// ---------------------------------------------------------------------------
__global__ void k_bd_invit(Slot *slots, const int *path, int kk, int cap) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n;
  const int K = cap ? min(min(kk, n), S.cp->k) : min(kk, n);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  const double *dd = S.bdws, *ee = S.bdws + n, *sig = S.bdws + 2 * n;
  double *base = S.bdws + bd_scratch(n, kk);
  double *U0 = base, *U1 = base + (size_t)N * K, *U2 = base + 2 * (size_t)N * K,
         *PV = base + 3 * (size_t)N * K, *Y = base + 4 * (size_t)N * K, *Z = base + 5 * (size_t)N * K;
#define AT(A, j) A[(size_t)(j) * K + i]
  const double lam = sig[i];
  if (lam <= 0.0) {  // an exactly zero value: FormLambda1 drops it, its vectors are zero
    for (int j = 0; j < N; ++j) AT(Z, j) = 0.0;
    return;
  }
  auto off = [&](int j) -> double { return (j & 1) ? ee[j >> 1] : dd[j >> 1]; };  // T(j, j+1)
  // pivots below eps ||T|| are raised to it (sign kept), as LAPACK's DLAGTS does,
  // so the solve stays finite when sigma_i is an eigenvalue to working precision
  double tnorm = 0.0;
  for (int j = 0; j < N - 1; ++j) tnorm = fmax(tnorm, fabs(off(j)));
  const double ptol = fmax(2.220446049250313e-16 * tnorm, 1e-300);
  auto guard = [&](double p) -> double { return fabs(p) >= ptol ? p : (p < 0.0 ? -ptol : ptol); };
  // LU with partial pivoting of T - lam I (diagonal -lam, off-diagonals off(j))
  double d0 = -lam, d1 = N > 1 ? off(0) : 0.0;
  for (int j = 0; j < N - 1; ++j) {
    const double sub = off(j);
    const double nd0 = -lam, nd1 = j + 1 < N - 1 ? off(j + 1) : 0.0;
    if (fabs(d0) >= fabs(sub)) {  // keep row j as the pivot row
      const double piv = guard(d0), rp = 1.0 / piv, mult = sub * rp;
      AT(U0, j) = rp;
      AT(U1, j) = d1;
      AT(U2, j) = 0.0;
      AT(PV, j) = mult;
      AT(Y, j) = 0.0;  // no swap
      d0 = nd0 - mult * d1;
      d1 = nd1;
    } else {  // row j+1 becomes the pivot row
      const double mult = d0 / sub;
      AT(U0, j) = 1.0 / sub;
      AT(U1, j) = nd0;
      AT(U2, j) = nd1;
      AT(PV, j) = mult;
      AT(Y, j) = 1.0;  // swapped
      d0 = d1 - mult * nd0;
      d1 = -mult * nd1;
    }
  }
  AT(U0, N - 1) = 1.0 / guard(d0);  // U0 holds the reciprocal pivots
  // start vector: fixed pseudo-random (splitmix-style hash of (i, j)), max-norm 1/2
  for (int j = 0; j < N; ++j) {
    unsigned long long x = (unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ull +
                           (unsigned long long)j * 0xBF58476D1CE4E5B9ull;
    x ^= x >> 31;
    x *= 0x94D049BB133111EBull;
    x ^= x >> 29;
    AT(Z, j) = (double)(x >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
  double scale = 1.0;  // the right-hand side is Z * scale
  for (int it = 0; it < 3; ++it) {
    // forward: the row operations (with swaps) applied to the right-hand side
    double carry = AT(Z, 0) * scale;
    for (int j = 0; j < N - 1; ++j) {
      const double next = AT(Z, j + 1) * scale;
      if (AT(Y, j) == 0.0) {
        AT(Z, j) = carry;
        carry = next - AT(PV, j) * carry;
      } else {
        AT(Z, j) = next;
        carry = carry - AT(PV, j) * next;
      }
    }
    AT(Z, N - 1) = carry;
    // back substitution with the upper factor (diagonal U0, super-diagonals U1, U2);
    // a partial result that grows past 2^500 is rescaled, with the values already
    // produced, so that nothing overflows
    double x1 = 0.0, x2 = 0.0, amax = 0.0;
    for (int j = N - 1; j >= 0; --j) {
      double sacc = AT(Z, j);
      if (j + 1 < N) sacc -= AT(U1, j) * x1;
      if (j + 2 < N) sacc -= AT(U2, j) * x2;
      double x = sacc * AT(U0, j);
      if (fabs(x) > 3.273390607896142e150) {
        const double r = 3.054936363499605e-151;  // 2^-500
        for (int q = j + 1; q < N; ++q) AT(Z, q) *= r;
        x *= r;
        x1 *= r;
        x2 *= r;
        amax *= r;
        // the remaining right-hand side entries scale with the solution
        for (int q = 0; q < j; ++q) AT(Z, q) *= r;
      }
      AT(Z, j) = x;
      amax = fmax(amax, fabs(x));
      x2 = x1;
      x1 = x;
    }
    scale = amax > 0.0 ? 1.0 / amax : 0.0;
  }
  double nrm = 0.0;
  for (int j = 0; j < N; ++j) {
    const double v = AT(Z, j) * scale;
    nrm = fma(v, v, nrm);
  }
  const double inv = nrm > 0.0 ? scale / sqrt(nrm) : 0.0;
  for (int j = 0; j < N; ++j) AT(Z, j) *= inv;
#undef AT
}

// 3b. split z into v (even rows) and u (odd rows) and re-orthogonalise each set in
// order of descending sigma by classical Gram-Schmidt, with a second pass only
// when the first removed more than 1 - 1/sqrt(2) of the vector's norm (the
// "twice is enough" test of Daniel, Gragg, Kaufman and Stewart).  A cluster of
// kOrthCluster CTAs per (bond, set) splits the rows; partial dot products and
// norms meet in the (free by now) inverse-iteration scratch, double-buffered.
// Z is row-major (element (j, i) at j*K + i): the dot products run one thread per
// earlier vector over a quarter of the CTA's rows (coalesced across threads), the
// subtraction one warp per row.
constexpr int kOrthThreads = 512;
constexpr int kOrthCluster = 2;
__global__ void __launch_bounds__(kOrthThreads) k_bd_orth(Slot *slots, const int *path, int kk, int cap) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks(), crank = (int)cluster.block_rank();
  const int s = blockIdx.y, part = blockIdx.x / C;  // part 0: v = z[2j], 1: u = z[2j+1]
  const int route = path[s];
  if (!on_route(route)) return;  // uniform per cluster
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = cap ? min(min(kk, n), S.cp->k) : min(kk, n);
  double *Z = S.bdws + bd_scratch(n, kk) + 5 * (size_t)N * K;
  double *xch = S.bdws + bd_scratch(n, kk) + (size_t)part * N * K;  // 2 x C x (K + 1)
  const int j0 = (int)((long long)n * crank / C), j1 = (int)((long long)n * (crank + 1) / C);
  extern __shared__ double dots[];  // K dot products, then 4 x K partial sums
  double *psum = dots + K;
  __shared__ double red[kOrthThreads / 32];
  __shared__ double nrm_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarp = kOrthThreads / 32;
  const int qt = tid & 127, jc = tid >> 7;  // 128 vector slots x 4 row quarters
  int post = 0;                             // postings so far (buffer = post & 1)
#define ZE(j, i) Z[(size_t)(2 * (j) + part) * K + (i)]
#define XC(buf, r, q) xch[((size_t)(buf) * C + (r)) * (K + 1) + (q)]
  // CTA sum of the squared norm of z_i over this CTA's rows
  auto norm_part = [&](int i) -> double {
    double a = 0.0;
    for (int j = j0 + tid; j < j1; j += kOrthThreads) a = fma(ZE(j, i), ZE(j, i), a);
    a = bsum(a);
    __syncthreads();
    if (lane == 0) red[warp] = a;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nwarp; ++w) t += red[w];
    return t;
  };
  // post this CTA's dot products of z_i with z_q (q < i) and, optionally, a norm
  auto post_dots = [&](int i, bool with_norm) {
    const int buf = post & 1;
    for (int q = qt; q < i; q += 128) {
      double a0 = 0.0, a1 = 0.0;
      int j = j0 + jc;
      for (; j + 4 < j1; j += 8) {
        a0 = fma(ZE(j, q), ZE(j, i), a0);
        a1 = fma(ZE(j + 4, q), ZE(j + 4, i), a1);
      }
      for (; j < j1; j += 4) a0 = fma(ZE(j, q), ZE(j, i), a0);
      psum[jc * K + q] = a0 + a1;
    }
    const double nr = with_norm ? norm_part(i) : 0.0;  // (its barriers also order psum)
    __syncthreads();
    for (int q = tid; q < i; q += kOrthThreads)
      XC(buf, crank, q) = (psum[q] + psum[K + q]) + (psum[2 * K + q] + psum[3 * K + q]);
    if (with_norm && tid == 0) XC(buf, crank, K) = nr;
  };
  // gather the posted dots (q < i) into shared memory and return the posted norm
  auto gather = [&](int i, bool dots_too) -> double {
    const int buf = post & 1;
    if (dots_too)
      for (int q = tid; q < i; q += kOrthThreads) {
        double t = 0.0;
        for (int r = 0; r < C; ++r) t += __ldcg(&XC(buf, r, q));
        dots[q] = t;
      }
    if (tid == 0) {
      double t = 0.0;
      for (int r = 0; r < C; ++r) t += __ldcg(&XC(buf, r, K));
      nrm_s = t;
    }
    __syncthreads();
    ++post;
    return nrm_s;
  };
  auto subtract = [&](int i) {
    for (int j = j0 + warp; j < j1; j += nwarp) {
      double a = 0.0;
      for (int q = lane; q < i; q += 32) a = fma(dots[q], ZE(j, q), a);
      a = bsum(a);
      if (lane == 0) ZE(j, i) -= a;
    }
    __syncthreads();
  };
  auto post_norm = [&](int i) {
    const double nr = norm_part(i);
    if (tid == 0) XC(post & 1, crank, K) = nr;
  };
  for (int i = 0; i < K; ++i) {
    post_dots(i, true);
    cluster.sync();
    const double nrm0 = gather(i, true);
    double nrm = nrm0;
    if (i > 0) {
      subtract(i);
      post_norm(i);
      cluster.sync();
      nrm = gather(i, false);
      if (nrm < 0.5 * nrm0) {  // second pass
        post_dots(i, false);
        cluster.sync();
        gather(i, true);
        subtract(i);
        post_norm(i);
        cluster.sync();
        nrm = gather(i, false);
      }
    }
    const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    for (int j = j0 + tid; j < j1; j += kOrthThreads) ZE(j, i) *= inv;
    __syncthreads();
  }
#undef ZE
#undef XC
}

// Precision form of step 3's re-orthogonalisation: the same schedule on Z held
// as double-float (float2 per real, converted in place by k_bd_z_df before and
// back after), so the dot products and the subtractions run on the FP32 pipe;
// the cross-lane and cross-CTA sums and the norms stay FP64.
__global__ void k_bd_z_df(Slot *slots, const int *path, int kk, int cap, int to_df) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = cap ? min(min(kk, n), S.cp->k) : min(kk, n);
  double *Z = S.bdws + bd_scratch(n, kk) + 5 * (size_t)N * K;
  float2 *Zf = reinterpret_cast<float2 *>(Z);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)N * K;
       e += (size_t)gridDim.x * blockDim.x) {
    if (to_df) {
      const double x = Z[e];
      const float h = (float)x;
      Zf[e] = make_float2(h, (float)(x - (double)h));
    } else {
      const float2 v = Zf[e];
      Z[e] = (double)v.x + (double)v.y;
    }
  }
}

__device__ __forceinline__ void df_fma2(float &h, float &l, float2 a, float2 b) { df_mac(h, l, a.x, a.y, b.x, b.y); }

__global__ void __launch_bounds__(kOrthThreads) k_bd_orth_df(Slot *slots, const int *path, int kk, int cap) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks(), crank = (int)cluster.block_rank();
  const int s = blockIdx.y, part = blockIdx.x / C;  // part 0: v = z[2j], 1: u = z[2j+1]
  const int route = path[s];
  if (!on_route(route)) return;  // uniform per cluster
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = cap ? min(min(kk, n), S.cp->k) : min(kk, n);
  float2 *Z = reinterpret_cast<float2 *>(S.bdws + bd_scratch(n, kk) + 5 * (size_t)N * K);
  double *xch = S.bdws + bd_scratch(n, kk) + (size_t)part * N * K;  // 2 x C x (K + 1)
  const int j0 = (int)((long long)n * crank / C), j1 = (int)((long long)n * (crank + 1) / C);
  extern __shared__ double dots[];  // K dot products, then 4 x K partial sums
  double *psum = dots + K;
  float2 *dotf = reinterpret_cast<float2 *>(psum);  // the dots as double-float for the subtraction
  __shared__ double red[kOrthThreads / 32];
  __shared__ double nrm_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarp = kOrthThreads / 32;
  const int qt = tid & 127, jc = tid >> 7;
  int post = 0;
#define ZE(j, i) Z[(size_t)(2 * (j) + part) * K + (i)]
#define XC(buf, r, q) xch[((size_t)(buf) * C + (r)) * (K + 1) + (q)]
  auto norm_part = [&](int i) -> double {
    float h = 0.f, l = 0.f;
    for (int j = j0 + tid; j < j1; j += kOrthThreads) df_fma2(h, l, ZE(j, i), ZE(j, i));
    const double a = bsum((double)h + (double)l);
    __syncthreads();
    if (lane == 0) red[warp] = a;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nwarp; ++w) t += red[w];
    return t;
  };
  auto post_dots = [&](int i, bool with_norm) {
    const int buf = post & 1;
    for (int q = qt; q < i; q += 128) {
      float h = 0.f, l = 0.f;
      for (int j = j0 + jc; j < j1; j += 4) df_fma2(h, l, ZE(j, q), ZE(j, i));
      psum[jc * K + q] = (double)h + (double)l;
    }
    const double nr = with_norm ? norm_part(i) : 0.0;  // (its barriers also order psum)
    __syncthreads();
    for (int q = tid; q < i; q += kOrthThreads)
      XC(buf, crank, q) = (psum[q] + psum[K + q]) + (psum[2 * K + q] + psum[3 * K + q]);
    if (with_norm && tid == 0) XC(buf, crank, K) = nr;
  };
  auto gather = [&](int i, bool dots_too) -> double {
    const int buf = post & 1;
    if (dots_too)
      for (int q = tid; q < i; q += kOrthThreads) {
        double t = 0.0;
        for (int r = 0; r < C; ++r) t += __ldcg(&XC(buf, r, q));
        dots[q] = t;
      }
    if (tid == 0) {
      double t = 0.0;
      for (int r = 0; r < C; ++r) t += __ldcg(&XC(buf, r, K));
      nrm_s = t;
    }
    __syncthreads();
    ++post;
    return nrm_s;
  };
  auto subtract = [&](int i) {
    for (int q = tid; q < i; q += kOrthThreads) {  // the dots as double-float (psum is free here)
      const double x = dots[q];
      const float hq = (float)x;
      dotf[q] = make_float2(hq, (float)(x - (double)hq));
    }
    __syncthreads();
    // one thread per row: row j of Z is contiguous in q, the dots are broadcast
    // from shared memory, and no cross-lane reduction is needed
    for (int j = j0 + tid; j < j1; j += kOrthThreads) {
      float h = 0.f, l = 0.f;
      for (int q = 0; q < i; ++q) df_fma2(h, l, dotf[q], ZE(j, q));
      const float2 z = ZE(j, i);
      const double r = ((double)z.x + (double)z.y) - ((double)h + (double)l);
      const float rh = (float)r;
      ZE(j, i) = make_float2(rh, (float)(r - (double)rh));
    }
    __syncthreads();
  };
  auto post_norm = [&](int i) {
    const double nr = norm_part(i);
    if (tid == 0) XC(post & 1, crank, K) = nr;
  };
  for (int i = 0; i < K; ++i) {
    post_dots(i, true);
    cluster.sync();
    const double nrm0 = gather(i, true);
    double nrm = nrm0;
    if (i > 0) {
      subtract(i);
      post_norm(i);
      cluster.sync();
      nrm = gather(i, false);
      if (nrm < 0.5 * nrm0) {  // second pass
        post_dots(i, false);
        cluster.sync();
        gather(i, true);
        subtract(i);
        post_norm(i);
        cluster.sync();
        nrm = gather(i, false);
      }
    }
    const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    for (int j = j0 + tid; j < j1; j += kOrthThreads) {
      const float2 z = ZE(j, i);
      const double r = ((double)z.x + (double)z.y) * inv;
      const float rh = (float)r;
      ZE(j, i) = make_float2(rh, (float)(r - (double)rh));
    }
    __syncthreads();
  }
#undef ZE
#undef XC
}

// ---------------------------------------------------------------------------
// 4. left vectors Q [Ub; 0] (M x K) and right vectors P Vb (N x K) of the
//    bidiagonalised matrix, one warp per kept column.
//    Theta route:   left -> Yu (scratch), right -> S.V (ld n).
//    Theta^H route: left -> Yu (= V of Theta), right -> Ru (= U of Theta, scratch
//    in the inverse-iteration LU area, free by now).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bd_apply(Slot *slots, const int *path, int kk, int cap) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = cap ? min(min(kk, n), S.cp->k) : min(kk, n);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = blockIdx.x * 8 + warp;
  if (col >= 2 * K) return;
  double *base = S.bdws + bd_scratch(n, kk);
  const double *Z = base + 5 * (size_t)N * K;
  double2 *Yu = reinterpret_cast<double2 *>(base + 6 * (size_t)N * K);
  double2 *Ru = route == kPathBidiagT ? reinterpret_cast<double2 *>(base) : S.V;
  const double2 *Pv = S.aux;
  if (col < K) {  // left: Y = H(0) ... H(n-1) [u; 0]
    const int i = col;
    double2 *Y = Yu + (size_t)m * i;
    for (int r = lane; r < m; r += 32)
      Y[r] = make_double2(r < n ? Z[(size_t)(2 * r + 1) * K + i] : 0.0, 0.0);
    __syncwarp();
    for (int j = n - 1; j >= 0; --j) {
      const double2 tq = S.tau[j];
      double wr = 0.0, wi = 0.0;
      for (int r = j + lane; r < m; r += 32) {
        const double2 y = Y[r];
        const double2 v = r == j ? make_double2(1.0, 0.0) : S.X[r + (size_t)m * j];
        wr = fma(v.x, y.x, fma(v.y, y.y, wr));
        wi = fma(v.x, y.y, fma(-v.y, y.x, wi));
      }
      wr = bsum(wr);
      wi = bsum(wi);
      const double fr = tq.x * wr - tq.y * wi, fi = tq.x * wi + tq.y * wr;
      for (int r = j + lane; r < m; r += 32) {
        const double2 v = r == j ? make_double2(1.0, 0.0) : S.X[r + (size_t)m * j];
        double2 y = Y[r];
        y.x -= v.x * fr - v.y * fi;
        y.y -= v.x * fi + v.y * fr;
        Y[r] = y;
      }
      __syncwarp();
    }
  } else {  // right: Y = G(0) ... G(n-2) v
    const int i = col - K;
    double2 *Y = Ru + (size_t)n * i;
    for (int r = lane; r < n; r += 32) Y[r] = make_double2(Z[(size_t)(2 * r) * K + i], 0.0);
    __syncwarp();
    for (int j = n - 2; j >= 0; --j) {
      const double2 tp = S.taup[j];
      double wr = 0.0, wi = 0.0;
      for (int r = j + 1 + lane; r < n; r += 32) {
        const double2 y = Y[r];
        const double2 u = Pv[r + (size_t)n * j];
        wr = fma(u.x, y.x, fma(u.y, y.y, wr));
        wi = fma(u.x, y.y, fma(-u.y, y.x, wi));
      }
      wr = bsum(wr);
      wi = bsum(wi);
      const double fr = tp.x * wr - tp.y * wi, fi = tp.x * wi + tp.y * wr;
      for (int r = j + 1 + lane; r < n; r += 32) {
        const double2 u = Pv[r + (size_t)n * j];
        double2 y = Y[r];
        y.x -= u.x * fr - u.y * fi;
        y.y -= u.x * fi + u.y * fr;
        Y[r] = y;
      }
      __syncwarp();
    }
  }
}

// X(:, i) = U(:, i) sigma_i (Theta's m rows, ld m) and, on the transposed route,
// V(:, i) = the left vectors of Theta^H (n rows, ld n).
__global__ void k_bd_store(Slot *slots, const int *path, int kk, int cap) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  const int m = S.cp->m, n = S.cp->n, K = cap ? min(min(kk, N), S.cp->k) : min(kk, N);
  double *base = S.bdws + bd_scratch(N, kk);
  const double *sig = S.bdws + 2 * N;
  const double2 *Yu = reinterpret_cast<const double2 *>(base + 12 * (size_t)N * K);
  const double2 *U = route == kPathBidiagT ? reinterpret_cast<const double2 *>(base) : Yu;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)m * K; e += stride) {
    const int i = (int)(e / m);
    const double2 y = U[e];
    S.X[e] = make_double2(y.x * sig[i], y.y * sig[i]);
  }
  if (route == kPathBidiagT)
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * K; e += stride)
      S.V[e] = Yu[e];
  if (cap) {  // columns past the capped count read as zero singular values
    for (size_t e = (size_t)m * K + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)m * n; e += stride)
      S.X[e] = make_double2(0.0, 0.0);
  } else if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.cp->k = K;
  }
}

// Precision form of step 4: the same reflector products in double-float, reading
// the left reflectors from the double-float matrix the bidiagonalisation left in
// S.X and the right ones from Pv converted in place (k_bd_pv_to_df); the vectors
// Yu / Ru are double-float too and k_bd_store_df converts them.
__global__ void __launch_bounds__(256) k_bd_apply_df(Slot *slots, const int *path, int kk, int cap,
                                                     int right_only) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = cap ? min(min(kk, n), S.cp->k) : min(kk, n);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = blockIdx.x * 8 + warp + (right_only ? K : 0);  // right only: columns K .. 2K-1
  if (col >= 2 * K) return;
  double *base = S.bdws + bd_scratch(n, kk);
  const double *Z = base + 5 * (size_t)N * K;
  float4 *Yu = reinterpret_cast<float4 *>(base + 6 * (size_t)N * K);
  float4 *Ru = route == kPathBidiagT ? reinterpret_cast<float4 *>(base) : reinterpret_cast<float4 *>(S.V);
  const float4 *Xf = reinterpret_cast<const float4 *>(S.X);
  const float4 *Pf = reinterpret_cast<const float4 *>(S.aux);
  const float4 one = make_float4(1.f, 0.f, 0.f, 0.f);
  const bool left = col < K;
  const int i = left ? col : col - K;
  const int len = left ? m : n;
  float4 *Y = left ? Yu + (size_t)m * i : Ru + (size_t)n * i;
  for (int r = lane; r < len; r += 32)
    Y[r] = dfs(make_double2(left ? (r < n ? Z[(size_t)(2 * r + 1) * K + i] : 0.0) : Z[(size_t)(2 * r) * K + i], 0.0));
  __syncwarp();
  for (int j = left ? n - 1 : n - 2; j >= 0; --j) {
    // reflector j: left v (rows j.., v(j) = 1) or right u (rows j+1.., u(j+1) = 1)
    const int r0 = left ? j : j + 1;
    const float4 *vc = left ? Xf + (size_t)m * j : Pf + (size_t)n * j;
    const double2 t = left ? S.tau[j] : S.taup[j];
    float wrh = 0.f, wrl = 0.f, wih = 0.f, wil = 0.f;  // w = sum conj(v) y
    for (int r = r0 + lane; r < len; r += 32)
      df_cmac_ca(wrh, wrl, wih, wil, (left && r == j) ? one : __ldcg(vc + r), Y[r]);
    const double wr = df_warp_sum(wrh, wrl), wi = df_warp_sum(wih, wil);
    const float4 f = dfs(make_double2(t.x * wr - t.y * wi, t.x * wi + t.y * wr));  // tau w
    const float4 nf = make_float4(-f.x, -f.y, -f.z, -f.w);
    for (int r = r0 + lane; r < len; r += 32) {  // y -= v f
      const float4 v = (left && r == j) ? one : __ldcg(vc + r);
      float4 y = Y[r];
      df_mac(y.x, y.y, v.x, v.y, nf.x, nf.y);
      df_mac(y.x, y.y, v.z, v.w, f.z, f.w);
      df_mac(y.z, y.w, v.x, v.y, nf.z, nf.w);
      df_mac(y.z, y.w, v.z, v.w, nf.x, nf.y);
      Y[r] = df_norm4(y);
    }
    __syncwarp();
  }
}

__global__ void k_bd_pv_to_df(Slot *slots, const int *path) {  // Pv in place, N x N
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  float4 *F = reinterpret_cast<float4 *>(S.aux);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)N * N; e += (size_t)gridDim.x * blockDim.x)
    F[e] = dfs(S.aux[e]);
}

__global__ void k_bd_store_df(Slot *slots, const int *path, int kk, int cap, int right_only) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  const int m = S.cp->m, n = S.cp->n, K = cap ? min(min(kk, N), S.cp->k) : min(kk, N);
  double *base = S.bdws + bd_scratch(N, kk);
  const double *sig = S.bdws + 2 * N;
  const float4 *Yu = reinterpret_cast<const float4 *>(base + 12 * (size_t)N * K);
  const float4 *U = route == kPathBidiagT ? reinterpret_cast<const float4 *>(base) : Yu;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; !right_only && e < (size_t)m * K; e += stride) {
    const int i = (int)(e / m);
    const double2 y = dfd(U[e]);
    S.X[e] = make_double2(y.x * sig[i], y.y * sig[i]);
  }
  const float4 *Vs = route == kPathBidiagT ? Yu : reinterpret_cast<const float4 *>(S.V);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * K; e += stride)
    S.V[e] = dfd(Vs[e]);  // in place on the tall route (same element, same size)
  if (cap) {  // columns past the capped count read as zero singular values
    for (size_t e = (size_t)m * K + blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)m * n; e += stride)
      S.X[e] = make_double2(0.0, 0.0);
  } else if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.cp->k = K;
  }
}

// Precision form: the M x N matrix of the route as double-float in place before
// the bidiagonalisation (float4 per complex element); its reflectors stay in that
// form for k_bd_apply_df.
__global__ void k_bd_to_df(Slot *slots, const int *path) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  float4 *F = reinterpret_cast<float4 *>(S.X);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)M * N; e += (size_t)gridDim.x * blockDim.x)
    F[e] = dfs(S.X[e]);
}

// Transposed route, before the bidiagonalisation: X (m x n, ld m) -> V (copy),
// then X <- V^H (n x m, ld n).
__global__ void k_bd_stage(Slot *slots, const int *path) {
  const int s = blockIdx.y;
  if (path[s] != kPathBidiagT) return;
  const Slot S = slots[s];
  const size_t e_end = (size_t)S.cp->m * S.cp->n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < e_end;
       e += (size_t)gridDim.x * blockDim.x)
    S.V[e] = S.X[e];
}

__global__ void k_bd_transpose(Slot *slots, const int *path) {
  __shared__ double2 tile[32][33];
  const int s = blockIdx.z;
  if (path[s] != kPathBidiagT) return;
  const Slot S = slots[s];
  const int m = S.cp->m, n = S.cp->n;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int tr = blockIdx.y * 32; tr < m; tr += gridDim.y * 32)
    for (int tc = blockIdx.x * 32; tc < n; tc += gridDim.x * 32) {
      for (int q = ty; q < 32; q += 8) {  // read V(tr + tx, tc + q)
        const int r = tr + tx, c = tc + q;
        if (r < m && c < n) tile[q][tx] = S.V[r + (size_t)m * c];
      }
      __syncthreads();
      for (int q = ty; q < 32; q += 8) {  // write X(tc + tx, tr + q) = conj(V(tr + q, tc + tx))
        const int c = tc + tx, r = tr + q;
        if (r < m && c < n) {
          const double2 v = tile[tx][q];
          S.X[c + (size_t)n * r] = make_double2(v.x, -v.y);
        }
      }
      __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host orchestration: bidiagonal route for the slots flagged kPathBidiag / kPathBidiagT
// ---------------------------------------------------------------------------
size_t bidiag_aux_elems(int n) { return bd_aux_elems(n, n); }

size_t bidiag_ws_doubles(int n, int chi) {
  const int K = std::min(chi, n);
  return bd_scratch(n, chi) + 6 * (size_t)(2 * n) * K + 2 * (size_t)n * K;
}

int run_bidiag_batch(tebd_handle *h, const BidiagBatch &b) {
  cudaStream_t st = h->stream;
  const int kk = b.kk, nb = b.nb, nmax = b.nmax, cap = b.cap;
  Slot *slots_d = b.slots_d;
  const int *path_d = b.path_d;
  int rc;
  if (b.phase != 2) {  // bidiagonalisation and singular values
  if (h->profiling) cudaEventRecord(h->ev[0], st);
  bool any_t = false;
  for (int s = 0; s < nb; ++s) any_t |= b.path_h[s] == kPathBidiagT;
  if (any_t) {
    k_bd_stage<<<dim3(128, nb), 256, 0, st>>>(slots_d, path_d);
    TEBD_LAUNCHED(h);
    const unsigned g = cdiv(nmax, 32) < 8 ? cdiv(nmax, 32) : 8;
    k_bd_transpose<<<dim3(g, g, nb), 256, 0, st>>>(slots_d, path_d);
    TEBD_LAUNCHED(h);
  }
  {
    cudaLaunchConfig_t cfg = {};
    const size_t smem = sizeof(double2) * ((size_t)nmax + 4 * kPanel) + sizeof(double) * kStageDoubles;
    const bool dfp = b.dfp;
    auto kern = dfp ? k_gebrd_df : k_gebrd;
    if ((rc = check_cuda(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "bidiagonalisation shared memory")))
      return rc;
    cfg.blockDim = dim3(kBW * 32, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // Cluster size: the kernel is bound by the SMs' FP64 pipes, so the batch's time
    // goes as waves / C; clusters must fit in one GPC, so the co-resident count
    // (occupancy query) decides how many waves a size needs.  Ties keep the
    // smaller size (fewer barriers' worth of idle SMs in a partial wave).
    // sizes up to 8, at least 4 (the autotuner measured 4 CTAs fastest for
    // 64..320-column batches of 32 bonds, where ceil(n / 128) had allowed 1..3)
    const int cmax = std::min(8, std::max(4, (nmax + 127) / 128));
    int nbd = 0;  // bonds on this route (the others' clusters exit at once)
    for (int s = 0; s < nb; ++s) nbd += b.path_h[s] != kPathQRJ;
    const TuneParams tp = tune_lookup(h, dfp ? 1 : 0, nmax, nbd);
    int C = 1;
    bool tuned_ok = false;
    double best = 1e300;
    for (int c = 1; c <= cmax; ++c) {
      cfg.gridDim = dim3(c, nb, 1);
      attr[0].val.clusterDim.x = c;
      int ncl = 0;
      if (cudaOccupancyMaxActiveClusters(&ncl, (const void *)kern, &cfg) != cudaSuccess || ncl < 1) {
        cudaGetLastError();
        continue;
      }
      tuned_ok |= c == tp.cluster;
      const double cost = (double)((nbd + ncl - 1) / ncl) / c;
      if (cost < best * (1.0 - 1e-9)) {
        best = cost;
        C = c;
      }
    }
    if (tp.cluster > cmax && tp.cluster <= 8) {  // beyond the default's range: every CTA
      cfg.gridDim = dim3(tp.cluster, nb, 1);      // still gets its share of the rows (or none)
      attr[0].val.clusterDim.x = tp.cluster;
      int ncl = 0;
      tuned_ok = cudaOccupancyMaxActiveClusters(&ncl, (const void *)kern, &cfg) == cudaSuccess && ncl >= 1;
      if (!tuned_ok) cudaGetLastError();
    }
    if (tp.cluster > 0) {  // the autotuner's size, when the launch can use it
      if (tuned_ok)
        C = tp.cluster;
      else
        tune_reject(h);
    }
    cfg.gridDim = dim3(C, nb, 1);
    attr[0].val.clusterDim.x = C;
    if (dfp) {
      k_bd_to_df<<<dim3(128, nb), 256, 0, st>>>(slots_d, path_d);
      TEBD_LAUNCHED(h);
    }
    if (h->profiling) cudaEventRecord(h->ev[4], st);
    rc = check_cuda(h, cudaLaunchKernelEx(&cfg, kern, slots_d, path_d),
                    "bidiagonalisation launch");
    if (rc) return rc;
    if (h->profiling) cudaEventRecord(h->ev[5], st);
    if (dfp) {  // the reflectors stay double-float for k_bd_apply_df; Pv follows
      k_bd_pv_to_df<<<dim3(128, nb), 256, 0, st>>>(slots_d, path_d);
      TEBD_LAUNCHED(h);
    }
    TEBD_LAUNCHED(h);
    ++h->stats.gebrd_launches;
  }
  {
    const size_t smem = (sizeof(double) + sizeof(float2) + sizeof(float)) * (size_t)(2 * nmax);
    // team size: multisection while the batch's values (nb x kk at most) leave the
    // GPU's resident threads idle, plain bisection once they fill them
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const double values = (double)nb * kk, slots_resident = 2048.0 * std::max(sms, 1);
    int team = values * 8 <= slots_resident ? 8 : values * 4 <= slots_resident ? 4
               : values * 2 <= slots_resident ? 2 : 1;
    const TuneParams tp = tune_lookup(h, b.dfp ? 1 : 0, nmax, nb);
    if (tp.team == 1 || tp.team == 2 || tp.team == 4 || tp.team == 8) team = tp.team;
    auto kern = team == 8 ? k_bd_sigma<8> : team == 4 ? k_bd_sigma<4> : team == 2 ? k_bd_sigma<2> : k_bd_sigma<1>;
    if ((rc = check_cuda(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "bisection shared memory")))
      return rc;
    kern<<<dim3(cdiv(kk, kSigmaThreads / team), nb), kSigmaThreads, smem, st>>>(slots_d, path_d, kk);
  }
  TEBD_LAUNCHED(h);
  if (b.phase == 1) return check_cuda(h, cudaGetLastError(), "bidiag launch");
  }  // vectors
  k_bd_invit<<<dim3(cdiv(kk, 32), nb), 32, 0, st>>>(slots_d, path_d, kk, cap);
  TEBD_LAUNCHED(h);
  {
    const size_t smem = sizeof(double) * 5 * (size_t)(kk > 1 ? kk : 1);
    auto okern = b.dfp ? k_bd_orth_df : k_bd_orth;
    if ((rc = check_cuda(h, cudaFuncSetAttribute(okern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "orthogonalisation shared memory")))
      return rc;
    if (b.dfp) {
      k_bd_z_df<<<dim3(64, nb), 256, 0, st>>>(slots_d, path_d, kk, cap, 1);
      TEBD_LAUNCHED(h);
    }
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(kOrthThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int oc = kOrthCluster;  // or the autotuner's size, when the launch can co-schedule it
    const TuneParams tpo = tune_lookup(h, b.dfp ? 1 : 0, nmax, nb);
    if (tpo.orth_cluster > 0) {
      cfg.gridDim = dim3((b.right_only ? 1 : 2) * tpo.orth_cluster, nb, 1);
      attr[0].val.clusterDim.x = tpo.orth_cluster;
      int ncl = 0;
      if (tpo.orth_cluster <= 8 &&
          cudaOccupancyMaxActiveClusters(&ncl, (const void *)okern, &cfg) == cudaSuccess && ncl >= 1) {
        oc = tpo.orth_cluster;
      } else {
        cudaGetLastError();
        tune_reject(h);
      }
    }
    cfg.gridDim = dim3((b.right_only ? 1 : 2) * oc, nb, 1);  // part 0 (right), then 1 (left)
    attr[0].val.clusterDim.x = oc;
    if ((rc = check_cuda(h, cudaLaunchKernelEx(&cfg, okern, slots_d, path_d, kk, cap),
                         "orthogonalisation launch")))
      return rc;
    if (b.dfp) {
      TEBD_LAUNCHED(h);
      k_bd_z_df<<<dim3(64, nb), 256, 0, st>>>(slots_d, path_d, kk, cap, 0);
    }
  }
  TEBD_LAUNCHED(h);
  if (b.dfp) {
    k_bd_apply_df<<<dim3(cdiv((b.right_only ? 1 : 2) * (size_t)kk, 8), nb), 256, 0, st>>>(slots_d, path_d, kk, cap,
                                                                                         b.right_only);
    TEBD_LAUNCHED(h);
    k_bd_store_df<<<dim3(256, nb), 256, 0, st>>>(slots_d, path_d, kk, cap, b.right_only);
    TEBD_LAUNCHED(h);
  } else {
    k_bd_apply<<<dim3(cdiv(2 * (size_t)kk, 8), nb), 256, 0, st>>>(slots_d, path_d, kk, cap);
    TEBD_LAUNCHED(h);
    k_bd_store<<<dim3(256, nb), 256, 0, st>>>(slots_d, path_d, kk, cap);
    TEBD_LAUNCHED(h);
  }
  if (h->profiling) {
    cudaEventRecord(h->ev[1], st);
    if ((rc = check_cuda(h, cudaStreamSynchronize(st), "bidiag"))) return rc;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess) h->stats.bidiag_ms += ms;
    if (cudaEventElapsedTime(&ms, h->ev[4], h->ev[5]) == cudaSuccess) h->stats.gebrd_ms += ms;
  }
  return check_cuda(h, cudaGetLastError(), "bidiag launch");
}

int run_bidiag(tebd_handle *h, int nb, int nmax) {
  BidiagBatch b;
  b.slots_d = h->slots_d;
  b.path_d = h->path_d;
  b.path_h = h->path_h.data();
  b.nb = nb;
  b.nmax = nmax;
  b.kk = h->chi;
  // the precision form, and the learned-rank form's bonds off the randomized route
  b.dfp = h->opts.svd_mode == TEBD_SVD_DF || h->opts.svd_mode == TEBD_SVD_RSVD;
  b.phase = 0;
  b.cap = 0;
  return run_bidiag_batch(h, b);
}

// Workspace of one bidiagonal problem of M x N (M >= N) computing all N triplets
// (kk = the batch's largest N): aux, tau, taup (complex) and bdws (doubles).
void bidiag_block_ws(int M, int N, int kk, size_t *aux_elems, size_t *bdws_doubles) {
  const int K = std::min(kk, N);
  *aux_elems = bd_aux_elems(M, N);
  *bdws_doubles = bd_scratch(N, kk) + 6 * (size_t)(2 * N) * K + 2 * (size_t)M * K + 4;
}

}  // namespace tebd
