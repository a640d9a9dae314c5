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

#include "tebd_internal.cuh"

namespace tebd {

namespace {
constexpr int kBW = 16;   // warps per CTA of the bidiagonalisation kernel
constexpr int kCC = 64;   // column chunk of the right-reflector update

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

// ZLARFG on (alpha, x[0..len)) with x strided; one warp.  Returns beta in *beta,
// tau in *tau and scales x in place (x <- x / (alpha - beta)).
__device__ void warp_larfg(double2 alpha, double2 *x, size_t stride, int len, int lane,
                           double *beta_out, double2 *tau_out, bool conj_in, bool conj_out) {
  double acc = 0.0;
  for (int r = lane; r < len; r += 32) {
    const double2 v = __ldcg(x + (size_t)r * stride);
    acc = fma(v.x, v.x, fma(v.y, v.y, acc));
  }
  const double xnorm = sqrt(bsum(acc));
  if (xnorm == 0.0 && alpha.y == 0.0) {
    *beta_out = alpha.x;
    *tau_out = make_double2(0.0, 0.0);
    if (conj_in != conj_out)
      for (int r = lane; r < len; r += 32) {
        const double2 v = __ldcg(x + (size_t)r * stride);
        x[(size_t)r * stride] = make_double2(v.x, -v.y);
      }
    return;
  }
  const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm), alpha.x);
  const double2 tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
  const double dr = alpha.x - beta, di = alpha.y, den = dr * dr + di * di;
  const double2 sc = make_double2(dr / den, -di / den);
  for (int r = lane; r < len; r += 32) {
    double2 v = __ldcg(x + (size_t)r * stride);
    if (conj_in) v.y = -v.y;
    double2 o = make_double2(v.x * sc.x - v.y * sc.y, v.x * sc.y + v.y * sc.x);
    if (conj_out) o.y = -o.y;
    x[(size_t)r * stride] = o;
  }
  *beta_out = beta;
  *tau_out = tau;
}
}  // namespace

// ---------------------------------------------------------------------------
// 1. Householder bidiagonalisation, in place on X (m x n, ld m), m >= n.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBW * 32) k_gebrd(Slot *slots, const int *path) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;  // uniform per cluster
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  double2 *X = S.X;
  double *dd = S.bdws, *ee = S.bdws + n;
  double2 *Pv = S.aux;                        // n x n: right reflector vectors by column
  double2 *part = S.aux + (size_t)n * n;      // column-chunk partial sums (<= n/kCC+1) x m
  const int crank = (int)cluster.block_rank(), C = (int)cluster.num_blocks();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = crank * kBW + warp, nw = C * kBW;
  for (int i = 0; i < n; ++i) {
    // (a) left reflector on column i, rows i..m-1
    if (crank == 0 && warp == 0) {
      double beta;
      double2 tau;
      const double2 alpha = __ldcg(X + i + (size_t)m * i);
      warp_larfg(alpha, X + (i + 1) + (size_t)m * i, 1, m - i - 1, lane, &beta, &tau, false, false);
      if (lane == 0) {
        dd[i] = beta;
        S.tau[i] = tau;
        X[i + (size_t)m * i] = make_double2(beta, 0.0);
      }
    }
    cluster.sync();
    if (i < n - 1) {
      // (b) H(i)^H = I - conj(tauq) v v^H on columns i+1..n-1
      const double2 tq = __ldcg(&S.tau[i]);
      for (int c = i + 1 + gw; c < n; c += nw) {
        double wr = 0.0, wi = 0.0;
        for (int r = i + lane; r < m; r += 32) {
          const double2 x = __ldcg(X + r + (size_t)m * c);
          const double2 v = r == i ? make_double2(1.0, 0.0) : __ldcg(X + r + (size_t)m * i);
          wr = fma(v.x, x.x, fma(v.y, x.y, wr));
          wi = fma(v.x, x.y, fma(-v.y, x.x, wi));
        }
        wr = bsum(wr);
        wi = bsum(wi);
        const double fr = tq.x * wr + tq.y * wi, fi = tq.x * wi - tq.y * wr;  // conj(tq) w
        for (int r = i + lane; r < m; r += 32) {
          const double2 v = r == i ? make_double2(1.0, 0.0) : __ldcg(X + r + (size_t)m * i);
          double2 x = __ldcg(X + r + (size_t)m * c);
          x.x -= v.x * fr - v.y * fi;
          x.y -= v.x * fi + v.y * fr;
          X[r + (size_t)m * c] = x;
        }
      }
      cluster.sync();
      // (c) right reflector on row i, columns i+1..n-1 (ZLACGV, ZLARFG, ZLACGV)
      if (crank == 0 && warp == 0) {
        double beta;
        double2 tau;
        double2 alpha = __ldcg(X + i + (size_t)m * (i + 1));
        alpha.y = -alpha.y;
        // scaled vector, unconjugated, goes to Pv(:, i); the row keeps its conjugate
        double2 *row = X + i + (size_t)m * (i + 2);
        warp_larfg(alpha, row, (size_t)m, n - i - 2, lane, &beta, &tau, true, false);
        __syncwarp();
        for (int c = i + 2 + lane; c < n; c += 32) {
          const double2 u = __ldcg(X + i + (size_t)m * c);
          Pv[c + (size_t)n * i] = u;
          X[i + (size_t)m * c] = make_double2(u.x, -u.y);
        }
        if (lane == 0) {
          ee[i] = beta;
          S.taup[i] = tau;
          X[i + (size_t)m * (i + 1)] = make_double2(beta, 0.0);
          Pv[(i + 1) + (size_t)n * i] = make_double2(1.0, 0.0);
        }
      }
      cluster.sync();
      // (d) C = X(i+1:m, i+1:n) <- C (I - taup u u^H): w = C u by column chunks
      const double2 tp = __ldcg(&S.taup[i]);
      const int rows = m - i - 1, cols = n - i - 1;
      const int nrc = (rows + 31) / 32, ncc = (cols + kCC - 1) / kCC;
      for (int t = gw; t < nrc * ncc; t += nw) {
        const int rc = t % nrc, cc = t / nrc;
        const int r = i + 1 + rc * 32 + lane;
        const int c0 = i + 1 + cc * kCC, c1 = min(n, c0 + kCC);
        double wr = 0.0, wi = 0.0;
        if (r < m)
          for (int c = c0; c < c1; ++c) {
            const double2 x = __ldcg(X + r + (size_t)m * c);
            const double2 u = __ldcg(Pv + c + (size_t)n * i);
            wr = fma(x.x, u.x, fma(-x.y, u.y, wr));
            wi = fma(x.x, u.y, fma(x.y, u.x, wi));
          }
        if (r < m) part[(size_t)cc * m + r] = make_double2(wr, wi);
      }
      cluster.sync();
      for (int t = gw; t < nrc * ncc; t += nw) {
        const int rc = t % nrc, cc = t / nrc;
        const int r = i + 1 + rc * 32 + lane;
        if (r >= m) continue;
        double wr = 0.0, wi = 0.0;
        for (int q = 0; q < ncc; ++q) {  // fixed order
          const double2 p = __ldcg(part + (size_t)q * m + r);
          wr += p.x;
          wi += p.y;
        }
        // f = taup * w
        const double fr = tp.x * wr - tp.y * wi, fi = tp.x * wi + tp.y * wr;
        const int c0 = i + 1 + cc * kCC, c1 = min(n, c0 + kCC);
        for (int c = c0; c < c1; ++c) {
          const double2 u = __ldcg(Pv + c + (size_t)n * i);  // subtract f conj(u)
          double2 x = __ldcg(X + r + (size_t)m * c);
          x.x -= fr * u.x + fi * u.y;
          x.y -= fi * u.x - fr * u.y;
          X[r + (size_t)m * c] = x;
        }
      }
      cluster.sync();
    } else if (crank == 0 && threadIdx.x == 0) {
      S.taup[i] = make_double2(0.0, 0.0);
    }
  }
}

// ---------------------------------------------------------------------------
// 2. bisection: sigma_i of B for i < kk (one thread each), Golub-Kahan Sturm counts
// ---------------------------------------------------------------------------
__device__ int gk_count_less(const double *dd, const double *ee, int n, double x) {
  // eigenvalues of the zero-diagonal tridiagonal with off-diagonals d0,e0,d1,... below x
  const double pivmin = 1e-290;
  double q = -x;
  int c = q < 0.0;
  for (int j = 1; j < 2 * n; ++j) {
    const double o = (j & 1) ? dd[j >> 1] : ee[(j >> 1) - 1];
    if (fabs(q) < pivmin) q = -pivmin;
    q = -x - (o * o) / q;
    c += q < 0.0;
  }
  return c;
}

__global__ void k_bd_sigma(Slot *slots, const int *path, int kk) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int kk_s = min(kk, n);
  if (i >= kk_s) return;
  const double *dd = S.bdws, *ee = S.bdws + n;
  double hi = 0.0;
  for (int j = 0; j < n; ++j) {
    const double a = fabs(dd[j]) + (j < n - 1 ? fabs(ee[j]) : 0.0) + (j > 0 ? fabs(ee[j - 1]) : 0.0);
    hi = fmax(hi, a);
  }
  hi = hi * (1.0 + 1e-12) + 1e-300;
  double lo = 0.0, h = hi;
  const int target = 2 * n - 1 - i;  // count(< x) <= target  <=>  x <= sigma_i
  for (int it = 0; it < 256; ++it) {
    const double mid = 0.5 * (lo + h);
    if (gk_count_less(dd, ee, n, mid) <= target)
      lo = mid;
    else
      h = mid;
    if (h - lo <= 4.440892098500626e-16 * h || h < 1e-30 * hi) break;
  }
  const double sg = 0.5 * (lo + h);
  S.bdws[2 * n + i] = sg < 1e-30 * hi ? 0.0 : sg;
}

// ---------------------------------------------------------------------------
// 3a. inverse iteration on (T_GK - sigma_i I), one thread per value.
// Scratch per value (transposed so that threads of a warp touch adjacent words):
//   U0, U1, U2 (upper factor of the pivoted LU), PV (multipliers), Y (swap flags),
//   then the vector Z itself.
// ---------------------------------------------------------------------------
__global__ void k_bd_invit(Slot *slots, const int *path, int kk) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n;
  const int K = min(kk, n);
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
      const double piv = guard(d0), mult = sub / piv;
      AT(U0, j) = piv;
      AT(U1, j) = d1;
      AT(U2, j) = 0.0;
      AT(PV, j) = mult;
      AT(Y, j) = 0.0;  // no swap
      d0 = nd0 - mult * d1;
      d1 = nd1;
    } else {  // row j+1 becomes the pivot row
      const double mult = d0 / sub;
      AT(U0, j) = sub;
      AT(U1, j) = nd0;
      AT(U2, j) = nd1;
      AT(PV, j) = mult;
      AT(Y, j) = 1.0;  // swapped
      d0 = d1 - mult * nd0;
      d1 = -mult * nd1;
    }
  }
  AT(U0, N - 1) = guard(d0);
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
      double x = sacc / AT(U0, j);
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

// 3b. split z into v (even) and u (odd) and re-orthogonalise each set, in order
// of descending sigma, by classical Gram-Schmidt applied twice.  One CTA per
// bond; the dot products of vector i against all earlier ones are one warp each.
__global__ void __launch_bounds__(512) k_bd_orth(Slot *slots, const int *path, int kk) {
  const int s = blockIdx.x;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = min(kk, n);
  double *Z = S.bdws + bd_scratch(n, kk) + 5 * (size_t)N * K;  // element (j, i) at [j * K + i]
  extern __shared__ double dots[];                        // K
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int part = 0; part < 2; ++part) {  // 0: v = z[2j], 1: u = z[2j+1]
#define ZE(j, i) Z[(size_t)(2 * (j) + part) * K + (i)]
    for (int i = 0; i < K; ++i) {
      for (int pass = 0; pass < 2; ++pass) {
        for (int q = warp; q < i; q += nw) {
          double a = 0.0;
          for (int j = lane; j < n; j += 32) a = fma(ZE(j, q), ZE(j, i), a);
          a = bsum(a);
          if (lane == 0) dots[q] = a;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          double v = ZE(j, i);
          for (int q = 0; q < i; ++q) v = fma(-dots[q], ZE(j, q), v);
          ZE(j, i) = v;
        }
        __syncthreads();
      }
      if (warp == 0) {
        double a = 0.0;
        for (int j = lane; j < n; j += 32) a = fma(ZE(j, i), ZE(j, i), a);
        a = bsum(a);
        if (lane == 0) dots[0] = a > 0.0 ? 1.0 / sqrt(a) : 0.0;
      }
      __syncthreads();
      const double inv = dots[0];
      for (int j = threadIdx.x; j < n; j += blockDim.x) ZE(j, i) *= inv;
      __syncthreads();
    }
#undef ZE
  }
}

// ---------------------------------------------------------------------------
// 4. left vectors Q [Ub; 0] (M x K) and right vectors P Vb (N x K) of the
//    bidiagonalised matrix, one warp per kept column.
//    Theta route:   left -> Yu (scratch), right -> S.V (ld n).
//    Theta^H route: left -> Yu (= V of Theta), right -> Ru (= U of Theta, scratch
//    in the inverse-iteration LU area, free by now).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bd_apply(Slot *slots, const int *path, int kk) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int m, n;
  bd_dims(*S.cp, route, m, n);
  const int N = 2 * n, K = min(kk, n);
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
__global__ void k_bd_store(Slot *slots, const int *path, int kk) {
  const int s = blockIdx.y;
  const int route = path[s];
  if (!on_route(route)) return;
  const Slot S = slots[s];
  int M, N;
  bd_dims(*S.cp, route, M, N);
  const int m = S.cp->m, n = S.cp->n, K = min(kk, N);
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
  if (blockIdx.x == 0 && threadIdx.x == 0) S.cp->k = K;
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
size_t bidiag_ws_doubles(int n, int chi) {
  const int K = std::min(chi, n);
  return bd_scratch(n, chi) + 6 * (size_t)(2 * n) * K + 2 * (size_t)n * K;
}

int run_bidiag(tebd_handle *h, int nb, int nmax) {
  cudaStream_t st = h->stream;
  const int kk = h->chi;
  int rc;
  if (h->profiling) cudaEventRecord(h->ev[0], st);
  bool any_t = false;
  for (int s = 0; s < nb; ++s) any_t |= h->path_h[s] == kPathBidiagT;
  if (any_t) {
    k_bd_stage<<<dim3(128, nb), 256, 0, st>>>(h->slots_d, h->path_d);
    TEBD_LAUNCHED(h);
    const unsigned g = cdiv(nmax, 32) < 8 ? cdiv(nmax, 32) : 8;
    k_bd_transpose<<<dim3(g, g, nb), 256, 0, st>>>(h->slots_d, h->path_d);
    TEBD_LAUNCHED(h);
  }
  {
    int C = (nmax + kBW * 8 - 1) / (kBW * 8);
    C = C < 1 ? 1 : (C > 8 ? 8 : C);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C, nb, 1);
    cfg.blockDim = dim3(kBW * 32, 1, 1);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    rc = check_cuda(h, cudaLaunchKernelEx(&cfg, k_gebrd, h->slots_d, (const int *)h->path_d),
                    "bidiagonalisation launch");
    if (rc) return rc;
    TEBD_LAUNCHED(h);
  }
  k_bd_sigma<<<dim3(cdiv(kk, 128), nb), 128, 0, st>>>(h->slots_d, h->path_d, kk);
  TEBD_LAUNCHED(h);
  k_bd_invit<<<dim3(cdiv(kk, 128), nb), 128, 0, st>>>(h->slots_d, h->path_d, kk);
  TEBD_LAUNCHED(h);
  k_bd_orth<<<nb, 512, sizeof(double) * (size_t)(kk > 1 ? kk : 1), st>>>(h->slots_d, h->path_d, kk);
  TEBD_LAUNCHED(h);
  k_bd_apply<<<dim3(cdiv(2 * (size_t)kk, 8), nb), 256, 0, st>>>(h->slots_d, h->path_d, kk);
  TEBD_LAUNCHED(h);
  k_bd_store<<<dim3(256, nb), 256, 0, st>>>(h->slots_d, h->path_d, kk);
  TEBD_LAUNCHED(h);
  if (h->profiling) {
    cudaEventRecord(h->ev[1], st);
    if ((rc = check_cuda(h, cudaStreamSynchronize(st), "bidiag"))) return rc;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess) h->stats.bidiag_ms += ms;
  }
  return check_cuda(h, cudaGetLastError(), "bidiag launch");
}

}  // namespace tebd
