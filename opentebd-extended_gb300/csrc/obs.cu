// obs.cu -- observables of the device-resident chain (the reference's
// VidalCore_v_2.0/observables_module.f90), so that a host does not download the
// chain to measure it:
//   tebd_single_site_rho   SingleSiteDensityMatrix / FormSingleSiteRho      :95-131
//   tebd_one_site_expval   OneSiteExpVal_c (complex Op), _r (real Op)        :194-252
//   tebd_two_site_rho      ThetaKernal + TwoSiteRho on sites link, link+1   :704-832
//   tebd_local_energy      LocalEnergy (open boundary)                       :1346-1387
//   tebd_total_energy      TotalEnergy (open boundary)                       :1432-1466
//   tebd_inner_product     InnerProduct                                     :1031-1089
//   tebd_chain_entropy     ChainEntropy for every link                       :1583-1602
// Sums run in a fixed order (deterministic), not in the reference's loop order,
// so results agree with it to rounding.  Two-site density matrices reuse the
// update's batched Theta formation (k_compact + k_theta_form with an identity
// gate) on the handle's SVD slots, so observables and updates of one handle are
// serialised on its stream.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "tebd_internal.cuh"

namespace tebd {

namespace {

constexpr int kObsThreads = 256;

inline unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

__device__ __forceinline__ void cacc(double2 &acc, double2 x, double2 y, double w) {  // acc += w x conj(y)
  const double re = x.x * y.x + x.y * y.y, im = x.y * y.x - x.x * y.y;
  acc.x = fma(w, re, acc.x);
  acc.y = fma(w, im, acc.y);
}

// rho_s(i,j) = sum_{a,b} l0(a)^2 l1(b)^2 G(a,i,b) conj(G(a,j,b)); one CTA per site,
// d^2 entries x (blockDim / d^2) chunks of (a,b), chunk sums added in chunk order.
__global__ void __launch_bounds__(kObsThreads) k_obs_rho1(const double2 *gam, const double *lam,
                                                          double2 *rho, int chi, int d) {
  __shared__ double2 part[kObsThreads];
  const int s = blockIdx.x;
  const double2 *G = gam + (size_t)s * chi * d * chi;
  const double *l0 = lam + (size_t)s * chi, *l1 = lam + (size_t)(s + 1) * chi;
  const int d2 = d * d, nch = kObsThreads / d2;
  const int t = threadIdx.x, ij = t % d2, ch = t / d2;
  double2 acc = make_double2(0.0, 0.0);
  if (ch < nch) {
    const int i = ij % d, j = ij / d;  // column-major position i + d j
    for (size_t e = ch; e < (size_t)chi * chi; e += nch) {
      const int a = (int)(e % chi), b = (int)(e / chi);
      const double w = l0[a] * l0[a] * l1[b] * l1[b];
      if (w == 0.0) continue;
      cacc(acc, G[a + (size_t)chi * (i + (size_t)d * b)], G[a + (size_t)chi * (j + (size_t)d * b)], w);
    }
  }
  part[t] = acc;
  __syncthreads();
  if (t < d2) {
    double2 r = make_double2(0.0, 0.0);
    for (int c = 0; c < nch; ++c) {
      r.x += part[t + c * d2].x;
      r.y += part[t + c * d2].y;
    }
    rho[(size_t)s * d2 + t] = r;
  }
}

// rho2[(i,j),(l,k)] = sum_{a,b} Theta(a,i,j,b) conj(Theta(a,l,k,b)) from the slot's
// compacted Theta X (row i*r0 + a', column j*r2 + b', ld m = d*r0); row index
// i*d + j, column l*d + k (the gate's order), column-major d^2 x d^2.  One CTA
// per (row, bond).
__global__ void __launch_bounds__(kObsThreads) k_obs_rho2(const Slot *slots, double2 *rho2, int d) {
  __shared__ double2 part[kObsThreads];
  const int s = blockIdx.y, row = blockIdx.x;
  const Slot S = slots[s];
  const Compact cp = *S.cp;
  const int r0 = cp.r0, r2 = cp.r2, m = cp.m;
  const int d2 = d * d, nch = kObsThreads / d2;
  const int t = threadIdx.x, col = t % d2, ch = t / d2;
  const int i = row / d, j = row % d, l = col / d, k = col % d;
  double2 acc = make_double2(0.0, 0.0);
  if (ch < nch)
    for (size_t e = ch; e < (size_t)r0 * r2; e += nch) {
      const int a = (int)(e % r0), b = (int)(e / r0);
      cacc(acc, S.X[(i * r0 + a) + (size_t)m * (j * r2 + b)], S.X[(l * r0 + a) + (size_t)m * (k * r2 + b)],
           1.0);
    }
  part[t] = acc;
  __syncthreads();
  if (t < d2) {
    double2 r = make_double2(0.0, 0.0);
    for (int c = 0; c < nch; ++c) {
      r.x += part[t + c * d2].x;
      r.y += part[t + c * d2].y;
    }
    rho2[(size_t)s * d2 * d2 + row + (size_t)d2 * t] = r;
  }
}

__global__ void k_obs_identity_gates(double2 *gates, int d2, int nb) {
  const size_t total = (size_t)nb * d2 * d2;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t q = e % ((size_t)d2 * d2);
    gates[e] = make_double2((q % d2) == (q / d2) ? 1.0 : 0.0, 0.0);
  }
}

// S(link) = -sum_{lambda != 0} lambda^2 ln|lambda^2| / ln(d), one warp per link
__global__ void k_obs_entropy(const double *lam, double *ent, int chi, int nlinks, double inv_logd) {
  const int link = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (link >= nlinks) return;
  const double *l = lam + (size_t)link * chi;
  double a = 0.0;
  for (int k = lane; k < chi; k += 32) {
    const double v = l[k];
    if (v != 0.0) a -= v * v * log(fabs(v * v));
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) ent[link] = a * inv_logd;
}

// C (M x N, ld ldc) = sum_k opA(m,k) B(k,n), FP64 complex, 64 x 64 tiles.
//   opA(m,k) = conjA ? conj(A[k + lda m]) * sa[m] : A[m + lda k]
//   B(k,n)   = B[k + ldb n] * (sb ? sb[n / sdiv] : 1)
constexpr int kGT = 64, kGK = 16;
__global__ void __launch_bounds__(256) k_obs_gemm(int M, int N, int K, const double2 *A, int lda, bool conjA,
                                                  const double *sa, const double2 *B, int ldb, const double *sb,
                                                  int sdiv, double2 *C, int ldc) {
  __shared__ double2 As[kGK][kGT + 1], Bs[kGK][kGT + 1];
  const int m0 = blockIdx.x * kGT, n0 = blockIdx.y * kGT;
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  double2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < K; k0 += kGK) {
    for (int e = t; e < kGK * kGT; e += 256) {
      int mm, kk;
      if (conjA) {
        kk = e % kGK;
        mm = e / kGK;
      } else {
        mm = e % kGT;
        kk = e / kGT;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      double2 a = make_double2(0.0, 0.0);
      if (gm < M && gk < K) {
        if (conjA) {
          a = A[gk + (size_t)lda * gm];
          const double w = sa ? sa[gm] : 1.0;
          a = make_double2(a.x * w, -a.y * w);
        } else {
          a = A[gm + (size_t)lda * gk];
        }
      }
      As[kk][mm] = a;
      const int nn = e / kGK, kb = e % kGK;  // B tile: k fastest
      const int gn = n0 + nn, gkb = k0 + kb;
      double2 b = make_double2(0.0, 0.0);
      if (gn < N && gkb < K) {
        b = B[gkb + (size_t)ldb * gn];
        if (sb) {
          const double w = sb[gn / sdiv];
          b = make_double2(b.x * w, b.y * w);
        }
      }
      Bs[kb][nn] = b;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kGK; ++kk) {
      double2 av[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) av[u] = As[kk][ty + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) bv[v] = Bs[kk][tx + 16 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          acc[u][v].x = fma(av[u].x, bv[v].x, fma(-av[u].y, bv[v].y, acc[u][v].x));
          acc[u][v].y = fma(av[u].x, bv[v].y, fma(av[u].y, bv[v].x, acc[u][v].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int gm = m0 + ty + 16 * u, gn = n0 + tx + 16 * v;
      if (gm < M && gn < N) C[gm + (size_t)ldc * gn] = acc[u][v];
    }
}

__global__ void k_obs_unit(double2 *E, int chi, double *e1) {  // E = e1 e1^T, e1 = unit vector
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)chi * chi;
       q += (size_t)gridDim.x * blockDim.x)
    E[q] = make_double2(q == 0 ? 1.0 : 0.0, 0.0);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < chi; q += gridDim.x * blockDim.x)
    e1[q] = q == 0 ? 1.0 : 0.0;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Workspace: rho1 (L d^2) or rho2 (nslots d^4) results, transfer matrices E, E'
// (chi^2 each), T (chi x d chi), a unit vector (chi doubles), entropies (L+1).
static int obs_ws(tebd_handle *h, size_t bytes) {
  if (h->obs_bytes >= bytes) return TEBD_OK;
  cudaFree(h->obs_buf);
  h->obs_buf = nullptr;
  h->obs_bytes = 0;
  int rc = check_cuda(h, cudaMalloc(&h->obs_buf, bytes), "alloc observables workspace");
  if (rc == TEBD_OK) h->obs_bytes = bytes;
  return rc;
}

static int obs_begin(tebd_handle *h) {
  int rc = check_cuda(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (rc) return rc;
  size_t n = (size_t)h->chi;
  size_t need = sizeof(double2) * std::max({(size_t)h->L * h->d * h->d,
                                            (size_t)h->nslots * h->d * h->d * h->d * h->d,
                                            3 * n * n + n * h->d * n}) +
                sizeof(double) * (n + h->L + 1) + 1024;
  return obs_ws(h, need);
}

static int obs_finish(tebd_handle *h, const char *what) {
  int rc = check_cuda(h, cudaGetLastError(), what);
  if (rc) return rc;
  return check_cuda(h, cudaStreamSynchronize(h->stream), what);
}

// rho2 of every bond in `links` (d^4 complex each, in list order) into `out`
static int obs_rho2(tebd_handle *h, const std::vector<int> &links, std::vector<double2> &out) {
  const int d = h->d, d2 = d * d, d4 = d2 * d2;
  out.assign((size_t)links.size() * d4, make_double2(0.0, 0.0));
  double2 *rho2_d = reinterpret_cast<double2 *>(h->obs_buf);
  // same-parity bonds share no site: odd links, then even links, nslots at a time
  std::vector<int> order;
  for (int par = 1; par >= 0; --par)
    for (size_t q = 0; q < links.size(); ++q)
      if ((links[q] & 1) == par) order.push_back((int)q);
  for (size_t base = 0; base < order.size();) {
    const int par = links[order[base]] & 1;
    std::vector<int> idx;
    while (base < order.size() && (int)idx.size() < h->nslots && (links[order[base]] & 1) == par)
      idx.push_back(order[base++]);
    const int nb = (int)idx.size();
    std::vector<int> lk(nb);
    for (int s = 0; s < nb; ++s) lk[s] = links[idx[s]];
    int rc;
    if ((rc = check_cuda(h, cudaMemcpyAsync(h->links_d, lk.data(), sizeof(int) * nb, cudaMemcpyHostToDevice,
                                            h->stream),
                         "upload links")))
      return rc;
    if ((rc = check_cuda(h, cudaMemsetAsync(h->status_d, 0, sizeof(int) * 4, h->stream), "reset status")))
      return rc;
    k_obs_identity_gates<<<64, 256, 0, h->stream>>>(h->gates_d, d2, nb);
    TEBD_LAUNCHED(h);
    if ((rc = launch_dense_prepare(h, nb, false))) return rc;
    k_obs_rho2<<<dim3(d2, nb), kObsThreads, 0, h->stream>>>(h->slots_d, rho2_d, d);
    TEBD_LAUNCHED(h);
    std::vector<double2> tmp((size_t)nb * d4);
    if ((rc = check_cuda(h, cudaMemcpyAsync(tmp.data(), rho2_d, sizeof(double2) * tmp.size(),
                                            cudaMemcpyDeviceToHost, h->stream),
                         "read two-site density matrices")))
      return rc;
    if ((rc = obs_finish(h, "two-site density matrices"))) return rc;
    for (int s = 0; s < nb; ++s)
      memcpy(out.data() + (size_t)idx[s] * d4, tmp.data() + (size_t)s * d4, sizeof(double2) * d4);
  }
  return TEBD_OK;
}

// Re Tr(H rho2) = Re sum_{a,b} H(a,b) rho2(b,a)  (TraceMatmul, TEBDtools_module.f90:401)
static double trace_matmul_re(const double *H, const double2 *rho2, int d2) {
  double acc = 0.0;
  for (int a = 0; a < d2; ++a)
    for (int b = 0; b < d2; ++b) {
      const double hr = H[2 * (a + (size_t)d2 * b)], hi = H[2 * (a + (size_t)d2 * b) + 1];
      const double2 r = rho2[b + (size_t)d2 * a];
      acc += hr * r.x - hi * r.y;
    }
  return acc;
}

}  // namespace tebd

using namespace tebd;

extern "C" int tebd_single_site_rho(tebd_handle *h, double *rho) {
  if (!h || !rho) return TEBD_ERR_ARG;
  int rc;
  if ((rc = obs_begin(h))) return rc;
  const size_t d2 = (size_t)h->d * h->d;
  double2 *rho_d = reinterpret_cast<double2 *>(h->obs_buf);
  k_obs_rho1<<<h->L, kObsThreads, 0, h->stream>>>(h->gam, h->lam, rho_d, h->chi, h->d);
  TEBD_LAUNCHED(h);
  if ((rc = check_cuda(h, cudaMemcpyAsync(rho, rho_d, sizeof(double2) * d2 * h->L, cudaMemcpyDeviceToHost,
                                          h->stream),
                       "read single-site density matrices")))
    return rc;
  return obs_finish(h, "single-site density matrices");
}

static int one_site(tebd_handle *h, const double *op, bool real_op, double *out) {
  if (!h || !op || !out) return TEBD_ERR_ARG;
  const int d = h->d, d2 = d * d;
  std::vector<double2> rho((size_t)h->L * d2);
  int rc;
  if ((rc = tebd_single_site_rho(h, reinterpret_cast<double *>(rho.data())))) return rc;
  for (int s = 0; s < h->L; ++s) {  // Tr(Op rho) = sum_{i,j} Op(i,j) rho(j,i)
    double re = 0.0, im = 0.0;
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) {
        const double2 r = rho[(size_t)s * d2 + j + (size_t)d * i];
        const double orr = real_op ? op[i + (size_t)d * j] : op[2 * (i + (size_t)d * j)];
        const double oi = real_op ? 0.0 : op[2 * (i + (size_t)d * j) + 1];
        re += orr * r.x - oi * r.y;
        im += orr * r.y + oi * r.x;
      }
    if (real_op) {
      out[s] = re;
    } else {
      out[2 * s] = re;
      out[2 * s + 1] = im;
    }
  }
  return TEBD_OK;
}

extern "C" int tebd_one_site_expval(tebd_handle *h, const double *op, double *exp_list) {
  return one_site(h, op, false, exp_list);
}

extern "C" int tebd_one_site_expval_r(tebd_handle *h, const double *op, double *exp_list) {
  return one_site(h, op, true, exp_list);
}

extern "C" int tebd_two_site_rho(tebd_handle *h, int link, double *rho2) {
  if (!h || !rho2) return TEBD_ERR_ARG;
  if (link < 1 || link > h->L - 1) return set_error(h, TEBD_ERR_ARG, "tebd_two_site_rho: link out of range");
  int rc;
  if ((rc = obs_begin(h))) return rc;
  std::vector<double2> out;
  const std::vector<int> one_link{link};
  if ((rc = obs_rho2(h, one_link, out))) return rc;
  memcpy(rho2, out.data(), sizeof(double2) * out.size());
  return TEBD_OK;
}

static int bond_energies(tebd_handle *h, int n_ops, const double *const *H, std::vector<double> &en) {
  if (!h || !H) return TEBD_ERR_ARG;
  if (n_ops < h->L - 1) return set_error(h, TEBD_ERR_ARG, "energy: need one bond operator per bond (L-1)");
  for (int l = 0; l < h->L - 1; ++l)
    if (!H[l]) return set_error(h, TEBD_ERR_ARG, "energy: null bond operator");
  int rc;
  if ((rc = obs_begin(h))) return rc;
  std::vector<int> links(h->L - 1);
  for (int l = 0; l < h->L - 1; ++l) links[l] = l + 1;
  std::vector<double2> rho2;
  if ((rc = obs_rho2(h, links, rho2))) return rc;
  const int d2 = h->d * h->d;
  en.resize(h->L - 1);
  for (int l = 0; l < h->L - 1; ++l) en[l] = trace_matmul_re(H[l], rho2.data() + (size_t)l * d2 * d2, d2);
  return TEBD_OK;
}

extern "C" int tebd_local_energy(tebd_handle *h, int n_ops, const double *const *H, double *energy) {
  if (!energy) return TEBD_ERR_ARG;
  std::vector<double> en;
  int rc = bond_energies(h, n_ops, H, en);
  if (rc) return rc;
  memcpy(energy, en.data(), sizeof(double) * en.size());
  return TEBD_OK;
}

extern "C" int tebd_total_energy(tebd_handle *h, int n_ops, const double *const *H, double *energy) {
  if (!energy) return TEBD_ERR_ARG;
  std::vector<double> en;
  int rc = bond_energies(h, n_ops, H, en);
  if (rc) return rc;
  double e = 0.0;
  for (double x : en) e += x;  // the reference's bond order
  *energy = e;
  return TEBD_OK;
}

extern "C" int tebd_inner_product(tebd_handle *left, tebd_handle *right, double *value) {
  if (!left || !right || !value) return TEBD_ERR_ARG;
  tebd_handle *h = left;
  if (left->L != right->L || left->d != right->d || left->chi != right->chi || left->device != right->device)
    return set_error(h, TEBD_ERR_ARG, "tebd_inner_product: chains differ in L, d, chi or device");
  int rc;
  if ((rc = obs_begin(h))) return rc;
  if (right != left && (rc = check_cuda(h, cudaStreamSynchronize(right->stream), "sync right chain"))) return rc;
  const int chi = h->chi, d = h->d, L = h->L;
  const size_t cc = (size_t)chi * chi;
  double2 *E = reinterpret_cast<double2 *>(h->obs_buf), *E2 = E + cc, *T = E2 + cc;
  double *e1 = reinterpret_cast<double *>(T + cc * d + cc);
  cudaStream_t st = h->stream;
  k_obs_unit<<<64, 256, 0, st>>>(E, chi, e1);
  TEBD_LAUNCHED(h);
  const size_t gsz = (size_t)chi * d * chi;
  for (int s = 0; s < L; ++s) {
    // the reference contracts the first site from left index 1 and the last site
    // into right index 1 (edge Lambdas e_1), without the edge Lambdas themselves
    const double *lr = s == L - 1 ? e1 : right->lam + (size_t)(s + 1) * chi;
    const double *ll = s == L - 1 ? e1 : left->lam + (size_t)(s + 1) * chi;
    // T = E (Gamma_R Lambda_R): chi x (d chi), column c = i + d beta
    k_obs_gemm<<<dim3(cdiv(chi, kGT), cdiv((size_t)d * chi, kGT)), 256, 0, st>>>(
        chi, d * chi, chi, E, chi, false, nullptr, right->gam + s * gsz, chi, lr, d, T, chi);
    TEBD_LAUNCHED(h);
    // E' = (Gamma_L Lambda_L)^H T over (gamma, i): chi x chi
    k_obs_gemm<<<dim3(cdiv(chi, kGT), cdiv(chi, kGT)), 256, 0, st>>>(chi, chi, d * chi, left->gam + s * gsz,
                                                                    d * chi, true, ll, T, d * chi, nullptr, 1,
                                                                    E2, chi);
    TEBD_LAUNCHED(h);
    std::swap(E, E2);
  }
  double2 v;
  if ((rc = check_cuda(h, cudaMemcpyAsync(&v, E, sizeof(double2), cudaMemcpyDeviceToHost, st), "read overlap")))
    return rc;
  if ((rc = obs_finish(h, "inner product"))) return rc;
  value[0] = v.x;
  value[1] = v.y;
  return TEBD_OK;
}

extern "C" int tebd_chain_entropy(tebd_handle *h, double *entropy) {
  if (!h || !entropy) return TEBD_ERR_ARG;
  int rc;
  if ((rc = obs_begin(h))) return rc;
  double *ent_d = reinterpret_cast<double *>(h->obs_buf);
  const int nl = h->L + 1;
  k_obs_entropy<<<cdiv(nl, 8), 256, 0, h->stream>>>(h->lam, ent_d, h->chi, nl, 1.0 / log((double)h->d));
  TEBD_LAUNCHED(h);
  if ((rc = check_cuda(h, cudaMemcpyAsync(entropy, ent_d, sizeof(double) * nl, cudaMemcpyDeviceToHost,
                                          h->stream),
                       "read entropies")))
    return rc;
  return obs_finish(h, "chain entropy");
}
