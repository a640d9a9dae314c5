// capi.cu -- the extern "C" boundary (include/tebd_capi.h) and its host orchestration.
//
// Host-side mirror of the reference's call structure:
//   tebd_two_site_op(_r)     TwoSiteOp_c/_r   local_operations_module.f90:430-494
//   tebd_two_site_op_nc(_r)  TwoSiteOpNC_c/_r local_operations_module.f90:1723-1964
//   tebd_trotter_step        TrotterStep2ndOrder / TrotterStep5thOrder (OBC) and the NC twins
//                            propagation_module.f90:82-114, 200-252, 956-1018
// The reference applies the bonds of one sweep one after another; bonds of one
// parity touch disjoint Gammas and Lambda(link+1) and only read the shared outer
// Lambdas, so here each sweep is one batch (tebd_apply_bonds).  Truncation errors
// are summed on the host in the reference's bond order.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "tebd_internal.cuh"

using tebd::Slot;

namespace tebd {

int set_error(tebd_handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

int check_cuda(tebd_handle *h, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return TEBD_OK;
  (void)cudaGetLastError();
  return set_error(h, e == cudaErrorMemoryAllocation ? TEBD_ERR_OOM : TEBD_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

// pinned staging layout
constexpr size_t kPinFlags = 0;        // 64 bytes: pending count, status flags
constexpr size_t kPinTrunc = 64;       // nslots doubles
static size_t pin_gates_off(const tebd_handle *h) {
  return (kPinTrunc + sizeof(double) * h->nslots + 255) & ~(size_t)255;
}
static size_t pin_links_off(const tebd_handle *h) {
  return pin_gates_off(h) + sizeof(double2) * (size_t)h->nslots * h->d * h->d * h->d * h->d;
}

}  // namespace tebd

using namespace tebd;

static thread_local std::string g_noh_err;
namespace tebd {
// the message tebd_last_error(NULL) returns (calls that take no handle)
void set_noh_error(const std::string &msg) { g_noh_err = msg; }
}  // namespace tebd

#define CK(expr, what)                                   \
  do {                                                   \
    int _rc = tebd::check_cuda(h, (expr), (what));       \
    if (_rc) return _rc;                                 \
  } while (0)

extern "C" void tebd_default_opts(tebd_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->version = TEBD_OPTS_VERSION;
}

static void free_all(tebd_handle *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->gam);
  cudaFree(h->lam);
  cudaFree(h->lab_l);
  cudaFree(h->lab_r);
  cudaFree(h->ws_base);
  cudaFree(h->slots_d);
  cudaFree(h->gates_d);
  cudaFree(h->cp_d);
  cudaFree(h->path_d);
  cudaFree(h->idx_d);
  cudaFree(h->nrm_part);
  cudaFree(h->nrm);
  cudaFree(h->truncerr_d);
  cudaFree(h->links_d);
  cudaFree(h->js.rot);
  cudaFree(h->js.done);
  cudaFree(h->js.sweeps);
  cudaFree(h->js.pending);
  cudaFree(h->js.counters);
  for (int e = 0; e < 6; ++e)
    if (h->ev[e]) cudaEventDestroy(h->ev[e]);
  cudaFree(h->jprob_d);
  cudaFree(h->jprobf_d);
  cudaFree(h->status_d);
  cudaFree(h->obs_buf);
  cudaFree(h->sig_link_d);
  cudaFree(h->sig_count_d);
  cudaFree(h->sweeps_link_d);
  tebd::nc_free(h);
  tebd::tc_free(h);
  tebd::rsvd_free(h);
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->stream) cudaStreamDestroy(h->stream);
}

template <typename P>
static int dalloc(tebd_handle *h, P **p, size_t bytes, const char *what) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  return tebd::check_cuda(h, cudaMalloc((void **)p, bytes), what);
}

extern "C" int tebd_create(int L, int d, int chi, int mode, const tebd_opts *opts,
                           tebd_handle **out) {
  if (!out) return TEBD_ERR_ARG;
  *out = nullptr;
  tebd_opts o;
  tebd_default_opts(&o);
  if (opts) {
    if (opts->version != TEBD_OPTS_VERSION) {
      g_noh_err = "tebd_create: opts.version mismatch";
      return TEBD_ERR_ARG;
    }
    o = *opts;
  }
  if (L < 2 || d < 1 || d > 8 || chi < 1 || (mode != TEBD_MODE_DENSE && mode != TEBD_MODE_NC) ||
      (o.svd_mode != TEBD_SVD_FP64 && o.svd_mode != TEBD_SVD_JACOBI &&
       o.svd_mode != TEBD_SVD_BIDIAG && o.svd_mode != TEBD_SVD_QRJ && o.svd_mode != TEBD_SVD_DF &&
       !(o.svd_mode == TEBD_SVD_RSVD && mode == TEBD_MODE_DENSE))) {
    g_noh_err = "tebd_create: invalid L/d/chi/mode (need L>=2, 1<=d<=8, chi>=1)";
    return TEBD_ERR_ARG;
  }
  if ((long long)d * chi > 8192) {
    g_noh_err = "tebd_create: d*chi > 8192 is not supported";
    return TEBD_ERR_ARG;
  }
  if (mode == TEBD_MODE_NC && (o.tot_num < 0 || o.tot_num >= 1000 || o.max_filling < 0)) {
    // labels >= 1000 mean "unused" in the reference, so particle numbers stay below 1000
    g_noh_err = "tebd_create: NC mode needs 0 <= tot_num < 1000 and max_filling >= 0";
    return TEBD_ERR_ARG;
  }
  tebd_handle *h = new (std::nothrow) tebd_handle();
  if (h) {  // randomized route defaults (tebd_set_rsvd)
    h->rs_oversample = 64;
    h->rs_power = 2;
    h->rs_tol = 1e-5;
    h->rs_slices = 7;
  }
  if (!h) return TEBD_ERR_OOM;
  h->L = L;
  h->d = d;
  h->chi = chi;
  h->mode = mode;
  h->n = d * chi;
  h->opts = o;
  h->device = o.device;
  h->launches = 0;
  int rc;
#define FAIL(code)                 \
  do {                             \
    g_noh_err = h->err;            \
    free_all(h);                   \
    delete h;                      \
    return (code);                 \
  } while (0)
  if ((rc = check_cuda(h, cudaSetDevice(o.device), "cudaSetDevice"))) FAIL(rc);
  cudaDeviceProp prop;
  if ((rc = check_cuda(h, cudaGetDeviceProperties(&prop, o.device), "cudaGetDeviceProperties")))
    FAIL(rc);
  if (prop.major * 10 + prop.minor != 103) {
    set_error(h, TEBD_ERR_CUDA,
              "this library is built for sm_103a (GB300); device is sm_" +
                  std::to_string(prop.major * 10 + prop.minor));
    FAIL(TEBD_ERR_CUDA);
  }
  if ((rc = check_cuda(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking),
                       "cudaStreamCreate")))
    FAIL(rc);
  const int n = h->n;
  const size_t csz = (size_t)chi * d * chi;
  // slots: at most one per bond of one parity
  int maxpar = L / 2;
  if (maxpar < 1) maxpar = 1;
  h->nslots = (o.max_batch > 0 && o.max_batch < maxpar) ? o.max_batch : maxpar;
  const int ns = h->nslots;
  if ((rc = dalloc(h, &h->gam, sizeof(double2) * csz * L, "alloc Gammas"))) FAIL(rc);
  if ((rc = dalloc(h, &h->lam, sizeof(double) * (size_t)chi * (L + 1), "alloc Lambdas"))) FAIL(rc);
  if ((rc = dalloc(h, &h->lab_l, sizeof(int) * (size_t)chi * (L + 1), "alloc labels"))) FAIL(rc);
  if ((rc = dalloc(h, &h->lab_r, sizeof(int) * (size_t)chi * (L + 1), "alloc labels"))) FAIL(rc);
  // workspace carve
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t nn = (size_t)n * n;
  // per slot: X, V (n^2 each), S, perm, QR buffers (jpvt, tau, 2n norms), aux (3 n^2)
  // (the QR buffers and aux serve the dense path only; NC blocks live in X and V)
  const size_t aux_elems = mode == TEBD_MODE_DENSE ? std::max(3 * nn, bidiag_aux_elems(n)) : 0;
  const size_t bd_elems = mode == TEBD_MODE_DENSE ? bidiag_ws_doubles(n, chi) : 0;
  size_t per = al(sizeof(double2) * nn) * 2 + al(sizeof(double) * n) + al(sizeof(int) * n) +
               al(sizeof(int) * n) + al(sizeof(double2) * n) * 2 + al(sizeof(double) * 2 * n) +
               al(sizeof(double2) * aux_elems) + al(sizeof(double) * bd_elems);
  h->ws_bytes = per * ns;
  if ((rc = dalloc(h, (char **)&h->ws_base, h->ws_bytes, "alloc SVD workspaces"))) FAIL(rc);
  if ((rc = dalloc(h, &h->gates_d, sizeof(double2) * (size_t)ns * d * d * d * d, "alloc gates")))
    FAIL(rc);
  if ((rc = dalloc(h, &h->cp_d, sizeof(Compact) * ns, "alloc compaction records"))) FAIL(rc);
  if ((rc = dalloc(h, &h->path_d, sizeof(int) * ns, "alloc SVD routes"))) FAIL(rc);
  h->path_h.assign(ns, kPathQRJ);
  if ((rc = dalloc(h, &h->idx_d, sizeof(int) * (size_t)ns * 5 * chi, "alloc index maps"))) FAIL(rc);
  h->slots.resize(ns);
  {
    char *p = (char *)h->ws_base;
    for (int s = 0; s < ns; ++s) {
      Slot &S = h->slots[s];
      memset(&S, 0, sizeof(S));
      S.X = (double2 *)p;
      p += al(sizeof(double2) * nn);
      S.V = (double2 *)p;
      p += al(sizeof(double2) * nn);
      S.S = (double *)p;
      p += al(sizeof(double) * n);
      S.perm = (int *)p;
      p += al(sizeof(int) * n);
      S.jpvt = (int *)p;
      p += al(sizeof(int) * n);
      S.tau = (double2 *)p;
      p += al(sizeof(double2) * n);
      S.vn = (double *)p;
      p += al(sizeof(double) * 2 * n);
      S.aux = aux_elems ? (double2 *)p : nullptr;
      p += al(sizeof(double2) * aux_elems);
      S.taup = (double2 *)p;
      p += al(sizeof(double2) * n);
      S.bdws = bd_elems ? (double *)p : nullptr;
      p += al(sizeof(double) * bd_elems);
      S.gate = h->gates_d + (size_t)s * d * d * d * d;
      int *ix = h->idx_d + (size_t)s * 5 * chi;
      S.idx0 = ix;
      S.idx1 = ix + chi;
      S.idx2 = ix + 2 * chi;
      S.inv0 = ix + 3 * chi;
      S.inv2 = ix + 4 * chi;
      S.cp = h->cp_d + s;
    }
  }
  if ((rc = dalloc(h, &h->slots_d, sizeof(Slot) * ns, "alloc slot table"))) FAIL(rc);
  if ((rc = check_cuda(h, cudaMemcpy(h->slots_d, h->slots.data(), sizeof(Slot) * ns,
                                     cudaMemcpyHostToDevice),
                       "upload slot table")))
    FAIL(rc);
  {
    std::vector<JacobiProblem<double>> jp(ns);
    for (int s = 0; s < ns; ++s) jp[s] = {h->slots[s].X, h->slots[s].V, n, n, n, n, 0.0};
    if ((rc = dalloc(h, (char **)&h->jprob_d, sizeof(JacobiProblem<double>) * ns, "alloc jprob")))
      FAIL(rc);
    if ((rc = check_cuda(h, cudaMemcpy(h->jprob_d, jp.data(), sizeof(JacobiProblem<double>) * ns,
                                       cudaMemcpyHostToDevice),
                         "upload jprob")))
      FAIL(rc);
  }
  if ((rc = dalloc(h, &h->nrm_part, sizeof(double) * ns * kNormParts, "alloc norm"))) FAIL(rc);
  if ((rc = dalloc(h, &h->nrm, sizeof(double) * ns, "alloc norm"))) FAIL(rc);
  if ((rc = dalloc(h, &h->truncerr_d, sizeof(double) * ns, "alloc truncerr"))) FAIL(rc);
  if ((rc = dalloc(h, &h->links_d, sizeof(int) * ns, "alloc links"))) FAIL(rc);
  h->js_cap = ns * (mode == TEBD_MODE_NC ? (o.tot_num + 2 > 64 ? o.tot_num + 2 : 64) : 1);
  if ((rc = dalloc(h, &h->js.rot, sizeof(int) * 2 * h->js_cap, "alloc jacobi state"))) FAIL(rc);
  if ((rc = dalloc(h, &h->js.done, sizeof(int) * h->js_cap, "alloc jacobi state"))) FAIL(rc);
  if ((rc = dalloc(h, &h->js.sweeps, sizeof(int) * h->js_cap, "alloc jacobi state"))) FAIL(rc);
  if ((rc = dalloc(h, &h->js.pending, sizeof(int) * 4, "alloc jacobi state"))) FAIL(rc);
  if ((rc = dalloc(h, &h->js.counters, sizeof(unsigned long long) * 4, "alloc counters"))) FAIL(rc);
  if ((rc = check_cuda(h, cudaMemset(h->js.counters, 0, sizeof(unsigned long long) * 4), "memset")))
    FAIL(rc);
  for (int e = 0; e < 6; ++e)
    if ((rc = check_cuda(h, cudaEventCreate(&h->ev[e]), "cudaEventCreate"))) FAIL(rc);
  if ((rc = dalloc(h, &h->status_d, sizeof(int) * 4, "alloc status"))) FAIL(rc);
  if ((rc = dalloc(h, &h->sig_link_d, sizeof(double) * (size_t)(L - 1) * n, "alloc spectra")))
    FAIL(rc);
  if ((rc = dalloc(h, &h->sig_count_d, sizeof(int) * (L - 1), "alloc spectra"))) FAIL(rc);
  if ((rc = dalloc(h, &h->sweeps_link_d, sizeof(int) * (L - 1), "alloc spectra"))) FAIL(rc);
  h->pinned_bytes = pin_links_off(h) + sizeof(int) * ns + 256;
  if ((rc = check_cuda(h, cudaMallocHost((void **)&h->pinned, h->pinned_bytes), "alloc pinned")))
    FAIL(rc);
  // initial state as AllocateGamLam / AllocateLabel leave it: zeros and label 10000
  if ((rc = check_cuda(h, cudaMemset(h->gam, 0, sizeof(double2) * csz * L), "memset"))) FAIL(rc);
  if ((rc = check_cuda(h, cudaMemset(h->lam, 0, sizeof(double) * (size_t)chi * (L + 1)), "memset")))
    FAIL(rc);
  if ((rc = check_cuda(h, cudaMemset(h->status_d, 0, sizeof(int) * 4), "memset"))) FAIL(rc);
  if ((rc = check_cuda(h, cudaMemset(h->sig_count_d, 0, sizeof(int) * (L - 1)), "memset"))) FAIL(rc);
  if ((rc = check_cuda(h, cudaMemset(h->sweeps_link_d, 0, sizeof(int) * (L - 1)), "memset")))
    FAIL(rc);
  {
    std::vector<int> lab((size_t)chi * (L + 1), kLabelUnused);
    if ((rc = check_cuda(h, cudaMemcpy(h->lab_l, lab.data(), sizeof(int) * lab.size(),
                                       cudaMemcpyHostToDevice), "init labels")))
      FAIL(rc);
    if ((rc = check_cuda(h, cudaMemcpy(h->lab_r, lab.data(), sizeof(int) * lab.size(),
                                       cudaMemcpyHostToDevice), "init labels")))
      FAIL(rc);
  }
  if (mode == TEBD_MODE_NC) {
    if ((rc = tebd::nc_alloc(h))) FAIL(rc);
  }
#undef FAIL
  *out = h;
  return TEBD_OK;
}

extern "C" int tebd_destroy(tebd_handle *h) {
  if (!h) return TEBD_ERR_ARG;
  free_all(h);
  delete h;
  return TEBD_OK;
}

extern "C" const char *tebd_last_error(tebd_handle *h) {
  return h ? h->err.c_str() : g_noh_err.c_str();
}

extern "C" long long tebd_kernel_launches(tebd_handle *h) { return h ? h->launches : -1; }

extern "C" int tebd_sync(tebd_handle *h) {
  if (!h) return TEBD_ERR_ARG;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(cudaStreamSynchronize(h->stream), "tebd_sync");
  return TEBD_OK;
}

static int xfer(tebd_handle *h, void *dst, const void *src, size_t bytes, cudaMemcpyKind k,
                const char *what) {
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  CK(cudaMemcpyAsync(dst, src, bytes, k, h->stream), what);
  CK(cudaStreamSynchronize(h->stream), what);
  return TEBD_OK;
}

extern "C" int tebd_set_gamma(tebd_handle *h, int site, const double *g) {
  if (!h || !g) return TEBD_ERR_ARG;
  if (site < 1 || site > h->L) return set_error(h, TEBD_ERR_ARG, "tebd_set_gamma: site out of range");
  const size_t csz = (size_t)h->chi * h->d * h->chi;
  return xfer(h, h->gam + (site - 1) * csz, g, sizeof(double2) * csz, cudaMemcpyHostToDevice,
              "tebd_set_gamma");
}

extern "C" int tebd_get_gamma(tebd_handle *h, int site, double *g) {
  if (!h || !g) return TEBD_ERR_ARG;
  if (site < 1 || site > h->L) return set_error(h, TEBD_ERR_ARG, "tebd_get_gamma: site out of range");
  const size_t csz = (size_t)h->chi * h->d * h->chi;
  return xfer(h, g, h->gam + (site - 1) * csz, sizeof(double2) * csz, cudaMemcpyDeviceToHost,
              "tebd_get_gamma");
}

extern "C" int tebd_set_lambda(tebd_handle *h, int link, const double *l) {
  if (!h || !l) return TEBD_ERR_ARG;
  if (link < 1 || link > h->L + 1)
    return set_error(h, TEBD_ERR_ARG, "tebd_set_lambda: link out of range");
  return xfer(h, h->lam + (size_t)(link - 1) * h->chi, l, sizeof(double) * h->chi,
              cudaMemcpyHostToDevice, "tebd_set_lambda");
}

extern "C" int tebd_get_lambda(tebd_handle *h, int link, double *l) {
  if (!h || !l) return TEBD_ERR_ARG;
  if (link < 1 || link > h->L + 1)
    return set_error(h, TEBD_ERR_ARG, "tebd_get_lambda: link out of range");
  return xfer(h, l, h->lam + (size_t)(link - 1) * h->chi, sizeof(double) * h->chi,
              cudaMemcpyDeviceToHost, "tebd_get_lambda");
}

extern "C" int tebd_set_labels(tebd_handle *h, int link, const int *ll, const int *lr) {
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_NC) return set_error(h, TEBD_ERR_STATE, "labels need TEBD_MODE_NC");
  if (link < 1 || link > h->L + 1)
    return set_error(h, TEBD_ERR_ARG, "tebd_set_labels: link out of range");
  int rc;
  if (ll && (rc = xfer(h, h->lab_l + (size_t)(link - 1) * h->chi, ll, sizeof(int) * h->chi,
                       cudaMemcpyHostToDevice, "tebd_set_labels")))
    return rc;
  if (lr && (rc = xfer(h, h->lab_r + (size_t)(link - 1) * h->chi, lr, sizeof(int) * h->chi,
                       cudaMemcpyHostToDevice, "tebd_set_labels")))
    return rc;
  return TEBD_OK;
}

extern "C" int tebd_get_labels(tebd_handle *h, int link, int *ll, int *lr) {
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_NC) return set_error(h, TEBD_ERR_STATE, "labels need TEBD_MODE_NC");
  if (link < 1 || link > h->L + 1)
    return set_error(h, TEBD_ERR_ARG, "tebd_get_labels: link out of range");
  int rc;
  if (ll && (rc = xfer(h, ll, h->lab_l + (size_t)(link - 1) * h->chi, sizeof(int) * h->chi,
                       cudaMemcpyDeviceToHost, "tebd_get_labels")))
    return rc;
  if (lr && (rc = xfer(h, lr, h->lab_r + (size_t)(link - 1) * h->chi, sizeof(int) * h->chi,
                       cudaMemcpyDeviceToHost, "tebd_get_labels")))
    return rc;
  return TEBD_OK;
}

extern "C" int tebd_get_singular_values(tebd_handle *h, int link, double *sigma, int *count) {
  if (!h || !sigma || !count) return TEBD_ERR_ARG;
  if (link < 1 || link > h->L - 1)
    return set_error(h, TEBD_ERR_ARG, "tebd_get_singular_values: link out of range");
  int rc;
  if ((rc = xfer(h, count, h->sig_count_d + (link - 1), sizeof(int), cudaMemcpyDeviceToHost,
                 "get spectrum count")))
    return rc;
  if (*count > 0)
    return xfer(h, sigma, h->sig_link_d + (size_t)(link - 1) * h->n, sizeof(double) * *count,
                cudaMemcpyDeviceToHost, "get spectrum");
  return TEBD_OK;
}

extern "C" int tebd_get_sweeps(tebd_handle *h, int link, int *sweeps) {
  if (!h || !sweeps) return TEBD_ERR_ARG;
  if (link < 1 || link > h->L - 1)
    return set_error(h, TEBD_ERR_ARG, "tebd_get_sweeps: link out of range");
  return xfer(h, sweeps, h->sweeps_link_d + (link - 1), sizeof(int), cudaMemcpyDeviceToHost,
              "get sweeps");
}

// A bond the randomized route may take: saturated (all chi of its Lambda in use)
// with Schmidt values spanning at most kRsvdSpan (the sketch is orthonormalised
// through Grams, which resolve directions down to ~1e-7 of the largest), a
// compacted Theta with room for a sketch beyond the kept rank, and within the
// bidiagonal route's size limit (its fallback).
constexpr float kRsvdSpan = 1e-6f;
static bool rsvd_candidate(const tebd_handle *h, const Compact &c) {
  const int mn = std::min(c.m, c.n);
  return c.r1 == h->chi && c.span >= kRsvdSpan && mn >= h->chi + 32 && std::max(c.m, c.n) <= kBidiagMaxDim;
}

// The learned model's choice for the randomized route of one batch: per bond
// the predicted log10 sigma_k / sigma_0 at k / chi = kMlpRanks (interpolated
// linearly, extended past the last point along its last segment).  A pair (p, q)
// is feasible for a bond when the weight the sketch can miss in the kept
// directions, (sigma_chi / sigma_0)^2 (sigma_{chi+p} / sigma_chi)^(2q + 2), is at
// most `target` (the directions near sigma_chi converge slowest and carry the
// least weight) and the judge's residual of the slowest kept direction,
// (sigma_chi / sigma_0) (sigma_{chi+p} / sigma_chi)^(2q + 1), is a decade inside
// its tolerance.  Its cost is the route's time model, in units of one product
// column over an n x n Theta: n^2 s (2q + 4) for the products (the sketch, q
// power iterations and the Rayleigh-Ritz and judge passes) plus s^3 (6 (q + 2) +
// 128) for the q + 2 Choleskys and the s x s Gram SVD (s = chi + p; weights
// measured on GB300 at chi = 512, where the Gram SVD is about as costly as all
// the products).  Each bond takes its cheapest feasible pair; bonds with none
// take the full SVD (allow = 0); the batch runs with the largest p and q chosen.
static int rsvd_model_choice(tebd_handle *h, int nb, const double *const *gates, const std::vector<Compact> &cps,
                             int *over, int *power, std::vector<char> &allow) {
  const int d2 = h->d * h->d;
  std::vector<float> gt(3 * (size_t)nb), pred((size_t)kMlpOut * nb);
  for (int s = 0; s < nb; ++s) {
    const double *g = gates[s];
    double off = 0.0, dev = 0.0;
    for (int c = 0; c < d2; ++c)
      for (int r = 0; r < d2; ++r) {
        const double re = g[2 * (r + (size_t)d2 * c)], im = g[2 * (r + (size_t)d2 * c) + 1];
        const double a2 = re * re + im * im;
        if (r != c) off += a2;
        dev += r == c ? (re - 1.0) * (re - 1.0) + im * im : a2;
      }
    gt[3 * s] = (float)(dev > 0.0 ? std::max(-16.0, 0.5 * log10(dev)) : -16.0);
    gt[3 * s + 1] = (float)(off > 0.0 ? std::max(-16.0, 0.5 * log10(off)) : -16.0);
    gt[3 * s + 2] = (float)h->d / 8.f;
  }
  int rc = mlp_features_forward(h->rs_model, h->lam, h->links_d, gt.data(), h->chi, nb, h->stream, pred.data());
  if (rc) return set_error(h, rc, std::string("rsvd model: ") + tebd_mlp_last_error(h->rs_model));
  auto at = [&](const float *y, double rho) {
    int j = 0;
    while (j < kMlpOut - 2 && rho > kMlpRanks[j + 1]) ++j;
    const double t = (rho - kMlpRanks[j]) / (kMlpRanks[j + 1] - kMlpRanks[j]);
    return (double)y[j] + t * ((double)y[j + 1] - (double)y[j]);
  };
  static const int kP[] = {16, 32, 48, 64, 96, 128};
  const double lt = log10(h->rs_target);
  // the judge's residual of the slowest kept direction is about
  // sigma_chi (sigma_{chi+p} / sigma_chi)^(2q+1): kept a decade inside its tolerance
  const double ltol = log10(h->rs_tol) - 1.0;
  int pmax = 0, qmax = 0;
  for (int s = 0; s < nb; ++s) {
    const float *y = pred.data() + (size_t)kMlpOut * s;
    const double y1 = std::min(0.0, at(y, 1.0));
    const double nn = (double)std::max(cps[s].m, cps[s].n);
    double best = 1e300;
    int bp = -1, bq = -1;
    for (int p : kP)
      for (int q = 0; q <= 3; ++q) {
        const double lr = at(y, (double)(h->chi + p) / h->chi) - y1;
        if (!(lr < 0.0) || 2.0 * y1 + (2.0 * q + 2.0) * lr > lt) continue;
        if (y1 + (2.0 * q + 1.0) * lr > ltol) continue;  // the judge would reject the slowest direction
        const double sk = (double)(h->chi + p);
        const double cost = nn * nn * sk * (2 * q + 4) + sk * sk * sk * (6.0 * (q + 2) + 128.0);
        if (cost < best) {
          best = cost;
          bp = p;
          bq = q;
        }
      }
    allow[s] = bp >= 0;
    if (bp >= 0) {
      pmax = std::max(pmax, bp);
      qmax = std::max(qmax, bq);
    }
  }
  *over = pmax ? pmax : h->rs_oversample;
  *power = pmax ? qmax : h->rs_power;
  return TEBD_OK;
}

// One batch of at most nslots non-overlapping bonds (complex gates).
static int run_batch(tebd_handle *h, int nb, const int *links, const double *const *gates,
                     double *truncerr) {
  const int d4 = h->d * h->d * h->d * h->d;
  char *pin = (char *)h->pinned;
  double2 *g_pin = (double2 *)(pin + pin_gates_off(h));
  int *l_pin = (int *)(pin + pin_links_off(h));
  for (int s = 0; s < nb; ++s) {
    memcpy(g_pin + (size_t)s * d4, gates[s], sizeof(double2) * d4);
    l_pin[s] = links[s];
  }
  CK(cudaMemcpyAsync(h->gates_d, g_pin, sizeof(double2) * (size_t)nb * d4, cudaMemcpyHostToDevice,
                     h->stream),
     "upload gates");
  CK(cudaMemcpyAsync(h->links_d, l_pin, sizeof(int) * nb, cudaMemcpyHostToDevice, h->stream),
     "upload links");
  CK(cudaMemsetAsync(h->status_d, 0, sizeof(int) * 4, h->stream), "reset status");
  if (h->profiling) cudaEventRecord(h->ev[2], h->stream);
  int rc;
  if (h->mode == TEBD_MODE_DENSE) {
    if ((rc = launch_dense_prepare(h, nb, false))) return rc;
    int nmax = 0;
    std::vector<Compact> cps;
    if ((rc = dense_compact_sizes(h, nb, &nmax, &cps))) return rc;
    if (h->opts.svd_mode == TEBD_SVD_JACOBI) {
      CK(cudaMemsetAsync(h->path_d, 0, sizeof(int) * nb, h->stream), "reset SVD routes");
      if ((rc = launch_eye(h, nb))) return rc;
      if ((rc = run_jacobi(h, nb, h->opts.svd_mode, nmax))) return rc;
    } else {
      // route per bond: bidiagonalisation when the compacted Theta is large in both
      // dimensions (default: min(m, n) >= kBidiagMinDim in a batch that holds a
      // saturated or large bond, below; a wide Theta is bidiagonalised as
      // Theta^H), pivoted QR + Jacobi on R^H otherwise (low rank, cheap sweeps)
      int nbd = 0, nbd_max = 0;
      // randomized route: bonds whose smaller compacted side exceeds the sketch
      // (kept rank + oversampling) by a margin; the judge may send some back
      std::vector<int> rank(nb, 0);
      int nrs = 0;
      if (h->opts.svd_mode == TEBD_SVD_RSVD && !h->unnormalized) {
        int over = h->rs_oversample, power = h->rs_power;
        std::vector<char> allow(nb, 1);
        bool any = false;
        for (int s = 0; s < nb; ++s) any |= rsvd_candidate(h, cps[s]);
        if (any && h->rs_model && (rc = rsvd_model_choice(h, nb, gates, cps, &over, &power, allow))) return rc;
        const int sketch = h->chi + over;
        for (int s = 0; s < nb; ++s) {
          const int mn = std::min(cps[s].m, cps[s].n);
          rank[s] = std::min(h->chi, mn);
          // the sketch is at most kRsvdMaxSketch wide (its Cholesky stages panels of R in shared memory)
          h->path_h[s] = (allow[s] && rsvd_candidate(h, cps[s]) && mn >= sketch + 16 && sketch <= kRsvdMaxSketch)
                             ? kPathRsvd
                             : kPathQRJ;
          nrs += h->path_h[s] == kPathRsvd;
        }
        h->stats.rsvd_skipped += std::count(allow.begin(), allow.end(), 0);
        if (nrs) {
          ++h->stats.rsvd_batches;
          h->stats.rsvd_oversample_sum += over;
          h->stats.rsvd_power_sum += power;
          std::vector<char> tried(nb, 0);
          for (int s = 0; s < nb; ++s) tried[s] = h->path_h[s] == kPathRsvd;
          if ((rc = run_rsvd(h, nb, cps, h->path_h, rank, sketch, power))) return rc;
          // with the model: the bonds its sketch did not pass the judge get one more
          // sketch, the conservative (p, q) = (128, 3), before the full SVD
          const int sk2 = h->chi + kRsvdRetryP;
          if (h->rs_model && (over < kRsvdRetryP || power < kRsvdRetryQ) && sk2 <= kRsvdMaxSketch) {
            int again = 0;
            for (int s = 0; s < nb; ++s)
              if (tried[s] && h->path_h[s] != kPathRsvd && std::min(cps[s].m, cps[s].n) >= sk2 + 16) {
                h->path_h[s] = kPathRsvd;
                ++again;
              }
            h->stats.rsvd_retries += again;
            if (again && (rc = run_rsvd(h, nb, cps, h->path_h, rank, sk2, kRsvdRetryQ))) return rc;
            h->stats.rsvd_updates -= again;    // counted once per bond,
            h->stats.rsvd_fallbacks -= again;  // and a fallback only if the second sketch failed too
          }
        }
      }
      // default routing: the bidiagonal route from 64 columns when the batch holds
      // a saturated bond (all chi of its Lambda in use: the gate fills Theta's
      // spectrum, rank ~ n, where the bidiagonal route's fixed O(n^3) is ~8x
      // cheaper than Jacobi sweeps; the batch's other bonds ride along in the same
      // launches) or a bond beyond kQrjMaxDim; a batch of unsaturated Thetas up to
      // kQrjMaxDim columns keeps the QR route, whose cost follows the numerical
      // rank (the chi = 128 run's steps 1..20, mean 177 columns: 1.30x faster than
      // bidiagonalising from 64 columns).  Mixing the routes in one batch would
      // serialise them (the QR batch, then the bidiagonal one).  A batch that took
      // the randomized route holds saturated bonds.
      bool full_batch = nrs > 0;
      for (int s = 0; s < nb; ++s) {
        const int mn = std::min(cps[s].m, cps[s].n);
        if (mn >= kBidiagMinDim && std::max(cps[s].m, cps[s].n) <= kBidiagMaxDim &&
            (cps[s].r1 >= h->chi || mn > kQrjMaxDim))
          full_batch = true;
      }
      for (int s = 0; s < nb; ++s) {
        if (nrs && h->path_h[s] != kPathQRJ) {  // randomized route, or its fallback to the full SVD
          if (h->path_h[s] != kPathRsvd) {
            const int mn = std::min(cps[s].m, cps[s].n), mx = std::max(cps[s].m, cps[s].n);
            ++nbd;
            nbd_max = std::max(nbd_max, mx);
            h->stats.gebrd_flops += 16.0 * mx * (double)mn * mn - 16.0 / 3.0 * (double)mn * mn * mn;
          }
          continue;
        }
        const int mn = std::min(cps[s].m, cps[s].n), mx = std::max(cps[s].m, cps[s].n);
        const bool bd = mx > kBidiagMaxDim                   ? false
                        : h->opts.svd_mode == TEBD_SVD_BIDIAG ? mn >= 2
                        : h->opts.svd_mode == TEBD_SVD_QRJ    ? false
                                                              : mn >= kBidiagMinDim && full_batch;
        h->path_h[s] = !bd ? kPathQRJ : (cps[s].m >= cps[s].n ? kPathBidiag : kPathBidiagT);
        if (bd) {
          ++nbd;
          nbd_max = std::max(nbd_max, mx);
          h->stats.gebrd_flops += 16.0 * mx * (double)mn * mn - 16.0 / 3.0 * (double)mn * mn * mn;
        }
      }
      h->stats.bidiag_updates += nbd;
      CK(cudaMemcpyAsync(h->path_d, h->path_h.data(), sizeof(int) * nb, cudaMemcpyHostToDevice,
                         h->stream),
         "upload SVD routes");
      int nqr = 0;
      for (int s = 0; s < nb; ++s) nqr += h->path_h[s] == kPathQRJ;
      if (nqr > 0 && (rc = run_qrj(h, nb, nmax))) return rc;
      if (nbd > 0 && (rc = run_bidiag(h, nb, nbd_max))) return rc;
    }
    if (h->unnormalized && (rc = launch_unit_norm(h, nb))) return rc;
    if ((rc = launch_dense_finish(h, nb))) return rc;
  } else {
    if ((rc = run_nc_batch(h, nb, links, nullptr))) return rc;
  }
  double *t_pin = (double *)(pin + kPinTrunc);
  int *f_pin = (int *)(pin + kPinFlags);
  CK(cudaMemcpyAsync(t_pin, h->truncerr_d, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream),
     "read truncerr");
  CK(cudaMemcpyAsync(f_pin + 4, h->status_d, sizeof(int) * 4, cudaMemcpyDeviceToHost, h->stream),
     "read status");
  f_pin[8] = 0;
  if (h->tc_err)  // a tensor-core product of the batch whose pipeline wait expired
    CK(cudaMemcpyAsync(f_pin + 8, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "read tensor-core flag");
  if (h->profiling) cudaEventRecord(h->ev[3], h->stream);
  CK(cudaStreamSynchronize(h->stream), "bond batch");
  for (int s = 0; s < nb; ++s) truncerr[s] = t_pin[s];
  if (h->profiling) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]) == cudaSuccess) h->stats.batch_ms += ms;
    tc_collect(h);
  }
  h->stats.updates += nb;
  if ((rc = jacobi_collect(h))) return rc;
  if (f_pin[8]) {
    cudaMemsetAsync(h->tc_err, 0, sizeof(int), h->stream);
    return set_error(h, TEBD_ERR_CUDA, "a tensor-core pipeline wait timed out");
  }
  if (f_pin[4] & 1) return set_error(h, TEBD_ERR_NONFINITE, "non-finite value in Theta or sigma");
  if (f_pin[5]) return set_error(h, TEBD_ERR_NC_BLOCKS, "charge label outside the block range");
  return TEBD_OK;
}

namespace tebd {
// one batch of at most nslots non-overlapping bonds (the autotuner's trials)
int run_bond_batch(tebd_handle *h, int nb, const int *links, const double *const *gates, double *truncerr) {
  return run_batch(h, nb, links, gates, truncerr);
}
}  // namespace tebd

static int apply_bonds_impl(tebd_handle *h, int nbonds, const int *links,
                            const double *const *gates, double *truncerr) {
  if (nbonds < 0 || (nbonds > 0 && (!links || !gates || !truncerr))) return TEBD_ERR_ARG;
  for (int k = 0; k < nbonds; ++k) {
    if (links[k] < 1 || links[k] > h->L - 1)
      return set_error(h, TEBD_ERR_ARG, "bond link out of range 1..L-1");
    if (!gates[k]) return set_error(h, TEBD_ERR_ARG, "null gate");
    for (int q = 0; q < k; ++q)
      if (abs(links[k] - links[q]) < 2)
        return set_error(h, TEBD_ERR_ARG, "batched bonds must not share a site");
  }
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  for (int c = 0; c < nbonds; c += h->nslots) {
    const int nb = std::min(h->nslots, nbonds - c);
    const int rc = run_batch(h, nb, links + c, gates + c, truncerr + c);
    if (rc) return rc;
  }
  return TEBD_OK;
}

extern "C" int tebd_apply_bonds(tebd_handle *h, int nbonds, const int *links,
                                const double *const *gates, double *truncerr) {
  if (!h) return TEBD_ERR_ARG;
  return apply_bonds_impl(h, nbonds, links, gates, truncerr);
}

static int one_bond(tebd_handle *h, int link, const double *op2, bool real, double *truncerr,
                    int want_mode) {
  if (!h || !op2 || !truncerr) return TEBD_ERR_ARG;
  if (h->mode != want_mode)
    return set_error(h, TEBD_ERR_STATE,
                     want_mode == TEBD_MODE_NC ? "TwoSiteOpNC needs a TEBD_MODE_NC handle"
                                               : "TwoSiteOp needs a TEBD_MODE_DENSE handle");
  const int d2 = h->d * h->d;
  std::vector<double> tmp;
  const double *g = op2;
  if (real) {  // ThetaOperation_r: the real gate enters as (op, 0)
    tmp.assign((size_t)2 * d2 * d2, 0.0);
    for (int e = 0; e < d2 * d2; ++e) tmp[2 * e] = op2[e];
    g = tmp.data();
  }
  return apply_bonds_impl(h, 1, &link, &g, truncerr);
}

extern "C" int tebd_two_site_op(tebd_handle *h, int link, const double *op2, double *truncerr) {
  return one_bond(h, link, op2, false, truncerr, TEBD_MODE_DENSE);
}
extern "C" int tebd_two_site_op_r(tebd_handle *h, int link, const double *op2, double *truncerr) {
  return one_bond(h, link, op2, true, truncerr, TEBD_MODE_DENSE);
}
extern "C" int tebd_two_site_op_nc(tebd_handle *h, int link, const double *op2, double *truncerr) {
  return one_bond(h, link, op2, false, truncerr, TEBD_MODE_NC);
}
extern "C" int tebd_two_site_op_nc_r(tebd_handle *h, int link, const double *op2,
                                     double *truncerr) {
  return one_bond(h, link, op2, true, truncerr, TEBD_MODE_NC);
}

// Sweep structure of TrotterStep2ndOrder (:82-114) and TrotterStep5thOrder (:200-252):
// 2nd order: odd, even, odd links with gate Udt(link);
// Forest-Ruth: odd,even,odd,even,odd,even,odd with gate Udt(2(link-1)+pick).
extern "C" int tebd_trotter_step(tebd_handle *h, int order, int n_gates, const double *const *gates,
                                 double *total_truncerr) {
  if (!h || !gates || !total_truncerr) return TEBD_ERR_ARG;
  if (order != 2 && order != 5)
    return set_error(h, TEBD_ERR_ARG, "trotter order must be 2 or 5 (Forest-Ruth)");
  const int L = h->L;
  const int need = order == 2 ? L - 1 : 2 * (L - 2) + 2;
  if (n_gates < need) return set_error(h, TEBD_ERR_ARG, "too few gates for this Trotter order");
  static const int pick5[7] = {1, 1, 2, 2, 2, 1, 1};
  const int nsweeps = order == 2 ? 3 : 7;
  std::vector<int> links;
  std::vector<const double *> gp;
  std::vector<double> te;
  double total = 0.0;
  for (int s = 0; s < nsweeps; ++s) {
    links.clear();
    gp.clear();
    for (int link = (s % 2 == 0) ? 1 : 2; link <= L - 1; link += 2) {
      links.push_back(link);
      const int gi = order == 2 ? link : 2 * (link - 1) + pick5[s];
      gp.push_back(gates[gi - 1]);
    }
    te.assign(links.size(), 0.0);
    const int rc = apply_bonds_impl(h, (int)links.size(), links.data(), gp.data(), te.data());
    if (rc) return rc;
    for (double v : te) total = total + v;
  }
  *total_truncerr = total;
  return TEBD_OK;
}

extern "C" int tebd_set_profiling(tebd_handle *h, int on) {
  if (!h) return TEBD_ERR_ARG;
  h->profiling = on ? 1 : 0;
  return TEBD_OK;
}

extern "C" int tebd_get_stats(tebd_handle *h, tebd_stats *st) {
  if (!h || !st) return TEBD_ERR_ARG;
  *st = h->stats;
  st->kernel_launches = h->launches;
  return TEBD_OK;
}

extern "C" int tebd_reset_stats(tebd_handle *h) {
  if (!h) return TEBD_ERR_ARG;
  memset(&h->stats, 0, sizeof(h->stats));
  return TEBD_OK;
}

extern "C" int tebd_measure_fp64_peak(int device, double *tflops) {
  if (!tflops) return TEBD_ERR_ARG;
  return tebd::measure_fp64_peak(device, tflops);
}

extern "C" void *tebd_get_stream(tebd_handle *h) { return h ? (void *)h->stream : nullptr; }

// ---------------------------------------------------------------------------
// Swapping, the periodic-boundary Trotter step, CanonicalFormAllNC
// ---------------------------------------------------------------------------
// SWAP in the gates' order: Op2((i-1)d+j, (k-1)d+l) = delta(i,l) delta(j,k)
static std::vector<double> swap_gate(int d) {
  const int d2 = d * d;
  std::vector<double> g((size_t)2 * d2 * d2, 0.0);
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) g[2 * ((size_t)(i * d + j) + (size_t)d2 * (j * d + i))] = 1.0;
  return g;
}

// Swapping (local_operations_module.f90:651-689): SwapTheta exchanges the two
// physical indices of the unnormalised Theta, which equals applying SWAP as the
// gate; the SVD then runs without ReshapeTheta's 1/||Theta||, as Swapping calls
// SVDTruncation directly (truncerr = |1 - sum of kept S^2| of the raw Theta).
// NC mode: SwappingNC (:1966-2095) -- SwapThetaNC moves the allowed entries
// (i, j) to (j, i), which is SWAP through ThetaOperationNC when every local
// number lies in [0, maxFilling] (enforced for both NC forms), and RenormThetaNC
// is skipped the same way.
extern "C" int tebd_swapping(tebd_handle *h, int link, double *truncerr) {
  if (!h || !truncerr) return TEBD_ERR_ARG;
  const std::vector<double> g = swap_gate(h->d);
  const double *gp = g.data();
  h->unnormalized = 1;
  const int rc = apply_bonds_impl(h, 1, &link, &gp, truncerr);
  h->unnormalized = 0;
  return rc;
}

// Kept-rank form: discarded-weight bound per bond update (0 = the reference's
// rule, keep chi values above the 1e-15 guard).
extern "C" int tebd_set_rank_bound(tebd_handle *h, double bound) {
  if (!h) return TEBD_ERR_ARG;
  if (!(bound >= 0.0 && bound < 1.0)) return set_error(h, TEBD_ERR_ARG, "rank bound must lie in [0, 1)");
  h->rank_bound = bound;
  return TEBD_OK;
}

// TrotterStep2ndOrderPBC (propagation_module.f90:116-198) and
// TrotterStep5thOrderPBC (:254-614); in NC mode TrotterStep2ndOrderPBCNC
// (:1019-1186) and TrotterStep5thOrderPBCNC (:1244-1940), the same sequences with
// TwoSiteOpNC and SwappingNC.  gates[g-1] = Udt(g) in the periodic layout
// of NEWConstructPropagators.  The edge gate acts on bond 1 between a swap of
// site L down to position 2 and the swap back; same-parity bulk bonds are
// batched; truncation errors of every update and swap are summed in the
// reference's order.
extern "C" int tebd_trotter_step_pbc(tebd_handle *h, int order, int n_gates, const double *const *gates,
                                     double *total_truncerr) {
  if (!h || !gates || !total_truncerr) return TEBD_ERR_ARG;
  if (order != 2 && order != 5) return set_error(h, TEBD_ERR_ARG, "periodic boundaries: order must be 2 or 5");
  const int L = h->L;
  if (L < 3) return set_error(h, TEBD_ERR_ARG, "periodic boundaries need L >= 3");
  const int need = order == 2 ? L : (L % 2 == 1 ? 3 * L : 2 * L);
  if (n_gates < need)
    return set_error(h, TEBD_ERR_ARG, order == 2 ? "periodic 2nd order needs L gates (Udt(L) = edge)"
                                                  : "periodic Forest-Ruth needs 3L gates (odd L) or 2L (even L)");
  for (int g = 0; g < need; ++g)
    if (!gates[g]) return set_error(h, TEBD_ERR_ARG, "NULL gate");
  double total = 0.0;
  std::vector<int> links;
  std::vector<const double *> gp;
  std::vector<double> te;
  // bonds first, first+2, ..., L-1 with Udt(base + step * (link - first0)) style indices
  auto sweep = [&](int first, int (*gidx)(int, int, int), int v) -> int {
    links.clear();
    gp.clear();
    for (int link = first; link <= L - 1; link += 2) {
      links.push_back(link);
      gp.push_back(gates[gidx(link, L, v) - 1]);
    }
    te.assign(links.size(), 0.0);
    const int rc = apply_bonds_impl(h, (int)links.size(), links.data(), gp.data(), te.data());
    for (double x : te) total = total + x;
    return rc;
  };
  auto edge = [&](int g) -> int {
    int rc;
    for (int i = L - 1; i >= 2; --i) {
      double t = 0.0;
      if ((rc = tebd_swapping(h, i, &t))) return rc;
      total = total + t;
    }
    double t = 0.0;
    const double *ge = gates[g - 1];
    const int link = 1;
    if ((rc = apply_bonds_impl(h, 1, &link, &ge, &t))) return rc;
    total = total + t;
    for (int i = 2; i <= L - 1; ++i) {
      double t2 = 0.0;
      if ((rc = tebd_swapping(h, i, &t2))) return rc;
      total = total + t2;
    }
    return TEBD_OK;
  };
  int rc = TEBD_OK;
#define PBC_DO(x) \
  if ((rc = (x))) return rc
  if (order == 2) {
    auto same = [](int link, int, int) { return link; };
    PBC_DO(sweep(1, same, 0));
    if (L % 2 == 1) PBC_DO(sweep(2, same, 0));
    PBC_DO(edge(L));
    PBC_DO(sweep(2, same, 0));
    PBC_DO(sweep(1, same, 0));
  } else if (L % 2 == 1) {
    // odd L: odd bonds Udt(3(i-1)+v), even bonds Udt(2+3(i-2)+v), edge Udt(3(L-1)+v)
    auto odd = [](int i, int, int v) { return 3 * (i - 1) + v; };
    auto even = [](int i, int, int v) { return 2 + 3 * (i - 2) + v; };
    const int e0 = 3 * (L - 1);
    // Forest-Ruth on the even bonds and the edge, nested in each even half-step
    auto nested = [&](int a, int b, int ea, int eb) -> int {
      int r;
      if ((r = sweep(2, even, a))) return r;
      if ((r = edge(e0 + ea))) return r;
      if ((r = sweep(2, even, b))) return r;
      if ((r = edge(e0 + eb))) return r;
      if ((r = sweep(2, even, b))) return r;
      if ((r = edge(e0 + ea))) return r;
      return sweep(2, even, a);
    };
    PBC_DO(sweep(1, odd, 1));
    PBC_DO(nested(1, 2, 1, 2));
    PBC_DO(sweep(1, odd, 2));
    PBC_DO(nested(3, 4, 2, 3));
    PBC_DO(sweep(1, odd, 2));
    PBC_DO(nested(1, 2, 1, 2));
    PBC_DO(sweep(1, odd, 1));
  } else {
    // even L: bond i Udt(2(i-1)+v), edge Udt(2(L-1)+v); the edge commutes with the even bonds
    auto both = [](int i, int, int v) { return 2 * (i - 1) + v; };
    const int e0 = 2 * (L - 1);
    PBC_DO(sweep(1, both, 1));
    PBC_DO(edge(e0 + 1));
    PBC_DO(sweep(2, both, 1));
    PBC_DO(sweep(1, both, 2));
    PBC_DO(edge(e0 + 2));
    PBC_DO(sweep(2, both, 2));
    PBC_DO(sweep(1, both, 2));
    PBC_DO(edge(e0 + 1));
    PBC_DO(sweep(2, both, 1));
    PBC_DO(sweep(1, both, 1));
  }
#undef PBC_DO
  *total_truncerr = total;
  return TEBD_OK;
}

// CanonicalFormAllNC (propagation_module.f90:1943-1983, no internal degrees of
// freedom): TwoSiteOpNC with the identity gate on links 1..L-1, then L-1..1, one
// bond at a time (each depends on the previous one).
extern "C" int tebd_canonical_form_all_nc(tebd_handle *h) {
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_NC) return set_error(h, TEBD_ERR_STATE, "CanonicalFormAllNC needs a TEBD_MODE_NC handle");
  const int d2 = h->d * h->d;
  std::vector<double> eye((size_t)2 * d2 * d2, 0.0);
  for (int k = 0; k < d2; ++k) eye[2 * ((size_t)k + (size_t)d2 * k)] = 1.0;
  const double *gp = eye.data();
  for (int pass = 0; pass < 2; ++pass)
    for (int q = 1; q <= h->L - 1; ++q) {
      const int link = pass == 0 ? q : h->L - q;
      double t = 0.0;
      const int rc = apply_bonds_impl(h, 1, &link, &gp, &t);
      if (rc) return rc;
    }
  return TEBD_OK;
}
