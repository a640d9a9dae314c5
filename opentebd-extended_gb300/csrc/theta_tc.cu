// theta_tc.cu -- FormTheta (VidalCore_v_2.0/local_operations_module.f90:184-211)
// as one batched complex product on the tensor cores.
//
// For every bond of the batch the two factors of Theta are gathered on the kept
// (compacted) indices into the slot's aux buffer, column-major and zero-filled to
// the batch's largest sizes:
//   A (m x r1): A[i*r0 + a', g'] = l0(a) G1(a, i, g),          a = idx0[a'], g = idx1[g']
//   B (r1 x n): B[g', j*r2 + b'] = l1(g) G2(g, j, b) l2(b),    b = idx2[b']
// and Theta = A B is written straight into the slot's X (m x n, ld m) -- the
// column order j*r2 + b' is the permuted order ReshapeTheta leaves, so nothing is
// moved afterwards.  The product runs in the handle's theta form: 3xTF32 (the
// split-precision form, ~FP32 accuracy) or S bf16 digit planes (S = 7: FP64
// class).  ThetaOperation, the norm and the SVD follow unchanged.
#include <stddef.h>

#include "tc_gemm.cuh"

namespace tebd {

int tc_reserve(tebd_handle *h, size_t bytes) {
  if (!h->tc_err) {
    int rc = check_cuda(h, cudaMalloc(&h->tc_err, sizeof(int)), "alloc tensor-core flag");
    if (rc) return rc;
    rc = check_cuda(h, cudaMemsetAsync(h->tc_err, 0, sizeof(int), h->stream), "clear tensor-core flag");
    if (rc) return rc;
  }
  if (bytes <= h->tc_ws_bytes) return TEBD_OK;
  int rc = check_cuda(h, cudaStreamSynchronize(h->stream), "tensor-core workspace");
  if (rc) return rc;
  cudaFree(h->tc_ws);
  h->tc_ws = nullptr;
  h->tc_ws_bytes = 0;
  rc = check_cuda(h, cudaMalloc(&h->tc_ws, bytes), "alloc tensor-core workspace");
  if (rc) return rc;
  h->tc_ws_bytes = bytes;
  return TEBD_OK;
}

void tc_events(tebd_handle *h, double flops, cudaEvent_t *e0, cudaEvent_t *e1) {
  *e0 = *e1 = nullptr;
  if (!h->profiling) return;
  const size_t need = 2 * (size_t)(h->tc_ev_used + 1);
  while (h->tc_ev.size() < need) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      (void)cudaGetLastError();
      return;
    }
    h->tc_ev.push_back(e);
  }
  h->tc_ev_flops.resize(h->tc_ev.size() / 2);
  *e0 = h->tc_ev[2 * h->tc_ev_used];
  *e1 = h->tc_ev[2 * h->tc_ev_used + 1];
  h->tc_ev_flops[h->tc_ev_used] = flops;
  ++h->tc_ev_used;
}

void tc_collect(tebd_handle *h) {
  for (int i = 0; i < h->tc_ev_used; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->tc_ev[2 * i], h->tc_ev[2 * i + 1]) == cudaSuccess) {
      h->stats.tc_ms += ms;
      h->stats.tc_launches++;
      h->stats.tc_mma_flops += h->tc_ev_flops[i];
    }
  }
  (void)cudaGetLastError();
  h->tc_ev_used = 0;
}

void tc_free(tebd_handle *h) {
  for (cudaEvent_t e : h->tc_ev) cudaEventDestroy(e);
  h->tc_ev.clear();
  h->tc_ev_used = 0;
  cudaFree(h->tc_ws);
  cudaFree(h->tc_err);
  h->tc_ws = nullptr;
  h->tc_err = nullptr;
  h->tc_ws_bytes = 0;
}

int tc_check(tebd_handle *h) {
  if (!h->tc_err) return TEBD_OK;
  int e = 0;
  int rc = check_cuda(h, cudaMemcpyAsync(&e, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream),
                      "read tensor-core flag");
  if (rc) return rc;
  rc = check_cuda(h, cudaStreamSynchronize(h->stream), "read tensor-core flag");
  if (rc) return rc;
  if (e) {
    cudaMemsetAsync(h->tc_err, 0, sizeof(int), h->stream);
    return set_error(h, TEBD_ERR_CUDA, "a tensor-core pipeline wait timed out");
  }
  return TEBD_OK;
}

namespace {

__global__ void __launch_bounds__(256) k_theta_operands(const double2 *__restrict__ gam,
                                                        const double *__restrict__ lam,
                                                        const int *__restrict__ links, const Slot *slots, int chi,
                                                        int d, int m_max, int r1_max, int n_max) {
  const int s = blockIdx.y;
  const Compact cp = *slots[s].cp;
  const int link = links[s];
  const size_t csz = (size_t)chi * d * chi;
  const double2 *G1 = gam + (size_t)(link - 1) * csz;
  const double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l1 = lam + (size_t)link * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  const int *idx0 = slots[s].idx0, *idx1 = slots[s].idx1, *idx2 = slots[s].idx2;
  double2 *A = slots[s].aux;
  double2 *B = A + (size_t)m_max * r1_max;
  const size_t na = (size_t)m_max * r1_max, total = na + (size_t)r1_max * n_max;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (e < na) {
      const int r = (int)(e % m_max), gk = (int)(e / m_max);
      if (r < cp.m && gk < cp.r1) {
        const int i = r / cp.r0, a = idx0[r - i * cp.r0], g = idx1[gk];
        v = cscale(G1[a + (size_t)chi * i + (size_t)chi * d * g], l0[a]);
      }
      A[e] = v;
    } else {
      const size_t f = e - na;
      const int gk = (int)(f % r1_max), c = (int)(f / r1_max);
      if (gk < cp.r1 && c < cp.n) {
        const int j = c / cp.r2, b = idx2[c - j * cp.r2], g = idx1[gk];
        v = cscale(G2[g + (size_t)chi * j + (size_t)chi * d * b], l1[g] * l2[b]);
      }
      B[f] = v;
    }
  }
}

}  // namespace

// Theta of the batch on the tensor cores; returns -1 (nothing launched) when a
// dimension of the batch is zero, so that the caller forms it on the CUDA cores.
int launch_theta_tc(tebd_handle *h, int nb) {
  std::vector<Compact> cp(nb);
  int rc = check_cuda(h, cudaMemcpyAsync(cp.data(), h->cp_d, sizeof(Compact) * nb, cudaMemcpyDeviceToHost,
                                         h->stream),
                      "read compaction");
  if (rc) return rc;
  if ((rc = check_cuda(h, cudaStreamSynchronize(h->stream), "read compaction"))) return rc;
  int m_max = 0, n_max = 0, r1_max = 0;
  for (const Compact &c : cp) {
    m_max = std::max(m_max, c.m);
    n_max = std::max(n_max, c.n);
    r1_max = std::max(r1_max, c.r1);
  }
  // small products (early, low-rank updates) stay on the CUDA cores: packing and
  // the extra synchronisation cost more than the tiled FP64 kernel there
  if (m_max == 0 || n_max == 0 || r1_max == 0 || (double)m_max * n_max * r1_max < (double)(1 << 21)) return -1;
  const Slot &s0 = h->slots[0];
  const long long aux_stride = nb > 1 ? (long long)(h->slots[1].aux - s0.aux) : 0;
  const size_t total = (size_t)m_max * r1_max + (size_t)r1_max * n_max;
  unsigned gx = (unsigned)std::min<size_t>((total + 255) / 256, 2048);
  k_theta_operands<<<dim3(gx, nb), 256, 0, h->stream>>>(h->gam, h->lam, h->links_d, h->slots_d, h->chi, h->d,
                                                         m_max, r1_max, n_max);
  TEBD_LAUNCHED(h);
  ZProd z = {};
  z.a = s0.aux;
  z.a_stride = aux_stride;
  z.lda = m_max;
  z.b = s0.aux + (size_t)m_max * r1_max;
  z.b_stride = aux_stride;
  z.ldb = r1_max;
  z.nprob = nb;
  z.m = m_max;
  z.n = n_max;
  z.k = r1_max;
  z.form = h->theta_form;
  z.rs = 1;
  z.cs = 0;  // column stride = the bond's own m
  z.m_d = &h->cp_d[0].m;
  z.n_d = &h->cp_d[0].n;
  z.dim_stride = (int)(sizeof(Compact) / sizeof(int));
  z.alpha = 1.0;
  z.optr = reinterpret_cast<const unsigned char *>(h->slots_d) + offsetof(Slot, X);
  z.optr_stride = (int)sizeof(Slot);
  if ((rc = tc_reserve(h, zprod_ws_bytes(z)))) return rc;
  tc_events(h, zprod_mma_flops(z, nb), &z.ev0, &z.ev1);
  if ((rc = check_cuda(h, zprod_run(z, h->tc_ws, h->tc_err, h->stream), "tensor-core Theta"))) return rc;
  h->launches += zprod_oz(z.form) ? 5 : 3;  // packs (+ exponent passes) and the product
  return TEBD_OK;
}

}  // namespace tebd

using namespace tebd;

extern "C" int tebd_set_theta_form(tebd_handle *h, int form) {
  if (!h) return TEBD_ERR_ARG;
  if (!(form == 0 || form == kTc3xTF32 || (form >= 103 && form <= 100 + kOzMaxS)))
    return set_error(h, TEBD_ERR_ARG, "theta form must be 0, 3 (3xTF32) or 103..107 (bf16 digit planes)");
  if (h->mode != TEBD_MODE_DENSE && form != 0 && !zprod_oz(form))
    return set_error(h, TEBD_ERR_STATE, "NC handles take theta form 0 or 103..107 (3xTF32 is for dense handles)");
  h->theta_form = form;
  return TEBD_OK;
}
