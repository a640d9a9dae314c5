// mlp.cu -- the learned part of the learned-rank form: a small FP32 network that
// reads a bond's previous Schmidt spectrum and its gate and predicts the
// post-update spectrum around the cut, trained on spectra the method itself
// produced, with hand-written forward, backward and Adam kernels.
//
// Network (fixed sizes): x (67) -> relu(W1 x + b1) (128) -> relu(W2 h1 + b2) (128)
// -> W3 h2 + b3 (8).  Parameters are one FP32 vector in the order W1, b1, W2, b2,
// W3, b3 (weights row-major: W[o * fan_in + i]).  Samples are stored column by
// column (sample j at x + 67 j).
//   inputs   64 values log10(lambda_k / lambda_0) of the bond's Lambda before the
//            update, at ranks k = floor(j chi / 64), floored at -16 (0 where
//            lambda_0 = 0); then log10 |U - I|_F, log10 |offdiag(U)|_F (floored at
//            -16) and d / 8 for the gate U;
//   outputs  log10(sigma_k / sigma_0) of the normalised Theta's singular values
//            at the relative ranks k / chi of kMlpRanks.
// Loss: mean squared error over the 8 outputs.  Every kernel is deterministic:
// each output element is one thread's fixed-order sum.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "tebd_internal.cuh"

namespace tebd {

namespace {

constexpr int kIn = kMlpIn, kH = kMlpHidden, kOut = kMlpOut;
constexpr size_t kW1 = 0, kB1 = kW1 + (size_t)kH * kIn, kW2 = kB1 + kH, kB2 = kW2 + (size_t)kH * kH,
                 kW3 = kB2 + kH, kB3 = kW3 + (size_t)kOut * kH, kNp = kB3 + kOut;

// out[o, j] = act(sum_i W[o, i] in[i, j] + b[o]); act = relu when relu != 0
__global__ void k_dense_fwd(const float *W, const float *b, const float *in, float *out, int fin, int fout, int n,
                            int relu) {
  const int o = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float *w = W + (size_t)o * fin;
  const float *x = in + (size_t)j * fin;
  float acc = b[o];
  for (int i = 0; i < fin; ++i) acc = fmaf(w[i], x[i], acc);
  out[(size_t)j * fout + o] = relu ? fmaxf(acc, 0.f) : acc;
}

// din[i, j] = (sum_o W[o, i] dout[o, j]) * (act[i, j] > 0): the gradient reaching
// the previous layer's relu output, masked by that relu
__global__ void k_dense_bwd_data(const float *W, const float *dout, const float *act, float *din, int fin, int fout,
                                 int n) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float acc = 0.f;
  for (int o = 0; o < fout; ++o) acc = fmaf(W[(size_t)o * fin + i], dout[(size_t)j * fout + o], acc);
  din[(size_t)j * fin + i] = act[(size_t)j * fin + i] > 0.f ? acc : 0.f;
}

// dW[o, i] = sum_j dout[o, j] in[i, j]; db[o] = sum_j dout[o, j] (one thread per
// weight, fixed sample order)
__global__ void k_dense_bwd_w(const float *dout, const float *in, float *dW, float *db, int fin, int fout, int n) {
  const int o = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > fin) return;
  float acc = 0.f;
  if (i < fin) {
    for (int j = 0; j < n; ++j) acc = fmaf(dout[(size_t)j * fout + o], in[(size_t)j * fin + i], acc);
    dW[(size_t)o * fin + i] = acc;
  } else {
    for (int j = 0; j < n; ++j) acc += dout[(size_t)j * fout + o];
    db[o] = acc;
  }
}

// dY = 2 (Y - T) / (n kOut); loss partials: one thread per sample
__global__ void k_mse(const float *Y, const float *T, float *dY, double *part, int n) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float sc = 2.f / ((float)n * kOut);
  double l = 0.0;
  for (int o = 0; o < kOut; ++o) {
    const float e = Y[(size_t)j * kOut + o] - T[(size_t)j * kOut + o];
    dY[(size_t)j * kOut + o] = sc * e;
    l += (double)e * e;
  }
  part[j] = l;
}

__global__ void k_sum(const double *part, int n, double *out) {  // one thread: fixed order
  if (blockIdx.x || threadIdx.x) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += part[j];
  *out = s / ((double)n * kOut);
}

// Adam (Kingma & Ba 2015): m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
// p -= lr * (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t)) + eps)
__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t np, float lr, float b1, float b2,
                       float c1, float c2, float eps) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= np) return;
  const float gg = g[e];
  const float mm = b1 * m[e] + (1.f - b1) * gg, vv = b2 * v[e] + (1.f - b2) * gg * gg;
  m[e] = mm;
  v[e] = vv;
  p[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// features of the bonds of a batch: Lambda(link) before the update, gate terms
// from the host (3 per bond)
__global__ void k_mlp_features(const double *lam, const int *links, const float *gate_terms, int chi, float *X,
                               int nb) {
  const int s = blockIdx.x;
  if (s >= nb) return;
  const double *l = lam + (size_t)links[s] * chi;
  const double l0 = l[0];
  for (int j = threadIdx.x; j < 64; j += blockDim.x) {
    const int k = (int)((long long)j * chi / 64);
    const double r = l0 > 0.0 ? l[k] / l0 : 0.0;
    X[(size_t)s * kIn + j] = (float)(r > 1e-16 ? log10(r) : -16.0);
  }
  if (threadIdx.x < 3) X[(size_t)s * kIn + 64 + threadIdx.x] = gate_terms[3 * s + threadIdx.x];
}

unsigned long long lcg(unsigned long long &s) {
  s = s * 6364136223846793005ULL + 1442695040888963407ULL;
  return s >> 11;
}

}  // namespace

const double kMlpRanks[kMlpOut] = {0.75, 1.0, 1.125, 1.25, 1.5, 1.75, 2.0, 2.5};

}  // namespace tebd

using namespace tebd;

struct tebd_mlp {
  int device;
  cudaStream_t stream;
  float *p, *g, *m, *v;  // parameters, gradient, Adam moments (kNp each)
  long long step;        // Adam steps taken
  int cap;               // samples the activation buffers hold
  float *x, *t, *h1, *h2, *y, *dy, *d2, *d1;
  double *part, *loss;
  std::string err;
};

namespace tebd {
namespace {

int mlp_fail(tebd_mlp *M, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return TEBD_OK;
  M->err = std::string(what) + ": " + cudaGetErrorString(e);
  (void)cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? TEBD_ERR_OOM : TEBD_ERR_CUDA;
}

void mlp_free_bufs(tebd_mlp *M) {
  for (float **q : {&M->x, &M->t, &M->h1, &M->h2, &M->y, &M->dy, &M->d2, &M->d1}) {
    cudaFree(*q);
    *q = nullptr;
  }
  cudaFree(M->part);
  cudaFree(M->loss);
  M->part = M->loss = nullptr;
  M->cap = 0;
}

int mlp_reserve(tebd_mlp *M, int n) {
  if (n <= M->cap) return TEBD_OK;
  int rc = mlp_fail(M, cudaStreamSynchronize(M->stream), "mlp buffers");
  if (rc) return rc;
  mlp_free_bufs(M);
  const size_t f = sizeof(float);
  cudaError_t e;
  if ((e = cudaMalloc(&M->x, f * kIn * n)) != cudaSuccess || (e = cudaMalloc(&M->t, f * kOut * n)) != cudaSuccess ||
      (e = cudaMalloc(&M->h1, f * kH * n)) != cudaSuccess || (e = cudaMalloc(&M->h2, f * kH * n)) != cudaSuccess ||
      (e = cudaMalloc(&M->y, f * kOut * n)) != cudaSuccess || (e = cudaMalloc(&M->dy, f * kOut * n)) != cudaSuccess ||
      (e = cudaMalloc(&M->d2, f * kH * n)) != cudaSuccess || (e = cudaMalloc(&M->d1, f * kH * n)) != cudaSuccess ||
      (e = cudaMalloc(&M->part, sizeof(double) * n)) != cudaSuccess ||
      (e = cudaMalloc(&M->loss, sizeof(double))) != cudaSuccess) {
    mlp_free_bufs(M);
    return mlp_fail(M, e, "alloc mlp buffers");
  }
  M->cap = n;
  return TEBD_OK;
}

inline unsigned cd(int a, int b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// forward on device inputs X (kIn x n) into M->y; keeps h1, h2 for backward
void mlp_forward_dev(tebd_mlp *M, const float *X, int n, cudaStream_t st) {
  k_dense_fwd<<<dim3(cd(n, 128), kH), 128, 0, st>>>(M->p + kW1, M->p + kB1, X, M->h1, kIn, kH, n, 1);
  k_dense_fwd<<<dim3(cd(n, 128), kH), 128, 0, st>>>(M->p + kW2, M->p + kB2, M->h1, M->h2, kH, kH, n, 1);
  k_dense_fwd<<<dim3(cd(n, 128), kOut), 128, 0, st>>>(M->p + kW3, M->p + kB3, M->h2, M->y, kH, kOut, n, 0);
}

// loss and gradient of the n samples X / T (device) into M->g, M->loss
static void mlp_loss_grad_dev(tebd_mlp *M, const float *X, const float *T, int n, cudaStream_t st) {
  mlp_forward_dev(M, X, n, st);
  k_mse<<<cd(n, 128), 128, 0, st>>>(M->y, T, M->dy, M->part, n);
  k_sum<<<1, 1, 0, st>>>(M->part, n, M->loss);
  k_dense_bwd_w<<<dim3(cd(kH + 1, 128), kOut), 128, 0, st>>>(M->dy, M->h2, M->g + kW3, M->g + kB3, kH, kOut, n);
  k_dense_bwd_data<<<dim3(cd(n, 128), kH), 128, 0, st>>>(M->p + kW3, M->dy, M->h2, M->d2, kH, kOut, n);
  k_dense_bwd_w<<<dim3(cd(kH + 1, 128), kH), 128, 0, st>>>(M->d2, M->h1, M->g + kW2, M->g + kB2, kH, kH, n);
  k_dense_bwd_data<<<dim3(cd(n, 128), kH), 128, 0, st>>>(M->p + kW2, M->d2, M->h1, M->d1, kH, kH, n);
  k_dense_bwd_w<<<dim3(cd(kIn + 1, 128), kH), 128, 0, st>>>(M->d1, X, M->g + kW1, M->g + kB1, kIn, kH, n);
}

int mlp_features_forward(tebd_mlp *M, const double *lam, const int *links, const float *gate_terms_host, int chi,
                         int nb, cudaStream_t st, float *out_host) {
  int rc = mlp_reserve(M, std::max(nb, 1));
  if (rc) return rc;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(M->t, gate_terms_host, sizeof(float) * 3 * nb, cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return mlp_fail(M, e, "upload gate terms");
  k_mlp_features<<<nb, 64, 0, st>>>(lam, links, M->t, chi, M->x, nb);
  mlp_forward_dev(M, M->x, nb, st);
  if ((e = cudaMemcpyAsync(out_host, M->y, sizeof(float) * kOut * nb, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return mlp_fail(M, e, "model forward");
  return TEBD_OK;
}

size_t mlp_param_count() { return kNp; }

}  // namespace tebd

// ---------------------------------------------------------------------------
// C ABI (no counterpart in the reference: the learned part of the learned-rank
// form, which stands in front of SVDTruncation, local_operations_module.f90:322-345)
// ---------------------------------------------------------------------------
extern "C" int tebd_mlp_create(int device, unsigned long long seed, tebd_mlp **out) {
  if (!out) return TEBD_ERR_ARG;
  *out = nullptr;
  tebd_mlp *M = new (std::nothrow) tebd_mlp();
  if (!M) return TEBD_ERR_OOM;
  M->device = device;
  cudaError_t e;
  const size_t b = sizeof(float) * kNp;
  if ((e = cudaSetDevice(device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&M->p, b)) != cudaSuccess || (e = cudaMalloc(&M->g, b)) != cudaSuccess ||
      (e = cudaMalloc(&M->m, b)) != cudaSuccess || (e = cudaMalloc(&M->v, b)) != cudaSuccess) {
    const int rc = e == cudaErrorMemoryAllocation ? TEBD_ERR_OOM : TEBD_ERR_CUDA;
    cudaFree(M->p);
    cudaFree(M->g);
    cudaFree(M->m);
    cudaFree(M->v);
    if (M->stream) cudaStreamDestroy(M->stream);
    (void)cudaGetLastError();
    delete M;
    return rc;
  }
  // He-uniform weights (fan-in), zero biases
  std::vector<float> p(kNp, 0.f);
  unsigned long long st = seed ^ 0x9e3779b97f4a7c15ULL;
  auto fill = [&](size_t off, int fo, int fi) {
    const double a = sqrt(6.0 / fi);
    for (size_t e2 = 0; e2 < (size_t)fo * fi; ++e2)
      p[off + e2] = (float)(a * (2.0 * (double)lcg(st) / 9007199254740992.0 - 1.0));
  };
  fill(kW1, kH, kIn);
  fill(kW2, kH, kH);
  fill(kW3, kOut, kH);
  if ((e = cudaMemcpy(M->p, p.data(), b, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(M->m, 0, b)) != cudaSuccess || (e = cudaMemset(M->v, 0, b)) != cudaSuccess) {
    (void)cudaGetLastError();
    cudaFree(M->p);
    cudaFree(M->g);
    cudaFree(M->m);
    cudaFree(M->v);
    cudaStreamDestroy(M->stream);
    delete M;
    return TEBD_ERR_CUDA;
  }
  *out = M;
  return TEBD_OK;
}

extern "C" int tebd_mlp_destroy(tebd_mlp *M) {
  if (!M) return TEBD_ERR_ARG;
  cudaSetDevice(M->device);
  cudaStreamSynchronize(M->stream);
  mlp_free_bufs(M);
  cudaFree(M->p);
  cudaFree(M->g);
  cudaFree(M->m);
  cudaFree(M->v);
  cudaStreamDestroy(M->stream);
  delete M;
  return TEBD_OK;
}

extern "C" int tebd_mlp_param_count(void) { return (int)kNp; }

extern "C" const char *tebd_mlp_last_error(tebd_mlp *M) { return M ? M->err.c_str() : "null model"; }

extern "C" int tebd_mlp_get_params(tebd_mlp *M, float *params) {
  if (!M || !params) return TEBD_ERR_ARG;
  cudaSetDevice(M->device);
  return mlp_fail(M, cudaMemcpy(params, M->p, sizeof(float) * kNp, cudaMemcpyDeviceToHost), "get params");
}

extern "C" int tebd_mlp_set_params(tebd_mlp *M, const float *params) {
  if (!M || !params) return TEBD_ERR_ARG;
  cudaSetDevice(M->device);
  int rc = mlp_fail(M, cudaMemcpy(M->p, params, sizeof(float) * kNp, cudaMemcpyHostToDevice), "set params");
  if (rc) return rc;
  M->step = 0;  // new parameters: the optimizer starts afresh
  if ((rc = mlp_fail(M, cudaMemset(M->m, 0, sizeof(float) * kNp), "reset moments"))) return rc;
  return mlp_fail(M, cudaMemset(M->v, 0, sizeof(float) * kNp), "reset moments");
}

extern "C" int tebd_mlp_forward(tebd_mlp *M, int n, const float *x, float *y) {
  if (!M || n < 1 || !x || !y) return TEBD_ERR_ARG;
  cudaSetDevice(M->device);
  int rc = mlp_reserve(M, n);
  if (rc) return rc;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(M->x, x, sizeof(float) * kIn * n, cudaMemcpyHostToDevice, M->stream)) != cudaSuccess)
    return mlp_fail(M, e, "upload inputs");
  mlp_forward_dev(M, M->x, n, M->stream);
  if ((e = cudaMemcpyAsync(y, M->y, sizeof(float) * kOut * n, cudaMemcpyDeviceToHost, M->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(M->stream)) != cudaSuccess)
    return mlp_fail(M, e, "forward");
  return TEBD_OK;
}

extern "C" int tebd_mlp_loss_grad(tebd_mlp *M, int n, const float *x, const float *t, double *loss, float *grad) {
  if (!M || n < 1 || !x || !t || !loss || !grad) return TEBD_ERR_ARG;
  cudaSetDevice(M->device);
  int rc = mlp_reserve(M, n);
  if (rc) return rc;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(M->x, x, sizeof(float) * kIn * n, cudaMemcpyHostToDevice, M->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(M->t, t, sizeof(float) * kOut * n, cudaMemcpyHostToDevice, M->stream)) != cudaSuccess)
    return mlp_fail(M, e, "upload samples");
  mlp_loss_grad_dev(M, M->x, M->t, n, M->stream);
  if ((e = cudaMemcpyAsync(loss, M->loss, sizeof(double), cudaMemcpyDeviceToHost, M->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(grad, M->g, sizeof(float) * kNp, cudaMemcpyDeviceToHost, M->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(M->stream)) != cudaSuccess)
    return mlp_fail(M, e, "loss and gradient");
  return TEBD_OK;
}

// Adam over `epochs` passes of minibatches of `batch` samples, in the samples'
// order (deterministic); *loss receives the mean loss of the last epoch.
extern "C" int tebd_mlp_train(tebd_mlp *M, int n, const float *x, const float *t, int epochs, int batch, float lr,
                              double *loss) {
  if (!M || n < 1 || !x || !t || epochs < 1 || batch < 1 || !(lr > 0.f) || !loss) return TEBD_ERR_ARG;
  cudaSetDevice(M->device);
  batch = std::min(batch, n);
  int rc = mlp_reserve(M, n);
  if (rc) return rc;
  cudaStream_t st = M->stream;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(M->x, x, sizeof(float) * kIn * n, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(M->t, t, sizeof(float) * kOut * n, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return mlp_fail(M, e, "upload samples");
  const float b1 = 0.9f, b2 = 0.999f;
  double sum = 0.0;
  int nbat = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    sum = 0.0;
    nbat = 0;
    for (int j0 = 0; j0 < n; j0 += batch) {
      const int nb = std::min(batch, n - j0);
      mlp_loss_grad_dev(M, M->x + (size_t)j0 * kIn, M->t + (size_t)j0 * kOut, nb, st);
      ++M->step;
      const float c1 = 1.f - powf(b1, (float)M->step), c2 = 1.f - powf(b2, (float)M->step);
      k_adam<<<cd((int)kNp, 256), 256, 0, st>>>(M->p, M->g, M->m, M->v, kNp, lr, b1, b2, c1, c2, 1e-8f);
      if (ep == epochs - 1) {
        double l = 0.0;
        if ((e = cudaMemcpyAsync(&l, M->loss, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
          return mlp_fail(M, e, "training");
        sum += l;
        ++nbat;
      }
    }
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess)
    return mlp_fail(M, e, "training");
  *loss = nbat ? sum / nbat : 0.0;
  return TEBD_OK;
}

extern "C" int tebd_set_rsvd_model(tebd_handle *h, tebd_mlp *M, double target) {
  if (!h) return TEBD_ERR_ARG;
  if (M && !(target > 0.0 && target < 1.0))
    return set_error(h, TEBD_ERR_ARG, "rsvd model: target must lie in (0, 1)");
  if (M && M->device != h->device) return set_error(h, TEBD_ERR_ARG, "rsvd model: on another device");
  h->rs_model = M;
  h->rs_target = target;
  return TEBD_OK;
}
