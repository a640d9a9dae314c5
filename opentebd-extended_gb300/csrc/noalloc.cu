// noalloc.cu -- tebd_two_site_op_noalloc: the dense two-site update on one bond
// of a caller-owned device chain, with no device or host allocation at all.
//
// Who needs it, and why they cannot allocate:
//  * a host whose device memory is handed out by a fixed pool sized at start-up
//    (a Fortran code that reserves its whole budget at once, or a process sharing
//    a GPU under a hard quota): a further cudaMalloc either fails or breaks the
//    pool's accounting;
//  * a host that keeps its own device-resident chain and cannot own a library
//    handle, which allocates SVD workspaces for every bond of a sweep (~1.3 GB at
//    d = 5, chi = 128) when it is created;
//  * a time-critical loop that overlaps other work on other streams: cudaFree
//    synchronises the whole device and cudaMalloc can stall it, so such a loop
//    keeps allocation out of its steady state.
// They pass their own device Gammas/Lambdas/gate; every temporary of the update
// lives in the one file-scope array below.
//
// Scratch: kNoAllocMaxN = 256 columns (d*chi <= 256, chi <= 256), about 2.1 MB,
// held by every GPU that loads the library until the process exits.  All calls on
// a device share it and it keeps the previous call's contents, so the counters
// and flags that must start at zero are cleared at the start of each call, and
// two calls that overlap on the GPU (different streams or host threads) race on
// it: serialise them.
//
// Host code cannot use `g_noalloc_scratch` as a device address (it names a host
// shadow); the device address is fetched once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on that
// device.  Make that first call before any stream capture begins.  The address
// is kept for the life of the process: after cudaDeviceReset on a device, this
// entry point must not be called again on that device.
//
// Errors: a CUDA error already pending on the calling thread is left in place and
// the call returns TEBD_ERR_CUDA without touching the chain.  Launch errors are
// checked before any kernel writes the caller's Gammas or Lambdas, and a
// non-finite Theta or singular value leaves them unmodified (TEBD_ERR_NONFINITE).
#include <string.h>

#include <mutex>

#include "tebd_internal.cuh"

namespace tebd {

cudaError_t raw_dense_prepare(cudaStream_t st, double2 *gam, const double *lam, const int *links_d,
                              Slot *slots_d, JacobiProblem<double> *jp, double *nrm_part, double *nrm,
                              int *status, int chi, int d);
cudaError_t raw_dense_finish(cudaStream_t st, double2 *gam, double *lam, const int *links_d,
                             Slot *slots_d, const double *nrm, double *truncerr, int *status, int chi,
                             int d);
void raw_jacobi_init(cudaStream_t st, int *rot, int *done, int *sweeps);
void raw_jacobi_sweep(cudaStream_t st, const JacobiProblem<double> *probs_d, int *rot, int *done,
                      int *sweeps, int *pending, unsigned long long *counters, int nmax,
                      double tol);

namespace {

constexpr int kNoAllocMaxN = 256;
constexpr int kNoAllocMaxChi = 256;
constexpr int kNoAllocMaxDevices = 64;
constexpr int kNoAllocSweepCap = 60;

constexpr size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// byte offsets inside the scratch array
constexpr size_t kOffX = 0;
constexpr size_t kOffV = kOffX + al256(sizeof(double2) * kNoAllocMaxN * kNoAllocMaxN);
constexpr size_t kOffS = kOffV + al256(sizeof(double2) * kNoAllocMaxN * kNoAllocMaxN);
constexpr size_t kOffPerm = kOffS + al256(sizeof(double) * kNoAllocMaxN);
constexpr size_t kOffIdx = kOffPerm + al256(sizeof(int) * kNoAllocMaxN);
constexpr size_t kOffCp = kOffIdx + al256(sizeof(int) * 5 * kNoAllocMaxChi);
constexpr size_t kOffSlot = kOffCp + al256(sizeof(Compact));
constexpr size_t kOffProb = kOffSlot + al256(sizeof(Slot));
constexpr size_t kOffLink = kOffProb + al256(sizeof(JacobiProblem<double>));
constexpr size_t kOffNormPart = kOffLink + al256(sizeof(int));
constexpr size_t kOffNorm = kOffNormPart + al256(sizeof(double) * kNormParts);
constexpr size_t kOffTrunc = kOffNorm + al256(sizeof(double));
constexpr size_t kOffState = kOffTrunc + al256(sizeof(double));  // rot, done, sweeps, pending
constexpr size_t kOffCounters = kOffState + al256(sizeof(int) * 4);
constexpr size_t kOffStatus = kOffCounters + al256(sizeof(unsigned long long) * 4);
constexpr size_t kScratchBytes = kOffStatus + al256(sizeof(int) * 4);

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_mu;
void *g_base[kNoAllocMaxDevices];

// Device address of the scratch array on the current device (set up once).
int scratch_base(int dev, char **base) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_base[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      (void)cudaGetLastError();
      return TEBD_ERR_CUDA;
    }
    g_base[dev] = p;
  }
  *base = static_cast<char *>(g_base[dev]);
  return TEBD_OK;
}

int fail(cudaError_t e) {
  (void)cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? TEBD_ERR_OOM : TEBD_ERR_CUDA;
}

}  // namespace
}  // namespace tebd

using namespace tebd;

extern "C" int tebd_two_site_op_noalloc(int L, int d, int chi, int link, double *gammas,
                                        double *lambdas, const double *op2, double *truncerr,
                                        void *stream) {
  if (L < 2 || d < 1 || d > 8 || chi < 1 || link < 1 || link > L - 1 || !gammas || !lambdas ||
      !op2 || !truncerr)
    return TEBD_ERR_ARG;
  if (d * chi > kNoAllocMaxN || chi > kNoAllocMaxChi) return TEBD_ERR_ARG;  // beyond the scratch
  // an error left by the caller's earlier work stays theirs: report, do not clear
  if (cudaPeekAtLastError() != cudaSuccess) return TEBD_ERR_CUDA;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(e);
  if (dev < 0 || dev >= kNoAllocMaxDevices) return TEBD_ERR_ARG;
  char *base = nullptr;
  int rc = scratch_base(dev, &base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n = d * chi;

  Slot slot;
  memset(&slot, 0, sizeof(slot));
  slot.X = reinterpret_cast<double2 *>(base + kOffX);
  slot.V = reinterpret_cast<double2 *>(base + kOffV);
  slot.S = reinterpret_cast<double *>(base + kOffS);
  slot.perm = reinterpret_cast<int *>(base + kOffPerm);
  slot.gate = reinterpret_cast<double2 *>(const_cast<double *>(op2));
  int *ix = reinterpret_cast<int *>(base + kOffIdx);
  slot.idx0 = ix;
  slot.idx1 = ix + chi;
  slot.idx2 = ix + 2 * chi;
  slot.inv0 = ix + 3 * chi;
  slot.inv2 = ix + 4 * chi;
  slot.cp = reinterpret_cast<Compact *>(base + kOffCp);
  JacobiProblem<double> prob = {slot.X, slot.V, n, n, n, n, 0.0};
  Slot *slot_d = reinterpret_cast<Slot *>(base + kOffSlot);
  JacobiProblem<double> *prob_d = reinterpret_cast<JacobiProblem<double> *>(base + kOffProb);
  int *link_d = reinterpret_cast<int *>(base + kOffLink);
  double *nrm_part = reinterpret_cast<double *>(base + kOffNormPart);
  double *nrm = reinterpret_cast<double *>(base + kOffNorm);
  double *trunc_d = reinterpret_cast<double *>(base + kOffTrunc);
  int *state = reinterpret_cast<int *>(base + kOffState);
  unsigned long long *counters = reinterpret_cast<unsigned long long *>(base + kOffCounters);
  int *status = reinterpret_cast<int *>(base + kOffStatus);

  // descriptors in, flags and counters cleared (the array keeps the last call's data)
  if ((e = cudaMemcpyAsync(slot_d, &slot, sizeof(slot), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(prob_d, &prob, sizeof(prob), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(link_d, &link, sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(state, 0, sizeof(int) * 4, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * 4, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(status, 0, sizeof(int) * 4, st)) != cudaSuccess)
    return fail(e);

  // Theta, gate, norm: reads the chain, writes only the scratch
  double2 *gam = reinterpret_cast<double2 *>(gammas);
  if ((e = raw_dense_prepare(st, gam, lambdas, link_d, slot_d, prob_d, nrm_part, nrm, status, chi,
                             d)) != cudaSuccess)
    return fail(e);
  Compact cp;
  if ((e = cudaMemcpyAsync(&cp, slot.cp, sizeof(cp), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(e);

  // one-sided Jacobi on the compacted Theta, one launch sequence per sweep
  const double tol = (double)(cp.n > 16 ? cp.n : 16) * 2.220446049250313e-16;
  raw_jacobi_init(st, state, state + 1, state + 2);
  int pending = 1;
  for (int sw = 0; sw < kNoAllocSweepCap && pending; ++sw) {
    raw_jacobi_sweep(st, prob_d, state, state + 1, state + 2, state + 3, counters, cp.n, tol);
    if ((e = cudaPeekAtLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(&pending, state + 3, sizeof(int), cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return fail(e);
  }
  if (pending) return TEBD_ERR_SVD_NOCONV;  // the chain has not been written

  // FormLambda1, FormGamma1/2: the only kernels that write the chain; they skip
  // their writes when the status flag marks a non-finite Theta or sigma
  if ((e = raw_dense_finish(st, gam, lambdas, link_d, slot_d, nrm, trunc_d, status, chi, d)) !=
      cudaSuccess)
    return fail(e);
  int flags[4];
  if ((e = cudaMemcpyAsync(truncerr, trunc_d, sizeof(double), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(flags, status, sizeof(flags), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(e);
  return (flags[0] & 1) ? TEBD_ERR_NONFINITE : TEBD_OK;
}
