// tune.cu -- the project's autotuner for the launch shapes of the SVD routes.
//
// Three launch parameters set how a batch of bonds maps onto the GPU without
// changing what is computed:
//   * the cluster size of the bidiagonalisation (k_gebrd / k_gebrd_df: one
//     cluster of 1..8 CTAs per bond; more CTAs share each column's passes but
//     fewer bonds run at once);
//   * the team size of the bisection (k_bd_sigma<team>: 1, 2, 4 or 8 lanes
//     evaluate Sturm counts at that many points per step for one value) and the
//     CTAs that share one side of a bond's vector re-orthogonalisation
//     (k_bd_orth, a cluster of 1, 2, 4 or 8);
//   * the panel height of the randomized route's Cholesky (k_rs_chol: 4, 8 or 16
//     rows of R staged in shared memory per panel), the CTAs that share one
//     bond's Cholesky (a cluster of 1..8), and the size below which its
//     recursive blocking factors a diagonal block directly (128 .. 768).
// Without a table the library picks them from occupancy queries and thread
// counts (bidiag.cu, rsvd.cu).  tebd_autotune times candidates on a batch of
// real bonds -- the default choice, then every cluster size, then every team
// size with the best cluster, then every re-orthogonalisation cluster size, then
// (randomized route only) every Cholesky cluster size, panel height and leaf
// size -- restoring the touched
// Gammas, Lambdas and labels after each trial, and keeps the fastest per
// (route, largest compacted dimension rounded up to 64, bonds in the batch
// rounded up to a power of two) in a table per device that every later batch on
// the device consults.  A trial that asked for a shape the launch cannot use
// (a cluster larger than the problem allows or than the GPC holds) is discarded.
#include <cuda_runtime.h>

#include <array>
#include <map>
#include <mutex>
#include <vector>

#include "tebd_internal.cuh"

namespace tebd {
namespace {

struct TuneEntry {
  TuneParams p;
  float us;
};

std::mutex g_mu;
std::map<std::array<int, 4>, TuneEntry> g_table;  // (device, route, n bucket, bonds bucket)

int n_bucket(int n) { return (n + 63) / 64 * 64; }
int nb_bucket(int nb) {
  int b = 1;
  while (b < nb) b <<= 1;
  return b;
}

}  // namespace

TuneParams tune_lookup(tebd_handle *h, int route, int n, int nb) {
  const std::array<int, 3> key = {route, n_bucket(n), nb_bucket(nb)};
  if (h->tune.active) {  // a trial: record the key, use the trial's shape (0 = default)
    bool seen = false;
    for (const auto &k : h->tune.seen) seen |= k == key;
    if (!seen) h->tune.seen.push_back(key);
    return h->tune.force;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  const auto it = g_table.find({h->device, key[0], key[1], key[2]});
  if (it == g_table.end()) return TuneParams{0, 0, 0, 0, 0, 0};
  return it->second.p;
}

void tune_reject(tebd_handle *h) {
  if (h->tune.active) h->tune.rejected = 1;
}

int run_bond_batch(tebd_handle *h, int nb, const int *links, const double *const *gates, double *truncerr);

}  // namespace tebd

using namespace tebd;

namespace {

// The state one batch of bonds writes: Gammas link-1 and link, Lambda row link,
// and (NC) the label rows link.
struct Snapshot {
  char *buf = nullptr;
  size_t per = 0;
};

int snap(tebd_handle *h, const std::vector<int> &links, Snapshot &s, bool restore) {
  const size_t gsz = sizeof(double2) * (size_t)h->chi * h->d * h->chi;
  const size_t lsz = sizeof(double) * (size_t)h->chi, isz = sizeof(int) * (size_t)h->chi;
  s.per = 2 * gsz + lsz + 2 * isz;
  if (!s.buf && check_cuda(h, cudaMalloc(&s.buf, s.per * links.size()), "autotune snapshot")) return TEBD_ERR_CUDA;
  for (size_t k = 0; k < links.size(); ++k) {
    const int link = links[k];
    char *o = s.buf + k * s.per;
    void *dev[5] = {h->gam + (size_t)(link - 1) * h->chi * h->d * h->chi, h->lam + (size_t)link * h->chi,
                    h->mode == TEBD_MODE_NC ? h->lab_l + (size_t)link * h->chi : nullptr,
                    h->mode == TEBD_MODE_NC ? h->lab_r + (size_t)link * h->chi : nullptr, nullptr};
    const size_t bytes[4] = {2 * gsz, lsz, isz, isz};
    size_t off = 0;
    for (int q = 0; q < 4; ++q) {
      if (dev[q]) {
        const cudaError_t e = restore ? cudaMemcpyAsync(dev[q], o + off, bytes[q], cudaMemcpyDeviceToDevice, h->stream)
                                      : cudaMemcpyAsync(o + off, dev[q], bytes[q], cudaMemcpyDeviceToDevice, h->stream);
        if (check_cuda(h, e, "autotune snapshot copy")) return TEBD_ERR_CUDA;
      }
      off += bytes[q];
    }
  }
  return TEBD_OK;
}

}  // namespace

extern "C" int tebd_autotune(tebd_handle *h, int nbonds, const int *links, const double *const *gates,
                             double *base_ms, double *best_ms) {
  if (!h || nbonds < 1 || !links || !gates) return TEBD_ERR_ARG;
  for (int k = 0; k < nbonds; ++k) {
    if (links[k] < 1 || links[k] > h->L - 1 || !gates[k])
      return set_error(h, TEBD_ERR_ARG, "tebd_autotune: bond link out of range 1..L-1 or null gate");
    for (int q = 0; q < k; ++q)
      if (abs(links[k] - links[q]) < 2) return set_error(h, TEBD_ERR_ARG, "batched bonds must not share a site");
  }
  if (check_cuda(h, cudaSetDevice(h->device), "cudaSetDevice")) return TEBD_ERR_CUDA;
  const int nb = std::min(nbonds, h->nslots);
  const std::vector<int> lk(links, links + nb);
  std::vector<double> te(nb);
  const tebd_stats stats0 = h->stats;
  const long long launches0 = h->launches;
  const int prof0 = h->profiling;
  h->profiling = 0;
  Snapshot s;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = snap(h, lk, s, false);
  if (!rc) rc = check_cuda(h, cudaEventCreate(&e0), "autotune event");
  if (!rc) rc = check_cuda(h, cudaEventCreate(&e1), "autotune event");
  // one timed trial of the batch with the shape `f` (0 entries: the default)
  // the keys the winning shape's launches used (the ones it is stored under)
  std::vector<std::array<int, 3>> win_keys;
  auto trial = [&](TuneParams f, float *ms) -> int {
    h->tune.active = 1;
    h->tune.force = f;
    h->tune.rejected = 0;
    h->tune.seen.clear();
    int r = check_cuda(h, cudaEventRecord(e0, h->stream), "autotune event");
    if (!r) r = run_bond_batch(h, nb, lk.data(), gates, te.data());
    if (!r) r = check_cuda(h, cudaEventRecord(e1, h->stream), "autotune event");
    if (!r) r = check_cuda(h, cudaEventSynchronize(e1), "autotune trial");
    if (!r) r = check_cuda(h, cudaEventElapsedTime(ms, e0, e1), "autotune timing");
    h->tune.active = 0;
    const int r2 = snap(h, lk, s, true);
    if (!r && h->tune.rejected) *ms = -1.f;
    return r ? r : r2;
  };
  float base = 0.f, best = 0.f;
  TuneParams win{0, 0, 0, 0, 0, 0};
  if (!rc) rc = trial(win, &base);  // warm-up of workspaces and kernels
  if (!rc) rc = trial(win, &base);
  best = base;
  win_keys = h->tune.seen;
  bool any_rsvd = false;
  for (const auto &k : h->tune.seen) any_rsvd |= k[0] == 2;
  auto sweep = [&](int which, const std::vector<int> &vals) -> int {
    for (int v : vals) {
      TuneParams f = win;
      (which == 0   ? f.cluster
       : which == 1 ? f.team
       : which == 2 ? f.chol_cluster
       : which == 3 ? f.panel
       : which == 4 ? f.chol_leaf
                    : f.orth_cluster) = v;
      float ms = 0.f;
      const int r = trial(f, &ms);
      if (r) return r;
      if (ms > 0.f && ms < 0.99f * best) {  // 1 %: above the trials' timing noise
        best = ms;
        win = f;
        win_keys = h->tune.seen;
      }
    }
    return TEBD_OK;
  };
  if (!rc) rc = sweep(0, {1, 2, 3, 4, 5, 6, 7, 8});
  if (!rc) rc = sweep(1, {1, 2, 4, 8});
  if (!rc) rc = sweep(5, {1, 2, 4, 8});
  if (!rc && any_rsvd) rc = sweep(2, {1, 2, 4, 8});
  if (!rc && any_rsvd) rc = sweep(3, {4, 8, 16});
  if (!rc && any_rsvd) rc = sweep(4, {128, 192, 256, 384, 768});
  if (!rc) {
    std::lock_guard<std::mutex> lock(g_mu);
    for (const auto &k : win_keys) g_table[{h->device, k[0], k[1], k[2]}] = TuneEntry{win, best * 1e3f};
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s.buf) cudaFree(s.buf);
  h->stats = stats0;
  h->launches = launches0;
  h->profiling = prof0;
  if (base_ms) *base_ms = base;
  if (best_ms) *best_ms = best;
  return rc;
}

extern "C" int tebd_get_tuning(int device, int *entries, int max_entries, int *count) {
  if (!count || max_entries < 0 || (max_entries > 0 && !entries)) return TEBD_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_mu);
  int n = 0, w = 0;
  for (const auto &kv : g_table) {
    if (kv.first[0] != device) continue;
    if (w < max_entries) {
      int *o = entries + 10 * w++;
      o[0] = kv.first[1];
      o[1] = kv.first[2];
      o[2] = kv.first[3];
      o[3] = kv.second.p.cluster;
      o[4] = kv.second.p.team;
      o[5] = kv.second.p.chol_cluster;
      o[6] = kv.second.p.panel;
      o[7] = kv.second.p.chol_leaf;
      o[8] = kv.second.p.orth_cluster;
      o[9] = (int)kv.second.us;
    }
    ++n;
  }
  *count = n;
  return TEBD_OK;
}

extern "C" int tebd_clear_tuning(int device) {
  std::lock_guard<std::mutex> lock(g_mu);
  for (auto it = g_table.begin(); it != g_table.end();)
    it = it->first[0] == device ? g_table.erase(it) : std::next(it);
  return TEBD_OK;
}
