// tebd_internal.cuh -- shared definitions of the sm_103a TEBD library.
//
// Device layout of one handle (all allocations made once in tebd_create):
//   gam     L Gammas, each chi x d x chi complex, Fortran column-major, site-major
//           (site s at offset s*chi*d*chi): the exact array a Fortran host holds.
//   lam     L+1 Lambdas of length chi (link-major).
//   lab_l/r L+1 label vectors of length chi (NC mode).
//   slots   one SVD workspace per concurrently updated bond: the reshaped Theta X
//           (n x n, n = d*chi, column-major, ld = n), the right factor V (n x n),
//           FP32 shadows of both for the mixed-precision SVD, sorted singular
//           values and their column permutation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <array>
#include <vector>

#include "tebd_capi.h"

namespace tebd {

// Fortran default-REAL literals used as guards by the reference:
// `1E-15` (local_operations_module.f90:362,373,396,421) and `10.0**(-10)`
// (:1591,1643,1679,1711) are single precision, widened to double at comparison.
constexpr double kGuardDense = (double)1e-15f;
constexpr double kGuardNC = (double)1e-10f;
constexpr int kLabelUnused = 10000;

// ---------------------------------------------------------------------------
// complex helpers (interleaved re/im, same storage as COMPLEX(8))
// ---------------------------------------------------------------------------
template <typename T>
struct cplx;
template <>
struct cplx<double> {
  using type = double2;
};
template <>
struct cplx<float> {
  using type = float2;
};

__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// ---------------------------------------------------------------------------
// batched one-sided Jacobi SVD problem descriptor
// ---------------------------------------------------------------------------
// Each problem is an m x n column-major matrix X (ld = ldx) whose columns are
// orthogonalised in place, with the right rotations accumulated into V
// (n x n, ld = ldv).  After convergence X = U*Sigma (column k = sigma_k u_k).
template <typename T>
struct JacobiProblem {
  typename cplx<T>::type *X;
  typename cplx<T>::type *V;
  int m, n, ldx, ldv;
  double floor;  // columns with squared norm <= floor are treated as zero (not rotated)
};

// Relative size below which a column of Theta is numerically zero for the SVD:
// |x| <= 2^-60 ||Theta||_F (~8.7e-19, three decades under the reference's 1e-15
// Lambda guard).  Such columns are not rotated; this only removes sweeps spent
// reorthogonalising rounding noise.
constexpr double kNegligibleColumn = 8.673617379884035e-19;

struct JacobiState {
  int *rot;                       // rotations applied in the current sweep, per problem
  int *done;                      // 1 once a sweep applied no rotation
  int *sweeps;                    // sweeps executed, per problem
  int *pending;                   // [0] problems not yet converged (host reads it)
  unsigned long long *counters;   // [0] rotations, [1] pairs visited, [2] pair-rows, [3] rotated
                                  // pair-rows (rows of X plus rows of V), summed over problems
};

// ---------------------------------------------------------------------------
// per-handle state
// ---------------------------------------------------------------------------
// Exact compaction of Theta.  Rows (i,alpha) with Lambda0(alpha) == 0 and columns
// (j,beta) with Lambda2(beta) == 0 are identically zero, and Lambda1(gamma) == 0
// removes gamma from the contraction; FormLambda1 leaves exact zeros below its
// guard, so most of a fixed-chi allocation is zero until the chain saturates.
// Theta is formed and decomposed as the (d r0) x (d r2) matrix of the kept
// indices: row i*r0 + a', column j*r2 + b'.  Its singular values are those of the
// full matrix; the dropped ones are exact zeros.
struct Compact {
  int r0, r1, r2;  // kept counts of Lambda0, Lambda1, Lambda2
  int m, n;        // d*r0 rows, d*r2 columns
  int k;           // singular triplets computed (numerical rank for the QR path, else n)
  float span;      // smallest / largest nonzero Lambda1 (the bond's own Schmidt values)
};

struct Slot {
  double2 *X, *V;    // FP64 Theta (m x n, ld m) / right factor (n x n, ld n)
  float2 *Xf, *Vf;   // FP32 shadows (mixed SVD)
  double2 *theta0;   // copy of the gated, unnormalised Theta (mixed SVD)
  double *S;         // n sorted singular values of the normalised Theta
  int *perm;         // n column permutation (descending sigma)
  double2 *gate;     // d^2 x d^2 gate for this slot
  int *idx0, *idx1, *idx2;  // kept alpha / gamma / beta (chi each)
  int *inv0, *inv2;         // alpha -> a' and beta -> b' (-1 if dropped)
  Compact *cp;              // device compaction record
  // QR-preconditioned SVD (qrj.cu)
  int *jpvt;                // n column permutation of the pivoted QR
  double2 *tau;             // n reflector scalars
  double *vn;               // 2n partial column norms (later: the k singular values)
  double2 *aux;             // 3 n^2: A = R^H (n x k), Z (k x k), Y = Q [Z; 0] (m x k);
                            // bidiagonal path: right reflectors (n x n), partial sums
  double2 *taup;            // n right-reflector scalars (bidiagonal path)
  double *bdws;             // bidiagonal path: d, e, sigma, inverse-iteration scratch, Z, U
};

// SVD route of one bond of a dense batch
constexpr int kPathQRJ = 0;      // pivoted QR + one-sided Jacobi on R^H (qrj.cu)
constexpr int kPathBidiag = 1;   // bidiagonalisation + bisection + inverse iteration (bidiag.cu)
constexpr int kPathBidiagT = 2;  // the same on Theta^H, for a wide compacted Theta (m < n)
constexpr int kPathRsvd = 3;     // randomized sketch + Rayleigh-Ritz (rsvd.cu), full SVD as fallback
constexpr int kBidiagMinDim = 64;  // default route switch: min(m, n) of the compacted Theta
constexpr int kQrjMaxDim = 384;    // a batch of unsaturated bonds up to this min(m, n) keeps the QR route

// learned model (mlp.cu): sizes and the relative ranks k / chi of its outputs
constexpr int kMlpIn = 67, kMlpHidden = 128, kMlpOut = 8;
extern const double kMlpRanks[kMlpOut];

// Launch shapes chosen by the autotuner (tune.cu); 0 = the library's default.
struct TuneParams {
  int cluster;       // CTAs per cluster of the bidiagonalisation
  int team;          // lanes per value of the bisection
  int panel;         // rows of R per panel of the randomized route's Cholesky
  int chol_cluster;  // CTAs per bond of that Cholesky
  int chol_leaf;     // largest diagonal block the recursive Cholesky factors directly
  int orth_cluster;  // CTAs per (bond, side) of the singular vectors' re-orthogonalisation
};

}  // namespace tebd

struct tebd_handle {
  int L, d, chi, mode, n;
  tebd_opts opts;
  int device;
  cudaStream_t stream;
  // chain
  double2 *gam;
  double *lam;
  int *lab_l, *lab_r;
  // workspaces
  int nslots;
  std::vector<tebd::Slot> slots;  // host copy of the slot table
  tebd::Slot *slots_d;            // device copy of the slot table
  void *ws_base;                  // single allocation carved into slots
  size_t ws_bytes;
  double2 *gates_d;               // nslots * d^4 gates of the current batch
  tebd::Compact *cp_d;            // nslots compaction records
  int *path_d;                    // nslots SVD route per slot (kPathQRJ / kPathBidiag)
  std::vector<int> path_h;        // host copy of the current batch's routes
  int *idx_d;                     // nslots * 5 * chi index maps
  double *nrm_part;       // nslots * kNormParts partial sums of |Theta|^2
  double *nrm;            // nslots Frobenius norms
  double *truncerr_d;     // nslots
  int *links_d;           // nslots link numbers of the current batch
  tebd::JacobiState js;
  void *jprob_d;          // device array of JacobiProblem<double>
  void *jprobf_d;         // device array of JacobiProblem<float>
  int *status_d;          // [0] non-finite flag, [1] NC block error flag
  void *obs_buf;          // observables workspace, allocated on first use (obs.cu)
  size_t obs_bytes;
  // NC workspaces (allocated in NC mode)
  void *nc_ws;
  size_t nc_ws_bytes;
  void *nc_meta;  // host-side NC slot table (nc.cu)
  // internal degrees of freedom (tebd_set_conserv): local particle numbers
  int nc_idf;                    // 1: the intDegFree branches, 0: local number i-1
  int nc_conserv[8];             // Conserv%vi(1..d)
  // last spectrum per link (tebd_get_singular_values / tebd_get_sweeps)
  double *sig_link_d;            // (L-1) * n
  int *sig_count_d;              // L-1
  int *sweeps_link_d;            // L-1
  int js_cap;                    // capacity of the JacobiState arrays (problems)
  double *pinned;                // pinned staging buffer (gates, truncation errors, flags)
  size_t pinned_bytes;
  std::string err;
  long long launches;
  // diagnostics
  tebd_stats stats;
  int profiling;
  int unnormalized;        // 1 while Swapping runs: Theta is decomposed without 1/||Theta||
  double rank_bound;       // kept-rank form: discarded weight bound per bond (0 = keep chi)
  cudaEvent_t ev[6];
  // tensor-core products (theta_tc.cu)
  int theta_form;          // 0: CUDA cores (FP64, or double-float with TEBD_SVD_DF);
                           // 3: 3xTF32; 100 + S: S bf16 digit planes (tcgen05)
  void *tc_ws;             // operand planes / digits, grown on demand
  size_t tc_ws_bytes;
  int *tc_err;             // set by a tensor-core kernel whose pipeline wait expired
  // randomized SVD route (rsvd.cu, TEBD_SVD_RSVD)
  void *rs;                // RsState, allocated on first use
  int rs_oversample;       // sketch columns beyond the kept rank
  int rs_power;            // power iterations (X^H X applications beyond the first)
  double rs_tol;           // judge: largest triplet residual / ||Theta||
  int rs_slices;           // bf16 digit planes of the products (7: FP64 class)
  int rs_sketch_cap;       // workspace sketch capacity requested so far
  // profiling: event pairs around the tensor-core product kernels of a batch
  std::vector<cudaEvent_t> tc_ev;
  std::vector<double> tc_ev_flops;
  int tc_ev_used;
  tebd_mlp *rs_model;      // learned model choosing the sketch per batch (mlp.cu), or null
  double rs_target;        // the model's bound on (sigma_{r+p} / sigma_r)^(2q+2)
  // autotuner trial in progress (tune.cu): the forced shape, the keys met, and
  // whether a launch could not use the forced shape
  struct {
    int active = 0, rejected = 0;
    tebd::TuneParams force{0, 0, 0, 0, 0, 0};
    std::vector<std::array<int, 3>> seen;
  } tune;
};

namespace tebd {

int set_error(tebd_handle *h, int code, const std::string &msg);
void set_noh_error(const std::string &msg);  // for tebd_last_error(NULL)
int check_cuda(tebd_handle *h, cudaError_t e, const char *what);

// kernels launched from capi.cu (defined in the .cu files)
int launch_dense_prepare(tebd_handle *h, int nb, bool real_gate);
int run_jacobi(tebd_handle *h, int nb, int svd_mode, int nmax);
int dense_compact_sizes(tebd_handle *h, int nb, int *nmax, std::vector<Compact> *out);
int launch_dense_finish(tebd_handle *h, int nb);
int launch_eye(tebd_handle *h, int nb);
int launch_unit_norm(tebd_handle *h, int nb);
int run_jacobi_problems(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob, int nmax);
int jacobi_persistent_double(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob,
                             int nmax, double tol, int max_sweeps);
int run_qrj(tebd_handle *h, int nb, int nmax);
int run_bidiag(tebd_handle *h, int nb, int nmax);
// A batch of bidiagonal problems described by slot entries (X, V, aux, tau, taup,
// bdws, cp) and routes; kk triplets per problem (min(kk, N) computed).
struct BidiagBatch {
  Slot *slots_d;
  const int *path_d;
  const int *path_h;
  int nb, nmax, kk;
  bool dfp;
  int phase;  // 0: whole route; 1: through the singular values; 2: the vectors
  int cap;    // 1: vectors only for the first cp->k values of each problem (set between phases)
  int right_only = 0;  // 1: right singular vectors only (double-float form; S.X keeps no left vectors)
};
int run_bidiag_batch(tebd_handle *h, const BidiagBatch &b);
// Autotuner table (tune.cu): the shape for route (0 FP64 bidiagonal, 1
// double-float bidiagonal, 2 randomized-route Cholesky leaf, 3 its blocking),
// largest dimension n and bonds nb; zeros where no entry exists.  tune_reject: the launch could not
// use the shape it was given.
TuneParams tune_lookup(tebd_handle *h, int route, int n, int nb);
void tune_reject(tebd_handle *h);
void bidiag_block_ws(int M, int N, int kk, size_t *aux_elems, size_t *bdws_doubles);
size_t bidiag_ws_doubles(int n, int chi);
size_t bidiag_aux_elems(int n);
constexpr int kBidiagMaxDim = 4096;  // larger compacted Theta take the QR + Jacobi route
constexpr int kRsvdMaxSketch = 1536;  // widest sketch of the randomized route (chi + oversampling)
constexpr int kRsvdRetryP = 128, kRsvdRetryQ = 3;  // the second sketch of a bond the judge sent back
int jacobi_collect(tebd_handle *h);
int measure_fp64_peak(int device, double *tflops);
int run_nc_batch(tebd_handle *h, int nb, const int *links_host, double *truncerr_host);
int nc_alloc(tebd_handle *h);
void nc_free(tebd_handle *h);

constexpr int kNormParts = 64;

// tensor-core Theta formation (theta_tc.cu)
int launch_theta_tc(tebd_handle *h, int nb);
int tc_reserve(tebd_handle *h, size_t bytes);
int tc_check(tebd_handle *h);  // reads and clears tc_err (synchronises the stream)
void tc_free(tebd_handle *h);
// profiling of the tensor-core product kernels: a fresh event pair for one launch
// issuing `flops` tensor-core flops (null events when profiling is off), and the
// collection of a batch's pairs into the stats once the stream is synchronised
void tc_events(tebd_handle *h, double flops, cudaEvent_t *e0, cudaEvent_t *e1);
void tc_collect(tebd_handle *h);
// randomized SVD route (rsvd.cu)
int run_rsvd(tebd_handle *h, int nb, const std::vector<Compact> &cps, std::vector<int> &route,
             const std::vector<int> &rank, int sketch, int power);
void rsvd_free(tebd_handle *h);
// model inference for the bonds of a batch: features from Lambda(link) on the
// device and 3 host gate terms per bond; kMlpOut predictions per bond to the host
int mlp_features_forward(tebd_mlp *M, const double *lam, const int *links, const float *gate_terms_host, int chi,
                         int nb, cudaStream_t st, float *out_host);

}  // namespace tebd

#define TEBD_LAUNCHED(h) ((h)->launches++)
