/*
 * tebd_capi.h -- C ABI of the GB300 (sm_103a) Vidal two-site TEBD update.
 *
 * This is the drop-in boundary for the reference's hot path.  Every entry point
 * replaces one routine of OpenTEBD-extended (paths relative to that tree) and is
 * callable from Fortran through ISO_C_BINDING (plain pointers, ints, doubles):
 *
 *   tebd_two_site_op       TwoSiteOp_c    VidalCore_v_2.0/local_operations_module.f90:463-494
 *   tebd_two_site_op_r     TwoSiteOp_r    local_operations_module.f90:430-461
 *   tebd_two_site_op_nc    TwoSiteOpNC_c  local_operations_module.f90:1845-1964
 *   tebd_two_site_op_nc_r  TwoSiteOpNC_r  local_operations_module.f90:1723-1843
 *   tebd_trotter_step      TrotterStep / TrotterStepNC with BoundaryCond='O'
 *                          VidalCore_v_2.0/propagation_module.f90:42-114,200-252,890-1018
 *   tebd_trotter_step_pbc  the same with BoundaryCond='P' (:116-614, 1019-1940)
 *   tebd_swapping          Swapping / SwappingNC  local_operations_module.f90:651-689,1966-2095
 *   tebd_set_conserv       the OPTIONAL intDegFree argument + Conserv%vi
 *   observables, record I/O and canonical forms: see their declarations below
 *   tebd_create/destroy    AllocateGamLam + AllocateLabel + SVDInit/SVDFinish
 *                          VidalCore_v_2.0/TEBDtools_module.f90:486-521,589-620;
 *                          local_operations_module.f90:84-151
 *   tebd_set/get_gamma, tebd_set/get_lambda, tebd_set/get_labels
 *                          the Gammas(:)%t / Lambdas(:)%v / LabelLeft,LabelRight(:)%vi
 *                          arrays the reference passes by pointer
 *                          (TEBDtools_module.f90:31-57)
 *
 * Layouts are exactly the Fortran ones, so a Fortran host passes C_LOC of its
 * arrays without any transpose:
 *   Gamma(site)   COMPLEX(8) (chi, d, chi), column-major, interleaved (re, im)
 *                 doubles: element (alpha,i,beta) at 2*(alpha + chi*(i + d*beta))
 *   Lambda(link)  REAL(8) (chi)
 *   Labels(link)  INTEGER(4) (chi); 10000 marks an unused Schmidt index
 *   Op2           (d*d, d*d) column-major; row index (i-1)*d + j (1-based): the
 *                 right site's index runs fastest.  Complex Op2 interleaved.
 * Sites are numbered 1..L and links 1..L+1, as in the reference; bond `link`
 * couples sites link and link+1.
 *
 * Truncation parameters are the reference's: keep chi singular values, zero
 * guard 1e-15 (dense, single-precision literal) and 1e-10 (number conserving).
 *
 * Threading: one handle per host thread; calls on one handle are serialised
 * on the handle's own CUDA stream.  No call aborts the process: every entry
 * point returns a status code and tebd_last_error() explains the last failure.
 */
#ifndef TEBD_CAPI_H
#define TEBD_CAPI_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define TEBD_OK 0
#define TEBD_ERR_ARG 1            /* invalid argument (size, index, mode)            */
#define TEBD_ERR_CUDA 2           /* a CUDA runtime call failed                       */
#define TEBD_ERR_OOM 3            /* device or host allocation failed                 */
#define TEBD_ERR_SVD_NOCONV 4     /* Jacobi SVD hit its sweep cap before converging   */
#define TEBD_ERR_NONFINITE 5      /* NaN/Inf met in Theta or in the singular values   */
/* On TEBD_ERR_SVD_NOCONV and TEBD_ERR_NONFINITE the bonds of the batch that met
 * the failure keep their Gammas, Lambdas and labels (nothing of that batch is
 * written); batches completed earlier in the same call (the previous sweeps of a
 * Trotter step) stay applied.  The reference ignores ZGESVD's info
 * (local_operations_module.f90:335-336). */
#define TEBD_ERR_STATE 6          /* call not valid in this handle's mode             */
#define TEBD_ERR_NC_BLOCKS 7      /* a charge label fell outside the block range      */

/* handle modes */
#define TEBD_MODE_DENSE 0         /* TwoSiteOp: no symmetry                            */
#define TEBD_MODE_NC 1            /* TwoSiteOpNC: U(1) number conservation             */

/* SVD algorithm (all FP64 but the precision form) */
#define TEBD_SVD_FP64 0           /* default: per bond, bidiagonalisation when both
                                     dimensions of the compacted Theta are >= 64 (a wide
                                     one as Theta^H) and its batch holds a saturated bond
                                     (all chi of its Lambda in use) or one above 384,
                                     else column-pivoted QR + one-sided Jacobi on R^H    */
#define TEBD_SVD_JACOBI 2         /* one-sided Jacobi on the whole (compacted) Theta    */
#define TEBD_SVD_BIDIAG 3         /* bidiagonalisation for every Theta (>= 2 x 2)       */
#define TEBD_SVD_QRJ 4            /* pivoted QR + Jacobi on R^H for every bond          */
#define TEBD_SVD_DF 5             /* precision form: as TEBD_SVD_FP64, but the bidiagonal
                                     route's passes over the trailing matrix, trailing
                                     updates, back-transformation and Gram-Schmidt, and
                                     the Theta formation, run in double-float (pairs of
                                     FP32, 48-bit significands) on the FP32 pipe; number-
                                     conserving blocks on the bidiagonal route too       */
#define TEBD_SVD_RSVD 6           /* learned-rank form: bonds whose compacted Theta is
                                     much larger than the kept rank r take a randomized
                                     sketch of width r + p with FP64-class products on
                                     the tensor cores and a Rayleigh-Ritz SVD (FP64);
                                     the full SVD is the fallback when a kept triplet's
                                     residual exceeds the tolerance (tebd_set_rsvd); the
                                     fallback and the other bonds as TEBD_SVD_DF         */

#define TEBD_OPTS_VERSION 1

typedef struct tebd_opts {
  int version;        /* must be TEBD_OPTS_VERSION                                     */
  int device;         /* CUDA device ordinal                                           */
  int tot_num;        /* NC mode: total particle number (reference global totNum)      */
  int max_filling;    /* NC mode: maximum occupation (reference global maxFilling);
                         d-1 unless tebd_set_conserv gives internal degrees of freedom */
  int svd_mode;       /* TEBD_SVD_FP64 (default), _JACOBI, _BIDIAG, _QRJ or _DF        */
  int max_sweeps;     /* Jacobi sweep cap; 0 selects the default (60)                  */
  int max_batch;      /* bonds updated concurrently; 0 = all bonds of one parity       */
  int reserved;
  double jacobi_tol;  /* relative orthogonality tolerance; 0 = sqrt(n)*eps             */
} tebd_opts;

typedef struct tebd_handle tebd_handle;

/* Fill *opts with defaults (dense-independent fields zero, version set). */
void tebd_default_opts(tebd_opts *opts);

/* Allocate the device-resident chain (L Gammas chi x d x chi, L+1 Lambdas, labels)
 * and the per-bond SVD workspaces.  Gammas and Lambdas start at zero and labels
 * at 10000, as AllocateGamLam/AllocateLabel leave them. */
int tebd_create(int L, int d, int chi, int mode, const tebd_opts *opts, tebd_handle **out);
int tebd_destroy(tebd_handle *h);

int tebd_set_gamma(tebd_handle *h, int site, const double *gamma);
int tebd_get_gamma(tebd_handle *h, int site, double *gamma);
int tebd_set_lambda(tebd_handle *h, int link, const double *lambda);
int tebd_get_lambda(tebd_handle *h, int link, double *lambda);
/* NC mode only: LabelLeft(link)%vi and LabelRight(link)%vi (either pointer may be NULL) */
int tebd_set_labels(tebd_handle *h, int link, const int *label_left, const int *label_right);
int tebd_get_labels(tebd_handle *h, int link, int *label_left, int *label_right);

/* One bond update; replaces TwoSiteOp(link, Op2, Gammas, Lambdas, truncerr).
 * op2 is complex (d^2 x d^2, interleaved) for tebd_two_site_op, real for _r. */
int tebd_two_site_op(tebd_handle *h, int link, const double *op2, double *truncerr);
int tebd_two_site_op_r(tebd_handle *h, int link, const double *op2, double *truncerr);

/* Number-conserving bond update; replaces TwoSiteOpNC(link, Op2, Gammas, Lambdas,
 * LabelLeft, LabelRight, truncerr[, intDegFree]) -- with intDegFree after
 * tebd_set_conserv.  Charge blocks with both sides >= 16 take the bidiagonal
 * route, the others the grouped Jacobi. */
int tebd_two_site_op_nc(tebd_handle *h, int link, const double *op2, double *truncerr);
int tebd_two_site_op_nc_r(tebd_handle *h, int link, const double *op2, double *truncerr);

/* Update several bonds that share no site (e.g. all odd links) in one batched
 * launch sequence.  gates[k] is the complex Op2 for links[k]; truncerr[k] out.
 * Dense or NC according to the handle's mode. */
int tebd_apply_bonds(tebd_handle *h, int nbonds, const int *links, const double *const *gates,
                     double *truncerr);

/* One open-boundary Trotter step; replaces TrotterStep(Udt, Gammas, Lambdas,
 * totalTruncerr) (dense mode) or TrotterStepNC(...) (NC mode).
 * order 2: gates[link-1] = Udt(link), link = 1..L-1 (n_gates >= L-1).
 * order 5 (Forest-Ruth): gates[g-1] = Udt(g), g = 1..2(L-1) (n_gates >= 2(L-2)+2).
 * Same-parity bonds of each sweep are batched. */
int tebd_trotter_step(tebd_handle *h, int order, int n_gates, const double *const *gates,
                      double *total_truncerr);

/* Swapping(link, truncerr, Gammas, Lambdas) (local_operations_module.f90:651-689):
 * exchange the physical indices of sites link and link+1 (SwapTheta), SVD of the
 * unnormalised Theta, FormLambda1/FormGamma1/FormGamma2.  In NC mode
 * SwappingNC(link, Gammas, Lambdas, LabelLeft, LabelRight, truncerr[, intDegFree])
 * (:1966-2095): SwapThetaNC and the block decomposition without RenormThetaNC. */
int tebd_swapping(tebd_handle *h, int link, double *truncerr);

/* Periodic-boundary Trotter step; replaces TrotterStep with BoundaryCond='P'
 * (propagation_module.f90:42-79) in dense mode and TrotterStep2ndOrderPBCNC /
 * TrotterStep5thOrderPBCNC (:1019-1940, same sequences with TwoSiteOpNC and
 * SwappingNC) in NC mode.  The edge bond (L,1) is
 * applied on bond 1 after Swapping site L down to site 2, and swapped back.
 * gates[g-1] = Udt(g) in NEWConstructPropagators' periodic layout
 * (TEBDtools_module.f90:1100-1190):
 *   order 2 (TrotterStep2ndOrderPBC :116-198): g = 1..L, Udt(L) the edge
 *     (n_gates >= L);
 *   order 5 (TrotterStep5thOrderPBC :254-614), odd L: odd bond i Udt(3(i-1)+1..2),
 *     even bond i Udt(2+3(i-2)+1..4), edge Udt(3(L-1)+1..3) (n_gates >= 3L);
 *     even L: bond i Udt(2(i-1)+1..2), edge Udt(2(L-1)+1..2) (n_gates >= 2L). */
int tebd_trotter_step_pbc(tebd_handle *h, int order, int n_gates, const double *const *gates,
                          double *total_truncerr);

/* CanonicalForm(Lambda0, Gamma1, Lambda1, Gamma2, Lambda2) on bond `link`
 * (local_operations_module.f90:496-610) and CanonicalFormAll (propagation_module.f90:
 * 617-634: links 1..L-1 then L-1..1), dense mode: the Schmidt bases of the bond are
 * re-orthogonalised from the chi x chi overlap matrices of the two sides (three
 * chi x chi SVDs, thresholds 1e-8 as the reference). */
int tebd_canonical_form(tebd_handle *h, int link);
int tebd_canonical_form_all(tebd_handle *h);

/* CanonicalFormAllNC (propagation_module.f90:1943-1983): the identity
 * TwoSiteOpNC on links 1..L-1 then L-1..1.  NC mode; follows tebd_set_conserv. */
int tebd_canonical_form_all_nc(tebd_handle *h);

/* Kept-rank form (no reference counterpart; the reference keeps chi values):
 * after each update keep the fewest leading singular values whose discarded
 * weight -- everything beyond them, relative to ||Theta||^2 = 1 -- is at most
 * `bound`; the remaining Lambda entries become exact zeros (NC: label 10000), so
 * the neighbouring updates compact them away.  truncerr reports the full
 * discarded weight.  bound = 0 restores the reference's rule.  Swapping keeps
 * the reference's rule. */
int tebd_set_rank_bound(tebd_handle *h, double bound);

/* Randomized route of TEBD_SVD_RSVD (no reference counterpart; it stands in for
 * ZGESVD, local_operations_module.f90:322-345, on bonds whose compacted Theta is
 * much larger than the kept rank).  oversample: sketch columns beyond the kept
 * rank (default 64); power_iters: extra X^H X applications (default 2, at most
 * 4); tol: a bond is accepted when every kept triplet's residual
 * rho = |Theta^H u - sigma v| is at most tol * ||Theta|| (default 1e-5), else its
 * full SVD is computed -- an accepted triplet's singular value is then within
 * ~rho^2 / gap and its vectors within ~rho / gap of the exact ones; slices: bf16
 * digit planes of the range finder's tensor-core products (3..7, default 7, FP64
 * class); the Rayleigh-Ritz products always use 7.  The route takes only
 * saturated bonds (all chi Schmidt values of the bond in use, spanning at most
 * six decades: the sketch is orthonormalised through Gram matrices, which
 * resolve directions down to ~1e-7 of the largest) with a compacted Theta at
 * least chi + p + 16 on its smaller side.  The learned model may set the sketch
 * per batch instead. */
int tebd_set_rsvd(tebd_handle *h, int oversample, int power_iters, double tol, int slices);

/* The learned part of the learned-rank form (no reference counterpart): a small
 * FP32 network, 67 -> 128 -> 128 -> 8 with ReLU, trained on the GPU by the
 * library's own forward/backward/Adam kernels.  Inputs (per bond, 67 floats):
 * log10(lambda_k / lambda_0) of the bond's Lambda before the update at ranks
 * k = floor(j chi / 64), j = 0..63 (floored at -16), then log10 |U - I|_F,
 * log10 |offdiag(U)|_F (floored at -16) and d / 8 of the gate U.  Outputs (8):
 * log10(sigma_k / sigma_0) of the normalised Theta at k / chi = 0.75, 1, 1.125,
 * 1.25, 1.5, 1.75, 2, 2.5.  Samples are stored one after another (x[67 j + i]).
 * Parameters: one float vector W1 (128 x 67, row-major), b1, W2 (128 x 128), b2,
 * W3 (8 x 128), b3.  Loss: mean squared error over the outputs.
 * Attached to a TEBD_SVD_RSVD handle, the model's predictions set, per batch,
 * the randomized route's oversampling p and power count q -- the cheapest pair
 * (by the route's time model: products n^2 s (2q + 4), Choleskys and Gram SVD
 * s^3 (6 (q + 2) + 128), s = chi + p) whose predicted missed weight
 * (sigma_chi / sigma_0)^2 (sigma_{chi+p} / sigma_chi)^(2q+2) is at most `target` --
 * and send bonds with no such pair straight to the full SVD; the judge still
 * checks every bond the sketch decomposes, and a bond it rejects is sketched once
 * more with (p, q) = (128, 3) before it falls back to the full SVD. */
typedef struct tebd_mlp tebd_mlp;
int tebd_mlp_create(int device, unsigned long long seed, tebd_mlp **out);
int tebd_mlp_destroy(tebd_mlp *m);
int tebd_mlp_param_count(void);
const char *tebd_mlp_last_error(tebd_mlp *m);
int tebd_mlp_get_params(tebd_mlp *m, float *params);
int tebd_mlp_set_params(tebd_mlp *m, const float *params);
/* host buffers; n samples */
int tebd_mlp_forward(tebd_mlp *m, int n, const float *x, float *y);
int tebd_mlp_loss_grad(tebd_mlp *m, int n, const float *x, const float *t, double *loss, float *grad);
/* Adam (lr, beta 0.9 / 0.999, eps 1e-8) over `epochs` passes of minibatches of
 * `batch` samples in order; *loss: mean minibatch loss of the last epoch */
int tebd_mlp_train(tebd_mlp *m, int n, const float *x, const float *t, int epochs, int batch, float lr,
                   double *loss);
/* attach (m != NULL) or detach the model; target in (0, 1) */
int tebd_set_rsvd_model(tebd_handle *h, tebd_mlp *m, double target);

/* Theta formation (FormTheta, local_operations_module.f90:184-211) on the tensor
 * cores (no counterpart in the reference, which forms Theta in FP64 loops).
 * form 0: CUDA cores (FP64, or double-float with TEBD_SVD_DF), the default; 3:
 * 3xTF32 split-precision product with FP32 accumulation (~FP32 accuracy; the
 * precision tier's Theta; dense handles only); 100 + S, S = 3..7: S bf16 digit
 * planes (error ~2^(-7S) of the largest terms; S = 7 is FP64 class).  On
 * TEBD_MODE_NC handles (0 or 103..107; 3 gives TEBD_ERR_STATE) FormThetaNC
 * (:748-818) runs as one product per charge block over its beta class, and
 * ThetaOperationNC is applied in the blocks afterwards.  ThetaOperation, the SVD
 * and the restoration are unchanged. */
int tebd_set_theta_form(tebd_handle *h, int form);

/* Internal degrees of freedom for every NC routine of the handle: the reference
 * passes the OPTIONAL argument intDegFree to TwoSiteOpNC, TrotterStepNC and
 * CanonicalFormAllNC (local_operations_module.f90:748-1443, 1723-1964;
 * propagation_module.f90:890-1018, 1943-1983) and then takes the particle number
 * of local state i from the module global Conserv%vi(i) instead of i-1
 * (set by the Hamiltonian builders, e.g. fermi_hubbard_module.f90:230-232).
 * conserv: d numbers in [0, max_filling] (Conserv%vi), or NULL for the form
 * without intDegFree (which needs max_filling = d-1).
 * NC mode, d <= 8; at most 16 local pairs (i, j) may share one pair total
 * n_i + n_j (TEBD_ERR_ARG otherwise). */
int tebd_set_conserv(tebd_handle *h, const int *conserv);

/* Singular values of the normalised Theta from the last update of `link`
 * (descending; NC mode: the flattened block values in the reference's order).
 * *count receives how many were written: all d*chi (zeros included) on the
 * Jacobi routes, the chi kept ones on the bidiagonal route; the buffer holds d*chi. */
int tebd_get_singular_values(tebd_handle *h, int link, double *sigma, int *count);

/* Jacobi sweeps used by the last update of `link` (diagnostics). */
int tebd_get_sweeps(tebd_handle *h, int link, int *sweeps);

int tebd_sync(tebd_handle *h);
const char *tebd_last_error(tebd_handle *h);
/* Number of CUDA kernel launches issued by this handle since creation. */
long long tebd_kernel_launches(tebd_handle *h);

/* Diagnostics (no counterpart in the reference, which only prints CPU_TIME):
 * work and device-time counters of the hot path, for roofline reporting. */
typedef struct tebd_stats {
  long long updates;           /* bond updates completed                                */
  long long kernel_launches;   /* all kernels launched by this handle                   */
  long long jacobi_launches;   /* Jacobi round kernels launched                         */
  long long jacobi_sweeps;     /* sweeps summed over problems                           */
  long long jacobi_pairs;      /* column pairs visited (each: one 3-term dot product)   */
  long long jacobi_rotations;  /* column pairs rotated                                  */
  double jacobi_flops;         /* algorithmic FP64 flops of the Jacobi rounds           */
  double jacobi_bytes;         /* algorithmic bytes moved by the Jacobi rounds          */
  double jacobi_ms;            /* device time of the Jacobi rounds (profiling on)       */
  double batch_ms;             /* device time of whole bond batches (profiling on)      */
  long long compact_rows;      /* sum over updates of the SVD's row count (d * kept chi) */
  long long compact_cols;      /* sum over updates of the SVD's column count            */
  double qr_flops;             /* algorithmic FP64 flops of the pivoted QR and of U = QZ */
  double qr_ms;                /* device time of the pivoted-QR kernel (profiling on)   */
  long long rank_sum;          /* sum over updates of the numerical rank k              */
  double bidiag_ms;            /* device time of the bidiagonal route (profiling on)     */
  long long bidiag_updates;    /* updates that took the bidiagonal route                */
  double gebrd_flops;          /* algorithmic FP64 flops of the bidiagonalisations:
                                  16 M N^2 - 16 N^3 / 3 per bond (M >= N)                  */
  double gebrd_ms;             /* device time of the bidiagonalisation kernel (profiling on) */
  long long gebrd_launches;    /* bidiagonalisation kernel launches                        */
  long long rsvd_updates;      /* updates that took the randomized route (TEBD_SVD_RSVD)   */
  long long rsvd_fallbacks;    /* of those, the ones the judge sent to the full SVD        */
  double rsvd_flops;           /* algorithmic flops (8 m n k per complex product) of the
                                  randomized route's tensor-core products                 */
  double rsvd_worst_residual;  /* largest triplet residual / ||Theta|| the judge saw        */
  long long rsvd_skipped;      /* bonds the learned model sent straight to the full SVD     */
  double tc_ms;                /* device time of the tensor-core product kernels (profiling on;
                                  the operand packing excluded)                           */
  long long tc_launches;       /* tensor-core product kernels timed                       */
  double tc_mma_flops;         /* flops those kernels issued on the tensor cores (2 per
                                  multiply-add, bf16 or TF32 operands, padding included)  */
  long long rsvd_batches;      /* batches that ran the randomized route                    */
  long long rsvd_oversample_sum; /* their sketch oversampling p, summed (mean = / batches) */
  long long rsvd_power_sum;    /* their power-iteration counts q, summed                   */
  long long rsvd_retries;      /* bonds re-sketched with (p, q) = (128, 3) after the judge
                                  rejected the model's sketch (then the full SVD if again) */
} tebd_stats;
int tebd_set_profiling(tebd_handle *h, int on);
int tebd_get_stats(tebd_handle *h, tebd_stats *stats);
int tebd_reset_stats(tebd_handle *h);
/* Measured FP64 FMA throughput of the device (TFLOP/s), by a short DFMA loop. */
int tebd_measure_fp64_peak(int device, double *tflops);

/* Autotuner of the SVD routes' launch shapes (no reference counterpart; the
 * reference has no GPU launches).  Times candidate shapes on the batch of bonds
 * `links` (at most one batch: the first nslots bonds, none sharing a site) with
 * their gates, as tebd_apply_bonds would update them: the default choice, each
 * cluster size 1..8 of the bidiagonalisation, each bisection team of 1, 2, 4, 8
 * lanes with the best cluster, each cluster of 1, 2, 4, 8 CTAs per side of the
 * singular vectors' re-orthogonalisation, and, when the randomized route runs, each
 * cluster of 1, 2, 4, 8 CTAs per bond, each panel of 4, 8, 16 rows and each leaf
 * size 128, 192, 256, 384, 768 of its recursively blocked Cholesky.  The fastest (by more than 1 %) is kept in
 * a table per device under (route, largest compacted dimension rounded up to
 * 64, bonds rounded up to a power of two), which every later batch on the device
 * uses.  Shapes change no result beyond rounding.  The chain is left as it was
 * (the touched Gammas, Lambdas and labels are restored after every trial) and
 * the statistics are not counted.  base_ms / best_ms (either may be NULL): the
 * batch's time with the default and with the chosen shape. */
int tebd_autotune(tebd_handle *h, int nbonds, const int *links, const double *const *gates, double *base_ms,
                  double *best_ms);
/* The device's table: up to max_entries rows of 10 ints (route: 0 FP64
 * bidiagonal, 1 double-float bidiagonal, 2 randomized-route Cholesky leaf, 3 its
 * blocking; dimension bucket; bonds bucket; bidiagonalisation cluster size;
 * bisection team size; Cholesky cluster size; Cholesky panel height; Cholesky
 * leaf size; re-orthogonalisation cluster size -- 0 = the default; batch time in
 * microseconds); *count = rows in the table. */
int tebd_get_tuning(int device, int *entries, int max_entries, int *count);
/* Empty the device's table (the defaults apply again). */
int tebd_clear_tuning(int device);
/* The handle's CUDA stream (a cudaStream_t), for callers that time or order
 * their own work against the library's. */
void *tebd_get_stream(tebd_handle *h);

/* Observables of the device-resident chain (VidalCore_v_2.0/observables_module.f90),
 * open boundary, computed on the GPU so that the chain is not downloaded to be
 * measured.  Complex outputs are interleaved (re, im); matrices column-major.
 * They run on the handle's stream after any pending update and use the handle's
 * SVD workspace, plus a small buffer allocated on first use.
 *   tebd_single_site_rho   SingleSiteDensityMatrix / FormSingleSiteRho (:95-131):
 *                          rho[s] (d x d) for s = 1..L, rho(i,j) = sum l0^2 l1^2 G(a,i,b) conj(G(a,j,b))
 *   tebd_one_site_expval   OneSiteExpVal_c (:224-252): Tr(Op rho_s), Op complex d x d,
 *                          exp_list: L complex
 *   tebd_one_site_expval_r OneSiteExpVal_r (:194-222): Op real d x d, exp_list: L real
 *   tebd_two_site_rho      ThetaKernal + TwoSiteRho (:704-832) on sites link, link+1:
 *                          d^2 x d^2 complex, rows (i-1)*d+j and columns (l-1)*d+k as the gates
 *   tebd_local_energy      LocalEnergy (:1346-1387): energy[l-1] = Re Tr(H(l) rho2(l)),
 *                          H[l-1] complex d^2 x d^2, l = 1..L-1 (n_ops >= L-1)
 *   tebd_total_energy      TotalEnergy (:1432-1466): sum of the bond energies
 *   tebd_inner_product     InnerProduct (:1031-1089): <left|right>, complex; the two handles
 *                          must have equal L, d, chi and device
 *   tebd_chain_entropy     ChainEntropy (:1583-1602) for links 1..L+1:
 *                          -sum_{lambda != 0} lambda^2 ln|lambda^2| / ln d */
int tebd_single_site_rho(tebd_handle *h, double *rho);
int tebd_one_site_expval(tebd_handle *h, const double *op, double *exp_list);
int tebd_one_site_expval_r(tebd_handle *h, const double *op, double *exp_list);
int tebd_two_site_rho(tebd_handle *h, int link, double *rho2);
int tebd_local_energy(tebd_handle *h, int n_ops, const double *const *H, double *energy);
int tebd_total_energy(tebd_handle *h, int n_ops, const double *const *H, double *energy);
int tebd_inner_product(tebd_handle *left, tebd_handle *right, double *value);
int tebd_chain_entropy(tebd_handle *h, double *entropy);

/* Chain state I/O in the reference's record formats (ToolsCore_v_2.0/io_module.f90),
 * for checkpoints shared with a Fortran host.  kind 'S': Fortran E30.15 text,
 * 15 significant digits; 'B': B80, the exact bit pattern in binary.  Files are
 * named by path (the reference passes open units); append != 0 appends as the
 * reference's openKind 'A' does, else the file is created or truncated.
 *   tebd_record_lambdas   RecordLambdas (:191-220): L+1 records of chi values
 *   tebd_record_gammas    RecordGammas (:222-264): per site, left index, right index a
 *                         record of the d real parts; then the imaginary parts
 *   tebd_record_labels    RecordLabel (:267-287) of LabelLeft and of LabelRight (NC mode;
 *                         either path may be NULL), I16
 *   tebd_read_gamma_lambda         readGammaLambda (:289-373): records of chi_now values
 *                                  (chi_now <= chi); entries beyond chi_now are kept
 *   tebd_read_gamma_lambda_labels  readGammaLambdaLabels (:376-472), NC mode */
int tebd_record_lambdas(tebd_handle *h, const char *path, char kind, int append);
int tebd_record_gammas(tebd_handle *h, const char *path, char kind, int append);
int tebd_record_labels(tebd_handle *h, const char *path_left, const char *path_right);
int tebd_read_gamma_lambda(tebd_handle *h, const char *lambda_path, const char *gamma_path, char kind,
                           int chi_now);
int tebd_read_gamma_lambda_labels(tebd_handle *h, const char *lambda_path, const char *gamma_path,
                                  const char *label_left_path, const char *label_right_path, char kind,
                                  int chi_now);

/* The split-precision complex product on the tensor cores (no counterpart in the
 * reference, which multiplies only inside FormTheta, local_operations_module.f90:
 * 184-211): C_p = A_p B_p for p = 0..nprob-1, all device pointers, complex
 * interleaved, column-major (A_p m x k at A + stride_a*p doubles... in complex
 * units: element (i, l) at A[2*(stride_a*p + i + lda*l)]), likewise B (k x n) and
 * C (m x n).  form 3: 3xTF32 (hi*hi + hi*lo + lo*hi, FP32 accumulation, about
 * FP32 accuracy); form 1: one TF32 pass; form 100 + S (S = 1..7): error-free
 * splitting into S bf16 digit planes of 7 bits per row (the Ozaki scheme), exact
 * FP32 accumulation of the digit products, combined in FP64 -- error about
 * 2^(-7S) x row max x column max per term (S = 7: FP64 class).  Runs on
 * `stream` and synchronises it; allocates its operand planes for the call. */
int tebd_zgemm_tc(int nprob, int m, int n, int k, const double *A, long long stride_a, int lda,
                  const double *B, long long stride_b, int ldb, double *C, long long stride_c, int ldc,
                  int form, void *stream);

/* Allocation-free dense update of bond `link` of a chain the caller already
 * holds in device memory.  No counterpart in the reference.  It exists for
 * callers that cannot allocate device memory when they run the update: a host
 * whose device memory comes from a fixed pool sized at start-up (a further
 * cudaMalloc fails or breaks the pool's budget), a host that keeps its own
 * device-resident chain and cannot own a handle (tebd_create allocates SVD
 * workspaces for a whole sweep), and time-critical loops that keep cudaMalloc
 * and cudaFree (which synchronises the device) out of their steady state.
 * It calls no cudaMalloc/cudaFree and no allocating library routine; every
 * temporary lives in one static device array of about 2.1 MB that each GPU
 * loading this library holds until exit.
 *   gammas   device, L Gammas back to back, each chi x d x chi complex (Fortran order)
 *   lambdas  device, L+1 Lambdas back to back, each chi doubles
 *   op2      device, complex (d^2 x d^2) gate, layout as for tebd_two_site_op
 *   truncerr host, receives the truncation error
 *   stream   cudaStream_t to run on (NULL: the legacy default stream); the call
 *            synchronises this stream before it returns
 * Limit: d*chi <= 256 (and chi <= 256, d <= 8); larger sizes return TEBD_ERR_ARG.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process: make that
 * first call before any stream capture begins, and do not call this entry point
 * on a device after cudaDeviceReset.  All calls share the array and it keeps the
 * last call's contents (what must start at zero is cleared by each call): calls
 * that overlap on the GPU race and must be serialised.
 * A CUDA error already pending on the calling thread is left in place and the
 * call returns TEBD_ERR_CUDA without running.  On TEBD_ERR_SVD_NOCONV and
 * TEBD_ERR_NONFINITE the caller's Gammas and Lambdas are left unmodified. */
int tebd_two_site_op_noalloc(int L, int d, int chi, int link, double *gammas, double *lambdas,
                             const double *op2, double *truncerr, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TEBD_CAPI_H */
