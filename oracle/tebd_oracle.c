/*
 * tebd_oracle.c -- CPU oracle for the Vidal two-site TEBD update.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
 * bench.py load it.  The shipped path is the CUDA library built from
 * opentebd-extended_gb300/csrc/.
 *
 * It restates, loop for loop, the reference's FP64 routines (paths relative to
 * the OpenTEBD-extended source tree):
 *
 *   dense update   VidalCore_v_2.0/local_operations_module.f90
 *       FormTheta        :184-211     ThetaOperation_c :248-280
 *       ThetaOperation_r :213-245     ReshapeTheta     :283-320
 *       SVDTruncation    :322-345     FormLambda1      :347-379
 *       FormGamma1       :381-404     FormGamma2       :406-428
 *       TwoSiteOp_c      :463-494
 *   number-conserving update (no internal degrees of freedom)
 *       FormThetaNC :748-851  ThetaOperationNC_c :950-1044  RenormThetaNC :1046-1130
 *       minmaxNLR :1201-1250  SizeOfBlocks :1252-1337  IndexLeft/Right :1339-1443
 *       FormBlockTheta :1445-1468  SVDNC :1470-1492  FlattenSS :1494-1513
 *       Ordering :1515-1538  JudgePosition :1540-1565  UpdateLabelLeft/Right :1567-1625
 *       FormLambdaNC :1627-1657  FormGamma1NC/2NC :1659-1721  TwoSiteOpNC_c :1845-1964
 *   sweeps        VidalCore_v_2.0/propagation_module.f90
 *       TrotterStep2ndOrder :82-114   TrotterStep5thOrder :200-252
 *       TrotterStep2ndOrderNC :956-1018 (5th-order NC twin follows :200-252's gate map)
 *
 * The SVD is LAPACK ZGESVD('A','A'), exactly as the reference calls it
 * (local_operations_module.f90:335 and :1486).  LAPACK is not part of the
 * reference tree and no version is pinned there; the host's LAPACK entry point
 * is handed in at run time by oracle_set_zgesvd() (the Python side passes the
 * address exported by scipy.linalg.cython_lapack).
 *
 * Fortran literals reproduced bit-for-bit: `1E-15` and `10.0**(-10)` are
 * default-REAL (single precision) constants in the reference, so the guards
 * compare against (double)1e-15f and (double)1e-10f.  The sentinel label is
 * 10000 and "unused" is tested as label >= 1000, as in the reference.
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists in the
 * build container, and the reference ships no tests or golden vectors.  This
 * restatement is therefore pinned only by analytic known answers (see
 * tests/test_oracle.py): parity unpinned against the reference binary itself.
 *
 * Layouts: every array is Fortran column-major, complex values are interleaved
 * (re, im) doubles (identical to COMPLEX(KIND=8) storage).
 *   Gamma(alpha,i,beta)  chi x d x chi   offset alpha + chi*(i + d*beta)
 *   Op2(r,c)             d^2 x d^2       offset r + d^2*c,  r = i*d + j (right site fastest)
 * Indices in this file are 0-based unless a comment says otherwise.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zc;

typedef void (*zgesvd_fn)(char *jobu, char *jobvt, int *m, int *n, zc *a, int *lda, double *s,
                          zc *u, int *ldu, zc *vt, int *ldvt, zc *work, int *lwork,
                          double *rwork, int *info);

static zgesvd_fn g_zgesvd = 0;

#define GUARD_DENSE ((double)1e-15f) /* Fortran `1E-15` (default REAL)      */
#define GUARD_CANON ((double)1e-8f)  /* CanonicalForm's `1E-8` (default REAL) */
#define GUARD_NC ((double)1e-10f)    /* Fortran `10.0**(-10)` (default REAL) */
#define LABEL_UNUSED 10000

/* status codes shared with the Python wrapper */
#define OR_OK 0
#define OR_ERR_NOLAPACK -1
#define OR_ERR_ALLOC -2
#define OR_ERR_LAPACK -3
#define OR_ERR_ARG -4

void oracle_set_zgesvd(void *fn) { g_zgesvd = (zgesvd_fn)fn; }
int oracle_has_zgesvd(void) { return g_zgesvd != 0; }

/* ZGESVD('A','A') on an m x n column-major matrix (destroyed), workspace as the
 * reference sizes it: dense 5*dchi (:90-94), NC 5*max(m,n) / 5*min(m,n) (:720-722). */
static int zgesvd_all(int m, int n, zc *a, double *s, zc *u, zc *vt, int lwork, int lrwork) {
  if (!g_zgesvd) return OR_ERR_NOLAPACK;
  zc *work = (zc *)malloc(sizeof(zc) * (size_t)(lwork > 1 ? lwork : 1));
  double *rwork = (double *)malloc(sizeof(double) * (size_t)(lrwork > 1 ? lrwork : 1));
  if (!work || !rwork) {
    free(work);
    free(rwork);
    return OR_ERR_ALLOC;
  }
  char ja = 'A', jb = 'A';
  int lda = m, ldu = m, ldvt = n, info = 0;
  g_zgesvd(&ja, &jb, &m, &n, a, &lda, s, u, &ldu, vt, &ldvt, work, &lwork, rwork, &info);
  free(work);
  free(rwork);
  return info == 0 ? OR_OK : OR_ERR_LAPACK;
}

/* ------------------------------------------------------------------------- */
/* Dense update                                                               */
/* ------------------------------------------------------------------------- */

/* FormTheta (:184-211): 5-deep loop, gamma innermost, product evaluated left to
 * right as Fortran does.  theta is chi x d x d x chi. */
static void form_theta(int chi, int d, zc *theta, const double *l0, const zc *g1, const double *l1,
                       const zc *g2, const double *l2) {
  const size_t sg = (size_t)chi * d; /* stride of the last Gamma index */
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
          zc acc = 0.0;
          for (int g = 0; g < chi; ++g)
            acc = acc + l0[a] * g1[a + (size_t)chi * i + sg * g] * l1[g] *
                            g2[g + (size_t)chi * j + sg * b] * l2[b];
          theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * b))] = acc;
        }
}

/* ThetaOperation_c (:248-280) / ThetaOperation_r (:213-245): the gate mixes the
 * two physical indices; op row index (i-1)*d+j, column (k-1)*d+l (1-based). */
static void theta_operation(int chi, int d, zc *theta, const zc *op_c, const double *op_r) {
  const size_t nt = (size_t)chi * d * d * chi;
  const int d2 = d * d;
  zc *tmp = (zc *)malloc(sizeof(zc) * nt);
  memcpy(tmp, theta, sizeof(zc) * nt);
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
          zc acc = 0.0;
          for (int k = 0; k < d; ++k)
            for (int l = 0; l < d; ++l) {
              const size_t oi = (size_t)(i * d + j) + (size_t)d2 * (k * d + l);
              const zc op = op_c ? op_c[oi] : (zc)op_r[oi];
              acc = acc + op * tmp[a + (size_t)chi * (k + (size_t)d * (l + (size_t)d * b))];
            }
          theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * b))] = acc;
        }
  free(tmp);
}

/* ReshapeTheta (:283-320): FP64 Frobenius norm in the reference's loop order,
 * then ThetaRS((i-1)chi+alpha, (j-1)chi+beta) = Theta/norm. */
static void reshape_theta(int chi, int d, const zc *theta, zc *rs) {
  const size_t n = (size_t)chi * d;
  zc nsq = 0.0;
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
          const zc t = theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * b))];
          nsq = nsq + conj(t) * t;
        }
  const double norm = sqrt(creal(nsq));
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j)
          rs[((size_t)i * chi + a) + n * ((size_t)j * chi + b)] =
              theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * b))] / norm;
}

/* FormLambda1 (:347-379) */
static void form_lambda1(int chi, double *lam1, double *truncerr, const double *s) {
  double norm = 0.0;
  for (int a = 0; a < chi; ++a)
    if (fabs(s[a]) > GUARD_DENSE) norm = norm + s[a] * s[a];
  *truncerr = fabs(1.0 - norm);
  for (int a = 0; a < chi; ++a) lam1[a] = (fabs(s[a]) > GUARD_DENSE) ? s[a] / sqrt(norm) : 0.0;
}

/* FormGamma1 (:381-404): Gamma1(alpha,i,beta) = U((i-1)chi+alpha, beta)/Lambda0(alpha) */
static void form_gamma1(int chi, int d, const double *l0, zc *g1, const zc *u) {
  const size_t n = (size_t)chi * d;
  for (int b = 0; b < chi; ++b)
    for (int a = 0; a < chi; ++a)
      for (int i = 0; i < d; ++i)
        g1[a + (size_t)chi * i + n * b] =
            (fabs(l0[a]) > GUARD_DENSE) ? u[((size_t)i * chi + a) + n * b] / l0[a] : 0.0;
}

/* FormGamma2 (:406-428): Gamma2(alpha,i,beta) = VT(alpha, (i-1)chi+beta)/Lambda2(beta) */
static void form_gamma2(int chi, int d, zc *g2, const double *l2, const zc *vt) {
  const size_t n = (size_t)chi * d;
  for (int b = 0; b < chi; ++b)
    for (int a = 0; a < chi; ++a)
      for (int i = 0; i < d; ++i)
        g2[a + (size_t)chi * i + n * b] =
            (fabs(l2[b]) > GUARD_DENSE) ? vt[a + n * ((size_t)i * chi + b)] / l2[b] : 0.0;
}

/* TwoSiteOp_c (:463-494) / TwoSiteOp_r (:430-461) on one bond.  Exactly one of
 * op_c / op_r is non-NULL.  Optionally returns all d*chi singular values of the
 * normalised Theta in s_out (may be NULL). */
int oracle_two_site_op(int chi, int d, double *g1_, double *g2_, const double *l0, double *l1,
                       const double *l2, const double *op_c_, const double *op_r, double *truncerr,
                       double *s_out) {
  if (chi < 1 || d < 1 || (!op_c_ && !op_r)) return OR_ERR_ARG;
  zc *g1 = (zc *)g1_, *g2 = (zc *)g2_;
  const zc *op_c = (const zc *)op_c_;
  const int n = chi * d;
  const size_t nn = (size_t)n * n;
  zc *theta = (zc *)malloc(sizeof(zc) * nn);
  zc *rs = (zc *)malloc(sizeof(zc) * nn);
  zc *u = (zc *)malloc(sizeof(zc) * nn);
  zc *vt = (zc *)malloc(sizeof(zc) * nn);
  double *s = (double *)malloc(sizeof(double) * n);
  int st = OR_ERR_ALLOC;
  if (theta && rs && u && vt && s) {
    form_theta(chi, d, theta, l0, g1, l1, g2, l2);
    theta_operation(chi, d, theta, op_c, op_r);
    reshape_theta(chi, d, theta, rs);
    st = zgesvd_all(n, n, rs, s, u, vt, 5 * n, 5 * n);
    if (st == OR_OK) {
      form_lambda1(chi, l1, truncerr, s);
      form_gamma1(chi, d, l0, g1, u);
      form_gamma2(chi, d, g2, l2, vt);
      if (s_out) memcpy(s_out, s, sizeof(double) * n);
    }
  }
  free(theta);
  free(rs);
  free(u);
  free(vt);
  free(s);
  return st;
}

/* Swapping (:651-689): Theta without a gate or normalisation, physical indices
 * exchanged by SwapTheta (:624-648): ThetaSW((j-1)chi+alpha, (i-1)chi+gamma) =
 * Theta(alpha,i,j,gamma); then SVDTruncation, FormLambda1, FormGamma1/2. */
int oracle_swapping(int chi, int d, double *g1_, double *g2_, const double *l0, double *l1,
                    const double *l2, double *truncerr) {
  if (chi < 1 || d < 1) return OR_ERR_ARG;
  zc *g1 = (zc *)g1_, *g2 = (zc *)g2_;
  const int n = chi * d;
  const size_t nn = (size_t)n * n;
  zc *theta = (zc *)malloc(sizeof(zc) * nn);
  zc *sw = (zc *)malloc(sizeof(zc) * nn);
  zc *u = (zc *)malloc(sizeof(zc) * nn);
  zc *vt = (zc *)malloc(sizeof(zc) * nn);
  double *s = (double *)malloc(sizeof(double) * n);
  int st = OR_ERR_ALLOC;
  if (theta && sw && u && vt && s) {
    form_theta(chi, d, theta, l0, g1, l1, g2, l2);
    for (int a = 0; a < chi; ++a)
      for (int g = 0; g < chi; ++g)
        for (int i = 0; i < d; ++i)
          for (int j = 0; j < d; ++j)
            sw[((size_t)j * chi + a) + (size_t)n * ((size_t)i * chi + g)] =
                theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * g))];
    st = zgesvd_all(n, n, sw, s, u, vt, 5 * n, 5 * n);
    if (st == OR_OK) {
      form_lambda1(chi, l1, truncerr, s);
      form_gamma1(chi, d, l0, g1, u);
      form_gamma2(chi, d, g2, l2, vt);
    }
  }
  free(theta);
  free(sw);
  free(u);
  free(vt);
  free(s);
  return st;
}

/* CanonicalForm (:496-610): loop for loop, with ZGESVD('A','A') on the chi x chi
 * matrices (SVD :612-622; workspaces 5 chi as SVDInit :84-122 sets them). */
int oracle_canonical_form(int chi, int d, const double *l0, double *g1_, double *l1, double *g2_,
                          const double *l2) {
  zc *g1 = (zc *)g1_, *g2 = (zc *)g2_;
  const size_t cc = (size_t)chi * chi, gs = (size_t)chi * d * chi;
  zc *M = (zc *)malloc(sizeof(zc) * cc), *X = (zc *)malloc(sizeof(zc) * cc), *Y = (zc *)malloc(sizeof(zc) * cc);
  zc *U = (zc *)malloc(sizeof(zc) * cc), *VT = (zc *)malloc(sizeof(zc) * cc);
  zc *g1t = (zc *)malloc(sizeof(zc) * gs), *g2t = (zc *)malloc(sizeof(zc) * gs);
  double *S = (double *)malloc(sizeof(double) * chi);
  int st = OR_ERR_ALLOC;
  if (!(M && X && Y && U && VT && g1t && g2t && S)) goto done;
#define G1(a, i, b) g1[(a) + (size_t)chi * ((i) + (size_t)d * (b))]
#define G2(a, i, b) g2[(a) + (size_t)chi * ((i) + (size_t)d * (b))]
#define T1(a, i, b) g1t[(a) + (size_t)chi * ((i) + (size_t)d * (b))]
#define T2(a, i, b) g2t[(a) + (size_t)chi * ((i) + (size_t)d * (b))]
#define MM(a, b) M[(a) + (size_t)chi * (b)]
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b) {
      zc acc = 0.0;
      for (int i = 0; i < d; ++i)
        for (int g = 0; g < chi; ++g) acc = acc + conj(G1(g, i, a)) * l0[g] * l0[g] * G1(g, i, b);
      MM(a, b) = acc;
    }
  if ((st = zgesvd_all(chi, chi, M, S, U, VT, 5 * chi, 5 * chi)) != OR_OK) goto done;
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i) {
        zc acc = 0.0;
        if (S[b] > GUARD_CANON)
          for (int g = 0; g < chi; ++g) acc = acc + G1(a, i, g) * U[g + (size_t)chi * b] * (1.0 / sqrt(S[b]));
        T1(a, i, b) = acc;
      }
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b) X[a + (size_t)chi * b] = sqrt(S[a]) * conj(U[b + (size_t)chi * a]);
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b) {
      zc acc = 0.0;
      for (int i = 0; i < d; ++i)
        for (int g = 0; g < chi; ++g) acc = acc + G2(a, i, g) * l2[g] * l2[g] * conj(G2(b, i, g));
      MM(a, b) = acc;
    }
  if ((st = zgesvd_all(chi, chi, M, S, U, VT, 5 * chi, 5 * chi)) != OR_OK) goto done;
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i) {
        zc acc = 0.0;
        if (S[a] > GUARD_CANON)
          for (int g = 0; g < chi; ++g) acc = acc + (1.0 / sqrt(S[a])) * conj(U[g + (size_t)chi * a]) * G2(g, i, b);
        T2(a, i, b) = acc;
      }
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b) Y[a + (size_t)chi * b] = l1[a] * U[a + (size_t)chi * b] * sqrt(S[b]);
  for (int a = 0; a < chi; ++a) /* M = MATMUL(X, Y) */
    for (int b = 0; b < chi; ++b) {
      zc acc = 0.0;
      for (int g = 0; g < chi; ++g) acc = acc + X[a + (size_t)chi * g] * Y[g + (size_t)chi * b];
      MM(a, b) = acc;
    }
  if ((st = zgesvd_all(chi, chi, M, S, U, VT, 5 * chi, 5 * chi)) != OR_OK) goto done;
  {
    double normsq = 0.0;
    for (int a = 0; a < chi; ++a) normsq = normsq + S[a] * S[a];
    for (int a = 0; a < chi; ++a) l1[a] = S[a] / sqrt(normsq);
  }
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i) {
        zc acc = 0.0;
        for (int g = 0; g < chi; ++g) acc = acc + T1(a, i, g) * U[g + (size_t)chi * b];
        G1(a, i, b) = acc;
      }
  for (int a = 0; a < chi; ++a)
    for (int b = 0; b < chi; ++b)
      for (int i = 0; i < d; ++i) {
        zc acc = 0.0;
        for (int g = 0; g < chi; ++g) acc = acc + VT[a + (size_t)chi * g] * T2(g, i, b);
        G2(a, i, b) = acc;
      }
#undef G1
#undef G2
#undef T1
#undef T2
#undef MM
done:
  free(M);
  free(X);
  free(Y);
  free(U);
  free(VT);
  free(g1t);
  free(g2t);
  free(S);
  return st;
}

/* ------------------------------------------------------------------------- */
/* Number-conserving update (U(1) labels)                                     */
/* ------------------------------------------------------------------------- */

/* Internal degrees of freedom.  The reference passes the OPTIONAL argument
 * intDegFree to every NC routine and reads the particle number of local state i
 * from the module global Conserv%vi(i) (set by the Hamiltonian builders, e.g.
 * fermi_hubbard_module.f90:230-232).  Here oracle_set_conserv(d, conserv) plays
 * both parts: a non-NULL table selects the intDegFree branches, NULL the plain
 * ones (local number i-1). */
static int g_idf = 0;
static int g_cons[64];

int oracle_set_conserv(int d, const int *conserv) {
  if (!conserv) {
    g_idf = 0;
    return OR_OK;
  }
  if (d < 1 || d > 64) return OR_ERR_ARG;
  for (int i = 0; i < d; ++i) g_cons[i] = conserv[i];
  g_idf = 1;
  return OR_OK;
}

/* particle number of local state i (0-based) */
static int nloc(int i) { return g_idf ? g_cons[i] : i; }

typedef struct {
  int nb;              /* number of blocks maxNL-minNL+1                       */
  int *rows, *cols;    /* BlockSize(k,2), BlockSize(k,3)                       */
  int *roff, *coff;    /* prefix offsets into the flat index lists             */
  int *l_alpha, *l_i;  /* indL(k)%mi(:,1:2) flattened by block                 */
  int *r_gamma, *r_j;  /* indR(k)%mi(:,1:2) flattened by block                 */
} nc_blocks;

static void nc_free(nc_blocks *b) {
  free(b->rows);
  free(b->cols);
  free(b->roff);
  free(b->coff);
  free(b->l_alpha);
  free(b->l_i);
  free(b->r_gamma);
  free(b->r_j);
}

/* FormThetaNC (:748-851).  ll0=LabelLeft(link), ll1=LabelLeft(link+1),
 * lr1=LabelRight(link+1), lr2=LabelRight(link+2). */
static void form_theta_nc(int chi, int d, int maxFilling, zc *theta, const double *l0, const zc *g1,
                          const double *l1, const zc *g2, const double *l2, const int *ll0,
                          const int *ll1, const int *lr1, const int *lr2) {
  const size_t sg = (size_t)chi * d;
  memset(theta, 0, sizeof(zc) * (size_t)chi * d * d * chi);
  if (g_idf) {
    /* FormThetaNC (:772-818), intDegFree present: sum over the local states
     * whose numbers close the label differences */
    for (int a = 0; a < chi; ++a)
      for (int g = 0; g < chi; ++g)
        for (int b = 0; b < chi; ++b)
          for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) {
              const int ni = g_cons[i], nj = g_cons[j];
              const int lftN1 = ll0[a], lftN2 = ll1[b], rgtN1 = lr2[g], rgtN2 = lr1[b];
              int mx = lftN1;
              if (lftN2 > mx) mx = lftN2;
              if (rgtN1 > mx) mx = rgtN1;
              if (rgtN2 > mx) mx = rgtN2;
              if (mx < 1000 && lftN2 - lftN1 <= maxFilling && lftN2 - lftN1 >= 0 &&
                  rgtN2 - rgtN1 <= maxFilling && rgtN2 - rgtN1 >= 0 && lftN1 + ni == lftN2 &&
                  rgtN1 + nj == rgtN2) {
                zc *t = &theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * g))];
                *t = *t + l0[a] * g1[a + (size_t)chi * i + sg * b] * l1[b] *
                              g2[b + (size_t)chi * j + sg * g] * l2[g];
              }
            }
    return;
  }
  for (int a = 0; a < chi; ++a)
    for (int g = 0; g < chi; ++g)
      for (int b = 0; b < chi; ++b) {
        const int lftN1 = ll0[a], lftN2 = ll1[b], rgtN1 = lr2[g], rgtN2 = lr1[b];
        int mx = lftN1;
        if (lftN2 > mx) mx = lftN2;
        if (rgtN1 > mx) mx = rgtN1;
        if (rgtN2 > mx) mx = rgtN2;
        const int i1 = lftN2 - lftN1 + 1, j1 = rgtN2 - rgtN1 + 1; /* 1-based */
        if (mx < 1000 && i1 <= d && i1 >= 1 && j1 <= d && j1 >= 1) {
          const int i = i1 - 1, j = j1 - 1;
          zc *t = &theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * g))];
          *t = *t + l0[a] * g1[a + (size_t)chi * i + sg * b] * l1[b] *
                        g2[b + (size_t)chi * j + sg * g] * l2[g];
        }
      }
}

/* ThetaOperationNC_c / _r (:950-1044 / :853-948) */
static void theta_operation_nc(int chi, int d, int totNum, int maxFilling, zc *theta,
                               const zc *op_c, const double *op_r, const int *ll0,
                               const int *lr2) {
  const size_t nt = (size_t)chi * d * d * chi;
  const int d2 = d * d;
  zc *tmp = (zc *)calloc(nt, sizeof(zc));
  if (g_idf) {
    /* intDegFree present (:970-1010): every (k, j) with n_k + n_j = totNum - lftN - rgtN */
    for (int a = 0; a < chi; ++a)
      for (int k = 0; k < d; ++k)
        for (int j = 0; j < d; ++j)
          for (int g = 0; g < chi; ++g) {
            const int nk = g_cons[k], nj = g_cons[j];
            const int lftN = ll0[a], rgtN = lr2[g];
            const int mx = lftN > rgtN ? lftN : rgtN;
            const int rest = totNum - lftN - rgtN - nk;
            if (mx < 1000 && rest >= 0 && rest <= maxFilling && nj == rest) {
              zc acc = 0.0;
              for (int i = 0; i < d; ++i)
                for (int l = 0; l < d; ++l) {
                  const int ni = g_cons[i], nl = g_cons[l];
                  const int ri = totNum - lftN - rgtN - ni;
                  if (ri >= 0 && ri <= maxFilling && nl == ri) {
                    const size_t oi = (size_t)(k * d + j) + (size_t)d2 * (i * d + l);
                    const zc op = op_c ? op_c[oi] : (zc)op_r[oi];
                    acc = acc + op * theta[a + (size_t)chi * (i + (size_t)d * (l + (size_t)d * g))];
                  }
                }
              tmp[a + (size_t)chi * (k + (size_t)d * (j + (size_t)d * g))] = acc;
            }
          }
    memcpy(theta, tmp, sizeof(zc) * nt);
    free(tmp);
    return;
  }
  for (int a = 0; a < chi; ++a)
    for (int k = 1; k <= d; ++k)
      for (int g = 0; g < chi; ++g) {
        const int lftN = ll0[a], rgtN = lr2[g];
        const int mx = lftN > rgtN ? lftN : rgtN;
        const int nk = totNum - lftN - rgtN - k + 1;
        if (mx < 1000 && nk >= 0 && nk <= maxFilling) {
          const int jj = totNum - lftN - rgtN - k + 2; /* 1-based */
          zc acc = 0.0;
          for (int i = 1; i <= d; ++i) {
            const int ni = totNum - lftN - rgtN - i + 1;
            if (ni >= 0 && ni <= maxFilling) {
              const int ll = totNum - lftN - rgtN - i + 2; /* 1-based */
              const size_t oi = (size_t)((k - 1) * d + jj - 1) + (size_t)d2 * ((i - 1) * d + ll - 1);
              const zc op = op_c ? op_c[oi] : (zc)op_r[oi];
              acc = acc + op * theta[a + (size_t)chi * ((i - 1) + (size_t)d * ((ll - 1) + (size_t)d * g))];
            }
          }
          tmp[a + (size_t)chi * ((k - 1) + (size_t)d * ((jj - 1) + (size_t)d * g))] = acc;
        }
      }
  memcpy(theta, tmp, sizeof(zc) * nt);
  free(tmp);
}

/* RenormThetaNC (:1046-1129) */
static void renorm_theta_nc(int chi, int d, int totNum, int maxFilling, zc *theta, const int *ll0,
                            const int *lr2) {
  zc nsq = 0.0;
  if (g_idf) {
    /* intDegFree present (:1062-1102) */
    for (int pass = 0; pass < 2; ++pass) {
      const double norm = sqrt(creal(nsq));
      for (int a = 0; a < chi; ++a)
        for (int g = 0; g < chi; ++g) {
          const int lftN = ll0[a], rgtN = lr2[g];
          for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) {
              const int ni = g_cons[i], nj = g_cons[j];
              const int r = totNum - lftN - rgtN - ni;
              if ((lftN > rgtN ? lftN : rgtN) < 1000 && r >= 0 && r <= maxFilling && nj == r) {
                zc *t = &theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * g))];
                if (pass == 0)
                  nsq = nsq + conj(*t) * *t;
                else
                  *t = *t / norm;
              }
            }
        }
    }
    return;
  }
  for (int a = 0; a < chi; ++a)
    for (int g = 0; g < chi; ++g) {
      const int lftN = ll0[a], rgtN = lr2[g];
      for (int i = 1; i <= d; ++i) {
        const int ni = totNum - lftN - rgtN - i + 1;
        if ((lftN > rgtN ? lftN : rgtN) < 1000 && ni >= 0 && ni <= maxFilling) {
          const zc t = theta[a + (size_t)chi * ((i - 1) + (size_t)d * ((ni) + (size_t)d * g))];
          nsq = nsq + conj(t) * t;
        }
      }
    }
  const double norm = sqrt(creal(nsq));
  for (int a = 0; a < chi; ++a)
    for (int g = 0; g < chi; ++g) {
      const int lftN = ll0[a], rgtN = lr2[g];
      for (int i = 1; i <= d; ++i) {
        const int ni = totNum - lftN - rgtN - i + 1;
        if ((lftN > rgtN ? lftN : rgtN) < 1000 && ni >= 0 && ni <= maxFilling) {
          zc *t = &theta[a + (size_t)chi * ((i - 1) + (size_t)d * ((ni) + (size_t)d * g))];
          *t = *t / norm;
        }
      }
    }
}

/* minmaxNLR (:1201-1250) */
static void minmax_nlr(int chi, int totNum, int maxFilling, const int *ll0, const int *lr2,
                       int *minNL, int *maxNL, int *minNR, int *maxNR) {
  int mnl = ll0[0], mxl = 0, mnr = lr2[0], mxr = 0;
  for (int a = 0; a < chi; ++a) {
    if (ll0[a] < mnl) mnl = ll0[a];
    const int l0v = ll0[a] == LABEL_UNUSED ? 0 : ll0[a];
    if (a == 0 || l0v > mxl) mxl = l0v;
  }
  for (int g = 0; g < chi; ++g) {
    if (lr2[g] < mnr) mnr = lr2[g];
    const int r0v = lr2[g] == LABEL_UNUSED ? 0 : lr2[g];
    if (g == 0 || r0v > mxr) mxr = r0v;
  }
  mxl += maxFilling;
  mxr += maxFilling;
  if (mxl > totNum - mnr)
    mxl = totNum - mnr;
  else
    mnr = totNum - mxl;
  if (mxr > totNum - mnl)
    mxr = totNum - mnl;
  else
    mnl = totNum - mxr;
  *minNL = mnl;
  *maxNL = mxl;
  *minNR = mnr;
  *maxNR = mxr;
}

/* SizeOfBlocks (:1252-1336) + IndexLeft (:1339-1391) + IndexRight (:1393-1443);
 * the local number is i-1, or Conserv(i) with intDegFree.  Returns OR_ERR_ARG if
 * a block index falls outside [1, nb] (the reference would write out of bounds
 * there). */
static int build_blocks(int chi, int d, int totNum, int minNL, int maxNL, int minNR, int maxNR,
                        const int *ll0, const int *lr2, nc_blocks *B) {
  memset(B, 0, sizeof(*B));
  const int nb = maxNL - minNL + 1;
  if (nb < 1) return OR_ERR_ARG;
  B->nb = nb;
  B->rows = (int *)calloc(nb, sizeof(int));
  B->cols = (int *)calloc(nb, sizeof(int));
  B->roff = (int *)calloc(nb + 1, sizeof(int));
  B->coff = (int *)calloc(nb + 1, sizeof(int));
  const size_t cap = (size_t)chi * d;
  B->l_alpha = (int *)malloc(sizeof(int) * cap);
  B->l_i = (int *)malloc(sizeof(int) * cap);
  B->r_gamma = (int *)malloc(sizeof(int) * cap);
  B->r_j = (int *)malloc(sizeof(int) * cap);
  if (!B->rows || !B->cols || !B->roff || !B->coff || !B->l_alpha || !B->l_i || !B->r_gamma || !B->r_j)
    return OR_ERR_ALLOC;
  for (int a = 0; a < chi; ++a)
    for (int i = 1; i <= d; ++i)
      if (ll0[a] < 1000) {
        const int NL = ll0[a] + nloc(i - 1);
        if (minNL <= NL && NL <= maxNL) B->rows[NL - minNL]++;
      }
  for (int g = 0; g < chi; ++g)
    for (int j = 1; j <= d; ++j)
      if (lr2[g] < 1000) {
        const int NR = lr2[g] + nloc(j - 1);
        if (minNR <= NR && NR <= maxNR) {
          const int k = totNum - NR - minNL;
          if (k < 0 || k >= nb) return OR_ERR_ARG;
          B->cols[k]++;
        }
      }
  for (int k = 0; k < nb; ++k) {
    B->roff[k + 1] = B->roff[k] + B->rows[k];
    B->coff[k + 1] = B->coff[k] + B->cols[k];
  }
  int *turn = (int *)calloc(nb, sizeof(int));
  if (!turn) return OR_ERR_ALLOC;
  for (int a = 0; a < chi; ++a)
    for (int i = 1; i <= d; ++i)
      if (ll0[a] < 1000 && minNL <= ll0[a] + nloc(i - 1) && ll0[a] + nloc(i - 1) <= maxNL) {
        const int k = ll0[a] + nloc(i - 1) - minNL;
        const int p = B->roff[k] + turn[k]++;
        B->l_alpha[p] = a;
        B->l_i[p] = i - 1;
      }
  memset(turn, 0, sizeof(int) * nb);
  for (int g = 0; g < chi; ++g)
    for (int j = 1; j <= d; ++j)
      if (lr2[g] < 1000 && minNR <= lr2[g] + nloc(j - 1) && lr2[g] + nloc(j - 1) <= maxNR) {
        const int k = totNum - (lr2[g] + nloc(j - 1)) - minNL;
        const int p = B->coff[k] + turn[k]++;
        B->r_gamma[p] = g;
        B->r_j[p] = j - 1;
      }
  free(turn);
  return OR_OK;
}

/* Ordering (:1515-1538): repeatedly take MINLOC (first occurrence) and place it
 * at the back.  Equal values therefore end up in descending index order. */
static void ordering(int sz, const double *arr, int *order /* 1-based values */) {
  double *def = (double *)malloc(sizeof(double) * (sz > 0 ? sz : 1));
  double mxv = -HUGE_VAL;
  for (int t = 0; t < sz; ++t) {
    def[t] = arr[t];
    if (arr[t] > mxv) mxv = arr[t];
  }
  /* MaxElement is declared INTEGER in the reference: the REAL maximum is truncated. */
  const int maxElement = sz > 0 ? (int)mxv : 0;
  for (int beta = sz - 1; beta >= 0; --beta) {
    int loc = 0;
    for (int t = 1; t < sz; ++t)
      if (def[t] < def[loc]) loc = t;
    order[beta] = loc + 1;
    def[loc] = (double)maxElement + 10.0;
  }
  free(def);
}

/* SwapThetaNC (:1144-1250): exchange the two physical indices on the allowed
 * entries (i, j) of each (alpha, gamma).  Without intDegFree the swapped array
 * starts from zero; with it the reference leaves the other entries unset, and
 * none of them is read afterwards when Conserv lies in [0, maxFilling]. */
static void swap_theta_nc(int chi, int d, int totNum, int maxFilling, zc *theta, const int *ll0,
                          const int *lr2) {
  const size_t nt = (size_t)chi * d * d * chi;
  zc *sw = (zc *)calloc(nt, sizeof(zc));
  for (int a = 0; a < chi; ++a)
    for (int g = 0; g < chi; ++g) {
      const int lftN = ll0[a], rgtN = lr2[g];
      if ((lftN > rgtN ? lftN : rgtN) >= 1000) continue;
      if (g_idf) {
        for (int i = 0; i < d; ++i)
          for (int j = 0; j < d; ++j) {
            const int r = totNum - lftN - rgtN - g_cons[i];
            if (r >= 0 && r <= maxFilling && g_cons[j] == r)
              sw[a + (size_t)chi * (j + (size_t)d * (i + (size_t)d * g))] =
                  theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * g))];
          }
      } else {
        for (int i = 1; i <= d; ++i) {
          const int r = totNum - lftN - rgtN - i + 1;
          if (r >= 0 && r <= maxFilling) {
            const int j = totNum - lftN - rgtN - i + 2; /* 1-based */
            sw[a + (size_t)chi * ((j - 1) + (size_t)d * ((i - 1) + (size_t)d * g))] =
                theta[a + (size_t)chi * ((i - 1) + (size_t)d * ((j - 1) + (size_t)d * g))];
          }
        }
      }
    }
  memcpy(theta, sw, sizeof(zc) * nt);
  free(sw);
}

static int nc_core(int chi, int d, int totNum, int maxFilling, double *g1_, double *g2_,
                   const double *l0, double *l1, const double *l2, const double *op_c_,
                   const double *op_r, const int *ll0, int *ll1, int *lr1, const int *lr2,
                   double *truncerr, double *s_out, int *sz_out, int swap);

/* TwoSiteOpNC_c (:1845-1964; intDegFree as set by oracle_set_conserv).  Labels are updated in place
 * for link+1.  Optional s_out receives the flattened block singular values
 * (ssflat) and *sz_out their count. */
int oracle_two_site_op_nc(int chi, int d, int totNum, int maxFilling, double *g1_, double *g2_,
                          const double *l0, double *l1, const double *l2, const double *op_c_,
                          const double *op_r, const int *ll0, int *ll1, int *lr1, const int *lr2,
                          double *truncerr, double *s_out, int *sz_out) {
  if (!op_c_ && !op_r) return OR_ERR_ARG;
  return nc_core(chi, d, totNum, maxFilling, g1_, g2_, l0, l1, l2, op_c_, op_r, ll0, ll1, lr1, lr2,
                 truncerr, s_out, sz_out, 0);
}

/* SwappingNC (:1966-2095): FormThetaNC, SwapThetaNC, then the block SVD and the
 * label / Lambda / Gamma updates of TwoSiteOpNC, without RenormThetaNC. */
int oracle_swapping_nc(int chi, int d, int totNum, int maxFilling, double *g1_, double *g2_,
                       const double *l0, double *l1, const double *l2, const int *ll0, int *ll1,
                       int *lr1, const int *lr2, double *truncerr) {
  return nc_core(chi, d, totNum, maxFilling, g1_, g2_, l0, l1, l2, 0, 0, ll0, ll1, lr1, lr2, truncerr,
                 0, 0, 1);
}

static int nc_core(int chi, int d, int totNum, int maxFilling, double *g1_, double *g2_,
                   const double *l0, double *l1, const double *l2, const double *op_c_,
                   const double *op_r, const int *ll0, int *ll1, int *lr1, const int *lr2,
                   double *truncerr, double *s_out, int *sz_out, int swap) {
  if (chi < 1 || d < 1) return OR_ERR_ARG;
  zc *g1 = (zc *)g1_, *g2 = (zc *)g2_;
  const zc *op_c = (const zc *)op_c_;
  const size_t nt = (size_t)chi * d * d * chi;
  zc *theta = (zc *)malloc(sizeof(zc) * nt);
  if (!theta) return OR_ERR_ALLOC;
  form_theta_nc(chi, d, maxFilling, theta, l0, g1, l1, g2, l2, ll0, ll1, lr1, lr2);
  if (swap) {
    swap_theta_nc(chi, d, totNum, maxFilling, theta, ll0, lr2);
  } else {
    theta_operation_nc(chi, d, totNum, maxFilling, theta, op_c, op_r, ll0, lr2);
    renorm_theta_nc(chi, d, totNum, maxFilling, theta, ll0, lr2);
  }
  int minNL, maxNL, minNR, maxNR;
  minmax_nlr(chi, totNum, maxFilling, ll0, lr2, &minNL, &maxNL, &minNR, &maxNR);
  nc_blocks B;
  int st = build_blocks(chi, d, totNum, minNL, maxNL, minNR, maxNR, ll0, lr2, &B);
  if (st != OR_OK) {
    nc_free(&B);
    free(theta);
    return st;
  }
  if (B.nb < 1) { /* build_blocks returns an error first; kept explicit for the allocations */
    nc_free(&B);
    free(theta);
    return OR_ERR_ARG;
  }
  /* per-block SVD (FormBlockTheta :1445-1468, SVDNC :1470-1492) */
  int sz = 0;
  for (int k = 0; k < B.nb; ++k) sz += B.rows[k] < B.cols[k] ? B.rows[k] : B.cols[k];
  double *ssfl = (double *)calloc(sz > 0 ? sz : 1, sizeof(double));
  zc **US = (zc **)calloc(B.nb, sizeof(zc *));
  zc **VS = (zc **)calloc(B.nb, sizeof(zc *));
  int *soff = (int *)calloc(B.nb + 1, sizeof(int));
  for (int k = 0; k < B.nb && st == OR_OK; ++k) {
    const int m = B.rows[k], n = B.cols[k], mn = m < n ? m : n;
    soff[k + 1] = soff[k] + mn;
    if (mn == 0) continue; /* an empty block contributes no singular values */
    zc *blk = (zc *)malloc(sizeof(zc) * (size_t)m * n);
    US[k] = (zc *)malloc(sizeof(zc) * (size_t)m * m);
    VS[k] = (zc *)malloc(sizeof(zc) * (size_t)n * n);
    for (int fa = 0; fa < m; ++fa)
      for (int fg = 0; fg < n; ++fg) {
        const int a = B.l_alpha[B.roff[k] + fa], i = B.l_i[B.roff[k] + fa];
        const int g = B.r_gamma[B.coff[k] + fg], j = B.r_j[B.coff[k] + fg];
        blk[fa + (size_t)m * fg] = theta[a + (size_t)chi * (i + (size_t)d * (j + (size_t)d * g))];
      }
    const int mxmn = m > n ? m : n;
    st = zgesvd_all(m, n, blk, &ssfl[soff[k]], US[k], VS[k], 5 * mxmn, 5 * mn);
    free(blk);
  }
  if (st == OR_OK) {
    int *order = (int *)malloc(sizeof(int) * (sz > 0 ? sz : 1));
    int *pos_b = (int *)malloc(sizeof(int) * (sz > 0 ? sz : 1));
    int *pos_p = (int *)malloc(sizeof(int) * (sz > 0 ? sz : 1));
    ordering(sz, ssfl, order);
    /* JudgePosition (:1540-1565) */
    for (int beta = 0; beta < sz; ++beta) {
      int ot = order[beta];
      pos_b[beta] = 0;
      pos_p[beta] = 0;
      for (int k = 0; k < B.nb; ++k) {
        if (ot <= 0) break;
        const int mn = B.rows[k] < B.cols[k] ? B.rows[k] : B.cols[k];
        ot -= mn;
        pos_b[beta] = k + 1;
        pos_p[beta] = ot + mn;
      }
    }
    /* UpdateLabelLeft (:1567-1605): order2(order(beta)) == beta <= chi always holds */
    for (int beta = 0; beta < chi; ++beta) {
      if (beta < sz)
        ll1[beta] = (ssfl[order[beta] - 1] > GUARD_NC) ? minNL + pos_b[beta] - 1 : LABEL_UNUSED;
      else
        ll1[beta] = LABEL_UNUSED;
    }
    /* UpdateLabelRight (:1607-1625) */
    for (int beta = 0; beta < chi; ++beta)
      lr1[beta] = ll1[beta] < 1000 ? totNum - ll1[beta] : LABEL_UNUSED;
    /* FormLambdaNC (:1627-1657) */
    double renorm = 0.0;
    double *tl = (double *)malloc(sizeof(double) * chi);
    for (int beta = 0; beta < chi; ++beta)
      tl[beta] = (beta < sz && ssfl[order[beta] - 1] > GUARD_NC) ? ssfl[order[beta] - 1] : 0.0;
    for (int beta = 0; beta < chi; ++beta) renorm = renorm + tl[beta] * tl[beta];
    *truncerr = fabs(1.0 - renorm);
    for (int beta = 0; beta < chi; ++beta) l1[beta] = tl[beta] / sqrt(renorm);
    free(tl);
    /* FormGamma1NC (:1659-1689) and FormGamma2NC (:1691-1721) */
    memset(g1, 0, sizeof(zc) * (size_t)chi * d * chi);
    memset(g2, 0, sizeof(zc) * (size_t)chi * d * chi);
    for (int beta = 0; beta < chi && beta < sz; ++beta) {
      const int k = pos_b[beta] - 1, psn = pos_p[beta] - 1;
      const int m = B.rows[k], n = B.cols[k];
      for (int fa = 0; fa < m; ++fa) {
        const int a = B.l_alpha[B.roff[k] + fa], i = B.l_i[B.roff[k] + fa];
        g1[a + (size_t)chi * i + (size_t)chi * d * beta] =
            (l0[a] > GUARD_NC) ? US[k][fa + (size_t)m * psn] / l0[a] : 0.0;
      }
      for (int fg = 0; fg < n; ++fg) {
        const int g = B.r_gamma[B.coff[k] + fg], j = B.r_j[B.coff[k] + fg];
        g2[beta + (size_t)chi * j + (size_t)chi * d * g] =
            (l2[g] > GUARD_NC) ? VS[k][psn + (size_t)n * fg] / l2[g] : 0.0;
      }
    }
    if (s_out) memcpy(s_out, ssfl, sizeof(double) * sz);
    if (sz_out) *sz_out = sz;
    free(order);
    free(pos_b);
    free(pos_p);
  }
  for (int k = 0; k < B.nb; ++k) {
    free(US[k]);
    free(VS[k]);
  }
  free(US);
  free(VS);
  free(soff);
  free(ssfl);
  nc_free(&B);
  free(theta);
  return st;
}

/* ------------------------------------------------------------------------- */
/* Trotter sweeps (open boundaries)                                           */
/* ------------------------------------------------------------------------- */

/* Gate index used for bond `link` (1-based) in sweep `s` of a step.
 * 2nd order (:82-114): sweeps odd, even, odd; gate Udt(link).
 * Forest-Ruth "5th order" (:200-252): sweeps odd,even,odd,even,odd,even,odd with
 * gates Udt(2(link-1)+1), (..+1), (..+2), (..+2), (..+2), (..+1), (..+1). */
static int sweep_count(int order) { return order == 2 ? 3 : 7; }
static int sweep_parity(int s) { return (s % 2 == 0) ? 1 : 2; } /* first link of the sweep */
static int sweep_gate(int order, int s, int link) {
  if (order == 2) return link;
  static const int pick[7] = {1, 1, 2, 2, 2, 1, 1};
  return 2 * (link - 1) + pick[s];
}

/* gammas[site-1], lambdas[link-1] (L+1 of them), gates[g-1] (complex d^2 x d^2). */
int oracle_trotter_step(int L, int chi, int d, int order, double **gammas, double **lambdas,
                        const double *const *gates, double *total_truncerr) {
  if (order != 2 && order != 5) return OR_ERR_ARG;
  double tot = 0.0;
  for (int s = 0; s < sweep_count(order); ++s)
    for (int link = sweep_parity(s); link <= L - 1; link += 2) {
      double te = 0.0;
      const int st = oracle_two_site_op(chi, d, gammas[link - 1], gammas[link], lambdas[link - 1],
                                        lambdas[link], lambdas[link + 1],
                                        gates[sweep_gate(order, s, link) - 1], 0, &te, 0);
      if (st != OR_OK) return st;
      tot += te;
    }
  *total_truncerr = tot;
  return OR_OK;
}

/* TrotterStep2ndOrderNC (:956-1018) and its 5th-order twin; labels[link-1] arrays. */
int oracle_trotter_step_nc(int L, int chi, int d, int totNum, int maxFilling, int order,
                           double **gammas, double **lambdas, int **label_left, int **label_right,
                           const double *const *gates, double *total_truncerr) {
  if (order != 2 && order != 5) return OR_ERR_ARG;
  double tot = 0.0;
  for (int s = 0; s < sweep_count(order); ++s)
    for (int link = sweep_parity(s); link <= L - 1; link += 2) {
      double te = 0.0;
      const int st = oracle_two_site_op_nc(
          chi, d, totNum, maxFilling, gammas[link - 1], gammas[link], lambdas[link - 1],
          lambdas[link], lambdas[link + 1], gates[sweep_gate(order, s, link) - 1], 0,
          label_left[link - 1], label_left[link], label_right[link], label_right[link + 1], &te, 0,
          0);
      if (st != OR_OK) return st;
      tot += te;
    }
  *total_truncerr = tot;
  return OR_OK;
}

/* Periodic-boundary steps.  One context carries the chain for the dense
 * routines (TwoSiteOp, Swapping) or the number-conserving ones (TwoSiteOpNC,
 * SwappingNC with the labels); the sequences are the reference's, which are the
 * same for both (propagation_module.f90:116-614 and 1019-1940).  The edge bond
 * (L,1) is applied on bond 1 after swapping site L down to site 2: the edge calls
 * of the NC Trotter routines pass the loop variable after
 * `DO i=systemSize-1,2,(-1)`, which is 1 there. */
typedef struct {
  int nc, chi, d, totNum, maxFilling;
  double **gammas, **lambdas;
  int **ll, **lr;
  const double *const *gates;
  double tot;
} pbc_ctx;

static int pbc_op(pbc_ctx *C, int link, int g) {
  double te = 0.0;
  int st;
  if (C->nc)
    st = oracle_two_site_op_nc(C->chi, C->d, C->totNum, C->maxFilling, C->gammas[link - 1],
                               C->gammas[link], C->lambdas[link - 1], C->lambdas[link],
                               C->lambdas[link + 1], C->gates[g - 1], 0, C->ll[link - 1], C->ll[link],
                               C->lr[link], C->lr[link + 1], &te, 0, 0);
  else
    st = oracle_two_site_op(C->chi, C->d, C->gammas[link - 1], C->gammas[link], C->lambdas[link - 1],
                            C->lambdas[link], C->lambdas[link + 1], C->gates[g - 1], 0, &te, 0);
  C->tot += te;
  return st;
}

static int pbc_sw(pbc_ctx *C, int link) {
  double te = 0.0;
  int st;
  if (C->nc)
    st = oracle_swapping_nc(C->chi, C->d, C->totNum, C->maxFilling, C->gammas[link - 1], C->gammas[link],
                            C->lambdas[link - 1], C->lambdas[link], C->lambdas[link + 1],
                            C->ll[link - 1], C->ll[link], C->lr[link], C->lr[link + 1], &te);
  else
    st = oracle_swapping(C->chi, C->d, C->gammas[link - 1], C->gammas[link], C->lambdas[link - 1],
                         C->lambdas[link], C->lambdas[link + 1], &te);
  C->tot += te;
  return st;
}

#define OP(link, g)                                 \
  do {                                              \
    if ((st = pbc_op(C, (link), (g))) != OR_OK) return st; \
  } while (0)
#define SW(link)                                    \
  do {                                              \
    if ((st = pbc_sw(C, (link))) != OR_OK) return st; \
  } while (0)
#define EDGE(g)                                   \
  do {                                            \
    for (int i = L - 1; i >= 2; --i) SW(i);       \
    OP(1, g);                                     \
    for (int i = 2; i <= L - 1; ++i) SW(i);       \
  } while (0)

/* TrotterStep2ndOrderPBC (:116-198) / TrotterStep2ndOrderPBCNC (:1019-1186):
 * gates[g-1] = Udt(g), g = 1..L, Udt(L) the edge. */
static int pbc2_run(pbc_ctx *C, int L) {
  int st;
  for (int i = 1; i <= L - 1; i += 2) OP(i, i);
  if (L % 2 == 1)
    for (int i = 2; i <= L - 1; i += 2) OP(i, i);
  EDGE(L);
  for (int i = 2; i <= L - 1; i += 2) OP(i, i);
  for (int i = 1; i <= L - 1; i += 2) OP(i, i);
  return OR_OK;
}

/* TrotterStep5thOrderPBC (:254-614) / TrotterStep5thOrderPBCNC (:1244-1940): the
 * Forest-Ruth sequence.  Gate layout (NEWConstructPropagators,
 * TEBDtools_module.f90:1149-1190): odd L -- odd bond i: Udt(3(i-1)+1..2), even
 * bond i: Udt(2+3(i-2)+1..4), edge: Udt(3(L-1)+1..3); even L -- bond i:
 * Udt(2(i-1)+1..2), edge Udt(2(L-1)+1..2).  gates[g-1] = Udt(g). */
static int pbc5_run(pbc_ctx *C, int L) {
  int st;
  if (L % 2 == 1) {
#define ODD3(v) for (int i = 1; i <= L - 1; i += 2) OP(i, 3 * (i - 1) + (v))
#define EVEN3(v) for (int i = 2; i <= L - 1; i += 2) OP(i, 2 + 3 * (i - 2) + (v))
#define EDGE3(v) EDGE(3 * (L - 1) + (v))
    ODD3(1);
    EVEN3(1); EDGE3(1); EVEN3(2); EDGE3(2); EVEN3(2); EDGE3(1); EVEN3(1);
    ODD3(2);
    EVEN3(3); EDGE3(2); EVEN3(4); EDGE3(3); EVEN3(4); EDGE3(2); EVEN3(3);
    ODD3(2);
    EVEN3(1); EDGE3(1); EVEN3(2); EDGE3(2); EVEN3(2); EDGE3(1); EVEN3(1);
    ODD3(1);
#undef ODD3
#undef EVEN3
#undef EDGE3
  } else {
#define ODD2(v) for (int i = 1; i <= L - 1; i += 2) OP(i, 2 * (i - 1) + (v))
#define EVEN2(v) for (int i = 2; i <= L - 1; i += 2) OP(i, 2 * (i - 1) + (v))
#define EDGE2(v) EDGE(2 * (L - 1) + (v))
    ODD2(1); EDGE2(1); EVEN2(1);
    ODD2(2); EDGE2(2); EVEN2(2);
    ODD2(2); EDGE2(1); EVEN2(1);
    ODD2(1);
#undef ODD2
#undef EVEN2
#undef EDGE2
  }
  return OR_OK;
}
#undef OP
#undef SW
#undef EDGE

int oracle_trotter_step_pbc(int L, int chi, int d, double **gammas, double **lambdas,
                            const double *const *gates, double *total_truncerr) {
  pbc_ctx C = {0, chi, d, 0, 0, gammas, lambdas, 0, 0, gates, 0.0};
  const int st = pbc2_run(&C, L);
  *total_truncerr = C.tot;
  return st;
}

int oracle_trotter_step_pbc5(int L, int chi, int d, double **gammas, double **lambdas,
                             const double *const *gates, double *total_truncerr) {
  pbc_ctx C = {0, chi, d, 0, 0, gammas, lambdas, 0, 0, gates, 0.0};
  const int st = pbc5_run(&C, L);
  *total_truncerr = C.tot;
  return st;
}

/* Number-conserving periodic steps (intDegFree as set by oracle_set_conserv). */
int oracle_trotter_step_pbc_nc(int L, int chi, int d, int totNum, int maxFilling, int order,
                               double **gammas, double **lambdas, int **label_left, int **label_right,
                               const double *const *gates, double *total_truncerr) {
  if (order != 2 && order != 5) return OR_ERR_ARG;
  pbc_ctx C = {1, chi, d, totNum, maxFilling, gammas, lambdas, label_left, label_right, gates, 0.0};
  const int st = order == 2 ? pbc2_run(&C, L) : pbc5_run(&C, L);
  *total_truncerr = C.tot;
  return st;
}
