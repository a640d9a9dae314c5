// nc.cu -- number-conserving (U(1) block-sparse) two-site update on the GPU.
//
// Replaces TwoSiteOpNC_c/_r, with or without internal degrees of freedom
// (VidalCore_v_2.0/local_operations_module.f90:748-1964) for a batch of
// same-parity bonds:
//   minmaxNLR :1201, SizeOfBlocks :1252, IndexLeft/Right :1339/:1393   -> k_nc_blocks
//   FormThetaNC :748, ThetaOperationNC :853/:950, RenormThetaNC :1046,
//   FormBlockTheta :1445                                                -> k_nc_theta
//     (theta form 103..107: FormThetaNC per charge block on the tensor cores,
//      k_nc_sizes / k_nc_oz_pack / k_tc_oz, then the rest in k_nc_mix)
//   SVDNC :1470 (one ZGESVD per block)                                  -> persistent Jacobi
//                                     (blocks with both sides >= 64: bidiagonalisation)
//   FlattenSS :1494, Ordering :1515, JudgePosition :1540,
//   UpdateLabelLeft/Right :1567/:1607, FormLambdaNC :1627               -> k_nc_select
//   FormGamma1NC :1659, FormGamma2NC :1691                               -> k_nc_gamma
//
// Structure.  Labels fix the physical indices: for Schmidt indices alpha (left,
// label a = LabelLeft(link)) and gamma (right, c = LabelRight(link+2)) the
// allowed entries of Theta have i + j = n_tot + 2 with n_tot = totNum - a - c,
// and FormThetaNC sums only the beta whose labels LabelLeft(link+1) = a+i-1 and
// LabelRight(link+1) = c+j-1.  Betas are therefore grouped by left label (a
// counting sort), and each allowed (alpha, i, gamma) entry is a short dot
// product over one class.  The gate mixes the <= d allowed entries of one
// (alpha, gamma) pair (ThetaOperationNC), and the result is written straight
// into the charge blocks (block k: left number minNL+k, rows (alpha,i) in
// IndexLeft order, columns (gamma,j) in IndexRight order).  Every block entry is
// an allowed entry, so no block needs clearing.  Blocks with fewer rows than
// columns are stored conjugate-transposed so the one-sided Jacobi always works
// on the narrow side.
//
// Internal degrees of freedom (intDegFree present, tebd_set_conserv): local state
// i carries Conserv(i) particles instead of i-1, so several (i, j) pairs share one
// pair total n_i + n_j.  The block bookkeeping reads the table; the Theta kernel
// runs a second form that lists the allowed pairs of each (alpha, gamma) in the
// reference's loop order (i outer, j inner) and mixes them with the gate.
//
// Guards and the sentinel are the reference's: labels >= 1000 are unused,
// 10000 is written for unused indices, and `10.0**(-10)` (single precision)
// decides kept singular values and the Lambda divisions.
#include <math.h>
#include <stddef.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <map>
#include <vector>

#include "df.cuh"
#include "oz_digits.cuh"
#include "tc_gemm.cuh"
#include "tebd_internal.cuh"

namespace tebd {

int run_jacobi_problems(tebd_handle *h, const JacobiProblem<double> *probs_d, int nprob, int nmax);

namespace {

// header fields of one slot
enum { H_NB = 0, H_MINNL, H_MAXNL, H_MINNR, H_MAXNR, H_SZ, H_MAXDIM, H_ERR, H_COUNT };

struct NcSlot {
  int *hdr;                       // H_COUNT ints
  int *rows, *cols;               // per block (B_max)
  int *roff, *coff;               // B_max + 1 prefix offsets into the index lists
  int *boffx, *boffv, *soff;      // B_max + 1 offsets: X elements, V elements, flat sigma
  int *l_alpha, *l_i, *r_gamma, *r_j;  // index lists (d*chi each)
  int *rowpos, *colpos;           // (alpha,i) -> block-local row / (gamma,j) -> local column, -1 if none
  int *cls_off, *cls_beta;        // betas sorted by LabelLeft(link+1): offsets (tot_num+2), list (chi)
  double *ssfl;                   // flattened normalised singular values (d*chi)
  int *blkperm;                   // column of X_k holding the p-th largest value of block k (flat)
  int *pos_b, *pos_p;             // Position(beta,1:2), 1-based (chi)
  double *part;                   // kNormParts partial sums of |Theta'|^2
};

// local particle numbers: Conserv(i) with intDegFree, i-1 (0-based i) without
struct NcLocal {
  int n[8];
};

// Tensor-core Theta: block k of a bond as stored in X (m >= n: the block itself,
// else its conjugate transpose), and the class size K of its betas
struct NcSize {
  int m, n, K, trans, boffx;
};
// one product of a grouped launch: X = the block's storage, (m, n) as stored,
// q = minNL + k the block's (and its betas' class) left number
struct NcProd {
  double2 *X;
  int m, n, K, s, k, trans, q, pad;
};
static_assert(sizeof(NcProd) == 40 && offsetof(NcProd, m) == 8 && offsetof(NcProd, n) == 12,
              "NcProd: per-problem sizes at a stride of 10 ints");

struct NcWorkspace {
  int bmax;
  std::vector<NcSlot> slots;
  NcSlot *slots_d;
  JacobiProblem<double> *probs_d;   // nslots * bmax problems
  JacobiProblem<double> *small_d;   // the same list with the bidiagonal blocks emptied
  // blocks on the bidiagonal route: slot table, records, routes and per-block
  // workspaces, in one allocation grown on demand
  char *bd_base = nullptr;
  size_t bd_bytes = 0;
  std::vector<JacobiProblem<double>> probs_h;
  std::vector<Slot> bslots_h;
  std::vector<Compact> bcp_h;
  std::vector<int> bpath_h;
  std::vector<int> blk2bs_h;  // (bond, block) -> bidiagonal block index, -1 for Jacobi
  int *blk2bs_d = nullptr;
  NcSize *sizes_d = nullptr;  // nslots * bmax block sizes (tensor-core Theta)
};


}  // namespace

// ---------------------------------------------------------------------------
// Block bookkeeping, one CTA per bond.  The order-defining loops (IndexLeft,
// IndexRight) run on one thread in the reference's loop order (alpha outer,
// i inner), so block rows/columns are in exactly the reference's order.
// ---------------------------------------------------------------------------
__global__ void k_nc_blocks(const int *__restrict__ lab_l, const int *__restrict__ lab_r,
                            const int *links, Slot *slots, NcSlot *nc, JacobiProblem<double> *probs,
                            int chi, int d, int totNum, int maxFilling, int bmax, NcLocal nl) {
  const int s = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int link = links[s];
  const int *ll0 = lab_l + (size_t)(link - 1) * chi;  // LabelLeft(link)
  const int *ll1 = lab_l + (size_t)link * chi;        // LabelLeft(link+1)
  const int *lr2 = lab_r + (size_t)(link + 1) * chi;  // LabelRight(link+2)
  NcSlot S = nc[s];
  // minmaxNLR (:1201-1250)
  int mnl = ll0[0], mxl = 0, mnr = lr2[0], mxr = 0;
  for (int a = 0; a < chi; ++a) {
    mnl = min(mnl, ll0[a]);
    const int v = ll0[a] == kLabelUnused ? 0 : ll0[a];
    mxl = a == 0 ? v : max(mxl, v);
  }
  for (int g = 0; g < chi; ++g) {
    mnr = min(mnr, lr2[g]);
    const int v = lr2[g] == kLabelUnused ? 0 : lr2[g];
    mxr = g == 0 ? v : max(mxr, v);
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
  const int nb = mxl - mnl + 1;
  S.hdr[H_MINNL] = mnl;
  S.hdr[H_MAXNL] = mxl;
  S.hdr[H_MINNR] = mnr;
  S.hdr[H_MAXNR] = mxr;
  S.hdr[H_ERR] = 0;
  for (int k = 0; k < bmax; ++k) probs[(size_t)s * bmax + k].n = 0;
  if (nb < 1 || nb > bmax) {
    S.hdr[H_NB] = 0;
    S.hdr[H_ERR] = 1;
    return;
  }
  S.hdr[H_NB] = nb;
  for (int k = 0; k < nb; ++k) S.rows[k] = S.cols[k] = 0;
  // SizeOfBlocks (:1252-1336)
  for (int a = 0; a < chi; ++a)
    for (int i = 0; i < d; ++i)
      if (ll0[a] < 1000) {
        const int NL = ll0[a] + nl.n[i];
        if (mnl <= NL && NL <= mxl) S.rows[NL - mnl]++;
      }
  for (int g = 0; g < chi; ++g)
    for (int j = 0; j < d; ++j)
      if (lr2[g] < 1000) {
        const int NR = lr2[g] + nl.n[j];
        if (mnr <= NR && NR <= mxr) {
          const int k = totNum - NR - mnl;
          if (k < 0 || k >= nb) {
            S.hdr[H_ERR] = 1;
            S.hdr[H_NB] = 0;
            return;
          }
          S.cols[k]++;
        }
      }
  S.roff[0] = S.coff[0] = S.boffx[0] = S.boffv[0] = S.soff[0] = 0;
  int maxdim = 0;
  for (int k = 0; k < nb; ++k) {
    const int m = S.rows[k], n = S.cols[k], mn = min(m, n);
    S.roff[k + 1] = S.roff[k] + m;
    S.coff[k + 1] = S.coff[k] + n;
    S.boffx[k + 1] = S.boffx[k] + m * n;
    S.boffv[k + 1] = S.boffv[k] + mn * mn;
    S.soff[k + 1] = S.soff[k] + mn;
    maxdim = max(maxdim, mn);
  }
  S.hdr[H_SZ] = S.soff[nb];
  S.hdr[H_MAXDIM] = maxdim;
  // IndexLeft (:1339-1391) and IndexRight (:1393-1443)
  for (int e = 0; e < chi * d; ++e) S.rowpos[e] = S.colpos[e] = -1;
  for (int k = 0; k < nb; ++k) S.rows[k] = 0;  // reused as fill counters
  for (int a = 0; a < chi; ++a)
    for (int i = 0; i < d; ++i)
      if (ll0[a] < 1000 && mnl <= ll0[a] + nl.n[i] && ll0[a] + nl.n[i] <= mxl) {
        const int k = ll0[a] + nl.n[i] - mnl;
        const int p = S.roff[k] + S.rows[k]++;
        S.l_alpha[p] = a;
        S.l_i[p] = i;
        S.rowpos[a * d + i] = p - S.roff[k];
      }
  for (int k = 0; k < nb; ++k) S.cols[k] = 0;
  for (int g = 0; g < chi; ++g)
    for (int j = 0; j < d; ++j)
      if (lr2[g] < 1000 && mnr <= lr2[g] + nl.n[j] && lr2[g] + nl.n[j] <= mxr) {
        const int k = totNum - (lr2[g] + nl.n[j]) - mnl;
        const int p = S.coff[k] + S.cols[k]++;
        S.r_gamma[p] = g;
        S.r_j[p] = j;
        S.colpos[g * d + j] = p - S.coff[k];
      }
  // betas of link+1 grouped by left label (stable counting sort, labels in [0, totNum])
  for (int q = 0; q <= totNum + 1; ++q) S.cls_off[q] = 0;
  for (int b = 0; b < chi; ++b)
    if (ll1[b] >= 0 && ll1[b] <= totNum) S.cls_off[ll1[b] + 1]++;
  for (int q = 0; q <= totNum; ++q) S.cls_off[q + 1] += S.cls_off[q];
  for (int b = 0; b < chi; ++b)
    if (ll1[b] >= 0 && ll1[b] <= totNum) S.cls_beta[S.cls_off[ll1[b]]++] = b;  // advances starts
  for (int q = totNum + 1; q > 0; --q) S.cls_off[q] = S.cls_off[q - 1];          // restore
  S.cls_off[0] = 0;
  // Jacobi problems: block k is X_k (rows x cols) or its conjugate transpose
  double2 *X = slots[s].X, *V = slots[s].V;
  for (int k = 0; k < nb; ++k) {
    const int m = S.rows[k], n = S.cols[k];
    JacobiProblem<double> P;
    P.X = X + S.boffx[k];
    P.V = V + S.boffv[k];
    if (m >= n) {
      P.m = m;
      P.n = n;
    } else {
      P.m = n;
      P.n = m;
    }
    P.ldx = P.m > 0 ? P.m : 1;
    P.ldv = P.n > 0 ? P.n : 1;
    P.floor = 0.0;
    probs[(size_t)s * bmax + k] = P;
  }
}

// ---------------------------------------------------------------------------
// FormThetaNC + ThetaOperationNC + RenormThetaNC partial sums + FormBlockTheta.
// One thread per (alpha, gamma); kNormParts CTAs per bond with a fixed chunk
// each, so the norm's summation order is fixed.
// ---------------------------------------------------------------------------
constexpr int kMaxDnc = 8;
constexpr int kNcBidiagMinDim = 16;  // smaller block side from which a block is bidiagonalised
constexpr int kMaxPairs = 16;  // allowed (i, j) pairs of one pair total, intDegFree form
static_assert(kMaxDnc <= 8, "NcLocal and the handle's table hold 8 local numbers");

// A = l0 G1 l1 and B = G2 l2 of each bond, once per update, so that each term of
// the Theta kernel's class dot products is one complex multiply-add: FP64
// (double2), or double-float (float4) in the precision form.  They live in the
// slot's V buffer, which the block SVDs only use after the Theta kernel
// (k_nc_prepare_svd resets it).
template <bool kDF>
__global__ void k_nc_scale(const double2 *__restrict__ gam, const double *__restrict__ lam,
                           const int *links, Slot *slots, int chi, int d) {
  const int s = blockIdx.y;
  const int link = links[s];
  const size_t csz = (size_t)chi * d * chi;
  const double2 *G1 = gam + (size_t)(link - 1) * csz;
  const double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l1 = lam + (size_t)link * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  float4 *A = reinterpret_cast<float4 *>(slots[s].V), *B = A + csz;  // double-float form
  double2 *Ad = slots[s].V, *Bd = Ad + csz;                           // FP64 form
  const size_t cd = (size_t)chi * d;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < csz; e += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(e % chi), b = (int)(e / cd);  // A: (a, i, b); B: (b, j, g) with g = e / (chi d)
    const double wa = l0[a] * l1[b];
    const double2 x = G1[e], y = G2[e];
    const double wb = l2[b];
    if (kDF) {
      A[e] = dfs(make_double2(wa * x.x, wa * x.y));
      B[e] = dfs(make_double2(wb * y.x, wb * y.y));
    } else {
      Ad[e] = make_double2(wa * x.x, wa * x.y);
      Bd[e] = make_double2(wb * y.x, wb * y.y);
    }
  }
}

// kDF (precision form): the class dot products read A = l0 G1 l1 and B = G2 l2,
// prepared as double-float in the slot's V buffer by k_nc_scale, and accumulate
// in double-float on the FP32 pipe; the gate mix and the norm stay FP64.
template <bool kIdf, bool kDF>
__global__ void __launch_bounds__(256) k_nc_theta(const double2 *__restrict__ gam,
                                                  const double *__restrict__ lam,
                                                  const int *__restrict__ lab_l,
                                                  const int *__restrict__ lab_r, const int *links,
                                                  Slot *slots, NcSlot *nc, int chi, int d,
                                                  int totNum, int maxFilling, NcLocal nl) {
  const int s = blockIdx.y;
  const NcSlot S = nc[s];
  __shared__ double red[256];
  const int nb = S.hdr[H_NB];
  const int link = links[s];
  const size_t csz = (size_t)chi * d * chi;
  const int *ll0 = lab_l + (size_t)(link - 1) * chi;
  const int *lr1 = lab_r + (size_t)link * chi;
  const int *lr2 = lab_r + (size_t)(link + 1) * chi;
  const double2 *op = slots[s].gate;
  const int d2 = d * d;
  const int mnl = S.hdr[H_MINNL];
  const float4 *Adf = reinterpret_cast<const float4 *>(slots[s].V);  // kDF: l0 G1 l1
  const float4 *Bdf = Adf + csz;                                      // kDF: G2 l2
  const double2 *Apre = slots[s].V, *Bpre = Apre + csz;               // FP64: l0 G1 l1, G2 l2
  // Theta(a, i, jj, g) = sum over the betas of class q with LabelRight(link+1) =
  // rgtN + r of l0 G1(a,i,b) l1 G2(b,jj,g) l2
  auto cdot = [&](int q, int i, int jj, int r, int a, int g, int rgtN) -> double2 {
    if constexpr (kDF) {
      float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
      for (int p = S.cls_off[q]; p < S.cls_off[q + 1]; ++p) {
        const int b = S.cls_beta[p];
        const int rgtN2 = lr1[b];
        if (rgtN2 >= 1000 || rgtN2 - rgtN != r) continue;
        df_cmac(rh, rl, ih, il, Adf[a + (size_t)chi * i + (size_t)chi * d * b],
                Bdf[b + (size_t)chi * jj + (size_t)chi * d * g]);
      }
      return make_double2((double)rh + (double)rl, (double)ih + (double)il);
    } else {
      double2 sacc = make_double2(0.0, 0.0);
      for (int p = S.cls_off[q]; p < S.cls_off[q + 1]; ++p) {
        const int b = S.cls_beta[p];
        const int rgtN2 = lr1[b];
        if (rgtN2 >= 1000 || rgtN2 - rgtN != r) continue;
        const double2 x = Apre[a + (size_t)chi * i + (size_t)chi * d * b];
        const double2 y = Bpre[b + (size_t)chi * jj + (size_t)chi * d * g];
        sacc.x = fma(x.x, y.x, fma(-x.y, y.y, sacc.x));
        sacc.y = fma(x.x, y.y, fma(x.y, y.x, sacc.y));
      }
      return sacc;
    }
  };
  const size_t total = (size_t)chi * chi;
  const size_t chunk = (total + kNormParts - 1) / kNormParts;
  const size_t beg = blockIdx.x * chunk, end = min(beg + chunk, total);
  double acc = 0.0;
  for (size_t t = beg + threadIdx.x; t < end; t += blockDim.x) {
    const int a = (int)(t % chi), g = (int)(t / chi);
    const int lftN = ll0[a], rgtN = lr2[g];
    if (max(lftN, rgtN) >= 1000) continue;
    const int ntot = totNum - lftN - rgtN;
    if constexpr (kIdf) {
      // intDegFree form.  Pairs (i, l) with 0 <= ntot - n_i <= maxFilling and
      // n_l = ntot - n_i, i outer and l inner: the entries ThetaOperationNC reads
      // and writes (:970-1010) and RenormThetaNC sums (:1062-1102).
      double2 th[kMaxPairs];
      int pi[kMaxPairs], pl[kMaxPairs];
      int np = 0;
      for (int i = 0; i < d; ++i) {
        const int r = ntot - nl.n[i];
        if (r < 0 || r > maxFilling) continue;
        for (int l = 0; l < d && np < kMaxPairs; ++l) {
          if (nl.n[l] != r) continue;
          // FormThetaNC (:772-818): betas with LabelLeft(link+1) = lftN + n_i and
          // LabelRight(link+1) = rgtN + n_l, both differences within [0, maxFilling]
          double2 sacc = make_double2(0.0, 0.0);
          const int q = lftN + nl.n[i];
          if (nl.n[i] <= maxFilling && q >= 0 && q <= totNum) sacc = cdot(q, i, l, r, a, g, rgtN);
          th[np] = sacc;
          pi[np] = i;
          pl[np] = l;
          ++np;
        }
      }
      for (int o = 0; o < np; ++o) {
        const int k = pi[o], jj = pl[o];
        double2 v = make_double2(0.0, 0.0);
        for (int p = 0; p < np; ++p) {
          const double2 gv = op[(size_t)(k * d + jj) + (size_t)d2 * (pi[p] * d + pl[p])];
          v.x += gv.x * th[p].x - gv.y * th[p].y;
          v.y += gv.x * th[p].y + gv.y * th[p].x;
        }
        acc += v.x * v.x + v.y * v.y;
        const int rp = S.rowpos[a * d + k], cpn = S.colpos[g * d + jj];
        if (nb == 0 || rp < 0 || cpn < 0) continue;
        const int blk = lftN + nl.n[k] - mnl;
        const int m = S.rows[blk], n = S.cols[blk];
        double2 *Xk = slots[s].X + S.boffx[blk];
        if (m >= n)
          Xk[rp + (size_t)m * cpn] = v;
        else
          Xk[cpn + (size_t)n * rp] = make_double2(v.x, -v.y);
      }
    } else {
      // FormThetaNC restricted to the entries ThetaOperationNC reads: (i, ll = ntot - i)
      double2 th[kMaxDnc];
      for (int i = 0; i < d; ++i) {
        th[i] = make_double2(0.0, 0.0);
        const int li = ntot - i;  // 0-based second physical index
        if (li < 0 || li > maxFilling) continue;
        const int q = lftN + i;  // LabelLeft(link+1) of the contributing betas
        if (q < 0 || q > totNum) continue;
        th[i] = cdot(q, i, li, li, a, g, rgtN);  // j = rgtN2 - rgtN1 + 1
      }
      // ThetaOperationNC: Theta'(a,k,jj,g) = sum_i Op2((k)d+jj, (i)d+ll) Theta(a,i,ll,g)
      for (int k = 0; k < d; ++k) {
        const int jj = ntot - k;
        if (jj < 0 || jj > maxFilling) continue;
        double2 o = make_double2(0.0, 0.0);
        for (int i = 0; i < d; ++i) {
          const int li = ntot - i;
          if (li < 0 || li > maxFilling) continue;
          const double2 gv = op[(size_t)(k * d + jj) + (size_t)d2 * (i * d + li)];
          o.x += gv.x * th[i].x - gv.y * th[i].y;
          o.y += gv.x * th[i].y + gv.y * th[i].x;
        }
        acc += o.x * o.x + o.y * o.y;  // RenormThetaNC sums every allowed entry
        // FormBlockTheta: row (a,k) of block NL = lftN + k, column (g,jj)
        const int NL = lftN + k;
        const int rp = S.rowpos[a * d + k], cpn = S.colpos[g * d + jj];
        if (nb == 0 || rp < 0 || cpn < 0) continue;
        const int blk = NL - mnl;
        const int m = S.rows[blk], n = S.cols[blk];
        double2 *Xk = slots[s].X + S.boffx[blk];
        if (m >= n)
          Xk[rp + (size_t)m * cpn] = o;
        else
          Xk[cpn + (size_t)n * rp] = make_double2(o.x, -o.y);
      }
    }  // plain form
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) S.part[blockIdx.x] = red[0];
}

// ---------------------------------------------------------------------------
// Theta on the tensor cores (theta form 103..107 on an NC handle).
//
// The class sums of FormThetaNC are, block by block, one dense product: for
// block k (left number q = minNL + k, rows (alpha, i) with LabelLeft(link) +
// n_i = q, columns (gamma, j) with LabelRight(link+2) + n_j = totNum - q)
//   P_k(r, c) = sum_beta A(alpha_r, i_r, beta) B(beta, j_c, gamma_c),
// beta over the class q betas with LabelRight(link+1) = totNum - q (the betas
// whose labels FormThetaNC's filter accepts for every entry of the block),
// A = l0 G1 l1, B = G2 l2.  Every allowed entry with a nonzero sum lies in a
// block (the block range is clipped to where rows and columns can meet), and
// every block entry is allowed, so the products written straight into the
// blocks' storage in X (conjugate-transposed blocks as P^H = B^H A^H) hold the
// whole pre-gate Theta.  k_nc_mix then applies ThetaOperationNC in place and
// sums RenormThetaNC's partials.  The products of all (bond, block) pairs run as
// grouped digit-plane products (tc_ozaki.cu), one launch per size bucket.
// ---------------------------------------------------------------------------
__global__ void k_nc_sizes(const NcSlot *nc, int totNum, int bmax, NcSize *out) {
  const int s = blockIdx.x;
  const NcSlot S = nc[s];
  const int nb = S.hdr[H_ERR] ? 0 : S.hdr[H_NB];
  const int mnl = S.hdr[H_MINNL];
  for (int k = threadIdx.x; k < bmax; k += blockDim.x) {
    NcSize z = {0, 0, 0, 0, 0};
    if (k < nb) {
      const int m = S.rows[k], n = S.cols[k], q = mnl + k;
      z.m = max(m, n);
      z.n = min(m, n);
      z.trans = m < n;
      z.K = (q >= 0 && q <= totNum) ? S.cls_off[q + 1] - S.cls_off[q] : 0;
      z.boffx = S.boffx[k];
    }
    out[(size_t)s * bmax + k] = z;
  }
}

// Digit planes of the grouped products' operands, one warp per line.  A line of
// the stored product's left factor (kB = false: its rows) or right factor (kB =
// true: its columns) is a row (alpha, i) of Theta or a column (gamma, j): rows
// when not transposed on the left and transposed on the right.  Its values over
// the class's betas (K, the class list order) are A(alpha, i, beta) and
// B(beta, j, gamma), conjugated for transposed blocks, zero for the betas that
// the label filter drops.
template <bool kB>
__global__ void __launch_bounds__(256) k_nc_oz_pack(const double2 *__restrict__ gam, const double *__restrict__ lam,
                                                    const int *__restrict__ lab_r, const int *links,
                                                    const NcSlot *nc, const NcProd *tab, int chi, int d,
                                                    int totNum, int nprob, int rows_pad, int k_pad, int S,
                                                    unsigned short *dig, int *exps) {
  const int p = blockIdx.y;
  const int lines = kB ? rows_pad / 2 : rows_pad;
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= lines) return;
  const NcProd P = tab[p];
  const NcSlot &Sl = nc[P.s];
  const int link = links[P.s];
  const bool live = r < (kB ? P.n : P.m);
  const bool theta_row = kB == (P.trans != 0);
  int x = 0, y = 0;  // (alpha, i) or (gamma, j)
  if (live) {
    if (theta_row) {
      const int e = Sl.roff[P.k] + r;
      x = Sl.l_alpha[e];
      y = Sl.l_i[e];
    } else {
      const int e = Sl.coff[P.k] + r;
      x = Sl.r_gamma[e];
      y = Sl.r_j[e];
    }
  }
  const size_t csz = (size_t)chi * d * chi;
  const double2 *G1 = gam + (size_t)(link - 1) * csz;
  const double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l1 = lam + (size_t)link * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  const int *lr1 = lab_r + (size_t)link * chi;  // LabelRight(link+1)
  const int *beta = Sl.cls_beta + (P.K > 0 ? Sl.cls_off[P.q] : 0);
  const int want = totNum - P.q;
  const bool cj = P.trans != 0;
  oz_pack_line<kB>(
      [&](int l) {
        const int b = beta[l];
        const int rb = lr1[b];
        double2 v = make_double2(0.0, 0.0);
        if (rb < 1000 && rb == want) {
          if (theta_row) {
            const double w = l0[x] * l1[b];
            const double2 g = G1[x + (size_t)chi * y + (size_t)chi * d * b];
            v = make_double2(w * g.x, w * g.y);
          } else {
            const double w = l2[x];
            const double2 g = G2[b + (size_t)chi * y + (size_t)chi * d * x];
            v = make_double2(w * g.x, w * g.y);
          }
          if (cj) v.y = -v.y;
        }
        return v;
      },
      live, P.K, p, r, nprob, rows_pad, k_pad, S, dig, exps);
}

// ThetaOperationNC + RenormThetaNC partials on the pre-gate Theta held in the
// blocks (the tensor-core form): one thread per (alpha, gamma) reads its <= d
// allowed entries (or its intDegFree pairs), mixes them with the gate and writes
// them back to the same places; the entries of different (alpha, gamma) are
// disjoint.  Same chunking and loop order as k_nc_theta.
template <bool kIdf>
__global__ void __launch_bounds__(256) k_nc_mix(const int *__restrict__ lab_l, const int *__restrict__ lab_r,
                                                const int *links, Slot *slots, NcSlot *nc, int chi, int d,
                                                int totNum, int maxFilling, NcLocal nl) {
  const int s = blockIdx.y;
  const NcSlot S = nc[s];
  __shared__ double red[256];
  const int nb = S.hdr[H_NB];
  const int link = links[s];
  const int *ll0 = lab_l + (size_t)(link - 1) * chi;
  const int *lr2 = lab_r + (size_t)(link + 1) * chi;
  const double2 *op = slots[s].gate;
  double2 *X = slots[s].X;
  const int d2 = d * d;
  const int mnl = S.hdr[H_MINNL];
  // storage of the allowed entry (alpha, i; j, gamma) in its block, or null
  auto at = [&](int a, int i, int j, int g, bool *cj) -> double2 * {
    const int rp = S.rowpos[a * d + i], cp = S.colpos[g * d + j];
    if (nb == 0 || rp < 0 || cp < 0) return nullptr;
    const int blk = ll0[a] + nl.n[i] - mnl;
    const int m = S.rows[blk], n = S.cols[blk];
    *cj = m < n;
    return X + S.boffx[blk] + (m >= n ? rp + (size_t)m * cp : cp + (size_t)n * rp);
  };
  auto get = [&](int a, int i, int j, int g) -> double2 {
    bool cj = false;
    const double2 *e = at(a, i, j, g, &cj);
    if (!e) return make_double2(0.0, 0.0);
    const double2 v = *e;
    return cj ? make_double2(v.x, -v.y) : v;
  };
  auto put = [&](int a, int i, int j, int g, double2 v) {
    bool cj = false;
    double2 *e = at(a, i, j, g, &cj);
    if (e) *e = cj ? make_double2(v.x, -v.y) : v;
  };
  const size_t total = (size_t)chi * chi;
  const size_t chunk = (total + kNormParts - 1) / kNormParts;
  const size_t beg = blockIdx.x * chunk, end = min(beg + chunk, total);
  double acc = 0.0;
  for (size_t t = beg + threadIdx.x; t < end; t += blockDim.x) {
    const int a = (int)(t % chi), g = (int)(t / chi);
    const int lftN = ll0[a], rgtN = lr2[g];
    if (max(lftN, rgtN) >= 1000) continue;
    const int ntot = totNum - lftN - rgtN;
    if constexpr (kIdf) {
      double2 th[kMaxPairs];
      int pi[kMaxPairs], pl[kMaxPairs];
      int np = 0;
      for (int i = 0; i < d; ++i) {
        const int r = ntot - nl.n[i];
        if (r < 0 || r > maxFilling) continue;
        for (int l = 0; l < d && np < kMaxPairs; ++l) {
          if (nl.n[l] != r) continue;
          const int q = lftN + nl.n[i];
          th[np] = (nl.n[i] <= maxFilling && q >= 0 && q <= totNum) ? get(a, i, l, g) : make_double2(0.0, 0.0);
          pi[np] = i;
          pl[np] = l;
          ++np;
        }
      }
      for (int o = 0; o < np; ++o) {
        const int k = pi[o], jj = pl[o];
        double2 v = make_double2(0.0, 0.0);
        for (int p = 0; p < np; ++p) {
          const double2 gv = op[(size_t)(k * d + jj) + (size_t)d2 * (pi[p] * d + pl[p])];
          v.x += gv.x * th[p].x - gv.y * th[p].y;
          v.y += gv.x * th[p].y + gv.y * th[p].x;
        }
        acc += v.x * v.x + v.y * v.y;
        put(a, k, jj, g, v);
      }
    } else {
      double2 th[kMaxDnc];
      for (int i = 0; i < d; ++i) {
        th[i] = make_double2(0.0, 0.0);
        const int li = ntot - i;
        if (li < 0 || li > maxFilling) continue;
        const int q = lftN + i;
        if (q < 0 || q > totNum) continue;
        th[i] = get(a, i, li, g);
      }
      for (int k = 0; k < d; ++k) {
        const int jj = ntot - k;
        if (jj < 0 || jj > maxFilling) continue;
        double2 o = make_double2(0.0, 0.0);
        for (int i = 0; i < d; ++i) {
          const int li = ntot - i;
          if (li < 0 || li > maxFilling) continue;
          const double2 gv = op[(size_t)(k * d + jj) + (size_t)d2 * (i * d + li)];
          o.x += gv.x * th[i].x - gv.y * th[i].y;
          o.y += gv.x * th[i].y + gv.y * th[i].x;
        }
        acc += o.x * o.x + o.y * o.y;
        put(a, k, jj, g, o);
      }
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) S.part[blockIdx.x] = red[0];
}

// V = identity for every block problem; norm from the fixed-order partials
// unnormalized = 1 for SwappingNC, which skips RenormThetaNC: the block singular
// values are taken as they are (norm 1 in the flattening).
__global__ void k_nc_prepare_svd(NcSlot *nc, JacobiProblem<double> *probs, double *nrm, int bmax,
                                 int *status, int unnormalized) {
  const int s = blockIdx.y;
  const NcSlot S = nc[s];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double acc = 0.0;
    for (int j = 0; j < kNormParts; ++j) acc += S.part[j];
    const double v = sqrt(acc);
    nrm[s] = unnormalized ? 1.0 : v;
    if (!isfinite(v) || v == 0.0) atomicOr(&status[0], 1);
    if (S.hdr[H_ERR]) atomicOr(&status[1], 1);
  }
  const int nb = S.hdr[H_NB];
  if (blockIdx.x == 0) {  // negligible-column floor, relative to this bond's ||Theta||
    double acc = 0.0;
    for (int j = 0; j < kNormParts; ++j) acc += S.part[j];
    const double f = kNegligibleColumn * sqrt(acc);
    for (int k = threadIdx.x; k < nb; k += blockDim.x) probs[(size_t)s * bmax + k].floor = f * f;
  }
  for (int k = blockIdx.x; k < nb; k += gridDim.x) {
    const JacobiProblem<double> P = probs[(size_t)s * bmax + k];
    for (int e = threadIdx.x; e < P.n * P.n; e += blockDim.x)
      P.V[e] = make_double2((e % P.n) == (e / P.n) ? 1.0 : 0.0, 0.0);
  }
}

// ---------------------------------------------------------------------------
// FlattenSS + Ordering + JudgePosition + UpdateLabelLeft/Right + FormLambdaNC.
// One CTA per bond.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_nc_select(int *lab_l, int *lab_r, double *lam,
                                                    const int *links, NcSlot *nc,
                                                    const JacobiProblem<double> *probs,
                                                    const double *nrm, double *truncerr,
                                                    double *sig_link, int *sig_count, int chi, int d,
                                                    int totNum, int bmax, int *status, double rank_bound) {
  extern __shared__ double sh[];  // colnorm[sz] | flat rank scratch
  if (status[0] & 1) return;  // non-finite ||Theta|| in the batch: the chain is left as it was
  const int s = blockIdx.x;
  const NcSlot S = nc[s];
  const int link = links[s];
  const int nb = S.hdr[H_NB], sz = S.hdr[H_SZ];
  double *cn = sh;  // column norms in flat (block-major, column) order, sz entries
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  // column norms: one warp per column
  for (int k = 0; k < nb; ++k) {
    const JacobiProblem<double> P = probs[(size_t)s * bmax + k];
    for (int c = warp; c < P.n; c += nw) {
      double acc = 0.0;
      for (int r = lane; r < P.m; r += 32) {
        const double2 v = P.X[r + (size_t)P.ldx * c];
        acc = fma(v.x, v.x, fma(v.y, v.y, acc));
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) cn[S.soff[k] + c] = sqrt(acc);
    }
  }
  __syncthreads();
  const double inv = 1.0 / nrm[s];
  // within each block: descending order (LAPACK's S order) -> ssfl, blkperm
  for (int k = 0; k < nb; ++k) {
    const int o = S.soff[k], n = S.soff[k + 1] - o;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      const double v = cn[o + c];
      if (!isfinite(v)) atomicOr(&status[0], 1);
      int rank = 0;
      for (int q = 0; q < n; ++q) {
        const double w = cn[o + q];
        rank += (w > v) || (w == v && q < c);
      }
      S.ssfl[o + rank] = v * inv;
      S.blkperm[o + rank] = c;
    }
  }
  __syncthreads();
  // Ordering (:1515-1538): descending; equal values in descending flat index.
  // order(beta) = flat index (1-based) of the beta-th largest; only beta < chi is used.
  int *ord = reinterpret_cast<int *>(sh);  // reuse: cn no longer needed
  for (int t = threadIdx.x; t < sz; t += blockDim.x) {
    const double v = S.ssfl[t];
    int rank = 0;
    for (int q = 0; q < sz; ++q) {
      const double w = S.ssfl[q];
      rank += (w > v) || (w == v && q > t);
    }
    if (rank < chi) ord[rank] = t + 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int mnl = S.hdr[H_MINNL];
    int *ll1 = lab_l + (size_t)link * chi;
    int *lr1 = lab_r + (size_t)link * chi;
    double *l1 = lam + (size_t)link * chi;
    // kept-rank form (no reference counterpart): the fewest leading values whose
    // discarded weight stays within rank_bound, as in the dense FormLambda1
    int keep = chi;
    if (rank_bound > 0.0) {
      const int top = min(chi, sz);
      double all = 0.0;
      for (int beta = 0; beta < top; ++beta) {
        const double v = S.ssfl[ord[beta] - 1];
        if (v > kGuardNC) all = all + v * v;
      }
      double w = fmax(1.0 - all, 0.0);
      keep = top;
      while (keep > 1) {
        const double v = S.ssfl[ord[keep - 1] - 1];
        const double q = v > kGuardNC ? v * v : 0.0;
        if (w + q > rank_bound) break;
        w += q;
        --keep;
      }
    }
    double renorm = 0.0;
    for (int beta = 0; beta < chi; ++beta) {
      int pb = 0, pp = 0;
      double v = 0.0;
      if (beta < sz) {
        // JudgePosition (:1540-1565)
        int ot = ord[beta];
        for (int k = 0; k < nb; ++k) {
          if (ot <= 0) break;
          const int mn = S.soff[k + 1] - S.soff[k];
          ot -= mn;
          pb = k + 1;
          pp = ot + mn;
        }
        v = S.ssfl[ord[beta] - 1];
      }
      S.pos_b[beta] = pb;
      S.pos_p[beta] = pp;
      // UpdateLabelLeft (:1583-1604) / UpdateLabelRight (:1615-1624)
      const bool kept = beta < sz && beta < keep && v > kGuardNC;
      const int lab = kept ? mnl + pb - 1 : kLabelUnused;
      ll1[beta] = lab;
      lr1[beta] = lab < 1000 ? totNum - lab : kLabelUnused;
      // FormLambdaNC (:1642-1656)
      const double tl = kept ? v : 0.0;
      l1[beta] = tl;
      renorm = renorm + tl * tl;
    }
    truncerr[s] = fabs(1.0 - renorm);
    const double rs = sqrt(renorm);
    for (int beta = 0; beta < chi; ++beta) l1[beta] = l1[beta] / rs;
    sig_count[link - 1] = sz;
  }
  for (int t = threadIdx.x; t < sz; t += blockDim.x) sig_link[(size_t)(link - 1) * d * chi + t] = S.ssfl[t];
}

// ---------------------------------------------------------------------------
// FormGamma1NC / FormGamma2NC: zero both Gammas, then scatter the kept columns.
// ---------------------------------------------------------------------------
__global__ void k_nc_zero_gammas(double2 *gam, const int *links, int chi, int d, const int *status) {
  if (status[0] & 1) return;  // non-finite batch: the chain is left as it was
  const int s = blockIdx.y;
  const size_t csz = (size_t)chi * d * chi;
  double2 *g = gam + (size_t)(links[s] - 1) * csz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < 2 * csz;
       e += (size_t)gridDim.x * blockDim.x)
    g[e] = make_double2(0.0, 0.0);
}

__global__ void k_nc_gamma(double2 *gam, const double *lam, const int *links, NcSlot *nc,
                           const JacobiProblem<double> *probs, const double *nrm, int chi, int d,
                           int bmax, const int *status) {
  if (status[0] & 1) return;  // non-finite batch: the chain is left as it was
  const int s = blockIdx.y;
  const int beta = blockIdx.x;
  const NcSlot S = nc[s];
  const int sz = S.hdr[H_SZ];
  if (beta >= chi || beta >= sz) return;
  const int link = links[s];
  const size_t csz = (size_t)chi * d * chi;
  double2 *G1 = gam + (size_t)(link - 1) * csz;
  double2 *G2 = gam + (size_t)link * csz;
  const double *l0 = lam + (size_t)(link - 1) * chi;
  const double *l2 = lam + (size_t)(link + 1) * chi;
  const int bn = S.pos_b[beta] - 1, psn = S.pos_p[beta] - 1;
  if (bn < 0 || psn < 0) return;
  const JacobiProblem<double> P = probs[(size_t)s * bmax + bn];
  const int m = S.rows[bn], n = S.cols[bn];
  const int col = S.blkperm[S.soff[bn] + psn];
  const double sigma = S.ssfl[S.soff[bn] + psn] * nrm[s];
  const bool trans = m < n;
  // U(:,psn) of the block (m rows) and V(:,psn) (n rows):
  //   m >= n: U = X(:,col)/sigma, V = V_J(:,col)
  //   m <  n: U = V_J(:,col),     V = X(:,col)/sigma   (X holds the block's conjugate transpose)
  for (int fa = threadIdx.x; fa < m; fa += blockDim.x) {
    const int a = S.l_alpha[S.roff[bn] + fa], i = S.l_i[S.roff[bn] + fa];
    double2 u;
    if (!trans) {
      const double2 x = P.X[fa + (size_t)P.ldx * col];
      u = sigma > 0.0 ? make_double2(x.x / sigma, x.y / sigma) : make_double2(0.0, 0.0);
    } else {
      // X = M^H = U' S V'^H, so M = V' S U'^H: the block's left vectors are V's columns
      u = P.V[fa + (size_t)P.ldv * col];
    }
    double2 out = make_double2(0.0, 0.0);
    if (l0[a] > kGuardNC) out = make_double2(u.x / l0[a], u.y / l0[a]);
    G1[a + (size_t)chi * i + (size_t)chi * d * beta] = out;
  }
  for (int fg = threadIdx.x; fg < n; fg += blockDim.x) {
    const int g = S.r_gamma[S.coff[bn] + fg], j = S.r_j[S.coff[bn] + fg];
    double2 vt;  // VT(psn, fg) = conj(V(fg, psn))
    if (!trans) {
      const double2 v = P.V[fg + (size_t)P.ldv * col];
      vt = make_double2(v.x, -v.y);
    } else {
      // the block's right vectors are U' = X(:,col)/sigma; VT = conj(U')
      const double2 x = P.X[fg + (size_t)P.ldx * col];
      vt = sigma > 0.0 ? make_double2(x.x / sigma, -x.y / sigma) : make_double2(0.0, 0.0);
    }
    double2 out = make_double2(0.0, 0.0);
    if (l2[g] > kGuardNC) out = make_double2(vt.x / l2[g], vt.y / l2[g]);
    G2[beta + (size_t)chi * j + (size_t)chi * d * g] = out;
  }
}

// The Jacobi list without the blocks that take the bidiagonal route (n = 0 there).
__global__ void k_nc_mask(const JacobiProblem<double> *probs, JacobiProblem<double> *small, int count,
                          int min_dim, int max_dim) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  JacobiProblem<double> P = probs[i];
  if (P.n >= min_dim && P.m <= max_dim) {
    P.m = 0;
    P.n = 0;
  }
  small[i] = P;
}

// Between the two phases of the bidiagonal route: every value of the bond --
// Jacobi blocks' column norms, bidiagonal blocks' bisection values -- is ranked,
// and each bidiagonal block computes vectors only for its values that can enter
// the global top chi (>= the chi-th largest, less a 1e-12 relative margin so that
// near-ties are decided by the final values).  One CTA per bond.
__global__ void __launch_bounds__(1024) k_nc_cut(NcSlot *nc, const JacobiProblem<double> *probs,
                                                 const int *blk2bs, Slot *bslots, int bmax, int chi) {
  extern __shared__ double val[];  // sz values of the bond
  const int s = blockIdx.x;
  const NcSlot S = nc[s];
  const int nb = S.hdr[H_NB], sz = S.hdr[H_SZ];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int k = 0; k < nb; ++k) {
    const JacobiProblem<double> P = probs[(size_t)s * bmax + k];
    const int bs = blk2bs[(size_t)s * bmax + k];
    const int o = S.soff[k];
    if (bs >= 0) {
      const double *sig = bslots[bs].bdws + 2 * P.n;
      for (int c = threadIdx.x; c < P.n; c += blockDim.x) val[o + c] = sig[c];
    } else {
      for (int c = warp; c < P.n; c += nw) {
        double acc = 0.0;
        for (int r = lane; r < P.m; r += 32) {
          const double2 v = P.X[r + (size_t)P.ldx * c];
          acc = fma(v.x, v.x, fma(v.y, v.y, acc));
        }
        for (int q = 16; q > 0; q >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, q);
        if (lane == 0) val[o + c] = sqrt(acc);
      }
    }
  }
  __syncthreads();
  // the chi-th largest value: the smallest one with fewer than chi values above it
  __shared__ double tau_s;
  if (threadIdx.x == 0) tau_s = 0.0;
  __syncthreads();
  if (sz > chi) {
    double best = INFINITY;
    for (int t = threadIdx.x; t < sz; t += blockDim.x) {
      const double v = val[t];
      int above = 0;
      for (int q = 0; q < sz; ++q) above += val[q] > v;
      if (above < chi) best = fmin(best, v);
    }
    for (int q = 16; q > 0; q >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, q));
    __shared__ double wmin[32];
    if (lane == 0) wmin[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = INFINITY;
      for (int w = 0; w < nw; ++w) b = fmin(b, wmin[w]);
      tau_s = b;
    }
    __syncthreads();
  }
  const double tau = tau_s * (1.0 - 1e-12);
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    const int bs = blk2bs[(size_t)s * bmax + k];
    if (bs < 0) continue;
    const int n = probs[(size_t)s * bmax + k].n, o = S.soff[k];
    int keep = 0;
    while (keep < n && val[o + keep] >= tau) ++keep;  // bisection values are descending
    bslots[bs].cp->k = keep > 0 ? keep : 1;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int nc_alloc(tebd_handle *h) {
  h->nc_ws = nullptr;
  h->nc_ws_bytes = 0;
  const int ns = h->nslots, chi = h->chi, d = h->d, nd = chi * d;
  const int bmax = h->opts.tot_num + 2;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t per = al(sizeof(int) * H_COUNT) + al(sizeof(int) * bmax) * 2 +
                     al(sizeof(int) * (bmax + 1)) * 5 + al(sizeof(int) * nd) * 6 +
                     al(sizeof(int) * (h->opts.tot_num + 3)) + al(sizeof(int) * chi) +
                     al(sizeof(double) * nd) + al(sizeof(int) * nd) + al(sizeof(int) * chi) * 2 +
                     al(sizeof(double) * kNormParts);
  NcWorkspace *w = new (std::nothrow) NcWorkspace();
  if (!w) return TEBD_ERR_OOM;
  w->bmax = bmax;
  char *base = nullptr;
  const size_t bytes = per * ns + al(sizeof(NcSlot) * ns) + 2 * al(sizeof(JacobiProblem<double>) * ns * bmax) +
                       sizeof(NcSize) * ns * bmax;
  int rc = check_cuda(h, cudaMalloc((void **)&base, bytes), "alloc NC workspace");
  if (rc) {
    delete w;
    return rc;
  }
  h->nc_ws_bytes = bytes;
  char *p = base;
  w->slots.resize(ns);
  for (int s = 0; s < ns; ++s) {
    NcSlot &S = w->slots[s];
    auto take = [&](size_t b) {
      char *q = p;
      p += al(b);
      return q;
    };
    S.hdr = (int *)take(sizeof(int) * H_COUNT);
    S.rows = (int *)take(sizeof(int) * bmax);
    S.cols = (int *)take(sizeof(int) * bmax);
    S.roff = (int *)take(sizeof(int) * (bmax + 1));
    S.coff = (int *)take(sizeof(int) * (bmax + 1));
    S.boffx = (int *)take(sizeof(int) * (bmax + 1));
    S.boffv = (int *)take(sizeof(int) * (bmax + 1));
    S.soff = (int *)take(sizeof(int) * (bmax + 1));
    S.l_alpha = (int *)take(sizeof(int) * nd);
    S.l_i = (int *)take(sizeof(int) * nd);
    S.r_gamma = (int *)take(sizeof(int) * nd);
    S.r_j = (int *)take(sizeof(int) * nd);
    S.rowpos = (int *)take(sizeof(int) * nd);
    S.colpos = (int *)take(sizeof(int) * nd);
    S.cls_off = (int *)take(sizeof(int) * (h->opts.tot_num + 3));
    S.cls_beta = (int *)take(sizeof(int) * chi);
    S.ssfl = (double *)take(sizeof(double) * nd);
    S.blkperm = (int *)take(sizeof(int) * nd);
    S.pos_b = (int *)take(sizeof(int) * chi);
    S.pos_p = (int *)take(sizeof(int) * chi);
    S.part = (double *)take(sizeof(double) * kNormParts);
  }
  w->slots_d = (NcSlot *)p;
  p += al(sizeof(NcSlot) * ns);
  w->probs_d = (JacobiProblem<double> *)p;
  p += al(sizeof(JacobiProblem<double>) * ns * bmax);
  w->small_d = (JacobiProblem<double> *)p;
  p += al(sizeof(JacobiProblem<double>) * ns * bmax);
  w->sizes_d = (NcSize *)p;
  h->nc_ws = base;
  rc = check_cuda(h, cudaMemcpy(w->slots_d, w->slots.data(), sizeof(NcSlot) * ns,
                                cudaMemcpyHostToDevice), "upload NC slot table");
  if (rc) {
    cudaFree(base);
    h->nc_ws = nullptr;
    delete w;
    return rc;
  }
  h->nc_meta = w;
  return TEBD_OK;
}

void nc_free(tebd_handle *h) {
  if (h->nc_ws) cudaFree(h->nc_ws);
  h->nc_ws = nullptr;
  NcWorkspace *w = reinterpret_cast<NcWorkspace *>(h->nc_meta);
  if (w && w->bd_base) cudaFree(w->bd_base);
  delete w;
  h->nc_meta = nullptr;
}

namespace {

// Blocks whose both sides are >= kNcBidiagMinDim (the Jacobi problem is always
// tall, m >= n) take the dense path's bidiagonal route, all n triplets each: the
// block slot table points at the block's X (ld m) and V (ld n), so the output has
// the Jacobi route's layout (X(:,c) = sigma_c u_c, V(:,c) = v_c) that the
// selection and the Gamma scatter read.  Returns the number of such blocks; the
// rest stay on the grouped Jacobi with `small_maxdim` its largest n.
int nc_route_blocks(tebd_handle *h, NcWorkspace *w, int nb, int *nbd, int *small_maxdim, BidiagBatch *out) {
  const int bmax = w->bmax, count = nb * bmax;
  cudaStream_t st = h->stream;
  w->probs_h.resize(count);
  int rc = check_cuda(h, cudaMemcpyAsync(w->probs_h.data(), w->probs_d, sizeof(JacobiProblem<double>) * count,
                                         cudaMemcpyDeviceToHost, st), "read NC block problems");
  if (rc) return rc;
  if ((rc = check_cuda(h, cudaStreamSynchronize(st), "NC block problems"))) return rc;
  w->bslots_h.clear();
  w->bcp_h.clear();
  w->blk2bs_h.assign(count, -1);
  // largest problems first (16 M N^2 flops), so that the long bidiagonalisations
  // start in the first wave and the small ones fill in behind them
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const JacobiProblem<double> &A = w->probs_h[a], &B = w->probs_h[b];
    return (double)A.m * A.n * A.n > (double)B.m * B.n * B.n;
  });
  int mmax = 0, nmaxb = 0, smax = 0;
  for (int i : order) {
    const JacobiProblem<double> &P = w->probs_h[i];
    if (P.n >= kNcBidiagMinDim && P.m <= kBidiagMaxDim) {
      w->blk2bs_h[i] = (int)w->bslots_h.size();
      Slot b = {};
      b.X = P.X;
      b.V = P.V;
      w->bslots_h.push_back(b);
      Compact c = {};
      c.m = P.m;
      c.n = P.n;
      c.k = P.n;
      w->bcp_h.push_back(c);
      mmax = std::max(mmax, P.m);
      nmaxb = std::max(nmaxb, P.n);
      h->stats.gebrd_flops += 16.0 * P.m * (double)P.n * P.n - 16.0 / 3.0 * (double)P.n * P.n * P.n;
    } else {
      smax = std::max(smax, P.n);
    }
  }
  const int nl = (int)w->bslots_h.size();
  *nbd = nl;
  *small_maxdim = smax;
  if (nl == 0) return TEBD_OK;
  // workspace: tables, then per block aux | tau | taup | bdws
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t need = al(sizeof(Slot) * nl) + al(sizeof(Compact) * nl) + al(sizeof(int) * nl) + al(sizeof(int) * count);
  std::vector<size_t> aux_e(nl), bd_d(nl);
  for (int i = 0; i < nl; ++i) {
    bidiag_block_ws(w->bcp_h[i].m, w->bcp_h[i].n, nmaxb, &aux_e[i], &bd_d[i]);
    need += al(sizeof(double2) * aux_e[i]) + 2 * al(sizeof(double2) * w->bcp_h[i].n) + al(sizeof(double) * bd_d[i]);
  }
  if (need > w->bd_bytes) {
    if (w->bd_base) {
      if ((rc = check_cuda(h, cudaStreamSynchronize(st), "NC bidiagonal workspace"))) return rc;
      cudaFree(w->bd_base);
      w->bd_base = nullptr;
      w->bd_bytes = 0;
    }
    const size_t grow = 2 * need;  // doubling: a few reallocations over a run whose blocks grow
    if ((rc = check_cuda(h, cudaMalloc((void **)&w->bd_base, grow), "alloc NC bidiagonal workspace"))) return rc;
    w->bd_bytes = grow;
  }
  char *p = w->bd_base;
  Slot *tab_d = (Slot *)p;
  p += al(sizeof(Slot) * nl);
  Compact *cp_d = (Compact *)p;
  p += al(sizeof(Compact) * nl);
  int *path_d = (int *)p;
  p += al(sizeof(int) * nl);
  w->blk2bs_d = (int *)p;
  p += al(sizeof(int) * count);
  for (int i = 0; i < nl; ++i) {
    Slot &b = w->bslots_h[i];
    b.cp = cp_d + i;
    b.aux = (double2 *)p;
    p += al(sizeof(double2) * aux_e[i]);
    b.tau = (double2 *)p;
    p += al(sizeof(double2) * w->bcp_h[i].n);
    b.taup = (double2 *)p;
    p += al(sizeof(double2) * w->bcp_h[i].n);
    b.bdws = (double *)p;
    p += al(sizeof(double) * bd_d[i]);
  }
  w->bpath_h.assign(nl, kPathBidiag);
  if ((rc = check_cuda(h, cudaMemcpyAsync(tab_d, w->bslots_h.data(), sizeof(Slot) * nl, cudaMemcpyHostToDevice, st),
                       "upload NC block slots")))
    return rc;
  if ((rc = check_cuda(h, cudaMemcpyAsync(cp_d, w->bcp_h.data(), sizeof(Compact) * nl, cudaMemcpyHostToDevice, st),
                       "upload NC block records")))
    return rc;
  if ((rc = check_cuda(h, cudaMemcpyAsync(path_d, w->bpath_h.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, st),
                       "upload NC block routes")))
    return rc;
  if ((rc = check_cuda(h, cudaMemcpyAsync(w->blk2bs_d, w->blk2bs_h.data(), sizeof(int) * count,
                                          cudaMemcpyHostToDevice, st),
                       "upload NC block map")))
    return rc;
  k_nc_mask<<<(count + 255) / 256, 256, 0, st>>>(w->probs_d, w->small_d, count, kNcBidiagMinDim, kBidiagMaxDim);
  TEBD_LAUNCHED(h);
  out->slots_d = tab_d;
  out->path_d = path_d;
  out->path_h = w->bpath_h.data();
  out->nb = nl;
  out->nmax = mmax;
  out->kk = nmaxb;
  out->dfp = h->opts.svd_mode == TEBD_SVD_DF;
  out->phase = 0;
  out->cap = 0;
  return TEBD_OK;
}

// The batch's Theta on the tensor cores (k_nc_sizes .. k_nc_mix above).  The
// bonds' headers are read into hdr first, since the products are sized from
// them; a bond whose labels fall outside its block range fails the batch here
// (TEBD_ERR_NC_BLOCKS), before anything is written.  Products are grouped in
// size buckets (stored rows up to 128 x 2^a, columns up to 64 x 2^b, class sizes
// up to 16 x 2^c), one grouped launch per bucket, padded to the bucket's largest
// problem; a launch skips the tiles outside each problem's own rows and columns.
int nc_theta_tc(tebd_handle *h, NcWorkspace *w, int nb, int N, int mf, const NcLocal &nl, std::vector<int> &hdr) {
  cudaStream_t st = h->stream;
  const int bmax = w->bmax, chi = h->chi, d = h->d, S = h->theta_form - 100;
  k_nc_sizes<<<nb, 128, 0, st>>>(w->slots_d, N, bmax, w->sizes_d);
  TEBD_LAUNCHED(h);
  std::vector<NcSize> sz((size_t)nb * bmax);
  hdr.assign((size_t)nb * H_COUNT, 0);
  int rc = check_cuda(h, cudaMemcpyAsync(sz.data(), w->sizes_d, sizeof(NcSize) * sz.size(), cudaMemcpyDeviceToHost,
                                         st),
                      "read NC block sizes");
  for (int s = 0; s < nb && !rc; ++s)
    rc = check_cuda(h, cudaMemcpyAsync(hdr.data() + (size_t)s * H_COUNT, w->slots[s].hdr, sizeof(int) * H_COUNT,
                                       cudaMemcpyDeviceToHost, st),
                    "read NC header");
  if (!rc) rc = check_cuda(h, cudaStreamSynchronize(st), "NC block sizes");
  if (rc) return rc;
  for (int s = 0; s < nb; ++s)
    if (hdr[(size_t)s * H_COUNT + H_ERR])
      return set_error(h, TEBD_ERR_NC_BLOCKS, "charge label outside the block range");
  auto level = [](int x, int unit) {
    int l = 0;
    while ((unit << l) < x) ++l;
    return l;
  };
  std::map<std::array<int, 3>, std::vector<NcProd>> buckets;
  for (int s = 0; s < nb; ++s)
    for (int k = 0; k < bmax; ++k) {
      const NcSize &z = sz[(size_t)s * bmax + k];
      if (z.m <= 0 || z.n <= 0) continue;
      NcProd P;
      P.X = h->slots[s].X + z.boffx;
      P.m = z.m;
      P.n = z.n;
      P.K = z.K;
      P.s = s;
      P.k = k;
      P.trans = z.trans;
      P.q = hdr[(size_t)s * H_COUNT + H_MINNL] + k;
      P.pad = 0;
      buckets[{level(z.m, kTcBM), level(z.n, kOzBN / 2), level(std::max(z.K, 1), 16)}].push_back(P);
    }
  struct Launch {
    int off, np, m, n, m_pad, n_pad, k_pad;
    double flops;
  };
  constexpr int kMaxProblems = 65535;  // the product's grid z and the packers' grid y
  const double pairs = S * (S + 1) / 2.0;
  std::vector<Launch> launches;
  std::vector<NcProd> tab;
  size_t da = 0, db = 0, ea = 0, eb = 0;
  for (const auto &kv : buckets) {
    const std::vector<NcProd> &v = kv.second;
    for (size_t c0 = 0; c0 < v.size(); c0 += kMaxProblems) {
      Launch L = {(int)tab.size(), (int)std::min(v.size() - c0, (size_t)kMaxProblems), 0, 0, 0, 0, 0, 0.0};
      int K = 1;
      for (int i = 0; i < L.np; ++i) {
        L.m = std::max(L.m, v[c0 + i].m);
        L.n = std::max(L.n, v[c0 + i].n);
        K = std::max(K, v[c0 + i].K);
      }
      L.m_pad = tc_pad(L.m, kTcBM);
      L.n_pad = tc_pad(2 * L.n, kOzBN);
      L.k_pad = tc_pad(2 * K, kOzBK);
      for (int i = 0; i < L.np; ++i)  // the tiles the launch runs
        L.flops += pairs * 2.0 * tc_pad(v[c0 + i].m, kTcBM) * (double)tc_pad(2 * v[c0 + i].n, kOzBN) * L.k_pad;
      da = std::max(da, (size_t)S * L.np * L.m_pad * L.k_pad);
      db = std::max(db, (size_t)S * L.np * L.n_pad * L.k_pad);
      ea = std::max(ea, (size_t)L.np * L.m_pad);
      eb = std::max(eb, (size_t)L.np * (L.n_pad / 2));
      tab.insert(tab.end(), v.begin() + c0, v.begin() + c0 + L.np);
      launches.push_back(L);
    }
  }
  if (!launches.empty()) {
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t tb = al(sizeof(NcProd) * tab.size()), ab = al(sizeof(unsigned short) * da),
                 bb = al(sizeof(unsigned short) * db), eab = al(sizeof(int) * ea);
    if ((rc = tc_reserve(h, tb + ab + bb + eab + al(sizeof(int) * eb)))) return rc;
    char *p = static_cast<char *>(h->tc_ws);
    NcProd *tab_d = reinterpret_cast<NcProd *>(p);
    auto *dA = reinterpret_cast<unsigned short *>(p + tb);
    auto *dB = reinterpret_cast<unsigned short *>(p + tb + ab);
    int *eA = reinterpret_cast<int *>(p + tb + ab + bb);
    int *eB = reinterpret_cast<int *>(p + tb + ab + bb + eab);
    if ((rc = check_cuda(h, cudaMemcpyAsync(tab_d, tab.data(), sizeof(NcProd) * tab.size(), cudaMemcpyHostToDevice, st),
                         "upload NC products")))
      return rc;
    for (const Launch &L : launches) {
      const NcProd *t = tab_d + L.off;
      k_nc_oz_pack<false><<<dim3(L.m_pad / 8, L.np), 256, 0, st>>>(h->gam, h->lam, h->lab_r, h->links_d, w->slots_d,
                                                                   t, chi, d, N, L.np, L.m_pad, L.k_pad, S, dA, eA);
      TEBD_LAUNCHED(h);
      k_nc_oz_pack<true><<<dim3(L.n_pad / 16, L.np), 256, 0, st>>>(h->gam, h->lam, h->lab_r, h->links_d, w->slots_d,
                                                                   t, chi, d, N, L.np, L.n_pad, L.k_pad, S, dB, eB);
      TEBD_LAUNCHED(h);
      const unsigned char *tp = reinterpret_cast<const unsigned char *>(t);
      OzBatch b = {};
      b.a_dig = dA;
      b.b_dig = dB;
      b.a_exp = eA;
      b.b_exp = eB;
      b.nprob = L.np;
      b.m_pad = L.m_pad;
      b.n_pad = L.n_pad;
      b.k_pad = L.k_pad;
      b.slices = S;
      b.rs = 1;
      b.cs = 0;  // column stride = the problem's own stored rows
      b.m_d = reinterpret_cast<const int *>(tp + offsetof(NcProd, m));
      b.n_d = reinterpret_cast<const int *>(tp + offsetof(NcProd, n));
      b.dim_stride = (int)(sizeof(NcProd) / sizeof(int));
      b.m = L.m;
      b.n = L.n;
      b.alpha = 1.0;
      b.optr = tp + offsetof(NcProd, X);
      b.optr_stride = (int)sizeof(NcProd);
      cudaEvent_t e0, e1;
      tc_events(h, L.flops, &e0, &e1);
      if (e0) cudaEventRecord(e0, st);
      if ((rc = check_cuda(h, oz_gemm_launch(b, h->tc_err, st), "NC tensor-core Theta"))) return rc;
      if (e1) cudaEventRecord(e1, st);
      TEBD_LAUNCHED(h);
    }
  }
  auto mix = h->nc_idf ? k_nc_mix<true> : k_nc_mix<false>;
  mix<<<dim3(kNormParts, nb), 256, 0, st>>>(h->lab_l, h->lab_r, h->links_d, h->slots_d, w->slots_d, chi, d, N, mf,
                                            nl);
  TEBD_LAUNCHED(h);
  return TEBD_OK;
}

}  // namespace

int run_nc_batch(tebd_handle *h, int nb, const int * /*links_host*/, double * /*truncerr*/) {
  NcWorkspace *w = reinterpret_cast<NcWorkspace *>(h->nc_meta);
  if (!w) return set_error(h, TEBD_ERR_STATE, "NC workspace missing");
  const int chi = h->chi, d = h->d, bmax = w->bmax;
  const int N = h->opts.tot_num, mf = h->opts.max_filling;
  if (d > kMaxDnc) return set_error(h, TEBD_ERR_ARG, "NC mode supports d <= 8");
  // Without intDegFree the physical index is the particle number: local states
  // 0..d-1 and at most maxFilling particles must be the same range (the reference
  // indexes past Gamma for maxFilling > d-1, and for maxFilling < d-1 its
  // SwapThetaNC keeps entries that ThetaOperationNC would drop).
  if (!h->nc_idf && mf != d - 1)
    return set_error(h, TEBD_ERR_ARG, "NC mode without internal degrees of freedom needs max_filling = d-1");
  NcLocal nl;
  for (int i = 0; i < 8; ++i) nl.n[i] = (h->nc_idf && i < d) ? h->nc_conserv[i] : i;
  cudaStream_t st = h->stream;
  k_nc_blocks<<<nb, 32, 0, st>>>(h->lab_l, h->lab_r, h->links_d, h->slots_d, w->slots_d, w->probs_d,
                                 chi, d, N, mf, bmax, nl);
  TEBD_LAUNCHED(h);
  if (d < 2) return set_error(h, TEBD_ERR_ARG, "NC mode needs d >= 2");
  const bool df = h->opts.svd_mode == TEBD_SVD_DF;
  std::vector<int> hdr;  // the bonds' headers: sizes for the launch configuration
  int rc = TEBD_OK;
  if (zprod_oz(h->theta_form)) {
    if ((rc = nc_theta_tc(h, w, nb, N, mf, nl, hdr))) return rc;
  } else {
    // A = l0 G1 l1 and B = G2 l2 of each bond, once per update, in the slot's V
    // buffer (they fill 2/d of it; d >= 2 in NC mode): FP64, or double-float in
    // the precision form
    if (df)
      k_nc_scale<true><<<dim3(64, nb), 256, 0, st>>>(h->gam, h->lam, h->links_d, h->slots_d, chi, d);
    else
      k_nc_scale<false><<<dim3(64, nb), 256, 0, st>>>(h->gam, h->lam, h->links_d, h->slots_d, chi, d);
    TEBD_LAUNCHED(h);
    auto kern = h->nc_idf ? (df ? k_nc_theta<true, true> : k_nc_theta<true, false>)
                          : (df ? k_nc_theta<false, true> : k_nc_theta<false, false>);
    kern<<<dim3(kNormParts, nb), 256, 0, st>>>(h->gam, h->lam, h->lab_l, h->lab_r, h->links_d, h->slots_d,
                                               w->slots_d, chi, d, N, mf, nl);
    TEBD_LAUNCHED(h);
  }
  k_nc_prepare_svd<<<dim3(32, nb), 256, 0, st>>>(w->slots_d, w->probs_d, h->nrm, bmax, h->status_d,
                                                 h->unnormalized);
  TEBD_LAUNCHED(h);
  if (hdr.empty()) {
    hdr.resize((size_t)nb * H_COUNT);
    for (int s = 0; s < nb; ++s)
      if ((rc = check_cuda(h, cudaMemcpyAsync(hdr.data() + (size_t)s * H_COUNT, w->slots[s].hdr,
                                              sizeof(int) * H_COUNT, cudaMemcpyDeviceToHost, st),
                           "read NC header")))
        return rc;
    if ((rc = check_cuda(h, cudaStreamSynchronize(st), "NC blocks"))) return rc;
  }
  int maxdim = 0, maxsz = 0;
  for (int s = 0; s < nb; ++s) {
    if (hdr[(size_t)s * H_COUNT + H_ERR])
      return set_error(h, TEBD_ERR_NC_BLOCKS, "charge label outside the block range");
    maxdim = std::max(maxdim, hdr[(size_t)s * H_COUNT + H_MAXDIM]);
    maxsz = std::max(maxsz, hdr[(size_t)s * H_COUNT + H_SZ]);
  }
  if (maxdim >= kNcBidiagMinDim) {
    // large blocks: bidiagonal route, the rest: grouped Jacobi.  The Jacobi blocks
    // and the bidiagonal singular values come first, then the cut decides how
    // many vectors each bidiagonal block needs.
    int nbd = 0, small_max = 0;
    BidiagBatch bb;
    if ((rc = nc_route_blocks(h, w, nb, &nbd, &small_max, &bb))) return rc;
    if (nbd == 0) {
      if ((rc = run_jacobi_problems(h, w->probs_d, nb * bmax, maxdim))) return rc;
    } else {
      if (small_max > 0 && (rc = run_jacobi_problems(h, w->small_d, nb * bmax, small_max))) return rc;
      bb.phase = 1;
      if ((rc = run_bidiag_batch(h, bb))) return rc;
      k_nc_cut<<<nb, 1024, sizeof(double) * (size_t)std::max(maxsz, 1), st>>>(w->slots_d, w->probs_d, w->blk2bs_d,
                                                                           bb.slots_d, bmax, chi);
      TEBD_LAUNCHED(h);
      bb.phase = 2;
      bb.cap = 1;
      if ((rc = run_bidiag_batch(h, bb))) return rc;
    }
  } else if ((rc = run_jacobi_problems(h, w->probs_d, nb * bmax, maxdim))) {
    return rc;
  }
  const size_t shb = std::max(sizeof(double) * (size_t)maxsz, sizeof(int) * (size_t)chi) + 16;
  k_nc_select<<<nb, 1024, shb, st>>>(h->lab_l, h->lab_r, h->lam, h->links_d, w->slots_d, w->probs_d,
                                     h->nrm, h->truncerr_d, h->sig_link_d, h->sig_count_d, chi, d, N,
                                     bmax, h->status_d, h->unnormalized ? 0.0 : h->rank_bound);
  TEBD_LAUNCHED(h);
  k_nc_zero_gammas<<<dim3(64, nb), 256, 0, st>>>(h->gam, h->links_d, chi, d, h->status_d);
  TEBD_LAUNCHED(h);
  k_nc_gamma<<<dim3(chi, nb), 128, 0, st>>>(h->gam, h->lam, h->links_d, w->slots_d, w->probs_d,
                                            h->nrm, chi, d, bmax, h->status_d);
  TEBD_LAUNCHED(h);
  return check_cuda(h, cudaGetLastError(), "NC launch");
}

}  // namespace tebd

// Internal degrees of freedom (intDegFree + Conserv%vi) for the handle's NC routines.
extern "C" int tebd_set_conserv(tebd_handle *h, const int *conserv) {
  using namespace tebd;
  if (!h) return TEBD_ERR_ARG;
  if (h->mode != TEBD_MODE_NC) return set_error(h, TEBD_ERR_STATE, "tebd_set_conserv needs a TEBD_MODE_NC handle");
  if (!conserv) {
    h->nc_idf = 0;
    return TEBD_OK;
  }
  const int d = h->d;
  if (d > kMaxDnc) return set_error(h, TEBD_ERR_ARG, "intDegFree: d <= 8");
  // Local numbers above maxFilling are dropped by FormThetaNC but can be filled by
  // ThetaOperationNC, a state the reference never builds; they are refused.
  int mx = 0;
  for (int i = 0; i < d; ++i) {
    if (conserv[i] < 0 || conserv[i] > h->opts.max_filling)
      return set_error(h, TEBD_ERR_ARG, "intDegFree: Conserv values must lie in [0, max_filling]");
    mx = std::max(mx, conserv[i]);
  }
  // pairs (i, j) per pair total, as the Theta kernel lists them
  for (int t = 0; t <= 2 * mx; ++t) {
    int np = 0;
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j) np += (conserv[i] + conserv[j] == t);
    if (np > kMaxPairs) return set_error(h, TEBD_ERR_ARG, "intDegFree: more than 16 local pairs share one pair total");
  }
  for (int i = 0; i < 8; ++i) h->nc_conserv[i] = i < d ? conserv[i] : 0;
  h->nc_idf = 1;
  return TEBD_OK;
}
