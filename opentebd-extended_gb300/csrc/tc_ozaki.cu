// tc_ozaki.cu -- FP64-class complex products on the sm_103a tensor cores by
// error-free splitting into bf16 integer digits (scheme and accuracy in
// tc_gemm.cuh).
//
// One CTA of 10 warps computes a 128 x 128 tile of the real product of one
// problem.  The S digit groups g = s + t do not fit the 512 TMEM columns at
// once for N = 128 (7 x 128), so K is streamed in passes: pass q accumulates the
// groups 4q .. 4q + 3 (four accumulators of 128 columns), reading the digit
// slices 0 .. min(S, 4q + 4) - 1 of A and B:
//   warp 8, lane 0   TMA producer: per 32-wide K block and pass the pass's digit
//                    tiles of A and of B (128 rows x 64 B each, 64-byte
//                    swizzle) into one of `stages` shared-memory stages;
//   warp 9, lane 0   MMA issuer: per K block two K-steps of 16, and per step
//                    one tcgen05.mma (M 128, N 128, K 16, kind::f16, bf16 in,
//                    FP32 accumulation) for every digit pair (s, t) of the
//                    pass's groups, into the TMEM accumulator of its group;
//   warps 0-7        epilogue (warp w reads TMEM lanes 32 (w mod 4) .. + 31,
//                    columns 64 (w div 4) .. + 63 of each group): after every
//                    chunk of 16 K blocks (512 real terms: the group sums are
//                    exact integers below 2^24) they read the pass's group
//                    accumulators and add them, exactly, into 64 int64
//                    registers, then release TMEM to the issuer; after the last
//                    chunk of the last pass the row and column exponents are
//                    applied and the complex FP64 result is written.
// N = 128 keeps the tensor pipe at its full op rate (an N = 64 MMA runs it at
// half) and halves the operand reads per multiply-add.  The issuer waits for
// the epilogue between chunks, so the two roles live in different warps (a
// warp's lanes reconverge before tcgen05.ld).  Every wait is bounded as in
// tc_gemm.cu; on expiry *err is set and nothing is written.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "oz_digits.cuh"
#include "tc_gemm.cuh"
#include "tc_ptx.cuh"

namespace tebd {
namespace {
using namespace tcx;

constexpr int kOzEpiWarps = 8;
constexpr int kOzThreads = 32 * (kOzEpiWarps + 2);
constexpr int kOzMaxStages = 4;
constexpr int kOzChunk = 16;   // K blocks per exact chunk (512 real terms)
constexpr int kOzGroups = 4;   // digit groups per pass (4 x 128 TMEM columns)
constexpr uint32_t kOzTileA = kTcBM * kOzBK * 2;  // 8 KB per digit tile of A
constexpr uint32_t kOzTileB = kOzBN * kOzBK * 2;  // 8 KB per digit tile of B
constexpr uint32_t kOzTmemCols = 512;
constexpr int kOzSmemMax = 232448;  // opt-in shared memory per block

// Instruction descriptor of kind::f16: D F32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdescBF16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kOzBN >> 3) << 17) |
                                ((uint32_t)(kTcBM >> 4) << 24);

__host__ __device__ constexpr int oz_passes(int S) { return (S + kOzGroups - 1) / kOzGroups; }
// digit slices pass q reads: 0 .. oz_pass_slices - 1
__host__ __device__ constexpr int oz_pass_slices(int S, int q) {
  return S < kOzGroups * (q + 1) ? S : kOzGroups * (q + 1);
}
__host__ __device__ constexpr int oz_stage_slices(int S) { return oz_pass_slices(S, oz_passes(S) - 1); }
__host__ __device__ constexpr int oz_stages(int S) {
  return (kOzSmemMax - 2048) / (oz_stage_slices(S) * (int)(kOzTileA + kOzTileB)) > kOzMaxStages
             ? kOzMaxStages
             : (kOzSmemMax - 2048) / (oz_stage_slices(S) * (int)(kOzTileA + kOzTileB));
}
size_t oz_smem(int S) { return 1024 + (size_t)oz_stages(S) * oz_stage_slices(S) * (kOzTileA + kOzTileB) + 512; }

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdescBF16), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

// 32 lanes x 16 columns of TMEM into r[0..15] without waiting; the caller waits
// once for several loads (tmem_wait) before it reads any of them.
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// Wait for this thread's TMEM loads; the empty asm statements that "modify" the
// registers afterwards keep every use of them behind the wait.
template <int N>
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[N]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < N; ++i) asm volatile("" : "+r"(r[i]));
}

// All MMAs of one K block (two K-steps of 16) for the digit pairs (sa, sb) of the
// groups GLO <= sa + sb < min(GHI, S): da, db are the descriptors of slice 0 of
// A and B in the stage; slice q starts q tiles further, a K-step 32 bytes further
// (descriptor units of 16 bytes); group g accumulates at TMEM column
// (g - GLO) x 128.  The first MMA into a group in a chunk (K-step 0 of its first
// K block, pair (0, g)) overwrites the accumulator.
template <int S, int GLO, int GHI>
__device__ __forceinline__ void oz_issue(uint32_t tmem, uint64_t da, uint64_t db, bool first) {
#pragma unroll
  for (int kk = 0; kk < kOzBK / 16; ++kk)
#pragma unroll
    for (int sa = 0; sa < S; ++sa)
#pragma unroll
      for (int sb = 0; sb < S; ++sb)
        if (sa + sb >= GLO && sa + sb < GHI && sa + sb < S)
          mma_bf16(tmem + (uint32_t)((sa + sb - GLO) * kOzBN), da + (uint64_t)((sa * kOzTileA + kk * 32) >> 4),
                   db + (uint64_t)((sb * kOzTileB + kk * 32) >> 4), (first && kk == 0 && sa == 0) ? 0u : 1u);
}

template <int S>
__global__ void __launch_bounds__(kOzThreads, 1)
    k_tc_oz(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, OzBatch b,
            int *err) {
  constexpr int stages = oz_stages(S), NSL = oz_stage_slices(S), NP = oz_passes(S);
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = smem;                                    // [stage][slice] kOzTileA
  unsigned char *sB = sA + (size_t)stages * NSL * kOzTileA;    // [stage][slice] kOzTileB
  uint64_t *full = reinterpret_cast<uint64_t *>(sB + (size_t)stages * NSL * kOzTileB);
  uint64_t *empty = full + kOzMaxStages;
  uint64_t *cfull = empty + kOzMaxStages;  // a chunk's MMAs are complete
  uint64_t *tfree = cfull + 1;             // the epilogue has read the chunk (8 arrivals)
  uint64_t *done = tfree + 1;              // every MMA issued has completed
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.z;
  const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * kOzBN;
  // a problem's own extent, never beyond the batch's (the operands end there)
  const int mp = b.m_d ? min(b.m_d[(size_t)p * b.dim_stride], b.m) : b.m;
  const int np = b.n_d ? min(b.n_d[(size_t)p * b.dim_stride], b.n) : b.n;
  if (m0 >= mp || n0 >= 2 * np) return;  // tile outside this problem: uniform over the CTA
  const int nk = b.k_pad / kOzBK;
  const int nchunks = (nk + kOzChunk - 1) / kOzChunk;
  const int total = NP * nk;  // K blocks over all passes

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(cfull, 1);
    mbar_init(tfree, kOzEpiWarps);
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(kOzTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == kOzEpiWarps) {
    // ---- TMA producer ----
    if (lane != 0) goto finish;
    int issued = 0;
    for (int it = 0; it < total; ++it) {
      const int s = it % stages, q = it / nk, kb = it % nk;
      if (it >= stages && !mbar_wait(&empty[s], ((it / stages) & 1) ^ 1, abort)) {
        *abort = 1;
        atomicExch(err, 1);
        break;
      }
      const int nsl = oz_pass_slices(S, q);
      mbar_expect_tx(&full[s], (uint32_t)nsl * (kOzTileA + kOzTileB));
      for (int sl = 0; sl < nsl; ++sl)
        tma_load_3d(sA + (size_t)(s * NSL + sl) * kOzTileA, &tmA, &full[s], kb * kOzBK, m0, sl * b.nprob + p);
      for (int sl = 0; sl < nsl; ++sl)
        tma_load_3d(sB + (size_t)(s * NSL + sl) * kOzTileB, &tmB, &full[s], kb * kOzBK, n0, sl * b.nprob + p);
      issued = it + 1;
    }
    if (*abort)
      for (int it = issued - stages < 0 ? 0 : issued - stages; it < issued; ++it)
        mbar_wait(&full[it % stages], (it / stages) & 1, nullptr);
    goto finish;
  }
  if (warp == kOzEpiWarps + 1) {
    // ---- MMA issuer ----
    if (lane != 0) goto finish;
    const uint64_t da0 = sw64_desc(su32(sA)), db0 = sw64_desc(su32(sB));
    for (int it = 0; it < total; ++it) {
      const int q = it / nk, kb = it % nk, s = it % stages;
      const int kc = kb % kOzChunk, gc = q * nchunks + kb / kOzChunk;
      if (kc == 0 && gc > 0 && !mbar_wait(tfree, (gc - 1) & 1, abort)) {
        *abort = 1;
        atomicExch(err, 1);
        break;
      }
      if (!mbar_wait(&full[s], (it / stages) & 1, abort)) {
        *abort = 1;
        atomicExch(err, 1);
        break;
      }
      tc_after();
      const uint64_t da = da0 + (uint64_t)((s * NSL * kOzTileA) >> 4), db = db0 + (uint64_t)((s * NSL * kOzTileB) >> 4);
      if (q == 0)
        oz_issue<S, 0, kOzGroups>(tmem, da, db, kc == 0);
      else
        oz_issue<S, kOzGroups, 2 * kOzGroups>(tmem, da, db, kc == 0);
      mma_commit(&empty[s]);
      if (kc == kOzChunk - 1 || kb == nk - 1) mma_commit(cfull);
    }
    mma_commit(done);
    goto finish;
  }

  {
  // ---- epilogue (warps 0-7): exact chunk sums into 64-bit integers ----
  // acc = sum_g G_g 2^(7 (S-1-g) - R) over the chunks, in units of
  // 2^(R - 7 (S+1)): R keeps the sum inside 63 bits (|G_0| < 2^23 per chunk);
  // groups shifted right by it are rounded, 2^-60 below the total at most.
  int lg = 0;
  while ((1 << lg) < nchunks) ++lg;
  const int R = max(0, 25 + lg + 7 * (S - 1) - 63);
  const int quad = warp & 3, half = warp >> 2;
  long long acc[64];
#pragma unroll
  for (int i = 0; i < 64; ++i) acc[i] = 0;
  bool ok = true;
  const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * 64);
  for (int gc = 0; gc < NP * nchunks; ++gc) {
    if (!mbar_wait(cfull, gc & 1, abort)) {
      ok = false;
      break;
    }
    tc_after();
    const int q = gc / nchunks;
    const int ghi = min(S, kOzGroups * (q + 1));
#pragma unroll 1
    for (int g = kOzGroups * q; g < ghi; ++g) {
      const int sh = 7 * (S - 1 - g) - R;
      const uint32_t col = (uint32_t)((g - kOzGroups * q) * kOzBN);
#pragma unroll
      for (int h = 0; h < 64; h += 16) {  // 16 columns at a time: 10 warps leave 168 registers a thread
        uint32_t r[16];
        tmem_ld16_async(lane_base + col + (uint32_t)h, r);
        tmem_wait(r);
        if (sh >= 0) {
#pragma unroll
          for (int i = 0; i < 16; ++i) acc[h + i] += (long long)__float2int_rn(__uint_as_float(r[i])) << sh;
        } else {
          const long long rnd = 1LL << (-sh - 1);
#pragma unroll
          for (int i = 0; i < 16; ++i)
            acc[h + i] += ((long long)__float2int_rn(__uint_as_float(r[i])) + rnd) >> (-sh);
        }
      }
    }
    tc_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(tfree);
  }
  const bool all_done = mbar_wait(done, 0, nullptr);
  tc_after();
  if (!all_done) atomicExch(err, 1);
  if (ok && all_done && !*abort) {
    const int row = m0 + quad * 32 + lane;
    if (row < mp) {
      double2 *out = b.optr ? *reinterpret_cast<double2 *const *>(b.optr + (size_t)p * b.optr_stride)
                            : b.out + (size_t)p * b.out_stride;
      const int ea = b.a_exp[(size_t)p * b.m_pad + row];
      const long long cs = b.cs ? b.cs : mp;  // cs == 0: column stride = this problem's row count
      const int eu = R - 7 * (S + 1);          // exponent of the accumulator's unit
#pragma unroll
      for (int t = 0; t < 32; ++t) {
        const int j = n0 / 2 + half * 32 + t;
        if (j < np) {
          const int eb = b.b_exp[(size_t)p * (b.n_pad / 2) + j];
          double2 r = make_double2(0.0, 0.0);
          if (ea > kExpZero && eb > kExpZero)
            r = make_double2(b.alpha * ldexp((double)acc[2 * t], ea + eb + eu),
                             b.alpha * ldexp((double)acc[2 * t + 1], ea + eb + eu));
          double2 *o = out + (long long)row * b.rs + (long long)j * cs;
          if (b.accumulate) {
            const double2 q = *o;
            r.x += q.x;
            r.y += q.y;
          }
          *o = r;
        }
      }
    }
  }
  }
finish:
  tc_before();
  __syncthreads();
  if (warp == 0) {
    tc_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOzTmemCols)
                 : "memory");
  }
}

// Load a 32 x 32 complex tile of the source as tile[row r][column c] with the
// same conventions as the TF32 packers: A (trans: element (i, k) at src[k + ld i],
// else src[i + ld k]); B (element (k, j) at src[j + ld k] if trans, else
// src[k + ld j]) is loaded as tile[j][k].
__device__ __forceinline__ void oz_tile_a(double2 (*tile)[33], const double2 *S, int ld, int rows, int cols,
                                          int trans, int conj, int i0, int k0) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int yy = ty; yy < 32; yy += 8) {
    const int i = trans ? i0 + yy : i0 + tx, k = trans ? k0 + tx : k0 + yy;
    double2 v = make_double2(0.0, 0.0);
    if (i < rows && k < cols) v = trans ? S[k + (size_t)ld * i] : S[i + (size_t)ld * k];
    if (conj) v.y = -v.y;
    if (trans)
      tile[yy][tx] = v;
    else
      tile[tx][yy] = v;
  }
}
__device__ __forceinline__ void oz_tile_b(double2 (*tile)[33], const double2 *S, int ld, int krows, int ncols,
                                          int trans, int conj, int j0, int k0) {
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int yy = ty; yy < 32; yy += 8) {
    const int j = trans ? j0 + tx : j0 + yy, k = trans ? k0 + yy : k0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (k < krows && j < ncols) v = trans ? S[j + (size_t)ld * k] : S[k + (size_t)ld * j];
    if (conj) v.y = -v.y;
    if (trans)
      tile[tx][yy] = v;
    else
      tile[yy][tx] = v;
  }
}

// Pass 1: the exponent of every row (A) or complex column (B): atomicMax of the
// tile's row maxima.  Pass 2 (digits = 1): the S digit planes.
template <bool kB>
__global__ void __launch_bounds__(256) k_oz_pack(const double2 *src, long long pstride, int ld, int r_ext,
                                                 int c_ext, int trans, int conj, int nprob, int rows_pad,
                                                 int k_pad, int S, unsigned short *dig, int *exps,
                                                 int digits) {
  __shared__ double2 tile[32][33];
  const int p = blockIdx.z;
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const double2 *Sp = src + (size_t)p * pstride;
  if (kB)
    oz_tile_b(tile, Sp, ld, r_ext, c_ext, trans, conj, r0, k0);
  else
    oz_tile_a(tile, Sp, ld, r_ext, c_ext, trans, conj, r0, k0);
  __syncthreads();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int nrow = kB ? rows_pad / 2 : rows_pad;  // complex rows (A) / complex columns (B)
  if (!digits) {
    for (int yy = ty; yy < 32; yy += 8) {
      const double2 v = tile[yy][tx];
      unsigned long long mx = max(oz_absbits(v.x), oz_absbits(v.y));
      for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      const int r = r0 + yy;
      if (tx == 0 && r < nrow && mx) atomicMax(&exps[(size_t)p * nrow + r], oz_exp_bits(mx));
    }
    return;
  }
  const size_t plane = (size_t)nprob * rows_pad * k_pad;
  for (int yy = ty; yy < 32; yy += 8) {
    const int r = r0 + yy, k = k0 + tx;
    if (r >= nrow || 2 * k >= k_pad) continue;
    const double2 v = tile[yy][tx];
    const int e = exps[(size_t)p * nrow + r];
    unsigned short dr[kOzMaxS], di[kOzMaxS];
    oz_digits(v.x, e, S, dr);
    oz_digits(v.y, e, S, di);
    if (!kB) {
      unsigned short *o = dig + ((size_t)p * rows_pad + r) * k_pad + 2 * k;
      for (int s = 0; s < S; ++s)
        *reinterpret_cast<uint32_t *>(o + s * plane) = (uint32_t)dr[s] | ((uint32_t)di[s] << 16);
    } else {
      // rows 2r: (re, -im); 2r+1: (im, re)
      unsigned short *o0 = dig + ((size_t)p * rows_pad + 2 * r) * k_pad + 2 * k;
      unsigned short *o1 = o0 + k_pad;
      for (int s = 0; s < S; ++s) {
        const unsigned short ni = di[s] ^ 0x8000u;  // -im (bf16 sign bit; -0 for 0 is harmless)
        *reinterpret_cast<uint32_t *>(o0 + s * plane) = (uint32_t)dr[s] | ((uint32_t)ni << 16);
        *reinterpret_cast<uint32_t *>(o1 + s * plane) = (uint32_t)di[s] | ((uint32_t)dr[s] << 16);
      }
    }
  }
}

// Digits of an operand whose K index is contiguous in memory (A read transposed,
// element (i, k) at src[k + ld i]; B read as stored, element (k, j) at
// src[k + ld j]): one warp per row of the packed operand (oz_pack_line),
// coalesced reads and writes, no atomics.  Rows beyond the source extent and K
// beyond it are packed as zeros.
template <bool kB>
__global__ void __launch_bounds__(256) k_oz_pack_rows(const double2 *src, long long pstride, int ld, int r_ext,
                                                      int c_ext, int conj, int nprob, int rows_pad, int k_pad,
                                                      int S, unsigned short *dig, int *exps) {
  const int p = blockIdx.y;
  const int nrow = kB ? rows_pad / 2 : rows_pad;
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= nrow) return;
  const double2 *row = src + (size_t)p * pstride + (size_t)ld * r;
  oz_pack_line<kB>(
      [&](int k) {
        double2 x = row[k];
        if (conj) x.y = -x.y;
        return x;
      },
      r < r_ext, c_ext, p, r, nprob, rows_pad, k_pad, S, dig, exps);
}

PFN_cuTensorMapEncodeTiled_v12000 oz_encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    (void)cudaGetLastError();
  });
  return fn;
}

// 3-D map over [depth][rows][k] bf16 with a 32 x box_rows box, 64-byte swizzle.
bool oz_map(CUtensorMap *map, const unsigned short *base, int k_pad, int rows, int depth, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = oz_encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)k_pad, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)k_pad * 2, (cuuint64_t)k_pad * 2 * rows};
  cuuint32_t box[3] = {(cuuint32_t)kOzBK, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<unsigned short *>(base), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t oz_gemm_launch(const OzBatch &b, int *err_d, cudaStream_t st) {
  if (b.m_pad % kTcBM || b.n_pad % kOzBN || b.k_pad % kOzBK || b.k_pad <= 0 || b.nprob <= 0 ||
      b.slices < 1 || b.slices > kOzMaxS)
    return cudaErrorInvalidValue;
  CUtensorMap ma, mb;
  if (!oz_map(&ma, b.a_dig, b.k_pad, b.m_pad, b.slices * b.nprob, kTcBM) ||
      !oz_map(&mb, b.b_dig, b.k_pad, b.n_pad, b.slices * b.nprob, kOzBN))
    return cudaErrorInvalidValue;
  const size_t smem = oz_smem(b.slices);
  dim3 grid(b.m_pad / kTcBM, b.n_pad / kOzBN, b.nprob);
  auto go = [&](auto kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, kOzThreads, smem, st>>>(ma, mb, b, err_d);
    return cudaPeekAtLastError();
  };
  switch (b.slices) {
    case 1: return go(k_tc_oz<1>);
    case 2: return go(k_tc_oz<2>);
    case 3: return go(k_tc_oz<3>);
    case 4: return go(k_tc_oz<4>);
    case 5: return go(k_tc_oz<5>);
    case 6: return go(k_tc_oz<6>);
    default: return go(k_tc_oz<7>);
  }
}

cudaError_t oz_pack_a(const double2 *src, long long pstride, int ld, int rows, int cols, int trans, int conj,
                      int nprob, int m_pad, int k_pad, int slices, unsigned short *dig, int *exps,
                      cudaStream_t st) {
  if (trans) {  // rows contiguous: one warp per row, one kernel
    k_oz_pack_rows<false><<<dim3((m_pad + 7) / 8, nprob), 256, 0, st>>>(src, pstride, ld, rows, cols, conj, nprob,
                                                                         m_pad, k_pad, slices, dig, exps);
    return cudaPeekAtLastError();
  }
  cudaError_t e = cudaMemsetAsync(exps, 0x80, sizeof(int) * (size_t)nprob * m_pad, st);
  if (e != cudaSuccess) return e;
  dim3 grid((m_pad + 31) / 32, (k_pad / 2 + 31) / 32, nprob);
  k_oz_pack<false><<<grid, 256, 0, st>>>(src, pstride, ld, rows, cols, trans, conj, nprob, m_pad, k_pad, slices,
                                         dig, exps, 0);
  k_oz_pack<false><<<grid, 256, 0, st>>>(src, pstride, ld, rows, cols, trans, conj, nprob, m_pad, k_pad, slices,
                                         dig, exps, 1);
  return cudaPeekAtLastError();
}

cudaError_t oz_pack_b(const double2 *src, long long pstride, int ld, int krows, int ncols, int trans, int conj,
                      int nprob, int n_pad, int k_pad, int slices, unsigned short *dig, int *exps,
                      cudaStream_t st) {
  if (!trans) {  // columns contiguous: one warp per complex column, one kernel
    k_oz_pack_rows<true><<<dim3((n_pad / 2 + 7) / 8, nprob), 256, 0, st>>>(src, pstride, ld, ncols, krows, conj,
                                                                            nprob, n_pad, k_pad, slices, dig, exps);
    return cudaPeekAtLastError();
  }
  cudaError_t e = cudaMemsetAsync(exps, 0x80, sizeof(int) * (size_t)nprob * (n_pad / 2), st);
  if (e != cudaSuccess) return e;
  dim3 grid((n_pad / 2 + 31) / 32, (k_pad / 2 + 31) / 32, nprob);
  k_oz_pack<true><<<grid, 256, 0, st>>>(src, pstride, ld, krows, ncols, trans, conj, nprob, n_pad, k_pad, slices,
                                        dig, exps, 0);
  k_oz_pack<true><<<grid, 256, 0, st>>>(src, pstride, ld, krows, ncols, trans, conj, nprob, n_pad, k_pad, slices,
                                        dig, exps, 1);
  return cudaPeekAtLastError();
}

}  // namespace tebd
