// tc_gemm.cu -- split-precision complex products on the sm_103a tensor cores:
// TMA-staged operands, tcgen05.mma with the accumulator in tensor memory (TMEM).
//
// One CTA of 4 warps computes a 128 x 128 tile of the real product C_r = A_r B_r^T
// of one problem of the batch (layouts in tc_gemm.cuh):
//   warp 0, lane 0   TMA producer: for each 32-wide K block, all planes of the A
//                    and B tiles (128 rows x 128 B each, 128-byte swizzle) into
//                    one of kStages shared-memory stages, completion counted on
//                    the stage's `full` mbarrier;
//   warp 1, lane 0   MMA issuer: per K block 4 K-steps of 8, and per step one
//                    tcgen05.mma (M 128, N 128, K 8, kind::tf32) per plane pair
//                    into the FP32 accumulator; tcgen05.commit frees the stage
//                    (`empty` mbarrier) once its MMAs have read it;
//   all 4 warps      epilogue: after the last commit (`done`), tcgen05.ld of
//                    their 32 TMEM lanes (rows), scaled, written as complex FP64
//                    (consecutive lanes write consecutive rows).
// Every mbarrier wait is bounded (~2 s of SM clock): on expiry the kernel sets
// *err, stops issuing, waits (bounded) for the copies and MMAs it issued, frees
// its TMEM and returns without writing the output.
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include <string>

#include "tc_gemm.cuh"
#include "tc_ptx.cuh"

namespace tebd {
namespace {
using namespace tcx;

constexpr int kStages = 3;
constexpr int kThreads = 128;
constexpr uint32_t kTileA = kTcBM * kTcBK * 4;  // bytes of one A plane tile (16 KB)
constexpr uint32_t kTileB = kTcBN * kTcBK * 4;  // bytes of one B plane tile (16 KB)

// Instruction descriptor of kind::tf32: D F32 (bits 4-5 = 1), A and B TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
constexpr uint32_t kIdescTF32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcBN >> 3) << 17) |
                                ((uint32_t)(kTcBM >> 4) << 24);

size_t smem_bytes(int planes) {
  return 1024 + (size_t)kStages * planes * (kTileA + kTileB) + 256;
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdescTF32), "r"(acc)
      : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcBatch b,
              int *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int planes = b.form == kTc3xTF32 ? 2 : 1;
  unsigned char *sA = smem;                                   // [stage][plane] kTileA
  unsigned char *sB = sA + (size_t)kStages * planes * kTileA;  // [stage][plane] kTileB
  uint64_t *full = reinterpret_cast<uint64_t *>(sB + (size_t)kStages * planes * kTileB);
  uint64_t *empty = full + kStages;
  uint64_t *done = empty + kStages;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.z;
  const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * kTcBN;
  // a problem's own extent, never beyond the batch's (the operands end there)
  const int mp = b.m_d ? min(b.m_d[(size_t)p * b.dim_stride], b.m) : b.m;
  const int np = b.n_d ? min(b.n_d[(size_t)p * b.dim_stride], b.n) : b.n;
  if (m0 >= mp || n0 >= 2 * np) return;  // tile outside this problem: uniform over the CTA
  const int nk = b.k_pad / kTcBK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // whole warp: allocate kTcBN TMEM columns (128 lanes x FP32)
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"((uint32_t)kTcBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer ----
    const uint32_t bytes = planes * (kTileA + kTileB);
    int issued = 0;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages;
      if (kb >= kStages && !mbar_wait(&empty[s], ((kb / kStages) & 1) ^ 1, abort)) {
        *abort = 1;
        atomicExch(err, 1);
        break;
      }
      mbar_expect_tx(&full[s], bytes);
      for (int q = 0; q < planes; ++q)
        tma_load_3d(sA + (size_t)(s * planes + q) * kTileA, &tmA, &full[s], kb * kTcBK, m0, q * b.nprob + p);
      for (int q = 0; q < planes; ++q)
        tma_load_3d(sB + (size_t)(s * planes + q) * kTileB, &tmB, &full[s], kb * kTcBK, n0, q * b.nprob + p);
      issued = kb + 1;
    }
    if (*abort)  // drain: the last copies issued into each stage must land before the CTA exits
      for (int kb = issued - kStages < 0 ? 0 : issued - kStages; kb < issued; ++kb)
        mbar_wait(&full[kb % kStages], (kb / kStages) & 1, nullptr);
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer ----
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages;
      if (!mbar_wait(&full[s], (kb / kStages) & 1, abort)) {
        *abort = 1;
        atomicExch(err, 1);
        break;
      }
      tc_after();
      const uint32_t a0 = su32(sA + (size_t)s * planes * kTileA);
      const uint32_t b0 = su32(sB + (size_t)s * planes * kTileB);
#pragma unroll
      for (int kk = 0; kk < kTcBK / 8; ++kk) {
        const uint32_t off = kk * 32;  // 8 TF32 = 32 bytes per K-step
        const uint32_t first = (kb == 0 && kk == 0) ? 0u : 1u;
        if (planes == 2) {
          // small terms first: lo*hi, hi*lo, then hi*hi
          mma_tf32(tmem, sw128_desc(a0 + kTileA + off), sw128_desc(b0 + off), first);
          mma_tf32(tmem, sw128_desc(a0 + off), sw128_desc(b0 + kTileB + off), 1u);
          mma_tf32(tmem, sw128_desc(a0 + off), sw128_desc(b0 + off), 1u);
        } else {
          mma_tf32(tmem, sw128_desc(a0 + off), sw128_desc(b0 + off), first);
        }
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();

  // ---- epilogue ----
  const bool ok = mbar_wait(done, 0, nullptr);
  tc_after();
  if (ok && !*abort) {
    const int row = m0 + warp * 32 + lane;
    double2 *out = b.optr ? *reinterpret_cast<double2 *const *>(b.optr + (size_t)p * b.optr_stride)
                          : b.out + (size_t)p * b.out_stride;
    const long long cs = b.cs ? b.cs : mp;  // cs == 0: column stride = this problem's row count
#pragma unroll 1
    for (int c0 = 0; c0 < kTcBN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (row < mp) {
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const int j = (n0 + c0) / 2 + t;
          if (j < np) {
            double2 *o = out + (long long)row * b.rs + (long long)j * cs;
            double2 r = make_double2(b.alpha * (double)v[2 * t], b.alpha * (double)v[2 * t + 1]);
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
  } else if (!ok) {
    atomicExch(err, 1);
  }
  tc_before();
  __syncthreads();
  if (warp == 0) {
    tc_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kTcBN)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// packing: complex FP64 -> TF32 planes (K-major, zero padded)
// ---------------------------------------------------------------------------
// Round an FP32 value to TF32 (10-bit significand), to nearest with ties away
// from zero, keeping the FP32 container (the low 13 bits become zero).
__device__ __forceinline__ float tf32r(float x) {
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  return __uint_as_float(u);
}

__device__ __forceinline__ void split(double x, int form, float &hi, float &lo) {
  hi = tf32r((float)x);
  lo = form == kTc3xTF32 ? tf32r((float)(x - (double)hi)) : 0.f;
}

// A planes: element (i, k) of the complex rows x cols matrix -> plane row i,
// columns 2k, 2k+1.  32 x 32 complex tile per block through shared memory, so
// that both the source reads (either orientation) and the plane writes coalesce.
__global__ void __launch_bounds__(256) k_tc_pack_a(const double2 *src, long long pstride, int ld, int rows,
                                                   int cols, int trans, int conj, int nprob, int m_pad,
                                                   int k_pad, int form, float *planes) {
  __shared__ double2 tile[32][33];
  const int p = blockIdx.z;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const double2 *S = src + (size_t)p * pstride;
  for (int yy = ty; yy < 32; yy += 8) {
    // trans == 0: column k0+yy, rows i0+tx (contiguous); trans == 1: row i0+yy, columns k0+tx
    const int i = trans ? i0 + yy : i0 + tx, k = trans ? k0 + tx : k0 + yy;
    double2 v = make_double2(0.0, 0.0);
    if (i < rows && k < cols) v = trans ? S[k + (size_t)ld * i] : S[i + (size_t)ld * k];
    if (conj) v.y = -v.y;
    if (trans)
      tile[yy][tx] = v;  // tile[i - i0][k - k0]
    else
      tile[tx][yy] = v;
  }
  __syncthreads();
  const size_t plane_sz = (size_t)nprob * m_pad * k_pad;
  for (int yy = ty; yy < 32; yy += 8) {
    const int i = i0 + yy, k = k0 + tx;
    if (i >= m_pad || 2 * k >= k_pad) continue;
    const double2 v = tile[yy][tx];
    float hr, lr, hi_, li;
    split(v.x, form, hr, lr);
    split(v.y, form, hi_, li);
    float2 *dst = reinterpret_cast<float2 *>(planes + ((size_t)p * m_pad + i) * k_pad + 2 * k);
    dst[0] = make_float2(hr, hi_);
    if (form == kTc3xTF32) dst[plane_sz / 2] = make_float2(lr, li);
  }
}

// B planes: element (k, j) of the complex krows x ncols matrix -> plane rows 2j
// (re, -im per k) and 2j+1 (im, re per k).
__global__ void __launch_bounds__(256) k_tc_pack_b(const double2 *src, long long pstride, int ld, int krows,
                                                   int ncols, int trans, int conj, int nprob, int n_pad,
                                                   int k_pad, int form, float *planes) {
  __shared__ double2 tile[32][33];
  const int p = blockIdx.z;
  const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const double2 *S = src + (size_t)p * pstride;
  for (int yy = ty; yy < 32; yy += 8) {
    // trans == 0: column j0+yy, rows k0+tx (contiguous); trans == 1: row k0+yy, columns j0+tx
    const int j = trans ? j0 + tx : j0 + yy, k = trans ? k0 + yy : k0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (k < krows && j < ncols) v = trans ? S[j + (size_t)ld * k] : S[k + (size_t)ld * j];
    if (conj) v.y = -v.y;
    if (trans)
      tile[tx][yy] = v;  // tile[j - j0][k - k0]
    else
      tile[yy][tx] = v;
  }
  __syncthreads();
  const size_t plane_sz = (size_t)nprob * n_pad * k_pad;
  for (int yy = ty; yy < 32; yy += 8) {
    const int j = j0 + yy, k = k0 + tx;
    if (2 * j + 1 >= n_pad || 2 * k >= k_pad) continue;
    const double2 v = tile[yy][tx];
    float hr, lr, hi_, li, hn, ln;
    split(v.x, form, hr, lr);
    split(v.y, form, hi_, li);
    hn = -hi_;
    ln = -li;
    float *r0 = planes + ((size_t)p * n_pad + 2 * j) * k_pad + 2 * k;
    float *r1 = r0 + k_pad;
    *reinterpret_cast<float2 *>(r0) = make_float2(hr, hn);
    *reinterpret_cast<float2 *>(r1) = make_float2(hi_, hr);
    if (form == kTc3xTF32) {
      *reinterpret_cast<float2 *>(r0 + plane_sz) = make_float2(lr, ln);
      *reinterpret_cast<float2 *>(r1 + plane_sz) = make_float2(li, lr);
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

// 3-D map over [depth][rows][k] FP32 with a 32 x box_rows box, 128-byte swizzle.
bool make_map(CUtensorMap *map, const float *base, int k_pad, int rows, int depth, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)k_pad, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)k_pad * 4, (cuuint64_t)k_pad * 4 * rows};
  cuuint32_t box[3] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t tc_gemm_launch(const TcBatch &b, int *err_d, cudaStream_t st) {
  if (b.m_pad % kTcBM || b.n_pad % kTcBN || b.k_pad % kTcBK || b.k_pad <= 0 || b.nprob <= 0 ||
      (b.form != kTc1xTF32 && b.form != kTc3xTF32))
    return cudaErrorInvalidValue;
  const int planes = tc_planes(b.form);
  CUtensorMap ma, mb;
  if (!make_map(&ma, b.a_planes, b.k_pad, b.m_pad, planes * b.nprob, kTcBM) ||
      !make_map(&mb, b.b_planes, b.k_pad, b.n_pad, planes * b.nprob, kTcBN))
    return cudaErrorInvalidValue;
  const size_t smem = smem_bytes(planes);
  cudaError_t e = cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(b.m_pad / kTcBM, b.n_pad / kTcBN, b.nprob);
  k_tc_gemm<<<grid, kThreads, smem, st>>>(ma, mb, b, err_d);
  return cudaPeekAtLastError();
}

cudaError_t tc_pack_a(const double2 *src, long long pstride, int ld, int rows, int cols, int trans, int conj,
                      int nprob, int m_pad, int k_pad, int form, float *planes, cudaStream_t st) {
  dim3 grid((m_pad + 31) / 32, (k_pad / 2 + 31) / 32, nprob);
  k_tc_pack_a<<<grid, 256, 0, st>>>(src, pstride, ld, rows, cols, trans, conj, nprob, m_pad, k_pad, form,
                                   planes);
  return cudaPeekAtLastError();
}

cudaError_t tc_pack_b(const double2 *src, long long pstride, int ld, int krows, int ncols, int trans,
                      int conj, int nprob, int n_pad, int k_pad, int form, float *planes, cudaStream_t st) {
  dim3 grid((n_pad / 2 + 31) / 32, (k_pad / 2 + 31) / 32, nprob);
  k_tc_pack_b<<<grid, 256, 0, st>>>(src, pstride, ld, krows, ncols, trans, conj, nprob, n_pad, k_pad, form,
                                   planes);
  return cudaPeekAtLastError();
}

}  // namespace tebd

namespace tebd {

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

struct ZDims {
  int m_pad, n_pad, k_pad, planes;
};
static ZDims zdims(const ZProd &z) {
  ZDims d;
  const bool oz = zprod_oz(z.form);
  d.m_pad = tc_pad(z.m, kTcBM);
  d.n_pad = tc_pad(2 * z.n, oz ? kOzBN : kTcBN);
  d.k_pad = tc_pad(2 * z.k, oz ? kOzBK : kTcBK);
  d.planes = oz ? z.form - 100 : tc_planes(z.form);
  return d;
}

double zprod_mma_flops(const ZProd &z, int active) {
  const ZDims d = zdims(z);
  const double pairs = zprod_oz(z.form) ? d.planes * (d.planes + 1) / 2.0 : (z.form == kTc3xTF32 ? 3.0 : 1.0);
  return pairs * 2.0 * d.m_pad * (double)d.n_pad * d.k_pad * active;
}

size_t zprod_ws_bytes(const ZProd &z) {
  const ZDims d = zdims(z);
  const size_t el = zprod_oz(z.form) ? 2 : 4;
  size_t b = al256(el * d.planes * (size_t)z.nprob * d.m_pad * d.k_pad) +
             al256(el * d.planes * (size_t)z.nprob * d.n_pad * d.k_pad);
  if (zprod_oz(z.form)) b += al256(sizeof(int) * (size_t)z.nprob * d.m_pad) + al256(sizeof(int) * (size_t)z.nprob * d.n_pad / 2);
  return b;
}

cudaError_t zprod_run(const ZProd &z, void *ws, int *err_d, cudaStream_t st) {
  const ZDims d = zdims(z);
  char *p = static_cast<char *>(ws);
  const size_t el = zprod_oz(z.form) ? 2 : 4;
  char *pa = p;
  p += al256(el * d.planes * (size_t)z.nprob * d.m_pad * d.k_pad);
  char *pb = p;
  p += al256(el * d.planes * (size_t)z.nprob * d.n_pad * d.k_pad);
  cudaError_t e;
  if (zprod_oz(z.form)) {
    int *ea = reinterpret_cast<int *>(p);
    p += al256(sizeof(int) * (size_t)z.nprob * d.m_pad);
    int *eb = reinterpret_cast<int *>(p);
    const int S = d.planes;
    auto *da = reinterpret_cast<unsigned short *>(pa);
    auto *db = reinterpret_cast<unsigned short *>(pb);
    if (z.a_dig) {  // packed by the caller, reused across products
      da = const_cast<unsigned short *>(z.a_dig);
      ea = const_cast<int *>(z.a_exp);
    } else if ((e = oz_pack_a(z.a, z.a_stride, z.lda, z.m, z.k, z.a_trans, z.a_conj, z.nprob, d.m_pad, d.k_pad,
                              S, da, ea, st)) != cudaSuccess) {
      return e;
    }
    if ((e = oz_pack_b(z.b, z.b_stride, z.ldb, z.k, z.n, z.b_trans, z.b_conj, z.nprob, d.n_pad, d.k_pad, S, db,
                       eb, st)) != cudaSuccess)
      return e;
    OzBatch b = {};
    b.a_dig = da;
    b.b_dig = db;
    b.a_exp = ea;
    b.b_exp = eb;
    b.nprob = z.nprob;
    b.m_pad = d.m_pad;
    b.n_pad = d.n_pad;
    b.k_pad = d.k_pad;
    b.slices = S;
    b.out = z.out;
    b.out_stride = z.out_stride;
    b.rs = z.rs;
    b.cs = z.cs;
    b.m_d = z.m_d;
    b.n_d = z.n_d;
    b.dim_stride = z.dim_stride;
    b.m = z.m;
    b.n = z.n;
    b.accumulate = z.accumulate;
    b.alpha = z.alpha;
    b.optr = z.optr;
    b.optr_stride = z.optr_stride;
    if (z.ev0) cudaEventRecord(z.ev0, st);
    e = oz_gemm_launch(b, err_d, st);
    if (z.ev1) cudaEventRecord(z.ev1, st);
    return e;
  }
  float *fa = reinterpret_cast<float *>(pa), *fb = reinterpret_cast<float *>(pb);
  if ((e = tc_pack_a(z.a, z.a_stride, z.lda, z.m, z.k, z.a_trans, z.a_conj, z.nprob, d.m_pad, d.k_pad, z.form,
                     fa, st)) != cudaSuccess ||
      (e = tc_pack_b(z.b, z.b_stride, z.ldb, z.k, z.n, z.b_trans, z.b_conj, z.nprob, d.n_pad, d.k_pad, z.form,
                     fb, st)) != cudaSuccess)
    return e;
  TcBatch b = {};
  b.a_planes = fa;
  b.b_planes = fb;
  b.nprob = z.nprob;
  b.m_pad = d.m_pad;
  b.n_pad = d.n_pad;
  b.k_pad = d.k_pad;
  b.form = z.form;
  b.out = z.out;
  b.out_stride = z.out_stride;
  b.rs = z.rs;
  b.cs = z.cs;
  b.m_d = z.m_d;
  b.n_d = z.n_d;
  b.dim_stride = z.dim_stride;
  b.m = z.m;
  b.n = z.n;
  b.accumulate = z.accumulate;
  b.alpha = z.alpha;
  b.optr = z.optr;
  b.optr_stride = z.optr_stride;
  if (z.ev0) cudaEventRecord(z.ev0, st);
  e = tc_gemm_launch(b, err_d, st);
  if (z.ev1) cudaEventRecord(z.ev1, st);
  return e;
}

}  // namespace tebd

// ---------------------------------------------------------------------------
// C ABI: the complex product on its own (diagnostics; no counterpart in the
// reference, which multiplies only inside FormTheta)
// ---------------------------------------------------------------------------
using namespace tebd;

extern "C" int tebd_zgemm_tc(int nprob, int m, int n, int k, const double *A, long long stride_a, int lda,
                             const double *B, long long stride_b, int ldb, double *C, long long stride_c,
                             int ldc, int form, void *stream) {
  if (nprob < 1 || m < 1 || n < 1 || k < 1 || !A || !B || !C || lda < m || ldb < k || ldc < m ||
      (form != kTc1xTF32 && form != kTc3xTF32 && !zprod_oz(form)))
    return TEBD_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ZProd z = {};
  z.a = reinterpret_cast<const double2 *>(A);
  z.a_stride = stride_a;
  z.lda = lda;
  z.b = reinterpret_cast<const double2 *>(B);
  z.b_stride = stride_b;
  z.ldb = ldb;
  z.nprob = nprob;
  z.m = m;
  z.n = n;
  z.k = k;
  z.form = form;
  z.out = reinterpret_cast<double2 *>(C);
  z.out_stride = stride_c;
  z.rs = 1;
  z.cs = ldc;
  z.alpha = 1.0;
  void *ws = nullptr;
  int *err = nullptr;
  int rc = TEBD_OK, herr = 0;
  cudaError_t e = cudaSuccess;
  if (cudaMalloc(&ws, zprod_ws_bytes(z)) != cudaSuccess || cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
    rc = TEBD_ERR_OOM;
    set_noh_error("tebd_zgemm_tc: out of device memory");
  } else if ((e = cudaMemsetAsync(err, 0, sizeof(int), st)) != cudaSuccess || (e = zprod_run(z, ws, err, st)) != cudaSuccess ||
             (e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
             (e = cudaStreamSynchronize(st)) != cudaSuccess || herr) {
    rc = TEBD_ERR_CUDA;
    set_noh_error(e != cudaSuccess ? std::string("tebd_zgemm_tc: ") + cudaGetErrorString(e)
                                   : std::string("tebd_zgemm_tc: a pipeline wait of the product kernel expired"));
  }
  (void)cudaGetLastError();
  cudaFree(ws);
  cudaFree(err);
  return rc;
}
