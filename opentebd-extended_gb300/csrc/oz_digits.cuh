// oz_digits.cuh -- the digit-plane operands of the FP64-class tensor-core
// products (tc_ozaki.cu): error-free splitting of FP64 values into bf16 integer
// digits relative to a row's exponent, and the one-warp-per-line packer shared
// by the strided packers and the gathered (number-conserving block) packers.
#pragma once

#include <stdint.h>

#include "tc_gemm.cuh"

namespace tebd {

constexpr int kExpZero = -2000;  // exponents below this mark an all-zero row

// bf16 bit pattern of an integer |D| <= 128 (exact: at most 8 significant bits)
__device__ __forceinline__ unsigned short oz_bf16_int(int D) {
  if (D == 0) return 0;
  const unsigned a = (unsigned)(D < 0 ? -D : D);
  const int p = 31 - __clz(a);  // 2^p <= a < 2^(p+1), p <= 7
  return (unsigned short)((D < 0 ? 0x8000u : 0u) | ((unsigned)(127 + p) << 7) | ((a << (7 - p)) & 0x7fu));
}

// Digits by integer arithmetic only (the FP64 pipe is the GPU's narrowest; these
// kernels then run at memory speed).  x = +-m 2^E exactly (m the 53-bit
// significand), q = rint(m 2^(E + 7S - e)) by a shift with rounding (ties away
// from zero), |q| < 2^(7S) because |x| < 2^e; then balanced 7-bit digits by
// integer shifts, rounding to nearest at every step: D_0 in [-128, 128], D_s in
// [-64, 64] after it, and x - 2^e sum_s D_s 2^(-7(s+1)) = 2^(e - 7S)(x 2^(7S-e) - q),
// at most 2^(e-7S-1).  Non-finite x and all-zero rows give zero digits.
__device__ __forceinline__ void oz_digits(double x, int e, int S, unsigned short *d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (e <= kExpZero || ex == 0x7ff) {
    for (int s = 0; s < S; ++s) d[s] = 0;
    return;
  }
  long long m = (long long)(b & 0xfffffffffffffULL);
  int E = -1074;
  if (ex) {
    m |= 1LL << 52;
    E = ex - 1075;
  }
  const int sh = E + 7 * S - e;
  long long q = sh >= 0 ? (m << sh) : (-sh <= 62 ? ((m + (1LL << (-sh - 1))) >> (-sh)) : 0LL);
  if (b >> 63) q = -q;
  for (int s = 0; s < S; ++s) {
    const int t = 7 * (S - 1 - s);
    const long long D = t ? ((q + (1LL << (t - 1))) >> t) : q;
    q -= D << t;
    d[s] = oz_bf16_int((int)D);
  }
}

// |x| as its bit pattern, which orders finite magnitudes; non-finite -> 0
__device__ __forceinline__ unsigned long long oz_absbits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  return (b >> 52) == 0x7ff ? 0ULL : b;
}

// e with mag = f 2^e, f in [1/2, 1), from the bit pattern of a positive finite mag
__device__ __forceinline__ int oz_exp_bits(unsigned long long b) {
  const int ex = (int)(b >> 52);
  if (ex) return ex - 1022;
  return (64 - __clzll((long long)b)) - 1074;  // subnormal: mag = b 2^-1074
}

// One warp packs one line of an operand: line r of problem p, an A row or a B
// complex column (stored as the two real rows 2r: (re, -im) and 2r+1: (im, re)),
// with values v(k) for k < ext; zero beyond ext, up to k_pad real K, and the
// whole line when !live.  Two passes over the line (largest magnitude, then
// the digits); the line's exponent goes to exps[p * lines + r].  Digit plane s
// of problem p starts at dig + s * nprob * rows_pad * k_pad.
template <bool kB, class Get>
__device__ __forceinline__ void oz_pack_line(Get v, bool live, int ext, int p, int r, int nprob, int rows_pad,
                                             int k_pad, int S, unsigned short *dig, int *exps) {
  const int lane = threadIdx.x & 31;
  const int lines = kB ? rows_pad / 2 : rows_pad;
  unsigned long long mx = 0;
  if (live)
    for (int k = lane; k < ext; k += 32) {
      const double2 x = v(k);
      mx = max(mx, max(oz_absbits(x.x), oz_absbits(x.y)));
    }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int e = mx ? oz_exp_bits(mx) : (int)0x80808080;
  if (lane == 0) exps[(size_t)p * lines + r] = e;
  const size_t plane = (size_t)nprob * rows_pad * k_pad;
  for (int k = lane; 2 * k < k_pad; k += 32) {
    double2 x = make_double2(0.0, 0.0);
    if (live && k < ext) x = v(k);
    unsigned short dr[kOzMaxS], di[kOzMaxS];
    oz_digits(x.x, e, S, dr);
    oz_digits(x.y, e, S, di);
    if (!kB) {
      unsigned short *o = dig + ((size_t)p * rows_pad + r) * k_pad + 2 * k;
      for (int q = 0; q < S; ++q)
        *reinterpret_cast<uint32_t *>(o + q * plane) = (uint32_t)dr[q] | ((uint32_t)di[q] << 16);
    } else {
      unsigned short *o0 = dig + ((size_t)p * rows_pad + 2 * r) * k_pad + 2 * k;
      unsigned short *o1 = o0 + k_pad;
      for (int q = 0; q < S; ++q) {
        const unsigned short ni = di[q] ^ 0x8000u;  // -im (bf16 sign bit; -0 for 0 is harmless)
        *reinterpret_cast<uint32_t *>(o0 + q * plane) = (uint32_t)dr[q] | ((uint32_t)ni << 16);
        *reinterpret_cast<uint32_t *>(o1 + q * plane) = (uint32_t)di[q] | ((uint32_t)dr[q] << 16);
      }
    }
  }
}

}  // namespace tebd
