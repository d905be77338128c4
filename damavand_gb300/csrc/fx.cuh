// Block fixed-point arithmetic for complex128 statevectors on the integer pipe.
//
// GB300 issues ~64 32-bit integer multiply-adds per clock per SM (IMAD,
// IMAD.WIDE) but only ~2 FP64 ones. Here a block of amplitudes (a shared
// memory tile, or one amplitude pair) is converted, with integer operations,
// to int64 fixed point with a shared exponent: with Emax the largest biased
// FP64 exponent in the block, component x becomes X = x * 2^(1076 - Emax),
// so the block's largest components have 54 fraction bits (FP64 has 53) and
// |X| < 2^54. Gates are unitary, so no component of a block ever exceeds the
// block's 2-norm, at most sqrt(block size) times its largest component: a
// 4096-amplitude tile needs 6 more bits, and every X stays below 2^60.
//
// Matrix entries (|m| <= 1) are Q.54 fixed point M = round(m * 2^54). A
// product is formed exactly from 31-bit limbs, x = xh*2^31 + xl and
// m = mh*2^31 + ml with xl, ml in [0, 2^31):
//   x*m = 2^62 xh mh + 2^31 (xh ml + xl mh) + xl ml
// and a sum of such products is rounded once, to nearest, back to Q.54.
// Each limb product is one IMAD.WIDE with the 64-bit accumulation folded in.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace dmv {

constexpr int kFxFrac = 54;

// Biased FP64 exponent field of x (0 for zero and subnormals).
__device__ __forceinline__ int fx_exponent(double x) {
  return (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FFull);
}

// x -> X = round(x * 2^(1076 - emax)); emax >= the exponent of x.
__device__ __forceinline__ long long fx_from_double(double x, int emax) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FFull);
  if (E == 0) return 0;  // zero or subnormal (below 2^-1022): flushed
  const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int s = emax - E - 1;  // right shift; -1 means a left shift by one
  unsigned long long X;
  if (s < 0) X = M << 1;
  else if (s == 0) X = M;
  else if (s < 63) X = (M + (1ull << (s - 1))) >> s;
  else X = 0;
  return (b >> 63) ? -(long long)X : (long long)X;
}

// X * 2^(emax - 1076) -> the nearest double (ties away from zero).
__device__ __forceinline__ double fx_to_double(long long X, int emax) {
  if (X == 0) return 0.0;
  const unsigned long long sign = X < 0 ? (1ull << 63) : 0ull;
  unsigned long long A = X < 0 ? (unsigned long long)(-X) : (unsigned long long)X;
  int p = 63 - __clzll((long long)A);  // position of the leading one
  unsigned long long Mn;
  if (p > 52) {
    const int s = p - 52;
    Mn = (A + (1ull << (s - 1))) >> s;
    if (Mn >> 53) {  // rounding carried into a new leading bit
      Mn >>= 1;
      ++p;
    }
  } else {
    Mn = A << (52 - p);
  }
  const int E = p + emax - 53;
  if (E <= 0) return 0.0;  // below the normal range: flushed
  return __longlong_as_double((long long)(sign | ((unsigned long long)E << 52) | (Mn & 0xFFFFFFFFFFFFFull)));
}

// A matrix as Q.54 limbs: entry k (m00r, m00i, m01r, m01i, m10r, m10i, m11r,
// m11i) is h[k] * 2^31 + l[k], l[k] in [0, 2^31).
struct FXMat {
  int h[8], l[8];
};

// Sum of limb products: S = 2^62 A + 2^31 B + C.
struct FXAcc {
  long long A, B;
  unsigned long long C;
};

__device__ __forceinline__ void fx_zero(FXAcc& a) {
  a.A = 0;
  a.B = 0;
  a.C = 0ull;
}

// acc += m * x, m = (mh, ml), x = (xh, xl) in limbs.
__device__ __forceinline__ void fx_mac(FXAcc& a, int mh, int ml, int xh, int xl) {
  a.A += (long long)xh * mh;
  a.B += (long long)xh * ml + (long long)xl * mh;
  a.C += (unsigned long long)(unsigned)xl * (unsigned)ml;
}

// round((S_pos - S_neg) / 2^54). C / 2^54 is folded in as (C >> 31) / 2^23,
// which drops less than 2^-23 of a unit before the single rounding.
__device__ __forceinline__ long long fx_result(const FXAcc& p, const FXAcc& n) {
  const long long A = p.A - n.A;
  const long long B = p.B - n.B + (long long)(p.C >> 31) - (long long)(n.C >> 31);
  return (A << 8) + ((B + (1ll << 22)) >> 23);
}

__device__ __forceinline__ long long fx_result(const FXAcc& p) {
  return (p.A << 8) + ((p.B + (long long)(p.C >> 31) + (1ll << 22)) >> 23);
}

__device__ __forceinline__ void fx_limbs(long long x, int& xh, int& xl) {
  xh = (int)(x >> 31);
  xl = (int)(x & 0x7FFFFFFFll);
}

// (a0, a1) <- M (a0, a1) on longlong2 (x = re, y = im) Q.54 values.
template <int CLS>
__device__ __forceinline__ void fx_apply_pair(const FXMat& m, longlong2& a0, longlong2& a1) {
  if constexpr (CLS == OP_SWAP) {
    const longlong2 t = a0;
    a0 = a1;
    a1 = t;
    return;
  } else {
    int r0h, r0l, i0h, i0l, r1h, r1l, i1h, i1l;
    fx_limbs(a0.x, r0h, r0l);
    fx_limbs(a0.y, i0h, i0l);
    fx_limbs(a1.x, r1h, r1l);
    fx_limbs(a1.y, i1h, i1l);
    FXAcc p, n;
    longlong2 b0, b1;
    if constexpr (CLS == OP_DIAG) {
      // out0 = m00 a0, out1 = m11 a1
      fx_zero(p); fx_zero(n);
      fx_mac(p, m.h[0], m.l[0], r0h, r0l); fx_mac(n, m.h[1], m.l[1], i0h, i0l);
      b0.x = fx_result(p, n);
      fx_zero(p);
      fx_mac(p, m.h[0], m.l[0], i0h, i0l); fx_mac(p, m.h[1], m.l[1], r0h, r0l);
      b0.y = fx_result(p);
      fx_zero(p); fx_zero(n);
      fx_mac(p, m.h[6], m.l[6], r1h, r1l); fx_mac(n, m.h[7], m.l[7], i1h, i1l);
      b1.x = fx_result(p, n);
      fx_zero(p);
      fx_mac(p, m.h[6], m.l[6], i1h, i1l); fx_mac(p, m.h[7], m.l[7], r1h, r1l);
      b1.y = fx_result(p);
    } else if constexpr (CLS == OP_ANTI) {
      // out0 = m01 a1, out1 = m10 a0
      fx_zero(p); fx_zero(n);
      fx_mac(p, m.h[2], m.l[2], r1h, r1l); fx_mac(n, m.h[3], m.l[3], i1h, i1l);
      b0.x = fx_result(p, n);
      fx_zero(p);
      fx_mac(p, m.h[2], m.l[2], i1h, i1l); fx_mac(p, m.h[3], m.l[3], r1h, r1l);
      b0.y = fx_result(p);
      fx_zero(p); fx_zero(n);
      fx_mac(p, m.h[4], m.l[4], r0h, r0l); fx_mac(n, m.h[5], m.l[5], i0h, i0l);
      b1.x = fx_result(p, n);
      fx_zero(p);
      fx_mac(p, m.h[4], m.l[4], i0h, i0l); fx_mac(p, m.h[5], m.l[5], r0h, r0l);
      b1.y = fx_result(p);
    } else if constexpr (CLS == OP_REAL) {
      fx_zero(p);
      fx_mac(p, m.h[0], m.l[0], r0h, r0l); fx_mac(p, m.h[2], m.l[2], r1h, r1l);
      b0.x = fx_result(p);
      fx_zero(p);
      fx_mac(p, m.h[0], m.l[0], i0h, i0l); fx_mac(p, m.h[2], m.l[2], i1h, i1l);
      b0.y = fx_result(p);
      fx_zero(p);
      fx_mac(p, m.h[4], m.l[4], r0h, r0l); fx_mac(p, m.h[6], m.l[6], r1h, r1l);
      b1.x = fx_result(p);
      fx_zero(p);
      fx_mac(p, m.h[4], m.l[4], i0h, i0l); fx_mac(p, m.h[6], m.l[6], i1h, i1l);
      b1.y = fx_result(p);
    } else {
      // out0.re = m00r a0r - m00i a0i + m01r a1r - m01i a1i
      fx_zero(p); fx_zero(n);
      fx_mac(p, m.h[0], m.l[0], r0h, r0l); fx_mac(n, m.h[1], m.l[1], i0h, i0l);
      fx_mac(p, m.h[2], m.l[2], r1h, r1l); fx_mac(n, m.h[3], m.l[3], i1h, i1l);
      b0.x = fx_result(p, n);
      // out0.im = m00r a0i + m00i a0r + m01r a1i + m01i a1r
      fx_zero(p);
      fx_mac(p, m.h[0], m.l[0], i0h, i0l); fx_mac(p, m.h[1], m.l[1], r0h, r0l);
      fx_mac(p, m.h[2], m.l[2], i1h, i1l); fx_mac(p, m.h[3], m.l[3], r1h, r1l);
      b0.y = fx_result(p);
      // out1.re = m10r a0r - m10i a0i + m11r a1r - m11i a1i
      fx_zero(p); fx_zero(n);
      fx_mac(p, m.h[4], m.l[4], r0h, r0l); fx_mac(n, m.h[5], m.l[5], i0h, i0l);
      fx_mac(p, m.h[6], m.l[6], r1h, r1l); fx_mac(n, m.h[7], m.l[7], i1h, i1l);
      b1.x = fx_result(p, n);
      // out1.im = m10r a0i + m10i a0r + m11r a1i + m11i a1r
      fx_zero(p);
      fx_mac(p, m.h[4], m.l[4], i0h, i0l); fx_mac(p, m.h[5], m.l[5], r0h, r0l);
      fx_mac(p, m.h[6], m.l[6], i1h, i1l); fx_mac(p, m.h[7], m.l[7], r1h, r1l);
      b1.y = fx_result(p);
    }
    a0 = b0;
    a1 = b1;
  }
}

}  // namespace dmv
