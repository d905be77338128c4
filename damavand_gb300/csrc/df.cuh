// FP32-pair ("double-float") arithmetic for complex128 statevectors.
//
// GB300 runs FP32 multiply-adds ~71x faster than FP64 ones (35.9 vs 0.50
// T/s measured), and FP64<->FP32 conversion instructions run at the FP64 rate.
// So a complex128 amplitude is split, with integer operations only, into two
// floats x = hi + lo (48 significant bits), gates are applied with error-free
// transformations (TwoProd through FMA, Knuth's TwoSum) -- the compensated dot
// product of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J.
// Sci. Comput. 26, 2005) with the cross terms of the pairs added to the
// compensation -- and the result is packed back into an IEEE double with
// integer operations. Every rounding step is written with __f*_rn intrinsics
// so the compiler cannot contract it into an FMA (that would break TwoSum).
//
// Range: |x| in [2^-126, 2^128). Smaller magnitudes flush to zero (absolute
// error below 2^-126, irrelevant next to a normalised state); below 2^-102 the
// low float leaves FP32's normal range and the pair keeps fewer than 48 bits.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace dmv {

// x -> (hi, lo): hi = x truncated to 24 significant bits, lo = the remaining
// 29 mantissa bits rounded to 24.
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int top = (unsigned int)(b >> 32);
  const unsigned int sign = top & 0x80000000u;
  const int E = (int)((top >> 20) & 0x7FFu);
  const int ef = E - 896;  // float exponent field (E - 1023 + 127)
  if (ef <= 0 || ef >= 255) {
    hi = 0.f;
    lo = 0.f;
    return;
  }
  const unsigned int m23 = (unsigned int)(b >> 29) & 0x7FFFFFu;
  hi = __uint_as_float(sign | ((unsigned int)ef << 23) | m23);
  // lo = r * 2^(E - 1075), r the low 29 mantissa bits, rounded to 24 bits.
  // No conversion instruction (those run at the FP64 rate): with r = 64 rh + rl,
  // rh * 2^-23 = bits(1.0f | rh) - 1 and rl = bits(2^23 | rl) - 2^23 are exact,
  // and one FMA forms r * 2^-29 rounded to nearest even (the same value as
  // converting r). The weight 2^(E - 1046) is a normal float for E >= 920; below
  // that it is applied in two factors (2^-64 and 2^(E - 982)), so lo keeps its
  // 24 bits while it stays in FP32's normal range (|x| >= 2^-102).
  const unsigned int r = (unsigned int)b & 0x1FFFFFFFu;
  const float fh = __fsub_rn(__uint_as_float(0x3F800000u | (r >> 6)), 1.0f);
  const float fl = __fsub_rn(__uint_as_float(0x4B000000u | (r & 63u)), 8388608.0f);
  const float u = __fmaf_rn(fl, 0x1p-29f, fh);
  float l;
  if (E >= 920) l = __fmul_rn(u, __uint_as_float((unsigned int)(E - 919) << 23));
  else l = __fmul_rn(__fmul_rn(u, 0x1p-64f), __uint_as_float((unsigned int)(E - 855) << 23));
  lo = __uint_as_float(__float_as_uint(l) | sign);
}

// (hi, lo) with |lo| <= ulp(hi) -> the nearest-ish double of hi + lo.
__device__ __forceinline__ double join_f64(float hi, float lo) {
  const unsigned int hb = __float_as_uint(hi);
  const int eh = (int)((hb >> 23) & 0xFFu);
  if (eh == 0 || eh == 255) return 0.0;
  long long X = (long long)((hb & 0x7FFFFFu) | 0x800000u) << 29;  // 53-bit significand of hi
  const unsigned int lb = __float_as_uint(lo);
  const int el = (int)((lb >> 23) & 0xFFu);
  if (el != 0) {
    long long L = (long long)((lb & 0x7FFFFFu) | 0x800000u);
    int d = el - eh + 29;  // weight of lo's unit in units of X's last bit
    if (d > 30) d = 30;    // only reachable with |lo| >> ulp(hi), which normalised pairs never have
    if (d >= 0) L <<= d;
    else if (d > -40) L = (L + (1LL << (-d - 1))) >> (-d);
    else L = 0;
    if ((lb ^ hb) & 0x80000000u) X -= L; else X += L;
  }
  int e = eh;
  if (X >= (1LL << 53)) {
    X = (X + 1) >> 1;
    e += 1;
  } else if (X < (1LL << 52)) {
    X <<= 1;
    e -= 1;
  }
  const unsigned long long bits = ((unsigned long long)(hb & 0x80000000u) << 32) |
                                  ((unsigned long long)(e + 896) << 52) |
                                  ((unsigned long long)X & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// Compensated dot-product accumulator: value = p + s, p the running sum of the
// high products, s the (small) sum of every rounding error and cross term.
struct DFAcc {
  float p, s;
};

__device__ __forceinline__ void df_first(DFAcc& a, float xh, float xl, float yh, float yl) {
  a.p = __fmul_rn(xh, yh);
  a.s = __fmaf_rn(xh, yh, -a.p);  // exact error of the product
  a.s = __fmaf_rn(xh, yl, a.s);
  a.s = __fmaf_rn(xl, yh, a.s);
}

__device__ __forceinline__ void df_add(DFAcc& a, float xh, float xl, float yh, float yl) {
  const float h = __fmul_rn(xh, yh);
  const float r = __fmaf_rn(xh, yh, -h);
  const float t = __fadd_rn(a.p, h);  // TwoSum(p, h) = t + q exactly
  const float z = __fsub_rn(t, a.p);
  const float q = __fadd_rn(__fsub_rn(a.p, __fsub_rn(t, z)), __fsub_rn(h, z));
  a.p = t;
  a.s = __fadd_rn(a.s, __fadd_rn(q, r));
  a.s = __fmaf_rn(xh, yl, a.s);
  a.s = __fmaf_rn(xl, yh, a.s);
}

__device__ __forceinline__ void df_finish(const DFAcc& a, float& hi, float& lo) {
  hi = __fadd_rn(a.p, a.s);  // FastTwoSum: |p| >= |s|
  lo = __fsub_rn(a.s, __fsub_rn(hi, a.p));
}

// A 2x2 matrix as FP32 pairs: h[k] + l[k] is entry k of (m00r, m00i, m01r,
// m01i, m10r, m10i, m11r, m11i).
struct DFMat {
  float h[8], l[8];
};

// Amplitude as float4: x = re_hi, y = re_lo, z = im_hi, w = im_lo.
// (a0, a1) <- M (a0, a1) for the op classes of internal.h.
template <int CLS>
__device__ __forceinline__ void df_apply_pair(const DFMat& m, float4& a0, float4& a1) {
  if constexpr (CLS == OP_SWAP) {
    const float4 t = a0;
    a0 = a1;
    a1 = t;
  } else if constexpr (CLS == OP_DIAG) {
    DFAcc re, im;
    float4 b0, b1;
    df_first(re, m.h[0], m.l[0], a0.x, a0.y);
    df_add(re, -m.h[1], -m.l[1], a0.z, a0.w);
    df_first(im, m.h[0], m.l[0], a0.z, a0.w);
    df_add(im, m.h[1], m.l[1], a0.x, a0.y);
    df_finish(re, b0.x, b0.y);
    df_finish(im, b0.z, b0.w);
    df_first(re, m.h[6], m.l[6], a1.x, a1.y);
    df_add(re, -m.h[7], -m.l[7], a1.z, a1.w);
    df_first(im, m.h[6], m.l[6], a1.z, a1.w);
    df_add(im, m.h[7], m.l[7], a1.x, a1.y);
    df_finish(re, b1.x, b1.y);
    df_finish(im, b1.z, b1.w);
    a0 = b0;
    a1 = b1;
  } else if constexpr (CLS == OP_ANTI) {
    DFAcc re, im;
    float4 b0, b1;
    df_first(re, m.h[2], m.l[2], a1.x, a1.y);
    df_add(re, -m.h[3], -m.l[3], a1.z, a1.w);
    df_first(im, m.h[2], m.l[2], a1.z, a1.w);
    df_add(im, m.h[3], m.l[3], a1.x, a1.y);
    df_finish(re, b0.x, b0.y);
    df_finish(im, b0.z, b0.w);
    df_first(re, m.h[4], m.l[4], a0.x, a0.y);
    df_add(re, -m.h[5], -m.l[5], a0.z, a0.w);
    df_first(im, m.h[4], m.l[4], a0.z, a0.w);
    df_add(im, m.h[5], m.l[5], a0.x, a0.y);
    df_finish(re, b1.x, b1.y);
    df_finish(im, b1.z, b1.w);
    a0 = b0;
    a1 = b1;
  } else if constexpr (CLS == OP_RXLIKE) {
    // m00 = m[0], m11 = m[6] real; m01 = i m[3], m10 = i m[5]: four 2-term dots
    DFAcc acc;
    float4 b0, b1;
    df_first(acc, m.h[0], m.l[0], a0.x, a0.y);  // m0 a0r - m3 a1i
    df_add(acc, -m.h[3], -m.l[3], a1.z, a1.w);
    df_finish(acc, b0.x, b0.y);
    df_first(acc, m.h[0], m.l[0], a0.z, a0.w);  // m0 a0i + m3 a1r
    df_add(acc, m.h[3], m.l[3], a1.x, a1.y);
    df_finish(acc, b0.z, b0.w);
    df_first(acc, -m.h[5], -m.l[5], a0.z, a0.w);  // -m5 a0i + m6 a1r
    df_add(acc, m.h[6], m.l[6], a1.x, a1.y);
    df_finish(acc, b1.x, b1.y);
    df_first(acc, m.h[5], m.l[5], a0.x, a0.y);  // m5 a0r + m6 a1i
    df_add(acc, m.h[6], m.l[6], a1.z, a1.w);
    df_finish(acc, b1.z, b1.w);
    a0 = b0;
    a1 = b1;
  } else if constexpr (CLS == OP_REAL) {
    DFAcc acc;
    float4 b0, b1;
    df_first(acc, m.h[0], m.l[0], a0.x, a0.y);
    df_add(acc, m.h[2], m.l[2], a1.x, a1.y);
    df_finish(acc, b0.x, b0.y);
    df_first(acc, m.h[0], m.l[0], a0.z, a0.w);
    df_add(acc, m.h[2], m.l[2], a1.z, a1.w);
    df_finish(acc, b0.z, b0.w);
    df_first(acc, m.h[4], m.l[4], a0.x, a0.y);
    df_add(acc, m.h[6], m.l[6], a1.x, a1.y);
    df_finish(acc, b1.x, b1.y);
    df_first(acc, m.h[4], m.l[4], a0.z, a0.w);
    df_add(acc, m.h[6], m.l[6], a1.z, a1.w);
    df_finish(acc, b1.z, b1.w);
    a0 = b0;
    a1 = b1;
  } else {
    DFAcc acc;
    float4 b0, b1;
    // out0.re = m00r a0r - m00i a0i + m01r a1r - m01i a1i
    df_first(acc, m.h[0], m.l[0], a0.x, a0.y);
    df_add(acc, -m.h[1], -m.l[1], a0.z, a0.w);
    df_add(acc, m.h[2], m.l[2], a1.x, a1.y);
    df_add(acc, -m.h[3], -m.l[3], a1.z, a1.w);
    df_finish(acc, b0.x, b0.y);
    // out0.im = m00r a0i + m00i a0r + m01r a1i + m01i a1r
    df_first(acc, m.h[0], m.l[0], a0.z, a0.w);
    df_add(acc, m.h[1], m.l[1], a0.x, a0.y);
    df_add(acc, m.h[2], m.l[2], a1.z, a1.w);
    df_add(acc, m.h[3], m.l[3], a1.x, a1.y);
    df_finish(acc, b0.z, b0.w);
    // out1.re = m10r a0r - m10i a0i + m11r a1r - m11i a1i
    df_first(acc, m.h[4], m.l[4], a0.x, a0.y);
    df_add(acc, -m.h[5], -m.l[5], a0.z, a0.w);
    df_add(acc, m.h[6], m.l[6], a1.x, a1.y);
    df_add(acc, -m.h[7], -m.l[7], a1.z, a1.w);
    df_finish(acc, b1.x, b1.y);
    // out1.im = m10r a0i + m10i a0r + m11r a1i + m11i a1r
    df_first(acc, m.h[4], m.l[4], a0.z, a0.w);
    df_add(acc, m.h[5], m.l[5], a0.x, a0.y);
    df_add(acc, m.h[6], m.l[6], a1.z, a1.w);
    df_add(acc, m.h[7], m.l[7], a1.x, a1.y);
    df_finish(acc, b1.z, b1.w);
    a0 = b0;
    a1 = b1;
  }
}

__device__ __forceinline__ float4 df_from_double2(const double2 v) {
  float4 o;
  split_f64(v.x, o.x, o.y);
  split_f64(v.y, o.z, o.w);
  return o;
}

__device__ __forceinline__ double2 df_to_double2(const float4 v) {
  return make_double2(join_f64(v.x, v.y), join_f64(v.z, v.w));
}

}  // namespace dmv
