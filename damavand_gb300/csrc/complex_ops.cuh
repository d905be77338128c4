// Device-side complex helpers and the 2x2 pair update, specialised per op class.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace dmv {

template <typename R> struct VecOf;
template <> struct VecOf<double> { using T = double2; };
template <> struct VecOf<float> { using T = float2; };

// 2x2 matrix held in registers in the storage precision.
template <typename R>
struct M2 {
  R r00, i00, r01, i01, r10, i10, r11, i11;
};

template <typename R>
__host__ __device__ inline M2<R> to_m2(const double m[8]) {
  M2<R> o;
  o.r00 = (R)m[0]; o.i00 = (R)m[1]; o.r01 = (R)m[2]; o.i01 = (R)m[3];
  o.r10 = (R)m[4]; o.i10 = (R)m[5]; o.r11 = (R)m[6]; o.i11 = (R)m[7];
  return o;
}

// (a0, a1) <- M (a0, a1). Written with explicit fma so each class costs the
// fewest multiply-adds: GENERAL 16 per pair, REAL/DIAG/ANTI 8, SWAP 0.
template <typename R, int CLS, typename V>
__device__ __forceinline__ void apply_pair(const M2<R>& m, V& a0, V& a1) {
  if constexpr (CLS == OP_SWAP) {
    V t = a0; a0 = a1; a1 = t;
  } else if constexpr (CLS == OP_DIAG) {
    V b0, b1;
    b0.x = fma(m.r00, a0.x, -m.i00 * a0.y);
    b0.y = fma(m.r00, a0.y, m.i00 * a0.x);
    b1.x = fma(m.r11, a1.x, -m.i11 * a1.y);
    b1.y = fma(m.r11, a1.y, m.i11 * a1.x);
    a0 = b0; a1 = b1;
  } else if constexpr (CLS == OP_ANTI) {
    V b0, b1;
    b0.x = fma(m.r01, a1.x, -m.i01 * a1.y);
    b0.y = fma(m.r01, a1.y, m.i01 * a1.x);
    b1.x = fma(m.r10, a0.x, -m.i10 * a0.y);
    b1.y = fma(m.r10, a0.y, m.i10 * a0.x);
    a0 = b0; a1 = b1;
  } else if constexpr (CLS == OP_RXLIKE) {
    // out0 = r00 a0 + i i01 a1, out1 = i i10 a0 + r11 a1
    V b0, b1;
    b0.x = fma(m.r00, a0.x, -m.i01 * a1.y);
    b0.y = fma(m.r00, a0.y, m.i01 * a1.x);
    b1.x = fma(m.r11, a1.x, -m.i10 * a0.y);
    b1.y = fma(m.r11, a1.y, m.i10 * a0.x);
    a0 = b0; a1 = b1;
  } else if constexpr (CLS == OP_REAL) {
    V b0, b1;
    b0.x = fma(m.r00, a0.x, m.r01 * a1.x);
    b0.y = fma(m.r00, a0.y, m.r01 * a1.y);
    b1.x = fma(m.r10, a0.x, m.r11 * a1.x);
    b1.y = fma(m.r10, a0.y, m.r11 * a1.y);
    a0 = b0; a1 = b1;
  } else {
    V b0, b1;
    b0.x = fma(m.r00, a0.x, fma(-m.i00, a0.y, fma(m.r01, a1.x, -m.i01 * a1.y)));
    b0.y = fma(m.r00, a0.y, fma(m.i00, a0.x, fma(m.r01, a1.y, m.i01 * a1.x)));
    b1.x = fma(m.r10, a0.x, fma(-m.i10, a0.y, fma(m.r11, a1.x, -m.i11 * a1.y)));
    b1.y = fma(m.r10, a0.y, fma(m.i10, a0.x, fma(m.r11, a1.y, m.i11 * a1.x)));
    a0 = b0; a1 = b1;
  }
}

template <typename R, typename V>
__device__ __forceinline__ void apply_pair_dyn(int cls, const M2<R>& m, V& a0, V& a1) {
  switch (cls) {
    case OP_SWAP: apply_pair<R, OP_SWAP>(m, a0, a1); break;
    case OP_DIAG: apply_pair<R, OP_DIAG>(m, a0, a1); break;
    case OP_ANTI: apply_pair<R, OP_ANTI>(m, a0, a1); break;
    case OP_REAL: apply_pair<R, OP_REAL>(m, a0, a1); break;
    case OP_RXLIKE: apply_pair<R, OP_RXLIKE>(m, a0, a1); break;
    default: apply_pair<R, OP_GENERAL>(m, a0, a1); break;
  }
}

// Index with a zero bit inserted at position b.
__device__ __forceinline__ int64_t insert_zero(int64_t j, int b) {
  const int64_t low = j & ((int64_t(1) << b) - 1);
  return ((j >> b) << (b + 1)) | low;
}
__device__ __forceinline__ uint32_t insert_zero32(uint32_t j, int b) {
  const uint32_t low = j & ((1u << b) - 1u);
  return ((j >> b) << (b + 1)) | low;
}

template <typename V>
__device__ __forceinline__ double norm2(const V& a) {
  const double x = (double)a.x, y = (double)a.y;
  return fma(x, x, y * y);
}

}  // namespace dmv
