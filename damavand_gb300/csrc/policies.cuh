// Arithmetic policies and the in-tile op loop shared by the single-state
// window kernel and the batched persistent kernel.
//
// A policy names G, the amplitude type in HBM; T, the working type in
// registers and shared memory; Mat, an op's matrix in registers; and how to
// convert and apply.
#pragma once

#include <cuda_runtime.h>

#include "complex_ops.cuh"
#include "df.cuh"
#include "internal.h"

namespace dmv {

struct PolF64 {  // complex128, IEEE FP64 multiply-adds
  using G = double2;
  using T = double2;
  using Mat = M2<double>;
  static Mat mat(const Op& op) { return to_m2<double>(op.m); }
  __device__ static Mat dmat(const Op& op) { return to_m2<double>(op.m); }
  template <int CLS>
  __device__ static void apply(const Mat& m, T& a0, T& a1) { apply_pair<double, CLS>(m, a0, a1); }
  __device__ static T in(const G& g) { return g; }
  __device__ static G out(const T& t) { return t; }
};

struct PolF32 {  // complex64, FP32 multiply-adds
  using G = float2;
  using T = float2;
  using Mat = M2<float>;
  static Mat mat(const Op& op) { return to_m2<float>(op.m); }
  __device__ static Mat dmat(const Op& op) { return to_m2<float>(op.m); }
  template <int CLS>
  __device__ static void apply(const Mat& m, T& a0, T& a1) { apply_pair<float, CLS>(m, a0, a1); }
  __device__ static T in(const G& g) { return g; }
  __device__ static G out(const T& t) { return t; }
};

struct PolDF {  // complex128 storage, FP32-pair arithmetic (df.cuh)
  using G = double2;
  using T = float4;
  using Mat = DFMat;
  static Mat mat(const Op& op) {
    Mat m;
    for (int i = 0; i < 8; ++i) {
      m.h[i] = op.mh[i];
      m.l[i] = op.ml[i];
    }
    return m;
  }
  __device__ static Mat dmat(const Op& op) {
    Mat m;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      m.h[i] = op.mh[i];
      m.l[i] = op.ml[i];
    }
    return m;
  }
  template <int CLS>
  __device__ static void apply(const Mat& m, T& a0, T& a1) { df_apply_pair<CLS>(m, a0, a1); }
  __device__ static T in(const G& g) { return df_from_double2(g); }
  __device__ static G out(const T& t) { return df_to_double2(t); }
};

// One op over a tile of T amplitudes in shared memory, all threads of the CTA.
template <typename P, int CLS>
__device__ __forceinline__ void tile_op(typename P::T* tile, int T, const Op& op) {
  using V = typename P::T;
  const typename P::Mat m = P::dmat(op);
  const int t = op.target;
  if (op.ctrl_kind == CTRL_LOCAL) {
    const int c = op.ctrl;
    const int lo = min(t, c), hi = max(t, c);
    for (int q = threadIdx.x; q < (T >> 2); q += blockDim.x) {
      const uint32_t l0 = insert_zero32(insert_zero32((uint32_t)q, lo), hi) | (1u << c);
      const uint32_t l1 = l0 | (1u << t);
      V a0 = tile[l0], a1 = tile[l1];
      P::template apply<CLS>(m, a0, a1);
      tile[l0] = a0;
      tile[l1] = a1;
    }
  } else {
    // Two independent pairs per iteration: both are loaded before either is
    // stored, so their arithmetic chains interleave.
    const int half = T >> 1;
    const int bd = blockDim.x;
    for (int q = threadIdx.x; q < half; q += 2 * bd) {
      const int q2 = q + bd;
      const uint32_t l0 = insert_zero32((uint32_t)q, t);
      const uint32_t l1 = l0 | (1u << t);
      V a0 = tile[l0], a1 = tile[l1];
      if (q2 < half) {
        const uint32_t m0 = insert_zero32((uint32_t)q2, t);
        const uint32_t m1 = m0 | (1u << t);
        V b0 = tile[m0], b1 = tile[m1];
        P::template apply<CLS>(m, a0, a1);
        P::template apply<CLS>(m, b0, b1);
        tile[m0] = b0;
        tile[m1] = b1;
      } else {
        P::template apply<CLS>(m, a0, a1);
      }
      tile[l0] = a0;
      tile[l1] = a1;
    }
  }
}

// Every op of a pass on one tile; `base` holds the tile's global index bits
// (controls outside the tile are read from it). Ends with a barrier after
// each applied op.
template <typename P>
__device__ __forceinline__ void tile_apply_ops(typename P::T* tile, int T, const Op* ops, int num_ops, int64_t base) {
  for (int o = 0; o < num_ops; ++o) {
    const Op& op = ops[o];
    if (op.ctrl_kind == CTRL_GLOBAL && !((base >> op.ctrl) & 1)) continue;  // uniform per tile
    switch (op.cls) {
      case OP_SWAP: tile_op<P, OP_SWAP>(tile, T, op); break;
      case OP_DIAG: tile_op<P, OP_DIAG>(tile, T, op); break;
      case OP_ANTI: tile_op<P, OP_ANTI>(tile, T, op); break;
      case OP_REAL: tile_op<P, OP_REAL>(tile, T, op); break;
      default: tile_op<P, OP_GENERAL>(tile, T, op); break;
    }
    __syncthreads();
  }
}

}  // namespace dmv
