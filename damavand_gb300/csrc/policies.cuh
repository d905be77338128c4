// Arithmetic policies and the in-tile op loop shared by the single-state
// window kernel and the batched persistent kernel.
//
// A policy names G, the amplitude type in HBM; T, the working type in
// registers and shared memory; Mat, an op's matrix in registers; and how to
// convert and apply.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "complex_ops.cuh"
#include "df.cuh"
#include "fx.cuh"
#include "internal.h"

namespace dmv {

struct PolF64 {  // complex128, IEEE FP64 multiply-adds
  static constexpr bool kBlockScaled = false;
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
  static constexpr bool kBlockScaled = false;
  using G = float2;
  using T = float2;
  using Mat = M2<float>;
  static Mat mat(const Op& op) { return to_m2<float>(op.m); }
  // op.mh holds the entries rounded to nearest FP32, the same values as
  // to_m2<float>(op.m), without device FP64->FP32 conversions (those run on
  // the FP64 pipe).
  __device__ static Mat dmat(const Op& op) {
    Mat m;
    m.r00 = op.mh[0]; m.i00 = op.mh[1]; m.r01 = op.mh[2]; m.i01 = op.mh[3];
    m.r10 = op.mh[4]; m.i10 = op.mh[5]; m.r11 = op.mh[6]; m.i11 = op.mh[7];
    return m;
  }
  template <int CLS>
  __device__ static void apply(const Mat& m, T& a0, T& a1) { apply_pair<float, CLS>(m, a0, a1); }
  __device__ static T in(const G& g) { return g; }
  __device__ static G out(const T& t) { return t; }
};

struct PolDF {  // complex128 storage, FP32-pair arithmetic (df.cuh)
  static constexpr bool kBlockScaled = false;
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

// complex128 storage, int64 block fixed-point arithmetic on the integer pipe
// (fx.cuh). Conversions need the block's exponent, so tiles are staged by
// tile_load_fx / tile_store_fx and pairs by pair_in / pair_out.
struct PolFX {
  static constexpr bool kBlockScaled = true;
  using G = double2;
  using T = longlong2;
  using Mat = FXMat;
  static Mat mat(const Op& op) {
    Mat m;
    for (int i = 0; i < 8; ++i) {
      m.h[i] = op.fh[i];
      m.l[i] = op.fl[i];
    }
    return m;
  }
  __device__ static Mat dmat(const Op& op) {
    Mat m;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      m.h[i] = op.fh[i];
      m.l[i] = op.fl[i];
    }
    return m;
  }
  template <int CLS>
  __device__ static void apply(const Mat& m, T& a0, T& a1) { fx_apply_pair<CLS>(m, a0, a1); }
  // A pair as its own block: 4 components, 2-norm at most 2x the largest.
  __device__ static int pair_exponent(const G& g0, const G& g1) {
    return max(max(fx_exponent(g0.x), fx_exponent(g0.y)), max(fx_exponent(g1.x), fx_exponent(g1.y)));
  }
  __device__ static T in(const G& g, int e) { return make_longlong2(fx_from_double(g.x, e), fx_from_double(g.y, e)); }
  __device__ static G out(const T& t, int e) { return make_double2(fx_to_double(t.x, e), fx_to_double(t.y, e)); }
};

// Staging view of a policy whose working type is already the HBM contents:
// the tile is loaded and stored without conversion (FP32-pair passes between
// the first and last of a gate list keep that form in HBM).
template <typename P>
struct PolRaw {
  static constexpr bool kBlockScaled = false;
  using G = typename P::T;
  using T = typename P::T;
  __device__ static T in(const G& g) { return g; }
  __device__ static G out(const T& t) { return t; }
};

// (a0, a1) <- M (a0, a1) with the op class chosen at run time.
template <typename P>
__device__ __forceinline__ void apply_dyn(int cls, const typename P::Mat& m, typename P::T& a0, typename P::T& a1) {
  switch (cls) {
    case OP_SWAP: P::template apply<OP_SWAP>(m, a0, a1); break;
    case OP_DIAG: P::template apply<OP_DIAG>(m, a0, a1); break;
    case OP_ANTI: P::template apply<OP_ANTI>(m, a0, a1); break;
    case OP_REAL: P::template apply<OP_REAL>(m, a0, a1); break;
    case OP_RXLIKE: P::template apply<OP_RXLIKE>(m, a0, a1); break;
    default: P::template apply<OP_GENERAL>(m, a0, a1); break;
  }
}

// ---------------------------------------------------------------------------
// Tile staging. Both tile kernels run 512 threads, so local index l of a tile
// splits as l = tid + 512*u: the low 9 bits come from the thread, the rest
// from the slot u. With `low` <= 9 always-local low qubits, the HBM offset of
// element l is (tid's part) | (u's part), both fixed for the whole pass:
// tid's part is computed once per thread, u's parts once per CTA into shared
// memory. Each thread then issues up to 8 loads before it writes any of them
// to shared memory, so a CTA keeps 8 x 512 x 16 bytes in flight.
// ---------------------------------------------------------------------------
constexpr int kTileThreads = 512;
constexpr int kTileThreadBits = 9;
constexpr int kMaxSlots = 16;  // tiles of up to 2^13 amplitudes

// Offsets of a tile's elements relative to the tile base. `high` are the
// global positions of the nh high local qubits (ascending).
template <typename HighArray>
__device__ __forceinline__ int64_t tile_thread_offset(int low, int nh, const HighArray& high) {
  const uint32_t tid = threadIdx.x;
  int64_t off = (int64_t)(tid & ((1u << low) - 1u));
  const int from_tid = min(nh, kTileThreadBits - low);
  for (int i = 0; i < from_tid; ++i) off |= (int64_t)((tid >> (low + i)) & 1u) << high[i];
  return off;
}

template <typename HighArray>
__device__ __forceinline__ void tile_slot_offsets(int low, int nh, const HighArray& high, int slots, int64_t* s_slot) {
  const int from_tid = min(nh, kTileThreadBits - low);
  if ((int)threadIdx.x < slots) {
    const uint32_t u = threadIdx.x;
    int64_t off = 0;
    for (int i = from_tid; i < nh; ++i) off |= (int64_t)((u >> (i - from_tid)) & 1u) << high[i];
    s_slot[threadIdx.x] = off;
  }
}

// HBM -> shared memory (converted to the working type). `cg` selects L2-only loads.
template <typename P, bool CG>
__device__ __forceinline__ void tile_load(typename P::T* tile, const typename P::G* a, int64_t base, int T,
                                          int64_t t_off, const int64_t* s_slot) {
  using G = typename P::G;
  // Loads in flight per thread: 4 x 16 B or 8 x 8 B, i.e. 64 KB per SM at
  // two CTAs, above what HBM latency needs, without spilling registers.
  constexpr int B = sizeof(G) >= 16 ? 4 : 8;
  const int slots = (T + kTileThreads - 1) >> kTileThreadBits;
  for (int u0 = 0; u0 < slots; u0 += B) {
    G v[B];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int l = (int)threadIdx.x + ((u0 + j) << kTileThreadBits);
      if (u0 + j < slots && l < T) {
        const G* p = a + (base | t_off | s_slot[u0 + j]);
        if constexpr (CG) v[j] = __ldcg(p);
        else v[j] = *p;
      }
    }
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int l = (int)threadIdx.x + ((u0 + j) << kTileThreadBits);
      if (u0 + j < slots && l < T) tile[l] = P::in(v[j]);
    }
  }
}

template <typename P>
__device__ __forceinline__ void tile_store(const typename P::T* tile, typename P::G* a, int64_t base, int T,
                                           int64_t t_off, const int64_t* s_slot) {
  const int slots = (T + kTileThreads - 1) >> kTileThreadBits;
  for (int u = 0; u < slots; ++u) {
    const int l = (int)threadIdx.x + (u << kTileThreadBits);
    if (l < T) a[base | t_off | s_slot[u]] = P::out(tile[l]);
  }
}

// Block-scaled staging (PolFX): the raw FP64 bits go to shared memory while
// each thread tracks its largest exponent; a block-wide maximum (s_red: 16
// ints) fixes the tile's exponent; each thread then converts the elements it
// loaded, in place. Returns the tile exponent. The caller synchronises before
// the ops, as after tile_load. Tiles of up to 4096 amplitudes keep every
// fixed-point component below 2^60.5 (fx.cuh).
template <bool CG>
__device__ __forceinline__ int tile_load_fx(longlong2* tile, const double2* a, int64_t base, int T, int64_t t_off,
                                            const int64_t* s_slot, int* s_red) {
  const int slots = (T + kTileThreads - 1) >> kTileThreadBits;
  unsigned emax = 0;
  for (int u0 = 0; u0 < slots; u0 += 4) {
    double2 v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int l = (int)threadIdx.x + ((u0 + j) << kTileThreadBits);
      if (u0 + j < slots && l < T) {
        const double2* p = a + (base | t_off | s_slot[u0 + j]);
        if constexpr (CG) v[j] = __ldcg(p);
        else v[j] = *p;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int l = (int)threadIdx.x + ((u0 + j) << kTileThreadBits);
      if (u0 + j < slots && l < T) {
        tile[l] = make_longlong2(__double_as_longlong(v[j].x), __double_as_longlong(v[j].y));
        emax = max(emax, (unsigned)max(fx_exponent(v[j].x), fx_exponent(v[j].y)));
      }
    }
  }
  emax = __reduce_max_sync(0xffffffffu, emax);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = (int)emax;
  __syncthreads();
  int e = 0;
#pragma unroll
  for (int w = 0; w < kTileThreads / 32; ++w) e = max(e, s_red[w]);
  for (int u = 0; u < slots; ++u) {
    const int l = (int)threadIdx.x + (u << kTileThreadBits);
    if (l < T) {
      const longlong2 r = tile[l];
      tile[l] = make_longlong2(fx_from_double(__longlong_as_double(r.x), e),
                               fx_from_double(__longlong_as_double(r.y), e));
    }
  }
  return e;
}

__device__ __forceinline__ void tile_store_fx(const longlong2* tile, double2* a, int64_t base, int T, int64_t t_off,
                                              const int64_t* s_slot, int e) {
  const int slots = (T + kTileThreads - 1) >> kTileThreadBits;
  for (int u = 0; u < slots; ++u) {
    const int l = (int)threadIdx.x + (u << kTileThreadBits);
    if (l < T) {
      const longlong2 x = tile[l];
      a[base | t_off | s_slot[u]] = make_double2(fx_to_double(x.x, e), fx_to_double(x.y, e));
    }
  }
}

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

// OP_ROT (FP64 window passes): the real rotation [[c, -s], [s, c]] of every
// pair along op.target, on the real parts and on the imaginary parts, as
// f M: M = [[1, -w], [w, 1]] (op.m[1] == 0) or [[w, -1], [1, w]] (op.m[1] ==
// 1), w = op.m[0]; one multiply-add per output (2 per amplitude). The factor
// f is not applied here: the plan multiplies the product of its rotations'
// factors back into the state once. Two pairs per iteration, as in tile_op.
template <bool FORM_B>
__device__ __forceinline__ void rot_pair(double w, double2& a0, double2& a1) {
  const double x0 = a0.x, x1 = a1.x, y0 = a0.y, y1 = a1.y;
  if constexpr (!FORM_B) {
    a0 = make_double2(fma(-w, x1, x0), fma(-w, y1, y0));
    a1 = make_double2(fma(w, x0, x1), fma(w, y0, y1));
  } else {
    a0 = make_double2(fma(w, x0, -x1), fma(w, y0, -y1));
    a1 = make_double2(fma(w, x1, x0), fma(w, y1, y0));
  }
}

template <bool FORM_B>
__device__ __forceinline__ void tile_rot_form(double2* tile, int T, int t, double w) {
  const int half = T >> 1;
  const int bd = blockDim.x;
  for (int q = threadIdx.x; q < half; q += 2 * bd) {
    const int q2 = q + bd;
    const uint32_t l0 = insert_zero32((uint32_t)q, t), l1 = l0 | (1u << t);
    double2 a0 = tile[l0], a1 = tile[l1];
    if (q2 < half) {
      const uint32_t m0 = insert_zero32((uint32_t)q2, t), m1 = m0 | (1u << t);
      double2 b0 = tile[m0], b1 = tile[m1];
      rot_pair<FORM_B>(w, a0, a1);
      rot_pair<FORM_B>(w, b0, b1);
      tile[m0] = b0;
      tile[m1] = b1;
    } else {
      rot_pair<FORM_B>(w, a0, a1);
    }
    tile[l0] = a0;
    tile[l1] = a1;
  }
}

__device__ __forceinline__ void tile_rot(double2* tile, int T, const Op& op) {
  if (op.m[1] == 0.0) tile_rot_form<false>(tile, T, op.target, op.m[0]);
  else tile_rot_form<true>(tile, T, op.target, op.m[0]);
}

// OP_PHASE (FP64 window passes): amplitude l times the phase of table entry
// op.fh[0] + (gsel << k) + l, in the 16-byte form of phase_tables_f64: three
// shears by (t, s), then for the factor i^q a swap and sign flips on the
// integer pipe, q read from bit 62 of t (q & 1: swap) and of s (q >> 1).
// gsel holds the tile's bits at the op.fh[1] global qubits op.fh[2..].
__device__ __forceinline__ void tile_phase(double2* tile, int T, const Op& op, const double2* tab, int64_t base) {
  const int k = 31 - __clz(T);
  int gsel = 0;
  for (int j = 0; j < op.fh[1]; ++j) gsel |= (int)((base >> op.fh[2 + j]) & 1) << j;
  const double2* e = tab + op.fh[0] + ((int64_t)gsel << k);
#pragma unroll 4
  for (int l = threadIdx.x; l < T; l += blockDim.x) {
    const double2 ts = __ldg(e + l);
    const int th = __double2hiint(ts.x), sh = __double2hiint(ts.y);
    const int b0 = (th >> 30) & 1, b1 = (sh >> 30) & 1;
    const double t = __hiloint2double(th & ~(1 << 30), __double2loint(ts.x));
    const double s = __hiloint2double(sh & ~(1 << 30), __double2loint(ts.y));
    const double2 v = tile[l];
    const double x1 = fma(t, v.y, v.x);
    const double y1 = fma(s, x1, v.y);
    const double x2 = fma(t, y1, x1);
    const double ox = b0 ? y1 : x2;
    const double oy = b0 ? x2 : y1;
    tile[l] = make_double2(__hiloint2double(__double2hiint(ox) ^ ((b0 ^ b1) << 31), __double2loint(ox)),
                           __hiloint2double(__double2hiint(oy) ^ (b1 << 31), __double2loint(oy)));
  }
}

// First table entry of an OP_PHASE op for the tile at `base` (2^k amplitudes).
__device__ __forceinline__ int64_t phase_slice(const Op& op, int k, int64_t base) {
  int gsel = 0;
  for (int j = 0; j < op.fh[1]; ++j) gsel |= (int)((base >> op.fh[2 + j]) & 1) << j;
  return (int64_t)op.fh[0] + ((int64_t)gsel << k);
}

// OP_PHASE in FP32-pair arithmetic: amplitude l times the table's pair
// (re_h, re_l, im_h, im_l), as the diagonal case of df_apply_pair.
__device__ __forceinline__ void tile_phase_df(float4* tile, int T, const Op& op, const float4* tab, int64_t base) {
  const float4* e = tab + phase_slice(op, 31 - __clz(T), base);
  for (int l = threadIdx.x; l < T; l += blockDim.x) {
    const float4 w = __ldg(e + l);
    const float4 a = tile[l];
    DFAcc re, im;
    df_first(re, w.x, w.y, a.x, a.y);
    df_add(re, -w.z, -w.w, a.z, a.w);
    df_first(im, w.x, w.y, a.z, a.w);
    df_add(im, w.z, w.w, a.x, a.y);
    float4 b;
    df_finish(re, b.x, b.y);
    df_finish(im, b.z, b.w);
    tile[l] = b;
  }
}

// OP_PHASE in int64 block fixed point: amplitude l times the table's Q.54
// phase (re_h, re_l, im_h, im_l limbs), one rounding per component.
__device__ __forceinline__ void tile_phase_fx(longlong2* tile, int T, const Op& op, const int4* tab, int64_t base) {
  const int4* e = tab + phase_slice(op, 31 - __clz(T), base);
  for (int l = threadIdx.x; l < T; l += blockDim.x) {
    const int4 w = __ldg(e + l);
    const longlong2 a = tile[l];
    int rh, rl, ih, il;
    fx_limbs(a.x, rh, rl);
    fx_limbs(a.y, ih, il);
    FXAcc p, n;
    fx_zero(p);
    fx_zero(n);
    fx_mac(p, w.x, w.y, rh, rl);
    fx_mac(n, w.z, w.w, ih, il);
    const long long x = fx_result(p, n);
    fx_zero(p);
    fx_mac(p, w.x, w.y, ih, il);
    fx_mac(p, w.z, w.w, rh, rl);
    tile[l] = make_longlong2(x, fx_result(p));
  }
}

// Every op of a pass on one tile; `base` holds the tile's global index bits
// (controls outside the tile are read from it). Ends with a barrier after
// each applied op. `tab` holds the phase tables of OP_PHASE ops in the
// policy's form: 16-byte packed entries (FP64, phase_tables_f64), float4 FP32 pairs (PolDF) or int4 Q.54
// limbs (PolFX).
template <typename P>
__device__ __forceinline__ void tile_apply_ops(typename P::T* tile, int T, const Op* ops, int num_ops, int64_t base,
                                               const void* tab = nullptr) {
  for (int o = 0; o < num_ops; ++o) {
    const Op& op = ops[o];
    if (op.ctrl_kind == CTRL_GLOBAL && !((base >> op.ctrl) & 1)) continue;  // uniform per tile
    if constexpr (std::is_same<P, PolF64>::value) {
      if (op.cls == OP_ROT) {
        tile_rot(tile, T, op);
        __syncthreads();
        continue;
      }
      if (op.cls == OP_PHASE) {
        tile_phase(tile, T, op, static_cast<const double2*>(tab), base);
        __syncthreads();
        continue;
      }
    } else if constexpr (std::is_same<P, PolDF>::value) {
      if (op.cls == OP_PHASE) {
        tile_phase_df(tile, T, op, static_cast<const float4*>(tab), base);
        __syncthreads();
        continue;
      }
    } else if constexpr (std::is_same<P, PolFX>::value) {
      if (op.cls == OP_PHASE) {
        tile_phase_fx(tile, T, op, static_cast<const int4*>(tab), base);
        __syncthreads();
        continue;
      }
    }
    switch (op.cls) {
      case OP_SWAP: tile_op<P, OP_SWAP>(tile, T, op); break;
      case OP_DIAG: tile_op<P, OP_DIAG>(tile, T, op); break;
      case OP_ANTI: tile_op<P, OP_ANTI>(tile, T, op); break;
      case OP_REAL: tile_op<P, OP_REAL>(tile, T, op); break;
      case OP_RXLIKE: tile_op<P, OP_RXLIKE>(tile, T, op); break;
      default: tile_op<P, OP_GENERAL>(tile, T, op); break;
    }
    __syncthreads();
  }
}

}  // namespace dmv
