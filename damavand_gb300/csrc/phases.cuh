// Register phases: the in-tile op loop of the TMA window kernel.
//
// The tile (2^k amplitudes, 1024-byte aligned, in the TMA 128-byte swizzle)
// is handled by 2^(k-rb) threads, each holding NR = 2^rb amplitudes in registers:
// the ones whose tile indices differ only in the phase's rb register bits.
// An op whose target is a register bit is a set of NR/2 register pairs per
// thread; its control is either another register bit (a compile-time-free,
// warp-uniform pair mask) or a bit the thread's amplitudes share (a
// per-thread predicate). Between phases the registers go back to shared
// memory and are re-read with the next phase's register bits.
#pragma once

#include <type_traits>

#include "policies.cuh"
#include "tma.cuh"

namespace dmv {

// Shared-memory slot of tile element l under the TMA 128-byte swizzle (each
// 16-byte chunk of a 128-byte row is XORed with the row index mod 8). ES is
// the element size: 16 (complex128) or 8 (complex64). Linear over GF(2), so
// the slot of l | m for disjoint bit sets is swz(l) ^ swz(m).
template <int ES>
__device__ __forceinline__ uint32_t swz(uint32_t l) {
  static_assert(ES == 16 || ES == 8, "element size");
  if constexpr (ES == 16) return l ^ ((l >> 3) & 7u);
  else return l ^ (((l >> 4) & 7u) << 1);
}

template <typename P>
__device__ __forceinline__ typename P::T cvt_in(const typename P::G& g, int e) {
  if constexpr (P::kBlockScaled) return P::in(g, e);
  else {
    (void)e;
    return P::in(g);
  }
}

template <typename P>
__device__ __forceinline__ typename P::G cvt_out(const typename P::T& t, int e) {
  if constexpr (P::kBlockScaled) return P::out(t, e);
  else {
    (void)e;
    return P::out(t);
  }
}

// Slot of register j: pbase ^ (XOR of pr[b] over the set bits b of j).
template <int RB>
__device__ __forceinline__ uint32_t reg_slot(uint32_t pbase, const uint32_t (&pr)[RB], int j) {
  uint32_t a = pbase;
#pragma unroll
  for (int b = 0; b < RB; ++b)
    if ((j >> b) & 1) a ^= pr[b];
  return a;
}

// Shared memory -> registers; FROM_G converts from the HBM type (first phase).
template <typename P, int RB, bool FROM_G>
__device__ __forceinline__ void regs_load(typename P::T (&r)[1 << RB], const void* tile, uint32_t pbase,
                                          const uint32_t (&pr)[RB], int e) {
#pragma unroll
  for (int j = 0; j < (1 << RB); ++j) {
    const uint32_t a = reg_slot<RB>(pbase, pr, j);
    if constexpr (FROM_G) r[j] = cvt_in<P>(static_cast<const typename P::G*>(tile)[a], e);
    else r[j] = static_cast<const typename P::T*>(tile)[a];
  }
}

// Registers -> shared memory; TO_G converts to the HBM type (last phase).
template <typename P, int RB, bool TO_G>
__device__ __forceinline__ void regs_store(const typename P::T (&r)[1 << RB], void* tile, uint32_t pbase,
                                           const uint32_t (&pr)[RB], int e) {
#pragma unroll
  for (int j = 0; j < (1 << RB); ++j) {
    const uint32_t a = reg_slot<RB>(pbase, pr, j);
    if constexpr (TO_G) static_cast<typename P::G*>(tile)[a] = cvt_out<P>(r[j], e);
    else static_cast<typename P::T*>(tile)[a] = r[j];
  }
}

// One op on the register pairs (j, j | 2^TP); cmask selects the pairs whose
// control register bit is set (0: all pairs).
template <typename P, int CLS, int RB, int TP>
__device__ __forceinline__ void regs_apply(typename P::T (&r)[1 << RB], const typename P::Mat& m, uint32_t cmask) {
#pragma unroll
  for (int j = 0; j < (1 << RB); ++j) {
    if (j & (1 << TP)) continue;
    if (((uint32_t)j & cmask) != cmask) continue;
    P::template apply<CLS>(m, r[j], r[j | (1 << TP)]);
  }
}

template <typename P, int CLS, int RB>
__device__ __forceinline__ void regs_apply_tp(typename P::T (&r)[1 << RB], const typename P::Mat& m, int tp,
                                              uint32_t cmask) {
  switch (tp) {
    case 0: regs_apply<P, CLS, RB, 0>(r, m, cmask); break;
    case 1: regs_apply<P, CLS, RB, 1>(r, m, cmask); break;
    case 2: regs_apply<P, CLS, RB, 2>(r, m, cmask); break;
    default:
      if constexpr (RB > 3) regs_apply<P, CLS, RB, 3>(r, m, cmask);
      break;
  }
}

// The FP32 matrix of a table op (complex64 arithmetic).
__device__ __forceinline__ M2<float> phase_mat(const PhaseOp& op) {
  M2<float> m;
  m.r00 = op.m[0]; m.i00 = op.m[1]; m.r01 = op.m[2]; m.i01 = op.m[3];
  m.r10 = op.m[4]; m.i10 = op.m[5]; m.r11 = op.m[6]; m.i11 = op.m[7];
  return m;
}

template <typename P, int RB>
__device__ __forceinline__ void regs_apply_op(typename P::T (&r)[1 << RB], const PhaseOp& op, int tp, uint32_t cmask) {
  static_assert(std::is_same<typename P::Mat, M2<float>>::value, "table ops carry FP32 matrices");
  const typename P::Mat m = phase_mat(op);
  switch (op.cls) {
    case OP_SWAP: regs_apply_tp<P, OP_SWAP, RB>(r, m, tp, cmask); break;
    case OP_DIAG: regs_apply_tp<P, OP_DIAG, RB>(r, m, tp, cmask); break;
    case OP_ANTI: regs_apply_tp<P, OP_ANTI, RB>(r, m, tp, cmask); break;
    case OP_REAL: regs_apply_tp<P, OP_REAL, RB>(r, m, tp, cmask); break;
    case OP_RXLIKE: regs_apply_tp<P, OP_RXLIKE, RB>(r, m, tp, cmask); break;
    default: regs_apply_tp<P, OP_GENERAL, RB>(r, m, tp, cmask); break;
  }
}

// Every op of a pass (the shared-memory op table `ops`) on a tile staged in
// HBM format (P::G, swizzled); leaves the tile in HBM format. `base` holds
// the tile's global index bits (controls outside the tile), `e` the block
// exponent (block-scaled policies). The NSYNC = 2^(k-RB) compute threads
// call it; it synchronises them (named barrier 1) at every phase start.
template <typename P, int RB, int NSYNC>
__device__ __forceinline__ void run_phases(void* tile, int k, const PhaseOp* ops, int num_ops, int64_t base,
                                           int e) {
  using V = typename P::T;
  constexpr int ES = (int)sizeof(typename P::G);
  static_assert(sizeof(V) == sizeof(typename P::G), "working and HBM types share the tile");
  (void)k;  // the thread count fixes k - RB
  V r[1 << RB];
  uint32_t pr[RB];
#pragma unroll
  for (int b = 0; b < RB; ++b) pr[b] = 0;
  uint32_t pbase = 0, lbase = 0;
  bool loaded = false;
  for (int o = 0; o < num_ops; ++o) {
    const PhaseOp& op = ops[o];
    const uint32_t ph = op.phase;
    if (ph & kPhaseStart) {
      if (loaded) regs_store<P, RB, false>(r, tile, pbase, pr, e);
      named_sync(1, NSYNC);
      uint32_t q[RB];
#pragma unroll
      for (int b = 0; b < RB; ++b) {
        q[b] = (ph >> (4 * b)) & 15u;
        pr[b] = swz<ES>(1u << q[b]);
      }
      // The thread's bits go to the non-register positions: insert a zero
      // at each register bit, lowest first (sorting network on RB values).
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j + 1 < RB - i; ++j) {
          const uint32_t lo = min(q[j], q[j + 1]), hi = max(q[j], q[j + 1]);
          q[j] = lo;
          q[j + 1] = hi;
        }
      lbase = threadIdx.x;
#pragma unroll
      for (int b = 0; b < RB; ++b) lbase = insert_zero32(lbase, (int)q[b]);
      pbase = swz<ES>(lbase);
      if (loaded) regs_load<P, RB, false>(r, tile, pbase, pr, e);
      else regs_load<P, RB, true>(r, tile, pbase, pr, e);
      loaded = true;
    }
    if (op.ctrl_kind == CTRL_GLOBAL && !((base >> op.ctrl) & 1)) continue;  // uniform per tile
    uint32_t cmask = 0;
    if (op.ctrl_kind == CTRL_LOCAL) {
      const uint32_t ci = (ph >> kPhaseCtrlShift) & 7u;
      if (ci) cmask = 1u << (ci - 1);
      else if (!((lbase >> op.ctrl) & 1u)) continue;  // control shared by this thread's amplitudes
    }
    regs_apply_op<P, RB>(r, op, (int)((ph >> kPhaseTargetShift) & 3u), cmask);
  }
  if (loaded) regs_store<P, RB, true>(r, tile, pbase, pr, e);
}

}  // namespace dmv
