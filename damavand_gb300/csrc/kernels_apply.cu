// Gate-application kernels.
//
//  * k_apply_single: one 2x2 op over the whole statevector. Each thread owns
//    whole amplitude pairs (i0, i0 + 2^t), so no amplitude is read after
//    another thread wrote it (the reference kernel, damavand-gpu/kernels.cu:
//    120-172, reads every amplitude twice and races across blocks). A
//    controlled op enumerates only the control=1 quarter-space pairs, so it
//    moves half the bytes of an uncontrolled one. 64-bit indices throughout.
//  * k_apply_window: a fused pass. Each CTA stages a tile of 2^k amplitudes
//    -- the pass's `low` lowest qubits (contiguous 2^low-amplitude chunks in
//    HBM) times its high local qubits -- in shared memory, applies every op
//    of the pass to it, and writes it back: one read and one write of the
//    statevector for the whole window of gates. A control qubit outside the
//    tile is constant over the tile and is tested once per tile.
//  * k_window_tma: the same pass for full-size tiles (2^12 complex128 or
//    2^13 complex64 amplitudes with at least three high qubits). One
//    persistent CTA per SM; tiles move HBM <-> shared memory by TMA
//    (cp.async.bulk.tensor over a per-pass 5-D tensor map), three buffers
//    deep: tile i+1 loads and tile i-1 drains while tile i computes. The ops
//    run in register phases (phases.cuh), so the tile crosses shared memory
//    once per phase instead of once per op.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "internal.h"
#include "phases.cuh"
#include "policies.cuh"
#include "tc.cuh"
#include "tma.cuh"

namespace dmv {

namespace {

constexpr int kSingleThreads = 256;
constexpr int kWindowThreads = 512;

int num_sms() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

template <typename P, int CLS, bool CTRL>
__global__ void __launch_bounds__(kSingleThreads)
k_apply_single(typename P::G* __restrict__ a, int64_t num_pairs, int target, int control, const typename P::Mat m) {
  using T = typename P::T;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int lo = CTRL ? min(target, control) : target;
  const int hi = CTRL ? max(target, control) : target;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < num_pairs; j += stride) {
    int64_t i0;
    if constexpr (CTRL) {
      i0 = insert_zero(insert_zero(j, lo), hi) | (int64_t(1) << control);
    } else {
      i0 = insert_zero(j, target);
    }
    const int64_t i1 = i0 | (int64_t(1) << target);
    if constexpr (CLS == OP_SWAP) {
      const typename P::G g0 = a[i0];
      a[i0] = a[i1];
      a[i1] = g0;
    } else if constexpr (P::kBlockScaled) {
      const typename P::G g0 = a[i0], g1 = a[i1];
      const int e = P::pair_exponent(g0, g1);
      T a0 = P::in(g0, e);
      T a1 = P::in(g1, e);
      P::template apply<CLS>(m, a0, a1);
      a[i0] = P::out(a0, e);
      a[i1] = P::out(a1, e);
    } else {
      T a0 = P::in(a[i0]);
      T a1 = P::in(a[i1]);
      P::template apply<CLS>(m, a0, a1);
      a[i0] = P::out(a0);
      a[i1] = P::out(a1);
    }
  }
}

template <typename P, int CLS, bool CTRL>
void launch_single_t(typename P::G* a, int32_t n, const Op& op, cudaStream_t stream) {
  const int64_t pairs = (int64_t(1) << n) >> (CTRL ? 2 : 1);
  const int64_t want = (pairs + kSingleThreads - 1) / kSingleThreads;
  const int64_t cap = (int64_t)num_sms() * 16;
  const int grid = (int)std::max<int64_t>(1, std::min(want, cap));
  k_apply_single<P, CLS, CTRL><<<grid, kSingleThreads, 0, stream>>>(a, pairs, op.target, op.ctrl, P::mat(op));
}

template <typename P, int CLS>
void launch_single_c(typename P::G* a, int32_t n, const Op& op, cudaStream_t stream) {
  if (op.ctrl_kind != CTRL_NONE && op.ctrl >= 0)
    launch_single_t<P, CLS, true>(a, n, op, stream);
  else
    launch_single_t<P, CLS, false>(a, n, op, stream);
}

template <typename P>
void launch_single(void* amps, int32_t n, const Op& op, cudaStream_t stream) {
  typename P::G* a = static_cast<typename P::G*>(amps);
  switch (op.cls) {
    case OP_SWAP: launch_single_c<P, OP_SWAP>(a, n, op, stream); break;
    case OP_DIAG: launch_single_c<P, OP_DIAG>(a, n, op, stream); break;
    case OP_ANTI: launch_single_c<P, OP_ANTI>(a, n, op, stream); break;
    case OP_REAL: launch_single_c<P, OP_REAL>(a, n, op, stream); break;
    case OP_RXLIKE: launch_single_c<P, OP_RXLIKE>(a, n, op, stream); break;
    default: launch_single_c<P, OP_GENERAL>(a, n, op, stream); break;
  }
}

struct WindowParams {
  int32_t k;         // log2 tile size
  int32_t low;       // low local qubits
  int32_t nh;        // high local qubits
  int32_t num_ops;
  int32_t high[16];  // ascending global positions of the high local qubits
  int64_t num_tiles;
  const Op* ops;
  const void* tab;   // phase tables of the pass's OP_PHASE ops, in the policy's form
};

static_assert(kWindowThreads == kTileThreads, "tile staging assumes 512 threads");

// FMT (FP32-pair arithmetic only): bit 0, the pass reads the FP32-pair form
// (float4 in place of each double2, the same 16 bytes); bit 1, it writes that
// form. Inside one gate list of window passes only the first pass reads IEEE
// complex128 and only the last one writes it, so the passes between skip the
// integer-heavy conversions.
template <typename P, int FMT = 0>
__global__ void __launch_bounds__(kWindowThreads, 2)
k_apply_window(typename P::G* __restrict__ a, const WindowParams p) {
  using V = typename P::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int64_t s_slot[kMaxSlots];
  V* tile = reinterpret_cast<V*>(smem_raw);
  const int T = 1 << p.k;
  const int64_t t_off = tile_thread_offset(p.low, p.nh, p.high);
  tile_slot_offsets(p.low, p.nh, p.high, (T + kTileThreads - 1) >> kTileThreadBits, s_slot);
  __syncthreads();
  __shared__ int s_red[kTileThreads / 32];
  for (int64_t tix = blockIdx.x; tix < p.num_tiles; tix += gridDim.x) {
    int64_t base = tix << p.low;
    for (int i = 0; i < p.nh; ++i) base = insert_zero(base, p.high[i]);
    if constexpr (P::kBlockScaled) {
      const int e = tile_load_fx<false>(tile, a, base, T, t_off, s_slot, s_red);
      __syncthreads();
      tile_apply_ops<P>(tile, T, p.ops, p.num_ops, base, p.tab);
      tile_store_fx(tile, a, base, T, t_off, s_slot, e);
    } else {
      (void)s_red;
      if constexpr (FMT & 1) tile_load<PolRaw<P>, false>(tile, reinterpret_cast<const V*>(a), base, T, t_off, s_slot);
      else tile_load<P, false>(tile, a, base, T, t_off, s_slot);
      __syncthreads();
      tile_apply_ops<P>(tile, T, p.ops, p.num_ops, base, p.tab);
      if constexpr (FMT & 2) tile_store<PolRaw<P>>(tile, reinterpret_cast<V*>(a), base, T, t_off, s_slot);
      else tile_store<P>(tile, a, base, T, t_off, s_slot);
    }
    __syncthreads();
  }
}

template <typename P, int FMT>
int launch_window_fmt(void* amps, int32_t n, const Pass& ps, const Op* ops_dev, cudaStream_t stream,
                      const void* tab) {
  using V = typename P::T;
  WindowParams p;
  p.k = ps.low_bits + ps.num_high;
  p.low = ps.low_bits;
  p.nh = ps.num_high;
  p.num_ops = (int32_t)ps.op_count;
  for (int i = 0; i < 16; ++i) p.high[i] = i < ps.num_high ? ps.high[i] : 0;
  p.num_tiles = int64_t(1) << (n - p.k);
  p.ops = ops_dev + ps.op_begin;
  p.tab = tab;
  const size_t smem = (size_t(1) << p.k) * sizeof(V);
  static size_t configured = 0;
  if (smem > configured) {
    DMV_CUDA_TRY(cudaFuncSetAttribute(k_apply_window<P, FMT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
    configured = smem;
  }
  int per_sm = 0;
  DMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_window<P, FMT>, kWindowThreads, smem));
  if (per_sm < 1) return set_error(DMV_ERR_CUDA, "window kernel cannot fit %zu bytes of shared memory", smem);
  const int64_t grid = std::min<int64_t>(p.num_tiles, (int64_t)per_sm * num_sms());
  k_apply_window<P, FMT><<<(int)grid, kWindowThreads, smem, stream>>>(static_cast<typename P::G*>(amps), p);
  return DMV_OK;
}

// fmt: the FMT bits of k_apply_window (FP32-pair arithmetic only).
template <typename P>
int launch_window(void* amps, int32_t n, const Pass& ps, const Op* ops_dev, cudaStream_t stream,
                  const void* tab = nullptr, int fmt = 0) {
  if constexpr (std::is_same<P, PolDF>::value) {
    switch (fmt) {
      case 1: return launch_window_fmt<P, 1>(amps, n, ps, ops_dev, stream, tab);
      case 2: return launch_window_fmt<P, 2>(amps, n, ps, ops_dev, stream, tab);
      case 3: return launch_window_fmt<P, 3>(amps, n, ps, ops_dev, stream, tab);
      default: break;
    }
  }
  return launch_window_fmt<P, 0>(amps, n, ps, ops_dev, stream, tab);
}

// ---------------------------------------------------------------------------
// TMA window pass
// ---------------------------------------------------------------------------
constexpr uint32_t kTmaWaitLimit = 1u << 22;  // polls before a load wait gives up
constexpr uint32_t kTmaDrainLimit = 1u << 22;

// Rows of the tensor map's innermost box dimension: 128 bytes, i.e. 2^3
// complex128 or 2^4 complex64 amplitudes.
template <int ES>
constexpr int row_bits() { return ES == 16 ? 3 : 4; }

// Two TMA kernels on 2^12-amplitude tiles:
//  * k_window_phases (complex64, FP32 arithmetic), warp-specialised: eight
//    compute warps hold 16 amplitudes per thread and run the ops in register
//    phases, synchronising among themselves on named barrier 1; one producer
//    warp issues every TMA load and store. Two tile buffers: the producer
//    refills a buffer with tile i+2 once the TMA store of tile i has read it,
//    while the compute warps work on tile i+1. Tiles are in the TMA 128-byte
//    swizzle so the phases' register gathers avoid bank conflicts; the pass's
//    ops sit in a shared-memory table.
//  * k_window_tma (complex128, FP64 arithmetic): two CTAs of 512 threads per
//    SM, one linear (unswizzled) tile buffer each; TMA loads the tile, the
//    ops run in the shared-memory op loop, the threads write the tile back
//    with their own stores, so the buffer is free for the next load as soon
//    as they are issued, and one CTA's copies overlap the other's
//    arithmetic.
constexpr int kPhaseRegBits = 4;
constexpr int kPhaseComputeThreads = 1 << (kTileThreadBits + 3 - kPhaseRegBits);  // 256
constexpr int kPhaseThreads = kPhaseComputeThreads + 32;                          // + producer warp
constexpr int kPhaseBuffers = 2;

struct TmaPassParams {
  int32_t k;         // log2 tile size
  int32_t low;       // low local qubits
  int32_t nh;        // high local qubits (>= 3)
  int32_t num_ops;
  int32_t high[16];  // ascending global positions of the high local qubits
  int32_t boxes;     // TMA boxes per tile: 2^(nh - 3)
  uint32_t wait_limit;
  int64_t num_tiles;
  const Op* ops;
  const PhaseOp* phase_ops;  // k_window_phases' op table (num_ops <= kMaxPhaseOps)
  const void* phase_tab;  // k_window_tma: tables of the pass's OP_PHASE ops (the policy's form)
  void* amps;        // the statevector (k_window_tma's thread stores)
  int* status;       // set to 1 when a wait gave up
};

__device__ int g_tma_status;

// Tile geometry shared by both TMA kernels: the tile's base index and the
// TMA coordinates of its boxes (high positions in shared memory).
template <int ES>
struct TileGeom {
  int low, nh;
  const int* high;
  __device__ int64_t base(int64_t tix) const {
    int64_t b = tix << low;
    for (int i = 0; i < nh; ++i) b = insert_zero(b, high[i]);
    return b;
  }
  // Box c of a tile: its origin has the tile's bits plus c's bits on high
  // qubits 3.. ; coordinates follow the tensor map's dimension cuts.
  __device__ void box(int64_t base, int c, int& c1, int& c2, int& c3, int& c4) const {
    constexpr int RBITS = row_bits<ES>();
    int64_t org = base;
    for (int i = 3; i < nh; ++i) org |= (int64_t)((c >> (i - 3)) & 1) << high[i];
    const int h0 = high[0], h1 = high[1], h2 = high[2];
    c1 = (int)((org >> RBITS) & ((int64_t(1) << (h0 - RBITS)) - 1));
    c2 = (int)((org >> h0) & ((int64_t(1) << (h1 - h0)) - 1));
    c3 = (int)((org >> h1) & ((int64_t(1) << (h2 - h1)) - 1));
    c4 = (int)(org >> h2);
  }
  // Lane `lane` of a warp issues boxes lane, lane+32, ...; lane 0 first
  // arms the barrier with the tile's bytes.
  __device__ void load(const CUtensorMap* map, uint64_t* bar, unsigned char* dst, int64_t tix, int boxes,
                       uint32_t tile_bytes, int lane) const {
    const int64_t b = base(tix);
    const uint32_t box_bytes = tile_bytes / (uint32_t)boxes;
    if (lane == 0) mbar_arrive_expect_tx(bar, tile_bytes);
    __syncwarp();
    for (int c = lane; c < boxes; c += 32) {
      int c1, c2, c3, c4;
      box(b, c, c1, c2, c3, c4);
      tma_load_5d(dst + (size_t)c * box_bytes, map, bar, 0, c1, c2, c3, c4);
    }
  }
  __device__ void store(const CUtensorMap* map, const unsigned char* src, int64_t tix, int boxes, uint32_t tile_bytes,
                        int lane) const {
    const int64_t b = base(tix);
    const uint32_t box_bytes = tile_bytes / (uint32_t)boxes;
    for (int c = lane; c < boxes; c += 32) {
      int c1, c2, c3, c4;
      box(b, c, c1, c2, c3, c4);
      tma_store_5d(map, src + (size_t)c * box_bytes, 0, c1, c2, c3, c4);
    }
    tma_commit_group();
  }
};

template <typename P>
__global__ void __launch_bounds__(kPhaseThreads, 3)
k_window_phases(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TmaPassParams p) {
  using G = typename P::G;
  constexpr int ES = (int)sizeof(G);
  constexpr int NB = kPhaseBuffers;
  constexpr int NC = kPhaseComputeThreads;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_full[NB];  // tile landed (TMA transaction count)
  __shared__ __align__(8) uint64_t s_done[NB];  // compute threads finished the tile
  __shared__ int s_high[16];
  unsigned char* tiles =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int k = p.k, boxes = p.boxes, num_ops = p.num_ops;
  const int64_t num_tiles = p.num_tiles;
  const uint32_t tile_bytes = (uint32_t)ES << k;
  const uint32_t wait_limit = p.wait_limit;
  PhaseOp* s_ops = reinterpret_cast<PhaseOp*>(tiles + (size_t)NB * tile_bytes);
  if (threadIdx.x < 16) s_high[threadIdx.x] = p.high[threadIdx.x];
  {
    const int4* src = reinterpret_cast<const int4*>(p.phase_ops);
    int4* dst = reinterpret_cast<int4*>(s_ops);
    const int words = num_ops * (int)(sizeof(PhaseOp) / sizeof(int4));
    for (int i = threadIdx.x; i < words; i += kPhaseThreads) dst[i] = src[i];
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < NB; ++b) {
      mbar_init(&s_full[b], 1);
      mbar_init(&s_done[b], NC);
    }
    fence_mbar_init();
    tma_prefetch_map(&tmap);
  }
  __syncthreads();
  const TileGeom<ES> geom{p.low, p.nh, s_high};
  const int64_t stride = gridDim.x;

  if (threadIdx.x >= NC) {
    // Producer warp.
    const int lane = (int)(threadIdx.x & 31);
    int64_t issued = 0;  // tiles whose loads were issued
    for (int b = 0; b < NB; ++b) {
      const int64_t tix = blockIdx.x + (int64_t)b * stride;
      if (tix >= num_tiles) break;
      geom.load(&tmap, &s_full[b], tiles + (size_t)b * tile_bytes, tix, boxes, tile_bytes, lane);
      ++issued;
    }
    for (int64_t it = 0;; ++it) {
      const int64_t tix = blockIdx.x + it * stride;
      if (tix >= num_tiles) break;
      const int buf = (int)(it % NB);
      const uint32_t parity = (uint32_t)((it / NB) & 1);
      if (!mbar_wait(&s_done[buf], parity, wait_limit)) {
        if (lane == 0) atomicExch(p.status, 1);
        // Drain this CTA's loads before leaving: tiles it .. issued-1.
        for (int64_t j = it; j < issued; ++j)
          mbar_wait(&s_full[j % NB], (uint32_t)((j / NB) & 1), kTmaDrainLimit);
        break;
      }
      unsigned char* tile = tiles + (size_t)buf * tile_bytes;
      geom.store(&tmap, tile, tix, boxes, tile_bytes, lane);
      const int64_t nxt = tix + NB * stride;
      if (nxt < num_tiles) {
        tma_wait_group_read<0>();  // the store has read the buffer
        geom.load(&tmap, &s_full[buf], tile, nxt, boxes, tile_bytes, lane);
        ++issued;
      }
    }
    tma_wait_group_all();
    return;
  }

  // Compute warps.
  for (int64_t it = 0;; ++it) {
    const int64_t tix = blockIdx.x + it * stride;
    if (tix >= num_tiles) break;
    const int buf = (int)(it % NB);
    const bool ok = mbar_wait(&s_full[buf], (uint32_t)((it / NB) & 1), wait_limit);
    if (named_sync_or(1, NC, !ok)) {
      if (threadIdx.x == 0) atomicExch(p.status, 1);
      return;
    }
    unsigned char* tile = tiles + (size_t)buf * tile_bytes;
    run_phases<P, kPhaseRegBits, NC>(tile, k, s_ops, num_ops, geom.base(tix), 0);
    fence_proxy_async_smem();
    mbar_arrive(&s_done[buf]);
  }
}

template <typename P>
__global__ void __launch_bounds__(kWindowThreads, 2)
k_window_tma(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TmaPassParams p) {
  using G = typename P::G;
  using V = typename P::T;
  constexpr int ES = (int)sizeof(G);
  constexpr int NT = kWindowThreads;
  static_assert(sizeof(V) == sizeof(G), "the tile is converted in place");
  static_assert(NT == kTileThreads, "the op loop's stores assume 512 threads");
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ int s_red[NT / 32];
  __shared__ int s_high[16];
  __shared__ int64_t s_slot[kMaxSlots];
  unsigned char* tile =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int k = p.k, low = p.low, nh = p.nh, boxes = p.boxes;
  const int64_t num_tiles = p.num_tiles;
  const int T = 1 << k;
  const uint32_t tile_bytes = (uint32_t)ES << k;
  if (threadIdx.x < 16) s_high[threadIdx.x] = p.high[threadIdx.x];
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    fence_mbar_init();
    tma_prefetch_map(&tmap);
  }
  const int64_t t_off = tile_thread_offset(low, nh, p.high);
  tile_slot_offsets(low, nh, p.high, (T + kTileThreads - 1) >> kTileThreadBits, s_slot);
  __syncthreads();
  const TileGeom<ES> geom{low, nh, s_high};
  const int lane = (int)(threadIdx.x & 31);
  const bool mover = threadIdx.x < 32;  // warp 0 issues the loads, lane c box c

  const uint32_t wait_limit = p.wait_limit;
  const Op* ops = p.ops;
  const int num_ops = p.num_ops;
  G* amps = static_cast<G*>(p.amps);
  int64_t tix = blockIdx.x;
  if (mover && tix < num_tiles) geom.load(&tmap, &s_bar, tile, tix, boxes, tile_bytes, lane);
  for (int64_t it = 0; tix < num_tiles; ++it, tix += gridDim.x) {
    const int64_t next = tix + gridDim.x;
    const uint32_t parity = (uint32_t)(it & 1);
    const bool ok = mbar_wait(&s_bar, parity, wait_limit);
    if (__syncthreads_or(!ok)) {
      if (mover) {
        if (lane == 0) atomicExch(p.status, 1);
        mbar_wait(&s_bar, parity, kTmaDrainLimit);  // drain the one load in flight
      }
      return;
    }
    const int64_t base = geom.base(tix);
    int e = 0;
    if constexpr (P::kBlockScaled) {
      // Tile exponent: the largest exponent of the raw FP64 components.
      const G* tg = reinterpret_cast<const G*>(tile);
      unsigned emax = 0;
      for (int l = threadIdx.x; l < T; l += NT) {
        const G g = tg[l];
        emax = max(emax, (unsigned)max(fx_exponent(g.x), fx_exponent(g.y)));
      }
      emax = __reduce_max_sync(0xffffffffu, emax);
      if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = (int)emax;
      __syncthreads();
#pragma unroll
      for (int w = 0; w < NT / 32; ++w) e = max(e, s_red[w]);
    } else {
      (void)s_red;
    }
    // HBM type -> working type in place (each thread its elements
    // l = tid + 512 u), every op, then the threads' stores convert back.
    V* tv = reinterpret_cast<V*>(tile);
    if constexpr (!std::is_same<V, G>::value) {
      const G* tg = reinterpret_cast<const G*>(tile);
      for (int l = threadIdx.x; l < T; l += NT) tv[l] = cvt_in<P>(tg[l], e);
      __syncthreads();
    }
    tile_apply_ops<P>(tv, T, ops, num_ops, base, p.phase_tab);
    if constexpr (P::kBlockScaled) tile_store_fx(tv, amps, base, T, t_off, s_slot, e);
    else tile_store<P>(tv, amps, base, T, t_off, s_slot);
    fence_proxy_async_smem();
    __syncthreads();
    if (mover && next < num_tiles) geom.load(&tmap, &s_bar, tile, next, boxes, tile_bytes, lane);
  }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
  });
  return fn;
}

uint32_t g_tma_wait_limit = kTmaWaitLimit;

int* tma_status_ptr() {
  static int* ptrs[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!ptrs[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tma_status) != cudaSuccess) return nullptr;
    ptrs[dev] = static_cast<int*>(p);
  }
  return ptrs[dev];
}

// The statevector as a dense 5-D tensor cut at the pass's local qubits:
// dim0 = one swizzle row (2^RBITS amplitudes, 128 bytes), dim1 = the qubits
// from RBITS up to the first high qubit, dims 2-4 start at high qubits 0-2;
// the box takes every low qubit and high qubits 0-2.
template <int ES>
int encode_pass_map(CUtensorMap* map, void* amps, int32_t n, const Pass& ps, bool swizzle) {
  EncodeTiledFn fn = encode_tiled_fn();
  if (!fn) return set_error(DMV_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  constexpr int RBITS = row_bits<ES>();
  const int32_t* h = ps.high;
  const cuuint64_t comp = ES / 2;  // bytes per real component
  cuuint64_t dims[5] = {cuuint64_t(2) << RBITS, cuuint64_t(1) << (h[0] - RBITS), cuuint64_t(1) << (h[1] - h[0]),
                        cuuint64_t(1) << (h[2] - h[1]), cuuint64_t(1) << (n - h[2])};
  cuuint64_t strides[4] = {(cuuint64_t)ES << RBITS, (cuuint64_t)ES << h[0], (cuuint64_t)ES << h[1],
                           (cuuint64_t)ES << h[2]};
  cuuint32_t box[5] = {cuuint32_t(2) << RBITS, cuuint32_t(1) << (ps.low_bits - RBITS), 2, 2, 2};
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  (void)comp;
  const CUresult r = fn(map, ES == 16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, amps,
                        dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(DMV_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return DMV_OK;
}

// The tensor-core window pass (ARITH_TC) and its launcher.
#include "tc_window.cuh"

// TMA kernels by policy: register phases for complex64 (FP32 arithmetic),
// the shared-memory op loop for complex128 in FP64. The complex128 FP32-pair
// and int64 arithmetics keep the shared-memory kernel (k_apply_window),
// which measured 7-12 % faster for them than a TMA-staged variant.
template <typename P>
constexpr bool tma_phases() { return std::is_same<P, PolF32>::value; }

template <typename P>
constexpr bool tma_policy() { return std::is_same<P, PolF64>::value || std::is_same<P, PolF32>::value; }

// Whether a window pass runs on a TMA kernel: a TMA policy, 2^12-amplitude
// tiles with at least three high qubits and the low qubits covering a
// 128-byte row.
template <typename P>
bool tma_eligible(const Pass& ps) {
  constexpr int ES = (int)sizeof(typename P::G);
  const int k = ps.low_bits + ps.num_high;
  return tma_policy<P>() && k == kTileThreadBits + 3 && ps.num_high >= 3 && ps.low_bits >= row_bits<ES>();
}

template <typename P>
int launch_window_tma(void* amps, int32_t n, const Pass& ps, const Op* ops_dev, const PhaseOp* phase_ops_dev,
                      cudaStream_t stream, const void* phase_tab = nullptr, int fmt = 0) {
  if constexpr (!tma_policy<P>()) {
    (void)phase_ops_dev;
    return launch_window<P>(amps, n, ps, ops_dev, stream, phase_tab, fmt);
  } else {
    (void)fmt;
    if (!tma_eligible<P>(ps)) return launch_window<P>(amps, n, ps, ops_dev, stream, phase_tab);
    constexpr int ES = (int)sizeof(typename P::G);
    constexpr bool PHASES = tma_phases<P>();
    if ((reinterpret_cast<uintptr_t>(amps) & 15u) != 0)
      return set_error(DMV_ERR_INVALID, "statevector not 16-byte aligned");
    CUtensorMap map;
    DMV_TRY(encode_pass_map<ES>(&map, amps, n, ps, PHASES));
    TmaPassParams p;
    p.k = ps.low_bits + ps.num_high;
    p.low = ps.low_bits;
    p.nh = ps.num_high;
    p.num_ops = (int32_t)ps.op_count;
    for (int i = 0; i < 16; ++i) p.high[i] = i < ps.num_high ? ps.high[i] : 0;
    p.boxes = 1 << (ps.num_high - 3);
    p.wait_limit = g_tma_wait_limit;
    p.num_tiles = int64_t(1) << (n - p.k);
    p.ops = ops_dev + ps.op_begin;
    p.phase_ops = phase_ops_dev ? phase_ops_dev + ps.op_begin : nullptr;
    p.phase_tab = phase_tab;
    p.amps = amps;
    p.status = tma_status_ptr();
    if (!p.status) return set_error(DMV_ERR_CUDA, "cannot resolve the TMA status word");
    const size_t tile = (size_t)ES << p.k;
    if constexpr (PHASES) {
      if (!p.phase_ops || ps.op_count > kMaxPhaseOps)
        return set_error(DMV_ERR_STATE, "register-phase pass without its op table (%lld ops)",
                         (long long)ps.op_count);
      const size_t smem = (size_t)kPhaseBuffers * tile + 1024 + (size_t)kMaxPhaseOps * sizeof(PhaseOp);
      static bool configured = false;
      if (!configured) {
        DMV_CUDA_TRY(cudaFuncSetAttribute(k_window_phases<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
      }
      int per_sm = 0;
      DMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_window_phases<P>, kPhaseThreads, smem));
      if (per_sm < 1) return set_error(DMV_ERR_CUDA, "phase kernel cannot fit %zu bytes of shared memory", smem);
      const int64_t grid = std::min<int64_t>(p.num_tiles, (int64_t)per_sm * num_sms());
      k_window_phases<P><<<(int)grid, kPhaseThreads, smem, stream>>>(map, p);
    } else {
      const size_t smem = tile + 1024;
      static bool configured = false;
      if (!configured) {
        DMV_CUDA_TRY(cudaFuncSetAttribute(k_window_tma<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
      }
      int per_sm = 0;
      DMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_window_tma<P>, kWindowThreads, smem));
      if (per_sm < 1) return set_error(DMV_ERR_CUDA, "TMA window kernel cannot fit %zu bytes of shared memory", smem);
      const int64_t grid = std::min<int64_t>(p.num_tiles, (int64_t)per_sm * num_sms());
      k_window_tma<P><<<(int)grid, kWindowThreads, smem, stream>>>(map, p);
    }
    return DMV_OK;
  }
}

}  // namespace

int upload_ops(dmv_state_s* s, const Op* ops, int64_t count) {
  if (count <= 0) return DMV_OK;
  DMV_TRY(s->ops_dev.reserve((size_t)count * sizeof(Op)));
  DMV_CUDA_TRY(cudaMemcpyAsync(s->ops_dev.ptr, ops, (size_t)count * sizeof(Op),
                               cudaMemcpyHostToDevice, s->stream));
  return DMV_OK;
}

// Arithmetic operations one op performs over the whole statevector. FP64 /
// FP32 storage arithmetic: multiply-adds, GENERAL 16 per amplitude pair,
// REAL / DIAG / ANTI 8, SWAP none. FP32-pair arithmetic: FP32 operations of
// the compensated dot products, 172 per pair (four 4-term dots) and 76 (four
// 2-term dots). A control halves the count.
// INT64 block fixed point: IMAD.WIDE limb products, 64 per pair (four 4-term
// sums of 4 limb products each) and 32.
double op_multiply_adds(const Op& op, int64_t N, int arith) {
  double per_pair = 0.;
  const bool pair_arith = arith == ARITH_FP32X2, fixed = arith == ARITH_INT64;
  switch (op.cls) {
    case OP_GENERAL: per_pair = pair_arith ? 172. : fixed ? 64. : 16.; break;
    case OP_RXLIKE: per_pair = pair_arith ? 76. : fixed ? 64. : 8.; break;  // int64: the general code
    case OP_SWAP: per_pair = 0.; break;
    case OP_ROT: per_pair = 4.; break;  // FP64 only: one multiply-add per output, re and im
    case OP_PHASE: per_pair = pair_arith ? 76. : fixed ? 32. : 6.; break;  // one complex product per amplitude
    default: per_pair = pair_arith ? 76. : fixed ? 32. : 8.; break;
  }
  const double pairs = (double)N / 2.0;
  return per_pair * pairs * (op.ctrl_kind != CTRL_NONE ? 0.5 : 1.0);
}

// Register bits of a window pass that runs in register phases (complex64
// passes on the TMA kernel), 0 otherwise.
int window_reg_bits(const dmv_state_s* s, const Pass& ps) {
  if (s->precision == DMV_C64 && tma_eligible<PolF32>(ps)) return kPhaseRegBits;
  return 0;
}

int launch_plan(dmv_state_s* s, const Plan& plan) {
  // The launches: every pass, except that a register-phase pass with more
  // ops than the kernel's op table holds runs as several launches over the
  // same qubits. Ops are copied so the phase scheduler may reorder them.
  std::vector<Pass>& passes = s->pass_staging;
  std::vector<Op>& ops = s->ops_staging;
  passes.clear();
  ops.assign(plan.ops.begin(), plan.ops.end());
  bool any_window = false, any_phases = false;
  // FP64 window passes on the TMA kernel: rotations and phase tables in place of
  // general 2x2 ops (rewrite_pass_rotations), appended to the staged ops.
  // The FP32-pair and int64 arithmetics take the same rewrite with the rotations
  // as real 2x2 ops and the tables in their own forms.
  const bool c128 = s->precision == DMV_C128;
  const bool rewrite = c128 && ((s->arith == ARITH_FP64 && s->fp64_rewrite) || s->arith == ARITH_FP32X2 ||
                                s->arith == ARITH_INT64);
  const bool rot_ops = s->arith == ARITH_FP64;
  s->phase_tab.clear();
  // Per staged pass, the product of its OP_ROT factors (1 elsewhere).
  std::vector<ScaleDD>& pass_scale = s->pass_scale;
  pass_scale.clear();
  // The window passes' rewrites run on host threads (each pass independent);
  // their tables are appended in pass order with the OP_PHASE offsets moved.
  std::vector<RewrittenPass> rewritten;
  std::vector<int64_t> rewritten_at(plan.passes.size(), -1);
  if (rewrite) {
    std::vector<int64_t> which;
    for (size_t i = 0; i < plan.passes.size(); ++i)
      if (plan.passes[i].kind == 1) {
        rewritten_at[i] = (int64_t)which.size();
        which.push_back((int64_t)i);
      }
    rewrite_passes(plan, which, rot_ops, rewritten);
  }
  for (size_t pi = 0; pi < plan.passes.size(); ++pi) {
    const Pass& ps = plan.passes[pi];
    const int rb = ps.kind == 1 ? window_reg_bits(s, ps) : 0;
    any_window |= ps.kind == 1;
    if (rewritten_at[pi] >= 0) {
      const RewrittenPass& r = rewritten[(size_t)rewritten_at[pi]];
      Pass rw = ps;
      rw.op_begin = (int64_t)ops.size();
      rw.op_count = (int64_t)r.ops.size();
      const int32_t tab_base = (int32_t)s->phase_tab.size();
      for (Op op : r.ops) {
        if (op.cls == OP_PHASE) op.fh[0] += tab_base;
        ops.push_back(op);
      }
      s->phase_tab.insert(s->phase_tab.end(), r.tab.begin(), r.tab.end());
      passes.push_back(rw);
      pass_scale.push_back(r.scale);
      continue;
    }
    if (rb <= 0) {
      passes.push_back(ps);
      pass_scale.push_back(ScaleDD());
      continue;
    }
    any_phases = true;
    for (int64_t o = 0; o < ps.op_count; o += kMaxPhaseOps) {
      Pass sub = ps;
      sub.op_begin = ps.op_begin + o;
      sub.op_count = std::min<int64_t>(kMaxPhaseOps, ps.op_count - o);
      assign_phases(ops.data() + sub.op_begin, sub.op_count, ps.low_bits + ps.num_high, rb);
      passes.push_back(sub);
      pass_scale.push_back(ScaleDD());
    }
  }
  if (any_window) DMV_TRY(upload_ops(s, ops.data(), (int64_t)ops.size()));
  const PhaseOp* phase_ops_dev = nullptr;
  if (any_phases) {
    std::vector<PhaseOp>& pops = s->phase_ops;
    pops.resize(ops.size());
    for (size_t i = 0; i < ops.size(); ++i) {
      PhaseOp& q = pops[i];
      for (int j = 0; j < 8; ++j) q.m[j] = ops[i].mh[j];
      q.phase = (uint32_t)ops[i].phase;
      q.ctrl = ops[i].ctrl;
      q.ctrl_kind = ops[i].ctrl_kind;
      q.cls = ops[i].cls;
    }
    DMV_TRY(s->phase_ops_dev.reserve(pops.size() * sizeof(PhaseOp)));
    DMV_CUDA_TRY(cudaMemcpyAsync(s->phase_ops_dev.ptr, pops.data(), pops.size() * sizeof(PhaseOp),
                                 cudaMemcpyHostToDevice, s->stream));
    phase_ops_dev = static_cast<const PhaseOp*>(s->phase_ops_dev.ptr);
  }
  const Op* ops_dev = static_cast<const Op*>(s->ops_dev.ptr);
  // Phase tables: the FP64 form (also read by an int64 pass that falls back to
  // FP64) and the FP32-pair or Q.54 form for those arithmetics.
  const void* phase_tab_dev = nullptr;
  const void* phase_tab2_dev = nullptr;
  int64_t tab2_bytes = 0;
  if (!s->phase_tab.empty()) {
    phase_tables_f64(s->phase_tab, s->phase_tab_f64);
    DMV_TRY(s->phase_tab_dev.reserve(s->phase_tab_f64.size() * sizeof(double2)));
    DMV_CUDA_TRY(cudaMemcpyAsync(s->phase_tab_dev.ptr, s->phase_tab_f64.data(),
                                 s->phase_tab_f64.size() * sizeof(double2), cudaMemcpyHostToDevice, s->stream));
    phase_tab_dev = s->phase_tab_dev.ptr;
    const void* src2 = nullptr;
    if (s->arith == ARITH_FP32X2) {
      phase_tables_df(s->phase_tab, s->phase_tab_df);
      src2 = s->phase_tab_df.data();
      tab2_bytes = (int64_t)(s->phase_tab_df.size() * sizeof(float4));
    } else if (s->arith == ARITH_INT64) {
      phase_tables_fx(s->phase_tab, s->phase_tab_fx);
      src2 = s->phase_tab_fx.data();
      tab2_bytes = (int64_t)(s->phase_tab_fx.size() * sizeof(int4));
    }
    if (src2) {
      DMV_TRY(s->phase_tab2_dev.reserve((size_t)tab2_bytes));
      DMV_CUDA_TRY(cudaMemcpyAsync(s->phase_tab2_dev.ptr, src2, (size_t)tab2_bytes, cudaMemcpyHostToDevice, s->stream));
      phase_tab2_dev = s->phase_tab2_dev.ptr;
    }
  }
  // Tensor-core arithmetic: the stages and block digit matrices of every
  // window pass it takes, uploaded once for the whole plan.
  const bool tc = s->precision == DMV_C128 && s->arith == ARITH_TC;
  std::vector<int64_t> tc_first(passes.size(), -1);
  std::vector<int32_t> tc_count(passes.size(), 0);
  std::vector<int32_t> tc_blocks(passes.size(), 0);
  std::vector<int32_t> tc_maps(passes.size() * 12, 0);
  std::vector<int32_t> tc_exchanges(passes.size(), 0);
  if (tc) {
    s->tc_stages.clear();
    s->tc_u.clear();
    for (size_t i = 0; i < passes.size(); ++i) {
      const Pass& ps = passes[i];
      if (ps.kind != 1 || !tma_eligible<PolF64>(ps)) continue;
      const size_t mark = s->tc_stages.size();
      const size_t umark = s->tc_u.size();
      if (!build_tc_pass(plan, ps, s->tc_stages, s->tc_u, &tc_maps[i * 12], &tc_exchanges[i])) continue;
      tc_first[i] = (int64_t)mark;
      tc_count[i] = (int32_t)(s->tc_stages.size() - mark);
      tc_blocks[i] = (int32_t)((s->tc_u.size() - umark) / (size_t)kTcUHalves);
    }
    if (!s->tc_stages.empty()) {
      DMV_TRY(s->tc_stages_dev.reserve(s->tc_stages.size() * sizeof(TcStage)));
      DMV_CUDA_TRY(cudaMemcpyAsync(s->tc_stages_dev.ptr, s->tc_stages.data(), s->tc_stages.size() * sizeof(TcStage),
                                   cudaMemcpyHostToDevice, s->stream));
    }
    if (!s->tc_u.empty()) {
      DMV_TRY(s->tc_u_dev.reserve(s->tc_u.size() * sizeof(uint16_t)));
      DMV_CUDA_TRY(cudaMemcpyAsync(s->tc_u_dev.ptr, s->tc_u.data(), s->tc_u.size() * sizeof(uint16_t),
                                   cudaMemcpyHostToDevice, s->stream));
    }
  }
  int64_t bytes = 0;
  const int64_t S = (int64_t)s->amp_bytes();
  // FP32-pair arithmetic: when every launch is a window pass, the state stays in
  // the FP32-pair form between them (k_apply_window's FMT bits).
  bool df_chain = c128 && s->arith == ARITH_FP32X2 && passes.size() >= 2;
  for (const Pass& ps : passes) df_chain = df_chain && ps.kind == 1;
  // The OP_ROT factors left out of the state so far (each in [1/sqrt 2, 1];
  // a pass leaves at most 2^200 out, rewrite_pass_rotations folds the rest
  // back itself): multiplied back at the end, or after a pass when the stored
  // values could have grown past 2^200.
  ScaleDD owed;
  for (size_t pi = 0; pi < passes.size(); ++pi) {
    if (pi > 0) {
      owed.mul(pass_scale[pi - 1]);
      if (std::fabs(owed.hi) < 0x1p-200) {
        DMV_TRY(launch_scale_state(s, owed.hi));
        owed = ScaleDD();
      }
    }
    const Pass& ps = passes[pi];
    const int df_fmt = df_chain ? ((pi > 0 ? 1 : 0) | (pi + 1 < passes.size() ? 2 : 0)) : 0;
    if (tc && tc_first[pi] >= 0) {
      // Tensor-core FLOPs: 34 digit products of a 128 x 64 x 64 real product per
      // 4096-amplitude tile and block (2 FLOPs per multiply-add).
      const double flops = (double)tc_blocks[pi] * 34.0 * 2.0 * 64.0 * 64.0 * 128.0 * (double)(s->N >> 12);
      const int64_t tok = prof_begin(DMV_KERNEL_WINDOW, s->stream, (double)(2 * S), flops);
      DMV_TRY(launch_window_tc(s->amps, s->n, ps,
                               static_cast<const TcStage*>(s->tc_stages_dev.ptr) + tc_first[pi], tc_count[pi],
                               static_cast<const uint16_t*>(s->tc_u_dev.ptr), &tc_maps[pi * 12], s->stream));
      prof_end(tok, s->stream);
      bytes += 2 * S;
      count_launch();
      continue;
    }
    // Block fixed point needs unitary ops; a pass with any other op runs in FP64.
    // Passes the tensor cores do not take run in the integer-pipe arithmetic.
    int arith = s->precision == DMV_C64 ? ARITH_FP64 : s->arith;
    if (arith == ARITH_TC) arith = ARITH_INT64;
    if (arith == ARITH_INT64)
      for (int64_t o = 0; o < ps.op_count; ++o)
        if (!ops[(size_t)(ps.op_begin + o)].unitary) arith = ARITH_FP64;
    if (ps.kind == 0) {
      const Op& op = ops[(size_t)ps.op_begin];
      const int64_t b = op.ctrl_kind != CTRL_NONE ? S : 2 * S;
      const int64_t tok = prof_begin(DMV_KERNEL_SINGLE, s->stream, (double)b, op_multiply_adds(op, s->N, arith));
      if (s->precision == DMV_C64) launch_single<PolF32>(s->amps, s->n, op, s->stream);
      else if (arith == ARITH_FP32X2) launch_single<PolDF>(s->amps, s->n, op, s->stream);
      else if (arith == ARITH_INT64) launch_single<PolFX>(s->amps, s->n, op, s->stream);
      else launch_single<PolF64>(s->amps, s->n, op, s->stream);
      prof_end(tok, s->stream);
      bytes += b;
    } else {
      double fmas = 0.;
      for (int64_t o = 0; o < ps.op_count; ++o)
        fmas += op_multiply_adds(ops[(size_t)(ps.op_begin + o)], s->N, arith);
      const int64_t tok = prof_begin(DMV_KERNEL_WINDOW, s->stream, (double)(2 * S), fmas);
      void* a = s->amps;
      cudaStream_t st = s->stream;
      if (s->precision == DMV_C64) DMV_TRY(launch_window_tma<PolF32>(a, s->n, ps, ops_dev, phase_ops_dev, st));
      else if (arith == ARITH_FP32X2)
        DMV_TRY(launch_window_tma<PolDF>(a, s->n, ps, ops_dev, phase_ops_dev, st, phase_tab2_dev, df_fmt));
      else if (arith == ARITH_INT64) DMV_TRY(launch_window_tma<PolFX>(a, s->n, ps, ops_dev, phase_ops_dev, st, phase_tab2_dev));
      else DMV_TRY(launch_window_tma<PolF64>(a, s->n, ps, ops_dev, phase_ops_dev, st, phase_tab_dev));
      prof_end(tok, s->stream);
      bytes += 2 * S;
    }
    count_launch();
  }
  if (!passes.empty()) {
    owed.mul(pass_scale.back());
  }
  if (owed.hi != 1.0 || owed.lo != 0.0) DMV_TRY(launch_scale_state(s, owed.hi + owed.lo));
  DMV_CUDA_TRY(cudaGetLastError());
  s->last_tc_passes = s->last_tc_blocks = s->last_tc_swaps = 0;
  for (size_t pi = 0; pi < passes.size(); ++pi)
    if (tc && tc_first[pi] >= 0) {
      ++s->last_tc_passes;
      s->last_tc_blocks += tc_blocks[pi];
      s->last_tc_swaps += tc_exchanges[pi];
    }
  s->last_passes = (int64_t)passes.size();
  s->last_ops = (int64_t)plan.ops.size();
  s->last_phase_tab_bytes = (int64_t)(s->phase_tab_f64.size() * sizeof(double2));
  s->last_upload_bytes = s->last_phase_tab_bytes + tab2_bytes + (any_window ? (int64_t)(ops.size() * sizeof(Op)) : 0) +
                         (any_phases ? (int64_t)(s->phase_ops.size() * sizeof(PhaseOp)) : 0) +
                         (tc ? (int64_t)(s->tc_stages.size() * sizeof(TcStage) + s->tc_u.size() * 2) : 0);
  s->last_bytes = bytes;
  return DMV_OK;
}

// The state times a real factor: the product of the FP64 rotations' factors
// (OP_ROT) that the window passes leave out.
__global__ void k_scale_state(double2* __restrict__ a, int64_t N, double f) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    const double2 v = a[i];
    a[i] = make_double2(v.x * f, v.y * f);
  }
}

int launch_scale_state(dmv_state_s* s, double f) {
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((s->N + 255) / 256, (int64_t)num_sms() * 8));
  k_scale_state<<<grid, 256, 0, s->stream>>>(static_cast<double2*>(s->amps), s->N, f);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

// |0...0>: clear the vector and set amplitude 0 to 1 (damavand-gpu/kernels.cu:62-81).
__global__ void k_set_one(void* amps, int precision) {
  if (precision == DMV_C128) static_cast<double2*>(amps)[0] = make_double2(1.0, 0.0);
  else static_cast<float2*>(amps)[0] = make_float2(1.0f, 0.0f);
}

int launch_set_zero(dmv_state_s* s) {
  DMV_CUDA_TRY(cudaMemsetAsync(s->amps, 0, s->amp_bytes(), s->stream));
  k_set_one<<<1, 1, 0, s->stream>>>(s->amps, s->precision);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

// A load wait of a TMA window kernel or of the bulk-staged chunk-mass pass
// that gave up leaves 1 in the device status word; report it (and clear it)
// as DMV_ERR_TIMEOUT.
int check_window_status() {
  int* p = tma_status_ptr();
  if (!p) return DMV_OK;
  int v = 0;
  DMV_CUDA_TRY(cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost));
  if (v != 0) {
    const int zero = 0;
    DMV_CUDA_TRY(cudaMemcpy(p, &zero, sizeof(int), cudaMemcpyHostToDevice));
    return set_error(DMV_ERR_TIMEOUT, "a TMA load did not complete within its wait limit");
  }
  return DMV_OK;
}

int* tma_status_word() { return tma_status_ptr(); }
uint32_t tma_wait_limit() { return g_tma_wait_limit; }

void set_tma_wait_limit(int64_t polls) {
  g_tma_wait_limit = polls < 0 ? kTmaWaitLimit : (uint32_t)std::min<int64_t>(polls, 0xffffffffLL);
}

}  // namespace dmv
