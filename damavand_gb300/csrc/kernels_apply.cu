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
#include <algorithm>

#include "internal.h"
#include "policies.cuh"

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
};

static_assert(kWindowThreads == kTileThreads, "tile staging assumes 512 threads");

template <typename P>
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
      tile_apply_ops<P>(tile, T, p.ops, p.num_ops, base);
      tile_store_fx(tile, a, base, T, t_off, s_slot, e);
    } else {
      (void)s_red;
      tile_load<P, false>(tile, a, base, T, t_off, s_slot);
      __syncthreads();
      tile_apply_ops<P>(tile, T, p.ops, p.num_ops, base);
      tile_store<P>(tile, a, base, T, t_off, s_slot);
    }
    __syncthreads();
  }
}

template <typename P>
int launch_window(void* amps, int32_t n, const Pass& ps, const Op* ops_dev, cudaStream_t stream) {
  using V = typename P::T;
  WindowParams p;
  p.k = ps.low_bits + ps.num_high;
  p.low = ps.low_bits;
  p.nh = ps.num_high;
  p.num_ops = (int32_t)ps.op_count;
  for (int i = 0; i < 16; ++i) p.high[i] = i < ps.num_high ? ps.high[i] : 0;
  p.num_tiles = int64_t(1) << (n - p.k);
  p.ops = ops_dev + ps.op_begin;
  const size_t smem = (size_t(1) << p.k) * sizeof(V);
  static size_t configured = 0;
  if (smem > configured) {
    DMV_CUDA_TRY(cudaFuncSetAttribute(k_apply_window<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
    configured = smem;
  }
  int per_sm = 0;
  DMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_window<P>, kWindowThreads, smem));
  if (per_sm < 1) return set_error(DMV_ERR_CUDA, "window kernel cannot fit %zu bytes of shared memory", smem);
  const int64_t grid = std::min<int64_t>(p.num_tiles, (int64_t)per_sm * num_sms());
  k_apply_window<P><<<(int)grid, kWindowThreads, smem, stream>>>(static_cast<typename P::G*>(amps), p);
  return DMV_OK;
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
    case OP_SWAP: per_pair = 0.; break;
    default: per_pair = pair_arith ? 76. : fixed ? 32. : 8.; break;
  }
  const double pairs = (double)N / 2.0;
  return per_pair * pairs * (op.ctrl_kind != CTRL_NONE ? 0.5 : 1.0);
}

int launch_plan(dmv_state_s* s, const Plan& plan) {
  bool any_window = false;
  for (const Pass& ps : plan.passes) any_window |= ps.kind == 1;
  if (any_window) DMV_TRY(upload_ops(s, plan.ops.data(), (int64_t)plan.ops.size()));
  const Op* ops_dev = static_cast<const Op*>(s->ops_dev.ptr);
  int64_t bytes = 0;
  const int64_t S = (int64_t)s->amp_bytes();
  for (const Pass& ps : plan.passes) {
    // Block fixed point needs unitary ops; a pass with any other op runs in FP64.
    int arith = s->precision == DMV_C64 ? ARITH_FP64 : s->arith;
    if (arith == ARITH_INT64)
      for (int64_t o = 0; o < ps.op_count; ++o)
        if (!plan.ops[(size_t)(ps.op_begin + o)].unitary) arith = ARITH_FP64;
    if (ps.kind == 0) {
      const Op& op = plan.ops[(size_t)ps.op_begin];
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
        fmas += op_multiply_adds(plan.ops[(size_t)(ps.op_begin + o)], s->N, arith);
      const int64_t tok = prof_begin(DMV_KERNEL_WINDOW, s->stream, (double)(2 * S), fmas);
      if (s->precision == DMV_C64) DMV_TRY(launch_window<PolF32>(s->amps, s->n, ps, ops_dev, s->stream));
      else if (arith == ARITH_FP32X2) DMV_TRY(launch_window<PolDF>(s->amps, s->n, ps, ops_dev, s->stream));
      else if (arith == ARITH_INT64) DMV_TRY(launch_window<PolFX>(s->amps, s->n, ps, ops_dev, s->stream));
      else DMV_TRY(launch_window<PolF64>(s->amps, s->n, ps, ops_dev, s->stream));
      prof_end(tok, s->stream);
      bytes += 2 * S;
    }
    count_launch();
  }
  DMV_CUDA_TRY(cudaGetLastError());
  s->last_passes = (int64_t)plan.passes.size();
  s->last_ops = (int64_t)plan.ops.size();
  s->last_bytes = bytes;
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

}  // namespace dmv
