// Batched execution of many independent circuits of uneven size and depth.
//
// All statevectors live in one device arena. The host plans every circuit
// into window passes (the single-state planner), cuts every pass into items
// of a few tiles, and orders the items pass by pass across circuits. One
// persistent, cooperative kernel then claims items from a global queue: an
// item of pass p of circuit b waits until every item of b's earlier passes
// has completed (a per-circuit completion counter), stages its tiles in shared
// memory, applies the pass's ops and writes the tiles back. An item only waits
// on items claimed before it by CTAs that are already running, so the wait
// always ends; it is nevertheless bounded, after which the kernel raises an
// error flag and every CTA returns. The arena reset, the kernel and the
// per-circuit Pauli-Z reductions are captured in one CUDA graph.
//
// An autotuner picks the tile size, the number of always-local low qubits
// and the tiles per item by timing graph runs of the batch itself.
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"
#include "policies.cuh"

namespace dmv {
namespace {

constexpr int kBatchThreads = 512;
constexpr long long kDefaultSpinLimit = 1LL << 22;  // x 1 us sleeps: ~4 s before giving up

struct BatchPass {
  int32_t k, low, nh, num_ops;
  int32_t high[16];
  int64_t amp_offset;  // first amplitude of the circuit in the arena
  int64_t op_begin;    // first op in the batch op array
  int32_t fmt;         // FP32-pair batches: bit 0 reads, bit 1 writes the pair form (not its
  int32_t pad;         // circuit's first / last pass), so the passes between skip the conversions
};

struct BatchItem {
  int32_t pass;
  int32_t circuit;
  int64_t tile_begin, tile_end;
  int64_t wait_count;  // items of this circuit that must have completed
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// counters[0]: queue head, counters[1]: error flag, counters[2 + b]: items of
// circuit b completed.
template <typename P>
__global__ void __launch_bounds__(kBatchThreads, 2)
k_batch(typename P::G* __restrict__ arena, const BatchPass* __restrict__ passes, const BatchItem* __restrict__ items,
        int64_t num_items, const Op* __restrict__ ops, unsigned long long* counters, long long spin_limit) {
  using V = typename P::T;
  using G = typename P::G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tile = reinterpret_cast<V*>(smem_raw);
  __shared__ long long s_item;
  __shared__ int s_stop;
  __shared__ int64_t s_slot[kMaxSlots];
  __shared__ int s_red[kTileThreads / 32];
  (void)s_red;
  for (;;) {
    if (threadIdx.x == 0) {
      const long long it = (long long)atomicAdd(&counters[0], 1ull);
      int stop = it >= num_items ? 1 : 0;
      if (!stop && items[it].wait_count > 0) {
        const unsigned long long* done = counters + 2 + items[it].circuit;
        const unsigned long long need = (unsigned long long)items[it].wait_count;
        long long spins = 0;
        while (ld_acquire_u64(done) < need) {
          if (++spins > spin_limit || *(volatile unsigned long long*)&counters[1] != 0ull) {
            stop = 2;
            break;
          }
          __nanosleep(1000);
        }
      }
      if (stop == 2) atomicExch(&counters[1], 1ull);
      s_item = it;
      s_stop = stop;
    }
    __syncthreads();
    if (s_stop) break;
    const BatchItem item = items[s_item];
    const BatchPass ps = passes[item.pass];
    G* a = arena + ps.amp_offset;
    const int T = 1 << ps.k;
    const int64_t t_off = tile_thread_offset(ps.low, ps.nh, ps.high);
    tile_slot_offsets(ps.low, ps.nh, ps.high, (T + kTileThreads - 1) >> kTileThreadBits, s_slot);
    __syncthreads();
    for (int64_t tix = item.tile_begin; tix < item.tile_end; ++tix) {
      int64_t base = tix << ps.low;
      for (int i = 0; i < ps.nh; ++i) base = insert_zero(base, ps.high[i]);
      // L2-coherent loads: another SM wrote these amplitudes in the previous pass.
      if constexpr (P::kBlockScaled) {
        const int e = tile_load_fx<true>(tile, a, base, T, t_off, s_slot, s_red);
        __syncthreads();
        tile_apply_ops<P>(tile, T, ops + ps.op_begin, ps.num_ops, base);
        tile_store_fx(tile, a, base, T, t_off, s_slot, e);
      } else {
        if constexpr (std::is_same<P, PolDF>::value) {
          if (ps.fmt & 1) tile_load<PolRaw<P>, true>(tile, reinterpret_cast<const V*>(a), base, T, t_off, s_slot);
          else tile_load<P, true>(tile, a, base, T, t_off, s_slot);
        } else {
          tile_load<P, true>(tile, a, base, T, t_off, s_slot);
        }
        __syncthreads();
        tile_apply_ops<P>(tile, T, ops + ps.op_begin, ps.num_ops, base);
        if constexpr (std::is_same<P, PolDF>::value) {
          if (ps.fmt & 2) tile_store<PolRaw<P>>(tile, reinterpret_cast<V*>(a), base, T, t_off, s_slot);
          else tile_store<P>(tile, a, base, T, t_off, s_slot);
        } else {
          tile_store<P>(tile, a, base, T, t_off, s_slot);
        }
      }
      __syncthreads();
    }
    __threadfence();  // publish this item's amplitudes before counting it done
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&counters[2 + item.circuit], 1ull);
  }
}

template <typename G>
__global__ void k_batch_init(G* arena, const int64_t* offsets, int count) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < count) {
    G one;
    one.x = 1;
    one.y = 0;
    arena[offsets[b]] = one;
  }
}

}  // namespace
}  // namespace dmv

using namespace dmv;

struct dmv_batch_s {
  int32_t count = 0;
  int32_t precision = DMV_C128;
  int32_t arith = ARITH_FP64;
  std::vector<int32_t> n;
  std::vector<std::vector<Gate>> gates;
  std::vector<int64_t> offsets;  // amplitudes
  int64_t total_amps = 0;
  void* arena = nullptr;
  cudaStream_t stream = nullptr;
  DeviceBuffer passes_dev, items_dev, ops_dev, counters_dev, offsets_dev, reduce_dev;
  std::vector<int64_t> red_partial, red_sums;  // per-circuit offsets (doubles) into reduce_dev
  int64_t num_items = 0, num_passes = 0, num_ops = 0;
  int32_t max_k = 0;
  PlanOptions opt;
  int32_t tiles_per_item = 4;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool use_graph = true;
  bool all_unitary = true;  // block fixed point needs unitary ops everywhere
  long long spin_limit = kDefaultSpinLimit;
  bool poison_next_plan = false;  // test hook: one item waits for a count that never arrives
  int grid = 0;
  float last_ms = 0.f;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t amp_size() const { return precision == DMV_C128 ? 16 : 8; }
};

namespace dmv {
namespace {

void destroy_graph(dmv_batch_s* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// Plans every circuit with b->opt / b->tiles_per_item and uploads the tables.
int batch_plan(dmv_batch_s* b) {
  std::vector<BatchPass> passes;
  std::vector<Op> ops;
  std::vector<std::vector<int32_t>> pass_ids((size_t)b->count);
  std::vector<std::vector<int64_t>> pass_tiles((size_t)b->count);
  b->max_k = 0;
  for (int32_t c = 0; c < b->count; ++c) {
    Plan plan;
    PlanOptions opt = b->opt;
    opt.windows_only = true;
    DMV_TRY(build_plan(b->gates[(size_t)c], b->n[(size_t)c], b->precision, opt, plan));
    for (const Pass& p : plan.passes) {
      BatchPass bp;
      std::memset(&bp, 0, sizeof(bp));
      bp.k = p.low_bits + p.num_high;
      bp.low = p.low_bits;
      bp.nh = p.num_high;
      bp.num_ops = (int32_t)p.op_count;
      for (int i = 0; i < p.num_high; ++i) bp.high[i] = p.high[i];
      bp.amp_offset = b->offsets[(size_t)c];
      bp.op_begin = (int64_t)ops.size();
      for (int64_t o = 0; o < p.op_count; ++o) ops.push_back(plan.ops[(size_t)(p.op_begin + o)]);
      b->max_k = std::max(b->max_k, bp.k);
      if (b->precision == DMV_C128 && b->arith == ARITH_FP32X2) {
        const size_t pi = (size_t)(&p - plan.passes.data());
        bp.fmt = (pi > 0 ? 1 : 0) | (pi + 1 < plan.passes.size() ? 2 : 0);
      }
      pass_ids[(size_t)c].push_back((int32_t)passes.size());
      pass_tiles[(size_t)c].push_back(int64_t(1) << (b->n[(size_t)c] - bp.k));
      passes.push_back(bp);
    }
  }
  // Items, wave by wave: pass 0 of every circuit, then pass 1, ...
  std::vector<BatchItem> items;
  std::vector<int64_t> items_done_before((size_t)b->count, 0);
  size_t max_passes = 0;
  for (const auto& v : pass_ids) max_passes = std::max(max_passes, v.size());
  const int64_t tpi = std::max<int32_t>(1, b->tiles_per_item);
  for (size_t p = 0; p < max_passes; ++p) {
    for (int32_t c = 0; c < b->count; ++c) {
      if (p >= pass_ids[(size_t)c].size()) continue;
      const int64_t tiles = pass_tiles[(size_t)c][p];
      const int64_t wait = items_done_before[(size_t)c];
      int64_t made = 0;
      for (int64_t t0 = 0; t0 < tiles; t0 += tpi) {
        BatchItem it;
        it.pass = pass_ids[(size_t)c][p];
        it.circuit = c;
        it.tile_begin = t0;
        it.tile_end = std::min(tiles, t0 + tpi);
        it.wait_count = p == 0 ? 0 : wait;
        items.push_back(it);
        ++made;
      }
      items_done_before[(size_t)c] += made;
    }
  }
  if (b->poison_next_plan) {
    // Test hook: the last dependent item waits for more completions than its
    // circuit will ever report, so its bounded wait must run out.
    for (size_t i = items.size(); i-- > 0;)
      if (items[i].wait_count > 0) {
        items[i].wait_count = int64_t(1) << 60;
        break;
      }
  }
  b->all_unitary = true;
  for (const Op& op : ops) b->all_unitary = b->all_unitary && op.unitary;
  b->num_items = (int64_t)items.size();
  b->num_passes = (int64_t)passes.size();
  b->num_ops = (int64_t)ops.size();
  DMV_TRY(b->passes_dev.reserve(std::max<size_t>(1, passes.size()) * sizeof(BatchPass)));
  DMV_TRY(b->items_dev.reserve(std::max<size_t>(1, items.size()) * sizeof(BatchItem)));
  DMV_TRY(b->ops_dev.reserve(std::max<size_t>(1, ops.size()) * sizeof(Op)));
  if (!passes.empty())
    DMV_CUDA_TRY(cudaMemcpy(b->passes_dev.ptr, passes.data(), passes.size() * sizeof(BatchPass), cudaMemcpyHostToDevice));
  if (!items.empty())
    DMV_CUDA_TRY(cudaMemcpy(b->items_dev.ptr, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
  if (!ops.empty())
    DMV_CUDA_TRY(cudaMemcpy(b->ops_dev.ptr, ops.data(), ops.size() * sizeof(Op), cudaMemcpyHostToDevice));
  return DMV_OK;
}

template <typename P>
int batch_launch_kernel(dmv_batch_s* b) {
  const size_t smem = (size_t(1) << b->max_k) * sizeof(typename P::T);
  DMV_CUDA_TRY(cudaFuncSetAttribute(k_batch<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)std::max<size_t>(smem, 48 * 1024)));
  int per_sm = 0;
  DMV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<P>, kBatchThreads, smem));
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (per_sm < 1) return set_error(DMV_ERR_CUDA, "batch kernel does not fit (%zu bytes of shared memory)", smem);
  b->grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)per_sm * sms, b->num_items));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)b->grid);
  cfg.blockDim = dim3(kBatchThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = b->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  DMV_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_batch<P>, static_cast<typename P::G*>(b->arena),
                                  static_cast<const BatchPass*>(b->passes_dev.ptr),
                                  static_cast<const BatchItem*>(b->items_dev.ptr), b->num_items,
                                  static_cast<const Op*>(b->ops_dev.ptr),
                                  static_cast<unsigned long long*>(b->counters_dev.ptr), b->spin_limit));
  count_launch();
  return DMV_OK;
}

// The whole run as stream work: counters and arena reset, |0...0> per
// circuit, the persistent kernel, then the per-circuit Pauli-Z reductions.
int batch_enqueue(dmv_batch_s* b) {
  DMV_CUDA_TRY(cudaMemsetAsync(b->counters_dev.ptr, 0, (size_t)(2 + b->count) * sizeof(unsigned long long), b->stream));
  DMV_CUDA_TRY(cudaMemsetAsync(b->arena, 0, (size_t)b->total_amps * b->amp_size(), b->stream));
  const int init_grid = (b->count + 255) / 256;
  if (b->precision == DMV_C128)
    k_batch_init<double2><<<init_grid, 256, 0, b->stream>>>(static_cast<double2*>(b->arena),
                                                            static_cast<const int64_t*>(b->offsets_dev.ptr), b->count);
  else
    k_batch_init<float2><<<init_grid, 256, 0, b->stream>>>(static_cast<float2*>(b->arena),
                                                           static_cast<const int64_t*>(b->offsets_dev.ptr), b->count);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  if (b->num_items > 0) {
    if (b->precision == DMV_C64) DMV_TRY(batch_launch_kernel<PolF32>(b));
    else if (b->arith == ARITH_FP32X2) DMV_TRY(batch_launch_kernel<PolDF>(b));
    else if (b->arith == ARITH_INT64 && b->all_unitary) DMV_TRY(batch_launch_kernel<PolFX>(b));
    else DMV_TRY(batch_launch_kernel<PolF64>(b));
  }
  double* red = static_cast<double*>(b->reduce_dev.ptr);
  for (int32_t c = 0; c < b->count; ++c) {
    const char* base = static_cast<const char*>(b->arena) + (size_t)b->offsets[(size_t)c] * b->amp_size();
    DMV_TRY(launch_chunk_mass_into(base, b->precision == DMV_C128 ? 0 : 1, b->n[(size_t)c],
                                   red + b->red_partial[(size_t)c], red + b->red_sums[(size_t)c], b->stream));
  }
  return DMV_OK;
}

int batch_build_graph(dmv_batch_s* b) {
  destroy_graph(b);
  DMV_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = batch_enqueue(b);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc != DMV_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_error(DMV_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  b->graph = g;
  DMV_CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return DMV_OK;
}

int batch_run(dmv_batch_s* b, float* ms) {
  if (!b->exec && b->use_graph) {
    if (batch_build_graph(b) != DMV_OK) {
      // Capture of this launch sequence is not available: enqueue it directly.
      cudaGetLastError();
      destroy_graph(b);
      b->use_graph = false;
    }
  }
  if (!b->ev0) DMV_CUDA_TRY(cudaEventCreate(&b->ev0));
  if (!b->ev1) DMV_CUDA_TRY(cudaEventCreate(&b->ev1));
  DMV_CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
  if (b->use_graph) DMV_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
  else DMV_TRY(batch_enqueue(b));
  DMV_CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
  DMV_CUDA_TRY(cudaEventSynchronize(b->ev1));
  float t = 0.f;
  DMV_CUDA_TRY(cudaEventElapsedTime(&t, b->ev0, b->ev1));
  b->last_ms = t;
  if (ms) *ms = t;
  unsigned long long err = 0;
  DMV_CUDA_TRY(cudaMemcpy(&err, static_cast<unsigned long long*>(b->counters_dev.ptr) + 1, sizeof(err),
                          cudaMemcpyDeviceToHost));
  if (err) return set_error(DMV_ERR_TIMEOUT, "batched kernel: a dependency wait gave up; results are incomplete");
  return DMV_OK;
}

}  // namespace
}  // namespace dmv

extern "C" int dmv_batch_create(int32_t num_circuits, const int32_t* num_qubits, const int64_t* gate_offsets,
                                const dmv_gate_t* gates, int32_t precision, int32_t arithmetic, dmv_batch_t* out) {
  clear_error();
  if (!out) return set_error(DMV_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (num_circuits < 1 || !num_qubits || !gate_offsets) return set_error(DMV_ERR_INVALID, "empty batch");
  if (precision != DMV_C128 && precision != DMV_C64) return set_error(DMV_ERR_INVALID, "unknown precision");
  if (arithmetic != DMV_ARITH_FP64 && arithmetic != DMV_ARITH_FP32X2 && arithmetic != DMV_ARITH_INT64 &&
      arithmetic != DMV_ARITH_FP64_DIRECT)
    return set_error(DMV_ERR_INVALID, "unknown arithmetic");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(DMV_ERR_NO_DEVICE, "no CUDA device visible");
  }
  dmv_batch_s* b = new dmv_batch_s();
  b->count = num_circuits;
  b->precision = precision;
  // Batches apply every fused 2x2 directly: the rotation/phase-table rewrite of
  // single states builds one table per pass, which many small circuits cannot
  // amortise (config-4-like batches: ~22k tables, 2.9 GB, for 512 circuits).
  b->arith = arithmetic == DMV_ARITH_FP64_DIRECT ? (int32_t)ARITH_FP64 : arithmetic;
  int64_t off = 0;
  for (int32_t c = 0; c < num_circuits; ++c) {
    const int32_t n = num_qubits[c];
    if (n < 1 || n > 30) {
      delete b;
      return set_error(DMV_ERR_INVALID, "circuit %d: %d qubits outside [1, 30]", c, n);
    }
    if (gate_offsets[c + 1] < gate_offsets[c]) {
      delete b;
      return set_error(DMV_ERR_INVALID, "circuit %d: decreasing gate offsets", c);
    }
    std::vector<Gate> parsed;
    const int rc = parse_gates(gates + gate_offsets[c], gate_offsets[c + 1] - gate_offsets[c], n, parsed);
    if (rc != DMV_OK) {
      delete b;
      return rc;
    }
    b->n.push_back(n);
    b->gates.push_back(std::move(parsed));
    b->offsets.push_back(off);
    off += (int64_t(1) << n) + 15;
    off &= ~int64_t(15);  // 256-byte aligned starts for complex128
  }
  b->total_amps = off;
  int rc = DMV_OK;
  do {
    if (injected_alloc_failure() || cudaMalloc(&b->arena, (size_t)b->total_amps * b->amp_size()) != cudaSuccess) {
      cudaGetLastError();
      b->arena = nullptr;
      rc = set_error(DMV_ERR_OOM, "cannot allocate the %.2f GB batch arena", (double)b->total_amps * b->amp_size() / 1e9);
      break;
    }
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      rc = set_error(DMV_ERR_CUDA, "cudaStreamCreate failed");
      break;
    }
    if ((rc = b->counters_dev.reserve((size_t)(2 + num_circuits) * sizeof(unsigned long long))) != DMV_OK) break;
    if ((rc = b->offsets_dev.reserve((size_t)num_circuits * sizeof(int64_t))) != DMV_OK) break;
    if (cudaMemcpy(b->offsets_dev.ptr, b->offsets.data(), (size_t)num_circuits * sizeof(int64_t),
                   cudaMemcpyHostToDevice) != cudaSuccess) {
      rc = set_error(DMV_ERR_CUDA, "offset upload failed");
      break;
    }
    int64_t red = 0;
    for (int32_t c = 0; c < num_circuits; ++c) {
      const ChunkMassShape sh = chunk_mass_shape(b->n[(size_t)c]);
      b->red_partial.push_back(red);
      red += sh.partial_elems;
      b->red_sums.push_back(red);
      red += b->n[(size_t)c] + 1;
    }
    if ((rc = b->reduce_dev.reserve((size_t)red * sizeof(double))) != DMV_OK) break;
    rc = batch_plan(b);
  } while (false);
  if (rc != DMV_OK) {
    dmv_batch_destroy(b);
    return rc;
  }
  *out = b;
  return DMV_OK;
}

extern "C" int dmv_batch_destroy(dmv_batch_t b) {
  if (!b) return DMV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  destroy_graph(b);
  if (b->arena) cudaFree(b->arena);
  b->passes_dev.release();
  b->items_dev.release();
  b->ops_dev.release();
  b->counters_dev.release();
  b->offsets_dev.release();
  b->reduce_dev.release();
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return DMV_OK;
}

extern "C" int dmv_batch_configure(dmv_batch_t b, int32_t tile_bits, int32_t low_bits, int32_t tiles_per_item) {
  clear_error();
  if (!b) return set_error(DMV_ERR_INVALID, "null batch");
  if (tile_bits < 2 || tile_bits > 13 || low_bits < 1 || low_bits > tile_bits || low_bits > 9 || tiles_per_item < 1)
    return set_error(DMV_ERR_INVALID, "bad batch configuration (%d, %d, %d)", tile_bits, low_bits, tiles_per_item);
  if (b->precision == DMV_C128 && tile_bits > 12)
    return set_error(DMV_ERR_INVALID, "complex128 tiles hold at most 2^12 amplitudes");
  b->opt.tile_bits = tile_bits;
  b->opt.low_bits = low_bits;
  b->tiles_per_item = tiles_per_item;
  destroy_graph(b);
  return batch_plan(b);
}

extern "C" int dmv_batch_debug_wait_limit(dmv_batch_t b, int64_t spin_limit, int32_t poison) {
  clear_error();
  if (!b || spin_limit < 1) return set_error(DMV_ERR_INVALID, "bad wait limit");
  b->spin_limit = spin_limit;
  b->poison_next_plan = poison != 0;
  destroy_graph(b);
  return batch_plan(b);
}

extern "C" int dmv_batch_run(dmv_batch_t b, double* elapsed_ms) {
  clear_error();
  if (!b) return set_error(DMV_ERR_INVALID, "null batch");
  float ms = 0.f;
  const int rc = batch_run(b, &ms);
  if (elapsed_ms) *elapsed_ms = ms;
  return rc;
}

extern "C" int dmv_batch_autotune(dmv_batch_t b, int32_t* tile_bits, int32_t* low_bits, int32_t* tiles_per_item,
                                  double* best_ms) {
  clear_error();
  if (!b) return set_error(DMV_ERR_INVALID, "null batch");
  const int max_tile = b->precision == DMV_C128 ? 12 : 13;
  struct Cand { int k, low, tpi; };
  std::vector<Cand> cands;
  for (int k : {10, 11, 12, 13})
    if (k <= max_tile)
      for (int low : {5, 6})
        for (int tpi : {1, 4, 16}) cands.push_back({k, low, tpi});
  Cand best{b->opt.tile_bits, b->opt.low_bits, b->tiles_per_item};
  float best_t = 1e30f;
  for (const Cand& c : cands) {
    DMV_TRY(dmv_batch_configure(b, c.k, c.low, c.tpi));
    float t = 0.f;
    DMV_TRY(batch_run(b, &t));  // build + warm
    DMV_TRY(batch_run(b, &t));
    if (t < best_t) {
      best_t = t;
      best = c;
    }
  }
  DMV_TRY(dmv_batch_configure(b, best.k, best.low, best.tpi));
  if (tile_bits) *tile_bits = best.k;
  if (low_bits) *low_bits = best.low;
  if (tiles_per_item) *tiles_per_item = best.tpi;
  if (best_ms) *best_ms = best_t;
  return DMV_OK;
}

extern "C" int dmv_batch_expect_z(dmv_batch_t b, double* out) {
  clear_error();
  if (!b || !out) return set_error(DMV_ERR_INVALID, "null batch or output");
  DMV_CUDA_TRY(cudaStreamSynchronize(b->stream));
  DMV_TRY(check_window_status());  // a mass pass whose chunk load wait gave up
  int64_t pos = 0;
  for (int32_t c = 0; c < b->count; ++c) {
    const int n = b->n[(size_t)c];
    std::vector<double> h((size_t)n + 1);
    DMV_CUDA_TRY(cudaMemcpy(h.data(), static_cast<double*>(b->reduce_dev.ptr) + b->red_sums[(size_t)c],
                            h.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int q = 0; q < n; ++q) out[pos + q] = h[(size_t)n] - 2.0 * h[(size_t)q];
    pos += n;
  }
  return DMV_OK;
}

extern "C" int dmv_batch_copy_state(dmv_batch_t b, int32_t index, double* interleaved) {
  clear_error();
  if (!b || !interleaved || index < 0 || index >= b->count) return set_error(DMV_ERR_INVALID, "bad batch index");
  const int64_t N = int64_t(1) << b->n[(size_t)index];
  const char* src = static_cast<const char*>(b->arena) + (size_t)b->offsets[(size_t)index] * b->amp_size();
  if (b->precision == DMV_C128) {
    DMV_CUDA_TRY(cudaMemcpy(interleaved, src, (size_t)N * 16, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> f((size_t)N * 2);
    DMV_CUDA_TRY(cudaMemcpy(f.data(), src, (size_t)N * 8, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < f.size(); ++i) interleaved[i] = (double)f[i];
  }
  return DMV_OK;
}

extern "C" int dmv_batch_stats(dmv_batch_t b, int64_t* items, int64_t* passes, int64_t* ops, int32_t* grid,
                               double* last_ms) {
  clear_error();
  if (!b) return set_error(DMV_ERR_INVALID, "null batch");
  if (items) *items = b->num_items;
  if (passes) *passes = b->num_passes;
  if (ops) *ops = b->num_ops;
  if (grid) *grid = b->use_graph ? b->grid : -b->grid;  // negative: enqueued without a CUDA graph
  if (last_ms) *last_ms = b->last_ms;
  return DMV_OK;
}
