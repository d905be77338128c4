// Pauli-Z expectation for callers that cannot allocate device memory.
//
// dmv_expect_z computes its per-CTA partial sums in device buffers that the
// library allocates (and keeps) on the state. Some callers cannot let a
// library allocate: a serving process may hand out all device memory from
// its own pool up front, and cudaMalloc/cudaFree synchronise the device,
// which a latency-bound loop cannot afford. dmv_expect_z_noalloc performs
// the same reduction with its scratch in a fixed-size array compiled into
// this library instead.
//
// The scratch is a file-scope __device__ array: every GPU that loads the
// library holds it (332.5 KiB) until the process exits. Host code must not
// use the array's name as an address (on the host it is only a stand-in), so
// the first call on each device looks its device address up with
// cudaGetSymbolAddress, with that device current, and caches it. That first
// call may also load the library's device code onto the device. All calls
// share the one array: calls whose kernels overlap on the GPU (different
// streams, or different host threads on one device) race on it and must be
// serialised by the caller.
#include <mutex>

#include "complex_ops.cuh"
#include "internal.h"

namespace dmv {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaChunkBits = 13;     // 8192 amplitudes per chunk
constexpr int kNaRows = 32;          // (1 << kNaChunkBits) / kNaThreads
constexpr int kNaTotalThread = kNaThreads - 1;  // writes the CTA's total mass
static_assert((1 << kNaChunkBits) == kNaThreads * kNaRows, "a chunk is one element per thread and row");
static_assert(kNaThreads == 256 && kNaRows == 32, "bits 0-7 of an element index come from the thread, 8-12 from the row");
static_assert(kNaChunkBits < kNaTotalThread, "the total's thread must not be one of the per-bit threads");
constexpr int kNaMaxQubits = 34;
constexpr int kNaMaxCtas = 1216;     // grid cap, fixed so the scratch bound holds on any GPU
constexpr int kNaScratchDoubles = kNaMaxCtas * (kNaMaxQubits + 1);  // 42,560 doubles

static __device__ __align__(256) double g_noalloc_scratch[kNaScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_na_mu;
double* g_na_ptr[kMaxDevices] = {};

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename V>
__device__ __forceinline__ double na_prob(const V* a, int64_t i) {
  const double x = (double)a[i].x, y = (double)a[i].y;
  return fma(x, x, y * y);
}

// Same reduction as the library's chunk-mass kernel, without the per-chunk
// output: row b of `partial` (n+1 doubles) receives CTA b's mass of the
// indices with bit q set (q < n) and its total mass (index n). Every row
// below gridDim.x is written on every call, so nothing needs clearing.
template <typename V>
__global__ void __launch_bounds__(kNaThreads)
k_expect_z_noalloc(const V* __restrict__ a, int n, int chunk_bits, int64_t num_chunks, double* __restrict__ partial) {
  __shared__ double red[32];
  __shared__ double tsum[kNaThreads];
  __shared__ double rsum[5][kNaThreads];
  __shared__ double hi_acc[kNaMaxQubits];
  const int C = 1 << chunk_bits;
  if (threadIdx.x < kNaMaxQubits) hi_acc[threadIdx.x] = 0.;
  double v[kNaRows];
#pragma unroll
  for (int r = 0; r < kNaRows; ++r) v[r] = 0.;
  for (int64_t ch = blockIdx.x; ch < num_chunks; ch += gridDim.x) {
    const int64_t base = ch << chunk_bits;
    double mine = 0.;
#pragma unroll
    for (int r = 0; r < kNaRows; ++r) {
      const int e = threadIdx.x + kNaThreads * r;
      if (e < C) {
        const double p = na_prob(a, base + e);
        v[r] += p;
        mine += p;
      }
    }
    mine = na_warp_sum(mine);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mine;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.;
      for (int w = 0; w < kNaThreads / 32; ++w) tot += red[w];
      for (int j = 0; j < n - chunk_bits; ++j)
        if ((ch >> j) & 1) hi_acc[j] += tot;
    }
  }
  double T = 0.;
  double R[5] = {0., 0., 0., 0., 0.};
#pragma unroll
  for (int r = 0; r < kNaRows; ++r) {
    T += v[r];
#pragma unroll
    for (int j = 0; j < 5; ++j)
      if ((r >> j) & 1) R[j] += v[r];
  }
  tsum[threadIdx.x] = T;
#pragma unroll
  for (int j = 0; j < 5; ++j) rsum[j][threadIdx.x] = R[j];
  __syncthreads();
  double* out = partial + (int64_t)blockIdx.x * (n + 1);
  const int q = threadIdx.x;
  if (q < chunk_bits) {
    double acc = 0.;
    if (q < 8) {
      for (int t = 0; t < kNaThreads; ++t)
        if ((t >> q) & 1) acc += tsum[t];
    } else {
      for (int t = 0; t < kNaThreads; ++t) acc += rsum[q - 8][t];
    }
    out[q] = acc;
  } else if (q == kNaTotalThread) {
    double acc = 0.;
    for (int t = 0; t < kNaThreads; ++t) acc += tsum[t];
    out[n] = acc;
  }
  if (threadIdx.x == 0)
    for (int j = 0; j < n - chunk_bits; ++j) out[chunk_bits + j] = hi_acc[j];
}

// out[q] = total - 2 * mass(bit q set) = <Z_q>, out[n] = total; rows summed in CTA order.
__global__ void k_expect_z_noalloc_finish(const double* __restrict__ partial, int n, int rows, double* __restrict__ out) {
  __shared__ double total;
  if (threadIdx.x == 0) {
    double acc = 0.;
    for (int r = 0; r < rows; ++r) acc += partial[(int64_t)r * (n + 1) + n];
    total = acc;
    out[n] = acc;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    double acc = 0.;
    for (int r = 0; r < rows; ++r) acc += partial[(int64_t)r * (n + 1) + q];
    out[q] = total - 2.0 * acc;
  }
}

// Device address of the scratch array for the current device (looked up once).
int scratch_for_current_device(double** out) {
  int dev = 0;
  DMV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(DMV_ERR_INVALID, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    double* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return set_error(DMV_ERR_CUDA, "cudaGetSymbolAddress of the expectation scratch failed: %s",
                       cudaGetErrorString(e));
    }
    g_na_ptr[dev] = p;
  }
  *out = g_na_ptr[dev];
  return DMV_OK;
}

}  // namespace
}  // namespace dmv

using namespace dmv;

extern "C" int dmv_expect_z_noalloc(const void* amps, int32_t num_qubits, int32_t precision, double* out_device,
                                    void* stream) {
  clear_error();
  if (!amps || !out_device) return set_error(DMV_ERR_INVALID, "dmv_expect_z_noalloc: null amplitude or output pointer");
  if (num_qubits < 1 || num_qubits > kNaMaxQubits)
    return set_error(DMV_ERR_INVALID,
                     "dmv_expect_z_noalloc: num_qubits %d outside [1, %d] (its fixed scratch holds %d x %d partial sums)",
                     num_qubits, kNaMaxQubits, kNaMaxCtas, kNaMaxQubits + 1);
  if (precision != DMV_C128 && precision != DMV_C64)
    return set_error(DMV_ERR_INVALID, "dmv_expect_z_noalloc: unknown precision %d", precision);
  const int cb = num_qubits < kNaChunkBits ? num_qubits : kNaChunkBits;
  const int64_t num_chunks = int64_t(1) << (num_qubits - cb);
  const int grid = (int)(num_chunks < kNaMaxCtas ? num_chunks : kNaMaxCtas);
  if ((int64_t)grid * (num_qubits + 1) > kNaScratchDoubles)
    return set_error(DMV_ERR_INVALID, "dmv_expect_z_noalloc: %d x %d partial sums exceed the %d-double scratch", grid,
                     num_qubits + 1, kNaScratchDoubles);
  double* scratch = nullptr;
  DMV_TRY(scratch_for_current_device(&scratch));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == DMV_C128)
    k_expect_z_noalloc<double2><<<grid, kNaThreads, 0, st>>>(static_cast<const double2*>(amps), num_qubits, cb,
                                                              num_chunks, scratch);
  else
    k_expect_z_noalloc<float2><<<grid, kNaThreads, 0, st>>>(static_cast<const float2*>(amps), num_qubits, cb,
                                                             num_chunks, scratch);
  k_expect_z_noalloc_finish<<<1, 64, 0, st>>>(scratch, num_qubits, grid, out_device);
  count_launch(2);
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}
