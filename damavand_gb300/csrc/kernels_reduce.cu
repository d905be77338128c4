// Reductions over the statevector: probabilities, Pauli-Z expectations with
// per-chunk probability mass, inverse-CDF sampling (segment and chunk
// prefixes, a chunk guide table, one warp per sample), sampled expectation
// values counted on the device, inner products, the Z-observable scaling and
// the adjoint sweep step. All sums accumulate in FP64 (also for complex64
// storage) in a fixed order, so results are reproducible run to run.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "complex_ops.cuh"
#include "df.cuh"
#include "internal.h"
#include "policies.cuh"
#include "tma.cuh"

namespace dmv {

namespace {

constexpr int kRedThreads = 256;
constexpr int kMaxChunkBits = 13;  // 8192 amplitudes per chunk

int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum (all threads get the result). `red` has >= 32 doubles.
__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.;
  const int nw = (blockDim.x + 31) >> 5;
  if (warp == 0) {
    t = lane < nw ? red[lane] : 0.;
    t = warp_sum(t);
    if (lane == 0) red[0] = t;
  }
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

// Probability of element i from one of three sources.
template <int SRC>
__device__ __forceinline__ double prob_at(const void* src, int64_t i) {
  if constexpr (SRC == 0) return norm2(static_cast<const double2*>(src)[i]);
  else if constexpr (SRC == 1) return norm2(static_cast<const float2*>(src)[i]);
  else return static_cast<const double*>(src)[i];
}

template <int SRC>
__global__ void __launch_bounds__(kRedThreads)
k_probabilities(const void* src, double* __restrict__ out, int64_t N) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride)
    out[i] = prob_at<SRC>(src, i);
}

// ---------------------------------------------------------------------------
// Pauli-Z masses: per qubit q the probability mass of the indices with bit q
// set, and the total (<Z_q> = total - 2 mass_q), in FP32 pairs.
//
// On GB300 an FP64 reduction spends 4 FP64 operations per amplitude and runs
// at about a third of HBM speed (8.8 ms at 30 qubits against 2.5 ms for the
// read). Here every probability is formed
// and summed as an unevaluated pair of floats hi + lo: the components of a
// complex128 amplitude are split into FP32 pairs with integer operations
// (split_f64), x^2 is hi^2 exactly by FMA (TwoProd) plus the cross terms,
// and sums use Knuth's TwoSum with the error kept in lo and the pair
// renormalised (Fast2Sum) after each addition. Each accumulator holds about
// 46 significant bits: the probabilities' relative error is at most ~2^-45,
// and an accumulator of k additions drifts by at most ~k 2^-47 of its value
// (k <= 2^17 per accumulator at 34 qubits). Amplitudes below 2^-126 count as
// zero (FP32 range; their probabilities are below 2^-252). FP64 runs once per
// accumulator at the end.
// ---------------------------------------------------------------------------
struct F2 {
  float h, l;
};

__device__ __forceinline__ void f2_add(F2& a, float bh, float bl) {
  const float t = __fadd_rn(a.h, bh);  // TwoSum(a.h, bh) = t + e exactly
  const float z = __fsub_rn(t, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(t, z)), __fsub_rn(bh, z));
  const float c = __fadd_rn(a.l, __fadd_rn(e, bl));
  a.h = __fadd_rn(t, c);  // Fast2Sum(t, c): |t| >= |c|
  a.l = __fsub_rn(c, __fsub_rn(a.h, t));
}

// |x|^2 + |y|^2 of one amplitude as an FP32 pair.
template <int SRC>
__device__ __forceinline__ F2 f2_prob(const void* src, int64_t i) {
  float xh, xl, yh, yl;
  if constexpr (SRC == 0) {
    const double2 a = static_cast<const double2*>(src)[i];
    split_f64(a.x, xh, xl);
    split_f64(a.y, yh, yl);
  } else {
    const float2 a = static_cast<const float2*>(src)[i];
    xh = a.x; yh = a.y;
    xl = 0.f; yl = 0.f;
  }
  const float px = __fmul_rn(xh, xh), py = __fmul_rn(yh, yh);
  float ex = __fmaf_rn(xh, xh, -px);  // exact error of hi^2
  float ey = __fmaf_rn(yh, yh, -py);
  ex = __fmaf_rn(__fadd_rn(xh, xh), xl, ex);  // + 2 hi lo
  ey = __fmaf_rn(__fadd_rn(yh, yh), yl, ey);
  ex = __fmaf_rn(xl, xl, ex);  // + lo^2
  ey = __fmaf_rn(yl, yl, ey);
  F2 r{px, __fadd_rn(ex, ey)};
  f2_add(r, py, 0.f);
  return r;
}

__device__ __forceinline__ double f2_val(const F2& a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ F2 f2_warp_sum(F2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, v.h, o);
    const float l = __shfl_xor_sync(0xffffffffu, v.l, o);
    f2_add(v, h, l);
  }
  return v;
}

constexpr int kF2Rows = 16;  // chunk of kRedThreads x 16 = 4096 amplitudes
constexpr int kF2ChunkBits = 12;

// Register-fed mass pass (states below 12 qubits; k_chunk_mass_bulk above),
// for complex128 (SRC 0) and complex64 (SRC 1) amplitudes, with
// 2^chunk_bits-amplitude chunks (chunk_bits = min(n, 12)). Element e of a
// chunk is e = tid + 256 r; each thread keeps one accumulator per r across
// the chunks it visits, and thread 0 adds each chunk's total to the masses of
// the chunk-index bits. Per CTA: partial[cta * (n+1) + q] = mass with bit q
// set (q < n), partial[cta * (n+1) + n] = the total.
template <int SRC>
__global__ void __launch_bounds__(kRedThreads)
k_chunk_mass_f2(const void* src, int n, int chunk_bits, int64_t num_chunks, double* __restrict__ partial) {
  __shared__ F2 red[kRedThreads / 32];
  __shared__ double tsum[kRedThreads];
  __shared__ double rsum[4][kRedThreads];
  __shared__ double hi_acc[34];  // only thread 0 updates it
  const int C = 1 << chunk_bits;
  F2 v[kF2Rows];
#pragma unroll
  for (int r = 0; r < kF2Rows; ++r) v[r] = F2{0.f, 0.f};
  if (threadIdx.x < 34) hi_acc[threadIdx.x] = 0.;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t ch = blockIdx.x; ch < num_chunks; ch += gridDim.x) {
    const int64_t base = ch << chunk_bits;
    F2 mine{0.f, 0.f};
#pragma unroll
    for (int r = 0; r < kF2Rows; ++r) {
      const int e = threadIdx.x + kRedThreads * r;
      if (e < C) {
        const F2 p = f2_prob<SRC>(src, base + e);
        f2_add(v[r], p.h, p.l);
        f2_add(mine, p.h, p.l);
      }
    }
    mine = f2_warp_sum(mine);
    __syncthreads();
    if (lane == 0) red[warp] = mine;
    __syncthreads();
    if (threadIdx.x == 0) {
      F2 tot{0.f, 0.f};
      for (int w = 0; w < kRedThreads / 32; ++w) f2_add(tot, red[w].h, red[w].l);
      const double t = f2_val(tot);
      for (int j = 0; j < n - chunk_bits; ++j)
        if ((ch >> j) & 1) hi_acc[j] += t;
    }
  }
  // fold the rows in FP32 pairs (FP64 only for the five results)
  F2 T{0.f, 0.f};
  F2 R[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
  for (int r = 0; r < kF2Rows; ++r) {
    f2_add(T, v[r].h, v[r].l);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if ((r >> j) & 1) f2_add(R[j], v[r].h, v[r].l);
  }
  tsum[threadIdx.x] = f2_val(T);
#pragma unroll
  for (int j = 0; j < 4; ++j) rsum[j][threadIdx.x] = f2_val(R[j]);
  __syncthreads();
  double* out = partial + (int64_t)blockIdx.x * (n + 1);
  const int q = threadIdx.x;
  if (q < chunk_bits) {
    double acc = 0.;
    if (q < 8) {
      for (int t = 0; t < kRedThreads; ++t)
        if ((t >> q) & 1) acc += tsum[t];
    } else {
      for (int t = 0; t < kRedThreads; ++t) acc += rsum[q - 8][t];
    }
    out[q] = acc;
  } else if (q == kRedThreads - 1) {
    double acc = 0.;
    for (int t = 0; t < kRedThreads; ++t) acc += tsum[t];
    out[n] = acc;
  }
  if (threadIdx.x == 0)
    for (int j = 0; j < n - chunk_bits; ++j) out[chunk_bits + j] = hi_acc[j];
}
static_assert((1 << kF2ChunkBits) == kRedThreads * kF2Rows, "a chunk is one amplitude per thread and row");
static_assert(kF2ChunkBits < kRedThreads - 1, "the total's thread is not a per-bit thread");

// ---------------------------------------------------------------------------
// k_chunk_mass_bulk: the same pass for states of 12 or more qubits, with one
// CTA per SM and the chunks staged in shared memory by the copy engine.
//
// The register-fed pass above keeps too few loads in flight per SM for HBM
// speed (its grid sweep: two CTAs per SM ran at a quarter of HBM bandwidth,
// eight at about half). Here a producer warp starts one untiled bulk copy
// (cp.async.bulk) per 4096-amplitude chunk into a ring of three buffers, so
// up to three chunks (192 KB of complex128) are in flight whatever the
// register count. Sixteen summing warps share no per-chunk barrier: each
// releases a buffer on its "empty" mbarrier as soon as it has read its part,
// and keeps everything else (row sums, its share of the high-bit masses) in
// registers until the end, so a slow warp does not hold up the others. The
// arithmetic is about 60 operations per amplitude (split47 below, a TwoSum in
// place of a full pair addition for |x|^2 + |y|^2). Each summing thread owns 8
// amplitudes of a chunk (elements tid + 512 r): the rows give bits 9..11, the
// thread index bits 0..8, and each warp's chunk sum the bits above 11 (lane j
// of every warp accumulates bit 12 + j).
// ---------------------------------------------------------------------------
constexpr int kMbSumWarps = 16;
constexpr int kMbSumThreads = 32 * kMbSumWarps;  // 512
constexpr int kMbThreads = kMbSumThreads + 32;   // + the producer warp
constexpr int kMbRows = 8;                       // 4096 / 512
constexpr int kMbStages = 3;
constexpr int kMbChunkBits = 12;
constexpr uint32_t kMbDrainLimit = 1u << 22;
static_assert(kMbSumThreads * kMbRows == (1 << kMbChunkBits), "a chunk is one amplitude per thread and row");
static_assert(kMbChunkBits == kF2ChunkBits, "both passes use the same chunks");

template <int SRC>
struct MbAmp {
  using T = double2;
};
template <>
struct MbAmp<1> {
  using T = float2;
};
template <int SRC>
constexpr size_t mass_bulk_smem() {
  return (size_t)kMbStages * ((size_t)1 << kMbChunkBits) * sizeof(typename MbAmp<SRC>::T);
}
static_assert(mass_bulk_smem<1>() >= 4 * kMbSumThreads * sizeof(double) + kMbSumWarps * 32 * sizeof(double),
              "the final fold reuses the ring");

// x -> (hi, lo) for a probability: hi = x truncated to 24 significant bits,
// lo = the remaining 29 bits rounded to 23 (x keeps 47 bits: relative error
// <= 2^-47, unbiased). Integer operations and one FP32 subtraction: with
// P = sign(x) 2^(e-23), e = x's exponent, lo = float(bits(P) + m) - P, m the
// rounded remainder (a carry of m into P's exponent field is exact as well).
// |x| outside [2^-103, 2^128) gives (0, 0): such squares are below 2^-206.
__device__ __forceinline__ void split47(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int top = (unsigned int)(b >> 32), low = (unsigned int)b;
  // (top << 3) | (low >> 29): the low 9 exponent bits, then 23 mantissa bits.
  const unsigned int f = __funnelshift_r(low, top, 29);
  // + 0x40000000 = - (896 << 23) mod 2^32: bits 30..23 become e + 127.
  const unsigned int hb = ((f + 0x40000000u) & 0x7FFFFFFFu) | (top & 0x80000000u);
  const unsigned int pb = (hb & 0xFF800000u) - (23u << 23);
  const unsigned int m = ((low & 0x1FFFFFFFu) + 32u) >> 6;
  const bool ok = (top & 0x7FFFFFFFu) - (920u << 20) < (231u << 20);  // exponent field in [920, 1150]
  hi = ok ? __uint_as_float(hb) : 0.f;
  lo = ok ? __fsub_rn(__uint_as_float(pb + m), __uint_as_float(pb)) : 0.f;
}

// x^2 as hi^2 (rounded) + its error: the exact FMA residual plus
// lo (2 hi + lo). Relative error of the pair about 2^-46.
__device__ __forceinline__ void sq_pair(float h, float l, float& p, float& e) {
  p = __fmul_rn(h, h);
  e = __fmaf_rn(h, h, -p);
  e = __fmaf_rn(l, __fmaf_rn(h, 2.f, l), e);
}

template <int SRC>
__device__ __forceinline__ F2 mb_prob(const typename MbAmp<SRC>::T a) {
  float px, ex, py, ey;
  if constexpr (SRC == 0) {
    float xh, xl, yh, yl;
    split47(a.x, xh, xl);
    split47(a.y, yh, yl);
    sq_pair(xh, xl, px, ex);
    sq_pair(yh, yl, py, ey);
  } else {
    sq_pair(a.x, 0.f, px, ex);
    sq_pair(a.y, 0.f, py, ey);
  }
  const float t = __fadd_rn(px, py);  // TwoSum(px, py) = t + q exactly
  const float z = __fsub_rn(t, px);
  const float q = __fadd_rn(__fsub_rn(px, __fsub_rn(t, z)), __fsub_rn(py, z));
  return F2{t, __fadd_rn(q, __fadd_rn(ex, ey))};
}

// The ring of a bulk-staged pass: full[s] completes when chunk i (i % 3 == s)
// has landed (one arrival with its byte count), empty[s] when all summing
// warps have read it (one arrival per warp). Every wait is bounded; a wait
// that gives up sets *status to 1, and the party that gave up stops waiting
// from then on (the producer stops issuing), so every thread still reaches
// the closing barrier. The producer waits, bounded, for its last copies
// before it gets there, so none is in flight when the CTA ends.
struct BulkRing {
  uint64_t full[kMbStages];
  uint64_t empty[kMbStages];
};

__device__ __forceinline__ void ring_init(BulkRing& r) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kMbStages; ++s) {
      mbar_init(&r.full[s], 1);
      mbar_init(&r.empty[s], kMbSumWarps);
    }
    fence_mbar_init();
  }
  __syncthreads();
}

// Producer warp, one lane: chunk i (global chunk blockIdx.x + i * gridDim.x)
// into buffer i % 3 once the summing warps have released chunk i - 3.
template <typename A>
__device__ void ring_produce(BulkRing& r, A* ring, const A* gsrc, int64_t count, uint32_t wait_limit,
                             int* status) {
  constexpr int C = 1 << kMbChunkBits;
  constexpr uint32_t kBytes = (uint32_t)(C * sizeof(A));
  int64_t issued = 0;
  for (int64_t i = 0; i < count; ++i) {
    const int s = (int)(i % kMbStages);
    if (i >= kMbStages && !mbar_wait(&r.empty[s], (uint32_t)((i / kMbStages - 1) & 1), wait_limit)) {
      atomicExch(status, 1);
      break;
    }
    mbar_arrive_expect_tx(&r.full[s], kBytes);
    bulk_load(ring + (size_t)s * C, gsrc + ((blockIdx.x + i * (int64_t)gridDim.x) << kMbChunkBits), kBytes,
              &r.full[s]);
    issued = i + 1;
  }
  // Chunks before issued - 3 were released, so read, so landed.
  for (int64_t j = issued > kMbStages ? issued - kMbStages : 0; j < issued; ++j)
    mbar_wait(&r.full[j % kMbStages], (uint32_t)((j / kMbStages) & 1), kMbDrainLimit);
}

// Summing warp: waits for chunk i; false (and *status set) if the wait gave up.
__device__ __forceinline__ bool ring_wait_full(BulkRing& r, int64_t i, uint32_t wait_limit, int* status) {
  const bool ok = __all_sync(0xffffffffu,
                             mbar_wait(&r.full[i % kMbStages], (uint32_t)((i / kMbStages) & 1), wait_limit));
  if (!ok && (threadIdx.x & 31) == 0) atomicExch(status, 1);
  return ok;
}

// Summing warp: its reads of chunk i are done.
__device__ __forceinline__ void ring_release(BulkRing& r, int64_t i) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(&r.empty[i % kMbStages]);
}

// Outputs as k_chunk_mass_f2 with chunk_bits = 12, except that no per-chunk
// masses are written (nothing reads them): per CTA the n + 1 sums in
// `partial`. The grid is at most num_chunks; CTA b takes chunks b, b + grid, ...
template <int SRC>
__global__ void __launch_bounds__(kMbThreads, 1)
k_chunk_mass_bulk(const void* src, int n, int64_t num_chunks, double* __restrict__ partial, uint32_t wait_limit,
                  int* __restrict__ status) {
  using A = typename MbAmp<SRC>::T;
  constexpr int C = 1 << kMbChunkBits;
  extern __shared__ __align__(128) unsigned char mb_smem[];
  A* ring = reinterpret_cast<A*>(mb_smem);
  __shared__ __align__(8) BulkRing rb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nh = n - kMbChunkBits;  // <= 22 (34 qubits): one lane per bit
  const int64_t G = gridDim.x;
  const int64_t count = (num_chunks - blockIdx.x + G - 1) / G;
  ring_init(rb);
  F2 v[kMbRows];
#pragma unroll
  for (int r = 0; r < kMbRows; ++r) v[r] = F2{0.f, 0.f};
  F2 hacc{0.f, 0.f};
  if (warp == kMbSumWarps) {
    if (lane == 0) ring_produce(rb, ring, static_cast<const A*>(src), count, wait_limit, status);
  } else {
    for (int64_t i = 0; i < count; ++i) {
      if (!ring_wait_full(rb, i, wait_limit, status)) break;
      const A* buf = ring + (size_t)(i % kMbStages) * C;
      A a[kMbRows];
#pragma unroll
      for (int r = 0; r < kMbRows; ++r) a[r] = buf[tid + kMbSumThreads * r];
      ring_release(rb, i);
      F2 p[kMbRows];
#pragma unroll
      for (int r = 0; r < kMbRows; ++r) {
        p[r] = mb_prob<SRC>(a[r]);
        f2_add(v[r], p[r].h, p[r].l);
      }
#pragma unroll
      for (int w = 1; w < kMbRows; w <<= 1)
#pragma unroll
        for (int r = 0; r < kMbRows; r += 2 * w) f2_add(p[r], p[r + w].h, p[r + w].l);
      F2 ws = f2_warp_sum(p[0]);
      ws.h = __shfl_sync(0xffffffffu, ws.h, 0);  // every lane adds the same value
      ws.l = __shfl_sync(0xffffffffu, ws.l, 0);
      const int64_t ch = blockIdx.x + i * G;
      if (lane < nh && ((ch >> lane) & 1)) f2_add(hacc, ws.h, ws.l);
    }
  }
  __syncthreads();  // every copy has landed: the ring is free for the fold
  // Rows folded in FP32 pairs; FP64 for the per-thread and per-warp results.
  double* tsum = reinterpret_cast<double*>(mb_smem);
  double* rsum = tsum + kMbSumThreads;         // [3][kMbSumThreads]
  double* hsum = rsum + 3 * kMbSumThreads;     // [kMbSumWarps][32]
  if (warp < kMbSumWarps) {
    F2 T{0.f, 0.f};
    F2 R[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
    for (int r = 0; r < kMbRows; ++r) {
      f2_add(T, v[r].h, v[r].l);
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if ((r >> j) & 1) f2_add(R[j], v[r].h, v[r].l);
    }
    tsum[tid] = f2_val(T);
#pragma unroll
    for (int j = 0; j < 3; ++j) rsum[j * kMbSumThreads + tid] = f2_val(R[j]);
    hsum[warp * 32 + lane] = f2_val(hacc);
  }
  __syncthreads();
  double* out = partial + (int64_t)blockIdx.x * (n + 1);
  if (tid < kMbChunkBits) {
    double acc = 0.;
    if (tid < 9) {
      for (int t = 0; t < kMbSumThreads; ++t)
        if ((t >> tid) & 1) acc += tsum[t];
    } else {
      for (int t = 0; t < kMbSumThreads; ++t) acc += rsum[(tid - 9) * kMbSumThreads + t];
    }
    out[tid] = acc;
  } else if (tid >= 32 && tid < 32 + nh) {
    double acc = 0.;
    for (int w = 0; w < kMbSumWarps; ++w) acc += hsum[w * 32 + (tid - 32)];
    out[kMbChunkBits + (tid - 32)] = acc;
  } else if (tid == kMbThreads - 1) {
    double acc = 0.;
    for (int t = 0; t < kMbSumThreads; ++t) acc += tsum[t];
    out[n] = acc;
  }
}

// The sampler's segment masses for states of 12 or more qubits, staged as in
// k_chunk_mass_bulk: 4096-amplitude chunks of 16 segments of 256; summing
// warp w sums segment w of each chunk (lane l: elements l + 32 r) and writes
// it to seg[c * 16 + w]. k_segment_scan then turns each chunk's 16 masses
// into running sums and the chunk mass.
constexpr int kSpSegBits = 8;
constexpr int kSpSegsPerChunk = 1 << (kMbChunkBits - kSpSegBits);
static_assert(kSpSegsPerChunk == kMbSumWarps, "one summing warp per segment");

template <int SRC>
__global__ void __launch_bounds__(kMbThreads, 1)
k_segment_mass_bulk(const void* src, int64_t num_chunks, double* __restrict__ seg, uint32_t wait_limit,
                    int* __restrict__ status) {
  using A = typename MbAmp<SRC>::T;
  constexpr int C = 1 << kMbChunkBits;
  extern __shared__ __align__(128) unsigned char mb_smem[];
  A* ring = reinterpret_cast<A*>(mb_smem);
  __shared__ __align__(8) BulkRing rb;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t G = gridDim.x;
  const int64_t count = (num_chunks - blockIdx.x + G - 1) / G;
  ring_init(rb);
  if (warp == kMbSumWarps) {
    if (lane == 0) ring_produce(rb, ring, static_cast<const A*>(src), count, wait_limit, status);
  } else {
    for (int64_t i = 0; i < count; ++i) {
      if (!ring_wait_full(rb, i, wait_limit, status)) break;
      const A* buf = ring + (size_t)(i % kMbStages) * C + (warp << kSpSegBits);
      A a[kMbRows];
#pragma unroll
      for (int r = 0; r < kMbRows; ++r) a[r] = buf[lane + 32 * r];
      ring_release(rb, i);
      F2 acc = mb_prob<SRC>(a[0]);
#pragma unroll
      for (int r = 1; r < kMbRows; ++r) {
        const F2 p = mb_prob<SRC>(a[r]);
        f2_add(acc, p.h, p.l);
      }
      acc = f2_warp_sum(acc);
      if (lane == 0) seg[(blockIdx.x + i * G) * kSpSegsPerChunk + warp] = f2_val(acc);
    }
  }
  __syncthreads();  // the producer has seen its last copies land
}

// In place, per chunk c: seg[c * 16 + j] <- seg[c * 16] + ... + seg[c * 16 + j]
// (FP64, in segment order), chunk_mass[c] <- the last of them.
__global__ void k_segment_scan(double* __restrict__ seg, int64_t num_chunks, double* __restrict__ chunk_mass) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= num_chunks) return;
  double* p = seg + c * kSpSegsPerChunk;
  double run = 0.;
#pragma unroll
  for (int j = 0; j < kSpSegsPerChunk; ++j) {
    run += p[j];
    p[j] = run;
  }
  chunk_mass[c] = run;
}

// Sum the per-CTA partials in CTA order.
__global__ void k_reduce_partials(const double* __restrict__ partial, int width, int rows,
                                  double* __restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= width) return;
  double acc = 0.;
  for (int r = 0; r < rows; ++r) acc += partial[(int64_t)r * width + q];
  out[q] = acc;
}

// out[r] = sum_c in[r * cols + c], in column order.
__global__ void k_reduce_rows(const double* __restrict__ in, int64_t rows, int cols, double* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double acc = 0.;
  for (int c = 0; c < cols; ++c) acc += in[r * cols + c];
  out[r] = acc;
}

// Inclusive prefix of the chunk masses (one CTA, fixed order).
__global__ void __launch_bounds__(1024)
k_scan_chunks(const double* __restrict__ mass, int64_t num_chunks, double* __restrict__ incl) {
  __shared__ double seg[1024];
  const int64_t per = (num_chunks + blockDim.x - 1) / blockDim.x;
  const int64_t b = (int64_t)threadIdx.x * per;
  const int64_t e = min(num_chunks, b + per);
  double s = 0.;
  for (int64_t i = b; i < e; ++i) s += mass[i];
  seg[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {  // 1024 serial adds: negligible next to the pass over HBM
    double run = 0.;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const double x = seg[t];
      seg[t] = run;
      run += x;
    }
  }
  __syncthreads();
  double run = seg[threadIdx.x];
  for (int64_t i = b; i < e; ++i) {
    run += mass[i];
    incl[i] = run;
  }
}

// Sampling works on segments of 2^seg_bits amplitudes (at most 256) inside
// chunks of 2^chunk_bits (at most 8192: at most 32 segments per chunk). Lane
// l of a segment's warp holds elements l*E .. l*E+E-1, E = 2^(seg_bits-5)
// (one element, and idle lanes, below 32 amplitudes).
__device__ __forceinline__ int seg_lane_elems(int seg_bits) { return seg_bits >= 5 ? 1 << (seg_bits - 5) : 1; }

// Per chunk c: seg_incl[c * spc + j] = t_0 + ... + t_j (in segment order),
// t_j the probability mass of segment j, and chunk_mass[c] = the chunk's last
// seg_incl. One warp per chunk; lane l sums elements l, l + 32, ... of a
// segment (coalesced loads), then a shuffle tree gives t_j to every lane.
// acc + |a_i|^2 as two chained FP64 multiply-adds (the square is not rounded
// on its own): the FP64 pipe, not HBM, bounds a pass over the state.
template <int SRC>
__device__ __forceinline__ double prob_acc(const void* src, int64_t i, double acc) {
  if constexpr (SRC == 0) {
    const double2 v = static_cast<const double2*>(src)[i];
    return fma(v.y, v.y, fma(v.x, v.x, acc));
  } else if constexpr (SRC == 1) {
    const float2 v = static_cast<const float2*>(src)[i];
    return fma((double)v.y, (double)v.y, fma((double)v.x, (double)v.x, acc));
  } else {
    return acc + static_cast<const double*>(src)[i];
  }
}

template <int SRC>
__global__ void __launch_bounds__(kRedThreads)
k_segment_prefix(const void* src, int seg_bits, int chunk_bits, int64_t num_chunks, double* __restrict__ seg_incl,
                 double* __restrict__ chunk_mass) {
  const int lane = threadIdx.x & 31;
  const int S = 1 << seg_bits, spc = 1 << (chunk_bits - seg_bits);
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < num_chunks; c += nwarps) {
    double run = 0.;
    for (int j = 0; j < spc; ++j) {
      const int64_t base = (c << chunk_bits) + ((int64_t)j << seg_bits);
      double ls = 0.;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        if (lane + 32 * e < S) ls = prob_acc<SRC>(src, base + lane + 32 * e, ls);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, off);
      run += ls;
      if (lane == 0) seg_incl[c * spc + j] = run;
    }
    if (lane == 0) chunk_mass[c] = run;
  }
}

// k_segment_prefix for amplitudes (SRC 0 complex128, 1 complex64) in FP32
// pairs: the same outputs, with the probabilities formed and summed as in
// k_chunk_mass_f2 (each segment sum and running prefix carries ~46 bits; the
// prefixes are written as FP64). Dyadic probabilities stay exact.
template <int SRC>
__global__ void __launch_bounds__(kRedThreads)
k_segment_prefix_f2(const void* src, int seg_bits, int chunk_bits, int64_t num_chunks, double* __restrict__ seg_incl,
                    double* __restrict__ chunk_mass) {
  const int lane = threadIdx.x & 31;
  const int S = 1 << seg_bits, spc = 1 << (chunk_bits - seg_bits);
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < num_chunks; c += nwarps) {
    F2 run{0.f, 0.f};
    for (int j = 0; j < spc; ++j) {
      const int64_t base = (c << chunk_bits) + ((int64_t)j << seg_bits);
      F2 ls{0.f, 0.f};
#pragma unroll
      for (int e = 0; e < 8; ++e)
        if (lane + 32 * e < S) {
          const F2 p = f2_prob<SRC>(src, base + lane + 32 * e);
          f2_add(ls, p.h, p.l);
        }
      ls = f2_warp_sum(ls);
      f2_add(run, ls.h, ls.l);
      if (lane == 0) seg_incl[c * spc + j] = f2_val(run);
    }
    if (lane == 0) chunk_mass[c] = f2_val(run);
  }
}

// Guide table of the chunk prefixes: guide[b] = least chunk c with
// incl[c] >= b * (total / M) for b < M, guide[M] = the last chunk. A value
// xsi with b * step <= xsi < (b + 1) * step has its chunk in
// [guide[b], guide[b + 1]] (the prefixes do not decrease).
__global__ void k_chunk_guide(const double* __restrict__ incl, int64_t num_chunks, int64_t M,
                              int32_t* __restrict__ guide) {
  const double step = incl[num_chunks - 1] / (double)M;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= M; b += stride) {
    if (b == M) {
      guide[b] = (int32_t)(num_chunks - 1);
      continue;
    }
    const double t = (double)b * step;
    int64_t lo = 0, hi = num_chunks - 1;
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if (t <= incl[mid]) hi = mid;
      else lo = mid + 1;
    }
    guide[b] = (int32_t)lo;
  }
}

// One warp per sample: the least index with u*total <= cdf(index), the rule
// of src/utils.rs:258-277 (cdf(index) = p_0 + ... + p_index), through the
// prefix levels: the chunk by binary search on the chunk prefixes, the segment
// by a ballot over the chunk's segment prefixes, the element by a scan of the
// segment (lane sums, a shuffle scan, then each lane's own elements in order).
// Where rounding between the levels leaves no element of the chosen segment
// reaching u*total, the segment's last element of nonzero probability is taken
// (the chosen segment has nonzero mass, so one exists).
template <int SRC>
__global__ void __launch_bounds__(kRedThreads)
k_sample_warp(const void* src, int seg_bits, int chunk_bits, int64_t num_chunks, const double* __restrict__ chunk_incl,
              const int32_t* __restrict__ guide, const double* __restrict__ seg_incl,
              const double* __restrict__ uniforms, int64_t k, uint64_t* __restrict__ samples) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int S = 1 << seg_bits, E = seg_lane_elems(seg_bits), spc = 1 << (chunk_bits - seg_bits);
  const double total = chunk_incl[num_chunks - 1];
  const int64_t M = num_chunks;  // guide buckets
  const double step = total / (double)M;
  for (int64_t s = warp0; s < k; s += nwarps) {
    const double xsi = uniforms[s] * total;
    if (!(xsi > 0.)) {  // xsi == 0 matches cdf[0] = 0: the reference returns 0 - 1
      if (lane == 0) samples[s] = ~uint64_t(0);
      continue;
    }
    // bucket b with b * step <= xsi < (b + 1) * step (the products as the guide
    // table computed them), then the least chunk whose inclusive mass
    // reaches xsi, between guide[b] and guide[b + 1]
    int64_t b = (int64_t)(xsi / step);
    b = b < 0 ? 0 : (b >= M ? M - 1 : b);
    while (b > 0 && (double)b * step > xsi) --b;
    while (b + 1 < M && (double)(b + 1) * step <= xsi) ++b;
    int64_t lo = guide[b], hi = guide[b + 1];
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if (xsi <= chunk_incl[mid]) hi = mid;
      else lo = mid + 1;
    }
    const double before = lo > 0 ? chunk_incl[lo - 1] : 0.;
    const double* sp = seg_incl + lo * spc;
    const unsigned segs = __ballot_sync(0xffffffffu, lane < spc && xsi <= before + sp[lane < spc ? lane : 0]);
    const int sg = segs ? __ffs((int)segs) - 1 : spc - 1;
    const double sbefore = sg > 0 ? before + sp[sg - 1] : before;
    const int64_t base = ((lo * spc + sg) << seg_bits) + (int64_t)lane * E;
    const int mine = lane * E < S ? E : 0;
    double p[8];
    double ls = 0.;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      p[e] = e < mine ? prob_at<SRC>(src, base + e) : 0.;
      ls += p[e];
    }
    double incl = ls;  // inclusive scan of the lane sums
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += t;
    }
    const double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    double run = sbefore + (lane > 0 ? excl : 0.);
    int hit = -1, last_nz = -1;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      if (e < mine) {
        run += p[e];
        if (p[e] > 0.) last_nz = e;
        if (hit < 0 && xsi <= run) hit = e;
      }
    }
    const unsigned hits = __ballot_sync(0xffffffffu, hit >= 0);
    const int64_t seg_base = (lo * spc + sg) << seg_bits;
    if (hits) {
      const int l = __ffs((int)hits) - 1;
      const int e = __shfl_sync(0xffffffffu, hit, l);
      if (lane == 0) samples[s] = (uint64_t)(seg_base + (int64_t)l * E + e);
    } else {
      const unsigned nz = __ballot_sync(0xffffffffu, last_nz >= 0);
      const int l = nz ? 31 - __clz((int)nz) : -1;
      const int e = __shfl_sync(0xffffffffu, last_nz, l >= 0 ? l : 0);
      if (lane == 0) samples[s] = (uint64_t)(l >= 0 ? seg_base + (int64_t)l * E + e : seg_base + S - 1);
    }
  }
}

// Uniform i of the seeded device stream: SplitMix64 (Steele, Lea and Flood,
// "Fast splittable pseudorandom number generators", OOPSLA 2014) of the
// counter state seed + (i + 1) * 0x9E3779B97F4A7C15, its top 53 bits scaled
// by 2^-53, so every value lies in [0, 1).
__device__ __forceinline__ double splitmix_uniform(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * 0x1.0p-53;
}

__global__ void k_uniforms(uint64_t seed, int64_t first, int64_t count, double* __restrict__ u) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    u[i] = splitmix_uniform(seed, (uint64_t)(first + i));
}

// counts[b] += number of samples with bit b set, b = 0 .. 63 (a sample of
// ~0, the reference's 0 - 1, has every bit set). Each warp takes 32 samples
// at a time and one ballot per bit; lane b keeps the counts of bits b and
// b + 32. Integer atomics: the totals do not depend on the order.
__global__ void __launch_bounds__(kRedThreads)
k_count_bits(const uint64_t* __restrict__ samples, int64_t k, unsigned long long* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  unsigned long long lo = 0, hi = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < k; i0 += stride) {
    const int64_t i = i0 + lane;
    const uint64_t x = i < k ? samples[i] : 0ull;  // lanes past the end set no bit
#pragma unroll
    for (int b = 0; b < 32; ++b) {
      const unsigned bl = __ballot_sync(0xffffffffu, (unsigned)(x >> b) & 1u);
      const unsigned bh = __ballot_sync(0xffffffffu, (unsigned)(x >> (b + 32)) & 1u);
      if (lane == b) {
        lo += (unsigned)__popc(bl);
        hi += (unsigned)__popc(bh);
      }
    }
  }
  if (lo) atomicAdd(&counts[lane], lo);
  if (hi) atomicAdd(&counts[lane + 32], hi);
}

template <typename V>
__global__ void __launch_bounds__(kRedThreads)
k_inner(const V* __restrict__ a, const V* __restrict__ b, int64_t N, double* __restrict__ partial) {
  __shared__ double red[32];
  double re = 0., im = 0.;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    const double ar = a[i].x, ai = a[i].y, br = b[i].x, bi = b[i].y;
    re = fma(ar, br, fma(ai, bi, re));
    im = fma(ar, bi, fma(-ai, br, im));
  }
  re = block_sum(re, red);
  im = block_sum(im, red);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = re;
    partial[2 * blockIdx.x + 1] = im;
  }
}

// dst_i = d(i) * src_i with d(i) = sum_q w_q (1 - 2 bit_q(i)), from four
// 1024-entry tables over 10-bit index fields.
template <typename V>
__global__ void __launch_bounds__(kRedThreads)
k_scale_z(V* __restrict__ dst, const V* __restrict__ src, int64_t N, const double* __restrict__ tables) {
  __shared__ double tab[4 * 1024];
  for (int i = threadIdx.x; i < 4 * 1024; i += blockDim.x) tab[i] = tables[i];
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
    const double d = tab[i & 1023] + tab[1024 + ((i >> 10) & 1023)] + tab[2048 + ((i >> 20) & 1023)] +
                     tab[3072 + ((i >> 30) & 1023)];
    V v = src[i];
    v.x = (decltype(v.x))((double)v.x * d);
    v.y = (decltype(v.y))((double)v.y * d);
    dst[i] = v;
  }
}

// Im <l| P |p> over one pair (P the generator: 1 X, 2 Y, 3 Z) as a
// compensated dot product of FP32 pairs (float4: re hi, re lo, im hi, im lo),
// pre-update values.
__device__ __forceinline__ F2 df_generator_term(int gen, const float4& p0, const float4& p1, const float4& l0,
                                                const float4& l1) {
  DFAcc a;
  if (gen == 1) {  // l0r p1i - l0i p1r + l1r p0i - l1i p0r
    df_first(a, l0.x, l0.y, p1.z, p1.w);
    df_add(a, -l0.z, -l0.w, p1.x, p1.y);
    df_add(a, l1.x, l1.y, p0.z, p0.w);
    df_add(a, -l1.z, -l1.w, p0.x, p0.y);
  } else if (gen == 2) {  // -l0r p1r - l0i p1i + l1r p0r + l1i p0i
    df_first(a, -l0.x, -l0.y, p1.x, p1.y);
    df_add(a, -l0.z, -l0.w, p1.z, p1.w);
    df_add(a, l1.x, l1.y, p0.x, p0.y);
    df_add(a, l1.z, l1.w, p0.z, p0.w);
  } else {  // l0r p0i - l0i p0r - l1r p1i + l1i p1r
    df_first(a, l0.x, l0.y, p0.z, p0.w);
    df_add(a, -l0.z, -l0.w, p0.x, p0.y);
    df_add(a, -l1.x, -l1.y, p1.z, p1.w);
    df_add(a, l1.z, l1.w, p1.x, p1.y);
  }
  F2 r;
  df_finish(a, r.h, r.l);
  return r;
}

// In place: complex128 amplitudes -> the FP32-pair form (float4: re hi, re
// lo, im hi, im lo; 16 bytes, like the double2 it replaces).
__global__ void k_df_pack(double2* __restrict__ v, int64_t N) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride)
    reinterpret_cast<float4*>(v)[i] = df_from_double2(v[i]);
}

// One step of the adjoint sweep for gate U (op holds U^dagger):
//   grad += Im <lam| P |psi>   (P the rotation's generator, pre-update values)
//   psi <- U^dagger psi, lam <- U^dagger lam.
// The state updates use the state's arithmetic policy (FP64, FP32, FP32-pair,
// int64 block fixed point). The gradient term is accumulated in FP64 from the
// loaded values, except under FP32-pair arithmetic, where it is a compensated
// FP32-pair dot product summed in FP32 pairs (FP64 once per thread): six FP64
// operations per pair would otherwise cost as much as the pass's HBM traffic.
// DF_RAW (FP32-pair only): psi and lam hold the FP32-pair form (k_df_pack)
// and keep it, so no step converts (the conversions' integer work made the
// step ALU-bound).
template <typename P, bool DF_RAW = false>
__global__ void __launch_bounds__(kRedThreads)
k_adjoint_step(typename P::G* __restrict__ psi, typename P::G* __restrict__ lam,
               int64_t num_pairs, Op op, int apply, double* __restrict__ partial) {
  static_assert(!DF_RAW || std::is_same<P, PolDF>::value, "the raw pair form is FP32-pair arithmetic's");
  using V = typename P::G;
  __shared__ double red[32];
  const typename P::Mat m = P::dmat(op);
  const int t = op.target;
  const bool ctrl = op.ctrl_kind != CTRL_NONE && op.ctrl >= 0;
  const int c = op.ctrl;
  const int lo = ctrl ? min(t, c) : t, hi = ctrl ? max(t, c) : t;
  const int gen = op.generator;
  double acc = 0.;
  F2 facc{0.f, 0.f};  // FP32-pair arithmetic's gradient sum
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < num_pairs; j += stride) {
    int64_t i0 = ctrl ? (insert_zero(insert_zero(j, lo), hi) | (int64_t(1) << c)) : insert_zero(j, t);
    const int64_t i1 = i0 | (int64_t(1) << t);
    if constexpr (std::is_same<P, PolDF>::value) {
      float4 q0, q1, m0, m1;
      if constexpr (DF_RAW) {
        float4* pf = reinterpret_cast<float4*>(psi);
        float4* lf = reinterpret_cast<float4*>(lam);
        q0 = pf[i0]; q1 = pf[i1]; m0 = lf[i0]; m1 = lf[i1];
      } else {
        q0 = P::in(psi[i0]); q1 = P::in(psi[i1]); m0 = P::in(lam[i0]); m1 = P::in(lam[i1]);
      }
      if (gen != 0) {
        const F2 g = df_generator_term(gen, q0, q1, m0, m1);
        f2_add(facc, g.h, g.l);
      }
      if (apply) {
        apply_dyn<P>(op.cls, m, q0, q1);
        apply_dyn<P>(op.cls, m, m0, m1);
        if constexpr (DF_RAW) {
          float4* pf = reinterpret_cast<float4*>(psi);
          float4* lf = reinterpret_cast<float4*>(lam);
          pf[i0] = q0; pf[i1] = q1; lf[i0] = m0; lf[i1] = m1;
        } else {
          psi[i0] = P::out(q0); psi[i1] = P::out(q1);
          lam[i0] = P::out(m0); lam[i1] = P::out(m1);
        }
      }
      continue;
    }
    V p0 = psi[i0], p1 = psi[i1], l0 = lam[i0], l1 = lam[i1];
    if (gen != 0) {
      const double p0r = p0.x, p0i = p0.y, p1r = p1.x, p1i = p1.y;
      const double l0r = l0.x, l0i = l0.y, l1r = l1.x, l1i = l1.y;
      if (gen == 1) {        // X: Im(l0* p1) + Im(l1* p0)
        acc += fma(l0r, p1i, -l0i * p1r) + fma(l1r, p0i, -l1i * p0r);
      } else if (gen == 2) { // Y: -Re(l0* p1) + Re(l1* p0)
        acc += -fma(l0r, p1r, l0i * p1i) + fma(l1r, p0r, l1i * p0i);
      } else {               // Z: Im(l0* p0) - Im(l1* p1)
        acc += fma(l0r, p0i, -l0i * p0r) - fma(l1r, p1i, -l1i * p1r);
      }
    }
    if (apply) {
      if constexpr (P::kBlockScaled) {  // each pair is its own block
        const int ep = P::pair_exponent(p0, p1), el = P::pair_exponent(l0, l1);
        typename P::T q0 = P::in(p0, ep), q1 = P::in(p1, ep), m0 = P::in(l0, el), m1 = P::in(l1, el);
        apply_dyn<P>(op.cls, m, q0, q1);
        apply_dyn<P>(op.cls, m, m0, m1);
        psi[i0] = P::out(q0, ep); psi[i1] = P::out(q1, ep);
        lam[i0] = P::out(m0, el); lam[i1] = P::out(m1, el);
      } else {
        typename P::T q0 = P::in(p0), q1 = P::in(p1), m0 = P::in(l0), m1 = P::in(l1);
        apply_dyn<P>(op.cls, m, q0, q1);
        apply_dyn<P>(op.cls, m, m0, m1);
        psi[i0] = P::out(q0); psi[i1] = P::out(q1);
        lam[i0] = P::out(m0); lam[i1] = P::out(m1);
      }
    }
  }
  if (gen != 0) {
    if constexpr (std::is_same<P, PolDF>::value) acc = f2_val(facc);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
  }
}

// ---------------------------------------------------------------------------
// Fused adjoint sweep in FP32-pair arithmetic: one launch per window of the
// reversed gate list (the forward planner's windows, gates unmerged, each op
// tagged with its parameter slot and generator). A CTA stages the tile of psi
// and the tile of lambda (the same 2^k local indices, FP32-pair form, 2 x 64
// KB), then runs the window's ops in order: for a rotation, every thread first
// adds Im <lam| P |psi> over its pairs (pre-update values) to its FP32-pair
// sum, folded per warp into a per-op, per-warp slot in shared memory; then the
// pair updates of both tiles. The tiles go back to HBM once per window (4S
// bytes per window instead of per gate). Reordering inside a window only
// moves gates past gates on other qubits, which leaves every Im <lam| P |psi>
// unchanged (V^dagger P V = P for V on other qubits).
// ---------------------------------------------------------------------------
constexpr int kAdjThreads = kTileThreads;  // 512
constexpr int kAdjWarps = kAdjThreads / 32;
constexpr int kAdjMaxOps = 256;  // ops per launch (a longer window runs as several launches)

struct AdjWindowParams {
  int32_t k, low, nh, num_ops;
  int32_t high[16];
  int64_t num_tiles;
  const Op* ops;
  double* partial;  // partial[param * cols + cta]
  int64_t cols;
};

template <int CLS>
__device__ __forceinline__ void adj_tile_op(float4* ps, float4* la, int T, const Op& op, F2& g) {
  const DFMat m = PolDF::dmat(op);
  const int t = op.target, gen = op.generator;
  const bool lctrl = op.ctrl_kind == CTRL_LOCAL;
  const int c = op.ctrl;
  const int lo = lctrl ? min(t, c) : t, hi = lctrl ? max(t, c) : t;
  const int pairs = lctrl ? (T >> 2) : (T >> 1);
  for (int q = threadIdx.x; q < pairs; q += kAdjThreads) {
    const uint32_t l0 = lctrl ? (insert_zero32(insert_zero32((uint32_t)q, lo), hi) | (1u << c))
                              : insert_zero32((uint32_t)q, t);
    const uint32_t l1 = l0 | (1u << t);
    float4 p0 = ps[l0], p1 = ps[l1], m0 = la[l0], m1 = la[l1];
    if (gen != 0) {
      const F2 d = df_generator_term(gen, p0, p1, m0, m1);
      f2_add(g, d.h, d.l);
    }
    PolDF::template apply<CLS>(m, p0, p1);
    PolDF::template apply<CLS>(m, m0, m1);
    ps[l0] = p0; ps[l1] = p1;
    la[l0] = m0; la[l1] = m1;
  }
}

__global__ void __launch_bounds__(kAdjThreads, 1)
k_adjoint_window(float4* __restrict__ psi, float4* __restrict__ lam, const AdjWindowParams p) {
  extern __shared__ __align__(16) unsigned char adj_smem[];
  const int T = 1 << p.k;
  float4* ps = reinterpret_cast<float4*>(adj_smem);
  float4* la = ps + T;
  F2* acc = reinterpret_cast<F2*>(la + T);  // [num_ops][kAdjWarps]
  __shared__ int64_t s_slot[kMaxSlots];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < p.num_ops * kAdjWarps; i += kAdjThreads) acc[i] = F2{0.f, 0.f};
  const int64_t t_off = tile_thread_offset(p.low, p.nh, p.high);
  tile_slot_offsets(p.low, p.nh, p.high, (T + kTileThreads - 1) >> kTileThreadBits, s_slot);
  __syncthreads();
  for (int64_t tix = blockIdx.x; tix < p.num_tiles; tix += gridDim.x) {
    int64_t base = tix << p.low;
    for (int i = 0; i < p.nh; ++i) base = insert_zero(base, p.high[i]);
    tile_load<PolRaw<PolDF>, false>(ps, psi, base, T, t_off, s_slot);
    tile_load<PolRaw<PolDF>, false>(la, lam, base, T, t_off, s_slot);
    __syncthreads();
    for (int o = 0; o < p.num_ops; ++o) {
      const Op& op = p.ops[o];
      if (op.ctrl_kind == CTRL_GLOBAL && !((base >> op.ctrl) & 1)) continue;  // uniform per tile
      F2 g{0.f, 0.f};
      switch (op.cls) {
        case OP_SWAP: adj_tile_op<OP_SWAP>(ps, la, T, op, g); break;
        case OP_DIAG: adj_tile_op<OP_DIAG>(ps, la, T, op, g); break;
        case OP_ANTI: adj_tile_op<OP_ANTI>(ps, la, T, op, g); break;
        case OP_REAL: adj_tile_op<OP_REAL>(ps, la, T, op, g); break;
        case OP_RXLIKE: adj_tile_op<OP_RXLIKE>(ps, la, T, op, g); break;
        default: adj_tile_op<OP_GENERAL>(ps, la, T, op, g); break;
      }
      if (op.generator != 0) {
        g = f2_warp_sum(g);
        if (lane == 0) f2_add(acc[o * kAdjWarps + warp], g.h, g.l);
      }
      __syncthreads();
    }
    tile_store<PolRaw<PolDF>>(ps, psi, base, T, t_off, s_slot);
    tile_store<PolRaw<PolDF>>(la, lam, base, T, t_off, s_slot);
    __syncthreads();
  }
  // Per op, this CTA's sum over its tiles (warps in order; FP64 once).
  for (int o = threadIdx.x; o < p.num_ops; o += kAdjThreads) {
    const Op& op = p.ops[o];
    if (op.generator == 0 || op.param < 0) continue;
    F2 t{0.f, 0.f};
    for (int w = 0; w < kAdjWarps; ++w) f2_add(t, acc[o * kAdjWarps + w].h, acc[o * kAdjWarps + w].l);
    p.partial[(int64_t)op.param * p.cols + blockIdx.x] = f2_val(t);
  }
}

size_t adjoint_window_smem(int k, int num_ops) {
  return ((size_t)2 << k) * sizeof(float4) + (size_t)num_ops * kAdjWarps * sizeof(F2);
}

// Grid of k_adjoint_window: one CTA per SM (the two tiles take 128 KB).
int adjoint_window_grid(int64_t num_tiles) { return (int)std::min<int64_t>(num_tiles, (int64_t)sm_count()); }

int launch_adjoint_window(dmv_state_s* psi, dmv_state_s* lam, int32_t n, const Pass& ps, const Op* ops_dev,
                          double* part, int64_t cols) {
  AdjWindowParams p;
  p.k = ps.low_bits + ps.num_high;
  p.low = ps.low_bits;
  p.nh = ps.num_high;
  for (int i = 0; i < 16; ++i) p.high[i] = i < ps.num_high ? ps.high[i] : 0;
  p.num_tiles = int64_t(1) << (n - p.k);
  p.partial = part;
  p.cols = cols;
  const int grid = adjoint_window_grid(p.num_tiles);
  static const cudaError_t attr = cudaFuncSetAttribute(
      k_adjoint_window, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)adjoint_window_smem(12, kAdjMaxOps));
  (void)attr;  // a refusal shows as the launch's error
  for (int64_t o = 0; o < ps.op_count; o += kAdjMaxOps) {
    p.ops = ops_dev + ps.op_begin + o;
    p.num_ops = (int32_t)std::min<int64_t>(kAdjMaxOps, ps.op_count - o);
    const int64_t tok = prof_begin(DMV_KERNEL_ADJOINT, psi->stream, 4.0 * (double)psi->amp_bytes());
    k_adjoint_window<<<grid, kAdjThreads, adjoint_window_smem(p.k, p.num_ops), psi->stream>>>(
        static_cast<float4*>(psi->amps), static_cast<float4*>(lam->amps), p);
    prof_end(tok, psi->stream);
    count_launch();
  }
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

int chunk_bits_for(int n) { return std::min(kMaxChunkBits, n); }
// Chunks of the Pauli-Z mass pass (k_chunk_mass_bulk, k_chunk_mass_f2 below
// 12 qubits): 4096 amplitudes.
int mass_chunk_bits_for(int n) { return std::min(kF2ChunkBits, n); }

// Amplitude states of 12 or more qubits take the bulk-staged pass.
bool mass_uses_bulk(int src_kind, int n) { return src_kind != 2 && n >= kMbChunkBits; }

// Its grid: one CTA per SM for the bulk-staged pass; eight CTAs per SM for
// k_chunk_mass_f2 (two measured 1.4x slower: too few loads in flight).
int mass_grid_for(int src_kind, int n, int64_t num_chunks) {
  const int64_t per_sm = mass_uses_bulk(src_kind, n) ? 1 : 8;
  return (int)std::max<int64_t>(1, std::min<int64_t>(num_chunks, (int64_t)sm_count() * per_sm));
}

// Opts the bulk-staged pass into its shared memory (once per process; done
// before any graph capture by the batch engine's setup).
template <int SRC>
void mass_bulk_attributes() {
  static const cudaError_t attr = cudaFuncSetAttribute(
      k_chunk_mass_bulk<SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mass_bulk_smem<SRC>());
  (void)attr;  // a refusal shows as the launch's error
}

template <int SRC>
void launch_mass_bulk(const void* src, int n, int64_t num_chunks, int grid, double* partial, cudaStream_t stream) {
  constexpr size_t smem = mass_bulk_smem<SRC>();
  mass_bulk_attributes<SRC>();
  k_chunk_mass_bulk<SRC><<<grid, kMbThreads, smem, stream>>>(src, n, num_chunks, partial, tma_wait_limit(),
                                                             tma_status_word());
}

// Segment masses (bulk-staged) and their per-chunk running sums.
template <int SRC>
void launch_segment_bulk(const void* src, int64_t num_chunks, int grid, double* seg, double* mass,
                         cudaStream_t stream) {
  constexpr size_t smem = mass_bulk_smem<SRC>();
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_segment_mass_bulk<SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  (void)attr;  // a refusal shows as the launch's error
  k_segment_mass_bulk<SRC><<<grid, kMbThreads, smem, stream>>>(src, num_chunks, seg, tma_wait_limit(),
                                                               tma_status_word());
  k_segment_scan<<<(int)((num_chunks + 255) / 256), 256, 0, stream>>>(seg, num_chunks, mass);
}

// The Pauli-Z mass pass over amplitudes (src_kind 0 complex128, 1
// complex64): per CTA the n + 1 sums in `partial`.
void launch_mass_kernel(const void* src, int src_kind, int n, int cb, int64_t num_chunks, int grid,
                        double* partial, cudaStream_t stream) {
  if (mass_uses_bulk(src_kind, n)) {
    if (src_kind == 0) launch_mass_bulk<0>(src, n, num_chunks, grid, partial, stream);
    else launch_mass_bulk<1>(src, n, num_chunks, grid, partial, stream);
  } else if (src_kind == 0) {
    k_chunk_mass_f2<0><<<grid, kRedThreads, 0, stream>>>(src, n, cb, num_chunks, partial);
  } else {
    k_chunk_mass_f2<1><<<grid, kRedThreads, 0, stream>>>(src, n, cb, num_chunks, partial);
  }
}

// Runs the mass pass and the partial reduction. Leaves the n+1 sums
// (bit-set mass per qubit, then total) in `sums_dev`.
int chunk_mass_pass(const void* src, int src_kind, int n, DeviceBuffer& reduce_dev, cudaStream_t stream,
                    double** sums_dev_out) {
  const int cb = mass_chunk_bits_for(n);
  const int64_t num_chunks = int64_t(1) << (n - cb);
  const int grid = mass_grid_for(src_kind, n, num_chunks);
  const size_t partial_elems = (size_t)grid * (n + 1);
  DMV_TRY(reduce_dev.reserve((partial_elems + (size_t)(n + 1)) * sizeof(double)));
  double* partial = static_cast<double*>(reduce_dev.ptr);
  double* sums = partial + partial_elems;
  launch_mass_kernel(src, src_kind, n, cb, num_chunks, grid, partial, stream);
  k_reduce_partials<<<1, 64, 0, stream>>>(partial, n + 1, grid, sums);
  count_launch(2);
  DMV_CUDA_TRY(cudaGetLastError());
  *sums_dev_out = sums;
  return DMV_OK;
}

// Prefix levels of the sampler, in `prefix`: chunk masses, their inclusive
// scan, then the per-chunk segment prefixes.
struct SamplePrefix {
  int seg_bits = 0, chunk_bits = 0;
  int64_t num_chunks = 0;
  const double* chunk_incl = nullptr;
  const int32_t* guide = nullptr;  // num_chunks + 1 entries
  const double* seg_incl = nullptr;
};

int sample_prefix_pass(const void* src, int src_kind, int n, DeviceBuffer& prefix, cudaStream_t stream,
                       SamplePrefix* out) {
  SamplePrefix sp;
  const bool bulk = mass_uses_bulk(src_kind, n);
  sp.seg_bits = std::min(kSpSegBits, n);
  sp.chunk_bits = bulk ? kMbChunkBits : chunk_bits_for(n);
  sp.num_chunks = int64_t(1) << (n - sp.chunk_bits);
  const int64_t nseg = int64_t(1) << (n - sp.seg_bits);
  DMV_TRY(prefix.reserve((size_t)(2 * sp.num_chunks + nseg) * sizeof(double) +
                         (size_t)(sp.num_chunks + 1) * sizeof(int32_t)));
  double* mass = static_cast<double*>(prefix.ptr);
  double* incl = mass + sp.num_chunks;
  double* seg = incl + sp.num_chunks;
  int32_t* guide = reinterpret_cast<int32_t*>(seg + nseg);
  if (bulk) {
    const int grid = mass_grid_for(src_kind, n, sp.num_chunks);
    if (src_kind == 0) launch_segment_bulk<0>(src, sp.num_chunks, grid, seg, mass, stream);
    else launch_segment_bulk<1>(src, sp.num_chunks, grid, seg, mass, stream);
    count_launch(2);
  } else {
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((sp.num_chunks + 7) / 8, (int64_t)sm_count() * 8));
    switch (src_kind) {
      case 0: k_segment_prefix_f2<0><<<grid, kRedThreads, 0, stream>>>(src, sp.seg_bits, sp.chunk_bits, sp.num_chunks, seg, mass); break;
      case 1: k_segment_prefix_f2<1><<<grid, kRedThreads, 0, stream>>>(src, sp.seg_bits, sp.chunk_bits, sp.num_chunks, seg, mass); break;
      default: k_segment_prefix<2><<<grid, kRedThreads, 0, stream>>>(src, sp.seg_bits, sp.chunk_bits, sp.num_chunks, seg, mass); break;
    }
    count_launch();
  }
  k_scan_chunks<<<1, 1024, 0, stream>>>(mass, sp.num_chunks, incl);
  const int gg = (int)std::max<int64_t>(1, std::min<int64_t>((sp.num_chunks + 256) / 256, (int64_t)sm_count() * 4));
  k_chunk_guide<<<gg, 256, 0, stream>>>(incl, sp.num_chunks, sp.num_chunks, guide);
  count_launch(2);
  DMV_CUDA_TRY(cudaGetLastError());
  sp.chunk_incl = incl;
  sp.guide = guide;
  sp.seg_incl = seg;
  *out = sp;
  return DMV_OK;
}

int launch_warp_sampler(const void* src, int src_kind, const SamplePrefix& sp, const double* u_dev, int64_t k,
                        uint64_t* out_dev, cudaStream_t stream) {
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((k + 7) / 8, (int64_t)sm_count() * 8));
  switch (src_kind) {
    case 0: k_sample_warp<0><<<grid, kRedThreads, 0, stream>>>(src, sp.seg_bits, sp.chunk_bits, sp.num_chunks, sp.chunk_incl, sp.guide, sp.seg_incl, u_dev, k, out_dev); break;
    case 1: k_sample_warp<1><<<grid, kRedThreads, 0, stream>>>(src, sp.seg_bits, sp.chunk_bits, sp.num_chunks, sp.chunk_incl, sp.guide, sp.seg_incl, u_dev, k, out_dev); break;
    default: k_sample_warp<2><<<grid, kRedThreads, 0, stream>>>(src, sp.seg_bits, sp.chunk_bits, sp.num_chunks, sp.chunk_incl, sp.guide, sp.seg_incl, u_dev, k, out_dev); break;
  }
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

int run_sampler(const void* src, int src_kind, int n, DeviceBuffer& prefix, DeviceBuffer& scratch,
                cudaStream_t stream, const double* uniforms_host, int64_t k, uint64_t* samples_host) {
  if (k <= 0) return DMV_OK;
  SamplePrefix sp;
  DMV_TRY(sample_prefix_pass(src, src_kind, n, prefix, stream, &sp));
  DMV_TRY(scratch.reserve((size_t)k * (sizeof(double) + sizeof(uint64_t))));
  double* u_dev = static_cast<double*>(scratch.ptr);
  uint64_t* out_dev = reinterpret_cast<uint64_t*>(u_dev + k);
  DMV_CUDA_TRY(cudaMemcpyAsync(u_dev, uniforms_host, (size_t)k * sizeof(double), cudaMemcpyHostToDevice, stream));
  DMV_TRY(launch_warp_sampler(src, src_kind, sp, u_dev, k, out_dev, stream));
  DMV_CUDA_TRY(cudaMemcpyAsync(samples_host, out_dev, (size_t)k * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
  DMV_CUDA_TRY(cudaStreamSynchronize(stream));
  DMV_TRY(check_window_status());  // the prefix pass's chunk load waits
  return DMV_OK;
}

}  // namespace

ChunkMassShape chunk_mass_shape(int n) {
  ChunkMassShape sh;
  sh.chunk_bits = mass_chunk_bits_for(n);
  sh.num_chunks = int64_t(1) << (n - sh.chunk_bits);
  sh.grid = mass_grid_for(0, n, sh.num_chunks);  // the same grid for complex64
  mass_bulk_attributes<0>();
  mass_bulk_attributes<1>();
  sh.partial_elems = (int64_t)sh.grid * (n + 1);
  return sh;
}

int launch_chunk_mass_into(const void* src, int src_kind, int n, double* partial, double* sums,
                           cudaStream_t stream) {
  if (src_kind != 0 && src_kind != 1)
    return set_error(DMV_ERR_INVALID, "launch_chunk_mass_into takes amplitudes (kinds 0, 1)");
  const ChunkMassShape sh = chunk_mass_shape(n);
  launch_mass_kernel(src, src_kind, n, sh.chunk_bits, sh.num_chunks, sh.grid, partial, stream);
  k_reduce_partials<<<1, 64, 0, stream>>>(partial, n + 1, sh.grid, sums);
  count_launch(2);
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

int launch_probabilities(dmv_state_s* s, double* probs_device) {
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((s->N + kRedThreads - 1) / kRedThreads,
                                                               (int64_t)sm_count() * 16));
  if (s->precision == DMV_C128)
    k_probabilities<0><<<grid, kRedThreads, 0, s->stream>>>(s->amps, probs_device, s->N);
  else
    k_probabilities<1><<<grid, kRedThreads, 0, s->stream>>>(s->amps, probs_device, s->N);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

int launch_expect_z(dmv_state_s* s, double* expect_host, double* norm_host) {
  double* sums = nullptr;
  DMV_TRY(chunk_mass_pass(s->amps, s->precision == DMV_C128 ? 0 : 1, s->n, s->reduce_dev, s->stream, &sums));
  std::vector<double> h((size_t)s->n + 1);
  DMV_CUDA_TRY(cudaMemcpyAsync(h.data(), sums, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
  DMV_TRY(check_window_status());  // the mass pass's chunk load waits
  const double total = h[(size_t)s->n];
  if (expect_host)
    for (int q = 0; q < s->n; ++q) expect_host[q] = total - 2.0 * h[(size_t)q];
  if (norm_host) *norm_host = total;
  return DMV_OK;
}

int launch_sample(dmv_state_s* s, const double* uniforms_host, int64_t k, uint64_t* samples_host) {
  return run_sampler(s->amps, s->precision == DMV_C128 ? 0 : 1, s->n, s->chunk_dev, s->reduce_dev, s->stream,
                     uniforms_host, k, samples_host);
}

// Samples per batch of the sampled-expectation pipeline (uniforms and samples
// of a batch: 256 MB of scratch).
constexpr int64_t kSampleBatch = int64_t(1) << 24;

int launch_sample_counts(dmv_state_s* s, const double* uniforms_host, uint64_t seed, int64_t k,
                         unsigned long long counts_host[64]) {
  for (int b = 0; b < 64; ++b) counts_host[b] = 0;
  if (k <= 0) return DMV_OK;
  const int src_kind = s->precision == DMV_C128 ? 0 : 1;
  SamplePrefix sp;
  DMV_TRY(sample_prefix_pass(s->amps, src_kind, s->n, s->chunk_dev, s->stream, &sp));
  const int64_t batch = std::min<int64_t>(k, kSampleBatch);
  DMV_TRY(s->reduce_dev.reserve((size_t)batch * (sizeof(double) + sizeof(uint64_t)) + 64 * sizeof(unsigned long long)));
  double* u_dev = static_cast<double*>(s->reduce_dev.ptr);
  uint64_t* out_dev = reinterpret_cast<uint64_t*>(u_dev + batch);
  unsigned long long* counts_dev = reinterpret_cast<unsigned long long*>(out_dev + batch);
  DMV_CUDA_TRY(cudaMemsetAsync(counts_dev, 0, 64 * sizeof(unsigned long long), s->stream));
  for (int64_t off = 0; off < k; off += batch) {
    const int64_t cnt = std::min(batch, k - off);
    if (uniforms_host) {
      DMV_CUDA_TRY(cudaMemcpyAsync(u_dev, uniforms_host + off, (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice,
                                   s->stream));
    } else {
      const int ug = (int)std::max<int64_t>(1, std::min<int64_t>((cnt + 255) / 256, (int64_t)sm_count() * 8));
      k_uniforms<<<ug, 256, 0, s->stream>>>(seed, off, cnt, u_dev);
      count_launch();
    }
    DMV_TRY(launch_warp_sampler(s->amps, src_kind, sp, u_dev, cnt, out_dev, s->stream));
    const int cg = (int)std::max<int64_t>(1, std::min<int64_t>((cnt + kRedThreads - 1) / kRedThreads,
                                                               (int64_t)sm_count() * 8));
    k_count_bits<<<cg, kRedThreads, 0, s->stream>>>(out_dev, cnt, counts_dev);
    count_launch();
    DMV_CUDA_TRY(cudaGetLastError());
  }
  DMV_CUDA_TRY(cudaMemcpyAsync(counts_host, counts_dev, 64 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               s->stream));
  DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
  DMV_TRY(check_window_status());  // the prefix pass's chunk load waits
  return DMV_OK;
}

int sample_from_device_probs(const double* probs_device, int64_t num_probs, int32_t num_bits,
                             cudaStream_t stream, const double* uniforms_host, int64_t k,
                             uint64_t* samples_host) {
  (void)num_probs;
  DeviceBuffer prefix, scratch;
  const int rc = run_sampler(probs_device, 2, num_bits, prefix, scratch, stream, uniforms_host, k, samples_host);
  cudaStreamSynchronize(stream);
  prefix.release();
  scratch.release();
  return rc;
}

int launch_inner_product(dmv_state_s* a, dmv_state_s* b, double* re, double* im) {
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((a->N + kRedThreads - 1) / kRedThreads,
                                                               (int64_t)sm_count() * 8));
  DMV_TRY(a->reduce_dev.reserve((size_t)(2 * grid + 2) * sizeof(double)));
  double* partial = static_cast<double*>(a->reduce_dev.ptr);
  double* sums = partial + 2 * grid;
  // b's pending work must be complete before a's stream reads it.
  if (a->stream != b->stream) {
    cudaEvent_t ev;
    DMV_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, b->stream);
    cudaStreamWaitEvent(a->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  if (a->precision == DMV_C128)
    k_inner<double2><<<grid, kRedThreads, 0, a->stream>>>(static_cast<const double2*>(a->amps),
                                                         static_cast<const double2*>(b->amps), a->N, partial);
  else
    k_inner<float2><<<grid, kRedThreads, 0, a->stream>>>(static_cast<const float2*>(a->amps),
                                                        static_cast<const float2*>(b->amps), a->N, partial);
  k_reduce_partials<<<1, 64, 0, a->stream>>>(partial, 2, grid, sums);
  count_launch(2);
  DMV_CUDA_TRY(cudaGetLastError());
  double h[2];
  DMV_CUDA_TRY(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, a->stream));
  DMV_CUDA_TRY(cudaStreamSynchronize(a->stream));
  *re = h[0];
  *im = h[1];
  return DMV_OK;
}

int launch_scale_by_z_observable(dmv_state_s* dst, dmv_state_s* src, const double* weights_host) {
  std::vector<double> tab(4 * 1024, 0.0);
  for (int f = 0; f < 4; ++f)
    for (int x = 0; x < 1024; ++x) {
      double acc = 0.;
      for (int b = 0; b < 10; ++b) {
        const int q = 10 * f + b;
        if (q >= src->n) break;
        acc += ((x >> b) & 1) ? -weights_host[q] : weights_host[q];
      }
      tab[(size_t)f * 1024 + (size_t)x] = acc;
    }
  DMV_TRY(dst->reduce_dev.reserve(tab.size() * sizeof(double)));
  DMV_CUDA_TRY(cudaMemcpyAsync(dst->reduce_dev.ptr, tab.data(), tab.size() * sizeof(double),
                               cudaMemcpyHostToDevice, dst->stream));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((src->N + kRedThreads - 1) / kRedThreads,
                                                               (int64_t)sm_count() * 8));
  if (src->precision == DMV_C128)
    k_scale_z<double2><<<grid, kRedThreads, 0, dst->stream>>>(
        static_cast<double2*>(dst->amps), static_cast<const double2*>(src->amps), src->N,
        static_cast<const double*>(dst->reduce_dev.ptr));
  else
    k_scale_z<float2><<<grid, kRedThreads, 0, dst->stream>>>(
        static_cast<float2*>(dst->amps), static_cast<const float2*>(src->amps), src->N,
        static_cast<const double*>(dst->reduce_dev.ptr));
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  // The table buffer is reused by the next call on this stream only after
  // this kernel, by stream order.
  return DMV_OK;
}

int adjoint_grid(int64_t num_pairs) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((num_pairs + kRedThreads - 1) / kRedThreads,
                                                      (int64_t)sm_count() * 8));
}

int launch_adjoint_step_impl(dmv_state_s* psi, dmv_state_s* lam, const Op& op, int apply,
                             double* partial_slot, bool df_raw = false) {
  const bool ctrl = op.ctrl_kind != CTRL_NONE && op.ctrl >= 0;
  const int64_t pairs = psi->N >> (ctrl ? 2 : 1);
  const int grid = adjoint_grid(pairs);
  const int64_t tok = prof_begin(DMV_KERNEL_ADJOINT, psi->stream, (double)(apply ? 4 : 2) * (double)psi->amp_bytes() *
                                                                       (ctrl ? 0.5 : 1.0));
  if (psi->precision == DMV_C64)
    k_adjoint_step<PolF32><<<grid, kRedThreads, 0, psi->stream>>>(
        static_cast<float2*>(psi->amps), static_cast<float2*>(lam->amps), pairs, op, apply, partial_slot);
  else if ((psi->arith == ARITH_INT64 || psi->arith == ARITH_TC) && op.unitary)
    k_adjoint_step<PolFX><<<grid, kRedThreads, 0, psi->stream>>>(
        static_cast<double2*>(psi->amps), static_cast<double2*>(lam->amps), pairs, op, apply, partial_slot);
  else if (psi->arith == ARITH_FP32X2 && df_raw)
    k_adjoint_step<PolDF, true><<<grid, kRedThreads, 0, psi->stream>>>(
        static_cast<double2*>(psi->amps), static_cast<double2*>(lam->amps), pairs, op, apply, partial_slot);
  else if (psi->arith == ARITH_FP32X2)
    k_adjoint_step<PolDF><<<grid, kRedThreads, 0, psi->stream>>>(
        static_cast<double2*>(psi->amps), static_cast<double2*>(lam->amps), pairs, op, apply, partial_slot);
  else
    k_adjoint_step<PolF64><<<grid, kRedThreads, 0, psi->stream>>>(
        static_cast<double2*>(psi->amps), static_cast<double2*>(lam->amps), pairs, op, apply, partial_slot);
  prof_end(tok, psi->stream);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

// The reverse sweep over psi and lam in the FP32-pair form, fused into
// windows (build_adjoint_plan): window passes run k_adjoint_window,
// single-gate passes k_adjoint_step.
int adjoint_sweep_windows(dmv_state_s* s, dmv_state_s* psi, dmv_state_s* lam, const std::vector<Gate>& gates,
                          double* part, int64_t cols, DeviceBuffer& ops_buf) {
  Plan plan;
  DMV_TRY(build_adjoint_plan(gates, s->n, s->precision, plan_options_for(s, DMV_FUSE_WINDOW), plan));
  if (!plan.ops.empty()) {
    DMV_TRY(ops_buf.reserve(plan.ops.size() * sizeof(Op)));
    DMV_CUDA_TRY(cudaMemcpyAsync(ops_buf.ptr, plan.ops.data(), plan.ops.size() * sizeof(Op), cudaMemcpyHostToDevice,
                                 s->stream));
  }
  const Op* ops_dev = static_cast<const Op*>(ops_buf.ptr);
  for (const Pass& ps : plan.passes) {
    if (ps.kind == 1) {
      DMV_TRY(launch_adjoint_window(psi, lam, s->n, ps, ops_dev, part, cols));
    } else {
      const Op& op = plan.ops[(size_t)ps.op_begin];
      double* slot = op.param >= 0 ? part + (size_t)op.param * cols : part;
      DMV_TRY(launch_adjoint_step_impl(psi, lam, op, 1, slot, true));
    }
  }
  return DMV_OK;
}

int adjoint_gradient(dmv_state_s* s, const std::vector<Gate>& gates, const double* weights,
                     double* loss, double* grads) {
  // Forward from |0...0> with the fused plan.
  DMV_TRY(launch_set_zero(s));
  Plan plan;
  const PlanOptions opt = plan_options_for(s, DMV_FUSE_WINDOW);
  DMV_TRY(build_plan(gates, s->n, s->precision, opt, plan));
  DMV_TRY(launch_plan(s, plan));
  std::vector<double> ez((size_t)s->n);
  DMV_TRY(launch_expect_z(s, ez.data(), nullptr));
  double L = 0.;
  for (int q = 0; q < s->n; ++q) L += weights[q] * ez[(size_t)q];
  if (loss) *loss = L;

  // Parameter slots in list order (Circuit::set_parameters order).
  std::vector<int64_t> slot_of(gates.size(), -1);
  int64_t num_params = 0;
  for (size_t i = 0; i < gates.size(); ++i)
    if (!gates[i].observable && is_parametrised(gates[i].kind)) slot_of[i] = num_params++;
  if (num_params == 0) return DMV_OK;

  dmv_state_t psi = nullptr, lam = nullptr;
  int rc = dmv_state_create(s->n, s->precision, s->stream, &psi);
  if (rc != DMV_OK) return rc;
  rc = dmv_state_create(s->n, s->precision, s->stream, &lam);
  if (rc != DMV_OK) { dmv_state_destroy(psi); return rc; }
  psi->arith = lam->arith = s->arith;  // the sweep runs in the state's arithmetic

  DeviceBuffer partial, adj_ops;
  const int64_t pairs_u = s->N >> 1;
  // Columns of the per-parameter partials: the widest grid of the sweep's kernels.
  const int grid = std::max(adjoint_grid(pairs_u), adjoint_window_grid(int64_t(1) << std::max(0, s->n - 12)));
  do {
    rc = partial.reserve((size_t)num_params * grid * sizeof(double) + (size_t)num_params * sizeof(double));
    if (rc != DMV_OK) break;
    double* part = static_cast<double*>(partial.ptr);
    double* out = part + (size_t)num_params * grid;
    if (cudaMemsetAsync(part, 0, (size_t)num_params * grid * sizeof(double), s->stream) != cudaSuccess) {
      rc = set_error(DMV_ERR_CUDA, "memset of gradient partials failed");
      break;
    }
    if (cudaMemcpyAsync(psi->amps, s->amps, s->amp_bytes(), cudaMemcpyDeviceToDevice, s->stream) != cudaSuccess) {
      rc = set_error(DMV_ERR_CUDA, "statevector copy failed");
      break;
    }
    rc = launch_scale_by_z_observable(lam, s, weights);
    if (rc != DMV_OK) break;
    // FP32-pair arithmetic: psi and lam are scratch, so they take the pair form
    // once and keep it for the whole sweep.
    const bool df_raw = s->precision == DMV_C128 && s->arith == ARITH_FP32X2;
    if (df_raw) {
      const int pg = (int)std::max<int64_t>(1, std::min<int64_t>((s->N + 255) / 256, (int64_t)sm_count() * 8));
      k_df_pack<<<pg, 256, 0, s->stream>>>(static_cast<double2*>(psi->amps), s->N);
      k_df_pack<<<pg, 256, 0, s->stream>>>(static_cast<double2*>(lam->amps), s->N);
      count_launch(2);
    }
    if (df_raw) {
      rc = adjoint_sweep_windows(s, psi, lam, gates, part, grid, adj_ops);
      if (rc != DMV_OK) break;
    }
    for (int64_t gi = df_raw ? -1 : (int64_t)gates.size() - 1; gi >= 0 && rc == DMV_OK; --gi) {
      const Gate& g = gates[(size_t)gi];
      if (g.observable) continue;
      Op op;
      std::memset(&op, 0, sizeof(op));
      adjoint2(g.m, op.m);
      split_matrix(op);
      op.target = g.target;
      op.ctrl = g.control;
      op.ctrl_kind = g.control >= 0 ? CTRL_GLOBAL : CTRL_NONE;
      op.cls = classify(op.m);
      op.param = (int32_t)slot_of[(size_t)gi];
      op.generator = slot_of[(size_t)gi] >= 0 ? rotation_generator(g.kind) : 0;
      // The grid of k_adjoint_step depends on the pair count; partials of
      // controlled parametrised gates use fewer CTAs and leave zeros behind.
      double* slot = op.param >= 0 ? part + (size_t)op.param * grid : part;
      const bool last = gi == 0;
      rc = launch_adjoint_step_impl(psi, lam, op, last ? 0 : 1, slot, df_raw);
    }
    if (rc != DMV_OK) break;
    k_reduce_rows<<<(int)((num_params + 127) / 128), 128, 0, s->stream>>>(part, num_params, grid, out);
    count_launch();
    if (cudaMemcpyAsync(grads, out, (size_t)num_params * sizeof(double), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess) {
      rc = set_error(DMV_ERR_CUDA, "gradient readback failed");
      break;
    }
  } while (false);
  cudaStreamSynchronize(s->stream);
  partial.release();
  adj_ops.release();
  dmv_state_destroy(psi);
  dmv_state_destroy(lam);
  return rc;
}

int launch_adjoint_step(dmv_state_s* psi, dmv_state_s* lam, const Op& op, double* grad_slot_device) {
  return launch_adjoint_step_impl(psi, lam, op, 1, grad_slot_device);
}

}  // namespace dmv
