// Tensor-core window pass (ARITH_TC, complex128 storage): included by
// kernels_apply.cu inside its anonymous namespace, after TileGeom and
// encode_pass_map.
//
// One persistent CTA of 512 threads per SM (it holds all 512 TMEM columns and
// 217 KB of shared memory). Per 2^12-amplitude tile:
//  1. The tile arrives by TMA (the FP64 5-D tensor map of the pass, two tile
//     buffers: the next tile loads while this one computes) and is converted
//     in place to int64 block fixed point with the tile's largest exponent
//     (56 fraction bits, tc_from_double). Amplitude l sits at
//     l ^ ((l >> 5) & 7), which keeps the column gathers below free of
//     bank conflicts.
//  2. Exchanges move no data: logical amplitude l of the tile is read at
//     A l xor c, A given by the host per block (CNOTs controlled inside the
//     tile), c updated per tile here (X, and CNOTs controlled outside it).
//  3. A block stage views the tile as 128 columns x 32 block rows. Threads
//     t, t + 128, t + 256, t + 384 gather quarters of column t, scale it so its largest
//     component is below 2^54, and write its 7 balanced 8-bit digits (FP16)
//     as row t of a 128 x 64 operand, one digit at a time into two
//     alternating buffers. After each
//     digit one thread issues the MMAs of that digit against the block's
//     stacked digit matrix (loaded by a bulk copy), N-stacked so one MMA
//     covers several matrix digits: digit product (i, j) accumulates into
//     TMEM columns 64(i+j) .. 64(i+j)+63 (exact: every sum stays below 2^24).
//     The same threads then read TMEM lane t, recombine the 8 accumulators into
//     int64 (sum of D_s 2^(42-8s), rounded once), undoes its column scale
//     and writes the column back.
//  4. The tile goes back to FP64 and out by TMA.
// Every wait is bounded; a wait that gives up sets the status word, drains
// the copies and MMAs in flight and ends the kernel.
// (cuda_fp16.h and tc.cuh are included by the including file.)

constexpr int kTcThreads = 512;
constexpr uint32_t kTcTileBytes = 4096u * 16u;               // 64 KB
constexpr uint32_t kTcDigitBytes = 128u * 64u * 2u;          // one digit of the 128 x 64 operand
constexpr uint32_t kTcUBytes = (uint32_t)kTcUHalves * 2u;    // 56 KB
constexpr size_t kTcSmem = 2 * (size_t)kTcTileBytes + 2 * (size_t)kTcDigitBytes + kTcUBytes + 1024;

// Stages a CTA copies to shared memory (a longer pass reads them from global memory).
constexpr int kTcSmemStages = 40;

struct TcPassParams {
  int k, low, nh, boxes;
  int high[16];
  int64_t num_tiles;
  void* amps;
  int* status;
  uint32_t wait_limit;
  int32_t num_stages;
  const TcStage* stages;
  const uint16_t* u;
  int32_t final_map[12];  // A e_b after the pass's last stage (the linear part of the final relabelling)
};

// Tile fixed point: with e the tile's largest biased FP64 exponent, x becomes
// X = round(x * 2^(1078 - e)), so the largest components have 56 fraction
// bits and |X| < 2^56. A unitary on a 4096-amplitude tile can concentrate its
// norm on one amplitude, at most 2^6 times the largest component: every value
// stays below 2^62.
__device__ __forceinline__ long long tc_from_double(double x, int e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FFull);
  if (E == 0) return 0;  // zero or subnormal: flushed
  const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int s = e - E - 3;  // right shift; negative is a left shift by up to 3
  unsigned long long X;
  if (s <= 0) X = M << (-s);
  else if (s < 63) X = (M + (1ull << (s - 1))) >> s;
  else X = 0;
  return (b >> 63) ? -(long long)X : (long long)X;
}

// Position of tile amplitude l in shared memory.
__device__ __forceinline__ int tc_pos(int l) { return l ^ ((l >> 5) & 7); }

__device__ __forceinline__ int tc_insert_zero(int x, int b) { return ((x >> b) << (b + 1)) | (x & ((1 << b) - 1)); }

// One MMA group of a state digit: matrix rows row0 .. row0+n-1 (matrix
// digits row0/64 ..) into TMEM columns col0 ..; `init` marks the first write
// of those columns in a block.
struct TcMma {
  int digit, row0, n, col0, init;
};
__device__ constexpr TcMma kTcMmas[12] = {{0, 0, 256, 0, 1},   {0, 256, 192, 256, 1}, {1, 0, 256, 64, 0},
                                          {1, 256, 128, 320, 0}, {1, 384, 64, 448, 1},  {2, 0, 256, 128, 0},
                                          {2, 256, 128, 384, 0}, {3, 0, 256, 192, 0},  {3, 256, 64, 448, 0},
                                          {4, 0, 256, 256, 0},  {5, 0, 192, 320, 0},   {6, 0, 128, 384, 0}};

// Two FP16 digits (byte `byte` of a and of b, each minus 128) as one word.
__device__ __forceinline__ uint32_t tc_digit_pair(uint64_t a, uint64_t b, int byte) {
  const uint32_t wa = byte < 4 ? (uint32_t)a : (uint32_t)(a >> 32);
  const uint32_t wb = byte < 4 ? (uint32_t)b : (uint32_t)(b >> 32);
  const int q = byte & 3;
  uint32_t t = __byte_perm(wa, wb, (uint32_t)(q | ((4 + q) << 8)));
  t = (t & 0x00FF00FFu) | 0x64006400u;  // FP16 1024 + digit byte, exact
  const __half2 h = __hsub2(*reinterpret_cast<const __half2*>(&t), __half2half2(__ushort_as_half((unsigned short)0x6480u)));
  return *reinterpret_cast<const uint32_t*>(&h);
}

// v * 2^ls, rounded to nearest (ties up) when ls < 0; the same code for
// both signs (the threads of a warp hold columns with different ls).
__device__ __forceinline__ long long tc_shift(long long v, int lsl, int lsr, long long rnd) {
  return ((long long)((unsigned long long)v << lsl) + rnd) >> lsr;
}

// bits(x + 1.5 * 2^23) = kTcMagic + x for an integer |x| < 2^22.
constexpr int kTcMagic = 0x4B400000;
// kTcMagic * (2^42 + 2^34 + 2^26 + 2^18 + 2^10 + 2^2) modulo 2^64.
constexpr unsigned long long kTcMagicSum =
    (unsigned long long)kTcMagic * ((1ull << 42) + (1ull << 34) + (1ull << 26) + (1ull << 18) + (1ull << 10) + (1ull << 2));

// An FP32 accumulator (an exact integer D) as kTcMagic + D: the magic-number
// addition when |D| < 2^22 is known, the conversion instruction otherwise.
template <bool MAGIC>
__device__ __forceinline__ unsigned tc_acc_biased(uint32_t bits) {
  if constexpr (MAGIC) return (unsigned)__float_as_int(__fadd_rn(__uint_as_float(bits), 12582912.0f));
  else return (unsigned)(__float2int_rn(__uint_as_float(bits)) + kTcMagic);
}

// Called by a whole warp (the descriptors are warp-uniform); the elected lane
// issues. A descriptor's address field is its low 14 bits (shared-memory byte
// address / 16, below 2^14 for addresses under 256 KB), so an offset is added
// to a base descriptor as offset / 16.
__device__ __forceinline__ void tc_issue_digit(int digit, uint32_t tbase, uint64_t a_desc, uint64_t u_desc,
                                               bool leader) {
#pragma unroll
  for (int e = 0; e < 12; ++e) {
    const TcMma m = kTcMmas[e];
    if (m.digit != digit) continue;
    const uint32_t idesc = tc_idesc_f16(128, m.n);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const uint64_t ad = a_desc + (uint64_t)(ks * 16);
      const uint64_t bd = u_desc + (uint64_t)((m.row0 >> 3) * 64 + ks * 16);
      if (leader) tc_mma_f16(tbase + (uint32_t)m.col0, ad, bd, idesc, m.init ? (uint32_t)(ks > 0) : 1u);
    }
  }
}

// Block row r (0..31) of a column as tile bits.
__device__ __forceinline__ int tc_dep(int r, const int (&d)[5]) {
  return ((r & 1) ? d[0] : 0) | ((r & 2) ? d[1] : 0) | ((r & 4) ? d[2] : 0) | ((r & 8) ? d[3] : 0) |
         ((r & 16) ? d[4] : 0);
}

// Output o of one TMEM chunk: sum_s D_s 2^(42-8s), rounded at 2^0. Groups
// 0..5 are integer terms, summed modulo 2^64 from the biased values (the
// true sum fits in int64, so the bias comes off at once); groups 6 and 7 are
// the fraction, rounded from their exact 32-bit sum D_6 2^8 + D_7.
template <bool MAGIC>
__device__ __forceinline__ long long tc_combine(const uint32_t (&g)[8][8], int o) {
  unsigned b[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) b[s] = tc_acc_biased<MAGIC>(g[s][o]);
  const int low = (int)(b[6] * 256u + b[7] + (8192u - 257u * (unsigned)kTcMagic));  // D_6 2^8 + D_7 + 2^13
  unsigned long long u = (unsigned long long)(long long)(low >> 14) - kTcMagicSum;
  u += (unsigned long long)b[5] * 4ull;
  u += (unsigned long long)b[4] * 1024ull;
  u += (unsigned long long)b[3] * 262144ull;
  u += (unsigned long long)b[2] * 67108864ull;
  u += (unsigned long long)(b[1] * 4u + b[0] * 1024u) << 32;
  return (long long)u;
}

// Thread (h, m) reads TMEM lane m, outputs 16h .. 16h+15 (block rows
// 8h .. 8h+7), undoes the column scale and writes them back.
template <bool MAGIC>
__device__ __forceinline__ void tc_epilogue(longlong2* tile, int hbase, int d0, int d1, int d2, int h, int ls,
                                            uint32_t tlane) {
  const int lsr = ls > 0 ? ls : 0, lsl = ls < 0 ? -ls : 0;
  const long long rnd = lsr ? (1ll << (lsr - 1)) : 0;
#pragma unroll 1
  for (int c = 0; c < 2; ++c) {
    const int q = 2 * h + c;
    uint32_t g[8][8];
#pragma unroll
    for (int s = 0; s < 8; ++s) tc_ld8(tlane + (uint32_t)(64 * s + 8 * q), g[s]);
    tc_wait_ld();
    const int cbase = hbase ^ (c ? d2 : 0);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const long long yr = tc_shift(tc_combine<MAGIC>(g, 2 * a), lsl, lsr, rnd);
      const long long yi = tc_shift(tc_combine<MAGIC>(g, 2 * a + 1), lsl, lsr, rnd);
      tile[tc_pos(cbase ^ ((a & 1) ? d0 : 0) ^ ((a & 2) ? d1 : 0))] = make_longlong2(yr, yi);
    }
  }
}

// Waits for phase `parity` of `bar`, each poll suspending the thread in
// hardware for up to ~0.5 us (no busy polling); gives up after `limit` polls.
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(500u)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Per-CTA progress of the barriers and the digit-matrix buffer (identical in
// every thread).
struct TcSync {
  uint32_t n_afree0 = 0, n_afree1 = 0, n_acc = 0, n_u = 0;
  int u_issued = -1;  // digit matrix of the last bulk copy into the buffer
  bool u_ready = true;
};

// One dense block on the tile. Returns false if a wait gave up (uniform over
// the CTA). Thread (h, m) = (tid / 128, tid % 128) owns block rows 8h .. 8h+7
// of column m: it gathers them, writes their digits (K columns 16h .. 16h+15
// of row m) and, from TMEM lane m, their 16 outputs. Each warp publishes a
// digit by one arrival on s_afull once its lanes' stores are fenced and the
// warp has synchronised; thread 0 waits there and issues that digit's MMAs.
template <bool MAGIC>
__device__ __forceinline__ bool tc_block(longlong2* tile, const TcStage& st, const TcPassParams& p, int basem,
                                         unsigned char* adig0, unsigned char* adig1, unsigned char* ubuf,
                                         uint32_t tbase, uint32_t tlane, uint64_t* s_afull, uint64_t* s_afree,
                                         uint64_t* s_acc, uint64_t* s_ufull, unsigned long long* s_cmax, TcSync& sy) {
  const int tid = threadIdx.x, h = tid >> 7, m = tid & 127;
  const uint32_t limit = p.wait_limit;
  if (st.u_index != sy.u_issued) {  // the first block of this CTA (later ones are prefetched)
    if (tid == 0) {
      mbar_arrive_expect_tx(s_ufull, kTcUBytes);
      bulk_load(ubuf, p.u + (size_t)st.u_index * (size_t)kTcUHalves, kTcUBytes, s_ufull);
    }
    sy.u_issued = st.u_index;
    ++sy.n_u;
    sy.u_ready = false;
  }
  // gather block rows 8h .. 8h+7 of column m (block-row bits 3, 4 come from h)
  // through the tile's relabelling (basem already holds A m xor c); the
  // column's scale from the bit length of its largest one's-complement magnitude
  const int d0 = st.img[0], d1 = st.img[1], d2 = st.img[2];
  const int hbase = basem ^ ((h & 1) ? st.img[3] : 0) ^ ((h & 2) ? st.img[4] : 0);
  longlong2 v[8];
  unsigned long long mx = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    v[j] = tile[tc_pos(hbase ^ ((j & 1) ? d0 : 0) ^ ((j & 2) ? d1 : 0) ^ ((j & 4) ? d2 : 0))];
    mx |= (unsigned long long)(v[j].x ^ (v[j].x >> 63)) | (unsigned long long)(v[j].y ^ (v[j].y >> 63));
  }
  s_cmax[tid] = mx;
  __syncthreads();
  mx = s_cmax[m] | s_cmax[m + 128] | s_cmax[m + 256] | s_cmax[m + 384];
  const int bl = mx ? 64 - __clzll((long long)mx) : 54;
  const int ls = 54 - bl;  // column scale 2^ls
  {
    const int lsl = ls > 0 ? ls : 0, lsr = ls < 0 ? -ls : 0;
    const long long rnd = lsr ? (1ll << (lsr - 1)) : 0;
    constexpr unsigned long long kBias = 0x0080808080808080ull;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      v[j].x = (long long)((unsigned long long)tc_shift(v[j].x, lsl, lsr, rnd) + kBias);
      v[j].y = (long long)((unsigned long long)tc_shift(v[j].y, lsl, lsr, rnd) + kBias);
    }
  }
  const uint64_t u_desc = tc_smem_desc((uint32_t)__cvta_generic_to_shared(ubuf), 128, 1024);
  bool ok = true;
#pragma unroll
  for (int i = 0; i < kTcDigits; ++i) {
    const int ab = i & 1;
    unsigned char* const abuf = ab ? adig1 : adig0;
    const uint32_t k = ab ? sy.n_afree1 : sy.n_afree0;  // earlier digits written into this buffer
    if (i >= 2) ok &= tc_wait(&s_afree[ab], (k - 1) & 1u, limit);
    unsigned char* row = abuf + (size_t)(m >> 3) * 1024 + (size_t)(m & 7) * 16 + (size_t)h * 256;
    const int byte = kTcDigits - 1 - i;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      uint4 w;
      w.x = tc_digit_pair((uint64_t)v[4 * c + 0].x, (uint64_t)v[4 * c + 0].y, byte);
      w.y = tc_digit_pair((uint64_t)v[4 * c + 1].x, (uint64_t)v[4 * c + 1].y, byte);
      w.z = tc_digit_pair((uint64_t)v[4 * c + 2].x, (uint64_t)v[4 * c + 2].y, byte);
      w.w = tc_digit_pair((uint64_t)v[4 * c + 3].x, (uint64_t)v[4 * c + 3].y, byte);
      if (ok) *reinterpret_cast<uint4*>(row + (size_t)c * 128) = w;
    }
    fence_proxy_async_smem();
    __syncwarp();
    if ((tid & 31) == 0) mbar_arrive(&s_afull[ab]);  // one arrival per warp
    if (tid < 32) {
      // warp 0 polls (a suspended wait would delay the MMAs) and one lane issues
      bool go = ok && mbar_wait(&s_afull[ab], k & 1u, limit);
      if (i == 0 && !sy.u_ready) go = go && mbar_wait(s_ufull, (sy.n_u - 1) & 1u, limit);
      go = __all_sync(0xffffffffu, go);
      const bool leader = tc_elect_one();
      if (go) {
        tc_fence_after_sync();
        tc_issue_digit(i, tbase, tc_smem_desc((uint32_t)__cvta_generic_to_shared(abuf), 128, 1024), u_desc, leader);
      }
      ok = go;
      // commits arrive even after a failure, so no thread waits on them forever
      if (leader) {
        tc_commit(&s_afree[ab]);
        if (i == kTcDigits - 1) tc_commit(s_acc);
      }
      __syncwarp();
    }
    if (ab) ++sy.n_afree1;
    else ++sy.n_afree0;
  }
  sy.u_ready = true;
  ++sy.n_acc;
  ok &= tc_wait(s_acc, (sy.n_acc - 1) & 1u, limit);
  if (__syncthreads_or(!ok)) return false;
  tc_fence_after_sync();
  // the MMAs have read the digit matrix: fetch the pass's next one during the epilogue
  if (st.next_u != sy.u_issued) {
    if (tid == 0) {
      mbar_arrive_expect_tx(s_ufull, kTcUBytes);
      bulk_load(ubuf, p.u + (size_t)st.next_u * (size_t)kTcUHalves, kTcUBytes, s_ufull);
    }
    sy.u_issued = st.next_u;
    ++sy.n_u;
    sy.u_ready = false;
  }
  tc_epilogue<MAGIC>(tile, hbase, d0, d1, d2, h, ls, tlane);
  tc_fence_before_sync();
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_window_tc(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TcPassParams p) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_full[2];
  __shared__ __align__(8) uint64_t s_afull[2];
  __shared__ __align__(8) uint64_t s_afree[2];
  __shared__ __align__(8) uint64_t s_acc;
  __shared__ __align__(8) uint64_t s_ufull;
  __shared__ uint32_t s_tbase;
  __shared__ int s_red[kTcThreads / 32];
  __shared__ int s_high[16];
  __shared__ unsigned long long s_cmax[kTcThreads];
  __shared__ TcStage s_stages[kTcSmemStages];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* const adig0 = base + 2 * kTcTileBytes;
  unsigned char* const adig1 = adig0 + kTcDigitBytes;
  unsigned char* ubuf = base + 2 * kTcTileBytes + 2 * kTcDigitBytes;
  const int tid = (int)threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < 16) s_high[tid] = p.high[tid];
  const TcStage* stages = p.stages;
  if (p.num_stages <= kTcSmemStages) {
    for (int i = tid; i < p.num_stages * (int)(sizeof(TcStage) / 4); i += kTcThreads)
      reinterpret_cast<int*>(s_stages)[i] = reinterpret_cast<const int*>(p.stages)[i];
    stages = s_stages;
  }
  if (warp == 0) tc_alloc(&s_tbase, 512);
  if (tid == 0) {
    mbar_init(&s_full[0], 1);
    mbar_init(&s_full[1], 1);
    mbar_init(&s_afull[0], kTcThreads / 32);
    mbar_init(&s_afull[1], kTcThreads / 32);
    mbar_init(&s_afree[0], 1);
    mbar_init(&s_afree[1], 1);
    mbar_init(&s_acc, 1);
    mbar_init(&s_ufull, 1);
    fence_mbar_init();
    tma_prefetch_map(&tmap);
  }
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t tbase = s_tbase;
  // warp w reads TMEM lanes 32 (w % 4) .. +31: the lanes of columns tid % 128
  const uint32_t tlane = tbase + ((uint32_t)((warp & 3) * 32) << 16);
  const TileGeom<16> geom{p.low, p.nh, s_high};
  const uint32_t limit = p.wait_limit;
  TcSync sy;
  bool failed = false;
  // loads issued into each tile buffer, and whether the last one is not yet consumed
  uint32_t n_load0 = 0u, n_load1 = 0u;
  bool pending0 = false, pending1 = false;
  int64_t tix = blockIdx.x;
  if (tix < p.num_tiles) {
    if (warp == 0) geom.load(&tmap, &s_full[0], base, tix, p.boxes, kTcTileBytes, lane);
    ++n_load0;
    pending0 = true;
  }
  for (int64_t it = 0; tix < p.num_tiles; ++it, tix += gridDim.x) {
    const int buf = (int)(it & 1);
    unsigned char* const tbytes = buf ? base + kTcTileBytes : base;
    unsigned char* const tother = buf ? base : base + kTcTileBytes;
    longlong2* tile = reinterpret_cast<longlong2*>(tbytes);
    const bool ok = tc_wait(&s_full[buf], ((buf ? n_load1 : n_load0) - 1) & 1u, limit);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    if (buf) pending1 = false;
    else pending0 = false;
    // FP64 -> int64 block fixed point, in place, at the swizzled positions
    double2 dd[8];
    const double2* td = reinterpret_cast<const double2*>(tile);
    unsigned emax = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      dd[j] = td[tid + kTcThreads * j];
      emax = max(emax, (unsigned)max(fx_exponent(dd[j].x), fx_exponent(dd[j].y)));
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
    if (lane == 0) s_red[warp] = (int)emax;
    __syncthreads();
    int e = 0;
#pragma unroll
    for (int w = 0; w < kTcThreads / 32; ++w) e = max(e, s_red[w]);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int l = tid + kTcThreads * j;
      tile[tc_pos(l)] = make_longlong2(tc_from_double(dd[j].x, e), tc_from_double(dd[j].y, e));
    }
    __syncthreads();
    // the next tile loads into the other buffer once that buffer's store has drained
    const int64_t next = tix + gridDim.x;
    if (next < p.num_tiles) {
      if (warp == 0) {
        tma_wait_group_read<0>();
        geom.load(&tmap, &s_full[buf ^ 1], tother, next, p.boxes, kTcTileBytes, lane);
      }
      if (buf) {
        ++n_load0;
        pending0 = true;
      } else {
        ++n_load1;
        pending1 = true;
      }
    }
    const int64_t tile_base = geom.base(tix);
    int cst = 0;  // the affine part c of the tile's relabelling
    for (int si = 0; si < p.num_stages; ++si) {
      const TcStage& st = stages[si];
      if (st.kind == TC_SWAP) {
        if (st.gctrl < 0 || ((tile_base >> st.gctrl) & 1)) cst ^= st.img[0];
        continue;
      }
      // dense block: the 7 tile bits outside it (images img[5..11]) index the 128 columns
      const int m = tid & 127;
      int basem = cst;
#pragma unroll
      for (int c = 0; c < 7; ++c) basem ^= ((m >> c) & 1) ? st.img[kTcBlockBits + c] : 0;
      const bool okb = st.magic ? tc_block<true>(tile, st, p, basem, adig0, adig1, ubuf, tbase, tlane, s_afull,
                                                 s_afree, &s_acc, &s_ufull, s_cmax, sy)
                                : tc_block<false>(tile, st, p, basem, adig0, adig1, ubuf, tbase, tlane, s_afull,
                                                  s_afree, &s_acc, &s_ufull, s_cmax, sy);
      if (!okb) {
        failed = true;
        break;
      }
    }
    if (failed) break;
    // int64 -> FP64, back to the linear layout, out by TMA
    // logical amplitude tid + 512 j sits at A (tid + 512 j) xor c
    int atid = cst;
#pragma unroll
    for (int b = 0; b < 9; ++b) atid ^= ((tid >> b) & 1) ? p.final_map[b] : 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int aj = ((j & 1) ? p.final_map[9] : 0) ^ ((j & 2) ? p.final_map[10] : 0) ^ ((j & 4) ? p.final_map[11] : 0);
      const longlong2 x = tile[tc_pos(atid ^ aj)];
      dd[j] = make_double2(fx_to_double(x.x, e - 2), fx_to_double(x.y, e - 2));  // X * 2^(e - 1078)
    }
    __syncthreads();
    double2* tw = reinterpret_cast<double2*>(tile);
#pragma unroll
    for (int j = 0; j < 8; ++j) tw[tid + kTcThreads * j] = dd[j];
    fence_proxy_async_smem();
    __syncthreads();
    if (warp == 0) geom.store(&tmap, tbytes, tix, p.boxes, kTcTileBytes, lane);
  }
  if (failed) {
    if (tid == 0) {
      atomicExch(p.status, 1);
      // every MMA issued so far completes before the TMEM is released
      tc_commit(&s_acc);
      mbar_wait(&s_acc, sy.n_acc & 1u, kTmaDrainLimit);
      if (sy.n_u > 0) mbar_wait(&s_ufull, (sy.n_u - 1) & 1u, kTmaDrainLimit);  // the last digit-matrix copy
    }
    if (warp == 0) {
      // loads in flight land before the CTA's shared memory is released
      if (pending0) mbar_wait(&s_full[0], (n_load0 - 1) & 1u, kTmaDrainLimit);
      if (pending1) mbar_wait(&s_full[1], (n_load1 - 1) & 1u, kTmaDrainLimit);
    }
  } else if (!sy.u_ready && tid == 0) {
    mbar_wait(&s_ufull, (sy.n_u - 1) & 1u, kTmaDrainLimit);  // a prefetched digit matrix still landing
  }
  if (warp == 0) tma_wait_group_all();
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_dealloc(tbase, 512);
}

int launch_window_tc(void* amps, int32_t n, const Pass& ps, const TcStage* stages_dev, int32_t num_stages,
                     const uint16_t* u_dev, const int32_t final_map[12], cudaStream_t stream) {
  if ((reinterpret_cast<uintptr_t>(amps) & 15u) != 0)
    return set_error(DMV_ERR_INVALID, "statevector not 16-byte aligned");
  CUtensorMap map;
  DMV_TRY(encode_pass_map<16>(&map, amps, n, ps, false));
  TcPassParams p;
  p.k = ps.low_bits + ps.num_high;
  p.low = ps.low_bits;
  p.nh = ps.num_high;
  for (int i = 0; i < 16; ++i) p.high[i] = i < ps.num_high ? ps.high[i] : 0;
  p.boxes = 1 << (ps.num_high - 3);
  p.num_tiles = int64_t(1) << (n - p.k);
  p.amps = amps;
  p.status = tma_status_ptr();
  if (!p.status) return set_error(DMV_ERR_CUDA, "cannot resolve the TMA status word");
  p.wait_limit = g_tma_wait_limit;
  p.num_stages = num_stages;
  p.stages = stages_dev;
  p.u = u_dev;
  for (int b = 0; b < 12; ++b) p.final_map[b] = final_map[b];
  static bool configured = false;
  if (!configured) {
    DMV_CUDA_TRY(cudaFuncSetAttribute(k_window_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    configured = true;
  }
  const int64_t grid = std::min<int64_t>(p.num_tiles, (int64_t)num_sms());
  k_window_tc<<<(int)grid, kTcThreads, kTcSmem, stream>>>(map, p);
  return DMV_OK;
}
