// Tensor-core window pass (ARITH_TC, complex128 storage): included by
// kernels_apply.cu inside its anonymous namespace, after TileGeom and
// encode_pass_map.
//
// One persistent CTA of 128 threads per SM (it holds all 512 TMEM columns and
// 209 KB of shared memory). Per 2^12-amplitude tile:
//  1. The tile arrives by TMA (the FP64 5-D tensor map of the pass, two tile
//     buffers: the next tile loads while this one computes) and is converted
//     in place to int64 block fixed point with the tile's largest exponent
//     (54 fraction bits, as the integer-pipe arithmetic). Amplitude l sits at
//     l ^ ((l >> 5) & 7), which keeps the column gathers below free of
//     bank conflicts.
//  2. Exchange stages swap amplitude pairs in shared memory.
//  3. A block stage views the tile as 128 columns x 32 block rows. Thread t
//     gathers column t, scales it so its largest component is below 2^54,
//     and writes its 7 balanced 8-bit digits (FP16) as row t of a 128 x 64
//     operand, one digit at a time into two alternating buffers. After each
//     digit one thread issues the MMAs of that digit against the block's
//     stacked digit matrix (loaded by a bulk copy), N-stacked so one MMA
//     covers several matrix digits: digit product (i, j) accumulates into
//     TMEM columns 64(i+j) .. 64(i+j)+63 (exact: every sum stays below 2^24).
//     Thread t then reads TMEM lane t, recombines the 8 accumulators into
//     int64 (sum of D_s 2^(42-8s), rounded once), undoes its column scale
//     and writes the column back.
//  4. The tile goes back to FP64 and out by TMA.
// Every wait is bounded; a wait that gives up sets the status word, drains
// the copies and MMAs in flight and ends the kernel.
// (cuda_fp16.h and tc.cuh are included by the including file.)

constexpr int kTcThreads = 128;
constexpr uint32_t kTcTileBytes = 4096u * 16u;               // 64 KB
constexpr uint32_t kTcDigitBytes = 128u * 64u * 2u;          // one digit of the 128 x 64 operand
constexpr uint32_t kTcUBytes = (uint32_t)kTcUHalves * 2u;    // 56 KB
constexpr size_t kTcSmem = 2 * (size_t)kTcTileBytes + 2 * (size_t)kTcDigitBytes + kTcUBytes + 1024;

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
};

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

__device__ __forceinline__ long long tc_scale(long long v, int ls) {
  if (ls >= 0) return v << ls;
  const int s = -ls;
  return (v + (1ll << (s - 1))) >> s;
}

__device__ __forceinline__ long long tc_unscale(long long y, int ls) {
  if (ls > 0) return (y + (1ll << (ls - 1))) >> ls;
  return y << (-ls);
}

// Recombines output o of one TMEM chunk: sum_s D_s 2^(42-8s), rounded at 2^0.
template <bool MAGIC>
__device__ __forceinline__ long long tc_combine(const uint32_t (&g)[8][8], int o) {
  int c[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    if constexpr (MAGIC) c[s] = __float_as_int(__fadd_rn(__uint_as_float(g[s][o]), 12582912.0f)) - 0x4B400000;
    else c[s] = __float2int_rn(__uint_as_float(g[s][o]));
  }
  const int p01 = c[0] * 256 + c[1], p23 = c[2] * 256 + c[3], p45 = c[4] * 256 + c[5], p67 = c[6] * 256 + c[7];
  return ((long long)p01 << 34) + ((long long)p23 << 18) + ((long long)p45 << 2) + (((long long)p67 + 8192) >> 14);
}

__device__ __forceinline__ void tc_issue_digit(int digit, uint32_t tbase, uint32_t a_addr, uint32_t u_addr) {
#pragma unroll
  for (int e = 0; e < 12; ++e) {
    const TcMma m = kTcMmas[e];
    if (m.digit != digit) continue;
    const uint32_t idesc = tc_idesc_f16(128, m.n);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const uint64_t ad = tc_smem_desc(a_addr + (uint32_t)ks * 256u, 128, 1024);
      const uint64_t bd = tc_smem_desc(u_addr + (uint32_t)(m.row0 >> 3) * 1024u + (uint32_t)ks * 256u, 128, 1024);
      tc_mma_f16(tbase + (uint32_t)m.col0, ad, bd, idesc, m.init ? (uint32_t)(ks > 0) : 1u);
    }
  }
}

// Gathers column `basem` of a block, computes its digits, runs the MMAs and
// writes the column back. Returns false if a wait gave up (uniform over the CTA).
template <bool MAGIC>
__device__ __forceinline__ bool tc_block(longlong2* tile, const TcStage& st, int basem, unsigned char* adig0,
                                         unsigned char* adig1, unsigned char* ubuf, uint32_t tbase, uint32_t tlane,
                                         uint64_t* s_afree, uint64_t* s_acc, uint64_t* s_ufull, uint32_t& n_afree0,
                                         uint32_t& n_afree1, uint32_t& n_acc, bool u_wait, uint32_t n_u,
                                         uint32_t limit) {
  const int tid = threadIdx.x;
  const int d0 = 1 << st.bits[0], d1 = 1 << st.bits[1], d2 = 1 << st.bits[2], d3 = 1 << st.bits[3],
            d4 = 1 << st.bits[4];
  longlong2 v[32];
#pragma unroll
  for (int r = 0; r < 32; ++r) {
    const int dep = ((r & 1) ? d0 : 0) | ((r & 2) ? d1 : 0) | ((r & 4) ? d2 : 0) | ((r & 8) ? d3 : 0) |
                    ((r & 16) ? d4 : 0);
    v[r] = tile[tc_pos(basem | dep)];
  }
  unsigned long long mx = 0;
#pragma unroll
  for (int r = 0; r < 32; ++r) {
    const long long x = v[r].x, y = v[r].y;
    mx |= (unsigned long long)((x ^ (x >> 63)) - (x >> 63)) | (unsigned long long)((y ^ (y >> 63)) - (y >> 63));
  }
  const int bl = mx ? 64 - __clzll((long long)mx) : 0;
  const int ls = mx ? 54 - bl : 0;
  constexpr unsigned long long kBias = 0x0080808080808080ull;
#pragma unroll
  for (int r = 0; r < 32; ++r) {
    v[r].x = (long long)((unsigned long long)tc_scale(v[r].x, ls) + kBias);
    v[r].y = (long long)((unsigned long long)tc_scale(v[r].y, ls) + kBias);
  }
  const uint32_t u_addr = (uint32_t)__cvta_generic_to_shared(ubuf);
  bool ok = true;
#pragma unroll
  for (int i = 0; i < kTcDigits; ++i) {
    const int ab = i & 1;
    unsigned char* const abuf = ab ? adig1 : adig0;
    if (i >= 2) ok = mbar_wait(&s_afree[ab], ((ab ? n_afree1 : n_afree0) - 1) & 1u, limit);
    if (i == 0 && u_wait) ok = mbar_wait(s_ufull, (n_u - 1) & 1u, limit);
    unsigned char* row = abuf + (size_t)(tid >> 3) * 1024 + (size_t)(tid & 7) * 16;
    const int byte = kTcDigits - 1 - i;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      uint4 w;
      w.x = tc_digit_pair((uint64_t)v[4 * c + 0].x, (uint64_t)v[4 * c + 0].y, byte);
      w.y = tc_digit_pair((uint64_t)v[4 * c + 1].x, (uint64_t)v[4 * c + 1].y, byte);
      w.z = tc_digit_pair((uint64_t)v[4 * c + 2].x, (uint64_t)v[4 * c + 2].y, byte);
      w.w = tc_digit_pair((uint64_t)v[4 * c + 3].x, (uint64_t)v[4 * c + 3].y, byte);
      if (ok) *reinterpret_cast<uint4*>(row + (size_t)c * 128) = w;
    }
    fence_proxy_async_smem();
    if (__syncthreads_or(!ok)) return false;
    if (tid == 0) {
      tc_fence_after_sync();
      tc_issue_digit(i, tbase, (uint32_t)__cvta_generic_to_shared(abuf), u_addr);
      tc_commit(&s_afree[ab]);
      if (i == kTcDigits - 1) tc_commit(s_acc);
    }
    if (ab) ++n_afree1;
    else ++n_afree0;
  }
  ++n_acc;
  ok = mbar_wait(s_acc, (n_acc - 1) & 1u, limit);
  if (__syncthreads_or(!ok)) return false;
  tc_fence_after_sync();
#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    uint32_t g[8][8];
#pragma unroll
    for (int s = 0; s < 8; ++s) tc_ld8(tlane + (uint32_t)(64 * s + 8 * q), g[s]);
    tc_wait_ld();
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int r = 4 * q + a;
      const int dep = ((r & 1) ? d0 : 0) | ((r & 2) ? d1 : 0) | ((r & 4) ? d2 : 0) | ((r & 8) ? d3 : 0) |
                      ((r & 16) ? d4 : 0);
      longlong2 o;
      o.x = tc_unscale(tc_combine<MAGIC>(g, 2 * a), ls);
      o.y = tc_unscale(tc_combine<MAGIC>(g, 2 * a + 1), ls);
      tile[tc_pos(basem | dep)] = o;
    }
  }
  tc_fence_before_sync();
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_window_tc(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ TcPassParams p) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t s_full[2];
  __shared__ __align__(8) uint64_t s_afree[2];
  __shared__ __align__(8) uint64_t s_acc;
  __shared__ __align__(8) uint64_t s_ufull;
  __shared__ uint32_t s_tbase;
  __shared__ int s_red[kTcThreads / 32];
  __shared__ int s_high[16];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* const adig0 = base + 2 * kTcTileBytes;
  unsigned char* const adig1 = adig0 + kTcDigitBytes;
  unsigned char* ubuf = base + 2 * kTcTileBytes + 2 * kTcDigitBytes;
  const int tid = (int)threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < 16) s_high[tid] = p.high[tid];
  if (warp == 0) tc_alloc(&s_tbase, 512);
  if (tid == 0) {
    mbar_init(&s_full[0], 1);
    mbar_init(&s_full[1], 1);
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
  const uint32_t tlane = tbase + ((uint32_t)(warp * 32) << 16);
  const TileGeom<16> geom{p.low, p.nh, s_high};
  const uint32_t limit = p.wait_limit;
  uint32_t n_afree0 = 0u, n_afree1 = 0u, n_acc = 0u, n_u = 0u;
  int u_resident = -1;
  bool failed = false;
  // loads issued into each tile buffer, and whether the last one is not yet consumed
  uint32_t n_load[2] = {0u, 0u};
  bool pending[2] = {false, false};
  int64_t tix = blockIdx.x;
  if (tix < p.num_tiles) {
    if (warp == 0) geom.load(&tmap, &s_full[0], base, tix, p.boxes, kTcTileBytes, lane);
    ++n_load[0];
    pending[0] = true;
  }
  for (int64_t it = 0; tix < p.num_tiles; ++it, tix += gridDim.x) {
    const int buf = (int)(it & 1);
    unsigned char* const tbytes = buf ? base + kTcTileBytes : base;
    unsigned char* const tother = buf ? base : base + kTcTileBytes;
    longlong2* tile = reinterpret_cast<longlong2*>(tbytes);
    const bool ok = mbar_wait(&s_full[buf], (n_load[buf] - 1) & 1u, limit);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    pending[buf] = false;
    // FP64 -> int64 block fixed point, in place, at the swizzled positions
    double2 d[32];
    const double2* td = reinterpret_cast<const double2*>(tile);
    unsigned emax = 0;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      d[j] = td[tid + 128 * j];
      emax = max(emax, (unsigned)max(fx_exponent(d[j].x), fx_exponent(d[j].y)));
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
    if (lane == 0) s_red[warp] = (int)emax;
    __syncthreads();
    const int e = max(max(s_red[0], s_red[1]), max(s_red[2], s_red[3]));
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int l = tid + 128 * j;
      tile[tc_pos(l)] = make_longlong2(fx_from_double(d[j].x, e), fx_from_double(d[j].y, e));
    }
    __syncthreads();
    // the next tile loads into the other buffer once that buffer's store has drained
    const int64_t next = tix + gridDim.x;
    if (next < p.num_tiles) {
      if (warp == 0) {
        tma_wait_group_read<0>();
        geom.load(&tmap, &s_full[buf ^ 1], tother, next, p.boxes, kTcTileBytes, lane);
      }
      ++n_load[buf ^ 1];
      pending[buf ^ 1] = true;
    }
    const int64_t tile_base = geom.base(tix);
    for (int si = 0; si < p.num_stages; ++si) {
      const TcStage st = p.stages[si];
      if (st.kind == TC_SWAP) {
        if (st.gctrl >= 0 && !((tile_base >> st.gctrl) & 1)) continue;
        const int tb = st.bits[0], cb = st.bits[1];
        if (cb < 0) {
#pragma unroll 4
          for (int j = 0; j < 16; ++j) {
            const int l0 = tc_insert_zero(tid + 128 * j, tb), l1 = l0 | (1 << tb);
            const int p0 = tc_pos(l0), p1 = tc_pos(l1);
            const longlong2 a0 = tile[p0], a1 = tile[p1];
            tile[p0] = a1;
            tile[p1] = a0;
          }
        } else {
          const int lo = min(tb, cb), hi = max(tb, cb);
#pragma unroll 4
          for (int j = 0; j < 8; ++j) {
            const int l0 = tc_insert_zero(tc_insert_zero(tid + 128 * j, lo), hi) | (1 << cb), l1 = l0 | (1 << tb);
            const int p0 = tc_pos(l0), p1 = tc_pos(l1);
            const longlong2 a0 = tile[p0], a1 = tile[p1];
            tile[p0] = a1;
            tile[p1] = a0;
          }
        }
        __syncthreads();
        continue;
      }
      // dense block: the 7 tile bits outside it index the 128 columns
      const uint32_t bmask = (1u << st.bits[0]) | (1u << st.bits[1]) | (1u << st.bits[2]) | (1u << st.bits[3]) |
                             (1u << st.bits[4]);
      int basem = 0;
      for (int b = 0, c = 0; b < 12; ++b)
        if (!(bmask & (1u << b))) {
          basem |= ((tid >> c) & 1) << b;
          ++c;
        }
      const bool u_wait = st.u_index != u_resident;
      if (u_wait) {
        if (tid == 0) {
          mbar_arrive_expect_tx(&s_ufull, kTcUBytes);
          bulk_load(ubuf, p.u + (size_t)st.u_index * (size_t)kTcUHalves, kTcUBytes, &s_ufull);
        }
        u_resident = st.u_index;
        ++n_u;
      }
      const bool okb = st.magic ? tc_block<true>(tile, st, basem, adig0, adig1, ubuf, tbase, tlane, s_afree, &s_acc,
                                                 &s_ufull, n_afree0, n_afree1, n_acc, u_wait, n_u, limit)
                                : tc_block<false>(tile, st, basem, adig0, adig1, ubuf, tbase, tlane, s_afree, &s_acc,
                                                  &s_ufull, n_afree0, n_afree1, n_acc, u_wait, n_u, limit);
      if (!okb) {
        failed = true;
        break;
      }
    }
    if (failed) break;
    // int64 -> FP64, back to the linear layout, out by TMA
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const longlong2 x = tile[tc_pos(tid + 128 * j)];
      d[j] = make_double2(fx_to_double(x.x, e), fx_to_double(x.y, e));
    }
    __syncthreads();
    double2* tw = reinterpret_cast<double2*>(tile);
#pragma unroll
    for (int j = 0; j < 32; ++j) tw[tid + 128 * j] = d[j];
    fence_proxy_async_smem();
    __syncthreads();
    if (warp == 0) geom.store(&tmap, tbytes, tix, p.boxes, kTcTileBytes, lane);
  }
  if (failed) {
    if (tid == 0) {
      atomicExch(p.status, 1);
      // every MMA issued so far completes before the TMEM is released
      tc_commit(&s_acc);
      mbar_wait(&s_acc, n_acc & 1u, kTmaDrainLimit);
    }
    if (warp == 0) {
      // loads in flight land before the CTA's shared memory is released
      for (int b = 0; b < 2; ++b)
        if (pending[b]) mbar_wait(&s_full[b], (n_load[b] - 1) & 1u, kTmaDrainLimit);
    }
  }
  if (warp == 0) tma_wait_group_all();
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tc_dealloc(tbase, 512);
}

int launch_window_tc(void* amps, int32_t n, const Pass& ps, const TcStage* stages_dev, int32_t num_stages,
                     const uint16_t* u_dev, cudaStream_t stream) {
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
  static bool configured = false;
  if (!configured) {
    DMV_CUDA_TRY(cudaFuncSetAttribute(k_window_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    configured = true;
  }
  const int64_t grid = std::min<int64_t>(p.num_tiles, (int64_t)num_sms());
  k_window_tc<<<(int)grid, kTcThreads, kTcSmem, stream>>>(map, p);
  return DMV_OK;
}
