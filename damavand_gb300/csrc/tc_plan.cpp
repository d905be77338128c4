// Host planning of tensor-core window passes (ARITH_TC): stages and the
// digit matrices of dense blocks.
//
// A window pass's ops (tile-local targets, in list order) are swept
// repeatedly, like the window planner sweeps gates: each sweep opens one
// dense block of at most 5 tile bits and takes, in order, every op whose bits
// fit and none of whose bits an earlier op of the sweep left behind. An
// exchange (X, CNOT) that touches no bit of the open block and none left
// behind commutes with everything taken so far and takes effect in front of
// the block, as a relabelling: the kernel reads logical amplitude l at
// A l xor c, A tracked here (CNOTs controlled inside the tile), c in the
// kernel (X and CNOTs controlled outside it). The block's matrix is the
// product of its ops, in order, as one 32 x 32 complex matrix.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"

namespace dmv {

namespace {

// IEEE half bits of an integer |v| <= 2048 (exactly representable).
uint16_t half_of_int(int v) {
  if (v == 0) return 0;
  const uint16_t sign = v < 0 ? 0x8000u : 0u;
  unsigned a = (unsigned)(v < 0 ? -v : v);
  int e = 31 - __builtin_clz(a);                      // a in [2^e, 2^(e+1))
  const unsigned mant = (a << (10 - e)) & 0x3FFu;      // exact: e <= 11 and a has at most e+1 bits
  return (uint16_t)(sign | (unsigned)((e + 15) << 10) | mant);
}

int popcount32(uint32_t x) { return __builtin_popcount(x); }

// Element (row, k) of a matrix with 64 columns of K in the canonical K-major
// layout without swizzle: 8 x 8 FP16 core matrices of 128 bytes, the 8 core
// matrices of a row group adjacent along K (128 bytes apart), row groups
// 1024 bytes apart.
inline int64_t kmajor_index(int row, int k) {
  return (int64_t)(((row >> 3) * 8 + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7));
}

constexpr uint64_t kDigitBias = 0x0080808080808080ull;  // 128 in each of bytes 0..6

int32_t g_tc_convert_mode = 0;

// Appends the digit matrix of the 32 x 32 block matrix (ur, ui row-major) and
// returns whether every FP32 group sum of the kernel stays below 2^22.
bool append_block_digits(const double* ur, const double* ui, std::vector<uint16_t>& u) {
  const size_t base = u.size();
  u.resize(base + (size_t)kTcUHalves, 0);
  // |digit| sums per (digit j, output n) for the accumulator bound
  static thread_local double esum[kTcDigits][64];
  for (int j = 0; j < kTcDigits; ++j)
    for (int n = 0; n < 64; ++n) esum[j][n] = 0.0;
  for (int n = 0; n < 64; ++n) {
    const int ro = n >> 1, co = n & 1;
    for (int k = 0; k < 64; ++k) {
      const int ri = k >> 1, ci = k & 1;
      // real form of the complex product: out.re = Re*re - Im*im, out.im = Im*re + Re*im
      const double re = ur[ro * 32 + ri], im = ui[ro * 32 + ri];
      const double val = co == 0 ? (ci == 0 ? re : -im) : (ci == 0 ? im : re);
      const long long w = std::llround(std::ldexp(val, 54));
      const uint64_t b = (uint64_t)w + kDigitBias;
      for (int j = 0; j < kTcDigits; ++j) {
        const int e = (int)((b >> (8 * (kTcDigits - 1 - j))) & 0xFFu) - 128;
        u[base + (size_t)kmajor_index(64 * j + n, k)] = half_of_int(e);
        esum[j][n] += std::abs((double)e);
      }
    }
  }
  // group s = i + j: state digit i (|d_0| <= 64, |d_i| <= 128 otherwise) times matrix digit j
  double worst = 0.0;
  for (int s = 0; s <= kTcDigits; ++s)
    for (int n = 0; n < 64; ++n) {
      double bound = 0.0;
      for (int i = std::max(0, s - (kTcDigits - 1)); i <= std::min(kTcDigits - 1, s); ++i)
        bound += (i == 0 ? 64.0 : 128.0) * esum[s - i][n];
      worst = std::max(worst, bound);
    }
  return worst < 4194304.0;
}

}  // namespace

bool build_tc_pass(const Plan& plan, const Pass& ps, std::vector<TcStage>& stages, std::vector<uint16_t>& u,
                   int32_t final_map[12], int32_t* exchanges) {
  const int32_t k = ps.low_bits + ps.num_high;
  if (k != 12) return false;
  const Op* ops = plan.ops.data() + ps.op_begin;
  const int64_t count = ps.op_count;
  for (int64_t i = 0; i < count; ++i) {
    if (!ops[i].unitary) return false;
    if (ops[i].ctrl_kind == CTRL_GLOBAL && ops[i].cls != OP_SWAP) return false;
  }
  const size_t first_stage = stages.size();
  // the affine map's linear part: amap[b] = A e_b
  int32_t amap[12];
  for (int b = 0; b < 12; ++b) amap[b] = 1 << b;
  int32_t nx = 0;
  std::vector<int64_t> rem(count), keep, take;
  for (int64_t i = 0; i < count; ++i) rem[i] = i;
  std::vector<double> ur(32 * 32), ui(32 * 32);
  while (!rem.empty()) {
    uint32_t S = 0, blocked = 0;
    keep.clear();
    take.clear();
    for (int64_t i : rem) {
      const Op& op = ops[i];
      uint32_t qs = 1u << op.target;
      if (op.ctrl_kind == CTRL_LOCAL) qs |= 1u << op.ctrl;
      if (qs & blocked) {
        blocked |= qs;
        keep.push_back(i);
        continue;
      }
      if (op.cls == OP_SWAP && !(qs & S)) {
        // new phys(l) = old phys(sigma(l)), sigma the exchange on logical indices
        ++nx;
        if (op.ctrl_kind == CTRL_LOCAL) {
          amap[op.ctrl] ^= amap[op.target];  // sigma(l) = l xor l_ctrl e_target: linear
        } else {
          TcStage st;  // sigma(l) = l xor e_target (on the tiles where the control is 1): c ^= A e_target
          std::memset(&st, 0, sizeof(st));
          st.kind = TC_SWAP;
          st.img[0] = amap[op.target];
          st.gctrl = op.ctrl_kind == CTRL_GLOBAL ? op.ctrl : -1;
          st.u_index = -1;
          stages.push_back(st);
        }
        continue;
      }
      if (op.ctrl_kind == CTRL_GLOBAL) {  // an exchange overlapping the open block: a later sweep
        blocked |= qs;
        keep.push_back(i);
        continue;
      }
      if (popcount32(S | qs) <= kTcBlockBits) {
        S |= qs;
        take.push_back(i);
      } else {
        blocked |= qs;
        keep.push_back(i);
      }
    }
    if (!take.empty()) {
      // pad the block to 5 bits with unused high tile bits (identity there)
      for (int b = k - 1; b >= 0 && popcount32(S) < kTcBlockBits; --b) S |= 1u << b;
      int bits[kTcBlockBits], nb = 0, pos_of[32];
      for (int b = 0; b < 32; ++b) pos_of[b] = -1;
      for (int b = 0; b < k; ++b)
        if (S & (1u << b)) {
          pos_of[b] = nb;
          bits[nb++] = b;
        }
      std::fill(ur.begin(), ur.end(), 0.0);
      std::fill(ui.begin(), ui.end(), 0.0);
      for (int r = 0; r < 32; ++r) ur[r * 32 + r] = 1.0;
      for (int64_t i : take) {
        const Op& op = ops[i];
        const int tq = pos_of[op.target];
        const int cq = op.ctrl_kind == CTRL_LOCAL ? pos_of[op.ctrl] : -1;
        const double* m = op.m;
        for (int r0 = 0; r0 < 32; ++r0) {
          if ((r0 >> tq) & 1) continue;
          if (cq >= 0 && !((r0 >> cq) & 1)) continue;
          const int r1 = r0 | (1 << tq);
          for (int c = 0; c < 32; ++c) {
            const double ar = ur[r0 * 32 + c], ai = ui[r0 * 32 + c];
            const double br = ur[r1 * 32 + c], bi = ui[r1 * 32 + c];
            ur[r0 * 32 + c] = m[0] * ar - m[1] * ai + m[2] * br - m[3] * bi;
            ui[r0 * 32 + c] = m[0] * ai + m[1] * ar + m[2] * bi + m[3] * br;
            ur[r1 * 32 + c] = m[4] * ar - m[5] * ai + m[6] * br - m[7] * bi;
            ui[r1 * 32 + c] = m[4] * ai + m[5] * ar + m[6] * bi + m[7] * br;
          }
        }
      }
      TcStage st;
      std::memset(&st, 0, sizeof(st));
      st.kind = TC_BLOCK;
      for (int b = 0; b < kTcBlockBits; ++b) st.img[b] = amap[bits[b]];
      for (int b = 0, c = 0; b < k; ++b)
        if (!(S & (1u << b))) st.img[kTcBlockBits + c++] = amap[b];
      st.gctrl = -1;
      st.u_index = (int32_t)(u.size() / (size_t)kTcUHalves);
      st.magic = append_block_digits(ur.data(), ui.data(), u) && g_tc_convert_mode == 0 ? 1 : 0;
      stages.push_back(st);
    }
    rem.swap(keep);
  }
  // each block names the digit matrix of the pass's next block, cyclically
  std::vector<size_t> blocks;
  for (size_t i = first_stage; i < stages.size(); ++i)
    if (stages[i].kind == TC_BLOCK) blocks.push_back(i);
  for (size_t b = 0; b < blocks.size(); ++b)
    stages[blocks[b]].next_u = stages[blocks[(b + 1) % blocks.size()]].u_index;
  for (int b = 0; b < 12; ++b) final_map[b] = amap[b];
  if (exchanges) *exchanges = nx;
  return true;
}

void set_tc_convert_mode(int32_t mode) { g_tc_convert_mode = mode; }

}  // namespace dmv
