// Fewer FP64 operations for FP64 window passes (host C++).
//
// On GB300 a complex128 window pass in IEEE FP64 is bound by the FP64
// multiply-add rate, not by HBM: a general 2x2 costs 8 multiply-adds per
// amplitude. The rewrite here spends fewer of them on the same unitary:
//
//  * An uncontrolled unitary U = [[a, b], [c, d]] is written as
//    U = D1 R D2 with R = [[cos t, -sin t], [sin t, cos t]] (t in [0, pi/2],
//    cos t = |a|, sin t = |b|), D2 = diag(1, e^{i g}) and
//    D1 = diag(e^{i arg a}, e^{i arg c}), g = arg b + pi - arg a. The
//    product is checked against U entry by entry; an op it does not
//    reproduce to 4e-15 stays as it was. R acts on the real parts and the
//    imaginary parts of a pair as the same real rotation, applied as f M with
//    M = [[1, -w], [w, 1]] (w = tan t, f = cos t) when cos t >= sin t, else
//    M = [[w, -1], [1, w]] (w = cot t, f = sin t): each output is one
//    multiply-add, 2 per amplitude instead of 8. The kernels apply M only; the
//    product of the factors f (each >= 1/sqrt 2) is multiplied back into the
//    state once, by the caller (three shears, x0 += T x1, x1 += S x0,
//    x0 += T x1, keep the norm but cost 3 multiply-adds per amplitude).
//  * Diagonal factors are not applied where they occur. Each is a phase per
//    amplitude that depends on a few tile bits. Moving a diagonal later in
//    time past an exchange (X, CNOT: a permutation P of the tile) re-indexes
//    it, D then P = P then D o P; past an op whose target is not one of its
//    bits it commutes. Moving it earlier past such ops also commutes. So the
//    factors collect into tables of one phase per amplitude, applied as one
//    op ("flush") where a rotation needs a bit the pending table depends on,
//    and at the end of the pass. A factor whose bits nothing has touched
//    since the last table joins that table instead of the pending one. An
//    exchange controlled from outside the tile re-indexes only the tiles
//    whose control bit is 1, so a table may depend on up to three global
//    bits (then it holds 2^(k+g) phases and each tile reads its slice).
//  * A table's phase phi becomes i^q e^{i phi'} with |phi'| <= pi/4: the
//    kernel rotates (re, im) by phi' with three shears (3 multiply-adds) and
//    multiplies by i^q with a swap and sign flips on the integer pipe.
//
// On the 30-qubit ladder forward (600 fused single-qubit unitaries in 85
// passes) this takes the FP64 work from 4800 to about 1900 multiply-adds
// per amplitude (600 rotations at 2 and 238 tables at 3).
#include <cmath>
#include <algorithm>
#include <cstring>
#include <atomic>
#include <thread>

#include "internal.h"

namespace dmv {
namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kHalfPi = 1.5707963267948966192313216916398;
constexpr double kZyzTol = 4e-15;  // per entry, about 18 ulp of 1

constexpr double kPi = 3.1415926535897932384626433832795;

inline double wrap(double a) { return std::remainder(a, kTwoPi); }

// x + a reduced to [-pi, pi] for x, a in [-pi, pi] (every term angle is).
inline double add_angle(double x, double a) {
  x += a;
  if (x > kPi) x -= kTwoPi;
  else if (x < -kPi) x += kTwoPi;
  return x;
}

// A diagonal phase over the tile (2^k amplitudes) and up to kMaxPhaseGlobals
// global bits: angle of amplitude l on tiles with global-bit pattern gsel at
// index (gsel << k) | l.
struct DiagTable {
  int g = 0;
  int gq[kMaxPhaseGlobals] = {0, 0, 0};
  uint32_t supp = 0;  // local bits it depends on
  bool used = false;
  std::vector<double> ang;
  void reset(int T) {
    g = 0;
    supp = 0;
    used = false;
    ang.assign((size_t)T, 0.0);
  }
};

// Adds the phase f(l) of one diagonal factor (local bits only, |f| <= pi) to every slice.
template <typename F>
void add_term(DiagTable& d, int k, uint32_t bits, F f) {
  const size_t T = size_t(1) << k;
  double* a = d.ang.data();
  for (size_t idx = 0; idx < d.ang.size(); ++idx) {
    const double v = f((uint32_t)(idx & (T - 1)));
    if (v != 0.0) a[idx] = add_angle(a[idx], v);
  }
  d.supp |= bits;
  d.used = true;
}

// The same for a factor on one bit t: p0 where the bit is clear, p1 where it is set.
void add_bit_term(DiagTable& d, int t, double p0, double p1) {
  const size_t n = d.ang.size(), tb = size_t(1) << t;
  double* a = d.ang.data();
  for (size_t base = 0; base < n; base += 2 * tb) {
    if (p0 != 0.0)
      for (size_t i = base; i < base + tb; ++i) a[i] = add_angle(a[i], p0);
    if (p1 != 0.0)
      for (size_t i = base + tb; i < base + 2 * tb; ++i) a[i] = add_angle(a[i], p1);
  }
  d.supp |= 1u << t;
  d.used = true;
}

// D o P for the exchange `op` (X or CNOT on tile bit op.target). Returns false,
// changing nothing, when the table would need a fourth global bit.
bool permute(DiagTable& d, int k, const Op& op) {
  const uint32_t tb = 1u << op.target;
  if (!(d.supp & tb)) return true;  // does not depend on the target: unchanged
  // the exchange is an involution: swap the entries of each pair it maps onto each other
  double* a = d.ang.data();
  const size_t n = d.ang.size();
  if (op.ctrl_kind == CTRL_NONE) {
    for (size_t idx = 0; idx < n; ++idx)
      if (!(idx & tb)) std::swap(a[idx], a[idx | tb]);
  } else if (op.ctrl_kind == CTRL_LOCAL) {
    const size_t cb = size_t(1) << op.ctrl;
    for (size_t idx = 0; idx < n; ++idx)
      if (!(idx & tb) && (idx & cb)) std::swap(a[idx], a[idx | tb]);
    d.supp |= 1u << op.ctrl;
  } else {
    int j = -1;
    for (int i = 0; i < d.g; ++i)
      if (d.gq[i] == op.ctrl) j = i;
    if (j < 0) {
      if (d.g == kMaxPhaseGlobals) return false;
      j = d.g++;
      d.gq[j] = op.ctrl;
      const size_t old = d.ang.size();
      d.ang.resize(old * 2);
      std::memcpy(d.ang.data() + old, d.ang.data(), old * sizeof(double));
    }
    a = d.ang.data();
    const size_t on = size_t(1) << (k + j);
    for (size_t idx = 0; idx < d.ang.size(); ++idx)
      if ((idx & on) && !(idx & tb)) std::swap(a[idx], a[idx | tb]);
  }
  return true;
}

inline double cabs(double re, double im) { return std::hypot(re, im); }

// U = D1 R D2 (see the file comment). Returns false when the product does not
// reproduce U to kZyzTol in every entry.
bool zyz(const double m[8], double& T, double& S, double& C, double& a1, double& a2, double& g2) {
  const double ra = cabs(m[0], m[1]), rb = cabs(m[2], m[3]);
  // c and s each rounded once from a wider quotient: dividing both by one
  // rounded double r biased c^2 + s^2 (by about 3e-17 per rotation on the
  // benchmark's unitaries, a norm drift of 1e-14 over 600 rotations).
  const long double rl = std::hypot((long double)ra, (long double)rb);
  if (!(rl > 0.0L)) return false;
  const double c = (double)((long double)ra / rl), s = (double)((long double)rb / rl);
  a1 = std::atan2(m[1], m[0]);
  a2 = std::atan2(m[5], m[4]);
  g2 = wrap(std::atan2(m[3], m[2]) + M_PI - a1);
  const double e[8] = {c * std::cos(a1),        c * std::sin(a1),
                       -s * std::cos(a1 + g2),  -s * std::sin(a1 + g2),
                       s * std::cos(a2),        s * std::sin(a2),
                       c * std::cos(a2 + g2),   c * std::sin(a2 + g2)};
  for (int i = 0; i < 8; ++i)
    if (!(std::fabs(e[i] - m[i]) <= kZyzTol)) return false;
  T = -s / (1.0 + c);  // -tan(t/2), t = atan2(s, c) in [0, pi/2]
  S = s;
  C = c;
  return true;
}

// |z| = 1 to kZyzTol: a diagonal entry that is a pure phase.
inline bool unit(double re, double im) { return std::fabs(cabs(re, im) - 1.0) <= kZyzTol; }

PhaseEntry entry_of(double phi) {
  // phi = q pi/2 + phi', |phi'| <= pi/4
  const double qf = std::nearbyint(phi / kHalfPi);
  const double p = phi - qf * kHalfPi;
  const int q = (((int)qf % 4) + 4) % 4;
  PhaseEntry e;
  double sh, ch;
  sincos(0.5 * p, &sh, &ch);  // t = -tan(p/2), s = sin p = 2 sin(p/2) cos(p/2)
  e.t = -sh / ch;
  e.s = 2.0 * sh * ch;
  e.swap_xy = (uint32_t)(q & 1);
  e.sign_x = (q == 1 || q == 2) ? 0x80000000u : 0u;
  e.sign_y = (q == 2 || q == 3) ? 0x80000000u : 0u;
  e.pad = 0;
  return e;
}

struct Item {
  bool flush;   // a table (index `table`) rather than `op`
  int table;
  Op op;
};

Op blank_op() {
  Op o;
  std::memset(&o, 0, sizeof(o));
  o.param = -1;
  o.unitary = 1;
  return o;
}

}  // namespace

// e^{i phi} of an entry in double: i^q (cos phi' + i sin phi') with
// cos phi' = 1 + s t (t = -tan(phi'/2), s = sin phi').
void phase_entry_value(const PhaseEntry& e, double& re, double& im) {
  const double c = 1.0 + e.s * e.t, sn = e.s;
  const int q = e.swap_xy ? (e.sign_y ? 3 : 1) : (e.sign_x ? 2 : 0);
  switch (q) {
    case 0: re = c; im = sn; break;
    case 1: re = -sn; im = c; break;
    case 2: re = -c; im = -sn; break;
    default: re = sn; im = -c; break;
  }
}

void phase_tables_df(const std::vector<PhaseEntry>& in, std::vector<float4>& out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    double re, im;
    phase_entry_value(in[i], re, im);
    const float rh = (float)re, ih = (float)im;
    out[i] = make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
  }
}

void rewrite_passes(const Plan& plan, const std::vector<int64_t>& which, bool rot_ops,
                    std::vector<RewrittenPass>& out) {
  out.assign(which.size(), RewrittenPass());
  auto work = [&](size_t j) {
    const Pass& ps = plan.passes[(size_t)which[j]];
    rewrite_pass_rotations(plan.ops.data() + ps.op_begin, ps.op_count, ps.low_bits + ps.num_high, rot_ops,
                           out[j].ops, out[j].tab, &out[j].scale);
  };
  const size_t nt = std::min<size_t>(std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 16),
                                     which.size());
  if (nt <= 1) {
    for (size_t j = 0; j < which.size(); ++j) work(j);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  pool.reserve(nt);
  for (size_t t = 0; t < nt; ++t)
    pool.emplace_back([&]() {
      for (size_t j = next.fetch_add(1); j < which.size(); j = next.fetch_add(1)) work(j);
    });
  for (std::thread& th : pool) th.join();
}

void phase_tables_f64(const std::vector<PhaseEntry>& in, std::vector<double2>& out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    const PhaseEntry& e = in[i];
    uint64_t tb, sb;
    std::memcpy(&tb, &e.t, 8);
    std::memcpy(&sb, &e.s, 8);
    // |t| <= tan(pi/8), |s| <= sin(pi/4): bit 62 (the exponent's top bit) is 0
    const uint64_t top = uint64_t(1) << 62;
    const uint64_t q = (uint64_t)e.swap_xy | ((uint64_t)(e.sign_y != 0) << 1);
    if (q & 1) tb |= top;
    if (q & 2) sb |= top;
    double t, sv;
    std::memcpy(&t, &tb, 8);
    std::memcpy(&sv, &sb, 8);
    out[i] = make_double2(t, sv);
  }
}

void phase_tables_fx(const std::vector<PhaseEntry>& in, std::vector<int4>& out) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    double re, im;
    phase_entry_value(in[i], re, im);
    const long long fr = std::llround(std::ldexp(re, 54)), fi = std::llround(std::ldexp(im, 54));
    out[i] = make_int4((int)(fr >> 31), (int)(fr & 0x7FFFFFFFll), (int)(fi >> 31), (int)(fi & 0x7FFFFFFFll));
  }
}

int64_t rewrite_pass_rotations(const Op* src, int64_t count, int32_t k, bool rot_ops, std::vector<Op>& dst,
                               std::vector<PhaseEntry>& tab, ScaleDD* scale) {
  const int T = 1 << k;
  std::vector<DiagTable> tables;  // flushes in time order; tables[0] may sit at the pass start
  bool start_table = false;
  std::vector<Item> items;
  int last = -1;          // table the next factor may join, -1: none yet
  uint32_t touched = 0;   // target bits of the ops emitted after `last` (after the pass start if none)
  DiagTable pend;
  pend.reset(T);
  ScaleDD acc;  // OP_ROT factors not yet in the state (rot_ops)

  auto flush = [&]() {
    if (!pend.used) return;
    tables.push_back(pend);
    items.push_back(Item{true, (int)tables.size() - 1, Op()});
    last = (int)tables.size() - 1;
    touched = 0;
    pend.reset(T);
  };
  // A diagonal factor on `bits` with phase f(l): into the last table when
  // nothing emitted since touches its bits, else pending.
  auto diag = [&](uint32_t bits, auto f) {
    if (!(bits & touched)) {
      if (last < 0) {
        DiagTable d;
        d.reset(T);
        tables.insert(tables.begin(), d);
        for (Item& it : items)
          if (it.flush) ++it.table;
        start_table = true;
        last = 0;
      }
      add_term(tables[(size_t)last], k, bits, f);
    } else {
      add_term(pend, k, bits, f);
    }
  };
  // The same for a factor on one bit t (p0 where clear, p1 where set).
  auto diag_bit = [&](int t, double p0, double p1) {
    const uint32_t bits = 1u << t;
    if (!(bits & touched)) {
      if (last < 0) {
        DiagTable d;
        d.reset(T);
        tables.insert(tables.begin(), d);
        start_table = true;
        last = 0;
      }
      add_bit_term(tables[(size_t)last], t, p0, p1);
    } else {
      add_bit_term(pend, t, p0, p1);
    }
  };
  auto emit = [&](const Op& op) {
    items.push_back(Item{false, -1, op});
    touched |= 1u << op.target;
  };

  for (int64_t i = 0; i < count; ++i) {
    const Op& op = src[i];
    const uint32_t tb = 1u << op.target;
    if (op.cls == OP_SWAP) {
      if (!permute(pend, k, op)) {
        flush();
        permute(pend, k, op);
      }
      emit(op);
      continue;
    }
    if (op.unitary && op.ctrl_kind == CTRL_NONE &&
        (op.cls == OP_GENERAL || op.cls == OP_REAL || op.cls == OP_RXLIKE)) {
      double Tq, Sq, Cq, a1, a2, g2;
      if (zyz(op.m, Tq, Sq, Cq, a1, a2, g2)) {
        const int t = op.target;
        if (g2 != 0.0) diag_bit(t, 0.0, g2);  // D2
        if (pend.supp & tb) flush();
        Op r = blank_op();
        r.target = t;
        r.ctrl = -1;
        r.ctrl_kind = CTRL_NONE;
        if (rot_ops) {
          // R = f M with one entry pair of M exactly 1: two multiply-adds per
          // component instead of three shears; f (>= 1/sqrt 2) goes to *scale.
          // f = 1 / sqrt(1 + w^2), rounded once from a wider result, so that
          // f M is orthogonal to within that rounding (no norm drift).
          // The factors left out since the last fold live in `acc`; before
          // the stored values could grow past 2^200 this rotation is applied
          // as the real 2x2 acc f M instead (8 multiply-adds per pair), which
          // gives the state its true scale back.
          (void)Tq;
          const bool form_b = Cq < Sq;
          const double w = form_b ? Cq / Sq : Sq / Cq;
          const long double wl = w;
          const double f = (double)(1.0L / std::sqrt(1.0L + wl * wl));
          if (acc.hi * f >= 0x1p-200) {
            r.cls = OP_ROT;
            r.m[0] = w;
            r.m[1] = form_b ? 1.0 : 0.0;
            acc.mul(f);
          } else {
            const long double F = ((long double)acc.hi + (long double)acc.lo) * (long double)f;
            const double one = (double)F, ww = (double)(F * wl);
            r.cls = OP_REAL;
            r.m[0] = form_b ? ww : one;
            r.m[2] = form_b ? -one : -ww;
            r.m[4] = form_b ? one : ww;
            r.m[6] = form_b ? ww : one;
            acc = ScaleDD();
          }
        } else {  // the rotation as a real 2x2 in the arithmetic's own form
          r.cls = OP_REAL;
          r.m[0] = Cq;
          r.m[2] = -Sq;
          r.m[4] = Sq;
          r.m[6] = Cq;
          split_matrix(r);
        }
        emit(r);
        // D1: after the rotation on its own bit, so it cannot join an earlier table
        add_bit_term(pend, t, a1, a2);
        continue;
      }
    }
    if (op.unitary && op.cls == OP_DIAG && unit(op.m[0], op.m[1]) && unit(op.m[6], op.m[7]) &&
        op.ctrl_kind != CTRL_GLOBAL) {
      const int t = op.target;
      const double p0 = std::atan2(op.m[1], op.m[0]), p1 = std::atan2(op.m[7], op.m[6]);
      if (op.ctrl_kind == CTRL_NONE) {
        diag_bit(t, p0, p1);
      } else {
        const int c = op.ctrl;
        diag(tb | (1u << c), [=](uint32_t l) { return ((l >> c) & 1u) ? (((l >> t) & 1u) ? p1 : p0) : 0.0; });
      }
      continue;
    }
    if (op.unitary && op.cls == OP_ANTI && op.ctrl_kind == CTRL_NONE && unit(op.m[2], op.m[3]) &&
        unit(op.m[4], op.m[5])) {
      // [[0, b], [c, 0]] = X diag(c, b)
      const int t = op.target;
      const double pc = std::atan2(op.m[5], op.m[4]), pb = std::atan2(op.m[3], op.m[2]);
      diag_bit(t, pc, pb);
      Op x = blank_op();
      x.cls = OP_SWAP;
      x.target = t;
      x.ctrl = -1;
      x.ctrl_kind = CTRL_NONE;
      x.m[2] = 1.0;
      x.m[4] = 1.0;
      if (!permute(pend, k, x)) {
        flush();
        permute(pend, k, x);
      }
      emit(x);
      continue;
    }
    // Anything else runs as it is, after the pending factors on its target.
    if (pend.supp & tb) flush();
    emit(op);
  }
  flush();

  const int64_t before = (int64_t)dst.size();
  auto put_table = [&](const DiagTable& d) {
    bool trivial = true;
    for (double a : d.ang)
      if (a != 0.0) {
        trivial = false;
        break;
      }
    if (trivial) return;
    Op p = blank_op();
    p.cls = OP_PHASE;
    p.target = 0;
    p.ctrl = -1;
    p.ctrl_kind = CTRL_NONE;
    p.fh[0] = (int32_t)tab.size();
    p.fh[1] = d.g;
    for (int j = 0; j < d.g; ++j) p.fh[2 + j] = d.gq[j];
    if (tab.capacity() < tab.size() + d.ang.size()) tab.reserve(2 * (tab.size() + d.ang.size()));
    for (double a : d.ang) tab.push_back(entry_of(a));
    dst.push_back(p);
  };
  if (start_table) put_table(tables[0]);
  for (const Item& it : items) {
    if (it.flush) put_table(tables[(size_t)it.table]);
    else dst.push_back(it.op);
  }
  if (scale) scale->mul(acc);
  return (int64_t)dst.size() - before;
}

}  // namespace dmv

// ---------------------------------------------------------------------------
// Host check of the rewrite (dmv_debug_check_fp64_rewrite): both op lists of
// every window pass applied to random tiles in host FP64, compared normwise.
// ---------------------------------------------------------------------------
namespace dmv {
namespace {

struct Cx {
  double re, im;
};

// value_form: apply table entries as the complex value phase_entry_value gives
// (the form the FP32-pair and int64 kernels read) instead of by shears.
// The FP64 kernels' decode of a packed entry (phase_tables_f64): t, s and the
// quadrant bits q & 1 (swap), q >> 1.
void unpack_entry(const double2& p, double& t, double& s, int& b0, int& b1) {
  uint64_t tb, sb;
  std::memcpy(&tb, &p.x, 8);
  std::memcpy(&sb, &p.y, 8);
  const uint64_t top = uint64_t(1) << 62;
  b0 = (int)((tb >> 62) & 1u);
  b1 = (int)((sb >> 62) & 1u);
  tb &= ~top;
  sb &= ~top;
  std::memcpy(&t, &tb, 8);
  std::memcpy(&s, &sb, 8);
}

// value_form false: the table applied as the FP64 kernels do, from the packed
// entries `packed` (phase_tables_f64 of `tab`).
void host_op(std::vector<Cx>& tile, int k, const Op& op, const std::vector<PhaseEntry>& tab, uint64_t base,
             bool value_form = false, const std::vector<double2>* packed = nullptr) {
  const uint32_t T = 1u << k;
  if (op.ctrl_kind == CTRL_GLOBAL && !((base >> op.ctrl) & 1u)) return;
  if (op.cls == OP_PHASE) {
    uint32_t gsel = 0;
    for (int j = 0; j < op.fh[1]; ++j) gsel |= (uint32_t)((base >> op.fh[2 + j]) & 1u) << j;
    for (uint32_t l = 0; l < T; ++l) {
      const PhaseEntry& e = tab[(size_t)op.fh[0] + ((size_t)gsel << k) + l];
      Cx v = tile[l];
      if (value_form) {
        double re, im;
        phase_entry_value(e, re, im);
        tile[l] = Cx{re * v.re - im * v.im, re * v.im + im * v.re};
        continue;
      }
      double t = e.t, sv = e.s;
      int b0 = (int)e.swap_xy, b1 = e.sign_y ? 1 : 0;
      if (packed) unpack_entry((*packed)[(size_t)op.fh[0] + ((size_t)gsel << k) + l], t, sv, b0, b1);
      const double x1 = std::fma(t, v.im, v.re);
      const double y1 = std::fma(sv, x1, v.im);
      const double x2 = std::fma(t, y1, x1);
      double ox = b0 ? y1 : x2, oy = b0 ? x2 : y1;
      if (b0 ^ b1) ox = -ox;  // sign_x: q = 1 or 2
      if (b1) oy = -oy;       // sign_y: q = 2 or 3
      tile[l] = Cx{ox, oy};
    }
    return;
  }
  const uint32_t tb = 1u << op.target;
  for (uint32_t l0 = 0; l0 < T; ++l0) {
    if (l0 & tb) continue;
    if (op.ctrl_kind == CTRL_LOCAL && !((l0 >> op.ctrl) & 1u)) continue;
    const uint32_t l1 = l0 | tb;
    Cx a0 = tile[l0], a1 = tile[l1];
    if (op.cls == OP_ROT) {
      const double w = op.m[0];
      const double x0 = a0.re, x1 = a1.re, y0 = a0.im, y1 = a1.im;
      if (op.m[1] == 0.0) {
        tile[l0] = Cx{std::fma(-w, x1, x0), std::fma(-w, y1, y0)};
        tile[l1] = Cx{std::fma(w, x0, x1), std::fma(w, y0, y1)};
      } else {
        tile[l0] = Cx{std::fma(w, x0, -x1), std::fma(w, y0, -y1)};
        tile[l1] = Cx{std::fma(w, x1, x0), std::fma(w, y1, y0)};
      }
    } else {
      const double* m = op.m;
      tile[l0] = Cx{m[0] * a0.re - m[1] * a0.im + m[2] * a1.re - m[3] * a1.im,
                    m[0] * a0.im + m[1] * a0.re + m[2] * a1.im + m[3] * a1.re};
      tile[l1] = Cx{m[4] * a0.re - m[5] * a0.im + m[6] * a1.re - m[7] * a1.im,
                    m[4] * a0.im + m[5] * a0.re + m[6] * a1.im + m[7] * a1.re};
    }
  }
}

}  // namespace
}  // namespace dmv

extern "C" int dmv_debug_check_fp64_rewrite(const dmv_gate_t* gates, int64_t num_gates, int32_t num_qubits,
                                            uint64_t seed, double* max_err, int64_t* counts) {
  using namespace dmv;
  clear_error();
  if (num_qubits < 12 || num_qubits > 34 || !max_err)
    return set_error(DMV_ERR_INVALID, "dmv_debug_check_fp64_rewrite: num_qubits %d outside [12, 34]", num_qubits);
  std::vector<Gate> g;
  DMV_TRY(parse_gates(gates, num_gates, num_qubits, g));
  PlanOptions opt;
  opt.fusion = DMV_FUSE_WINDOW;
  opt.tile_bits = 12;
  Plan plan;
  DMV_TRY(build_plan(g, num_qubits, DMV_C128, opt, plan));
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto rnd = [&]() {  // SplitMix64
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  double worst = 0.0;
  int64_t n_rot = 0, n_phase = 0, n_general = 0, n_passes = 0;
  // the threaded rewrite (what launch_plan runs) must give every pass exactly
  // the sequential result
  std::vector<int64_t> which;
  for (size_t i = 0; i < plan.passes.size(); ++i)
    if (plan.passes[i].kind == 1) which.push_back((int64_t)i);
  std::vector<RewrittenPass> threaded[2];
  rewrite_passes(plan, which, true, threaded[0]);
  rewrite_passes(plan, which, false, threaded[1]);
  size_t wi = 0;
  for (const Pass& ps : plan.passes) {
    if (ps.kind != 1) continue;
    const size_t j = wi++;
    const int k = ps.low_bits + ps.num_high;
    for (int form = 0; form < 2; ++form) {
      std::vector<Op> rw;
      std::vector<PhaseEntry> tab;
      ScaleDD scale;
      rewrite_pass_rotations(plan.ops.data() + ps.op_begin, ps.op_count, k, form == 0, rw, tab, &scale);
      const RewrittenPass& t = threaded[form][j];
      if (t.ops.size() != rw.size() || t.tab.size() != tab.size() || t.scale.hi != scale.hi ||
          t.scale.lo != scale.lo || (!rw.empty() && std::memcmp(t.ops.data(), rw.data(), rw.size() * sizeof(Op))) ||
          (!tab.empty() && std::memcmp(t.tab.data(), tab.data(), tab.size() * sizeof(PhaseEntry))))
        return set_error(DMV_ERR_INVALID, "threaded rewrite of pass %zu differs from the sequential one", j);
    }
    if (k != 12 || ps.num_high < 3) continue;
    ++n_passes;
    for (int form = 0; form < 2; ++form) {  // rotations as OP_ROT (FP64), then as real 2x2 ops
    std::vector<Op> rw;
    std::vector<PhaseEntry> tab;
    ScaleDD scale;
    rewrite_pass_rotations(plan.ops.data() + ps.op_begin, ps.op_count, k, form == 0, rw, tab, &scale);
    std::vector<double2> packed;
    phase_tables_f64(tab, packed);
    if (form == 0)
      for (const Op& o : rw) {
        n_rot += o.cls == OP_ROT;
        n_phase += o.cls == OP_PHASE;
      }
    if (form == 0)
      for (int64_t o = 0; o < ps.op_count; ++o) n_general += plan.ops[(size_t)(ps.op_begin + o)].cls != OP_SWAP;
    // local bit j of the tile index sits at global qubit pos[j]
    int pos[12];
    for (int j = 0; j < ps.low_bits; ++j) pos[j] = j;
    for (int j = 0; j < ps.num_high; ++j) pos[ps.low_bits + j] = ps.high[j];
    for (int trial = 0; trial < 2; ++trial) {
      uint64_t base = rnd() & ((num_qubits >= 64 ? ~0ull : (1ull << num_qubits) - 1));
      for (int j = 0; j < k; ++j) base &= ~(1ull << pos[j]);
      std::vector<Cx> a(size_t(1) << k), b;
      for (Cx& v : a) v = Cx{((double)(rnd() >> 11) * 0x1.0p-53) - 0.5, ((double)(rnd() >> 11) * 0x1.0p-53) - 0.5};
      b = a;
      // the original ops index controls outside the tile by global qubit; the host
      // emulation reads them from `base`, as the kernel does
      for (int64_t o = 0; o < ps.op_count; ++o) host_op(a, k, plan.ops[(size_t)(ps.op_begin + o)], tab, base);
      for (const Op& o : rw) host_op(b, k, o, tab, base, form == 1, form == 0 ? &packed : nullptr);
      for (Cx& v : b) v = Cx{v.re * scale.hi, v.im * scale.hi};  // the rotations' factors
      double num = 0.0, den = 0.0;
      for (size_t i = 0; i < a.size(); ++i) {
        num = std::max(num, std::hypot(a[i].re - b[i].re, a[i].im - b[i].im));
        den = std::max(den, std::hypot(a[i].re, a[i].im));
      }
      const double e = den > 0 ? num / den : num;
      worst = std::isfinite(e) ? std::max(worst, e) : INFINITY;  // NaN must not pass as 0
    }
    }
  }
  *max_err = worst;
  if (counts) {
    counts[0] = n_passes;
    counts[1] = n_general;
    counts[2] = n_rot;
    counts[3] = n_phase;
  }
  return DMV_OK;
}
