// Gate matrices, op classification and the pass planner (host C++).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"

namespace dmv {

// Matrices follow src/qubit_backend/gates.rs: Hadamard :97-119 (1/sqrt(2)),
// PauliX :223-233, PauliY :288-298, PauliZ :352-362, RotationX :417-439,
// RotationY :489-511, RotationZ :561-577. CNOT uses the PauliX matrix
// (src/qubit_backend/circuit_multithreading.rs:14-20). The same libm calls as
// the oracle produce the coefficients, so both sides start from identical
// doubles.
void gate_matrix(int32_t kind, double theta, double m[8]) {
  std::memset(m, 0, 8 * sizeof(double));
  switch (kind) {
    case DMV_GATE_H: {
      const double h = 1. / std::sqrt(2.0);
      m[0] = h; m[2] = h; m[4] = h; m[6] = -1. / std::sqrt(2.0);
      break;
    }
    case DMV_GATE_X:
    case DMV_GATE_CNOT:
      m[2] = 1.; m[4] = 1.;
      break;
    case DMV_GATE_Y:
      m[3] = -1.; m[5] = 1.;
      break;
    case DMV_GATE_Z:
      m[0] = 1.; m[6] = -1.;
      break;
    case DMV_GATE_RX:
      m[0] = std::cos(theta / 2.); m[3] = -std::sin(theta / 2.);
      m[5] = -std::sin(theta / 2.); m[6] = std::cos(theta / 2.);
      break;
    case DMV_GATE_RY:
      m[0] = std::cos(theta / 2.); m[2] = -std::sin(theta / 2.);
      m[4] = std::sin(theta / 2.); m[6] = std::cos(theta / 2.);
      break;
    case DMV_GATE_RZ:
      m[0] = std::cos(-theta / 2.); m[1] = std::sin(-theta / 2.);
      m[6] = std::cos(theta / 2.); m[7] = std::sin(theta / 2.);
      break;
    default:
      break;
  }
}

bool is_parametrised(int32_t kind) {
  return kind == DMV_GATE_RX || kind == DMV_GATE_RY || kind == DMV_GATE_RZ;
}

int32_t rotation_generator(int32_t kind) {
  switch (kind) {
    case DMV_GATE_RX: return 1;
    case DMV_GATE_RY: return 2;
    case DMV_GATE_RZ: return 3;
    default: return 0;
  }
}

int32_t classify(const double m[8]) {
  const bool off_zero = m[2] == 0. && m[3] == 0. && m[4] == 0. && m[5] == 0.;
  const bool diag_zero = m[0] == 0. && m[1] == 0. && m[6] == 0. && m[7] == 0.;
  if (diag_zero && m[2] == 1. && m[3] == 0. && m[4] == 1. && m[5] == 0.) return OP_SWAP;
  if (off_zero) return OP_DIAG;
  if (diag_zero) return OP_ANTI;
  if (m[1] == 0. && m[3] == 0. && m[5] == 0. && m[7] == 0.) return OP_REAL;
  if (m[1] == 0. && m[7] == 0. && m[2] == 0. && m[4] == 0.) return OP_RXLIKE;
  return OP_GENERAL;
}

void split_matrix(Op& op) {
  bool bounded = true;
  for (int i = 0; i < 8; ++i) {
    const float hi = (float)op.m[i];
    op.mh[i] = hi;
    op.ml[i] = (float)(op.m[i] - (double)hi);
    if (!(std::fabs(op.m[i]) <= 1.0)) bounded = false;
    const long long f = bounded ? std::llround(std::ldexp(op.m[i], 54)) : 0;  // |f| <= 2^54
    op.fh[i] = (int32_t)(f >> 31);
    op.fl[i] = (int32_t)(f & 0x7FFFFFFFll);
  }
  // U^dagger U = I to 1e-12: the fixed-point headroom argument needs unitarity.
  double worst = bounded ? 0.0 : 1.0;
  for (int r = 0; r < 2 && bounded; ++r)
    for (int c = 0; c < 2; ++c) {
      double re = 0., im = 0.;
      for (int k = 0; k < 2; ++k) {  // sum_k conj(m[k][r]) m[k][c]
        const double ar = op.m[2 * (2 * k + r)], ai = -op.m[2 * (2 * k + r) + 1];
        const double br = op.m[2 * (2 * k + c)], bi = op.m[2 * (2 * k + c) + 1];
        re += ar * br - ai * bi;
        im += ar * bi + ai * br;
      }
      worst = std::max(worst, std::fabs(re - (r == c ? 1.0 : 0.0)) + std::fabs(im));
    }
  op.unitary = worst <= 1e-12 ? 1 : 0;
}

void matmul2(const double a[8], const double b[8], double out[8]) {
  double r[8];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      double re = 0., im = 0.;
      for (int k = 0; k < 2; ++k) {
        const double ar = a[2 * (2 * i + k)], ai = a[2 * (2 * i + k) + 1];
        const double br = b[2 * (2 * k + j)], bi = b[2 * (2 * k + j) + 1];
        re += ar * br - ai * bi;
        im += ar * bi + ai * br;
      }
      r[2 * (2 * i + j)] = re;
      r[2 * (2 * i + j) + 1] = im;
    }
  std::memcpy(out, r, sizeof(r));
}

void adjoint2(const double a[8], double out[8]) {
  double r[8];
  r[0] = a[0]; r[1] = -a[1];  // m00*
  r[2] = a[4]; r[3] = -a[5];  // m10*
  r[4] = a[2]; r[5] = -a[3];  // m01*
  r[6] = a[6]; r[7] = -a[7];  // m11*
  std::memcpy(out, r, sizeof(r));
}

int parse_gates(const dmv_gate_t* gates, int64_t num_gates, int32_t n, std::vector<Gate>& out) {
  out.clear();
  if (num_gates < 0 || (num_gates > 0 && gates == nullptr))
    return set_error(DMV_ERR_INVALID, "gate list: null pointer or negative count");
  out.reserve((size_t)num_gates);
  for (int64_t i = 0; i < num_gates; ++i) {
    const dmv_gate_t& g = gates[i];
    if (g.kind < DMV_GATE_H || g.kind > DMV_GATE_MATRIX)
      return set_error(DMV_ERR_INVALID, "gate %lld: unknown kind %d", (long long)i, g.kind);
    if (g.target < 0 || g.target >= n)
      return set_error(DMV_ERR_INVALID, "gate %lld: target qubit %d out of range [0,%d)",
                       (long long)i, g.target, n);
    int32_t control = g.control;
    if (g.kind == DMV_GATE_CNOT && control < 0)
      return set_error(DMV_ERR_INVALID, "gate %lld: CNOT needs a control qubit", (long long)i);
    if (control >= n || control < -1)
      return set_error(DMV_ERR_INVALID, "gate %lld: control qubit %d out of range", (long long)i,
                       control);
    if (control == g.target)
      return set_error(DMV_ERR_INVALID, "gate %lld: control equals target (%d)", (long long)i,
                       control);
    Gate h;
    h.kind = g.kind;
    h.target = g.target;
    h.control = control;
    h.theta = g.theta;
    h.observable = false;
    if (g.kind == DMV_GATE_MATRIX) {
      std::memcpy(h.m, g.m, sizeof(h.m));
      for (double v : h.m)
        if (!std::isfinite(v)) return set_error(DMV_ERR_INVALID, "gate %lld: non-finite matrix", (long long)i);
    } else {
      gate_matrix(g.kind, g.theta, h.m);
    }
    out.push_back(h);
  }
  return DMV_OK;
}

// ---------------------------------------------------------------------------
// Planner
// ---------------------------------------------------------------------------
namespace {

struct PGate {
  int32_t target, control;
  double m[8];
  int32_t param, generator;  // adjoint tags (PlanOptions::param_of), else -1 / 0
};

Op make_op(const PGate& g, int32_t target_pos, int32_t ctrl, int32_t ctrl_kind) {
  Op op;
  std::memset(&op, 0, sizeof(op));
  std::memcpy(op.m, g.m, sizeof(op.m));
  split_matrix(op);
  op.target = target_pos;
  op.ctrl = ctrl;
  op.ctrl_kind = ctrl_kind;
  op.cls = classify(g.m);
  op.param = g.param;
  op.generator = g.generator;
  return op;
}

inline uint64_t qbit(int32_t q) { return q >= 0 ? (uint64_t(1) << q) : 0; }

}  // namespace

int build_plan(const std::vector<Gate>& gates, int32_t n, int32_t precision,
               const PlanOptions& opt, Plan& plan) {
  plan.passes.clear();
  plan.ops.clear();
  plan.num_gates = 0;

  // 1. Merge runs of uncontrolled gates on one qubit into one 2x2 (later
  //    gate multiplies from the left). A run ends at any gate that touches
  //    the qubit, as target or as control.
  std::vector<PGate> fg;
  fg.reserve(gates.size());
  std::vector<int64_t> last_on((size_t)n, -1);
  const bool tagged = opt.param_of != nullptr;
  for (size_t gi = 0; gi < gates.size(); ++gi) {
    const Gate& g = gates[gi];
    if (g.observable) continue;
    ++plan.num_gates;
    if (opt.fusion != DMV_FUSE_NONE && g.control < 0 && !tagged) {
      const int64_t j = last_on[(size_t)g.target];
      if (j >= 0 && fg[(size_t)j].control < 0 && fg[(size_t)j].target == g.target) {
        matmul2(g.m, fg[(size_t)j].m, fg[(size_t)j].m);
        continue;
      }
    }
    PGate p;
    p.target = g.target;
    p.control = g.control;
    std::memcpy(p.m, g.m, sizeof(p.m));
    p.param = tagged ? opt.param_of[gi] : -1;
    p.generator = tagged && opt.generator_of ? opt.generator_of[gi] : 0;
    fg.push_back(p);
    last_on[(size_t)g.target] = (int64_t)fg.size() - 1;
    if (g.control >= 0) last_on[(size_t)g.control] = (int64_t)fg.size() - 1;
  }

  auto emit_single = [&](const PGate& g) {
    Pass ps;
    std::memset(&ps, 0, sizeof(ps));
    ps.kind = 0;
    ps.op_begin = (int64_t)plan.ops.size();
    ps.op_count = 1;
    plan.ops.push_back(make_op(g, g.target, g.control, g.control >= 0 ? CTRL_GLOBAL : CTRL_NONE));
    plan.passes.push_back(ps);
  };

  const int32_t k = std::min(opt.tile_bits, n);
  if (!opt.windows_only && (opt.fusion == DMV_FUSE_NONE || k < 2)) {
    for (const PGate& g : fg) emit_single(g);
    return DMV_OK;
  }
  const int32_t low = std::min(opt.low_bits, k);
  const uint64_t all_mask = n >= 64 ? ~uint64_t(0) : ((uint64_t(1) << n) - 1);
  (void)precision;

  // 2. Qubit-window passes. Each pass keeps `k` qubits local to a tile: the
  //    `low` lowest ones (contiguous chunks in HBM) and the first other
  //    targets met in the pending list. A list-order sweep then takes every
  //    gate whose target is local and none of whose qubits is blocked by an
  //    earlier gate left pending; a gate left pending blocks its qubits.
  std::vector<int64_t> pending(fg.size());
  for (size_t i = 0; i < fg.size(); ++i) pending[i] = (int64_t)i;
  std::vector<int64_t> keep, take;
  while (!pending.empty()) {
    uint64_t local = (uint64_t(1) << low) - 1;
    int32_t nlocal = low;
    for (int64_t gi : pending) {
      if (nlocal >= k) break;
      const int32_t t = fg[(size_t)gi].target;
      if (!(local & qbit(t))) { local |= qbit(t); ++nlocal; }
    }
    for (int32_t q = 0; q < n && nlocal < k; ++q)
      if (!(local & qbit(q))) { local |= qbit(q); ++nlocal; }

    keep.clear();
    take.clear();
    uint64_t blocked = 0;
    for (size_t idx = 0; idx < pending.size(); ++idx) {
      const int64_t gi = pending[idx];
      const PGate& g = fg[(size_t)gi];
      const uint64_t qs = qbit(g.target) | qbit(g.control);
      if (blocked == all_mask) { keep.insert(keep.end(), pending.begin() + (int64_t)idx, pending.end()); break; }
      if ((qs & blocked) || !(local & qbit(g.target))) {
        blocked |= qs;
        keep.push_back(gi);
      } else {
        take.push_back(gi);
      }
    }
    if (take.empty()) {  // cannot happen (the first pending gate's target is local); guard anyway
      emit_single(fg[(size_t)pending.front()]);
      pending.erase(pending.begin());
      continue;
    }
    if (take.size() == 1 && !opt.windows_only) {
      emit_single(fg[(size_t)take.front()]);
    } else {
      Pass ps;
      std::memset(&ps, 0, sizeof(ps));
      ps.kind = 1;
      ps.low_bits = low;
      ps.num_high = 0;
      int32_t pos_of[64];
      for (int32_t q = 0; q < 64; ++q) pos_of[q] = -1;
      for (int32_t q = 0; q < low; ++q) pos_of[q] = q;
      for (int32_t q = low; q < n; ++q)
        if (local & qbit(q)) {
          pos_of[q] = low + ps.num_high;
          ps.high[ps.num_high++] = q;
        }
      ps.op_begin = (int64_t)plan.ops.size();
      for (int64_t gi : take) {
        const PGate& g = fg[(size_t)gi];
        int32_t ctrl = -1, ck = CTRL_NONE;
        if (g.control >= 0) {
          if (pos_of[g.control] >= 0) { ctrl = pos_of[g.control]; ck = CTRL_LOCAL; }
          else { ctrl = g.control; ck = CTRL_GLOBAL; }
        }
        plan.ops.push_back(make_op(g, pos_of[g.target], ctrl, ck));
      }
      ps.op_count = (int64_t)take.size();
      plan.passes.push_back(ps);
    }
    pending.swap(keep);
  }
  return DMV_OK;
}

int64_t assign_phases(Op* ops, int64_t count, int32_t tile_bits, int32_t rb) {
  // Phases are built by list scheduling: each phase sweeps the remaining ops
  // in order (up to kLookahead of them) and takes every op whose target is,
  // or can still become, one of the phase's rb register bits and none of
  // whose tile bits is used by an op the sweep left behind. Ops that share
  // no tile bit commute, so the order within the pass may change; ops that
  // share one keep their order.
  constexpr int64_t kLookahead = 256;
  const std::vector<Op> in(ops, ops + count);
  std::vector<char> done((size_t)count, 0);
  int64_t out = 0, first = 0, phases = 0;
  while (out < count) {
    while (done[(size_t)first]) ++first;
    int32_t reg[kMaxRegBits] = {0, 0, 0, 0};
    int32_t nr = 0;
    uint32_t rmask = 0, blocked = 0;
    const int64_t begin = out;
    int64_t seen = 0;
    for (int64_t i = first; i < count && seen < kLookahead; ++i) {
      if (done[(size_t)i]) continue;
      ++seen;
      const Op& op = in[(size_t)i];
      uint32_t qs = 1u << op.target;
      if (op.ctrl_kind == CTRL_LOCAL) qs |= 1u << op.ctrl;
      if (qs & blocked) {
        blocked |= qs;
        continue;
      }
      if (!((rmask >> op.target) & 1u)) {
        if (nr == rb) {
          blocked |= qs;
          continue;
        }
        reg[nr++] = op.target;
        rmask |= 1u << op.target;
      }
      ops[out++] = op;
      done[(size_t)i] = 1;
    }
    for (int32_t pos = 0; nr < rb && pos < tile_bits; ++pos)
      if (!((rmask >> pos) & 1u)) {
        reg[nr++] = pos;
        rmask |= 1u << pos;
      }
    for (int64_t j = begin; j < out; ++j) {
      Op& op = ops[j];
      uint32_t v = 0;
      if (j == begin) {
        v |= kPhaseStart;
        for (int32_t b = 0; b < rb; ++b) v |= (uint32_t)reg[b] << (4 * b);
      }
      for (int32_t b = 0; b < rb; ++b) {
        if (reg[b] == op.target) v |= (uint32_t)b << kPhaseTargetShift;
        if (op.ctrl_kind == CTRL_LOCAL && reg[b] == op.ctrl) v |= (uint32_t)(b + 1) << kPhaseCtrlShift;
      }
      op.phase = (int32_t)v;
    }
    ++phases;
  }
  return phases;
}

int build_adjoint_plan(const std::vector<Gate>& gates, int32_t n, int32_t precision, const PlanOptions& base,
                       Plan& plan) {
  std::vector<Gate> rev;
  std::vector<int32_t> param, gen;
  int32_t slots = 0;
  for (const Gate& g : gates)
    if (!g.observable && is_parametrised(g.kind)) ++slots;
  rev.reserve(gates.size());
  for (int64_t gi = (int64_t)gates.size() - 1; gi >= 0; --gi) {
    const Gate& g = gates[(size_t)gi];
    if (g.observable) continue;
    Gate h = g;
    adjoint2(g.m, h.m);
    rev.push_back(h);
    const bool p = is_parametrised(g.kind);
    if (p) --slots;  // slots now the list-order index of this gate's parameter
    param.push_back(p ? slots : -1);
    gen.push_back(p ? rotation_generator(g.kind) : 0);
  }
  PlanOptions opt = base;
  opt.param_of = param.data();
  opt.generator_of = gen.data();
  return build_plan(rev, n, precision, opt, plan);
}

}  // namespace dmv

extern "C" int dmv_debug_adjoint_plan(const dmv_gate_t* gates, int64_t num_gates, int32_t num_qubits,
                                      int64_t* counts) {
  using namespace dmv;
  clear_error();
  if (!counts) return set_error(DMV_ERR_INVALID, "dmv_debug_adjoint_plan: null counts");
  std::vector<Gate> g;
  DMV_TRY(parse_gates(gates, num_gates, num_qubits, g));
  PlanOptions opt;
  opt.fusion = DMV_FUSE_WINDOW;
  opt.tile_bits = 12;
  Plan plan;
  DMV_TRY(build_adjoint_plan(g, num_qubits, DMV_C128, opt, plan));
  int64_t windows = 0, tagged = 0, max_param = -1, mismatched = 0;
  for (const Pass& ps : plan.passes) windows += ps.kind == 1;
  for (const Op& op : plan.ops) {
    if (op.param >= 0) {
      ++tagged;
      max_param = std::max<int64_t>(max_param, op.param);
    }
    if ((op.param >= 0) != (op.generator != 0)) ++mismatched;
  }
  counts[0] = (int64_t)plan.passes.size();
  counts[1] = windows;
  counts[2] = (int64_t)plan.ops.size();
  counts[3] = tagged;
  counts[4] = max_param + 1;
  counts[5] = mismatched;
  return DMV_OK;
}
