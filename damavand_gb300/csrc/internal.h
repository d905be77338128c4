// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <cmath>
#include <vector>

#include "../../include/damavand_gpu.h"

namespace dmv {

// ---------------------------------------------------------------------------
// Error reporting: every entry point returns a status and records the last
// error (thread-local) with a message. Nothing calls exit().
// ---------------------------------------------------------------------------
int set_error(int code, const char* fmt, ...);
void clear_error();
int last_error();

#define DMV_CUDA_TRY(expr)                                                           \
  do {                                                                               \
    cudaError_t dmv_e_ = (expr);                                                     \
    if (dmv_e_ != cudaSuccess) {                                                     \
      return ::dmv::set_error(dmv_e_ == cudaErrorMemoryAllocation ? DMV_ERR_OOM      \
                                                                  : DMV_ERR_CUDA,    \
                              "%s failed: %s (%s:%d)", #expr,                        \
                              cudaGetErrorString(dmv_e_), __FILE__, __LINE__);       \
    }                                                                                \
  } while (0)

#define DMV_TRY(expr)                       \
  do {                                      \
    int dmv_rc_ = (expr);                   \
    if (dmv_rc_ != DMV_OK) return dmv_rc_;  \
  } while (0)

// Counts the library's own kernel launches (reported by the benchmark).
void count_launch(int64_t n = 1);

// Test hook (dmv_debug_fail_allocations): true when this device allocation
// must fail as if the device were out of memory.
bool injected_alloc_failure();

// Optional per-launch CUDA-event profiling (dmv_profile_*). prof_begin
// returns a token (or -1 when profiling is off); prof_end closes it.
int64_t prof_begin(int family, cudaStream_t stream, double algorithmic_bytes, double multiply_adds = 0.0);
void prof_end(int64_t token, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Gate matrices and fused-op encoding
// ---------------------------------------------------------------------------
// Op arithmetic classes: the kernels specialise on them to spend as few
// FP64 operations as the matrix allows (FP64 is ~1/70 of FP32 on GB300).
enum OpClass : int32_t {
  OP_GENERAL = 0,  // full complex 2x2
  OP_DIAG = 1,     // m01 = m10 = 0
  OP_SWAP = 2,     // exactly [[0,1],[1,0]] (X, CNOT): a pure exchange
  OP_REAL = 3,     // all four entries real
  OP_ANTI = 4,     // m00 = m11 = 0 (Y and scaled exchanges)
  OP_RXLIKE = 5,   // m00, m11 real and m01, m10 imaginary (RX and its adjoint): 8 multiply-adds
  // Only in window passes rewritten by rewrite_pass_rotations (diag_plan.cpp):
  OP_ROT = 6,      // FP64: real rotation R = [[c, -s], [s, c]] applied as f * M, two multiply-adds per component:
                   //   m[1] == 0: M = [[1, -w], [w, 1]] (w = s/c, f = c); m[1] == 1: M = [[w, -1], [1, w]] (w = c/s, f = s);
                   //   m[0] = w. The state is left divided by f; the caller multiplies the product of the f's back.
  OP_PHASE = 7     // every amplitude times a phase from a table (PhaseEntry); fields below
};

// Control kinds inside a fused pass.
enum CtrlKind : int32_t {
  CTRL_NONE = 0,
  CTRL_LOCAL = 1,   // control qubit is one of the pass's local bits
  CTRL_GLOBAL = 2   // control qubit is outside the tile: constant per tile
};

// One operation as the kernels see it (224 bytes).
struct alignas(16) Op {
  double m[8];        // row-major 2x2, (re, im) pairs
  float mh[8];        // m split into FP32 pairs: m = mh + ml (FP32-pair arithmetic)
  float ml[8];
  int32_t fh[8];      // m as Q.54 fixed point: round(m * 2^54) = fh * 2^31 + fl, fl in [0, 2^31)
  int32_t fl[8];
  int32_t target;     // local bit (fused) or qubit (unfused)
  int32_t ctrl;       // local bit or global qubit, per ctrl_kind
  int32_t ctrl_kind;  // CtrlKind
  int32_t cls;        // OpClass
  int32_t param;      // index of the gradient slot (adjoint) or -1
  int32_t generator;  // 0 none, 1 X, 2 Y, 3 Z: generator of a rotation (adjoint)
  int32_t unitary;    // 1 when m is unitary to 1e-12 (block fixed point relies on it)
  int32_t phase;      // register phase of a fused op (kPhase* below), 0 elsewhere
};
static_assert(sizeof(Op) == 224, "Op layout");

// An OP_PHASE op multiplies amplitude l of a tile (2^k amplitudes) by the
// phase of table entry fh[0] + (gsel << k) + l, where gsel collects the
// tile's bits at the fh[1] (at most 3) global qubits fh[2..4]. An entry holds
// the phase e^{i phi} as i^q e^{i phi'} with |phi'| <= pi/4: (x, y) is
// rotated by phi' with three shears, x += t y, y += s x, x += t y
// (t = -tan(phi'/2), s = sin phi'), then multiplied by i^q: swapped when q is
// odd and the sign words xored into the high halves of x and y.
struct alignas(32) PhaseEntry {
  double t;
  double s;
  uint32_t swap_xy;
  uint32_t sign_x;  // 0 or 0x80000000
  uint32_t sign_y;
  uint32_t pad;
};
static_assert(sizeof(PhaseEntry) == 32, "PhaseEntry layout");
constexpr int kMaxPhaseGlobals = 3;

// Register phases of a fused pass run by the TMA window kernel: each thread
// keeps 2^rb amplitudes of the tile in registers, the ones that differ in rb
// "register bits" of the tile index, and applies every op whose target is a
// register bit without touching shared memory. An op that starts a phase
// carries the phase's register bits; the tile goes through shared memory only
// between phases.
constexpr uint32_t kPhaseStart = 0x80000000u;  // this op starts a phase
// bits 0..15: the phase's register bits, 4 bits each (valid on a phase start)
// bits 16..17: index of the op's target among the register bits
// bits 20..22: 1 + index of the op's local control among them, 0 if not one
constexpr int kPhaseTargetShift = 16;
constexpr int kPhaseCtrlShift = 20;
constexpr int kMaxRegBits = 4;

// An op as the register-phase kernel reads it from its shared-memory op
// table (complex64 passes): the FP32 matrix and the fields the loop tests.
struct alignas(16) PhaseOp {
  float m[8];         // op.mh: the matrix rounded to FP32
  uint32_t phase;     // op.phase
  int32_t ctrl;
  int32_t ctrl_kind;
  int32_t cls;
};
static_assert(sizeof(PhaseOp) == 48, "PhaseOp layout");
// Ops one launch of the register-phase kernel holds in shared memory; a
// longer pass runs as several launches over the same qubits.
constexpr int64_t kMaxPhaseOps = 128;

// Orders one fused pass's ops (tile-local targets) into register phases and
// marks them: each phase holds ops whose targets span at most rb tile bits
// (padded with unused tile bits); ops move across others only where they
// share no tile bit. Returns the number of phases.
int64_t assign_phases(Op* ops, int64_t count, int32_t tile_bits, int32_t rb);

// Fills op.mh / op.ml (FP32 pair: hi = nearest float, lo = nearest float of
// the rest), op.fh / op.fl (Q.54 limbs) and op.unitary from op.m.
void split_matrix(Op& op);

// Rewrites the ops src[0 .. count) of one FP64 window pass over a tile of
// 2^k amplitudes so that it spends fewer FP64 operations: every uncontrolled
// unitary 2x2 becomes D1 R D2 (R a real rotation; D1, D2 diagonal), and the
// diagonal factors of the whole pass (with Z-type
// and controlled-phase ops and the diagonals of Y-type ops) are collected
// into as few per-amplitude phase tables as the rotations allow: a diagonal
// factor moves later in time through exchanges (re-indexed) and through
// rotations on other bits, and earlier into the last table when nothing in
// between touches its bits. Appends the new ops to `dst` and the tables to
// `tab`; returns the number of ops appended.
// `rot_ops` true: rotations as OP_ROT (the FP64 kernels: two multiply-adds
// per component, the state left divided by each rotation's factor f, whose
// product over the pass is multiplied into *scale); false: as OP_REAL 2x2 ops
// (with their FP32-pair, Q.54 and FP32 forms), for the other arithmetics,
// which read the tables converted by phase_entry_value.
// A product of many factors kept to about 2^-100 relative (error-free
// products through fma), for the OP_ROT factors.
struct ScaleDD {
  double hi = 1.0, lo = 0.0;
  void mul(double f) {
    const double p = hi * f;
    const double e = std::fma(hi, f, -p);
    const double l = std::fma(lo, f, e);
    hi = p + l;
    lo = l - (hi - p);
  }
  void mul(const ScaleDD& o) {
    const double p = hi * o.hi;
    const double e = std::fma(hi, o.hi, -p);
    const double l = std::fma(hi, o.lo, std::fma(lo, o.hi, e));
    hi = p + l;
    lo = l - (hi - p);
  }
};
int64_t rewrite_pass_rotations(const Op* src, int64_t count, int32_t k, bool rot_ops, std::vector<Op>& dst,
                               std::vector<PhaseEntry>& tab, ScaleDD* scale = nullptr);
// e^{i phi} of a table entry in double.
void phase_entry_value(const PhaseEntry& e, double& re, double& im);
// The tables in the FP32-pair form (re_h, re_l, im_h, im_l) and as Q.54 limbs
// (re_h, re_l, im_h, im_l: value = h * 2^31 + l, l in [0, 2^31)).
void phase_tables_df(const std::vector<PhaseEntry>& in, std::vector<float4>& out);
// The FP64 kernels' 16-byte form: (t, s) with the quadrant in bit 62 of each
// (0 in both, as |t|, |s| < 2): bit 62 of t = swap_xy = q & 1, bit 62 of s =
// q >> 1 (sign_y); sign_x = the xor of the two.
void phase_tables_f64(const std::vector<PhaseEntry>& in, std::vector<double2>& out);
void phase_tables_fx(const std::vector<PhaseEntry>& in, std::vector<int4>& out);

// Arithmetic used for complex128 storage.
enum Arith : int32_t {
  ARITH_FP64 = 0,    // IEEE FP64 multiply-adds
  ARITH_FP32X2 = 1,  // FP32-pair (double-float) error-free transformations
  ARITH_INT64 = 2,   // int64 block fixed point on the integer pipe
  ARITH_TC = 3       // int64 block fixed point, dense blocks as exact digit products on the tensor cores
};

// Host-side gate after parsing.
struct Gate {
  int32_t kind;
  int32_t target;
  int32_t control;  // -1 none
  double theta;
  double m[8];      // the gate's matrix, computed on the host (gates.cpp)
  bool observable;
};

// Matrix of a gate kind, the formulas of the reference's gates.rs.
void gate_matrix(int32_t kind, double theta, double m[8]);
int32_t classify(const double m[8]);
bool is_parametrised(int32_t kind);
// Generator P of R(theta) = exp(-i theta P / 2): 1 X, 2 Y, 3 Z, 0 none.
int32_t rotation_generator(int32_t kind);
// m = a * b (2x2 complex)
void matmul2(const double a[8], const double b[8], double out[8]);
// Conjugate transpose.
void adjoint2(const double a[8], double out[8]);
int parse_gates(const dmv_gate_t* gates, int64_t num_gates, int32_t n, std::vector<Gate>& out);

// ---------------------------------------------------------------------------
// Execution plan: a sequence of passes over the statevector.
// ---------------------------------------------------------------------------
struct Pass {
  // kind 0: single op on global qubit indices (unfused kernel).
  // kind 1: fused window: local bits = [0, low_bits) + high[0..num_high).
  int32_t kind;
  int32_t low_bits;
  int32_t num_high;
  int32_t high[16];
  int64_t op_begin;  // range in Plan::ops
  int64_t op_count;
};

struct Plan {
  std::vector<Pass> passes;
  std::vector<Op> ops;
  int64_t num_gates = 0;
};

struct PlanOptions {
  int32_t fusion = DMV_FUSE_WINDOW;
  int32_t tile_bits = 12;  // log2 amplitudes per tile
  int32_t low_bits = 6;    // always-local low qubits (coalesced chunks)
  bool windows_only = false;  // every pass a window pass (the batched kernel runs only those)
  // Adjoint sweeps: when set, no gates are merged and the op made from
  // gates[i] carries param_of[i] / generator_of[i] (Op::param, Op::generator).
  const int32_t* param_of = nullptr;
  const int32_t* generator_of = nullptr;
};

int build_plan(const std::vector<Gate>& gates, int32_t n, int32_t precision,
               const PlanOptions& opt, Plan& plan);
// The reverse sweep of an adjoint gradient as a plan: the non-observable gates
// in reverse order, each replaced by U^dagger, unmerged, each op tagged with
// its gate's parameter slot (list order of the parametrised gates) and
// generator (PlanOptions::param_of / generator_of).
int build_adjoint_plan(const std::vector<Gate>& gates, int32_t n, int32_t precision, const PlanOptions& base,
                       Plan& plan);
// rewrite_pass_rotations of several window passes, on host threads: pass
// which[j] of `plan` into out[j] (its own ops, its own tables with OP_PHASE
// offsets from 0, its factor product). Results do not depend on the threads.
struct RewrittenPass {
  std::vector<Op> ops;
  std::vector<PhaseEntry> tab;
  ScaleDD scale;
};
void rewrite_passes(const Plan& plan, const std::vector<int64_t>& which, bool rot_ops,
                    std::vector<RewrittenPass>& out);

// ---------------------------------------------------------------------------
// Tensor-core window passes (ARITH_TC, complex128 storage).
//
// The tile (2^12 amplitudes) is held as int64 block fixed point. A pass is
// cut into stages: exchanges (X, CNOT: integer swaps in shared memory) and
// dense blocks, the product of consecutive ops on at most 5 tile bits as one
// 32 x 32 complex matrix. A block is applied to the tile viewed as 128
// columns of 32 amplitudes: every integer is split into 7 balanced 8-bit
// digits (FP16, exact), the matrix likewise, and the 34 digit products
// whose weights 2^(-8s) have s = i + j <= 7 accumulate exactly in FP32 on the
// tensor cores (tcgen05.mma), one TMEM accumulator per weight.
// ---------------------------------------------------------------------------
constexpr int kTcBlockBits = 5;                             // qubits of a dense block
constexpr int kTcDigits = 7;                                // balanced 8-bit digits of a 56-bit integer
constexpr int kTcURows = 64 * kTcDigits;                    // rows of a block's stacked digit matrix
constexpr int64_t kTcUHalves = (int64_t)kTcURows * 64;      // FP16 elements per block (56 KB)
enum TcStageKind : int32_t { TC_BLOCK = 0, TC_SWAP = 1 };

// Exchanges are not applied to the data: the tile stays where it is and the
// kernel reads logical amplitude l at phys(l) = A l xor c, an affine map over
// the 12 tile bits. A CNOT with a control inside the tile changes A (the host
// tracks it), X and CNOTs controlled from outside the tile change c (the
// kernel, per tile).
struct TcStage {
  int32_t kind;       // TcStageKind
  int32_t img[12];    // block: A e_b for the block's 5 bits (img[0..4], block-row bits 0..4) and its 7
                      // other tile bits (img[5..11], column-index bits 0..6); swap: img[0] = mask xored into c
  int32_t gctrl;      // swap: control qubit outside the tile (c changes on tiles where it is 1), or -1
  int32_t u_index;    // block: index of its digit matrix in the plan's array
  int32_t magic;      // block: 1 when every FP32 accumulator stays below 2^22 in magnitude
  int32_t next_u;     // block: u_index of the pass's next block (cyclically), fetched during this one's epilogue
  int32_t pad[3];
};
static_assert(sizeof(TcStage) == 80, "TcStage layout");

// Cuts window pass `ps` of `plan` (a 2^12-amplitude tile) into stages,
// appended to `stages`, and appends each block's digit matrix (kTcUHalves
// FP16 bit patterns in the tensor cores' K-major layout) to `u`. Returns
// false, appending nothing, when the pass holds an op the tensor-core kernel
// does not take (a non-unitary op, or a non-exchange op controlled from
// outside the tile).
// `final_map` receives A e_b (b = 0..11) after the pass's last stage and
// `exchanges` the number of X / CNOT ops applied as relabellings.
bool build_tc_pass(const Plan& plan, const Pass& ps, std::vector<TcStage>& stages, std::vector<uint16_t>& u,
                   int32_t final_map[12], int32_t* exchanges);
// Test hook (dmv_debug_tc_convert): 1 forces the exact conversion in every block.
void set_tc_convert_mode(int32_t mode);

// ---------------------------------------------------------------------------
// Device state
// ---------------------------------------------------------------------------
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  int reserve(size_t n);
  void release();
};

}  // namespace dmv

struct dmv_state_s {
  int32_t n = 0;
  int64_t N = 0;
  int32_t precision = DMV_C128;
  int32_t arith = dmv::ARITH_FP64;  // complex128 arithmetic (ignored for complex64)
  int device = 0;
  void* amps = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  dmv::DeviceBuffer ops_dev;     // plan ops uploaded for the last apply
  dmv::DeviceBuffer reduce_dev;  // reduction partials
  dmv::DeviceBuffer chunk_dev;   // per-chunk probability sums (sampling)
  std::vector<dmv::Op> ops_host_pinned;  // (regular host memory; copied async from a pinned staging)
  std::vector<dmv::Op> ops_staging;      // plan ops with register phases marked, as uploaded
  std::vector<dmv::Pass> pass_staging;   // the launches of the last plan (long phase passes split)
  std::vector<dmv::PhaseOp> phase_ops;   // compact ops of the register-phase launches
  dmv::DeviceBuffer phase_ops_dev;
  std::vector<dmv::PhaseEntry> phase_tab;  // phase tables of the rewritten passes
  std::vector<dmv::ScaleDD> pass_scale;  // launch_plan: OP_ROT factor product per staged pass
  dmv::DeviceBuffer phase_tab_dev;
  std::vector<double2> phase_tab_f64;      // the tables in the FP64 kernels' 16-byte form
  std::vector<float4> phase_tab_df;        // the same tables for the FP32-pair arithmetic
  std::vector<int4> phase_tab_fx;          // and for the int64 arithmetic
  dmv::DeviceBuffer phase_tab2_dev;
  std::vector<dmv::TcStage> tc_stages;  // tensor-core passes of the last plan
  std::vector<uint16_t> tc_u;
  dmv::DeviceBuffer tc_stages_dev, tc_u_dev;
  void* pinned = nullptr;        // pinned host staging
  size_t pinned_bytes = 0;
  int64_t last_passes = 0, last_ops = 0, last_bytes = 0;
  int64_t last_tc_passes = 0, last_tc_blocks = 0, last_tc_swaps = 0;
  int64_t last_phase_tab_bytes = 0;  // phase tables uploaded by the last plan
  int64_t last_upload_bytes = 0;     // every host-to-device byte of the last plan (ops, tables, digit matrices)
  bool fp64_rewrite = true;          // FP64 window passes as rotations and phase tables
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  size_t amp_bytes() const { return (size_t)N * (precision == DMV_C128 ? 16 : 8); }
};

namespace dmv {
int ensure_pinned(dmv_state_s* s, size_t bytes);

// Planner settings for a state: tiles of 2^12 amplitudes (the TMA window
// kernel's register phases hold 8 per thread of 512).
inline PlanOptions plan_options_for(const dmv_state_s* s, int32_t fusion) {
  (void)s;
  PlanOptions opt;
  opt.fusion = fusion;
  opt.tile_bits = 12;
  return opt;
}

// Kernel launchers (kernels_*.cu). All stream-ordered on s->stream.
int launch_set_zero(dmv_state_s* s);
// The state times a real factor (complex128).
int launch_scale_state(dmv_state_s* s, double f);
int launch_plan(dmv_state_s* s, const Plan& plan);
int launch_probabilities(dmv_state_s* s, double* probs_device);
int launch_expect_z(dmv_state_s* s, double* expect_host, double* norm_host);
int launch_sample(dmv_state_s* s, const double* uniforms_host, int64_t k, uint64_t* samples_host);
// Draws k samples on the device (uniforms from the host, or from the seeded
// SplitMix64 stream when uniforms_host is null) and counts, per bit position,
// the samples with that bit set; the samples never leave the device.
int launch_sample_counts(dmv_state_s* s, const double* uniforms_host, uint64_t seed, int64_t k,
                         unsigned long long counts_host[64]);
int sample_from_device_probs(const double* probs_device, int64_t num_probs, int32_t num_bits,
                             cudaStream_t stream, const double* uniforms_host, int64_t k,
                             uint64_t* samples_host);
int launch_inner_product(dmv_state_s* a, dmv_state_s* b, double* re, double* im);
int launch_scale_by_z_observable(dmv_state_s* dst, dmv_state_s* src, const double* weights_host);
int launch_adjoint_step(dmv_state_s* psi, dmv_state_s* lam, const Op& op, double* grad_slot_device);
int adjoint_gradient(dmv_state_s* s, const std::vector<Gate>& gates, const double* weights,
                     double* loss, double* grads);
int upload_ops(dmv_state_s* s, const Op* ops, int64_t count);
// DMV_ERR_TIMEOUT (and clears the flag) when a TMA window pass or the
// bulk-staged chunk-mass pass gave up waiting for a load since the last
// check; synchronises the device.
int check_window_status();
// Polls before a TMA load wait gives up; negative restores the default.
void set_tma_wait_limit(int64_t polls);
uint32_t tma_wait_limit();
// The device word those waits set to 1 when they give up.
int* tma_status_word();

// Pauli-Z mass reduction into caller-provided device buffers: `partial`
// holds partial_elems doubles, `sums` n+1 (mass with bit q set for q < n,
// then the total).
struct ChunkMassShape {
  int chunk_bits;
  int64_t num_chunks;
  int grid;
  int64_t partial_elems;
};
ChunkMassShape chunk_mass_shape(int n);
int launch_chunk_mass_into(const void* src, int src_kind, int n, double* partial, double* sums,
                           cudaStream_t stream);
}  // namespace dmv
