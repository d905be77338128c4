/*
 * damavand_gpu.h -- C ABI of libdamavand_gpu.so, the GB300 (sm_103a)
 * statevector gate-application library.
 *
 * Two layers:
 *
 *  1. LEGACY entry points. Same names and C types as the functions the
 *     reference's Rust front-end declares (src/qubit_backend/circuit.rs:27-51,
 *     src/qubit_backend/circuit_gpu.rs:3-24,
 *     src/qubit_backend/circuit_distributed_gpu.rs:6-33) and defines in
 *     damavand-gpu/rust_communication.cu, so an unchanged
 *     `cargo build --features gpu` links against this library. They drive one
 *     process-global state on device 0. The `int` sizes limit them to 30 qubits.
 *     Errors no longer exit() the process: they print one line to stderr and
 *     set the code returned by dmv_last_error().
 *
 *  2. dmv_* entry points: an opaque state handle, int64 sizes (up to 34
 *     qubits, memory permitting), an int status return, stream-ordered
 *     execution, batched gate lists (fused into few passes over HBM),
 *     probabilities / Pauli-Z expectation / sampling with injected uniforms,
 *     an adjoint gradient, and complex128 or complex64 storage.
 *
 * Amplitude layout on the device: interleaved complex (re, im), 16 bytes per
 * amplitude for complex128 and 8 for complex64. Qubit q is bit q of the
 * amplitude index (little-endian), as in the reference.
 */
#ifndef DAMAVAND_GPU_H
#define DAMAVAND_GPU_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes (dmv_* return values; also dmv_last_error())                 */
/* ------------------------------------------------------------------------ */
enum {
  DMV_OK = 0,
  DMV_ERR_INVALID = 1,     /* bad argument: qubit index, size, null pointer, ... */
  DMV_ERR_OOM = 2,         /* device or pinned-host allocation failed */
  DMV_ERR_CUDA = 3,        /* CUDA runtime error (message in dmv_last_error_string) */
  DMV_ERR_NO_DEVICE = 4,   /* no CUDA device visible */
  DMV_ERR_UNSUPPORTED = 5, /* multi-GPU / distributed entry points */
  DMV_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
  DMV_ERR_STATE = 7        /* call out of order (e.g. legacy call before init) */
};

/* Precision of the stored amplitudes. */
enum { DMV_C128 = 0, DMV_C64 = 1 };

/* Arithmetic of complex128 gate application (complex64 always computes in FP32).
 * The amplitudes are IEEE complex128 in device memory between calls in every mode.
 * DMV_ARITH_FP64: IEEE FP64 arithmetic (default). Fused window passes on the
 *   TMA kernel write each uncontrolled unitary 2x2 as diagonal x real rotation
 *   x diagonal, apply the rotation as a scaled matrix with one FP64
 *   multiply-add per output (2 per amplitude instead of 8; the product of the
 *   scale factors is multiplied back into the state once per forward) and
 *   collect the diagonals of a pass into a few per-amplitude phase tables,
 *   each applied with three shears (3 multiply-adds per amplitude).
 * DMV_ARITH_FP64_DIRECT: IEEE FP64 with every fused 2x2 applied as a full
 *   complex multiply-add (8 per amplitude for a general matrix).
 * The FP32-pair and int64 arithmetics below take the same rotation and phase
 * table rewrite of their fused passes, with each rotation a real 2x2.
 * DMV_ARITH_FP32X2: the FP64 amplitudes are split into FP32 pairs (about 48
 *   significant bits) inside each kernel and combined with error-free
 *   transformations, then stored back as FP64; GB300 runs FP32 ~71x faster
 *   than FP64. Between the window passes of one gate list the state keeps the
 *   pair form (the same 16 bytes per amplitude); it is IEEE complex128 again
 *   when the call returns. Measured error on deep circuits ~1e-13 normwise.
 * DMV_ARITH_INT64: each tile (or pair) is converted to int64 fixed point with
 *   one shared exponent (54 fraction bits for its largest components) and
 *   multiplied exactly in 31-bit limbs on the integer pipe, with one rounding
 *   per output. Passes holding a non-unitary matrix fall back to FP64.
 * DMV_ARITH_TC: the same int64 block fixed point, but each fused window pass
 *   is cut into dense blocks (the product of its gates on up to 5 qubits, one
 *   32 x 32 unitary) and exchanges (X, CNOT). A block is applied to 128
 *   columns of the tile at once as exact products of balanced 8-bit digits
 *   (7 per 56-bit integer, FP16) on the tensor cores (tcgen05.mma, FP32
 *   accumulators in tensor memory, every sum exact), rounded once per
 *   output. Passes it does not take run as DMV_ARITH_INT64. Single states
 *   only (batches accept FP64, FP64_DIRECT, FP32X2 and INT64; a batch applies
 *   every fused 2x2 directly, as DMV_ARITH_FP64_DIRECT does). */
enum { DMV_ARITH_FP64 = 0, DMV_ARITH_FP32X2 = 1, DMV_ARITH_INT64 = 2, DMV_ARITH_TC = 3, DMV_ARITH_FP64_DIRECT = 4 };

/* Gate kinds (numbering shared with the oracle). DMV_GATE_MATRIX takes an
 * explicit 2x2 matrix; every kind may carry a control qubit. */
enum {
  DMV_GATE_H = 0, DMV_GATE_X = 1, DMV_GATE_Y = 2, DMV_GATE_Z = 3,
  DMV_GATE_RX = 4, DMV_GATE_RY = 5, DMV_GATE_RZ = 6, DMV_GATE_CNOT = 7,
  DMV_GATE_MATRIX = 8
};

/* Fusion modes for dmv_apply_gates. */
enum {
  DMV_FUSE_NONE = 0,   /* one kernel pass per gate (reference order, one pass each) */
  DMV_FUSE_WINDOW = 1  /* merge same-qubit runs, then qubit-window passes */
};

/* One gate of a gate list. `control` is -1 for none. `theta` is the rotation
 * angle of RX/RY/RZ. For DMV_GATE_MATRIX, `m` holds the row-major 2x2 matrix
 * as (re, im) pairs [m00, m01, m10, m11]; it is ignored otherwise. */
typedef struct {
  int32_t kind;
  int32_t target;
  int32_t control;
  int32_t reserved;
  double theta;
  double m[8];
} dmv_gate_t;

typedef struct dmv_state_s* dmv_state_t;
typedef struct dmv_circuit_s* dmv_circuit_t;

/* ------------------------------------------------------------------------ */
/* Library / device                                                          */
/* ------------------------------------------------------------------------ */
int dmv_last_error(void);
const char* dmv_last_error_string(void);
const char* dmv_version(void);
/* Number of the library's own kernel launches since load (bench bookkeeping). */
int64_t dmv_kernel_launch_count(void);
/* Selects the CUDA device used by the calling thread for new states. */
int dmv_set_device(int32_t device);
/* Page-locks (or releases) caller-owned host memory so host<->device copies
 * of states run at full link speed. */
int dmv_host_register(void* ptr, int64_t bytes);
int dmv_host_unregister(void* ptr);

/* Kernel families reported by the profiler. */
enum {
  DMV_KERNEL_WINDOW = 0,  /* fused qubit-window pass */
  DMV_KERNEL_SINGLE = 1,  /* one-op pass */
  DMV_KERNEL_REDUCE = 2,  /* probabilities / expectation / sampling / inner product */
  DMV_KERNEL_ADJOINT = 3, /* adjoint sweep step */
  DMV_KERNEL_OTHER = 4,   /* init, layout conversion */
  DMV_KERNEL_FAMILIES = 5
};
/* While enabled, every launch of the gate-application kernels is bracketed by
 * CUDA events on its stream. dmv_profile_read synchronizes and returns, per
 * family, the launch count, the summed event time, the algorithmic bytes and
 * the algorithmic multiply-adds (in the storage precision's arithmetic). */
int dmv_profile_enable(int32_t on);
int dmv_profile_reset(void);
int dmv_profile_read(int32_t family, int64_t* launches, double* total_ms, double* algorithmic_bytes,
                     double* multiply_adds);

/* ------------------------------------------------------------------------ */
/* State                                                                     */
/* ------------------------------------------------------------------------ */
/* Allocates 2^num_qubits amplitudes on the current device and sets |0...0>.
 * `stream` may be NULL (the library then creates its own non-blocking stream). */
int dmv_state_create(int32_t num_qubits, int32_t precision, void* stream, dmv_state_t* out);
int dmv_state_destroy(dmv_state_t s);
int dmv_state_info(dmv_state_t s, int32_t* num_qubits, int32_t* precision, int64_t* num_amplitudes);
int dmv_state_set_zero(dmv_state_t s);
int dmv_state_synchronize(dmv_state_t s);
/* DMV_ARITH_* for later gate applications on this state. */
int dmv_state_set_arithmetic(dmv_state_t s, int32_t arithmetic);
/* Device pointer of the amplitudes (interleaved complex) and its stream. */
int dmv_state_device_ptr(dmv_state_t s, void** amps, void** stream);
/* Host <-> device copies of all amplitudes. `re`/`im` are split real and
 * imaginary parts (the reference's SoA host layout); `interleaved` is
 * (re, im) pairs. Always complex128 on the host side. Synchronous. */
int dmv_state_copy_to_host(dmv_state_t s, double* re, double* im);
int dmv_state_copy_to_host_interleaved(dmv_state_t s, double* interleaved);
int dmv_state_load_from_host(dmv_state_t s, const double* re, const double* im);
int dmv_state_load_from_host_interleaved(dmv_state_t s, const double* interleaved);
/* dst <- src (same size and precision), stream-ordered on dst's stream. */
int dmv_state_copy(dmv_state_t dst, dmv_state_t src);
/* CUDA-event timing of everything enqueued on the state's stream between
 * the two calls; _end synchronizes and returns the elapsed milliseconds. */
int dmv_state_event_begin(dmv_state_t s);
int dmv_state_event_end(dmv_state_t s, double* elapsed_ms);

/* ------------------------------------------------------------------------ */
/* Gate application (stream-ordered; returns once the work is enqueued)      */
/* ------------------------------------------------------------------------ */
/* One 2x2 gate given as split real/imag row-major parts, control -1 = none.
 * Same argument meaning as the reference's apply_one_qubit_gate_gpu_local. */
int dmv_apply_matrix(dmv_state_t s, const double m_re[4], const double m_im[4],
                     int32_t control, int32_t target);
/* A gate list, fused according to `fusion` (DMV_FUSE_*). */
int dmv_apply_gates(dmv_state_t s, const dmv_gate_t* gates, int64_t num_gates, int32_t fusion);
/* Number of HBM passes the last dmv_apply_gates call used (plan statistics). */
int dmv_last_plan_stats(int64_t* num_passes, int64_t* num_fused_ops, int64_t* bytes_moved);
/* Tensor-core statistics of the last dmv_apply_gates call on a state with
 * DMV_ARITH_TC: window passes that ran on the tensor cores, their dense
 * blocks and their exchange stages (zeros for other arithmetics). */
int dmv_last_tc_stats(dmv_state_t s, int64_t* tc_passes, int64_t* blocks, int64_t* exchanges);
/* Bytes the last gate application on `s` copied from the host to the device
 * (the plan's op list, phase tables, tensor-core stages and digit matrices),
 * and of those the phase tables of the FP64 rotation passes. No reference
 * counterpart. */
int dmv_last_upload_bytes(dmv_state_t s, int64_t* total, int64_t* phase_tables);
/* Plans a gate list without touching a GPU (host only): the number of HBM
 * passes, of window passes, of ops after merging, and the largest number of
 * local qubits of a window. tile_bits 0 picks the default for the precision. */
int dmv_plan_describe(int32_t num_qubits, int32_t precision, const dmv_gate_t* gates, int64_t num_gates,
                      int32_t fusion, int32_t tile_bits, int64_t* num_passes, int64_t* num_window_passes,
                      int64_t* num_ops, int32_t* max_local_qubits);

/* ------------------------------------------------------------------------ */
/* Measurement (synchronous: results are on the host when these return)      */
/* ------------------------------------------------------------------------ */
/* probs[i] = |a_i|^2 for all 2^n amplitudes (host array). */
int dmv_measure(dmv_state_t s, double* probs);
/* Same, into a device buffer of 2^n doubles; stream-ordered. */
int dmv_measure_device(dmv_state_t s, double* probs_device);
/* <Z_q> = sum_i |a_i|^2 (1 - 2 bit_q(i)) for q = 0..n-1, and the norm
 * sum_i |a_i|^2 (may be NULL). FP64 accumulation in both precisions. */
int dmv_expect_z(dmv_state_t s, double* expect, double* norm);
/* Inverse-CDF sampling with caller-supplied uniforms in [0,1): sample j is
 * the least index with u_j * total <= cdf(index) (the reference's rule,
 * src/utils.rs:258-277); u = 0 gives UINT64_MAX like the reference. */
int dmv_sample(dmv_state_t s, const double* uniforms, int64_t k, uint64_t* samples);
/* Same rule on a caller-supplied host probability vector (Circuit.sample_local). */
int dmv_sample_probabilities(const double* probs, int64_t num_probs, const double* uniforms,
                             int64_t k, uint64_t* samples);
/* Sampled expectation values, samples kept on the device: k samples drawn by
 * dmv_sample's rule, then for each of the num_obs qubits the mean over the
 * samples of +1 (bit clear) / -1 (bit set): the per-sample values of
 * extract_expectation_values (src/qubit_backend/circuit.rs:494-513) averaged,
 * without moving the samples to the host. `uniforms`: k host values in
 * [0,1), or NULL to draw them on the device from `seed` (SplitMix64: uniform
 * i = (mix64(seed + (i+1) * 0x9E3779B97F4A7C15) >> 11) * 2^-53). `set_counts`
 * (may be NULL) receives, per qubit, the number of samples with the bit set;
 * means[j] = (k - 2 set_counts[j]) / k exactly. k is processed in batches of
 * 2^24 (256 MB of scratch). */
int dmv_sample_expect_z(dmv_state_t s, const double* uniforms, uint64_t seed, int64_t k,
                        const int32_t* qubits, int32_t num_obs, double* means, int64_t* set_counts);
/* <a|b> (conjugate-linear in a), FP64 accumulation. */
int dmv_inner_product(dmv_state_t a, dmv_state_t b, double* re, double* im);

/* Allocation-free <Z_q> for callers that must not let a library allocate
 * device memory: applications that hand all device memory out from their
 * own pool up front, and latency-bound loops that cannot take the
 * device-wide synchronisation of cudaMalloc/cudaFree. It has no counterpart
 * in the reference.
 * `amps` are the caller's 2^num_qubits device amplitudes (interleaved, in
 * `precision`); `out_device` receives num_qubits + 1 doubles on the device:
 * <Z_0> ... <Z_{n-1}>, then the norm. Stream-ordered on `stream`. It calls
 * no cudaMalloc/cudaFree: its partial sums live in one fixed device array
 * compiled into the library (1216 x 35 doubles, 332.5 KiB, held on every GPU
 * that loads the library until exit), hence num_qubits <= 34; larger sizes
 * are rejected with DMV_ERR_INVALID. The first call on each device looks the
 * array's device address up (and may load the library's device code). Every
 * call shares the array, so calls whose kernels overlap on the GPU race;
 * serialise them. */
int dmv_expect_z_noalloc(const void* amps, int32_t num_qubits, int32_t precision, double* out_device,
                         void* stream);

/* ------------------------------------------------------------------------ */
/* Adjoint gradient                                                          */
/* ------------------------------------------------------------------------ */
/* Runs the gate list from |0...0> on `s`, then the adjoint sweep for the loss
 * L = sum_q weights[q] <Z_q>. grads[j] is dL/dtheta for the j-th RX/RY/RZ gate
 * in list order. `s` holds the forward state on return. Uses two more
 * statevectors of the same size (allocated and freed inside). */
int dmv_adjoint_gradient(dmv_state_t s, const dmv_gate_t* gates, int64_t num_gates,
                         const double* weights, double* loss, double* grads);

/* ------------------------------------------------------------------------ */
/* Batched circuits (no counterpart in the reference: it runs one circuit per */
/* process). Many independent circuits of uneven qubit count and depth share  */
/* one device arena and run in one persistent launch captured in a CUDA graph. */
/* ------------------------------------------------------------------------ */
typedef struct dmv_batch_s* dmv_batch_t;
/* Circuit c has num_qubits[c] (1..30) qubits and the gates
 * gates[gate_offsets[c] .. gate_offsets[c+1]). */
int dmv_batch_create(int32_t num_circuits, const int32_t* num_qubits, const int64_t* gate_offsets,
                     const dmv_gate_t* gates, int32_t precision, int32_t arithmetic, dmv_batch_t* out);
int dmv_batch_destroy(dmv_batch_t b);
/* Tile size (log2 amplitudes), always-local low qubits and tiles per work item. */
int dmv_batch_configure(dmv_batch_t b, int32_t tile_bits, int32_t low_bits, int32_t tiles_per_item);
/* Times graph runs over a grid of configurations and keeps the fastest. */
int dmv_batch_autotune(dmv_batch_t b, int32_t* tile_bits, int32_t* low_bits, int32_t* tiles_per_item,
                       double* best_ms);
/* One graph launch: every state reset to |0...0>, every circuit applied, every
 * <Z_q> reduced. Synchronous; DMV_ERR_TIMEOUT if a bounded wait gave up. */
int dmv_batch_run(dmv_batch_t b, double* elapsed_ms);
/* <Z_q> of every circuit after the last run, concatenated (sum of num_qubits). */
int dmv_batch_expect_z(dmv_batch_t b, double* out);
int dmv_batch_copy_state(dmv_batch_t b, int32_t index, double* interleaved);
int dmv_batch_stats(dmv_batch_t b, int64_t* items, int64_t* passes, int64_t* ops, int32_t* grid,
                    double* last_ms);
/* Test hook: sets the dependency-wait limit (iterations of ~1 us) and, with
 * poison != 0, re-plans so one item waits for a count that never arrives; the
 * next run must then end with DMV_ERR_TIMEOUT instead of hanging. */
int dmv_batch_debug_wait_limit(dmv_batch_t b, int64_t spin_limit, int32_t poison);
/* Test hook: the next `count` device allocations of the library fail (as if
 * out of memory). */
int dmv_debug_fail_allocations(int32_t count);
/* Test hook: mode 1 makes every dense block of later DMV_ARITH_TC passes read
 * its tensor-memory accumulators with the exact float-to-integer conversion
 * instead of the magic-number addition the planner picks when every
 * accumulator provably stays below 2^22; mode 0 restores the choice. */
int dmv_debug_tc_convert(int32_t mode);
/* Test hook: the number of polls after which a TMA window pass stops waiting
 * for a tile load (negative: the default). The pass then drains its copies,
 * leaves the state undefined and the next dmv_state_synchronize returns
 * DMV_ERR_TIMEOUT. The same limit bounds the chunk-load waits of the
 * bulk-staged readout passes (dmv_expect_z, dmv_sample, dmv_sample_expect_z
 * from 12 qubits), which then return DMV_ERR_TIMEOUT themselves with
 * undefined outputs; the state is unchanged. No reference counterpart. */
int dmv_debug_tma_wait_limit(int64_t polls);
/* Test hook (host only, no GPU): plans `gates` for num_qubits (12..34) with
 * 2^12-amplitude windows, rewrites every window pass into rotations and phase
 * tables in both forms (scaled rotations and tables by shears, as the FP64
 * kernels apply them; rotations as real 2x2 ops and tables as complex values,
 * as the FP32-pair and int64 kernels do), applies the original and the
 * rewritten ops to two random tiles each in host FP64, and returns the
 * largest normwise difference. counts (may be NULL) receives 4 values: passes
 * checked, non-exchange ops before, rotations and phase tables after. No
 * reference counterpart. */
int dmv_debug_check_fp64_rewrite(const dmv_gate_t* gates, int64_t num_gates, int32_t num_qubits, uint64_t seed,
                                 double* max_err, int64_t* counts);
/* Test hook (host only, no GPU): plans the reverse sweep of an adjoint
 * gradient over `gates` (reversed, each gate's adjoint, unmerged, ops tagged
 * with parameter slots and generators, 2^12-amplitude windows) and writes 6
 * counts: passes, window passes, ops, tagged ops, the largest slot + 1, and
 * ops whose slot and generator disagree (one set, the other not). No
 * reference counterpart. */
int dmv_debug_adjoint_plan(const dmv_gate_t* gates, int64_t num_gates, int32_t num_qubits, int64_t* counts);

/* ------------------------------------------------------------------------ */
/* Circuit front-end (the reference's pyo3 Circuit, src/qubit_backend/circuit.rs:78-770) */
/* ------------------------------------------------------------------------ */
/* apply_method: NULL or "gpu" (only the GPU backend lives in this library). */
int dmv_circuit_create(int32_t num_qubits, const char* apply_method, int32_t precision,
                       dmv_circuit_t* out);
int dmv_circuit_destroy(dmv_circuit_t c);
int dmv_circuit_add_gate(dmv_circuit_t c, int32_t kind, int32_t target, int32_t control,
                         double theta, int32_t is_observable);
int dmv_circuit_num_gates(dmv_circuit_t c, int64_t* num_gates, int64_t* num_params,
                          int64_t* num_observables);
int dmv_circuit_get_gate(dmv_circuit_t c, int64_t index, dmv_gate_t* gate, int32_t* is_observable);
int dmv_circuit_set_parameters(dmv_circuit_t c, const double* params, int64_t num_params);
int dmv_circuit_set_fusion(dmv_circuit_t c, int32_t fusion);
int dmv_circuit_set_arithmetic(dmv_circuit_t c, int32_t arithmetic);
int dmv_circuit_reset_amplitudes(dmv_circuit_t c);
int dmv_circuit_reset(dmv_circuit_t c);
int dmv_circuit_forward(dmv_circuit_t c);
int dmv_circuit_state(dmv_circuit_t c, dmv_state_t* state);
/* Readout qubits of the observables, in the order they were added. */
int dmv_circuit_observables(dmv_circuit_t c, int32_t* readout_qubits);
/* out[s*num_obs + j] = -1 if bit readout_j of samples[s] is set else +1 (circuit.rs:494-513). */
int dmv_circuit_extract_expectation_values(dmv_circuit_t c, const uint64_t* samples, int64_t k,
                                           double* out);
/* dmv_sample_expect_z over the circuit's observables (their readout qubits,
 * in the order they were added): means[j] is the average over k device-drawn
 * samples of column j of extract_expectation_values. */
int dmv_circuit_sample_expectation_values(dmv_circuit_t c, const double* uniforms, uint64_t seed, int64_t k,
                                          double* means);
/* |<psi(params1)|psi(params2)>|^2; clears the gate list afterwards like
 * the reference's get_fidelity (circuit_metrics.rs:11-32). */
int dmv_circuit_fidelity_with_parameters(dmv_circuit_t c, const double* p1, int64_t n1,
                                         const double* p2, int64_t n2, double* fidelity);
/* Adjoint gradient of sum_q w_q <Z_q> over the circuit's non-observable gates. */
int dmv_circuit_adjoint(dmv_circuit_t c, const double* weights, double* loss, double* grads);

/* ------------------------------------------------------------------------ */
/* LEGACY ABI (damavand-gpu/rust_communication.cu); process-global state     */
/* ------------------------------------------------------------------------ */
/* rust_communication.cu:24-29 */
int get_number_of_available_gpus(void);
/* rust_communication.cu:31-37, MiB of device memory */
double get_memory_for_gpu(int local_gpu_rank);
/* rust_communication.cu:39-47; this library never enables peer access: 0 */
int peer_access_allowed(int source_gpu_id, int target_gpu_id);
/* rust_communication.cu:49-104; prints call and kernel-launch counts */
void print_timers(void);
/* rust_communication.cu:143-198; one GPU only (num_gpus_per_node must be 1).
 * The Rust side passes an int for the bool; both are accepted (nonzero = true). */
void init_quantum_state(int num_amplitudes_per_gpu, int num_gpus_per_node, int is_first_node);
/* rust_communication.cu:339-359 */
void apply_one_qubit_gate_gpu_local(double* gate_matrix_real, double* gate_matrix_imaginary,
                                    int num_qubits, int num_amplitudes_per_gpu,
                                    int control_qubit, int target_qubit);
/* rust_communication.cu:330-337, :200-252, :254-328 (all three fill the host array) */
void measure_on_gpu(int num_amplitudes_per_gpu, double* probabilities);
void sequential_measure_on_gpu(int num_amplitudes_per_gpu, double* probabilities);
void concurrent_measure_on_gpu(int num_amplitudes_per_gpu, double* probabilities);
/* rust_communication.cu:450-482 */
void retrieve_amplitudes_on_host(int num_amplitudes_per_gpu, double* local_amplitudes_real,
                                 double* local_amplitudes_imaginary);
/* rust_communication.cu:384-398 (a stub there; a real host->device upload here) */
void load_amplitudes_local_on_device(int num_amplitudes_per_gpu, double* local_amplitudes_real,
                                     double* local_amplitudes_imaginary);
/* Distributed entry points (rust_communication.cu:106-141, :361-382, :400-448):
 * exported so the link succeeds; they set DMV_ERR_UNSUPPORTED and do nothing. */
void exchange_amplitudes_between_gpus(int current_gpu_rank, int partner_gpu_rank,
                                      int num_amplitudes_per_gpu);
void apply_one_qubit_gate_gpu_distributed(double* gate_matrix_real, double* gate_matrix_imaginary,
                                          int num_qubits, int num_amplitudes_per_gpu,
                                          int control_qubit, int target_qubit);
void split_amplitudes_between_gpus(int num_amplitudes_per_gpu, double* local_amplitudes_real,
                                   double* local_amplitudes_imaginary,
                                   double* partner_amplitudes_real,
                                   double* partner_amplitudes_imaginary);

#ifdef __cplusplus
}
#endif
#endif /* DAMAVAND_GPU_H */
