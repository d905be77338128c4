/*
 * CPU oracle for the damavand statevector gate-application path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * `apply_method="multithreading"` path (the rayon per-amplitude update), its
 * gate matrices, its sampler and its expectation-value extraction. Only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark load
 * it. The product path (damavand_gb300) never links or calls it.
 *
 * Parity pin: the reference's only state known-answer test is
 * src/qubit_backend/circuit.rs:802-837 (H(0), H(1), CNOT(0,1) on 2 qubits ->
 * every amplitude 1/2). The oracle is checked against it and against analytic
 * known answers (tests/golden/). Everything else rests on this restatement.
 *
 * Layout: a state of n qubits is 2^n complex128 amplitudes stored interleaved
 * (re, im), the memory layout of ndarray's Array1<Complex<f64>>. Qubit q is
 * bit q of the amplitude index (little-endian), as in
 * src/qubit_backend/circuit_multithreading.rs:36,41.
 *
 * Build with -O3 -ffp-contract=off -fopenmp: the reference (Rust) performs no
 * FMA contraction, and num-complex's multiply is the textbook 4-mul/2-add form.
 */
#ifndef DAMAVAND_ORACLE_H
#define DAMAVAND_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gate kinds; same numbering as the product library's DMV_GATE_* values. */
enum {
  ORC_H = 0, ORC_X = 1, ORC_Y = 2, ORC_Z = 3,
  ORC_RX = 4, ORC_RY = 5, ORC_RZ = 6, ORC_CNOT = 7
};

typedef struct {
  int32_t kind;
  int32_t target;
  int32_t control;       /* -1 when the gate has no control qubit */
  int32_t is_observable; /* skipped by forward, read by expectation extraction */
  double theta;          /* rotation angle for RX/RY/RZ, ignored otherwise */
} orc_gate;

/* 2x2 matrix of a gate, row-major [m00, m01, m10, m11], each (re, im). */
void orc_gate_matrix(int32_t kind, double theta, double m[8]);

/* |0...0> */
void orc_zero_state(double* state, int32_t n);

/* One gate, exactly as apply_multithreading_local: clone the state, then
 * update every amplitude from the clone. `scratch` holds 2^n complex. */
void orc_apply_gate(double* state, double* scratch, int32_t n, const double m[8],
                    int32_t control, int32_t target);

/* The same gate in place over amplitude pairs, without the clone; each output
 * is the reference's expression on the same inputs, so the bits are those of
 * orc_apply_gate (checked by the oracle tests). */
void orc_apply_gate_inplace(double* state, int32_t n, const double m[8], int32_t control,
                            int32_t target);

/* Circuit::forward: every non-observable gate in order. Does NOT reset.
 * orc_forward clones per gate (the reference's algorithm); orc_forward_mode
 * with clone_per_gate = 0 uses orc_apply_gate_inplace. */
void orc_forward(double* state, int32_t n, const orc_gate* gates, int64_t num_gates);
void orc_forward_mode(double* state, int32_t n, const orc_gate* gates, int64_t num_gates,
                      int32_t clone_per_gate);

/* Circuit::measure on the CPU path: norm_sqr of every amplitude. */
void orc_measure(const double* state, int32_t n, double* probs);

/* utils::sample_from_discrete_distribution with an injected uniform u in
 * [0,1): returns index-1 for the least index with u*cdf[N] <= cdf[index]
 * (wrapping to UINT64_MAX for index 0, as the release-mode usize does). */
uint64_t orc_sample_one(const double* probs, int64_t num_probs, double u);

/* Circuit::sample_local with injected uniforms. rebuild_per_sample=1 repeats
 * the reference's O(k*N) rebuild of the cumulative sum for every sample;
 * 0 builds it once and binary-searches (same result: the search finds the
 * least index of a non-decreasing sequence). */
void orc_sample(const double* probs, int64_t num_probs, const double* uniforms,
                int64_t k, uint64_t* samples, int32_t rebuild_per_sample);

/* Exact <Z_q> = sum_i p_i (1 - 2 bit_q(i)), q = 0..n-1 (sign convention of
 * Circuit::extract_expectation_values). */
void orc_expect_z(const double* probs, int32_t n, double* out);

/* The same from the amplitudes, without a probability vector (n <= 64). */
void orc_expect_z_from_state(const double* state, int32_t n, double* out);

/* Circuit::extract_expectation_values: out[s*num_obs+j] = -1 if bit
 * readout[j] of samples[s] is set, else +1. */
void orc_extract_expectation_values(const uint64_t* samples, int64_t k,
                                    const int32_t* readout_qubits, int32_t num_obs,
                                    double* out);

/* Loss sum_q w_q <Z_q> of the circuit run from |0...0>, with its RX/RY/RZ
 * angles replaced in gate order by `params` (Circuit::set_parameters). */
double orc_loss(int32_t n, const orc_gate* gates, int64_t num_gates,
                const double* params, int64_t num_params, const double* weights);

double orc_loss_mode(int32_t n, const orc_gate* gates, int64_t num_gates, const double* params,
                     int64_t num_params, const double* weights, int32_t clone_per_gate);

/* Parameter shift for the parameters with indices which[0..num_which). */
void orc_param_shift_subset(int32_t n, const orc_gate* gates, int64_t num_gates,
                            const double* params, int64_t num_params, const double* weights,
                            const int64_t* which, int64_t num_which, double* grads,
                            int32_t clone_per_gate);

/* Parameter-shift gradient of orc_loss: g_k = (L(th_k + pi/2) - L(th_k - pi/2))/2,
 * the rule sketched (commented out) at src/qubit_backend/circuit.rs:529-546. */
void orc_param_shift_grad(int32_t n, const orc_gate* gates, int64_t num_gates,
                          const double* params, int64_t num_params,
                          const double* weights, double* grads);

/* Threads OpenMP will use (for reporting the CPU baseline's core count). */
int32_t orc_num_threads(void);
void orc_set_num_threads(int32_t t);

#ifdef __cplusplus
}
#endif
#endif
