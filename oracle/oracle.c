/*
 * CPU oracle (test infrastructure only) -- see oracle.h for scope and pinning.
 * Each function cites the reference lines it restates.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* num-complex Mul: (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re), no FMA. */
static inline void cmul(double ar, double ai, double br, double bi, double* cr, double* ci) {
  *cr = ar * br - ai * bi;
  *ci = ar * bi + ai * br;
}

/* Matrices of src/qubit_backend/gates.rs: Hadamard :97-119, PauliX :223-233,
 * PauliY :288-298, PauliZ :352-362, RotationX :417-439, RotationY :489-511,
 * RotationZ :561-577; CNOT uses the PauliX matrix (circuit_multithreading.rs:14-20). */
void orc_gate_matrix(int32_t kind, double theta, double m[8]) {
  memset(m, 0, 8 * sizeof(double));
  switch (kind) {
    case ORC_H: {
      double h = 1. / sqrt(2.0);
      m[0] = h; m[2] = h; m[4] = h; m[6] = -1. / sqrt(2.0);
      break;
    }
    case ORC_X:
    case ORC_CNOT:
      m[2] = 1.; m[4] = 1.;
      break;
    case ORC_Y:
      m[3] = -1.; m[5] = 1.;
      break;
    case ORC_Z:
      m[0] = 1.; m[6] = -1.;
      break;
    case ORC_RX:
      m[0] = cos(theta / 2.); m[3] = -sin(theta / 2.);
      m[5] = -sin(theta / 2.); m[6] = cos(theta / 2.);
      break;
    case ORC_RY:
      m[0] = cos(theta / 2.); m[2] = -sin(theta / 2.);
      m[4] = sin(theta / 2.); m[6] = cos(theta / 2.);
      break;
    case ORC_RZ:
      m[0] = cos(-theta / 2.); m[1] = sin(-theta / 2.);
      m[6] = cos(theta / 2.); m[7] = sin(theta / 2.);
      break;
    default:
      break;
  }
}

/* Circuit::new / reset_amplitudes for the CPU paths: zeros, amplitude 0 = 1
 * (src/qubit_backend/circuit.rs:172-175, :262-267). */
void orc_zero_state(double* state, int32_t n) {
  int64_t N = (int64_t)1 << n;
  memset(state, 0, (size_t)N * 2 * sizeof(double));
  state[0] = 1.;
}

/* Circuit::compute_partner_rank(i, 1, gap), src/qubit_backend/circuit.rs:781-795. */
static inline int64_t partner_index(int64_t i, int64_t gap) {
  return (i % (2 * gap)) < gap ? i + gap : i - gap;
}

/* apply_multithreading_local, src/qubit_backend/circuit_multithreading.rs:9-54. */
void orc_apply_gate(double* state, double* scratch, int32_t n, const double m[8],
                    int32_t control, int32_t target) {
  int64_t N = (int64_t)1 << n;
  int64_t gap = (int64_t)1 << target;
  memcpy(scratch, state, (size_t)N * 2 * sizeof(double)); /* :31 clone */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    int apply = control < 0 ? 1 : (int)((i >> control) & 1); /* :35-39 */
    if (!apply) continue;
    int64_t p = partner_index(i, gap); /* :40-41 */
    double ar = state[2 * i], ai = state[2 * i + 1];
    double pr = scratch[2 * p], pi = scratch[2 * p + 1];
    double t0r, t0i, t1r, t1i;
    if (p > i) { /* :46-47  a*m00 + partner*m01 */
      cmul(ar, ai, m[0], m[1], &t0r, &t0i);
      cmul(pr, pi, m[2], m[3], &t1r, &t1i);
    } else {     /* :48-49  partner*m10 + a*m11 */
      cmul(pr, pi, m[4], m[5], &t0r, &t0i);
      cmul(ar, ai, m[6], m[7], &t1r, &t1i);
    }
    state[2 * i] = t0r + t1r;
    state[2 * i + 1] = t0i + t1i;
  }
}

/* The same update as orc_apply_gate without the clone: every amplitude pair
 * (i, i + 2^target) with bit `target` of i clear is read once and both
 * outputs are written in place. Each output is the expression of
 * circuit_multithreading.rs:46-49 on the same two inputs, in the same order
 * of operations (a*m00 + partner*m01 for the lower index, partner*m10 +
 * a*m11 for the upper), so the result is bit-identical to orc_apply_gate:
 * the clone only guarantees that every read sees the pre-gate values, which
 * reading each pair before writing it guarantees as well. The control is
 * tested on the lower index; both indices of a pair share every bit but
 * `target` (control != target). */
void orc_apply_gate_inplace(double* state, int32_t n, const double m[8], int32_t control,
                            int32_t target) {
  int64_t half = (int64_t)1 << (n - 1);
  int64_t gap = (int64_t)1 << target;
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < half; ++j) {
    int64_t i = ((j >> target) << (target + 1)) | (j & (gap - 1)); /* bit `target` clear */
    if (control >= 0 && !((i >> control) & 1)) continue;
    int64_t p = i + gap;
    double ar = state[2 * i], ai = state[2 * i + 1];
    double pr = state[2 * p], pi = state[2 * p + 1];
    double t0r, t0i, t1r, t1i, u0r, u0i, u1r, u1i;
    cmul(ar, ai, m[0], m[1], &t0r, &t0i); /* lower: a*m00 + partner*m01 */
    cmul(pr, pi, m[2], m[3], &t1r, &t1i);
    cmul(ar, ai, m[4], m[5], &u0r, &u0i); /* upper: partner*m10 + a*m11 */
    cmul(pr, pi, m[6], m[7], &u1r, &u1i);
    state[2 * i] = t0r + t1r;
    state[2 * i + 1] = t0i + t1i;
    state[2 * p] = u0r + u1r;
    state[2 * p + 1] = u0i + u1i;
  }
}

/* Circuit::forward, src/qubit_backend/circuit.rs:341-369: observables skipped.
 * clone_per_gate = 1 runs orc_apply_gate (the reference's clone and sweep, the
 * algorithm the CPU baseline times); 0 runs orc_apply_gate_inplace (same
 * bits, half the memory traffic and no scratch vector). */
void orc_forward_mode(double* state, int32_t n, const orc_gate* gates, int64_t num_gates,
                      int32_t clone_per_gate) {
  int64_t N = (int64_t)1 << n;
  double* scratch = NULL;
  if (clone_per_gate) {
    scratch = (double*)malloc((size_t)N * 2 * sizeof(double));
    if (!scratch) return;
  }
  for (int64_t g = 0; g < num_gates; ++g) {
    if (gates[g].is_observable) continue;
    double m[8];
    orc_gate_matrix(gates[g].kind, gates[g].theta, m);
    int32_t control = gates[g].kind == ORC_CNOT ? gates[g].control : -1;
    if (clone_per_gate) orc_apply_gate(state, scratch, n, m, control, gates[g].target);
    else orc_apply_gate_inplace(state, n, m, control, gates[g].target);
  }
  free(scratch);
}

void orc_forward(double* state, int32_t n, const orc_gate* gates, int64_t num_gates) {
  orc_forward_mode(state, n, gates, num_gates, 1);
}

/* Circuit::measure CPU branch, src/qubit_backend/circuit.rs:579-581 (norm_sqr). */
void orc_measure(const double* state, int32_t n, double* probs) {
  int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i)
    probs[i] = state[2 * i] * state[2 * i] + state[2 * i + 1] * state[2 * i + 1];
}

/* utils::sample_from_discrete_distribution + sample_from_discrete_cumulative,
 * src/utils.rs:258-277, with the thread_rng draw replaced by `u`. */
uint64_t orc_sample_one(const double* probs, int64_t num_probs, double u) {
  /* cumulative = [0, p0, p0+p1, ...] built sequentially (:270-274) */
  double* cdf = (double*)malloc((size_t)(num_probs + 1) * sizeof(double));
  if (!cdf) return UINT64_MAX;
  cdf[0] = 0.;
  for (int64_t j = 0; j < num_probs; ++j) cdf[j + 1] = cdf[j] + probs[j];
  double xsi = u * cdf[num_probs]; /* :260 */
  uint64_t result = UINT64_MAX;    /* None -> the caller panics (circuit.rs:478-482) */
  for (int64_t idx = 0; idx <= num_probs; ++idx) { /* :262-266 */
    if (xsi <= cdf[idx]) { result = (uint64_t)idx - 1u; break; }
  }
  free(cdf);
  return result;
}

void orc_sample(const double* probs, int64_t num_probs, const double* uniforms,
                int64_t k, uint64_t* samples, int32_t rebuild_per_sample) {
  if (rebuild_per_sample) { /* Circuit::sample_local, circuit.rs:468-485 */
    for (int64_t s = 0; s < k; ++s) samples[s] = orc_sample_one(probs, num_probs, uniforms[s]);
    return;
  }
  double* cdf = (double*)malloc((size_t)(num_probs + 1) * sizeof(double));
  if (!cdf) return;
  cdf[0] = 0.;
  for (int64_t j = 0; j < num_probs; ++j) cdf[j + 1] = cdf[j] + probs[j];
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < k; ++s) {
    double xsi = uniforms[s] * cdf[num_probs];
    int64_t lo = 0, hi = num_probs + 1; /* least idx in [0, N] with xsi <= cdf[idx] */
    while (lo < hi) {
      int64_t mid = lo + (hi - lo) / 2;
      if (xsi <= cdf[mid]) hi = mid; else lo = mid + 1;
    }
    samples[s] = lo <= num_probs ? (uint64_t)lo - 1u : UINT64_MAX;
  }
  free(cdf);
}

/* Compensated accumulation (Neumaier's variant of Kahan summation). */
static inline void acc_add(double* s, double* c, double x) {
  double t = *s + x;
  if (fabs(*s) >= fabs(x)) *c += (*s - t) + x;
  else *c += (x - t) + *s;
  *s = t;
}

/* Per-bit masses of p_0 .. p_{N-1}: out[q] = sum of p_i with bit q of i set,
 * total = sum of all. Blocks of 1024 consecutive indices are summed plainly
 * (bits 0-9 inside the block, the block's total for the bits above) and the
 * block sums accumulate with compensation, so the error stays near one
 * rounding of each block sum even at 2^31 terms (a plain running sum of 2^30
 * similar terms drifts by ~1e-10). `get(i)` is p_i. */
#define ORC_BLOCK_BITS 10
#define ORC_BIT_MASSES(N, n, GET, out, total_out)                                  \
  do {                                                                             \
    double tot_s = 0., tot_c = 0.;                                                 \
    double set_s[64], set_c[64];                                                   \
    for (int32_t q = 0; q < (n); ++q) set_s[q] = set_c[q] = 0.;                     \
    int64_t bsz = (int64_t)1 << ((n) < ORC_BLOCK_BITS ? (n) : ORC_BLOCK_BITS);      \
    int64_t nblk = (N) / bsz;                                                      \
    _Pragma("omp parallel")                                                        \
    {                                                                              \
      double ts = 0., tc = 0., ss[64], sc[64];                                     \
      for (int32_t q = 0; q < (n); ++q) ss[q] = sc[q] = 0.;                         \
      _Pragma("omp for schedule(static) nowait")                                   \
      for (int64_t b = 0; b < nblk; ++b) {                                         \
        double bt = 0., bb[ORC_BLOCK_BITS];                                        \
        for (int j = 0; j < ORC_BLOCK_BITS; ++j) bb[j] = 0.;                       \
        for (int64_t e = 0; e < bsz; ++e) {                                        \
          int64_t i = b * bsz + e;                                                 \
          double p = GET(i);                                                       \
          bt += p;                                                                 \
          for (int j = 0; j < ORC_BLOCK_BITS; ++j)                                 \
            if ((e >> j) & 1) bb[j] += p;                                          \
        }                                                                          \
        acc_add(&ts, &tc, bt);                                                     \
        for (int32_t q = 0; q < (n); ++q) {                                         \
          if (q < ORC_BLOCK_BITS) { if ((int64_t)1 << q < bsz) acc_add(&ss[q], &sc[q], bb[q]); } \
          else if ((b >> (q - ORC_BLOCK_BITS)) & 1) acc_add(&ss[q], &sc[q], bt);   \
        }                                                                          \
      }                                                                            \
      _Pragma("omp critical")                                                      \
      {                                                                            \
        acc_add(&tot_s, &tot_c, ts + tc);                                          \
        for (int32_t q = 0; q < (n); ++q) acc_add(&set_s[q], &set_c[q], ss[q] + sc[q]); \
      }                                                                            \
    }                                                                              \
    for (int32_t q = 0; q < (n); ++q) (out)[q] = set_s[q] + set_c[q];               \
    *(total_out) = tot_s + tot_c;                                                  \
  } while (0)

/* Exact Pauli-Z expectation; sign convention of circuit.rs:503-508 (+1 for bit 0):
 * <Z_q> = total - 2 * (mass with bit q set). */
void orc_expect_z(const double* probs, int32_t n, double* out) {
  int64_t N = (int64_t)1 << n;
  double total = 0.;
#define ORC_GET_P(i) (probs[(i)])
  ORC_BIT_MASSES(N, n, ORC_GET_P, out, &total);
#undef ORC_GET_P
  for (int32_t q = 0; q < n; ++q) out[q] = total - 2. * out[q];
}

/* The same <Z_q> straight from the amplitudes (p_i = norm_sqr, circuit.rs:579-581),
 * for states whose probability vector would not fit beside them. */
void orc_expect_z_from_state(const double* state, int32_t n, double* out) {
  int64_t N = (int64_t)1 << n;
  double total = 0.;
#define ORC_GET_A(i) (state[2 * (i)] * state[2 * (i)] + state[2 * (i) + 1] * state[2 * (i) + 1])
  ORC_BIT_MASSES(N, n, ORC_GET_A, out, &total);
#undef ORC_GET_A
  for (int32_t q = 0; q < n; ++q) out[q] = total - 2. * out[q];
}

/* Circuit::extract_expectation_values, src/qubit_backend/circuit.rs:494-513. */
void orc_extract_expectation_values(const uint64_t* samples, int64_t k,
                                    const int32_t* readout_qubits, int32_t num_obs,
                                    double* out) {
  for (int64_t s = 0; s < k; ++s)
    for (int32_t j = 0; j < num_obs; ++j)
      out[s * num_obs + j] = ((samples[s] >> (readout_qubits[j] & 63)) & 1) ? -1. : 1.;
}

static int is_parametrised(int32_t kind) {
  return kind == ORC_RX || kind == ORC_RY || kind == ORC_RZ;
}

double orc_loss_mode(int32_t n, const orc_gate* gates, int64_t num_gates, const double* params,
                     int64_t num_params, const double* weights, int32_t clone_per_gate) {
  int64_t N = (int64_t)1 << n;
  orc_gate* g = (orc_gate*)malloc((size_t)num_gates * sizeof(orc_gate));
  double* state = (double*)malloc((size_t)N * 2 * sizeof(double));
  double* probs = (double*)malloc((size_t)N * sizeof(double));
  double* ez = (double*)malloc((size_t)n * sizeof(double));
  double loss = NAN;
  if (g && state && probs && ez) {
    memcpy(g, gates, (size_t)num_gates * sizeof(orc_gate));
    /* Circuit::set_parameters, circuit.rs:308-322: parametrised gates in order */
    int64_t p = 0;
    for (int64_t i = 0; i < num_gates && p < num_params; ++i)
      if (is_parametrised(g[i].kind)) g[i].theta = params[p++];
    orc_zero_state(state, n);
    orc_forward_mode(state, n, g, num_gates, clone_per_gate);
    orc_measure(state, n, probs);
    orc_expect_z(probs, n, ez);
    loss = 0.;
    for (int32_t q = 0; q < n; ++q) loss += weights[q] * ez[q];
  }
  free(g); free(state); free(probs); free(ez);
  return loss;
}

double orc_loss(int32_t n, const orc_gate* gates, int64_t num_gates,
                const double* params, int64_t num_params, const double* weights) {
  return orc_loss_mode(n, gates, num_gates, params, num_params, weights, 1);
}

/* Parameter shift for the parameters listed in `which` (num_which of them):
 * grads[j] = (L(th_k + pi/2) - L(th_k - pi/2)) / 2 for k = which[j]. */
void orc_param_shift_subset(int32_t n, const orc_gate* gates, int64_t num_gates,
                            const double* params, int64_t num_params, const double* weights,
                            const int64_t* which, int64_t num_which, double* grads,
                            int32_t clone_per_gate) {
  const double half_pi = 1.5707963267948966;
  double* shifted = (double*)malloc((size_t)num_params * sizeof(double));
  if (!shifted) return;
  memcpy(shifted, params, (size_t)num_params * sizeof(double));
  for (int64_t j = 0; j < num_which; ++j) {
    int64_t k = which[j];
    shifted[k] = params[k] + half_pi;
    double up = orc_loss_mode(n, gates, num_gates, shifted, num_params, weights, clone_per_gate);
    shifted[k] = params[k] - half_pi;
    double down = orc_loss_mode(n, gates, num_gates, shifted, num_params, weights, clone_per_gate);
    shifted[k] = params[k];
    grads[j] = 0.5 * (up - down);
  }
  free(shifted);
}

void orc_param_shift_grad(int32_t n, const orc_gate* gates, int64_t num_gates,
                          const double* params, int64_t num_params,
                          const double* weights, double* grads) {
  const double half_pi = 1.5707963267948966;
  double* shifted = (double*)malloc((size_t)num_params * sizeof(double));
  if (!shifted) return;
  memcpy(shifted, params, (size_t)num_params * sizeof(double));
  for (int64_t k = 0; k < num_params; ++k) {
    shifted[k] = params[k] + half_pi;
    double up = orc_loss(n, gates, num_gates, shifted, num_params, weights);
    shifted[k] = params[k] - half_pi;
    double down = orc_loss(n, gates, num_gates, shifted, num_params, weights);
    shifted[k] = params[k];
    grads[k] = 0.5 * (up - down);
  }
  free(shifted);
}

int32_t orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int32_t t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}
