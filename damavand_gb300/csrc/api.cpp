// C ABI of libdamavand_gpu.so: state management, gate application,
// measurement, the Circuit front-end and the legacy entry points.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace dmv {

namespace {
thread_local int g_last_error = DMV_OK;
thread_local char g_last_msg[1024] = "";
std::atomic<int64_t> g_launches{0};
}  // namespace

int set_error(int code, const char* fmt, ...) {
  g_last_error = code;
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_last_msg, sizeof(g_last_msg), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() {
  g_last_error = DMV_OK;
  g_last_msg[0] = '\0';
}

int last_error() { return g_last_error; }

void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {
struct ProfRecord {
  int family;
  cudaEvent_t a, b;
  double bytes;
  double fmas;
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<ProfRecord> g_prof;
int64_t g_prof_launches[DMV_KERNEL_FAMILIES] = {};
double g_prof_ms[DMV_KERNEL_FAMILIES] = {};
double g_prof_bytes[DMV_KERNEL_FAMILIES] = {};
double g_prof_fmas[DMV_KERNEL_FAMILIES] = {};

// Folds finished records into the per-family totals (caller holds the lock).
void prof_drain(bool wait) {
  size_t keep = 0;
  for (size_t i = 0; i < g_prof.size(); ++i) {
    ProfRecord& r = g_prof[i];
    if (wait) cudaEventSynchronize(r.b);
    if (cudaEventQuery(r.b) == cudaSuccess) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.a, r.b);
      g_prof_launches[r.family] += 1;
      g_prof_ms[r.family] += ms;
      g_prof_bytes[r.family] += r.bytes;
      g_prof_fmas[r.family] += r.fmas;
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    } else {
      g_prof[keep++] = r;
    }
  }
  g_prof.resize(keep);
  cudaGetLastError();
}
}  // namespace

int64_t prof_begin(int family, cudaStream_t stream, double algorithmic_bytes, double multiply_adds) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (!g_prof_on || family < 0 || family >= DMV_KERNEL_FAMILIES) return -1;
  if (g_prof.size() > 4096) prof_drain(false);
  ProfRecord r{family, nullptr, nullptr, algorithmic_bytes, multiply_adds};
  if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  cudaEventRecord(r.a, stream);
  g_prof.push_back(r);
  return (int64_t)g_prof.size() - 1;
}

void prof_end(int64_t token, cudaStream_t stream) {
  if (token < 0) return;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  if (token < (int64_t)g_prof.size()) cudaEventRecord(g_prof[(size_t)token].b, stream);
}

namespace {
std::atomic<int32_t> g_fail_allocs{0};
}

bool injected_alloc_failure() {
  int32_t v = g_fail_allocs.load();
  while (v > 0)
    if (g_fail_allocs.compare_exchange_weak(v, v - 1)) return true;
  return false;
}

int DeviceBuffer::reserve(size_t n) {
  if (n <= bytes && ptr) return DMV_OK;
  release();
  if (injected_alloc_failure()) return set_error(DMV_ERR_OOM, "cudaMalloc(%zu) failed: injected failure", n);
  void* p = nullptr;
  const cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 256));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? DMV_ERR_OOM : DMV_ERR_CUDA,
                     "cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
  }
  ptr = p;
  bytes = std::max<size_t>(n, 256);
  return DMV_OK;
}

void DeviceBuffer::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

int ensure_pinned(dmv_state_s* s, size_t bytes) {
  if (s->pinned && s->pinned_bytes >= bytes) return DMV_OK;
  if (s->pinned) cudaFreeHost(s->pinned);
  s->pinned = nullptr;
  s->pinned_bytes = 0;
  void* p = nullptr;
  DMV_CUDA_TRY(cudaMallocHost(&p, bytes));
  s->pinned = p;
  s->pinned_bytes = bytes;
  return DMV_OK;
}

namespace {

constexpr int32_t kMaxQubits = 34;
constexpr int64_t kStageAmps = int64_t(1) << 24;  // host-copy staging: 16M amplitudes per chunk

int check_state(dmv_state_s* s) {
  if (!s || !s->amps) return set_error(DMV_ERR_INVALID, "null or destroyed state handle");
  return DMV_OK;
}

// Device-side split / join between interleaved storage and the host layouts.
int copy_out(dmv_state_s* s, double* re, double* im, double* inter);
int copy_in(dmv_state_s* s, const double* re, const double* im, const double* inter);

}  // namespace
}  // namespace dmv

using namespace dmv;

// Staging kernels live in kernels_copy.cu.
namespace dmv {
int launch_split(const void* amps, int precision, int64_t offset, int64_t count, double* re_dev, double* im_dev,
                 double* inter_dev, cudaStream_t stream);
int launch_join(void* amps, int precision, int64_t offset, int64_t count, const double* re_dev,
                const double* im_dev, const double* inter_dev, cudaStream_t stream);
}  // namespace dmv

namespace dmv {
namespace {

// Device address of page-locked (cudaHostRegister'ed or cudaMallocHost'ed)
// host memory, or nullptr for ordinary pageable memory.
void* mapped_device_pointer(const void* host) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (attr.type != cudaMemoryTypeHost) return nullptr;
  void* dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, const_cast<void*>(host), 0) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return dev;
}

int copy_out(dmv_state_s* s, double* re, double* im, double* inter) {
  const int64_t chunk = std::min<int64_t>(s->N, kStageAmps);
  // Fast path: complex128 interleaved output is a straight copy.
  if (inter && s->precision == DMV_C128) {
    DMV_CUDA_TRY(cudaMemcpyAsync(inter, s->amps, s->amp_bytes(), cudaMemcpyDeviceToHost, s->stream));
    DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return DMV_OK;
  }
  // Page-locked host buffers: the split kernel writes them directly over the link.
  {
    double* dre = re ? static_cast<double*>(mapped_device_pointer(re)) : nullptr;
    double* dim = im ? static_cast<double*>(mapped_device_pointer(im)) : nullptr;
    double* dint = inter ? static_cast<double*>(mapped_device_pointer(inter)) : nullptr;
    if ((inter && dint) || (!inter && dre && dim)) {
      DMV_TRY(launch_split(s->amps, s->precision, 0, s->N, dre, dim, dint, s->stream));
      DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
      return DMV_OK;
    }
  }
  DeviceBuffer stage;
  DMV_TRY(stage.reserve((size_t)chunk * 2 * sizeof(double)));
  double* a = static_cast<double*>(stage.ptr);
  double* b = a + chunk;
  int rc = DMV_OK;
  for (int64_t off = 0; off < s->N && rc == DMV_OK; off += chunk) {
    const int64_t cnt = std::min(chunk, s->N - off);
    if (inter) {
      rc = launch_split(s->amps, s->precision, off, cnt, nullptr, nullptr, a, s->stream);
      if (rc == DMV_OK && cudaMemcpyAsync(inter + 2 * off, a, (size_t)cnt * 2 * sizeof(double),
                                          cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
        rc = set_error(DMV_ERR_CUDA, "device-to-host copy failed");
    } else {
      rc = launch_split(s->amps, s->precision, off, cnt, a, b, nullptr, s->stream);
      if (rc == DMV_OK && (cudaMemcpyAsync(re + off, a, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost,
                                           s->stream) != cudaSuccess ||
                           cudaMemcpyAsync(im + off, b, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost,
                                           s->stream) != cudaSuccess))
        rc = set_error(DMV_ERR_CUDA, "device-to-host copy failed");
    }
    if (rc == DMV_OK && cudaStreamSynchronize(s->stream) != cudaSuccess)
      rc = set_error(DMV_ERR_CUDA, "stream synchronize failed");
  }
  cudaStreamSynchronize(s->stream);
  stage.release();
  return rc;
}

int copy_in(dmv_state_s* s, const double* re, const double* im, const double* inter) {
  const int64_t chunk = std::min<int64_t>(s->N, kStageAmps);
  if (inter && s->precision == DMV_C128) {
    DMV_CUDA_TRY(cudaMemcpyAsync(s->amps, inter, s->amp_bytes(), cudaMemcpyHostToDevice, s->stream));
    DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return DMV_OK;
  }
  {
    const double* dre = re ? static_cast<const double*>(mapped_device_pointer(re)) : nullptr;
    const double* dim = im ? static_cast<const double*>(mapped_device_pointer(im)) : nullptr;
    const double* dint = inter ? static_cast<const double*>(mapped_device_pointer(inter)) : nullptr;
    if ((inter && dint) || (!inter && dre && dim)) {
      DMV_TRY(launch_join(s->amps, s->precision, 0, s->N, dre, dim, dint, s->stream));
      DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
      return DMV_OK;
    }
  }
  DeviceBuffer stage;
  DMV_TRY(stage.reserve((size_t)chunk * 2 * sizeof(double)));
  double* a = static_cast<double*>(stage.ptr);
  double* b = a + chunk;
  int rc = DMV_OK;
  for (int64_t off = 0; off < s->N && rc == DMV_OK; off += chunk) {
    const int64_t cnt = std::min(chunk, s->N - off);
    if (inter) {
      if (cudaMemcpyAsync(a, inter + 2 * off, (size_t)cnt * 2 * sizeof(double), cudaMemcpyHostToDevice,
                          s->stream) != cudaSuccess)
        rc = set_error(DMV_ERR_CUDA, "host-to-device copy failed");
      if (rc == DMV_OK) rc = launch_join(s->amps, s->precision, off, cnt, nullptr, nullptr, a, s->stream);
    } else {
      if (cudaMemcpyAsync(a, re + off, (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice, s->stream) !=
              cudaSuccess ||
          cudaMemcpyAsync(b, im + off, (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice, s->stream) !=
              cudaSuccess)
        rc = set_error(DMV_ERR_CUDA, "host-to-device copy failed");
      if (rc == DMV_OK) rc = launch_join(s->amps, s->precision, off, cnt, a, b, nullptr, s->stream);
    }
    if (rc == DMV_OK && cudaStreamSynchronize(s->stream) != cudaSuccess)
      rc = set_error(DMV_ERR_CUDA, "stream synchronize failed");
  }
  cudaStreamSynchronize(s->stream);
  stage.release();
  return rc;
}

int apply_gate_list(dmv_state_s* s, const std::vector<Gate>& gates, int32_t fusion) {
  Plan plan;
  const PlanOptions opt = plan_options_for(s, fusion);
  DMV_TRY(build_plan(gates, s->n, s->precision, opt, plan));
  return launch_plan(s, plan);
}

}  // namespace
}  // namespace dmv

// ===========================================================================
// Library / device
// ===========================================================================
extern "C" int dmv_last_error(void) { return dmv::last_error(); }
extern "C" const char* dmv_last_error_string(void) { return dmv::g_last_msg; }
extern "C" const char* dmv_version(void) { return "damavand_gb300 0.1.0 (sm_103a)"; }
extern "C" int64_t dmv_kernel_launch_count(void) { return dmv::g_launches.load(); }

extern "C" int dmv_debug_fail_allocations(int32_t count) {
  dmv::g_fail_allocs.store(count > 0 ? count : 0);
  return DMV_OK;
}

extern "C" int dmv_debug_tc_convert(int32_t mode) {
  clear_error();
  if (mode != 0 && mode != 1) return set_error(DMV_ERR_INVALID, "tensor-core conversion mode must be 0 or 1");
  dmv::set_tc_convert_mode(mode);
  return DMV_OK;
}

extern "C" int dmv_debug_tma_wait_limit(int64_t polls) {
  dmv::set_tma_wait_limit(polls);
  return DMV_OK;
}

extern "C" int dmv_set_device(int32_t device) {
  clear_error();
  DMV_CUDA_TRY(cudaSetDevice(device));
  return DMV_OK;
}

extern "C" int dmv_host_register(void* ptr, int64_t bytes) {
  clear_error();
  if (!ptr || bytes <= 0) return set_error(DMV_ERR_INVALID, "dmv_host_register: bad buffer");
  DMV_CUDA_TRY(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterPortable));
  return DMV_OK;
}

extern "C" int dmv_host_unregister(void* ptr) {
  clear_error();
  if (!ptr) return set_error(DMV_ERR_INVALID, "dmv_host_unregister: null pointer");
  DMV_CUDA_TRY(cudaHostUnregister(ptr));
  return DMV_OK;
}

extern "C" int dmv_profile_enable(int32_t on) {
  std::lock_guard<std::mutex> lk(dmv::g_prof_mu);
  dmv::g_prof_on = on != 0;
  return DMV_OK;
}

extern "C" int dmv_profile_reset(void) {
  std::lock_guard<std::mutex> lk(dmv::g_prof_mu);
  dmv::prof_drain(true);
  for (int f = 0; f < DMV_KERNEL_FAMILIES; ++f) {
    dmv::g_prof_launches[f] = 0;
    dmv::g_prof_ms[f] = 0.;
    dmv::g_prof_bytes[f] = 0.;
    dmv::g_prof_fmas[f] = 0.;
  }
  return DMV_OK;
}

extern "C" int dmv_profile_read(int32_t family, int64_t* launches, double* total_ms, double* algorithmic_bytes,
                                double* multiply_adds) {
  clear_error();
  if (family < 0 || family >= DMV_KERNEL_FAMILIES) return set_error(DMV_ERR_INVALID, "unknown kernel family");
  std::lock_guard<std::mutex> lk(dmv::g_prof_mu);
  dmv::prof_drain(true);
  if (launches) *launches = dmv::g_prof_launches[family];
  if (total_ms) *total_ms = dmv::g_prof_ms[family];
  if (algorithmic_bytes) *algorithmic_bytes = dmv::g_prof_bytes[family];
  if (multiply_adds) *multiply_adds = dmv::g_prof_fmas[family];
  return DMV_OK;
}

// ===========================================================================
// State
// ===========================================================================
extern "C" int dmv_state_create(int32_t num_qubits, int32_t precision, void* stream, dmv_state_t* out) {
  clear_error();
  if (!out) return set_error(DMV_ERR_INVALID, "dmv_state_create: null output handle");
  *out = nullptr;
  if (num_qubits < 1 || num_qubits > kMaxQubits)
    return set_error(DMV_ERR_INVALID, "num_qubits %d outside [1, %d]", num_qubits, kMaxQubits);
  if (precision != DMV_C128 && precision != DMV_C64)
    return set_error(DMV_ERR_INVALID, "unknown precision %d", precision);
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(DMV_ERR_NO_DEVICE, "no CUDA device visible");
  }
  dmv_state_s* s = new dmv_state_s();
  s->n = num_qubits;
  s->N = int64_t(1) << num_qubits;
  s->precision = precision;
  cudaGetDevice(&s->device);
  const cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation : cudaMalloc(&s->amps, s->amp_bytes());
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return set_error(e == cudaErrorMemoryAllocation ? DMV_ERR_OOM : DMV_ERR_CUDA,
                     "cannot allocate %d-qubit state (%.1f GB): %s", num_qubits,
                     (double)(size_t(1) << num_qubits) * (precision == DMV_C128 ? 16 : 8) / 1e9,
                     cudaGetErrorString(e));
  }
  if (stream) {
    s->stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaFree(s->amps);
      delete s;
      return set_error(DMV_ERR_CUDA, "cudaStreamCreate failed");
    }
    s->own_stream = true;
  }
  const int rc = launch_set_zero(s);
  if (rc != DMV_OK) {
    dmv_state_destroy(s);
    return rc;
  }
  *out = s;
  return DMV_OK;
}

extern "C" int dmv_state_destroy(dmv_state_t s) {
  if (!s) return DMV_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->amps) cudaFree(s->amps);
  s->amps = nullptr;
  s->ops_dev.release();
  s->phase_ops_dev.release();
  s->reduce_dev.release();
  s->chunk_dev.release();
  if (s->pinned) cudaFreeHost(s->pinned);
  if (s->ev_begin) cudaEventDestroy(s->ev_begin);
  if (s->ev_end) cudaEventDestroy(s->ev_end);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return DMV_OK;
}

extern "C" int dmv_state_info(dmv_state_t s, int32_t* num_qubits, int32_t* precision, int64_t* num_amplitudes) {
  clear_error();
  DMV_TRY(check_state(s));
  if (num_qubits) *num_qubits = s->n;
  if (precision) *precision = s->precision;
  if (num_amplitudes) *num_amplitudes = s->N;
  return DMV_OK;
}

extern "C" int dmv_state_set_zero(dmv_state_t s) {
  clear_error();
  DMV_TRY(check_state(s));
  return launch_set_zero(s);
}

extern "C" int dmv_state_set_arithmetic(dmv_state_t s, int32_t arithmetic) {
  clear_error();
  DMV_TRY(check_state(s));
  if (arithmetic != DMV_ARITH_FP64 && arithmetic != DMV_ARITH_FP32X2 && arithmetic != DMV_ARITH_INT64 &&
      arithmetic != DMV_ARITH_TC && arithmetic != DMV_ARITH_FP64_DIRECT)
    return set_error(DMV_ERR_INVALID, "unknown arithmetic %d", arithmetic);
  s->arith = arithmetic == DMV_ARITH_FP64_DIRECT ? (int32_t)dmv::ARITH_FP64 : arithmetic;
  s->fp64_rewrite = arithmetic == DMV_ARITH_FP64;
  return DMV_OK;
}

extern "C" int dmv_state_synchronize(dmv_state_t s) {
  clear_error();
  DMV_TRY(check_state(s));
  DMV_CUDA_TRY(cudaStreamSynchronize(s->stream));
  DMV_TRY(dmv::check_window_status());
  return DMV_OK;
}

extern "C" int dmv_state_device_ptr(dmv_state_t s, void** amps, void** stream) {
  clear_error();
  DMV_TRY(check_state(s));
  if (amps) *amps = s->amps;
  if (stream) *stream = s->stream;
  return DMV_OK;
}

extern "C" int dmv_state_copy_to_host(dmv_state_t s, double* re, double* im) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!re || !im) return set_error(DMV_ERR_INVALID, "null host buffer");
  return copy_out(s, re, im, nullptr);
}

extern "C" int dmv_state_copy_to_host_interleaved(dmv_state_t s, double* interleaved) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!interleaved) return set_error(DMV_ERR_INVALID, "null host buffer");
  return copy_out(s, nullptr, nullptr, interleaved);
}

extern "C" int dmv_state_load_from_host(dmv_state_t s, const double* re, const double* im) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!re || !im) return set_error(DMV_ERR_INVALID, "null host buffer");
  return copy_in(s, re, im, nullptr);
}

extern "C" int dmv_state_load_from_host_interleaved(dmv_state_t s, const double* interleaved) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!interleaved) return set_error(DMV_ERR_INVALID, "null host buffer");
  return copy_in(s, nullptr, nullptr, interleaved);
}

extern "C" int dmv_state_copy(dmv_state_t dst, dmv_state_t src) {
  clear_error();
  DMV_TRY(check_state(dst));
  DMV_TRY(check_state(src));
  if (dst->n != src->n || dst->precision != src->precision)
    return set_error(DMV_ERR_INVALID, "dmv_state_copy: size or precision mismatch");
  if (dst->stream != src->stream) DMV_CUDA_TRY(cudaStreamSynchronize(src->stream));
  DMV_CUDA_TRY(cudaMemcpyAsync(dst->amps, src->amps, src->amp_bytes(), cudaMemcpyDeviceToDevice, dst->stream));
  return DMV_OK;
}

extern "C" int dmv_state_event_begin(dmv_state_t s) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!s->ev_begin) DMV_CUDA_TRY(cudaEventCreate(&s->ev_begin));
  if (!s->ev_end) DMV_CUDA_TRY(cudaEventCreate(&s->ev_end));
  DMV_CUDA_TRY(cudaEventRecord(s->ev_begin, s->stream));
  return DMV_OK;
}

extern "C" int dmv_state_event_end(dmv_state_t s, double* elapsed_ms) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!s->ev_begin || !s->ev_end) return set_error(DMV_ERR_STATE, "dmv_state_event_end before _begin");
  DMV_CUDA_TRY(cudaEventRecord(s->ev_end, s->stream));
  DMV_CUDA_TRY(cudaEventSynchronize(s->ev_end));
  float ms = 0.f;
  DMV_CUDA_TRY(cudaEventElapsedTime(&ms, s->ev_begin, s->ev_end));
  if (elapsed_ms) *elapsed_ms = ms;
  return DMV_OK;
}

// ===========================================================================
// Gate application
// ===========================================================================
extern "C" int dmv_apply_matrix(dmv_state_t s, const double m_re[4], const double m_im[4], int32_t control,
                                int32_t target) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!m_re || !m_im) return set_error(DMV_ERR_INVALID, "null matrix");
  dmv_gate_t g;
  std::memset(&g, 0, sizeof(g));
  g.kind = DMV_GATE_MATRIX;
  g.target = target;
  g.control = control;
  for (int i = 0; i < 4; ++i) {
    g.m[2 * i] = m_re[i];
    g.m[2 * i + 1] = m_im[i];
  }
  std::vector<Gate> gates;
  DMV_TRY(parse_gates(&g, 1, s->n, gates));
  return apply_gate_list(s, gates, DMV_FUSE_NONE);
}

namespace {
// Launch statistics of the last gate list applied on this thread (dmv_last_plan_stats).
thread_local int64_t g_stat_passes = 0, g_stat_ops = 0, g_stat_bytes = 0;
void record_stats(dmv_state_s* s) {
  g_stat_passes = s->last_passes;
  g_stat_ops = s->last_ops;
  g_stat_bytes = s->last_bytes;
}
}  // namespace

extern "C" int dmv_apply_gates(dmv_state_t s, const dmv_gate_t* gates, int64_t num_gates, int32_t fusion) {
  clear_error();
  DMV_TRY(check_state(s));
  if (fusion != DMV_FUSE_NONE && fusion != DMV_FUSE_WINDOW)
    return set_error(DMV_ERR_INVALID, "unknown fusion mode %d", fusion);
  std::vector<Gate> parsed;
  DMV_TRY(parse_gates(gates, num_gates, s->n, parsed));
  DMV_TRY(apply_gate_list(s, parsed, fusion));
  record_stats(s);
  return DMV_OK;
}

extern "C" int dmv_plan_describe(int32_t num_qubits, int32_t precision, const dmv_gate_t* gates, int64_t num_gates,
                                 int32_t fusion, int32_t tile_bits, int64_t* num_passes, int64_t* num_window_passes,
                                 int64_t* num_ops, int32_t* max_local_qubits) {
  clear_error();
  if (num_qubits < 1 || num_qubits > 34) return set_error(DMV_ERR_INVALID, "num_qubits %d outside [1, 34]", num_qubits);
  if (precision != DMV_C128 && precision != DMV_C64) return set_error(DMV_ERR_INVALID, "unknown precision");
  if (fusion != DMV_FUSE_NONE && fusion != DMV_FUSE_WINDOW) return set_error(DMV_ERR_INVALID, "unknown fusion mode");
  if (tile_bits < 0 || tile_bits > 13) return set_error(DMV_ERR_INVALID, "tile_bits %d outside [0, 13]", tile_bits);
  std::vector<Gate> parsed;
  DMV_TRY(parse_gates(gates, num_gates, num_qubits, parsed));
  dmv_state_s probe;
  probe.n = num_qubits;
  probe.precision = precision;
  PlanOptions opt = plan_options_for(&probe, fusion);
  if (tile_bits > 0) opt.tile_bits = tile_bits;
  Plan plan;
  DMV_TRY(build_plan(parsed, num_qubits, precision, opt, plan));
  int64_t windows = 0;
  int32_t max_local = 0;
  for (const Pass& p : plan.passes) {
    if (p.kind == 1) {
      ++windows;
      max_local = std::max(max_local, p.low_bits + p.num_high);
    }
  }
  if (num_passes) *num_passes = (int64_t)plan.passes.size();
  if (num_window_passes) *num_window_passes = windows;
  if (num_ops) *num_ops = (int64_t)plan.ops.size();
  if (max_local_qubits) *max_local_qubits = max_local;
  return DMV_OK;
}

extern "C" int dmv_last_upload_bytes(dmv_state_t s, int64_t* total, int64_t* phase_tables) {
  clear_error();
  DMV_TRY(check_state(s));
  if (total) *total = s->last_upload_bytes;
  if (phase_tables) *phase_tables = s->last_phase_tab_bytes;
  return DMV_OK;
}

extern "C" int dmv_last_tc_stats(dmv_state_t s, int64_t* tc_passes, int64_t* blocks, int64_t* exchanges) {
  clear_error();
  DMV_TRY(check_state(s));
  if (tc_passes) *tc_passes = s->last_tc_passes;
  if (blocks) *blocks = s->last_tc_blocks;
  if (exchanges) *exchanges = s->last_tc_swaps;
  return DMV_OK;
}

extern "C" int dmv_last_plan_stats(int64_t* num_passes, int64_t* num_fused_ops, int64_t* bytes_moved) {
  if (num_passes) *num_passes = g_stat_passes;
  if (num_fused_ops) *num_fused_ops = g_stat_ops;
  if (bytes_moved) *bytes_moved = g_stat_bytes;
  return DMV_OK;
}

// ===========================================================================
// Measurement
// ===========================================================================
extern "C" int dmv_measure_device(dmv_state_t s, double* probs_device) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!probs_device) return set_error(DMV_ERR_INVALID, "null probability buffer");
  return launch_probabilities(s, probs_device);
}

extern "C" int dmv_measure(dmv_state_t s, double* probs) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!probs) return set_error(DMV_ERR_INVALID, "null probability buffer");
  DeviceBuffer buf;
  DMV_TRY(buf.reserve((size_t)s->N * sizeof(double)));
  int rc = launch_probabilities(s, static_cast<double*>(buf.ptr));
  if (rc == DMV_OK && (cudaMemcpyAsync(probs, buf.ptr, (size_t)s->N * sizeof(double), cudaMemcpyDeviceToHost,
                                       s->stream) != cudaSuccess ||
                       cudaStreamSynchronize(s->stream) != cudaSuccess))
    rc = set_error(DMV_ERR_CUDA, "probability readback failed");
  cudaStreamSynchronize(s->stream);
  buf.release();
  return rc;
}

extern "C" int dmv_expect_z(dmv_state_t s, double* expect, double* norm) {
  clear_error();
  DMV_TRY(check_state(s));
  return launch_expect_z(s, expect, norm);
}

extern "C" int dmv_sample(dmv_state_t s, const double* uniforms, int64_t k, uint64_t* samples) {
  clear_error();
  DMV_TRY(check_state(s));
  if (k < 0 || (k > 0 && (!uniforms || !samples))) return set_error(DMV_ERR_INVALID, "bad sample buffers");
  for (int64_t i = 0; i < k; ++i)
    if (!(uniforms[i] >= 0.0 && uniforms[i] < 1.0))
      return set_error(DMV_ERR_INVALID, "uniform %lld = %g outside [0,1)", (long long)i, uniforms[i]);
  return launch_sample(s, uniforms, k, samples);
}

namespace dmv {
namespace {

int check_uniforms(const double* uniforms, int64_t k) {
  for (int64_t i = 0; i < k; ++i)
    if (!(uniforms[i] >= 0.0 && uniforms[i] < 1.0))
      return set_error(DMV_ERR_INVALID, "uniform %lld = %g outside [0,1)", (long long)i, uniforms[i]);
  return DMV_OK;
}

int sample_expect(dmv_state_s* s, const double* uniforms, uint64_t seed, int64_t k, const int32_t* qubits,
                  int32_t num_obs, double* means, int64_t* set_counts) {
  if (k <= 0) return set_error(DMV_ERR_INVALID, "sampled expectation needs k >= 1 samples (got %lld)", (long long)k);
  if (k >= (int64_t(1) << 53)) return set_error(DMV_ERR_INVALID, "k = %lld samples: at most 2^53", (long long)k);
  if (num_obs < 0 || (num_obs > 0 && (!qubits || !means)))
    return set_error(DMV_ERR_INVALID, "bad observable buffers");
  for (int32_t j = 0; j < num_obs; ++j)
    if (qubits[j] < 0 || qubits[j] >= s->n)
      return set_error(DMV_ERR_INVALID, "observable %d: qubit %d outside [0, %d)", j, qubits[j], s->n);
  if (uniforms) DMV_TRY(check_uniforms(uniforms, k));
  unsigned long long counts[64];
  DMV_TRY(launch_sample_counts(s, uniforms, seed, k, counts));
  for (int32_t j = 0; j < num_obs; ++j) {
    const unsigned long long c = counts[qubits[j]];
    means[j] = (double)(k - 2 * (int64_t)c) / (double)k;
    if (set_counts) set_counts[j] = (int64_t)c;
  }
  return DMV_OK;
}

}  // namespace
}  // namespace dmv

extern "C" int dmv_sample_expect_z(dmv_state_t s, const double* uniforms, uint64_t seed, int64_t k,
                                   const int32_t* qubits, int32_t num_obs, double* means, int64_t* set_counts) {
  clear_error();
  DMV_TRY(check_state(s));
  return sample_expect(s, uniforms, seed, k, qubits, num_obs, means, set_counts);
}

extern "C" int dmv_sample_probabilities(const double* probs, int64_t num_probs, const double* uniforms, int64_t k,
                                        uint64_t* samples) {
  clear_error();
  if (!probs || num_probs <= 0 || (num_probs & (num_probs - 1)) != 0)
    return set_error(DMV_ERR_INVALID, "probability vector length must be a power of two");
  if (k < 0 || (k > 0 && (!uniforms || !samples))) return set_error(DMV_ERR_INVALID, "bad sample buffers");
  for (int64_t i = 0; i < k; ++i)
    if (!(uniforms[i] >= 0.0 && uniforms[i] < 1.0))
      return set_error(DMV_ERR_INVALID, "uniform %lld = %g outside [0,1)", (long long)i, uniforms[i]);
  int bits = 0;
  while ((int64_t(1) << bits) < num_probs) ++bits;
  cudaStream_t stream;
  DMV_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  DeviceBuffer buf;
  int rc = buf.reserve((size_t)num_probs * sizeof(double));
  if (rc == DMV_OK && cudaMemcpyAsync(buf.ptr, probs, (size_t)num_probs * sizeof(double), cudaMemcpyHostToDevice,
                                      stream) != cudaSuccess)
    rc = set_error(DMV_ERR_CUDA, "probability upload failed");
  if (rc == DMV_OK)
    rc = sample_from_device_probs(static_cast<const double*>(buf.ptr), num_probs, bits, stream, uniforms, k,
                                  samples);
  cudaStreamSynchronize(stream);
  buf.release();
  cudaStreamDestroy(stream);
  return rc;
}

extern "C" int dmv_inner_product(dmv_state_t a, dmv_state_t b, double* re, double* im) {
  clear_error();
  DMV_TRY(check_state(a));
  DMV_TRY(check_state(b));
  if (a->n != b->n || a->precision != b->precision)
    return set_error(DMV_ERR_INVALID, "inner product: size or precision mismatch");
  double r = 0., i = 0.;
  DMV_TRY(launch_inner_product(a, b, &r, &i));
  if (re) *re = r;
  if (im) *im = i;
  return DMV_OK;
}

extern "C" int dmv_adjoint_gradient(dmv_state_t s, const dmv_gate_t* gates, int64_t num_gates, const double* weights,
                                    double* loss, double* grads) {
  clear_error();
  DMV_TRY(check_state(s));
  if (!weights) return set_error(DMV_ERR_INVALID, "null weights");
  std::vector<Gate> parsed;
  DMV_TRY(parse_gates(gates, num_gates, s->n, parsed));
  int64_t np = 0;
  for (const Gate& g : parsed) np += is_parametrised(g.kind) ? 1 : 0;
  if (np > 0 && !grads) return set_error(DMV_ERR_INVALID, "null gradient buffer");
  return adjoint_gradient(s, parsed, weights, loss, grads);
}

// ===========================================================================
// Circuit front-end: src/qubit_backend/circuit.rs:78-770 with apply_method
// "gpu". Holds the gate list, observables and the device state.
// ===========================================================================
struct dmv_circuit_s {
  int32_t n = 0;
  int32_t precision = DMV_C128;
  int32_t fusion = DMV_FUSE_WINDOW;
  std::vector<Gate> gates;
  std::vector<int64_t> observables;  // gate indices (circuit.rs:652-654)
  dmv_state_t state = nullptr;
};

namespace {

int check_circuit(dmv_circuit_s* c) {
  if (!c || !c->state) return set_error(DMV_ERR_INVALID, "null or destroyed circuit handle");
  return DMV_OK;
}

bool is_observable_index(const dmv_circuit_s* c, int64_t i) {
  return std::find(c->observables.begin(), c->observables.end(), i) != c->observables.end();
}

// Gate list with observable gates flagged (skipped by forward, circuit.rs:347-349).
std::vector<Gate> flagged_gates(const dmv_circuit_s* c) {
  std::vector<Gate> g = c->gates;
  for (size_t i = 0; i < g.size(); ++i) g[i].observable = is_observable_index(c, (int64_t)i);
  return g;
}

void assign_parameters(dmv_circuit_s* c, const double* params, int64_t num) {
  // circuit.rs:308-322: parametrised gates in order, zipped with the list.
  int64_t p = 0;
  for (Gate& g : c->gates) {
    if (p >= num) break;
    if (is_parametrised(g.kind)) {
      g.theta = params[p++];
      gate_matrix(g.kind, g.theta, g.m);
    }
  }
}

}  // namespace

extern "C" int dmv_circuit_create(int32_t num_qubits, const char* apply_method, int32_t precision,
                                  dmv_circuit_t* out) {
  clear_error();
  if (!out) return set_error(DMV_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (apply_method && std::strcmp(apply_method, "gpu") != 0) {
    static const char* known[] = {"brute_force", "shuffle", "multithreading", "distributed_cpu", "distributed_gpu"};
    for (const char* k : known)
      if (std::strcmp(apply_method, k) == 0)
        return set_error(DMV_ERR_UNSUPPORTED,
                         "apply_method '%s' is not provided by this library (only 'gpu')", apply_method);
    return set_error(DMV_ERR_INVALID, "Apply method not recognized: %s", apply_method);
  }
  dmv_state_t s = nullptr;
  DMV_TRY(dmv_state_create(num_qubits, precision, nullptr, &s));
  dmv_circuit_s* c = new dmv_circuit_s();
  c->n = num_qubits;
  c->precision = precision;
  c->state = s;
  *out = c;
  return DMV_OK;
}

extern "C" int dmv_circuit_destroy(dmv_circuit_t c) {
  if (!c) return DMV_OK;
  dmv_state_destroy(c->state);
  delete c;
  return DMV_OK;
}

extern "C" int dmv_circuit_add_gate(dmv_circuit_t c, int32_t kind, int32_t target, int32_t control, double theta,
                                    int32_t is_observable) {
  clear_error();
  DMV_TRY(check_circuit(c));
  dmv_gate_t g;
  std::memset(&g, 0, sizeof(g));
  g.kind = kind;
  g.target = target;
  g.control = kind == DMV_GATE_CNOT ? control : -1;
  g.theta = theta;
  std::vector<Gate> parsed;
  DMV_TRY(parse_gates(&g, 1, c->n, parsed));
  c->gates.push_back(parsed[0]);
  if (is_observable) c->observables.push_back((int64_t)c->gates.size() - 1);
  return DMV_OK;
}

extern "C" int dmv_circuit_num_gates(dmv_circuit_t c, int64_t* num_gates, int64_t* num_params,
                                     int64_t* num_observables) {
  clear_error();
  DMV_TRY(check_circuit(c));
  int64_t np = 0;
  for (const Gate& g : c->gates) np += is_parametrised(g.kind) ? 1 : 0;
  if (num_gates) *num_gates = (int64_t)c->gates.size();
  if (num_params) *num_params = np;
  if (num_observables) *num_observables = (int64_t)c->observables.size();
  return DMV_OK;
}

extern "C" int dmv_circuit_get_gate(dmv_circuit_t c, int64_t index, dmv_gate_t* gate, int32_t* is_observable) {
  clear_error();
  DMV_TRY(check_circuit(c));
  if (index < 0 || index >= (int64_t)c->gates.size() || !gate)
    return set_error(DMV_ERR_INVALID, "gate index %lld out of range", (long long)index);
  const Gate& g = c->gates[(size_t)index];
  std::memset(gate, 0, sizeof(*gate));
  gate->kind = g.kind;
  gate->target = g.target;
  gate->control = g.control;
  gate->theta = g.theta;
  std::memcpy(gate->m, g.m, sizeof(g.m));
  if (is_observable) *is_observable = is_observable_index(c, index) ? 1 : 0;
  return DMV_OK;
}

extern "C" int dmv_circuit_set_parameters(dmv_circuit_t c, const double* params, int64_t num_params) {
  clear_error();
  DMV_TRY(check_circuit(c));
  if (num_params > 0 && !params) return set_error(DMV_ERR_INVALID, "null parameter buffer");
  assign_parameters(c, params, num_params);
  return DMV_OK;
}

extern "C" int dmv_circuit_set_fusion(dmv_circuit_t c, int32_t fusion) {
  clear_error();
  DMV_TRY(check_circuit(c));
  if (fusion != DMV_FUSE_NONE && fusion != DMV_FUSE_WINDOW)
    return set_error(DMV_ERR_INVALID, "unknown fusion mode %d", fusion);
  c->fusion = fusion;
  return DMV_OK;
}

extern "C" int dmv_circuit_set_arithmetic(dmv_circuit_t c, int32_t arithmetic) {
  clear_error();
  DMV_TRY(check_circuit(c));
  return dmv_state_set_arithmetic(c->state, arithmetic);
}

extern "C" int dmv_circuit_reset_amplitudes(dmv_circuit_t c) {
  clear_error();
  DMV_TRY(check_circuit(c));
  return launch_set_zero(c->state);
}

extern "C" int dmv_circuit_reset(dmv_circuit_t c) {
  clear_error();
  DMV_TRY(check_circuit(c));
  DMV_TRY(launch_set_zero(c->state));
  c->gates.clear();  // circuit.rs:303-306 clears the gates only (observable indices stay)
  return DMV_OK;
}

extern "C" int dmv_circuit_forward(dmv_circuit_t c) {
  clear_error();
  DMV_TRY(check_circuit(c));
  const int rc = apply_gate_list(c->state, flagged_gates(c), c->fusion);
  record_stats(c->state);
  return rc;
}

extern "C" int dmv_circuit_state(dmv_circuit_t c, dmv_state_t* state) {
  clear_error();
  DMV_TRY(check_circuit(c));
  if (state) *state = c->state;
  return DMV_OK;
}

extern "C" int dmv_circuit_observables(dmv_circuit_t c, int32_t* readout_qubits) {
  clear_error();
  DMV_TRY(check_circuit(c));
  for (size_t j = 0; j < c->observables.size(); ++j) {
    const int64_t gi = c->observables[j];
    // A reset() keeps stale observable indices; one past the gate list reads as -1.
    readout_qubits[j] = gi < (int64_t)c->gates.size() ? c->gates[(size_t)gi].target : -1;
  }
  return DMV_OK;
}

extern "C" int dmv_circuit_extract_expectation_values(dmv_circuit_t c, const uint64_t* samples, int64_t k,
                                                      double* out) {
  clear_error();
  DMV_TRY(check_circuit(c));
  const size_t nobs = c->observables.size();
  std::vector<int32_t> q(nobs);
  for (size_t j = 0; j < nobs; ++j) {
    const int64_t gi = c->observables[j];
    if (gi >= (int64_t)c->gates.size())
      return set_error(DMV_ERR_STATE, "observable %zu refers to gate %lld, past the gate list", j, (long long)gi);
    q[j] = c->gates[(size_t)gi].target;
  }
  for (int64_t s = 0; s < k; ++s)
    for (size_t j = 0; j < nobs; ++j)
      out[(size_t)s * nobs + j] = ((samples[s] >> (q[j] & 63)) & 1) ? -1. : 1.;
  return DMV_OK;
}

extern "C" int dmv_circuit_sample_expectation_values(dmv_circuit_t c, const double* uniforms, uint64_t seed,
                                                     int64_t k, double* means) {
  clear_error();
  DMV_TRY(check_circuit(c));
  const size_t nobs = c->observables.size();
  std::vector<int32_t> q(nobs);
  for (size_t j = 0; j < nobs; ++j) {
    const int64_t gi = c->observables[j];
    if (gi >= (int64_t)c->gates.size())
      return set_error(DMV_ERR_STATE, "observable %zu refers to gate %lld, past the gate list", j, (long long)gi);
    q[j] = c->gates[(size_t)gi].target;
  }
  return sample_expect(c->state, uniforms, seed, k, q.data(), (int32_t)nobs, means, nullptr);
}

extern "C" int dmv_circuit_fidelity_with_parameters(dmv_circuit_t c, const double* p1, int64_t n1, const double* p2,
                                                    int64_t n2, double* fidelity) {
  // circuit.rs:753-769 then circuit_metrics.rs:11-32: |<psi1|psi2>|^2, then reset().
  clear_error();
  DMV_TRY(check_circuit(c));
  dmv_state_t first = nullptr;
  DMV_TRY(dmv_state_create(c->n, c->precision, c->state->stream, &first));
  int rc = DMV_OK;
  do {
    if ((rc = launch_set_zero(c->state)) != DMV_OK) break;
    assign_parameters(c, p1, n1);
    if ((rc = apply_gate_list(c->state, flagged_gates(c), c->fusion)) != DMV_OK) break;
    if ((rc = dmv_state_copy(first, c->state)) != DMV_OK) break;
    if ((rc = launch_set_zero(c->state)) != DMV_OK) break;
    assign_parameters(c, p2, n2);
    if ((rc = apply_gate_list(c->state, flagged_gates(c), c->fusion)) != DMV_OK) break;
    double re = 0., im = 0.;
    if ((rc = launch_inner_product(first, c->state, &re, &im)) != DMV_OK) break;
    if (fidelity) *fidelity = re * re + im * im;
    if ((rc = launch_set_zero(c->state)) != DMV_OK) break;
    c->gates.clear();
  } while (false);
  dmv_state_destroy(first);
  return rc;
}

extern "C" int dmv_circuit_adjoint(dmv_circuit_t c, const double* weights, double* loss, double* grads) {
  clear_error();
  DMV_TRY(check_circuit(c));
  if (!weights) return set_error(DMV_ERR_INVALID, "null weights");
  return adjoint_gradient(c->state, flagged_gates(c), weights, loss, grads);
}

// ===========================================================================
// Legacy ABI (damavand-gpu/rust_communication.cu). One process-global state.
// ===========================================================================
namespace {
std::mutex g_legacy_mu;
dmv_state_t g_legacy = nullptr;
int64_t g_n_apply = 0;
// Gates applied through the per-gate legacy call are queued and run as one
// fused gate list (qubit-window passes) when the state is next read, loaded
// or when the queue is long: the reference front-end calls once per gate
// (src/qubit_backend/circuit_gpu.rs:31-60), and every read of the state goes
// through this library, so the deferral is invisible to it.
std::vector<dmv_gate_t> g_legacy_pending;
constexpr size_t kLegacyQueue = 8192;

void legacy_report(const char* where) {
  std::fprintf(stderr, "damavand_gb300: %s: %s\n", where, g_last_msg);
}

// Runs the queued legacy gates (caller holds g_legacy_mu).
void legacy_flush(const char* where) {
  if (g_legacy_pending.empty() || !g_legacy) {
    g_legacy_pending.clear();
    return;
  }
  const int rc = dmv_apply_gates(g_legacy, g_legacy_pending.data(), (int64_t)g_legacy_pending.size(),
                                 DMV_FUSE_WINDOW);
  g_legacy_pending.clear();
  if (rc != DMV_OK) legacy_report(where);
}

// Complex128 arithmetic of the legacy state: DAMAVAND_GB300_ARITHMETIC = fp64
// (default), fp64-direct, fp32x2, int64 or tc, so an unchanged front-end can select it.
int32_t legacy_arithmetic() {
  const char* v = std::getenv("DAMAVAND_GB300_ARITHMETIC");
  if (!v || !*v) return DMV_ARITH_FP64;
  const std::string a(v);
  if (a == "fp32x2") return DMV_ARITH_FP32X2;
  if (a == "int64") return DMV_ARITH_INT64;
  if (a == "tc") return DMV_ARITH_TC;
  if (a == "fp64-direct") return DMV_ARITH_FP64_DIRECT;
  if (a != "fp64") std::fprintf(stderr, "damavand_gb300: unknown DAMAVAND_GB300_ARITHMETIC '%s': fp64\n", v);
  return DMV_ARITH_FP64;
}

int log2_exact(int64_t v) {
  if (v <= 0 || (v & (v - 1)) != 0) return -1;
  int b = 0;
  while ((int64_t(1) << b) < v) ++b;
  return b;
}

bool legacy_ready(const char* where, int num_amplitudes) {
  if (!g_legacy) {
    set_error(DMV_ERR_STATE, "init_quantum_state has not been called");
    legacy_report(where);
    return false;
  }
  if ((int64_t)num_amplitudes != g_legacy->N) {
    set_error(DMV_ERR_INVALID, "num_amplitudes_per_gpu %d does not match the state (%lld)", num_amplitudes,
              (long long)g_legacy->N);
    legacy_report(where);
    return false;
  }
  return true;
}
}  // namespace

extern "C" int get_number_of_available_gpus(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count;
}

extern "C" double get_memory_for_gpu(int local_gpu_rank) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, local_gpu_rank) != cudaSuccess) {
    cudaGetLastError();
    set_error(DMV_ERR_INVALID, "no device %d", local_gpu_rank);
    legacy_report("get_memory_for_gpu");
    return 0.0;
  }
  return (double)prop.totalGlobalMem / 1048576.0;
}

extern "C" int peer_access_allowed(int, int) { return 0; }

extern "C" void print_timers(void) {
  // Kernel timings come from CUDA events and ncu; this prints call counts.
  std::lock_guard<std::mutex> lk(g_legacy_mu);
  legacy_flush("print_timers");
  std::printf("apply calls %lld\n", (long long)g_n_apply);
  std::printf("kernel launches %lld\n", (long long)dmv_kernel_launch_count());
}

extern "C" void init_quantum_state(int num_amplitudes_per_gpu, int num_gpus_per_node, int is_first_node) {
  std::lock_guard<std::mutex> lk(g_legacy_mu);
  clear_error();
  if (num_gpus_per_node != 1) {
    set_error(DMV_ERR_UNSUPPORTED, "only one GPU is supported (got %d)", num_gpus_per_node);
    legacy_report("init_quantum_state");
    return;
  }
  const int n = log2_exact(num_amplitudes_per_gpu);
  if (n < 1) {
    set_error(DMV_ERR_INVALID, "num_amplitudes_per_gpu %d is not a power of two >= 2", num_amplitudes_per_gpu);
    legacy_report("init_quantum_state");
    return;
  }
  g_legacy_pending.clear();  // gates queued for the state being replaced
  if (g_legacy && g_legacy->n != n) {
    dmv_state_destroy(g_legacy);
    g_legacy = nullptr;
  }
  if (!g_legacy) {
    if (dmv_state_create(n, DMV_C128, nullptr, &g_legacy) != DMV_OK) {
      legacy_report("init_quantum_state");
      g_legacy = nullptr;
      return;
    }
    dmv_state_set_arithmetic(g_legacy, legacy_arithmetic());
  }
  // |0...0> on the first node, the zero vector otherwise (rust_communication.cu:185-194).
  if (is_first_node) {
    if (launch_set_zero(g_legacy) != DMV_OK) legacy_report("init_quantum_state");
  } else if (cudaMemsetAsync(g_legacy->amps, 0, g_legacy->amp_bytes(), g_legacy->stream) != cudaSuccess) {
    set_error(DMV_ERR_CUDA, "memset failed");
    legacy_report("init_quantum_state");
  }
}

extern "C" void apply_one_qubit_gate_gpu_local(double* gate_matrix_real, double* gate_matrix_imaginary,
                                               int num_qubits, int num_amplitudes_per_gpu, int control_qubit,
                                               int target_qubit) {
  std::lock_guard<std::mutex> lk(g_legacy_mu);
  clear_error();
  if (!legacy_ready("apply_one_qubit_gate_gpu_local", num_amplitudes_per_gpu)) return;
  if (num_qubits != g_legacy->n) {
    set_error(DMV_ERR_INVALID, "num_qubits %d does not match the state (%d)", num_qubits, g_legacy->n);
    legacy_report("apply_one_qubit_gate_gpu_local");
    return;
  }
  if (!gate_matrix_real || !gate_matrix_imaginary) {
    set_error(DMV_ERR_INVALID, "null matrix");
    legacy_report("apply_one_qubit_gate_gpu_local");
    return;
  }
  const int control = control_qubit < 0 ? -1 : control_qubit;
  if (target_qubit < 0 || target_qubit >= g_legacy->n || control >= g_legacy->n || control == target_qubit) {
    set_error(DMV_ERR_INVALID, "bad qubits: target %d control %d for %d qubits", target_qubit, control_qubit,
              g_legacy->n);
    legacy_report("apply_one_qubit_gate_gpu_local");
    return;
  }
  dmv_gate_t g;
  std::memset(&g, 0, sizeof(g));
  g.kind = DMV_GATE_MATRIX;
  g.target = target_qubit;
  g.control = control;
  for (int k = 0; k < 4; ++k) {
    g.m[2 * k] = gate_matrix_real[k];
    g.m[2 * k + 1] = gate_matrix_imaginary[k];
  }
  g_legacy_pending.push_back(g);
  if (g_legacy_pending.size() >= kLegacyQueue) legacy_flush("apply_one_qubit_gate_gpu_local");
  ++g_n_apply;
}

extern "C" void measure_on_gpu(int num_amplitudes_per_gpu, double* probabilities) {
  std::lock_guard<std::mutex> lk(g_legacy_mu);
  clear_error();
  if (!legacy_ready("measure_on_gpu", num_amplitudes_per_gpu)) return;
  legacy_flush("measure_on_gpu");
  if (dmv_measure(g_legacy, probabilities) != DMV_OK) legacy_report("measure_on_gpu");
}

extern "C" void sequential_measure_on_gpu(int num_amplitudes_per_gpu, double* probabilities) {
  measure_on_gpu(num_amplitudes_per_gpu, probabilities);
}

extern "C" void concurrent_measure_on_gpu(int num_amplitudes_per_gpu, double* probabilities) {
  measure_on_gpu(num_amplitudes_per_gpu, probabilities);
}

extern "C" void retrieve_amplitudes_on_host(int num_amplitudes_per_gpu, double* local_amplitudes_real,
                                            double* local_amplitudes_imaginary) {
  std::lock_guard<std::mutex> lk(g_legacy_mu);
  clear_error();
  if (!legacy_ready("retrieve_amplitudes_on_host", num_amplitudes_per_gpu)) return;
  legacy_flush("retrieve_amplitudes_on_host");
  if (dmv_state_copy_to_host(g_legacy, local_amplitudes_real, local_amplitudes_imaginary) != DMV_OK)
    legacy_report("retrieve_amplitudes_on_host");
}

extern "C" void load_amplitudes_local_on_device(int num_amplitudes_per_gpu, double* local_amplitudes_real,
                                                double* local_amplitudes_imaginary) {
  std::lock_guard<std::mutex> lk(g_legacy_mu);
  clear_error();
  if (!legacy_ready("load_amplitudes_local_on_device", num_amplitudes_per_gpu)) return;
  g_legacy_pending.clear();  // the load replaces every amplitude the queued gates would change
  if (dmv_state_load_from_host(g_legacy, local_amplitudes_real, local_amplitudes_imaginary) != DMV_OK)
    legacy_report("load_amplitudes_local_on_device");
}

extern "C" void exchange_amplitudes_between_gpus(int, int, int) {
  set_error(DMV_ERR_UNSUPPORTED, "distributed_gpu is not provided: one GPU only");
  legacy_report("exchange_amplitudes_between_gpus");
}

extern "C" void apply_one_qubit_gate_gpu_distributed(double*, double*, int, int, int, int) {
  set_error(DMV_ERR_UNSUPPORTED, "distributed_gpu is not provided: one GPU only");
  legacy_report("apply_one_qubit_gate_gpu_distributed");
}

extern "C" void split_amplitudes_between_gpus(int, double*, double*, double*, double*) {
  set_error(DMV_ERR_UNSUPPORTED, "distributed_gpu is not provided: one GPU only");
  legacy_report("split_amplitudes_between_gpus");
}
