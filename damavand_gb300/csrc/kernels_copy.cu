// Layout conversion between the device's interleaved amplitudes (complex128
// or complex64) and the host-side layouts: split real/imag doubles (the
// reference's SoA retrieve_amplitudes_on_host) or interleaved doubles.
#include <algorithm>

#include "internal.h"

namespace dmv {

namespace {

template <typename V>
__global__ void k_split(const V* __restrict__ amps, int64_t offset, int64_t count, double* __restrict__ re,
                        double* __restrict__ im, double* __restrict__ inter) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const V v = amps[offset + i];
    if (inter) {
      reinterpret_cast<double2*>(inter)[i] = make_double2((double)v.x, (double)v.y);
    } else {
      re[i] = (double)v.x;
      im[i] = (double)v.y;
    }
  }
}

template <typename V, typename R>
__global__ void k_join(V* __restrict__ amps, int64_t offset, int64_t count, const double* __restrict__ re,
                       const double* __restrict__ im, const double* __restrict__ inter) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    V v;
    if (inter) {
      const double2 d = reinterpret_cast<const double2*>(inter)[i];
      v.x = (R)d.x;
      v.y = (R)d.y;
    } else {
      v.x = (R)re[i];
      v.y = (R)im[i];
    }
    amps[offset + i] = v;
  }
}

int grid_for(int64_t count) { return (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, 4096)); }

}  // namespace

int launch_split(const void* amps, int precision, int64_t offset, int64_t count, double* re_dev, double* im_dev,
                 double* inter_dev, cudaStream_t stream) {
  if (precision == DMV_C128)
    k_split<double2><<<grid_for(count), 256, 0, stream>>>(static_cast<const double2*>(amps), offset, count, re_dev,
                                                         im_dev, inter_dev);
  else
    k_split<float2><<<grid_for(count), 256, 0, stream>>>(static_cast<const float2*>(amps), offset, count, re_dev,
                                                        im_dev, inter_dev);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

int launch_join(void* amps, int precision, int64_t offset, int64_t count, const double* re_dev, const double* im_dev,
                const double* inter_dev, cudaStream_t stream) {
  if (precision == DMV_C128)
    k_join<double2, double><<<grid_for(count), 256, 0, stream>>>(static_cast<double2*>(amps), offset, count, re_dev,
                                                                 im_dev, inter_dev);
  else
    k_join<float2, float><<<grid_for(count), 256, 0, stream>>>(static_cast<float2*>(amps), offset, count, re_dev,
                                                               im_dev, inter_dev);
  count_launch();
  DMV_CUDA_TRY(cudaGetLastError());
  return DMV_OK;
}

}  // namespace dmv
