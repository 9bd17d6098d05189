// Element conversion kernels between the FP64 user layout and the
// compute-precision internal layout.
#include "ptf_internal.h"

namespace ptf {

template <typename T>
__global__ void real_in_kernel(const double* __restrict__ src, T* __restrict__ dst, long long n, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (T)(src[i] * scale);
}
template <typename T>
__global__ void real_out_kernel(const T* __restrict__ src, double* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}
template <typename T>
__global__ void spec_in_kernel(const double2* __restrict__ src, typename cplx_of<T>::type* __restrict__ dst, int nkr,
                               int pitch, long long rows) {
  const long long n = rows * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / pitch;
    const int k = (int)(i - r * pitch);
    typename cplx_of<T>::type z;
    if (k < nkr) { const double2 s = src[r * nkr + k]; z.x = (T)s.x; z.y = (T)s.y; }
    else { z.x = 0; z.y = 0; }
    dst[i] = z;
  }
}
template <typename T>
__global__ void spec_out_kernel(const typename cplx_of<T>::type* __restrict__ src, double2* __restrict__ dst, int nkr,
                                int pitch, long long rows) {
  const long long n = rows * nkr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / nkr;
    const int k = (int)(i - r * nkr);
    const typename cplx_of<T>::type z = src[r * pitch + k];
    dst[i] = make_double2((double)z.x, (double)z.y);
  }
}

static inline int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

template <typename T> cudaError_t launch_real_in(const double* src, T* dst, long long n, double scale, cudaStream_t st) {
  real_in_kernel<T><<<grid_for(n), 256, 0, st>>>(src, dst, n, scale);
  return cudaGetLastError();
}
template <typename T> cudaError_t launch_real_out(const T* src, double* dst, long long n, cudaStream_t st) {
  real_out_kernel<T><<<grid_for(n), 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_spec_in(const double2* src, typename cplx_of<T>::type* dst, int nkr, int pitch, long long rows, cudaStream_t st) {
  spec_in_kernel<T><<<grid_for(rows * pitch), 256, 0, st>>>(src, dst, nkr, pitch, rows);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_spec_out(const typename cplx_of<T>::type* src, double2* dst, int nkr, int pitch, long long rows, cudaStream_t st) {
  spec_out_kernel<T><<<grid_for(rows * nkr), 256, 0, st>>>(src, dst, nkr, pitch, rows);
  return cudaGetLastError();
}

template cudaError_t launch_real_in<double>(const double*, double*, long long, double, cudaStream_t);
template cudaError_t launch_real_in<float>(const double*, float*, long long, double, cudaStream_t);
template cudaError_t launch_real_out<double>(const double*, double*, long long, cudaStream_t);
template cudaError_t launch_real_out<float>(const float*, double*, long long, cudaStream_t);
template cudaError_t launch_spec_in<double>(const double2*, double2*, int, int, long long, cudaStream_t);
template cudaError_t launch_spec_in<float>(const double2*, float2*, int, int, long long, cudaStream_t);
template cudaError_t launch_spec_out<double>(const double2*, double2*, int, int, long long, cudaStream_t);
template cudaError_t launch_spec_out<float>(const float2*, double2*, int, int, long long, cudaStream_t);

}  // namespace ptf
