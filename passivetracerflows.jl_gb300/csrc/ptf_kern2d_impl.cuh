// Launch dispatch of the 2D pass kernels over the supported lengths.
#pragma once
#include "ptf_internal.h"

namespace ptf {

template <typename T, int N> struct PassLaunch {
  typedef typename cplx_of<T>::type C;
  static size_t line_bytes() { return (size_t)line_stride(N) * sizeof(C); }
  // Largest block the compiled kernel can launch with (register bound).
  template <typename K> static int max_threads(K kern) {
    cudaFuncAttributes at;
    if (cudaFuncGetAttributes(&at, kern) != cudaSuccess) return 0;
    return at.maxThreadsPerBlock;
  }
  static cudaError_t col(const ColArgs<T>& a, int W, int nbx, int batch, cudaStream_t st) {
    if (W * (N / FFT_E) > max_threads(col_pass_kernel<T, N>)) return cudaErrorInvalidConfiguration;
    const size_t smem = (size_t)W * line_bytes();
    cudaError_t e = cudaFuncSetAttribute(col_pass_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    col_pass_kernel<T, N><<<dim3(nbx, batch), dim3(W * (N / FFT_E)), smem, st>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t row(const RowArgs<T>& a, int P, int nby, int batch, cudaStream_t st) {
    if (P * (N / FFT_E) > max_threads(row_pass_kernel<T, N>)) return cudaErrorInvalidConfiguration;
    const size_t smem = (size_t)P * line_bytes();
    cudaError_t e = cudaFuncSetAttribute(row_pass_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    row_pass_kernel<T, N><<<dim3(nby, batch), dim3(P * (N / FFT_E)), smem, st>>>(a);
    return cudaGetLastError();
  }
};

#define PTF_FOR_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

template <typename T>
cudaError_t launch_col2d_impl(int ny, const ColArgs<T>& a, int W, int nbx, int batch, cudaStream_t st) {
  switch (ny) {
#define PTF_CASE(n) case n: return PassLaunch<T, n>::col(a, W, nbx, batch, st);
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return cudaErrorInvalidValue;
  }
}
template <typename T>
cudaError_t launch_row2d_impl(int nx, const RowArgs<T>& a, int P, int nby, int batch, cudaStream_t st) {
  switch (nx) {
#define PTF_CASE(n) case n: return PassLaunch<T, n>::row(a, P, nby, batch, st);
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return cudaErrorInvalidValue;
  }
}
template <typename T, int N> int max_lines_n(bool col) {
  typedef typename cplx_of<T>::type C;
  const size_t lb = (size_t)line_stride(N) * sizeof(C);
  int m = (int)((160u * 1024u) / lb);
  const int tpl = N / FFT_E;
  const int mt = col ? PassLaunch<T, N>::max_threads(col_pass_kernel<T, N>)
                     : PassLaunch<T, N>::max_threads(row_pass_kernel<T, N>);
  while (m > 1 && m * tpl > mt) --m;
  return m < 1 ? 1 : m;
}
// Largest number of lines (columns W or row pairs P) per block for length n.
template <typename T> int max_lines_impl(int n, bool col) {
  switch (n) {
#define PTF_CASE(v) case v: return max_lines_n<T, v>(col);
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return 1;
  }
}

}  // namespace ptf

#define PTF_INSTANTIATE_2D(T)                                                                            \
  namespace ptf {                                                                                        \
  template <> cudaError_t launch_col2d<T>(int ny, const ColArgs<T>& a, int W, int nbx, int batch,       \
                                          cudaStream_t st) {                                             \
    return launch_col2d_impl<T>(ny, a, W, nbx, batch, st);                                               \
  }                                                                                                      \
  template <> cudaError_t launch_row2d<T>(int nx, const RowArgs<T>& a, int P, int nby, int batch,       \
                                          cudaStream_t st) {                                             \
    return launch_row2d_impl<T>(nx, a, P, nby, batch, st);                                               \
  }                                                                                                      \
  template <> int max_lines_per_block<T>(int n, bool col) { return max_lines_impl<T>(n, col); }                         \
  }
