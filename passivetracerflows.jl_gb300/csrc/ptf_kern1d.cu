// 1D stage-pass launchers: one (precision, length) per ptf_k1d_inst.cu object,
// dispatched here over the length and the stepper mode.
#include "ptf_internal.h"
#include "ptf_pass1d.cuh"

namespace ptf {

template <typename T, int N> struct Line1DLaunch {
  template <int MODE> static cudaError_t run_m(const Line1DArgs<T>& a, int P, int nblk, cudaStream_t st) {
    const size_t smem = line1d_smem_bytes<T, N>(P);
    cudaError_t e = cudaFuncSetAttribute(line1d_kernel<T, N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    line1d_kernel<T, N, MODE><<<nblk, P * (N / PassE<T, N>::value), smem, st>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t run(int mode, const Line1DArgs<T>& a, int P, int nblk, cudaStream_t st);
};

template <typename T, int N>
cudaError_t Line1DLaunch<T, N>::run(int mode, const Line1DArgs<T>& a, int P, int nblk, cudaStream_t st) {
  switch (mode) {
    case COL_FWD_N: return run_m<COL_FWD_N>(a, P, nblk, st);
    case COL_RK4_1: return run_m<COL_RK4_1>(a, P, nblk, st);
    case COL_RK4_2: return run_m<COL_RK4_2>(a, P, nblk, st);
    case COL_RK4_3: return run_m<COL_RK4_3>(a, P, nblk, st);
    case COL_RK4_4: return run_m<COL_RK4_4>(a, P, nblk, st);
    case COL_ETD_1: return run_m<COL_ETD_1>(a, P, nblk, st);
    case COL_ETD_2: return run_m<COL_ETD_2>(a, P, nblk, st);
    case COL_ETD_3: return run_m<COL_ETD_3>(a, P, nblk, st);
    case COL_ETD_4: return run_m<COL_ETD_4>(a, P, nblk, st);
    default: return cudaErrorInvalidValue;
  }
}

#ifdef PTF_K1D_INST
template struct Line1DLaunch<PTF_T, PTF_N>;
#else
#define PTF_EXTERN(n)                             \
  extern template struct Line1DLaunch<float, n>;  \
  extern template struct Line1DLaunch<double, n>;
PTF_EXTERN(16) PTF_EXTERN(32) PTF_EXTERN(64) PTF_EXTERN(128) PTF_EXTERN(256) PTF_EXTERN(512) PTF_EXTERN(1024)
PTF_EXTERN(2048) PTF_EXTERN(4096)
#undef PTF_EXTERN

template <typename T>
cudaError_t launch_line1d(int nx, int mode, const Line1DArgs<T>& a, int P, int nblk, cudaStream_t st) {
  switch (nx) {
#define PTF_CASE(n) case n: return Line1DLaunch<T, n>::run(mode, a, P, nblk, st);
    PTF_CASE(16) PTF_CASE(32) PTF_CASE(64) PTF_CASE(128) PTF_CASE(256) PTF_CASE(512) PTF_CASE(1024)
    PTF_CASE(2048) PTF_CASE(4096)
#undef PTF_CASE
    default: return cudaErrorInvalidValue;
  }
}
template <typename T> int line1d_tpl(int nx) {
  switch (nx) {
#define PTF_CASE(n) case n: return n / PassE<T, n>::value;
    PTF_CASE(16) PTF_CASE(32) PTF_CASE(64) PTF_CASE(128) PTF_CASE(256) PTF_CASE(512) PTF_CASE(1024)
    PTF_CASE(2048) PTF_CASE(4096)
#undef PTF_CASE
    default: return 1;
  }
}
template cudaError_t launch_line1d<float>(int, int, const Line1DArgs<float>&, int, int, cudaStream_t);
template cudaError_t launch_line1d<double>(int, int, const Line1DArgs<double>&, int, int, cudaStream_t);
template int line1d_tpl<float>(int);
template int line1d_tpl<double>(int);
#endif

}  // namespace ptf
