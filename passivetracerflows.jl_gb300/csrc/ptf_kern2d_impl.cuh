// Launchers of the 2D pass kernels for one (precision, length).  Each pair is
// explicitly instantiated in its own object (ptf_k2d_inst.cu) so the
// kernels compile in parallel; ptf_kern2d.cu dispatches over them.
#pragma once
#include "ptf_internal.h"

#ifndef PTF_COL_CSTRIDE
#define PTF_COL_CSTRIDE 1
#endif

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
  template <int MODE, int CS>
  static cudaError_t col_k(const ColArgs<T>& a, int W, int nbx, int batch, cudaStream_t st, int carve) {
    auto kern = col_pass_kernel<T, N, MODE, CS>;
    if (W * col_tpl<T, N>() > max_threads(kern)) return cudaErrorInvalidConfiguration;
    const size_t smem = col_smem_bytes_mode<T, N>(W, MODE);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, carve < 0 ? -1 : carve);
    if (e != cudaSuccess) return e;
    kern<<<dim3(nbx, batch), dim3(W * col_tpl<T, N>()), smem, st>>>(a);
    return cudaGetLastError();
  }
  // Square grids (the row pitch equals square_pitch<N>) take the kernel with
  // the pitch compiled in; others the runtime-stride kernel.
  template <int MODE>
  static cudaError_t col_m(const ColArgs<T>& a, int W, int nbx, int batch, cudaStream_t st, int carve) {
#if PTF_COL_CSTRIDE
    constexpr bool stage = MODE >= COL_RK4_1 && MODE <= COL_ETD_4;
    if (a.stride == square_pitch<N>() && (!stage || a.tplane == (long long)N * square_pitch<N>()))
      return col_k<MODE, square_pitch<N>()>(a, W, nbx, batch, st, carve);
#endif
    return col_k<MODE, 0>(a, W, nbx, batch, st, carve);
  }
  static cudaError_t col(const ColArgs<T>& a, int W, int nbx, int batch, cudaStream_t st, int carve = -1) {
    // the layout's row groups must divide every register's row offset
    if (a.ylog < 0 || a.ylog > col_ylog_max<T, N>()) return cudaErrorInvalidValue;
    switch (a.mode) {
      case COL_PROLOGUE: return col_m<COL_PROLOGUE>(a, W, nbx, batch, st, carve);
      case COL_FWD_STORE: return col_m<COL_FWD_STORE>(a, W, nbx, batch, st, carve);
      case COL_FWD_N: return col_m<COL_FWD_N>(a, W, nbx, batch, st, carve);
      case COL_RK4_1: return col_m<COL_RK4_1>(a, W, nbx, batch, st, carve);
      case COL_RK4_2: return col_m<COL_RK4_2>(a, W, nbx, batch, st, carve);
      case COL_RK4_3: return col_m<COL_RK4_3>(a, W, nbx, batch, st, carve);
      case COL_RK4_4: return col_m<COL_RK4_4>(a, W, nbx, batch, st, carve);
      case COL_ETD_1: return col_m<COL_ETD_1>(a, W, nbx, batch, st, carve);
      case COL_ETD_2: return col_m<COL_ETD_2>(a, W, nbx, batch, st, carve);
      case COL_ETD_3: return col_m<COL_ETD_3>(a, W, nbx, batch, st, carve);
      case COL_ETD_4: return col_m<COL_ETD_4>(a, W, nbx, batch, st, carve);
      case COL_YINV3: return col_m<COL_YINV3>(a, W, nbx, batch, st, carve);
      default: return cudaErrorInvalidValue;
    }
  }
  static cudaError_t row(const RowArgs<T>& a, int P, int nby, int batch, cudaStream_t st) {
    // the staged variant (plain layout only) when its shared memory fits,
    // else the direct kernel
    if (a.ylog < 0 || a.ylog > 2) return cudaErrorInvalidValue;
    if (a.tma && a.ylog == 0 && a.mode == ROW_RHS && row_tma_smem_bytes<T, N>(P, a.pitch) <= 227u * 1024u &&
        P * pass_tpl<T, N>() <= max_threads(row_rhs_tma_kernel<T, N>)) {
      const size_t smem = row_tma_smem_bytes<T, N>(P, a.pitch);
      cudaError_t e = cudaFuncSetAttribute(row_rhs_tma_kernel<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) return e;
      row_rhs_tma_kernel<T, N><<<dim3(nby, batch), dim3(P * pass_tpl<T, N>()), smem, st>>>(a);
      return cudaGetLastError();
    }
    return a.ylog > 0 ? row_k<true>(a, P, nby, batch, st) : row_k<false>(a, P, nby, batch, st);
  }
  // rows of a pair interleaved (PAIRED: spectral layout ylog >= 1) or not
  template <bool PAIRED> static cudaError_t row_k(const RowArgs<T>& a, int P, int nby, int batch, cudaStream_t st) {
    auto kern = row_pass_kernel<T, N, PAIRED>;
    if (P * pass_tpl<T, N>() > max_threads(kern)) return cudaErrorInvalidConfiguration;
    const size_t smem = row_smem_bytes<T, N>(P, a.park_slots < 1 ? 1 : a.park_slots);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3(nby, batch), dim3(P * pass_tpl<T, N>()), smem, st>>>(a);
    return cudaGetLastError();
  }
};

template <typename T, int N> int max_lines_n(bool col) {
  typedef typename cplx_of<T>::type C;
  const size_t lb = col ? col_smem_bytes_mode<T, N>(1, COL_ETD_4) : row_smem_bytes<T, N>(1, 2);
  (void)sizeof(C);
  int m = (int)((200u * 1024u) / lb);
  const int tpl = col ? col_tpl<T, N>() : pass_tpl<T, N>();
  // the ETDRK4 stage-1 kernel carries the most state: it bounds every mode
  const int mt = col ? PassLaunch<T, N>::max_threads(col_pass_kernel<T, N, COL_ETD_1>)
                     : PassLaunch<T, N>::max_threads(row_pass_kernel<T, N>);
  while (m > 1 && m * tpl > mt) --m;
  return m < 1 ? 1 : m;
}

#define PTF_FOR_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

}  // namespace ptf
