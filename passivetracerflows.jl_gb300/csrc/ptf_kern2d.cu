// Dispatch of the 2D pass launchers over precision and length.  The
// launchers themselves are instantiated per (precision, length) in
// ptf_k2d_inst.cu objects.
#include "ptf_kern2d_impl.cuh"

namespace ptf {

#define PTF_EXTERN(n)                                  \
  extern template struct PassLaunch<float, n>;         \
  extern template struct PassLaunch<double, n>;        \
  extern template int max_lines_n<float, n>(bool col); \
  extern template int max_lines_n<double, n>(bool col);
PTF_FOR_SIZES(PTF_EXTERN)
#undef PTF_EXTERN

template <typename T>
cudaError_t launch_col(int n, const ColArgs<T>& a, int W, int nbx, int batch, cudaStream_t st, int carve) {
  switch (n) {
#define PTF_CASE(n) case n: return PassLaunch<T, n>::col(a, W, nbx, batch, st, carve);
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return cudaErrorInvalidValue;
  }
}
template <typename T>
cudaError_t launch_row(int nx, const RowArgs<T>& a, int P, int nby, int batch, cudaStream_t st) {
  switch (nx) {
#define PTF_CASE(n) case n: return PassLaunch<T, n>::row(a, P, nby, batch, st);
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return cudaErrorInvalidValue;
  }
}
// Largest number of lines (columns W or row pairs P) per block for length n.
template <typename T> int max_lines_per_block(int n, bool col) {
  switch (n) {
#define PTF_CASE(v) case v: return max_lines_n<T, v>(col);
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return 1;
  }
}
template <typename T> static int tpl_of(int n, bool col) {
  switch (n) {
#define PTF_CASE(v) case v: return col ? col_tpl<T, v>() : pass_tpl<T, v>();
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return 1;
  }
}
// Default lines per block.  Column pass: FP32 takes 8 columns (64-byte row
// segments, memory bound) when registers allow; FP64 takes 2 (compute bound:
// more, smaller blocks balance 152 SMs better).  Row pass: enough pairs for
// >= 64 threads.  `divisor` must be divisible by the result.
template <typename T> int default_lines_per_block(int n, bool col, int divisor) {
  const int tpl = tpl_of<T>(n, col);
  const int mx = max_lines_per_block<T>(n, col);
  int m;
  if (col) {
    m = sizeof(T) == 4 ? 8 : 2;
    while (m * tpl < 64 && m < 64) m *= 2;
  } else {
    m = 1;
    while (m * tpl < 64 && m < 64) m *= 2;
  }
  while (m > mx) m /= 2;
  while (m > 1 && divisor % m) m /= 2;
  return m < 1 ? 1 : m;
}

template <typename T> int col_ylog_limit(int n) {
  switch (n) {
#define PTF_CASE(v) case v: return col_ylog_max<T, v>();
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: return 0;
  }
}

template <typename T> void col_line_shape(int n, int* tpl, int* rf) {
  switch (n) {
#define PTF_CASE(v) case v: *tpl = col_tpl<T, v>(); *rf = LastRadix<v, -1, ColE<T, v>::value>::value; return;
    PTF_FOR_SIZES(PTF_CASE)
#undef PTF_CASE
    default: *tpl = 1; *rf = 1;
  }
}

template void col_line_shape<float>(int, int*, int*);
template void col_line_shape<double>(int, int*, int*);
template int col_ylog_limit<float>(int);
template int col_ylog_limit<double>(int);
template cudaError_t launch_col<float>(int, const ColArgs<float>&, int, int, int, cudaStream_t, int);
template cudaError_t launch_col<double>(int, const ColArgs<double>&, int, int, int, cudaStream_t, int);
template cudaError_t launch_row<float>(int, const RowArgs<float>&, int, int, int, cudaStream_t);
template cudaError_t launch_row<double>(int, const RowArgs<double>&, int, int, int, cudaStream_t);
template int max_lines_per_block<float>(int, bool);
template int max_lines_per_block<double>(int, bool);
template int default_lines_per_block<float>(int, bool, int);
template int default_lines_per_block<double>(int, bool, int);

}  // namespace ptf
