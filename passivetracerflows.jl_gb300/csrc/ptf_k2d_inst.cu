// Explicit instantiation of the 2D pass kernels for one precision and one
// length, selected at compile time: -DPTF_T=float|double -DPTF_N=16..4096.
#include "ptf_kern2d_impl.cuh"

#if !defined(PTF_T) || !defined(PTF_N)
#error "compile with -DPTF_T=<float|double> -DPTF_N=<length>"
#endif

namespace ptf {
template struct PassLaunch<PTF_T, PTF_N>;
template int max_lines_n<PTF_T, PTF_N>(bool col);
}  // namespace ptf
