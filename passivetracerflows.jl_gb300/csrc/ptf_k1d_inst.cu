// Explicit instantiation of the 1D stage-pass kernels for one precision and
// one length: -DPTF_T=float|double -DPTF_N=16..4096.
#if !defined(PTF_T) || !defined(PTF_N)
#error "compile with -DPTF_T=<float|double> -DPTF_N=<length>"
#endif
#define PTF_K1D_INST 1
#include "ptf_kern1d.cu"
