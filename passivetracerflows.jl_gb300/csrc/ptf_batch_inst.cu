// Explicit instantiation of the batched stage kernels for one precision and
// one RK4 stage (the per-item row and column launches and the persistent
// form): -DPTF_T=float|double -DPTF_MODE=<RK4 stage ColMode 2..5>.
#include "ptf_batch_kern.cuh"

#if !defined(PTF_T) || !defined(PTF_MODE)
#error "compile with -DPTF_T=<float|double> -DPTF_MODE=<2..5>"
#endif

namespace ptf {
template cudaError_t launch_batch_stage<PTF_T, PTF_MODE>(const BatchPlan<PTF_T>*, unsigned int*, int*, PTF_T, int,
                                                         size_t, cudaStream_t);
template cudaError_t setup_batch_stage<PTF_T, PTF_MODE>(size_t, int*);
template cudaError_t launch_batch_cols<PTF_T, PTF_MODE>(const BatchPlan<PTF_T>*, int, size_t, cudaStream_t);
template cudaError_t setup_batch_items<PTF_T, PTF_MODE>(size_t);
#if PTF_MODE == 2
template cudaError_t launch_batch_rows<PTF_T>(const BatchPlan<PTF_T>*, PTF_T, int, size_t, cudaStream_t);
#endif
}  // namespace ptf
