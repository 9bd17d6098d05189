// FP64 instantiation of the 2D pass kernels.
#include "ptf_kern2d_impl.cuh"
PTF_INSTANTIATE_2D(double)
