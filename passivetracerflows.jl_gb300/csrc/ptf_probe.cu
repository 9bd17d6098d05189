// Arithmetic-throughput probe of the current device: the FP64 (and FP32) FMA
// rate that bounds the FP64 path, measured on the GPU the library runs on.
//
// Every thread runs 8 independent FMA chains x <- x * a + b for `iters`
// iterations (a, b kernel arguments, so nothing folds at compile time); the
// chains converge to 0.1 and their sum is stored (to a file-scope device
// variable) only when it equals an impossible value, so the work is kept and
// nothing is written.  One launch of 4 blocks of 256 threads per
// SM; the loop bound is a kernel argument and every thread runs it to the
// end (no waits, no data dependence between threads).
#include <cuda_runtime.h>

#include <string>

#include "../../include/ptf.h"
#include "ptf_internal.h"

namespace {

__device__ double g_probe_sink[2];  // written only if a chain sum were impossible

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T a, T b, int iters) {
  T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == (T)-1.2345e30) g_probe_sink[sizeof(T) == 8 ? 0 : 1] = (double)s;
}

template <typename T> int probe(double* flops_per_s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    ptf::set_global_error(std::string("fma probe: ") + cudaGetErrorString(e));
    return PTF_ERR_CUDA;
  }
  const int blocks = 4 * sms, threads = 256;
  // FP64: about 2^27 DFMA per SM at a few DFMA per SM per clock, tens of ms
  const int iters = sizeof(T) == 8 ? 256 : 8192;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // rep 0 warms up
    e = cudaEventRecord(e0, st);
    fma_probe_kernel<T><<<blocks, threads, 0, st>>>((T)0.999999, (T)1e-7, iters);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && ms < best) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess) {
    ptf::set_global_error(std::string("fma probe: ") + cudaGetErrorString(e));
    return PTF_ERR_CUDA;
  }
  const double fmas = (double)blocks * threads * (double)iters * 64.0;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  return PTF_OK;
}

}  // namespace

extern "C" int ptf_measure_fma_peak(int32_t precision, double* flops_per_s) {
  if (!flops_per_s) {
    ptf::set_global_error("ptf_measure_fma_peak: null output");
    return PTF_ERR_ARG;
  }
  if (precision == PTF_FP64) return probe<double>(flops_per_s);
  if (precision == PTF_FP32) return probe<float>(flops_per_s);
  ptf::set_global_error("ptf_measure_fma_peak: precision must be PTF_FP64 or PTF_FP32");
  return PTF_ERR_ARG;
}
