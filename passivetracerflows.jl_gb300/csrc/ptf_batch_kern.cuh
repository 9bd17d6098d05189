// Stage kernels of the batched form (per-item row and column launches, and
// the persistent per-stage kernel) and their work plan.  See
// ptf_batch.cu for the design; the kernels are instantiated per (precision,
// stage) in ptf_batch_inst.cu so they compile in parallel.
#pragma once
#include <algorithm>
#include "ptf_internal.h"

namespace ptf {

constexpr int kBatchThreads = 256;
constexpr int kMaxBuckets = 32;
// Slot fields use the single-handle layouts: rows interleaved in fours
// (every bucket size is >= 64) and the state in the column pass's register
// order.
constexpr int kBatchYlog = 2;

template <typename T> struct BucketPlan {
  ColArgs<T> col;
  RowArgs<T> row;
  int n;
  int row_items, col_items;
  int row_begin, col_begin;  // first global item of the bucket's row / column tiles
};
template <typename T> struct BatchPlan {
  int nb, row_total, total;
  // bounded wait of the persistent kernel: sleeps of about 128 ns before a
  // column item gives up (0: kSpinLimit), and extra row items a column item
  // waits for (0; > 0 only through the test hook that makes the wait run out)
  unsigned long long spin_limit;
  unsigned int wait_extra;
  BucketPlan<T> b[kMaxBuckets];
};

#define PTF_BATCH_SIZES(X) X(64) X(128) X(256) X(512) X(1024)

template <typename T> struct BatchBounds { static constexpr int blocks = 1; };
template <> struct BatchBounds<float> { static constexpr int blocks = 2; };

template <typename T, int N> __host__ __device__ constexpr size_t batch_smem_n() {
  // W = 256 / col_tpl columns, P = 256 / pass_tpl row pairs per block
  return col_smem_bytes<T, N>(kBatchThreads / col_tpl<T, N>()) > row_smem_bytes<T, N>(kBatchThreads / pass_tpl<T, N>(), 1)
             ? col_smem_bytes<T, N>(kBatchThreads / col_tpl<T, N>())
             : row_smem_bytes<T, N>(kBatchThreads / pass_tpl<T, N>(), 1);
}
template <typename T> size_t batch_smem_bytes() {
  size_t m = 0;
#define PTF_MAXS(n) m = std::max(m, batch_smem_n<T, n>());
  PTF_BATCH_SIZES(PTF_MAXS)
#undef PTF_MAXS
  return m;
}

constexpr unsigned long long kSpinLimit = 1ull << 24;  // x 128 ns sleeps: about 2 s

// The bodies of one work item as real calls: the item loop of the persistent
// kernel then holds few values across an item, and each body gets the
// registers it needs instead of competing with hoisted loop state.
template <typename T, int N>
__device__ __noinline__ void batch_row_item(const RowArgs<T>* ra, T stage_c, int local, unsigned char* smem) {
  RowArgs<T> a = *ra;
  a.stage_c = stage_c;
  row_body<T, N, true, true>(a, local, 0, smem);
}
template <typename T, int N, int MODE>
__device__ __noinline__ void batch_col_item(const ColArgs<T>* ca, int local, unsigned char* smem) {
  // buckets hold square grids: the row pitch is square_pitch<N>()
  col_body<T, N, MODE, true, square_pitch<N>()>(*ca, local, 0, smem);
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kBatchThreads, BatchBounds<T>::blocks)
batch_stage_kernel(const BatchPlan<T>* __restrict__ plan, unsigned int* ctr, int* err, T stage_c) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item, s_ok;
  const int nb = plan->nb, row_total = plan->row_total, total = plan->total;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(&ctr[0], 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= total) return;  // uniform
    if (item < row_total) {
      int b = 0;
      while (b + 1 < nb && item >= plan->b[b + 1].row_begin) ++b;
      const int local = item - plan->b[b].row_begin;
      switch (plan->b[b].n) {
#define PTF_CASE(n) case n: batch_row_item<T, n>(&plan->b[b].row, stage_c, local, smem); break;
        PTF_BATCH_SIZES(PTF_CASE)
#undef PTF_CASE
        default: break;
      }
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&ctr[1 + b], 1u);
    } else {
      int b = 0;
      while (b + 1 < nb && item >= plan->b[b + 1].col_begin) ++b;
      if (threadIdx.x == 0) {
        const unsigned need = (unsigned)plan->b[b].row_items + plan->wait_extra;
        const unsigned long long limit = plan->spin_limit ? plan->spin_limit : kSpinLimit;
        unsigned long long spins = 0;
        int ok = 1;
        while (*((volatile unsigned int*)&ctr[1 + b]) < need) {
          if (++spins > limit) { atomicExch(err, 1); ok = 0; break; }
          __nanosleep(128);
        }
        __threadfence();
        s_ok = ok;
      }
      __syncthreads();
      if (s_ok) {
        const int local = item - plan->b[b].col_begin;
        switch (plan->b[b].n) {
#define PTF_CASE(n) case n: batch_col_item<T, n, MODE>(&plan->b[b].col, local, smem); break;
          PTF_BATCH_SIZES(PTF_CASE)
#undef PTF_CASE
          default: break;
        }
      }
    }
    __syncthreads();  // s_item / s_ok are rewritten by the next item
  }
}

// ---------------------------------------------------------------------------
// One block per work item instead: a row launch over every bucket's row
// items, then a column launch over the column items; the hardware schedules
// the blocks and the kernel boundary is the dependency.  Same items, same
// bodies as the persistent kernel.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kBatchThreads, BatchBounds<T>::blocks)
batch_row_kernel(const BatchPlan<T>* __restrict__ plan, T stage_c) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int item = blockIdx.x, nb = plan->nb;
  int b = 0;
  while (b + 1 < nb && item >= plan->b[b + 1].row_begin) ++b;
  RowArgs<T> ra = plan->b[b].row;
  ra.stage_c = stage_c;
  const int local = item - plan->b[b].row_begin;
  switch (plan->b[b].n) {
#define PTF_CASE(n) case n: row_body<T, n, true, true>(ra, local, 0, smem); break;
    PTF_BATCH_SIZES(PTF_CASE)
#undef PTF_CASE
    default: break;
  }
}
template <typename T, int MODE>
__global__ void __launch_bounds__(kBatchThreads, BatchBounds<T>::blocks)
batch_col_kernel(const BatchPlan<T>* __restrict__ plan) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int item = plan->row_total + blockIdx.x, nb = plan->nb;
  int b = 0;
  while (b + 1 < nb && item >= plan->b[b + 1].col_begin) ++b;
  const int local = item - plan->b[b].col_begin;
  // each size's body as a real call (batch_col_item): inlined side by side
  // in one kernel they shared one register allocation and spilled 370-540 B
  // per thread in the RK4 stages 2-4; as calls, 0-28 B
  switch (plan->b[b].n) {
#define PTF_CASE(n) case n: batch_col_item<T, n, MODE>(&plan->b[b].col, local, smem); break;
    PTF_BATCH_SIZES(PTF_CASE)
#undef PTF_CASE
    default: break;
  }
}
template <typename T>
cudaError_t launch_batch_rows(const BatchPlan<T>* plan, T stage_c, int nitems, size_t smem, cudaStream_t st) {
  batch_row_kernel<T><<<nitems, kBatchThreads, smem, st>>>(plan, stage_c);
  return cudaGetLastError();
}
template <typename T, int MODE>
cudaError_t launch_batch_cols(const BatchPlan<T>* plan, int nitems, size_t smem, cudaStream_t st) {
  batch_col_kernel<T, MODE><<<nitems, kBatchThreads, smem, st>>>(plan);
  return cudaGetLastError();
}
template <typename T, int MODE> cudaError_t setup_batch_items(size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(batch_col_kernel<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && MODE == COL_RK4_1)
    e = cudaFuncSetAttribute(batch_row_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e;
}

// Launcher and set-up of one (precision, stage) kernel; instantiated in
// ptf_batch_inst.cu objects.
template <typename T, int MODE>
cudaError_t launch_batch_stage(const BatchPlan<T>* plan, unsigned int* ctr, int* err, T stage_c, int grid, size_t smem,
                               cudaStream_t st) {
  batch_stage_kernel<T, MODE><<<grid, kBatchThreads, smem, st>>>(plan, ctr, err, stage_c);
  return cudaGetLastError();
}
template <typename T, int MODE> cudaError_t setup_batch_stage(size_t smem, int* occ) {
  cudaError_t e = cudaFuncSetAttribute(batch_stage_kernel<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, batch_stage_kernel<T, MODE>, kBatchThreads, smem);
}
template <typename T> __global__ void batch_clock_kernel(SlotParams<T>* slots, int n);

}  // namespace ptf
