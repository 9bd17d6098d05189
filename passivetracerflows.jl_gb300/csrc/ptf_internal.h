// Internal declarations shared by the translation units of libptf.so.
#pragma once
#include <cuda_runtime.h>
#include "ptf_passes.cuh"
#include "ptf_pass1d.cuh"
#include "../../include/ptf.h"

#include <string>

namespace ptf {

// Message returned by ptf_last_error(NULL) (calls without a handle).
void set_global_error(const std::string& msg);

// Device bytes a batch holds besides its buckets (slot table, plan, staging),
// and the bytes one slot of an n x n solve needs (ptf_batch.cu): the request
// server refuses a request that could not fit even in an empty batch.
int64_t batch_fixed_bytes(const ptf_batch* b);
int64_t batch_slot_bytes(const ptf_batch* b, int n);

// Pass launchers (ptf_kern2d.cu dispatching to ptf_k2d_inst.cu objects).
// Column pass over transform length n: grid (nbx, nby), W columns per block.
// carve: preferred shared-memory carve-out in percent (-1: the CUDA driver's choice).
template <typename T>
cudaError_t launch_col(int n, const ColArgs<T>& a, int W, int nbx, int nby, cudaStream_t st, int carve = -1);
// Row pass over x length nx: grid (nbx, batch), P row pairs per block.
template <typename T> cudaError_t launch_row(int nx, const RowArgs<T>& a, int P, int nbx, int batch, cudaStream_t st);
// Largest W / P that a launch may use for a given length (shared-memory bound).
template <typename T> int max_lines_per_block(int n, bool col);
// Default W (col) or P (row) for length n; `divisor` must be divisible by it.
template <typename T> int default_lines_per_block(int n, bool col, int divisor);
// Largest spectral layout (ylog of spec_index) a column pass of length n takes.
template <typename T> int col_ylog_limit(int n);
// Threads per line and last forward radix of a column pass of length n
// (the register order of SpecMap).
template <typename T> void col_line_shape(int n, int* tpl, int* rf);

// 1D stage passes (ptf_kern1d.cu): nblk blocks of P solve pairs; mode is a
// stepper stage (COL_RK4_*, COL_ETD_*) or COL_FWD_N (N into xout).
template <typename T>
cudaError_t launch_line1d(int nx, int mode, const Line1DArgs<T>& a, int P, int nblk, cudaStream_t st);
template <typename T> int line1d_tpl(int nx);  // threads per solve pair

// Element conversions (ptf_util.cu).
template <typename T> cudaError_t launch_real_in(const double* src, T* dst, long long n, double scale, cudaStream_t st);
template <typename T> cudaError_t launch_real_out(const T* src, double* dst, long long n, cudaStream_t st);
// user spectral layout (nkr complex per row) <-> pitched internal layout:
// the plain [rows][pitch] layout without a map, else spec_map(*map, r, k)
// within each solve of rows_per_solve rows
// (lo: the low part of a compensated state, written as the FP64 value's
// remainder after rounding / added back; null: none)
template <typename T>
cudaError_t launch_spec_in(const double2* src, typename cplx_of<T>::type* dst, int nkr, int pitch, long long rows,
                           cudaStream_t st, const SpecMap* map = nullptr, long long rows_per_solve = 0,
                           typename cplx_of<T>::type* lo = nullptr);
template <typename T>
cudaError_t launch_spec_out(const typename cplx_of<T>::type* src, double2* dst, int nkr, int pitch, long long rows,
                            cudaStream_t st, const SpecMap* map = nullptr, long long rows_per_solve = 0,
                            const typename cplx_of<T>::type* lo = nullptr);

// FP64 k = 0 mode (ptf_util.cu).  Per-solve sums of x (n values per solve):
// out[b * out_stride]; partials holds 64 doubles per solve.
template <typename Tin>
cudaError_t launch_solve_sums(const Tin* x, long long n, int batch, double* partials, double* out, int out_stride,
                              cudaStream_t st);
// k0[4b] = Re src[b * per_solve]; dst[b * per_solve] = (k0[4b], 0)
cudaError_t launch_k0_from_spec(const double2* src, long long per_solve, int batch, double* k0, cudaStream_t st);
cudaError_t launch_k0_to_spec(double2* dst, long long per_solve, int batch, const double* k0, cudaStream_t st);
// analytic flows (ptf_set_flow_analytic) evaluated at time t, pre-scaled
template <typename T>
cudaError_t launch_flow_analytic(T* u, T* v, T* w, int nx, int ny, int nz, double Lx, double Ly, double Lz,
                                 const ptf_flow_desc& d, double t, double scale, cudaStream_t st);
// per-solve flows: dst[b n + i] = (src[b n + i] + U[b]) * scale (U may be null)
template <typename T>
cudaError_t launch_layers_in(const double* src, T* dst, long long n, int batch, const double* U, double scale,
                             cudaStream_t st);
// dst = src + (k0[4b] - sums[b]) / n per solve b
template <typename T>
cudaError_t launch_real_out_shift(const T* src, double* dst, long long n, int batch, const double* k0,
                                  const double* sums, cudaStream_t st);

}  // namespace ptf
