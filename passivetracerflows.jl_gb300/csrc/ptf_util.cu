// Element conversion kernels between the FP64 user layout and the
// compute-precision internal layout.
#include "ptf_internal.h"
#include "../../include/ptf.h"

namespace ptf {

template <typename T>
__global__ void real_in_kernel(const double* __restrict__ src, T* __restrict__ dst, long long n, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (T)(src[i] * scale);
}
template <typename T>
__global__ void real_out_kernel(const T* __restrict__ src, double* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}
// User row r (of rows_per_solve per solve), bin k <-> element spec_map(m, .)
// of the solve's plane (rows_per_solve * pitch elements).  Bins k >= nkr of
// the pitch are written as zero.
// lo non-null: dst and lo receive the value split into its rounding and the
// remainder (x = hi + lo exactly for FP32 parts of an FP64 value near hi).
template <typename T>
__global__ void spec_in_kernel(const double2* __restrict__ src, typename cplx_of<T>::type* __restrict__ dst, int nkr,
                               long long rows, long long rows_per_solve, SpecMap m,
                               typename cplx_of<T>::type* __restrict__ lo) {
  const long long n = rows * m.pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long rg = i / m.pitch;
    const int k = (int)(i - rg * m.pitch);
    const long long b = rg / rows_per_solve, r = rg - b * rows_per_solve;
    typename cplx_of<T>::type z, zl;
    zl.x = 0; zl.y = 0;
    if (k < nkr) {
      const double2 s = src[rg * nkr + k];
      z.x = (T)s.x; z.y = (T)s.y;
      zl.x = (T)(s.x - (double)z.x); zl.y = (T)(s.y - (double)z.y);
    } else {
      z.x = 0; z.y = 0;
    }
    const long long at = b * rows_per_solve * m.pitch + spec_map(m, r, k);
    dst[at] = z;
    if (lo) lo[at] = zl;
  }
}
template <typename T>
__global__ void spec_out_kernel(const typename cplx_of<T>::type* __restrict__ src, double2* __restrict__ dst, int nkr,
                                long long rows, long long rows_per_solve, SpecMap m,
                                const typename cplx_of<T>::type* __restrict__ lo) {
  const long long n = rows * nkr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long rg = i / nkr;
    const int k = (int)(i - rg * nkr);
    const long long b = rg / rows_per_solve, r = rg - b * rows_per_solve;
    const long long at = b * rows_per_solve * m.pitch + spec_map(m, r, k);
    const typename cplx_of<T>::type z = src[at];
    double2 d = make_double2((double)z.x, (double)z.y);
    if (lo) { d.x += (double)lo[at].x; d.y += (double)lo[at].y; }
    dst[i] = d;
  }
}

static inline int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

template <typename T> cudaError_t launch_real_in(const double* src, T* dst, long long n, double scale, cudaStream_t st) {
  real_in_kernel<T><<<grid_for(n), 256, 0, st>>>(src, dst, n, scale);
  return cudaGetLastError();
}
template <typename T> cudaError_t launch_real_out(const T* src, double* dst, long long n, cudaStream_t st) {
  real_out_kernel<T><<<grid_for(n), 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_spec_in(const double2* src, typename cplx_of<T>::type* dst, int nkr, int pitch, long long rows,
                           cudaStream_t st, const SpecMap* map, long long rows_per_solve,
                           typename cplx_of<T>::type* lo) {
  SpecMap m;
  if (map) m = *map;
  m.pitch = pitch;
  if (!map || rows_per_solve <= 0) rows_per_solve = rows;
  spec_in_kernel<T><<<grid_for(rows * pitch), 256, 0, st>>>(src, dst, nkr, rows, rows_per_solve, m, lo);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_spec_out(const typename cplx_of<T>::type* src, double2* dst, int nkr, int pitch, long long rows,
                            cudaStream_t st, const SpecMap* map, long long rows_per_solve,
                            const typename cplx_of<T>::type* lo) {
  SpecMap m;
  if (map) m = *map;
  m.pitch = pitch;
  if (!map || rows_per_solve <= 0) rows_per_solve = rows;
  spec_out_kernel<T><<<grid_for(rows * nkr), 256, 0, st>>>(src, dst, nkr, rows, rows_per_solve, m, lo);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 k = 0 mode helpers.  Per-solve sums run as kSumBlocks blocks per solve
// writing FP64 partials (plain FP64 accumulation per thread over a short
// strided run, then a block tree), then one warp per solve adding the
// partials with a compensated (Kahan) sum.
// ---------------------------------------------------------------------------
constexpr int kSumBlocks = 64;

__device__ __forceinline__ void kahan_add(double& s, double& c, double x) {
  const double y = x - c;
  const double u = s + y;
  c = (u - s) - y;
  s = u;
}

template <typename Tin>
__global__ void __launch_bounds__(256) solve_partials_kernel(const Tin* __restrict__ x, long long n, double* part) {
  const long long b = blockIdx.y;
  const long long chunk = (n + kSumBlocks - 1) / kSumBlocks;
  const long long lo = blockIdx.x * chunk, hi = lo + chunk < n ? lo + chunk : n;
  const Tin* xs = x + b * n;
  // four independent FP64 accumulators per thread (each covers a few dozen
  // values: error ~ count * eps64), then compensated sums across threads
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  const long long step = blockDim.x;
  long long i = lo + threadIdx.x;
  for (; i + 3 * step < hi; i += 4 * step) {
    a0 += (double)xs[i];
    a1 += (double)xs[i + step];
    a2 += (double)xs[i + 2 * step];
    a3 += (double)xs[i + 3 * step];
  }
  for (; i < hi; i += step) a0 += (double)xs[i];
  double s = (a0 + a1) + (a2 + a3);
  for (int off = 16; off > 0; off /= 2) s += __shfl_xor_sync(0xffffffffu, s, off);
  __shared__ double ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0, tc = 0;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) kahan_add(t, tc, ws[k]);
    part[b * kSumBlocks + blockIdx.x] = t;
  }
}

__global__ void solve_sums_finish_kernel(const double* __restrict__ part, double* out, int out_stride) {
  const int b = blockIdx.x;
  double s = 0, c = 0;
  for (int k = threadIdx.x; k < kSumBlocks; k += 32) kahan_add(s, c, part[b * kSumBlocks + k]);
  for (int off = 16; off > 0; off /= 2) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (threadIdx.x == 0) out[(long long)b * out_stride] = s;
}

template <typename Tin>
cudaError_t launch_solve_sums(const Tin* x, long long n, int batch, double* partials, double* out, int out_stride,
                              cudaStream_t st) {
  solve_partials_kernel<Tin><<<dim3(kSumBlocks, batch), 256, 0, st>>>(x, n, partials);
  solve_sums_finish_kernel<<<batch, 32, 0, st>>>(partials, out, out_stride);
  return cudaGetLastError();
}

// k0[4b] = Re src[b * per_solve] (the (0,0) element of a solve's spectrum)
__global__ void k0_from_spec_kernel(const double2* __restrict__ src, long long per_solve, int batch, double* k0) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) k0[4 * b] = src[(long long)b * per_solve].x;
}
// dst[b * per_solve] = (k0[4b], 0)
__global__ void k0_to_spec_kernel(double2* dst, long long per_solve, int batch, const double* __restrict__ k0) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) dst[(long long)b * per_solve] = make_double2(k0[4 * b], 0.0);
}
cudaError_t launch_k0_from_spec(const double2* src, long long per_solve, int batch, double* k0, cudaStream_t st) {
  k0_from_spec_kernel<<<(batch + 127) / 128, 128, 0, st>>>(src, per_solve, batch, k0);
  return cudaGetLastError();
}
cudaError_t launch_k0_to_spec(double2* dst, long long per_solve, int batch, const double* k0, cudaStream_t st) {
  k0_to_spec_kernel<<<(batch + 127) / 128, 128, 0, st>>>(dst, per_solve, batch, k0);
  return cudaGetLastError();
}

// dst = src + (k0[4b] - sums[b]) / n for solve b: the field's sum becomes the
// FP64 (0,0) mode.
template <typename T>
__global__ void real_out_shift_kernel(const T* __restrict__ src, double* __restrict__ dst, long long n,
                                      const double* __restrict__ k0, const double* __restrict__ sums) {
  const long long b = blockIdx.y;  // solve
  const double shift = (k0[4 * b] - sums[b]) / (double)n;
  const T* s = src + b * n;
  double* d = dst + b * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[i] = (double)s[i] + shift;
}
template <typename T>
cudaError_t launch_real_out_shift(const T* src, double* dst, long long n, int batch, const double* k0,
                                  const double* sums, cudaStream_t st) {
  const int gx = (grid_for(n * batch) + batch - 1) / batch;
  real_out_shift_kernel<T><<<dim3(gx < 1 ? 1 : gx, batch), 256, 0, st>>>(src, dst, n, k0, sums);
  return cudaGetLastError();
}

// dst[b n + i] = (src[b n + i] + (U ? U[b] : 0)) * scale: per-solve flows
template <typename T>
__global__ void layers_in_kernel(const double* __restrict__ src, T* __restrict__ dst, long long n,
                                 const double* __restrict__ U, double scale) {
  const long long b = blockIdx.y;
  const double off = U ? U[b] : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[b * n + i] = (T)((src[b * n + i] + off) * scale);
}
template <typename T>
cudaError_t launch_layers_in(const double* src, T* dst, long long n, int batch, const double* U, double scale,
                             cudaStream_t st) {
  const int gx = (grid_for(n * batch) + batch - 1) / batch;
  layers_in_kernel<T><<<dim3(gx < 1 ? 1 : gx, batch), 256, 0, st>>>(src, dst, n, U, scale);
  return cudaGetLastError();
}
// Analytic flows on the grid x_i = -L/2 + i L/n, pre-scaled like the array
// flows (scale = -1/(2 points)); FP64 evaluation, stored in T.
// kind 1 (cellular, 2D): u = U ky cos(kx x + phi) sin(ky y), v = -U kx sin(kx x + phi) cos(ky y),
//   phi = eps sin(omega t); kind 2 (ABC, 3D).
template <typename T>
__global__ void flow_analytic_kernel(T* __restrict__ u, T* __restrict__ v, T* __restrict__ w, int nx, int ny, int nz,
                                     double Lx, double Ly, double Lz, ptf_flow_desc d, double t, double scale) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nx);
    const long long r = i / nx;
    const int iy = (int)(r % ny), iz = (int)(r / ny);
    const double x = -Lx / 2 + Lx / nx * ix, y = -Ly / 2 + Ly / ny * iy, z = -Lz / 2 + Lz / nz * iz;
    if (d.kind == PTF_FLOW_CELLULAR) {
      const double kx = d.Kx * 2 * M_PI / Lx, ky = d.Ky * 2 * M_PI / Ly;
      const double arg = kx * x + d.eps * sin(d.omega * t);
      u[i] = (T)(scale * d.U * ky * cos(arg) * sin(ky * y));
      v[i] = (T)(scale * -d.U * kx * sin(arg) * cos(ky * y));
    } else {
      u[i] = (T)(scale * (d.A * sin(z) + d.C * cos(y)));
      v[i] = (T)(scale * (d.B * sin(x) + d.A * cos(z)));
      w[i] = (T)(scale * (d.C * sin(y) + d.B * cos(x)));
    }
  }
}
template <typename T>
cudaError_t launch_flow_analytic(T* u, T* v, T* w, int nx, int ny, int nz, double Lx, double Ly, double Lz,
                                 const ptf_flow_desc& d, double t, double scale, cudaStream_t st) {
  flow_analytic_kernel<T><<<grid_for((long long)nx * ny * nz), 256, 0, st>>>(u, v, w, nx, ny, nz, Lx, Ly, Lz, d, t,
                                                                              scale);
  return cudaGetLastError();
}
template cudaError_t launch_flow_analytic<float>(float*, float*, float*, int, int, int, double, double, double,
                                                 const ptf_flow_desc&, double, double, cudaStream_t);
template cudaError_t launch_flow_analytic<double>(double*, double*, double*, int, int, int, double, double, double,
                                                  const ptf_flow_desc&, double, double, cudaStream_t);

template cudaError_t launch_layers_in<float>(const double*, float*, long long, int, const double*, double, cudaStream_t);
template cudaError_t launch_layers_in<double>(const double*, double*, long long, int, const double*, double, cudaStream_t);

template cudaError_t launch_solve_sums<double>(const double*, long long, int, double*, double*, int, cudaStream_t);
template cudaError_t launch_solve_sums<float>(const float*, long long, int, double*, double*, int, cudaStream_t);
template cudaError_t launch_real_out_shift<float>(const float*, double*, long long, int, const double*, const double*,
                                                  cudaStream_t);
template cudaError_t launch_real_out_shift<double>(const double*, double*, long long, int, const double*, const double*,
                                                   cudaStream_t);

template cudaError_t launch_real_in<double>(const double*, double*, long long, double, cudaStream_t);
template cudaError_t launch_real_in<float>(const double*, float*, long long, double, cudaStream_t);
template cudaError_t launch_real_out<double>(const double*, double*, long long, cudaStream_t);
template cudaError_t launch_real_out<float>(const float*, double*, long long, cudaStream_t);
template cudaError_t launch_spec_in<double>(const double2*, double2*, int, int, long long, cudaStream_t, const SpecMap*,
                                            long long, double2*);
template cudaError_t launch_spec_in<float>(const double2*, float2*, int, int, long long, cudaStream_t, const SpecMap*,
                                           long long, float2*);
template cudaError_t launch_spec_out<double>(const double2*, double2*, int, int, long long, cudaStream_t, const SpecMap*,
                                             long long, const double2*);
template cudaError_t launch_spec_out<float>(const float2*, double2*, int, int, long long, cudaStream_t, const SpecMap*,
                                            long long, const float2*);

}  // namespace ptf
