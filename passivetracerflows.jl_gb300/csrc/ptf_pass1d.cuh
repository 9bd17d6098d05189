// 1D problems (src/traceradvectiondiffusion.jl:143-163 Problem, :695-706 /
// :744-754 calcN!): one kernel per stepper stage.  A block takes P pairs of
// solves; per pair, one inverse complex x-FFT of Z = P0 + i P1 (P_j the
// Hermitian extension of i kr X_j, X the stage input) gives c_x of both
// solves, the product with the flow u (pre-scaled by -1/(2 nx)), one forward
// FFT of n_0 + i n_1 separated into the two half spectra, then the stage
// combination (the same code as the 2D column pass) for both solves.
#pragma once
#include "ptf_passes.cuh"

namespace ptf {

template <typename T> struct Line1DArgs {
  typedef typename cplx_of<T>::type C;
  const C* xin;  // stage input, pitch complex per solve
  C* xout;       // next stage input (ETDRK4 stages 1-3; may alias xin); N for COL_FWD_N
  C *s, *si, *acc;
  const T* u;  // flow on the grid, pre-scaled by -1/(2 nx), shared by the batch
  const T* Ltab;
  const T* coef;
  const T* filt;  // filtered steppers: spectral filter (null: none)
  const C* tw;
  T dkx, dt;
  int pitch, rows;  // rows = solves (even: an odd batch carries one zero solve)
  // FP64 k = 0 mode (FP32 handles): per-solve {s, stage input (ETDRK4: d), acc, -}, coefficients
  double* k0;
  const double* k0c;
  double dt64;
};

// Z[k] = P0[k] + i P1[k] with P_j the Hermitian extension of i kr X_j; the
// imaginary parts at the self-conjugate bins (k = 0, nx/2) are dropped.
template <typename T, typename C>
__device__ __forceinline__ C zsrc_1d(const C* X0, const C* X1, int k, int NX, T dkx) {
  C z;
  const int h = NX / 2;
  if (k == 0) {
    z.x = 0; z.y = 0;
  } else if (k == h) {
    const T kr = (T)h * dkx;
    z.x = -kr * X0[h].y; z.y = -kr * X1[h].y;
  } else if (k < h) {
    const T kr = (T)k * dkx;
    const C a = X0[k], b = X1[k];
    // P0 = (-kr a.y, kr a.x), P1 = (-kr b.y, kr b.x); Z = P0 + i P1
    z.x = -kr * a.y - kr * b.x; z.y = kr * a.x - kr * b.y;
  } else {
    const int kk = NX - k;
    const T kr = (T)kk * dkx;
    const C a = X0[kk], b = X1[kk];
    // P0 = conj(i kr a) = (-kr a.y, -kr a.x), P1 likewise
    z.x = -kr * a.y + kr * b.x; z.y = -kr * a.x - kr * b.y;
  }
  return z;
}

template <typename T, int NX> __host__ __device__ constexpr size_t line1d_smem_bytes(int P) {
  return (size_t)P * line_stride(NX) * sizeof(typename cplx_of<T>::type);
}

template <typename T, int NX, int MODE>
__global__ void __launch_bounds__(256) line1d_kernel(Line1DArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = PassE<T, NX>::value;
  constexpr int TPL = NX / E;
  constexpr int LS = line_stride(NX);
  constexpr int RI0 = FirstRadix<NX, +1, E>::value;
  constexpr int RIL = LastRadix<NX, +1, E>::value;
  constexpr int RFL = LastRadix<NX, -1, E>::value;
  static_assert(RIL == FirstRadix<NX, -1, E>::value, "inverse-last and forward-first radices must match");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int P = blockDim.x / TPL;
  const int pr = threadIdx.x / TPL, t = threadIdx.x % TPL;
  const int y0 = 2 * (blockIdx.x * P + pr);
  const bool valid = y0 < a.rows;  // grids are sized exactly; kept for safety
  const int yy0 = valid ? y0 : 0;
  const int pitch = a.pitch;
  C* line = sm + pr * LS;
  const C* X0 = a.xin + (size_t)yy0 * pitch;
  const C* X1 = X0 + pitch;

  C v[E];
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = zsrc_1d<T, C>(X0, X1, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
  fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const T uu = a.u[reg_pos<NX, RIL, E>(t, i)];
    v[i].x *= uu;
    v[i].y *= uu;
  }
  // FP64 k = 0 mode: N(0) of both solves as compensated FP64 sums of the
  // products (Re: solve y0, Im: solve y1) rather than the FP32 transform's
  // k = 0 bin; they land in the pair's thread t = 0, which handles k = 0.
  double n0sum[2] = {0.0, 0.0};
  if (a.k0 != nullptr && MODE != COL_FWD_N) {  // uniform across the block
    double* part = reinterpret_cast<double*>(line);  // 2 TPL doubles fit in the line
    double s0 = 0, c0 = 0, s1 = 0, c1 = 0;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      double y = (double)v[i].x - c0, u0 = s0 + y;
      c0 = (u0 - s0) - y; s0 = u0;
      y = (double)v[i].y - c1; const double u1 = s1 + y;
      c1 = (u1 - s1) - y; s1 = u1;
    }
    part[2 * t] = s0;
    part[2 * t + 1] = s1;
    __syncthreads();
    if (t == 0) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        double tot = 0, c = 0;
        for (int q = 0; q < TPL; ++q) {
          const double y = part[2 * q + j] - c, u = tot + y;
          c = (u - tot) - y;
          tot = u;
        }
        n0sum[j] = 2.0 * tot;  // the k = 0 bin of the separated spectra is twice the sum
      }
    }
    __syncthreads();
  }
  fft_line<NX, -1, E>(v, t, line, a.tw);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E; ++i) line[smem_pad(reg_pos<NX, RFL, E>(t, i))] = v[i];
  __syncthreads();
  if (!valid) return;
  for (int k = t; k <= NX / 2; k += TPL) {
    const C wk = line[smem_pad(k)];
    const C wn = line[smem_pad((NX - k) & (NX - 1))];
    C o[2];
    // solve y0: W[k] + conj(W[n-k]) ; solve y1: -i (W[k] - conj(W[n-k]))
    o[0].x = wk.x + wn.x; o[0].y = wk.y - wn.y;
    o[1].x = wk.y + wn.y; o[1].y = wn.x - wk.x;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const size_t r = (size_t)(y0 + j) * pitch;
      C x;
      if (MODE == COL_FWD_N) {
        a.xout[r + k] = o[j];
        continue;
      }
      x = stage_combine<T, MODE>(o[j], k, a.s + r, a.si + r, a.acc + r, a.coef, (size_t)pitch, a.dt, true,
                                 [&]() { return a.Ltab[k]; }, a.filt);
      if (a.k0 != nullptr && k == 0) {
        double* q = a.k0 + (size_t)(y0 + j) * 4;
        const double xd = k0_combine<MODE>(q, a.k0c, a.dt64, n0sum[j]);
        x.x = (T)xd; x.y = 0;
        if (MODE == COL_RK4_4 || MODE == COL_ETD_4) a.s[r] = x;
        else if (MODE == COL_RK4_1 || MODE == COL_RK4_2 || MODE == COL_RK4_3) a.si[r] = x;
      }
      // ETDRK4 stage inputs a, b, c go to xout (SI holds d = E2 a - zeta N(s))
      if (MODE == COL_ETD_1 || MODE == COL_ETD_2 || MODE == COL_ETD_3) a.xout[r + k] = x;
    }
  }
}

}  // namespace ptf
