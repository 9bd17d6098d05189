// 2D pass kernels of the tracer advection-diffusion right-hand side.
//
// Spectral arrays are [ny][pitch] complex with kr fastest (the layout of
// the reference's (nkr, nl) column-major arrays, padded to `pitch`);
// physical arrays are [ny][nx] real, x fastest.  One RHS evaluation
// (calcN!, src/traceradvectiondiffusion.jl:756-769) is split into
//
//   column pass (y): forward y-FFT of the previous row-pass output, the
//       time-stepper stage combination with the linear operator, then the
//       inverse y-FFTs of the next stage input s and of i*l*s -> A, B
//   row pass (x):    per pair of rows, inverse x-FFT of Z = i(kr A + B)
//       (Hermitian-extended; Re z = c_x, Im z = c_y), the product
//       n = -(u c_x + v c_y), and one forward x-FFT of n_y0 + i n_y1,
//       separated into the two rows' half spectra -> Nx
//
// so one RK4/ETDRK4 stage is two kernels.  The flow passed to the row pass
// is pre-scaled by -1/(2 nx ny): that folds the inverse normalisation, the
// minus sign and the 1/2 of the two-for-one separation into the product.
#pragma once
#include "ptf_fft.cuh"

namespace ptf {

enum ColMode : int {
  COL_PROLOGUE = 0,   // s -> A, B
  COL_FWD_STORE = 1,  // s = Fy(Nx) ; then A, B of s
  COL_RK4_1 = 2, COL_RK4_2 = 3, COL_RK4_3 = 4, COL_RK4_4 = 5,
  COL_ETD_1 = 6, COL_ETD_2 = 7, COL_ETD_3 = 8, COL_ETD_4 = 9,
  COL_FWD_N = 10,     // nout = Fy(Nx), nothing else (calcN)
};
enum RowMode : int { ROW_RHS = 0, ROW_C2R = 1, ROW_R2C = 2 };

template <typename T> struct ColArgs {
  typedef typename cplx_of<T>::type C;
  const C* nxin;   // row-pass output (forward input)
  C* s;            // state (sol)
  C* si;           // RK4: current stage input; ETDRK4: sol1 ("a")
  C* acc;          // accumulator of the update
  C* n1;           // ETDRK4: N(sol)
  C* A;            // Fy^-1(s_next)
  C* B;            // Fy^-1(i l s_next)
  C* nout;         // COL_FWD_N output
  const C* tw;     // NY-point twiddles
  const T* Ltab;   // linear operator [ny][pitch]
  const T* coef;   // ETDRK4 tables E, E2, zeta, alpha, beta, gamma, each ny*pitch
  T dt, dky;
  int pitch, mode, do_inverse;
  long long bstride;    // complex elements between solves of a batch
  int tab_per_solve;    // 1: each solve of the batch has its own L / ETDRK4 tables
};

template <typename T> struct RowArgs {
  typedef typename cplx_of<T>::type C;
  const C* A;
  const C* B;
  C* out;          // ROW_RHS / ROW_R2C: half spectra [ny][pitch]
  const T* u;      // ROW_RHS: scaled flow [ny][nx]
  const T* v;
  const T* cin;    // ROW_R2C: physical input [ny][nx]
  T* cout;         // ROW_C2R: physical output
  const C* tw;     // NX-point twiddles
  T dkx, scale;    // scale: C2R normalisation / R2C 1/2
  int ny, pitch, mode;
  long long bstride, pstride, fstride;
};

template <typename T, int NY>
__device__ __forceinline__ T lval(int p, T dky) { return (T)(p < NY / 2 ? p : p - NY) * dky; }

// ---------------------------------------------------------------------------
// Column pass.  blockDim.x = W * (NY/16); w = tid % W selects the column
// (kr = blockIdx.x*W + w), t = tid / W the thread within the column's line.
// ---------------------------------------------------------------------------
template <typename T, int NY>
__global__ void col_pass_kernel(ColArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = FFT_E;
  constexpr int LS = line_stride(NY);
  constexpr int RF = LastRadix<NY, -1>::value;   // forward output pattern
  constexpr int RI = FirstRadix<NY, +1>::value;  // inverse input pattern (== RF)
  constexpr int RO = LastRadix<NY, +1>::value;   // inverse output pattern
  static_assert(RF == RI, "forward-last and inverse-first radices must match");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int W = blockDim.x / (NY / E);
  const int w = threadIdx.x % W, t = threadIdx.x / W;
  const int kr = blockIdx.x * W + w;
  const long long boff = (long long)blockIdx.y * a.bstride;
  const long long plane = (long long)NY * a.pitch;
  const long long toff = a.tab_per_solve ? (long long)blockIdx.y * plane : 0;
  const int pitch = a.pitch;
  C* line = sm + w * LS;
  const int mode = a.mode;

  C v[E];
  if (mode != COL_PROLOGUE) {
    constexpr int R0 = FirstRadix<NY, -1>::value;
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = a.nxin[boff + (long long)reg_pos<NY, R0>(t, i) * pitch + kr];
    fft_line<NY, -1>(v, t, line, a.tw);
  }

  // Stage combination at the positions p = reg_pos<NY, RF>(t, i).
  const T dt = a.dt;
  C sn[E];
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int p = reg_pos<NY, RF>(t, i);
    const long long o = boff + (long long)p * pitch + kr;
    const long long to = toff + (long long)p * pitch + kr;       // L table
    const long long co = 6 * toff + (long long)p * pitch + kr;   // ETDRK4 tables
    const C N = v[i];
    C x;
    switch (mode) {
      case COL_PROLOGUE: x = a.s[o]; break;
      case COL_FWD_STORE: x = N; a.s[o] = x; break;
      case COL_FWD_N: x = N; a.nout[o] = N; break;
      case COL_RK4_1: {
        const T L = a.Ltab[to];
        const C s = a.s[o];
        C k; k.x = L * s.x + N.x; k.y = L * s.y + N.y;
        C ac; ac.x = s.x + (dt / 6) * k.x; ac.y = s.y + (dt / 6) * k.y;
        a.acc[o] = ac;
        x.x = s.x + (dt / 2) * k.x; x.y = s.y + (dt / 2) * k.y;
        a.si[o] = x;
      } break;
      case COL_RK4_2:
      case COL_RK4_3: {
        const T L = a.Ltab[to];
        const C si = a.si[o], s = a.s[o];
        C k; k.x = L * si.x + N.x; k.y = L * si.y + N.y;
        C ac = a.acc[o];
        ac.x += (dt / 3) * k.x; ac.y += (dt / 3) * k.y;
        a.acc[o] = ac;
        const T h = (mode == COL_RK4_2) ? dt / 2 : dt;
        x.x = s.x + h * k.x; x.y = s.y + h * k.y;
        a.si[o] = x;
      } break;
      case COL_RK4_4: {
        const T L = a.Ltab[to];
        const C si = a.si[o];
        C k; k.x = L * si.x + N.x; k.y = L * si.y + N.y;
        const C ac = a.acc[o];
        x.x = ac.x + (dt / 6) * k.x; x.y = ac.y + (dt / 6) * k.y;
        a.s[o] = x;
      } break;
      case COL_ETD_1: {
        const T* cf = a.coef + co;
        const T Ee = cf[0], E2 = cf[plane], ze = cf[2 * plane], al = cf[3 * plane];
        const C s = a.s[o];
        a.n1[o] = N;
        C ac; ac.x = Ee * s.x + al * N.x; ac.y = Ee * s.y + al * N.y;
        a.acc[o] = ac;
        x.x = E2 * s.x + ze * N.x; x.y = E2 * s.y + ze * N.y;
        a.si[o] = x;
      } break;
      case COL_ETD_2: {
        const T* cf = a.coef + co;
        const T E2 = cf[plane], ze = cf[2 * plane], be = cf[4 * plane];
        const C s = a.s[o];
        C ac = a.acc[o];
        ac.x += 2 * be * N.x; ac.y += 2 * be * N.y;
        a.acc[o] = ac;
        x.x = E2 * s.x + ze * N.x; x.y = E2 * s.y + ze * N.y;
      } break;
      case COL_ETD_3: {
        const T* cf = a.coef + co;
        const T E2 = cf[plane], ze = cf[2 * plane], be = cf[4 * plane];
        const C s1 = a.si[o], N1 = a.n1[o];
        C ac = a.acc[o];
        ac.x += 2 * be * N.x; ac.y += 2 * be * N.y;
        a.acc[o] = ac;
        x.x = E2 * s1.x + ze * (2 * N.x - N1.x); x.y = E2 * s1.y + ze * (2 * N.y - N1.y);
      } break;
      default: {  // COL_ETD_4
        const T ga = a.coef[co + 5 * plane];
        const C ac = a.acc[o];
        x.x = ac.x + ga * N.x; x.y = ac.y + ga * N.y;
        a.s[o] = x;
      } break;
    }
    sn[i] = x;
  }
  if (!a.do_inverse) return;  // uniform across the block

  // A = Fy^-1(s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = sn[i];
  fft_line<NY, +1>(v, t, line, a.tw);
#pragma unroll
  for (int i = 0; i < E; ++i) a.A[boff + (long long)reg_pos<NY, RO>(t, i) * pitch + kr] = v[i];
  // B = Fy^-1(i l s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const T l = lval<T, NY>(reg_pos<NY, RI>(t, i), a.dky);
    v[i].x = -l * sn[i].y;
    v[i].y = l * sn[i].x;
  }
  fft_line<NY, +1>(v, t, line, a.tw);
#pragma unroll
  for (int i = 0; i < E; ++i) a.B[boff + (long long)reg_pos<NY, RO>(t, i) * pitch + kr] = v[i];
}

// ---------------------------------------------------------------------------
// Row pass.  blockDim.x = P * (NX/16); pair pr = tid / (NX/16) handles rows
// y0 = 2*(blockIdx.x*P + pr) and y0+1; t = tid % (NX/16).
// ---------------------------------------------------------------------------
template <typename T, typename C>
__device__ __forceinline__ C zsrc_rhs(const C* Arow, const C* Brow, int k, int NX, T dkx) {
  // Z[k] = P[k] + i Q[k], P = Hermitian extension of i kr A, Q of B;
  // the imaginary parts of P and Q at the self-conjugate bins are dropped.
  C z;
  const int h = NX / 2;
  if (k == 0) {
    z.x = 0; z.y = Brow[0].x;
  } else if (k == h) {
    const T kr = (T)h * dkx;
    const C av = Arow[h], bv = Brow[h];
    z.x = -kr * av.y; z.y = bv.x;
  } else if (k < h) {
    const T kr = (T)k * dkx;
    const C av = Arow[k], bv = Brow[k];
    // i (kr A + B)
    z.x = -(kr * av.y + bv.y); z.y = kr * av.x + bv.x;
  } else {
    const int kk = NX - k;
    const T kr = (T)kk * dkx;
    const C av = Arow[kk], bv = Brow[kk];
    // i (conj(B) - kr conj(A)) = i ((b.x - kr a.x) + i(-b.y + kr a.y))
    const T re = bv.x - kr * av.x, im = -bv.y + kr * av.y;
    z.x = -im; z.y = re;
  }
  return z;
}
template <typename C>
__device__ __forceinline__ C zsrc_c2r(const C* A0, const C* A1, int k, int NX) {
  // Z[k] = P0[k] + i P1[k] with P0, P1 the Hermitian extensions of rows y0, y1.
  C z;
  const int h = NX / 2;
  if (k == 0 || k == h) {
    z.x = A0[k].x; z.y = A1[k].x;
  } else if (k < h) {
    const C p = A0[k], q = A1[k];
    z.x = p.x - q.y; z.y = p.y + q.x;
  } else {
    const int kk = NX - k;
    const C p = A0[kk], q = A1[kk];
    // conj(p) + i conj(q)
    z.x = p.x + q.y; z.y = -p.y + q.x;
  }
  return z;
}

template <typename T, int NX>
__global__ void row_pass_kernel(RowArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = FFT_E;
  constexpr int TPL = NX / E;
  constexpr int LS = line_stride(NX);
  constexpr int RI0 = FirstRadix<NX, +1>::value;
  constexpr int RIL = LastRadix<NX, +1>::value;   // == 16
  constexpr int RF0 = FirstRadix<NX, -1>::value;  // == 16
  constexpr int RFL = LastRadix<NX, -1>::value;
  static_assert(RIL == RF0, "inverse-last and forward-first radices must match");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int P = blockDim.x / TPL;
  const int pr = threadIdx.x / TPL, t = threadIdx.x % TPL;
  const int y0 = 2 * (blockIdx.x * P + pr);
  const long long boff = (long long)blockIdx.y * a.bstride;
  const long long poff = (long long)blockIdx.y * a.pstride;
  const long long foff = (long long)blockIdx.y * a.fstride;
  const int pitch = a.pitch;
  C* line = sm + pr * LS;
  const bool valid = y0 < a.ny;  // grids are sized exactly; kept for safety
  const int yy0 = valid ? y0 : 0;
  const long long r0 = boff + (long long)yy0 * pitch, r1 = r0 + pitch;
  const long long q0 = (long long)yy0 * NX, q1 = q0 + NX;

  C v[E];
  if (a.mode == ROW_R2C) {
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int x = reg_pos<NX, RF0>(t, i);
      v[i].x = a.cin[poff + q0 + x];
      v[i].y = a.cin[poff + q1 + x];
    }
  } else if (a.mode == ROW_C2R) {
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_c2r<C>(a.A + r0, a.A + r1, reg_pos<NX, RI0>(t, i), NX);
    fft_line<NX, +1>(v, t, line, a.tw);
    if (valid) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int x = reg_pos<NX, RIL>(t, i);
        a.cout[poff + q0 + x] = v[i].x * a.scale;
        a.cout[poff + q1 + x] = v[i].y * a.scale;
      }
    }
    return;
  } else {  // ROW_RHS
    C z0[E];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(a.A + r0, a.B + r0, reg_pos<NX, RI0>(t, i), NX, a.dkx);
    fft_line<NX, +1>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) z0[i] = v[i];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(a.A + r1, a.B + r1, reg_pos<NX, RI0>(t, i), NX, a.dkx);
    fft_line<NX, +1>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int x = reg_pos<NX, RIL>(t, i);
      const T u0 = a.u[foff + q0 + x], v0 = a.v[foff + q0 + x];
      const T u1 = a.u[foff + q1 + x], v1 = a.v[foff + q1 + x];
      C w;
      w.x = u0 * z0[i].x + v0 * z0[i].y;
      w.y = u1 * v[i].x + v1 * v[i].y;
      v[i] = w;
    }
  }
  // forward x-FFT of n_y0 + i n_y1
  fft_line<NX, -1>(v, t, line, a.tw);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E; ++i) line[smem_pad(reg_pos<NX, RFL>(t, i))] = v[i];
  __syncthreads();
  const T sc = a.scale;
  if (valid) {
    for (int k = t; k <= NX / 2; k += TPL) {
      const C wk = line[smem_pad(k)];
      const C wn = line[smem_pad((NX - k) & (NX - 1))];
      C o0, o1;
      // row y0: W[k] + conj(W[n-k]) ; row y1: -i (W[k] - conj(W[n-k]))
      o0.x = (wk.x + wn.x) * sc; o0.y = (wk.y - wn.y) * sc;
      o1.x = (wk.y + wn.y) * sc; o1.y = (wn.x - wk.x) * sc;
      a.out[r0 + k] = o0;
      a.out[r1 + k] = o1;
    }
  }
}

}  // namespace ptf
