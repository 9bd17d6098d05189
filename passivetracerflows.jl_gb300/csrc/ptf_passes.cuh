// Pass kernels of the tracer advection-diffusion right-hand side (2D and 3D).
//
// Spectral arrays are [nz][ny][pitch] complex with kr fastest (the layout of
// the reference's (nkr, nl[, nm]) column-major arrays, padded to `pitch`);
// physical arrays are [nz][ny][nx] real, x fastest (nz = 1 in 2D).  One RHS
// evaluation (calcN!, src/traceradvectiondiffusion.jl:756-786) is split into
// passes along one axis each:
//
//   column pass: along y (2D) or z (3D): forward FFT of the previous pass's
//       output, the time-stepper stage combination with the linear
//       operator, then the inverse FFTs of the next stage input s and of
//       i*k_axis*s -> A, B.  The same kernel, in other modes, is the 3D
//       y-forward pass and the 3D y-inverse pass (three outputs).
//   row pass (x): per pair of rows, inverse x-FFT of Z = i(kr A + B)
//       (Hermitian-extended; Re z = c_x, Im z = c_y; in 3D one more packed
//       inverse gives c_z of both rows), the product n = -(u.grad c), and one
//       forward x-FFT of n_y0 + i n_y1, separated into the two rows' half
//       spectra.
//
// The flow passed to the row pass is pre-scaled by -1/(2 N) (N = grid
// points): that folds the inverse normalisation, the minus sign and the 1/2
// of the two-for-one separation into the product.
#pragma once
#include "ptf_fft.cuh"

namespace ptf {

enum ColMode : int {
  COL_PROLOGUE = 0,   // s -> A, B
  COL_FWD_STORE = 1,  // s = F(nxin) ; then A, B of s
  COL_RK4_1 = 2, COL_RK4_2 = 3, COL_RK4_3 = 4, COL_RK4_4 = 5,   // RK4 stages
  COL_ETD_1 = 6, COL_ETD_2 = 7, COL_ETD_3 = 8, COL_ETD_4 = 9,   // ETDRK4 stages
  COL_FWD_N = 10,     // nout = F(nxin), nothing else (calcN, 3D y-forward)
  COL_YINV3 = 11,     // 3D y-inverse: A = F^-1(s), B = F^-1(i l s), C = F^-1(z2in)
};
constexpr int COL_NMODES = 12;
enum RowMode : int { ROW_RHS = 0, ROW_C2R = 1, ROW_R2C = 2, ROW_RHS3 = 3 };

template <typename T> struct ColArgs {
  typedef typename cplx_of<T>::type C;
  const C* nxin;   // forward input
  C* s;            // state (sol); COL_YINV3: the z-inverse Z1
  C* si;           // RK4: current stage input; ETDRK4: sol1 ("a")
  C* acc;          // accumulator of the update
  C* n1;           // ETDRK4: N(sol)
  C* A;            // F^-1(s_next)
  C* B;            // F^-1(i k s_next)
  C* Cout;         // COL_YINV3: F^-1(z2in)
  const C* z2in;   // COL_YINV3: the z-inverse Z2
  C* nout;         // COL_FWD_N output
  const C* tw;     // transform-length twiddles
  const T* Ltab;   // linear operator, one value per spectral element
  const T* coef;   // ETDRK4 tables E, E2, zeta, alpha, beta, gamma, `tplane` apart
  T dt, dk;        // dk: 2*pi/L of the transform axis
  int stride;      // elements between consecutive points of a line
  int mode, do_inverse;
  long long bstride;    // elements between blockIdx.y blocks of fields
  long long tplane;     // elements of one table plane
  int tab_per_block;    // 1: tables advance with blockIdx.y (per-solve tables)
};

template <typename T> struct RowArgs {
  typedef typename cplx_of<T>::type C;
  const C* A;
  const C* B;
  const C* Cin;    // ROW_RHS3: F_y^-1 F_z^-1 (i m s)
  C* out;          // ROW_RHS* / ROW_R2C: half spectra [rows][pitch]
  const T* u;      // ROW_RHS*: scaled flow [rows][nx]
  const T* v;
  const T* w;
  const T* cin;    // ROW_R2C: physical input [rows][nx]
  T* cout;         // ROW_C2R: physical output
  const C* tw;     // NX-point twiddles
  T dkx, scale;    // scale: C2R normalisation / R2C 1/2 / RHS 1
  int rows, pitch, mode;
  long long bstride, pstride, fstride;
};

template <typename T, int N>
__device__ __forceinline__ T kval(int p, T dk) { return (T)(p < N / 2 ? p : p - N) * dk; }

// ---------------------------------------------------------------------------
// Column pass.  blockDim.x = W * (N/E); w = tid % W selects the column
// (col = blockIdx.x*W + w, a flat index over the non-transformed axes whose
// elements are contiguous), t = tid / W the thread within the column's line.
// Consecutive threads therefore touch consecutive columns: a warp reads
// W-element segments.  MODE is a compile-time ColMode.
// ---------------------------------------------------------------------------
#ifndef PTF_COL_MINB_F32
#define PTF_COL_MINB_F32 2
#endif
#ifndef PTF_COL_MINB_F64
#define PTF_COL_MINB_F64 1
#endif
template <typename T> struct ColBounds { static constexpr int threads = 256, blocks = PTF_COL_MINB_F64; };
template <> struct ColBounds<float> { static constexpr int threads = 256, blocks = PTF_COL_MINB_F32; };
// Dynamic shared memory of a column-pass block with W lines: the W FFT
// lines, then a private slot array holding each thread's values between
// transforms.
template <typename T, int N> __host__ __device__ constexpr size_t col_smem_bytes(int W) {
  return (size_t)W * (line_stride(N) + N) * sizeof(typename cplx_of<T>::type);
}
template <typename T, int N> __host__ __device__ constexpr int pass_tpl() { return N / PassE<T, N>::value; }

template <typename T, int N, int MODE>
__global__ void __launch_bounds__(ColBounds<T>::threads, ColBounds<T>::blocks) col_pass_kernel(ColArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = PassE<T, N>::value;
  constexpr int TPL = N / E;
  constexpr int LS = line_stride(N);
  constexpr int RF0 = FirstRadix<N, -1, E>::value;  // forward input pattern
  constexpr int RF = LastRadix<N, -1, E>::value;    // forward output pattern
  constexpr int RI = FirstRadix<N, +1, E>::value;   // inverse input pattern (== RF)
  constexpr int RO = LastRadix<N, +1, E>::value;    // inverse output pattern
  static_assert(RF == RI, "forward-last and inverse-first radices must match");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int W = blockDim.x / TPL;
  const int w = threadIdx.x % W, t = threadIdx.x / W;
  const int col = blockIdx.x * W + w;
  const int stride = a.stride;
  const size_t boff = (size_t)blockIdx.y * (size_t)a.bstride;
  const size_t plane = (size_t)a.tplane;
  const size_t toff = a.tab_per_block ? (size_t)blockIdx.y * plane : 0;
  C* line = sm + w * LS;
  C* park = sm + W * LS;  // slot i of this thread: park[i*blockDim + tid]
  const int nthr = blockDim.x;
  const int tb = t * stride + col;  // this thread's offset inside one field
  // offset of register i for a first/last stage of radix R
#define PTF_OFF(R, i) (tb + (((i) / (R)) * TPL + ((i) % (R)) * (N / (R))) * stride)

  C v[E];
  if (MODE != COL_PROLOGUE && MODE != COL_YINV3) {
    const C* __restrict__ src = a.nxin + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = src[PTF_OFF(RF0, i)];
    fft_line<N, -1, E>(v, t, line, a.tw);
  }

  // Stage combination at the positions p = reg_pos<N, RF, E>(t, i); the
  // next stage input is parked (each thread reads back only its own slots,
  // so no barrier is needed).
  const T dt = a.dt;
  {
    C* __restrict__ S = a.s + boff;
    C* __restrict__ SI = a.si + boff;
    C* __restrict__ AC = a.acc + boff;
    C* __restrict__ N1p = a.n1 + boff;
    const T* __restrict__ Lt = a.Ltab + toff;
    const T* __restrict__ cf = a.coef + 6 * toff;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int o = PTF_OFF(RF, i);
      const C N = v[i];
      C x;
      if (MODE == COL_PROLOGUE || MODE == COL_YINV3) {
        x = S[o];
      } else if (MODE == COL_FWD_STORE) {
        x = N; S[o] = x;
      } else if (MODE == COL_FWD_N) {
        x = N; a.nout[boff + o] = N;
      } else if (MODE == COL_RK4_1) {
        const T L = Lt[o];
        const C s = S[o];
        C k; k.x = L * s.x + N.x; k.y = L * s.y + N.y;
        C ac; ac.x = s.x + (dt / 6) * k.x; ac.y = s.y + (dt / 6) * k.y;
        AC[o] = ac;
        x.x = s.x + (dt / 2) * k.x; x.y = s.y + (dt / 2) * k.y;
        SI[o] = x;
      } else if (MODE == COL_RK4_2 || MODE == COL_RK4_3) {
        const T L = Lt[o];
        const C si = SI[o], s = S[o];
        C ac = AC[o];
        C k; k.x = L * si.x + N.x; k.y = L * si.y + N.y;
        ac.x += (dt / 3) * k.x; ac.y += (dt / 3) * k.y;
        AC[o] = ac;
        const T h = (MODE == COL_RK4_2) ? dt / 2 : dt;
        x.x = s.x + h * k.x; x.y = s.y + h * k.y;
        SI[o] = x;
      } else if (MODE == COL_RK4_4) {
        const T L = Lt[o];
        const C si = SI[o], ac = AC[o];
        C k; k.x = L * si.x + N.x; k.y = L * si.y + N.y;
        x.x = ac.x + (dt / 6) * k.x; x.y = ac.y + (dt / 6) * k.y;
        S[o] = x;
      } else if (MODE == COL_ETD_1) {
        const T Ee = cf[o], E2 = cf[o + plane], ze = cf[o + 2 * plane], al = cf[o + 3 * plane];
        const C s = S[o];
        N1p[o] = N;
        C ac; ac.x = Ee * s.x + al * N.x; ac.y = Ee * s.y + al * N.y;
        AC[o] = ac;
        x.x = E2 * s.x + ze * N.x; x.y = E2 * s.y + ze * N.y;
        SI[o] = x;
      } else if (MODE == COL_ETD_2) {
        const T E2 = cf[o + plane], ze = cf[o + 2 * plane], be = cf[o + 4 * plane];
        const C s = S[o];
        C ac = AC[o];
        ac.x += 2 * be * N.x; ac.y += 2 * be * N.y;
        AC[o] = ac;
        x.x = E2 * s.x + ze * N.x; x.y = E2 * s.y + ze * N.y;
      } else if (MODE == COL_ETD_3) {
        const T E2 = cf[o + plane], ze = cf[o + 2 * plane], be = cf[o + 4 * plane];
        const C s1 = SI[o], N1 = N1p[o];
        C ac = AC[o];
        ac.x += 2 * be * N.x; ac.y += 2 * be * N.y;
        AC[o] = ac;
        x.x = E2 * s1.x + ze * (2 * N.x - N1.x); x.y = E2 * s1.y + ze * (2 * N.y - N1.y);
      } else {  // COL_ETD_4
        const T ga = cf[o + 5 * plane];
        const C ac = AC[o];
        x.x = ac.x + ga * N.x; x.y = ac.y + ga * N.y;
        S[o] = x;
      }
      park[i * nthr + threadIdx.x] = x;
    }
  }
  if (MODE == COL_FWD_N || !a.do_inverse) return;  // uniform across the block

  // A = F^-1(s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = park[i * nthr + threadIdx.x];
  fft_line<N, +1, E>(v, t, line, a.tw);
  {
    C* __restrict__ Ap = a.A + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) Ap[PTF_OFF(RO, i)] = v[i];
  }
  // Keep the second transform from being interleaved with the first (that
  // doubles the live registers): memory operations cannot cross this.
  asm volatile("" ::: "memory");
  // B = F^-1(i k s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const T k = kval<T, N>(reg_pos<N, RI, E>(t, i), a.dk);
    const C x = park[i * nthr + threadIdx.x];
    v[i].x = -k * x.y;
    v[i].y = k * x.x;
  }
  fft_line<N, +1, E>(v, t, line, a.tw);
  {
    C* __restrict__ Bp = a.B + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) Bp[PTF_OFF(RO, i)] = v[i];
  }
  if (MODE == COL_YINV3) {
    asm volatile("" ::: "memory");
    // C = F^-1(z2in)
    const C* __restrict__ Z2 = a.z2in + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = Z2[PTF_OFF(RI, i)];
    fft_line<N, +1, E>(v, t, line, a.tw);
    C* __restrict__ Cp = a.Cout + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) Cp[PTF_OFF(RO, i)] = v[i];
  }
#undef PTF_OFF
}

// ---------------------------------------------------------------------------
// Row pass.  blockDim.x = P * (NX/E); pair pr = tid / (NX/E) handles rows
// y0 = 2*(blockIdx.x*P + pr) and y0+1 (a flat row index over (z, y));
// t = tid % (NX/E).
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

// Shared memory of a row-pass block with P pairs: one FFT line and two
// parking slots per point of each pair.
template <typename T, int NX> __host__ __device__ constexpr size_t row_smem_bytes(int P) {
  return (size_t)P * (line_stride(NX) + 2 * NX) * sizeof(typename cplx_of<T>::type);
}

template <typename T, int NX>
__global__ void __launch_bounds__(256) row_pass_kernel(RowArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = PassE<T, NX>::value;
  constexpr int TPL = NX / E;
  constexpr int LS = line_stride(NX);
  constexpr int RI0 = FirstRadix<NX, +1, E>::value;
  constexpr int RIL = LastRadix<NX, +1, E>::value;   // == E
  constexpr int RF0 = FirstRadix<NX, -1, E>::value;  // == E
  constexpr int RFL = LastRadix<NX, -1, E>::value;
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
  C* park = sm + P * LS + pr * 2 * NX;  // this pair's slots: park[i*TPL + t], park[NX + i*TPL + t]
  const bool valid = y0 < a.rows;  // grids are sized exactly; kept for safety
  const int yy0 = valid ? y0 : 0;
  const long long r0 = boff + (long long)yy0 * pitch, r1 = r0 + pitch;
  const long long q0 = (long long)yy0 * NX, q1 = q0 + NX;

  C v[E];
  if (a.mode == ROW_R2C) {
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int x = reg_pos<NX, RF0, E>(t, i);
      v[i].x = a.cin[poff + q0 + x];
      v[i].y = a.cin[poff + q1 + x];
    }
  } else if (a.mode == ROW_C2R) {
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_c2r<C>(a.A + r0, a.A + r1, reg_pos<NX, RI0, E>(t, i), NX);
    fft_line<NX, +1, E>(v, t, line, a.tw);
    if (valid) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int x = reg_pos<NX, RIL, E>(t, i);
        a.cout[poff + q0 + x] = v[i].x * a.scale;
        a.cout[poff + q1 + x] = v[i].y * a.scale;
      }
    }
    return;
  } else {  // ROW_RHS / ROW_RHS3
    const bool three = (a.mode == ROW_RHS3);
    if (three) {
      // c_z of both rows: Z = C0 + i C1 (Hermitian extensions) -> park
#pragma unroll
      for (int i = 0; i < E; ++i) v[i] = zsrc_c2r<C>(a.Cin + r0, a.Cin + r1, reg_pos<NX, RI0, E>(t, i), NX);
      fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
      for (int i = 0; i < E; ++i) park[NX + i * TPL + t] = v[i];
      asm volatile("" ::: "memory");
    }
    // row y0: c_x + i c_y -> park the product's first half
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(a.A + r0, a.B + r0, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
    fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int x = reg_pos<NX, RIL, E>(t, i);
      T n0 = a.u[foff + q0 + x] * v[i].x + a.v[foff + q0 + x] * v[i].y;
      if (three) n0 += a.w[foff + q0 + x] * park[NX + i * TPL + t].x;
      C pk; pk.x = n0; pk.y = 0;
      park[i * TPL + t] = pk;
    }
    asm volatile("" ::: "memory");
    // row y1
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(a.A + r1, a.B + r1, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
    fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int x = reg_pos<NX, RIL, E>(t, i);
      T n1 = a.u[foff + q1 + x] * v[i].x + a.v[foff + q1 + x] * v[i].y;
      if (three) n1 += a.w[foff + q1 + x] * park[NX + i * TPL + t].y;
      C w;
      w.x = park[i * TPL + t].x;
      w.y = n1;
      v[i] = w;
    }
  }
  // forward x-FFT of n_y0 + i n_y1
  fft_line<NX, -1, E>(v, t, line, a.tw);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E; ++i) line[smem_pad(reg_pos<NX, RFL, E>(t, i))] = v[i];
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
