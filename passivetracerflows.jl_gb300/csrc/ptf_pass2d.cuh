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
  COL_RK4_1 = 2, COL_RK4_2 = 3, COL_RK4_3 = 4, COL_RK4_4 = 5,   // RK4 stages
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
// Consecutive threads therefore touch consecutive kr of one row: a warp
// reads W-element row segments.  MODE is a compile-time ColMode.
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
// lines, then a private slot array holding each thread's 16 stage outputs
// between the two inverse transforms.
template <typename T, int NY> __host__ __device__ constexpr size_t col_smem_bytes(int W) {
  return (size_t)W * (line_stride(NY) + NY) * sizeof(typename cplx_of<T>::type);
}
template <typename T, int N> __host__ __device__ constexpr int pass_tpl() { return N / PassE<T, N>::value;
}

template <typename T, int NY, int MODE>
__global__ void __launch_bounds__(ColBounds<T>::threads, ColBounds<T>::blocks) col_pass_kernel(ColArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = PassE<T, NY>::value;
  constexpr int TPL = NY / E;
  constexpr int LS = line_stride(NY);
  constexpr int RF0 = FirstRadix<NY, -1, E>::value;  // forward input pattern
  constexpr int RF = LastRadix<NY, -1, E>::value;    // forward output pattern
  constexpr int RI = FirstRadix<NY, +1, E>::value;   // inverse input pattern (== RF)
  constexpr int RO = LastRadix<NY, +1, E>::value;    // inverse output pattern
  static_assert(RF == RI, "forward-last and inverse-first radices must match");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int W = blockDim.x / TPL;
  const int w = threadIdx.x % W, t = threadIdx.x / W;
  const int kr = blockIdx.x * W + w;
  const int pitch = a.pitch;
  const size_t boff = (size_t)blockIdx.y * (size_t)a.bstride;
  const size_t plane = (size_t)NY * (size_t)pitch;
  const size_t toff = a.tab_per_solve ? (size_t)blockIdx.y * plane : 0;
  C* line = sm + w * LS;
  const int tb = t * pitch + kr;  // this thread's offset inside one field
  // offset of register i for a first/last stage of radix R
#define PTF_OFF(R, i) (tb + (((i) / (R)) * TPL + ((i) % (R)) * (NY / (R))) * pitch)

  C v[E];
  if (MODE != COL_PROLOGUE) {
    const C* __restrict__ src = a.nxin + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = src[PTF_OFF(RF0, i)];
    fft_line<NY, -1, E>(v, t, line, a.tw);
  }

  // Stage combination at the positions p = reg_pos<NY, RF, E>(t, i).  The next
  // stage input is parked in this thread's slots of `park` (slot i at
  // park[i*blockDim + tid]: conflict-free, no barrier needed since each
  // thread reads back only what it wrote).
  const T dt = a.dt;
  C* park = sm + W * LS;
  const int nthr = blockDim.x;
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
      if (MODE == COL_PROLOGUE) {
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

  // A = Fy^-1(s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = park[i * nthr + threadIdx.x];
  fft_line<NY, +1, E>(v, t, line, a.tw);
  {
    C* __restrict__ Ap = a.A + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) Ap[PTF_OFF(RO, i)] = v[i];
  }
  // Keep the second transform from being interleaved with the first (that
  // doubles the live registers): memory operations cannot cross this.
  asm volatile("" ::: "memory");
  // B = Fy^-1(i l s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const T l = lval<T, NY>(reg_pos<NY, RI, E>(t, i), a.dky);
    const C x = park[i * nthr + threadIdx.x];
    v[i].x = -l * x.y;
    v[i].y = l * x.x;
  }
  fft_line<NY, +1, E>(v, t, line, a.tw);
  {
    C* __restrict__ Bp = a.B + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) Bp[PTF_OFF(RO, i)] = v[i];
  }
#undef PTF_OFF
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
  const bool valid = y0 < a.ny;  // grids are sized exactly; kept for safety
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
  } else {  // ROW_RHS
    C z0[E];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(a.A + r0, a.B + r0, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
    fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) z0[i] = v[i];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(a.A + r1, a.B + r1, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
    fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int x = reg_pos<NX, RIL, E>(t, i);
      const T u0 = a.u[foff + q0 + x], v0 = a.v[foff + q0 + x];
      const T u1 = a.u[foff + q1 + x], v1 = a.v[foff + q1 + x];
      C w;
      w.x = u0 * z0[i].x + v0 * z0[i].y;
      w.y = u1 * v[i].x + v1 * v[i].y;
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
