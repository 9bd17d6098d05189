// Shared-memory Stockham FFT building blocks for sm_103a.
//
// A "line" of N complex values (N a power of two, 16 <= N <= 4096) is
// transformed by N/E threads that each hold E = 16 values in registers.
// Stages are radix-16 except one radix-2/4/8 stage when N is not a power
// of 16.  Between stages the line is exchanged through shared memory
// (padded index i + i/16 so that the stride-16 write pattern of the first
// stage is bank-conflict free).  The algorithm is the Stockham autosort
// decimation-in-time formulation (Govindaraju et al., SC'08): stage with
// radix R after sub-transforms of size NS reads x[j + r*N/R], multiplies by
// w_{NS*R}^{r*(j mod NS)}, does a radix-R DFT and writes
// y[(j/NS)*NS*R + (j mod NS) + r*NS].  Output is in natural order.
//
// Register convention: thread t owns butterflies j = t + q*(N/E),
// q = 0..E/R-1, and register v[q*R + r] holds element j + r*(N/R) at the
// first-stage input and at the last-stage output (R = that stage's radix).
// An inverse transform whose last radix equals the next forward
// transform's first radix can therefore feed it with no shared-memory
// exchange; the row pass relies on this.
//
// Twiddles come from a per-N table tw[m] = exp(-2*pi*i*m/N) computed on the
// host in FP64 (octant symmetry on host libm values) and read through the
// read-only cache; the inverse uses the conjugate.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ptf {

template <typename T> struct cplx_of;
template <> struct cplx_of<double> { typedef double2 type; };
template <> struct cplx_of<float> { typedef float2 type; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename C> __device__ __forceinline__ C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }
// (DIR*i) * v ; DIR = -1 forward, +1 inverse
template <int DIR, typename C> __device__ __forceinline__ C mul_dir_i(C v) {
  C r;
  if (DIR < 0) { r.x = v.y; r.y = -v.x; } else { r.x = -v.y; r.y = v.x; }
  return r;
}
// v * (c + i s)
template <typename C, typename T> __device__ __forceinline__ C cmul_cs(C v, T c, T s) {
  C r; r.x = v.x * c - v.y * s; r.y = v.x * s + v.y * c; return r;
}
// v * w (forward twiddle) or v * conj(w) (inverse)
template <typename C> __device__ __forceinline__ C cmul_plain(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// FP32 stages of radix 8 and 16 apply a butterfly's twiddles W^r in a
// factored form (twiddled_dft below): only table values, none formed by
// multiplying rounded twiddles together.  PTF_TW_POW2 (radix 32 only, FP32)
// loads the power-of-two powers and multiplies out the rest.
#ifndef PTF_TW_POW2
#define PTF_TW_POW2 1
#endif

template <int DIR, typename C> __device__ __forceinline__ C cmul_tw(C v, C w) {
  C r;
  if (DIR < 0) { r.x = v.x * w.x - v.y * w.y; r.y = v.x * w.y + v.y * w.x; }
  else         { r.x = v.x * w.x + v.y * w.y; r.y = v.y * w.x - v.x * w.y; }
  return r;
}

// cos and sin of m*pi/8 (exact mathematical constants).
__host__ __device__ constexpr double cos_pi8(int m) {
  return (m & 15) == 0 ? 1.0 : (m & 15) == 1 ? 0.92387953251128674 : (m & 15) == 2 ? 0.70710678118654752
       : (m & 15) == 3 ? 0.38268343236508977 : (m & 15) == 4 ? 0.0 : (m & 15) == 5 ? -0.38268343236508977
       : (m & 15) == 6 ? -0.70710678118654752 : (m & 15) == 7 ? -0.92387953251128674 : (m & 15) == 8 ? -1.0
       : (m & 15) == 9 ? -0.92387953251128674 : (m & 15) == 10 ? -0.70710678118654752
       : (m & 15) == 11 ? -0.38268343236508977 : (m & 15) == 12 ? 0.0 : (m & 15) == 13 ? 0.38268343236508977
       : (m & 15) == 14 ? 0.70710678118654752 : 0.92387953251128674;
}
__host__ __device__ constexpr double sin_pi8(int m) { return cos_pi8(m - 4); }

// cos of m*pi/16 by symmetry from the first-quadrant values.
__host__ __device__ constexpr double cos_q16(int k) {  // 0 <= k <= 8
  return k == 0 ? 1.0 : k == 1 ? 0.98078528040323044 : k == 2 ? 0.92387953251128674 : k == 3 ? 0.83146961230254524
       : k == 4 ? 0.70710678118654752 : k == 5 ? 0.55557023301960218 : k == 6 ? 0.38268343236508977
       : k == 7 ? 0.19509032201612826 : 0.0;
}
__host__ __device__ constexpr double cos_pi16(int m) {
  return ((m % 32) + 32) % 32 <= 8 ? cos_q16(((m % 32) + 32) % 32)
       : ((m % 32) + 32) % 32 <= 16 ? -cos_q16(16 - ((m % 32) + 32) % 32)
       : ((m % 32) + 32) % 32 <= 24 ? -cos_q16(((m % 32) + 32) % 32 - 16)
       : cos_q16(32 - ((m % 32) + 32) % 32);
}
__host__ __device__ constexpr double sin_pi16(int m) { return cos_pi16(m - 8); }

// v * exp(DIR * 2*pi*i * m / 16) for a compile-time m.
template <int DIR, int M, typename C> __device__ __forceinline__ C rot16(C v) {
  typedef decltype(v.x) T;
  constexpr int m = ((M % 16) + 16) % 16;
  if (m == 0) return v;
  if (m == 8) { C r; r.x = -v.x; r.y = -v.y; return r; }
  if (m == 4) return mul_dir_i<DIR>(v);
  if (m == 12) return mul_dir_i<-DIR>(v);
  constexpr double c = cos_pi8(m);  // angle 2*pi*m/16 = m*pi/8
  constexpr double s = (DIR < 0 ? -1.0 : 1.0) * sin_pi8(m);
  return cmul_cs(v, (T)c, (T)s);
}

// v * exp(DIR * 2*pi*i * m / 32) for a compile-time m.
template <int DIR, int M, typename C> __device__ __forceinline__ C rot32(C v) {
  typedef decltype(v.x) T;
  constexpr int m = ((M % 32) + 32) % 32;
  if (m % 2 == 0) return rot16<DIR, m / 2>(v);
  constexpr double c = cos_pi16(m);  // angle 2*pi*m/32 = m*pi/16
  constexpr double s = (DIR < 0 ? -1.0 : 1.0) * sin_pi16(m);
  return cmul_cs(v, (T)c, (T)s);
}

template <int DIR, typename C> __device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a; a = cadd(t, b); b = csub(t, b);
}
// natural-order in place DFT-4 of (a0, a1, a2, a3)
template <int DIR, typename C> __device__ __forceinline__ void dft4(C& a0, C& a1, C& a2, C& a3) {
  C s02 = cadd(a0, a2), d02 = csub(a0, a2), s13 = cadd(a1, a3), d13 = mul_dir_i<DIR>(csub(a1, a3));
  a0 = cadd(s02, s13); a2 = csub(s02, s13); a1 = cadd(d02, d13); a3 = csub(d02, d13);
}

// DFT-R on v[0..R) (stride 1), natural order output.
template <int R, int DIR, typename C> struct DFT;
template <int DIR, typename C> struct DFT<2, DIR, C> {
  static __device__ __forceinline__ void run(C* v) { dft2<DIR>(v[0], v[1]); }
};
template <int DIR, typename C> struct DFT<4, DIR, C> {
  static __device__ __forceinline__ void run(C* v) { dft4<DIR>(v[0], v[1], v[2], v[3]); }
};
// 8 = 2 (inner, over n1) x 4 (outer, over n2): X[k1 + 2 k2]
template <int DIR, typename C> struct DFT<8, DIR, C> {
  static __device__ __forceinline__ void run(C* v) {
    dft2<DIR>(v[0], v[4]); dft2<DIR>(v[1], v[5]); dft2<DIR>(v[2], v[6]); dft2<DIR>(v[3], v[7]);
    // y[n2][k1] : k1=0 -> v[n2], k1=1 -> v[4+n2]; twiddle w8^(n2*k1) = w16^(2*n2)
    v[5] = rot16<DIR, 2>(v[5]); v[6] = rot16<DIR, 4>(v[6]); v[7] = rot16<DIR, 6>(v[7]);
    dft4<DIR>(v[0], v[1], v[2], v[3]);   // k1 = 0 -> X[0,2,4,6]
    dft4<DIR>(v[4], v[5], v[6], v[7]);   // k1 = 1 -> X[1,3,5,7]
    C t[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) t[i] = v[i];
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) { v[2 * k2] = t[k2]; v[2 * k2 + 1] = t[4 + k2]; }
  }
};
// 16 = 4 (inner, over n1) x 4 (outer, over n2): X[k1 + 4 k2]
template <int DIR, typename C> struct DFT<16, DIR, C> {
  static __device__ __forceinline__ void run(C* v) {
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4<DIR>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
    // y[n2][k1] now in v[n2 + 4*k1]; twiddle by w16^(n2*k1)
    v[5] = rot16<DIR, 1>(v[5]);  v[6] = rot16<DIR, 2>(v[6]);  v[7] = rot16<DIR, 3>(v[7]);
    v[9] = rot16<DIR, 2>(v[9]);  v[10] = rot16<DIR, 4>(v[10]); v[11] = rot16<DIR, 6>(v[11]);
    v[13] = rot16<DIR, 3>(v[13]); v[14] = rot16<DIR, 6>(v[14]); v[15] = rot16<DIR, 9>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // X[k1 + 4 k2] = v[4 k1 + k2]: transpose 4x4
    C t[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = v[i];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[4 * k1 + k2];
  }
};

// 32 = 4 (inner, over n1; inputs stride 8) x 8 (outer, over n2): X[k1 + 4 k2]
template <int DIR, typename C> struct DFT<32, DIR, C> {
  static __device__ __forceinline__ void run(C* v) {
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) dft4<DIR>(v[n2], v[n2 + 8], v[n2 + 16], v[n2 + 24]);
    // y[n2][k1] in v[n2 + 8*k1]; twiddle by w32^(n2*k1)
#define PTF_R32(n2, k1) v[n2 + 8 * k1] = rot32<DIR, n2 * k1>(v[n2 + 8 * k1]);
    PTF_R32(1, 1) PTF_R32(2, 1) PTF_R32(3, 1) PTF_R32(4, 1) PTF_R32(5, 1) PTF_R32(6, 1) PTF_R32(7, 1)
    PTF_R32(1, 2) PTF_R32(2, 2) PTF_R32(3, 2) PTF_R32(4, 2) PTF_R32(5, 2) PTF_R32(6, 2) PTF_R32(7, 2)
    PTF_R32(1, 3) PTF_R32(2, 3) PTF_R32(3, 3) PTF_R32(4, 3) PTF_R32(5, 3) PTF_R32(6, 3) PTF_R32(7, 3)
#undef PTF_R32
    // outer DFT-8 over n2 for each k1 (contiguous v[8*k1 .. 8*k1+7]) -> X[k1 + 4 k2] at v[8 k1 + k2]
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) DFT<8, DIR, C>::run(v + 8 * k1);
    C t[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) t[i] = v[i];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 8; ++k2) v[k1 + 4 * k2] = t[8 * k1 + k2];
  }
};

// A radix-16 or radix-8 Stockham butterfly with its input twiddles
// t_r = W^r (W = this butterfly's base twiddle, r = 0..R-1) applied in
// factored form.  The DFT splits r = n2 + 4 n1 (inner DFT over n1, the
// stride-4 elements; outer over n2): t_r = W^(4 n1) W^n2, and W^n2 is
// constant across each inner DFT, so it is applied to the inner DFT's
// outputs instead of its inputs.  The twiddles used are W, W^2, W^3, W^4,
// W^8, W^12 (radix 16) or W..W^4 (radix 8), each a correctly rounded table
// value: no twiddle is a product of rounded twiddles.  Radix 16: 24 complex
// products (the direct form needs 15, plus 11 to build W^r from four table
// values), 6 table loads.  Same arithmetic as DFT<R> after the twiddles.
template <int R, int DIR, typename C> struct TwiddledDFT;
template <int DIR, typename C> struct TwiddledDFT<16, DIR, C> {
  static __device__ __forceinline__ void run(C* v, const C* __restrict__ tw, int b) {
    const C w1 = __ldg(tw + b), w2 = __ldg(tw + 2 * b), w3 = __ldg(tw + 3 * b);
    const C w4 = __ldg(tw + 4 * b), w8 = __ldg(tw + 8 * b), w12 = __ldg(tw + 12 * b);
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      v[n2 + 4] = cmul_tw<DIR>(v[n2 + 4], w4);
      v[n2 + 8] = cmul_tw<DIR>(v[n2 + 8], w8);
      v[n2 + 12] = cmul_tw<DIR>(v[n2 + 12], w12);
      dft4<DIR>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
    }
    // y[n2][k1] in v[n2 + 4*k1]: times W^n2, then the internal twiddle w16^(n2*k1)
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      v[1 + 4 * k1] = cmul_tw<DIR>(v[1 + 4 * k1], w1);
      v[2 + 4 * k1] = cmul_tw<DIR>(v[2 + 4 * k1], w2);
      v[3 + 4 * k1] = cmul_tw<DIR>(v[3 + 4 * k1], w3);
    }
    v[5] = rot16<DIR, 1>(v[5]);  v[6] = rot16<DIR, 2>(v[6]);  v[7] = rot16<DIR, 3>(v[7]);
    v[9] = rot16<DIR, 2>(v[9]);  v[10] = rot16<DIR, 4>(v[10]); v[11] = rot16<DIR, 6>(v[11]);
    v[13] = rot16<DIR, 3>(v[13]); v[14] = rot16<DIR, 6>(v[14]); v[15] = rot16<DIR, 9>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    C t[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = v[i];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[4 * k1 + k2];
  }
};
template <int DIR, typename C> struct TwiddledDFT<8, DIR, C> {
  static __device__ __forceinline__ void run(C* v, const C* __restrict__ tw, int b) {
    const C w1 = __ldg(tw + b), w2 = __ldg(tw + 2 * b), w3 = __ldg(tw + 3 * b), w4 = __ldg(tw + 4 * b);
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      v[n2 + 4] = cmul_tw<DIR>(v[n2 + 4], w4);
      dft2<DIR>(v[n2], v[n2 + 4]);
    }
    // y[n2][k1] in v[n2 + 4*k1]: times W^n2, then the internal twiddle w8^(n2*k1)
#pragma unroll
    for (int k1 = 0; k1 < 2; ++k1) {
      v[1 + 4 * k1] = cmul_tw<DIR>(v[1 + 4 * k1], w1);
      v[2 + 4 * k1] = cmul_tw<DIR>(v[2 + 4 * k1], w2);
      v[3 + 4 * k1] = cmul_tw<DIR>(v[3 + 4 * k1], w3);
    }
    v[5] = rot16<DIR, 2>(v[5]); v[6] = rot16<DIR, 4>(v[6]); v[7] = rot16<DIR, 6>(v[7]);
    dft4<DIR>(v[0], v[1], v[2], v[3]);
    dft4<DIR>(v[4], v[5], v[6], v[7]);
    C t[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) t[i] = v[i];
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) { v[2 * k2] = t[k2]; v[2 * k2 + 1] = t[4 + k2]; }
  }
};

constexpr int FFT_E = 16;  // default complex values per thread

// Values per thread of the row (and 1D, batched) passes: 16; FP32 lengths
// from PTF_ROW_E32_MIN on take 32 (radix-32 stages: fewer shared-memory
// exchanges, at twice the registers per thread).
#ifndef PTF_ROW_E32_MIN
#define PTF_ROW_E32_MIN 0x7fffffff  // lengths from which FP32 row passes take 32 values per thread
#endif
template <typename T, int N> struct PassE { static constexpr int value = 16; };
template <int N> struct PassE<float, N> { static constexpr int value = N >= PTF_ROW_E32_MIN ? 32 : 16; };

// Radix schedule for N with E = 16: NB16 radix-16 stages plus one radix
// REM stage (REM = 1 means none).  Forward order puts REM last; inverse
// order puts REM first, so that inverse-last and forward-first radices are
// both 16 and the row pass can chain them through registers.
template <int N> struct Log2 { static constexpr int value = 1 + Log2<N / 2>::value; };
template <> struct Log2<1> { static constexpr int value = 0; };
// Radix schedule for N with E values per thread: NBE radix-E stages plus one
// radix-REM stage (REM = 1: none).
template <int N, int E = FFT_E> struct Sched {
  static constexpr int log2n = Log2<N>::value;
  static constexpr int log2e = Log2<E>::value;
  static constexpr int NBE = log2n / log2e;
  static constexpr int REM = 1 << (log2n % log2e);
  static constexpr int NSTAGES = NBE + (REM > 1 ? 1 : 0);
  static constexpr int TPL = N / E;  // threads per line
};

__host__ __device__ constexpr int smem_pad(int i) { return i + (i >> 4); }
// line stride in elements: padded length rounded to 32, plus 2 (see bank notes)
__host__ __device__ constexpr int line_stride(int n) { return ((smem_pad(n - 1) + 1 + 31) / 32) * 32 + 2; }

template <typename C> __device__ __forceinline__ C ldtw(const C* __restrict__ tw, int m) { return __ldg(tw + m); }

// One Stockham stage.  Input: v[] holds this stage's read pattern
// (x[j + r*N/R]).  Twiddle + DFT in registers.  Output written to the
// line in shared memory with the Stockham write pattern (STORE=true), or
// left in registers (last stage).
template <int N, int R, int NS, int DIR, int E, typename C>
__device__ __forceinline__ void stage_compute(C* v, int t, const C* __restrict__ tw) {
#pragma unroll
  for (int q = 0; q < E / R; ++q) {
    const int j = t + q * (N / E);
    if constexpr (NS > 1 && (R == 8 || R == 16) && sizeof(C) == 8) {
      // FP32: twiddles applied in factored form inside the butterfly
      TwiddledDFT<R, DIR, C>::run(v + q * R, tw, (j % NS) * (N / (NS * R)));
      continue;
    }
    if (NS > 1) {
      const int k = j % NS;
      if (PTF_TW_POW2 && R >= 8 && sizeof(v[0].x) == 4) {
        // FP32: load the power-of-two powers w^1, w^2, w^4, ... of this
        // butterfly's twiddle and form each other power as w^hb * w^(r-hb)
        // (hb the highest power of two in r): at most log2(R)-1 products
        // (error a few ulp), log2(R) table loads instead of R-1
        const int b = k * (N / (NS * R));
        C w[R];
#pragma unroll
        for (int p = 1; p < R; p *= 2) w[p] = ldtw(tw, p * b);
#pragma unroll
        for (int r = 3; r < R; ++r) {
          if ((r & (r - 1)) == 0) continue;
          int hb = 1;
          while (hb * 2 <= r) hb *= 2;
          w[r] = cmul_plain(w[hb], w[r - hb]);
        }
#pragma unroll
        for (int r = 1; r < R; ++r) v[q * R + r] = cmul_tw<DIR>(v[q * R + r], w[r]);
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) v[q * R + r] = cmul_tw<DIR>(v[q * R + r], ldtw(tw, r * k * (N / (NS * R))));
      }
    }
    DFT<R, DIR, C>::run(v + q * R);
  }
}
template <int N, int R, int NS, int E, typename C>
__device__ __forceinline__ void stage_store(const C* v, int t, C* line) {
#pragma unroll
  for (int q = 0; q < E / R; ++q) {
    const int j = t + q * (N / E);
    const int k = j % NS;
    const int base = (j / NS) * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) line[smem_pad(base + r * NS)] = v[q * R + r];
  }
}
template <int N, int R, int E, typename C>
__device__ __forceinline__ void stage_load(C* v, int t, const C* line) {
#pragma unroll
  for (int q = 0; q < E / R; ++q) {
    const int j = t + q * (N / E);
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = line[smem_pad(j + r * (N / R))];
  }
}

// Position of register v[q*R + r] for a first/last stage of radix R.
template <int N, int R, int E = FFT_E> __device__ __forceinline__ int reg_pos(int t, int idx) {
  return t + (idx / R) * (N / E) + (idx % R) * (N / R);
}

// Radix of stage s of an N-point transform in direction DIR (E per thread).
template <int N, int DIR, int E = FFT_E> __host__ __device__ constexpr int stage_radix(int s) {
  return (Sched<N, E>::REM > 1)
             ? ((DIR > 0) ? (s == 0 ? Sched<N, E>::REM : E) : (s == Sched<N, E>::NSTAGES - 1 ? Sched<N, E>::REM : E))
             : E;
}

// Full transform of one line.  On entry v[] holds the first stage's read
// pattern; on exit v[] holds the result in the last stage's pattern.
// `line` is this line's shared-memory buffer.  Every thread of the block
// must call this: it contains __syncthreads().
template <int N, int DIR, int E, int S> struct StageNS {  // product of the radices of stages 0..S-1
  static constexpr int value = stage_radix<N, DIR, E>(S - 1) * StageNS<N, DIR, E, S - 1>::value;
};
template <int N, int DIR, int E> struct StageNS<N, DIR, E, 0> { static constexpr int value = 1; };

// Stages S..NST-1 of a transform: exchange through shared memory, then
// compute stage S in registers.
template <int N, int DIR, int E, int S, int NST> struct StagesFrom {
  template <typename C> static __device__ __forceinline__ void run(C* v, int t, C* line, const C* __restrict__ tw) {
    if constexpr (S < NST) {
      constexpr int RP = stage_radix<N, DIR, E>(S - 1);
      constexpr int R = stage_radix<N, DIR, E>(S);
      constexpr int NSP = StageNS<N, DIR, E, S - 1>::value;
      constexpr int NS = StageNS<N, DIR, E, S>::value;
      __syncthreads();
      stage_store<N, RP, NSP, E>(v, t, line);
      __syncthreads();
      stage_load<N, R, E>(v, t, line);
      stage_compute<N, R, NS, DIR, E>(v, t, tw);
      StagesFrom<N, DIR, E, S + 1, NST>::run(v, t, line, tw);
    }
  }
};

// Full transform of one line.  On entry v[] holds the first stage's read
// pattern; on exit v[] holds the result in the last stage's pattern.
// `line` is this line's shared-memory buffer.  Every thread of the block
// must call this: it contains __syncthreads().
template <int N, int DIR, int E = FFT_E, typename C>
__device__ __forceinline__ void fft_line(C* v, int t, C* line, const C* __restrict__ tw) {
  constexpr int NST = Sched<N, E>::NSTAGES;
  static_assert(NST >= 1 && NST <= 6, "unsupported FFT length / values per thread");
  constexpr int R0 = stage_radix<N, DIR, E>(0);
  stage_compute<N, R0, 1, DIR, E>(v, t, tw);
  StagesFrom<N, DIR, E, 1, NST>::run(v, t, line, tw);
}

// ---------------------------------------------------------------------------
// Mirror-paired last stage.  When the last stage of a forward transform has
// a radix R < E (a remainder stage), each thread holds E/R >= 2 of its
// butterflies, and they can be chosen so that a thread holds both X[p] and
// X[N - p] for every output p it holds: butterfly j's outputs are
// j + r B (B = N/R) and N - (j + r B) = (B - j) + (R - 1 - r) B, so j and
// B - j are paired (0 with B/2, each of which mirrors itself).  Thread t
// holds j = t + q TPL for q < m (m = E/(2R)) in slots q, and their partners
// in slots q + m.  The row pass then separates the two rows' spectra of a
// packed transform in registers instead of through shared memory.
template <int N, int E> struct MirrorLast {
  static constexpr int R = Sched<N, E>::REM;
  static constexpr bool ok = R > 1 && E / R >= 2;
  static constexpr int B = N / (R > 1 ? R : 1), TPL = N / E, M = E / (2 * (R > 1 ? R : 1));
};
template <int N, int E> __device__ __forceinline__ int mirror_butterfly(int t, int q) {
  constexpr int B = MirrorLast<N, E>::B, TPL = MirrorLast<N, E>::TPL, M = MirrorLast<N, E>::M;
  if (q < M) return t + q * TPL;
  const int jl = t + (q - M) * TPL;
  return jl == 0 ? B / 2 : B - jl;
}

// Forward transform (DIR = -1) of one line whose last (remainder) stage runs
// on the mirror-paired butterflies: on exit v[q R + r] holds X at position
// mirror_butterfly(t, q) + r B.  Every thread of the block must call this.
template <int N, int E = FFT_E, typename C>
__device__ __forceinline__ void fft_line_mirror_last(C* v, int t, C* line, const C* __restrict__ tw) {
  constexpr int DIR = -1;
  constexpr int NST = Sched<N, E>::NSTAGES;
  constexpr int R = MirrorLast<N, E>::R, B = MirrorLast<N, E>::B;
  static_assert(MirrorLast<N, E>::ok && NST >= 2, "mirror-paired last stage needs a remainder stage");
  static_assert(stage_radix<N, DIR, E>(NST - 1) == R, "the forward transform's remainder stage is its last");
  constexpr int R0 = stage_radix<N, DIR, E>(0);
  stage_compute<N, R0, 1, DIR, E>(v, t, tw);
  StagesFrom<N, DIR, E, 1, NST - 1>::run(v, t, line, tw);
  constexpr int RP = stage_radix<N, DIR, E>(NST - 2);
  constexpr int NSP = StageNS<N, DIR, E, NST - 2>::value;
  constexpr int NS = StageNS<N, DIR, E, NST - 1>::value;
  static_assert(NS == B, "the last stage's sub-transform size");
  __syncthreads();
  stage_store<N, RP, NSP, E>(v, t, line);
  __syncthreads();
#pragma unroll
  for (int q = 0; q < E / R; ++q) {
    const int j = mirror_butterfly<N, E>(t, q);
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = line[smem_pad(j + r * B)];
    // twiddles w^(r j) (k = j mod NS = j), then the radix-R DFT; outputs at j + r B
    if constexpr ((R == 8) && sizeof(C) == 8) {
      TwiddledDFT<R, DIR, C>::run(v + q * R, tw, j);
    } else {
#pragma unroll
      for (int r = 1; r < R; ++r) v[q * R + r] = cmul_tw<DIR>(v[q * R + r], ldtw(tw, r * j));
      DFT<R, DIR, C>::run(v + q * R);
    }
  }
}

template <int N, int DIR, int E = FFT_E> struct FirstRadix {
  static constexpr int value = (Sched<N, E>::REM > 1 && DIR > 0) ? Sched<N, E>::REM : E;
};
template <int N, int DIR, int E = FFT_E> struct LastRadix {
  static constexpr int value = (Sched<N, E>::REM > 1 && DIR < 0) ? Sched<N, E>::REM : E;
};

}  // namespace ptf
