// Pass kernels of the tracer advection-diffusion right-hand side (2D and 3D).
//
// Spectral arrays are [nz][ny][pitch] complex with kr fastest (the layout of
// the reference's (nkr, nl[, nm]) column-major arrays, padded to `pitch`),
// rows interleaved in small groups (spec_index below);
// physical arrays are [nz][ny][nx] real, x fastest (nz = 1 in 2D).  One RHS
// evaluation (calcN!, src/traceradvectiondiffusion.jl:756-786) is split into
// passes along one axis each:
//
//   column pass: along y (2D) or z (3D): forward FFT of the previous pass's
//       output, the time-stepper stage combination with the linear
//       operator, then the inverse FFTs of the next stage input s and of
//       i*k_axis*s -> A, B.  The same kernel, in other modes, is the 3D
//       y-forward pass and the 3D y-inverse pass (three outputs).
//   row pass (x): per pair of rows, one inverse x-FFT of the two rows' i kr A
//       (Hermitian-extended, packed as row 0 + i row 1) gives c_x of both
//       rows, one of B gives c_y (in 3D one of C gives c_z), then the
//       products n = -(u.grad c) of the two rows form one forward x-FFT of
//       n_y0 + i n_y1, separated into the two rows' half spectra.
//
// The flow passed to the row pass is pre-scaled by -1/(2 N) (N = grid
// points): that folds the inverse normalisation, the minus sign and the 1/2
// of the two-for-one separation into the product.
#pragma once
#include "ptf_fft.cuh"
#include "ptf_tma.cuh"

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

enum FlowKind : int { FLOW_ARRAYS = 0, FLOW_CELLULAR = 1 };

// Spectral layout.  A field is `rows` (the flat (z, y) index) by `pitch`
// complex values, its rows interleaved in groups of 2^ylog: element (r, k)
// sits at (((r >> ylog) * pitch + k) << ylog) + (r & (2^ylog - 1)).  ylog = 0
// is the plain [rows][pitch] layout.  With ylog >= 1 the two rows of a row
// pair are adjacent (one 16-byte access serves both in FP32), and a column
// pass block of W columns moves runs of W * 2^ylog values instead of W.
__host__ __device__ __forceinline__ long long spec_row_base(long long r, int pitch, int ylog) {
  return (((r >> ylog) * (long long)pitch) << ylog) + (r & ((1LL << ylog) - 1));
}
__host__ __device__ __forceinline__ long long spec_index(long long r, long long k, int pitch, int ylog) {
  return spec_row_base(r, pitch, ylog) + (k << ylog);
}

// Register order.  The fields only the main column pass touches -- the
// stepper state (sol, stage input, accumulator) and the tables (L, ETDRK4
// coefficients, filter) -- are stored in the order the pass holds them:
// for column c (2D: kr; 3D: the in-plane offset) and position p along the
// line, held by thread t in register i (p = t + (i / RF) TPL + (i % RF) n / RF,
// the last forward stage's pattern), at (((c >> pl) n + i TPL + t) << pl) +
// (c & (2^pl - 1)).  A warp's access of one register is then one contiguous
// run, whatever the columns per block.  pl = 2 in FP32, 1 in FP64.
struct SpecMap {
  int pitch = 0, ylog = 0;      // rows interleaved in groups of 2^ylog (spec_index)
  int priv = 0;                 // 1: register order of the main column pass
  int n = 0, tpl = 0, rf = 0;   // main pass: line length, threads per line, last forward radix
  int pl = 0;                   // log2 columns per register-order group
  int ny = 0, three = 0;        // 3D: the main pass runs along z over planes of ny rows
};
__host__ __device__ __forceinline__ long long priv_index(const SpecMap& m, long long p, long long c) {
  const int t = (int)(p % m.tpl);
  const int rest = (int)(p - t), nr = m.n / m.rf;
  const int i = ((rest % nr) / m.tpl) * m.rf + rest / nr;
  return ((((c >> m.pl) * m.n) + (long long)i * m.tpl + t) << m.pl) + (c & ((1LL << m.pl) - 1));
}
// Element (row r of a solve, bin k) under map m.
__host__ __device__ __forceinline__ long long spec_map(const SpecMap& m, long long r, long long k) {
  if (!m.priv) return spec_index(r, k, m.pitch, m.ylog);
  if (m.three) return priv_index(m, r / m.ny, spec_index(r % m.ny, k, m.pitch, m.ylog));
  return priv_index(m, r, k);
}

// Per-solve parameters of the batched form (one entry per slot of a bucket
// of equally sized square 2D solves).  The clock (t, step) advances on the
// device after every step; a solve that reaches nsteps is deactivated and
// its state is no longer written.
template <typename T> struct SlotParams {
  double t;                 // clock.t at the start of the current step
  double dtd;               // dt in FP64 (the clock advances by it)
  long long step, nsteps;   // clock.step and the solve's target
  T kappa, eta, kappah;     // L = -(kappa kr^2 + eta l^2 + kappah |k|^(2 nkappah))
  T dt;
  T dkx, dky;               // 2 pi / Lx, 2 pi / Ly
  T U, eps, omega;          // FLOW_CELLULAR: psi = U cos(Kx x + eps sin(omega t)) cos(Ky y)
  int nkappah, active, flow_kind, time_mode;
  int Kx, Ky;
  // FLOW_CELLULAR: cos and sin of the phase eps sin(omega te) at the stage
  // times te = t + c dt, c = 0, 1/2, 1 (all at t in clock.t mode); set by
  // slot_phases whenever t changes, so the passes evaluate no trigonometry
  T ph_c[3], ph_s[3];
};

__device__ __forceinline__ void sin_cos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sin_cos(float x, float* s, float* c) { sincosf(x, s, c); }
template <typename T> __device__ __forceinline__ void slot_phases(SlotParams<T>& sp) {
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const double te = sp.t + (sp.time_mode ? 0.5 * q * (double)sp.dt : 0.0);
    const T phi = sp.eps * (T)sin((double)sp.omega * te);
    sin_cos(phi, &sp.ph_s[q], &sp.ph_c[q]);
  }
}

template <typename T> struct ColArgs {
  typedef typename cplx_of<T>::type C;
  const C* nxin;   // forward input
  C* s;            // state (sol); COL_YINV3: the z-inverse Z1
  C* si;           // RK4: current stage input; ETDRK4: d = E2 a - zeta N(sol)
  C* acc;          // accumulator of the update
  C* slo;          // FP32 compensated state: the low part of s (null: s alone; see stage_combine)
  const T* filt;   // filtered steppers: the spectral filter the new state is multiplied by (null: none)
  C* A;            // F^-1(s_next)
  C* B;            // F^-1(i k s_next)
  C* Cout;         // COL_YINV3: F^-1(z2in)
  const C* z2in;   // COL_YINV3: the z-inverse Z2
  C* nout;         // COL_FWD_N output
  const C* tw;     // transform-length twiddles
  const T* Ltab;   // linear operator, one value per spectral element
  const T* coef;   // ETDRK4 tables E, E2, zeta, alpha, beta, gamma, `tplane` apart
  T dt, dk;        // dk: 2*pi/L of the transform axis
  int stride;      // elements between consecutive points of a line (the row pitch when ylog > 0)
  int ylog;        // spectral layout (spec_index): lines along the interleaved row axis
  int priv;        // 1: s, si, acc and the tables are in register order (SpecMap)
  int mode, do_inverse;
  long long bstride;    // elements between blockIdx.y blocks of fields
  long long tplane;     // elements of one table plane
  int tab_per_block;    // 1: tables advance with blockIdx.y (per-solve tables)
  // batched form only: per-slot parameters, the slots to process
  // (slot_list[k], k < nslots) and columns per slot
  const SlotParams<T>* slots;
  const int* slot_list;
  int nslots, slot_cols;
  // FP64 k = 0 mode (FP32 handles, main column pass): per-solve FP64 state
  // {s, stage input (ETDRK4: d), acc, -} of the (0,0[,0]) mode and its FP64
  // coefficients {L, E, E2, zeta, alpha, beta, gamma}; null when off.
  // Batched form: {s, stage input, acc, L(0,0)} per slot of the bucket
  // (RK4 needs no other coefficient; dt comes from the slot), k0c unused.
  double* k0;
  const double* k0c;
  double dt64;
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
  int ylog;        // spectral layout of A, B, Cin, out (spec_index)
  int park_slots;  // parking slots per point: 1 (2D) or 2 (3D)
  long long bstride, pstride, fstride;
  // batched form only
  const SlotParams<T>* slots;
  const int* slot_list;
  int nslots;
  T stage_c;       // stage time offset in units of dt (0, 1/2, 1/2, 1 for RK4)
  T fscale;        // analytic flow scale: -1/(2 nx ny)
  int* err;        // device error flag (bounded waits that ran out)
  int tma;         // 1: ROW_RHS stages its rows in shared memory with bulk copies
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
// FP32 column blocks: up to 512 threads at 128 registers each -- two blocks
// of 256 threads (4 columns of 1024) or one of 512 (8 columns: 64-byte row
// segments, which DRAM serves markedly better than 32-byte ones; measured 5%
// faster per 1024-point column launch, and 2 instead of 1 column per block
// at 4096).  The register budget is the same for both shapes; the tuner picks.
#ifndef PTF_COL_MINB_F32
#define PTF_COL_MINB_F32 1
#endif
#ifndef PTF_COL_MINB_F64
#define PTF_COL_MINB_F64 1
#endif
#ifndef PTF_COL_THREADS_F32
#define PTF_COL_THREADS_F32 512
#endif
#ifndef PTF_EARLY_OPERAND
#define PTF_EARLY_OPERAND 1  // fetch a stage operand ahead with cp.async (see col_body)
#endif
template <typename T> struct ColBounds { static constexpr int threads = 256, blocks = PTF_COL_MINB_F64; };
template <> struct ColBounds<float> { static constexpr int threads = PTF_COL_THREADS_F32, blocks = PTF_COL_MINB_F32; };

// Dynamic shared memory of a column-pass block with W lines: the W FFT
// lines, then a private slot array holding each thread's next stage input
// between the two inverse transforms.
template <typename T, int N> __host__ __device__ constexpr size_t col_smem_bytes(int W) {
  return (size_t)W * (line_stride(N) + N) * sizeof(typename cplx_of<T>::type);
}
// The stepper's last stage parks one more operand (the state, for the
// compensated sum): its blocks take a second slot array.
__host__ __device__ constexpr bool col_second_park(int mode) { return mode == COL_RK4_4 || mode == COL_ETD_4; }
template <typename T, int N> __host__ __device__ constexpr size_t col_smem_bytes_mode(int W, int mode) {
  return col_smem_bytes<T, N>(W) + (col_second_park(mode) ? (size_t)W * N * sizeof(typename cplx_of<T>::type) : 0);
}
// Values per thread of the column pass (may differ from the row pass's: the
// column pass is bound by latency, the row pass by shared-memory traffic).
#ifndef PTF_COL_E_F32
#define PTF_COL_E_F32 16
#endif
template <typename T, int N> struct ColE { static constexpr int value = PassE<T, N>::value; };
template <int N> struct ColE<float, N> { static constexpr int value = N >= 256 ? PTF_COL_E_F32 : PassE<float, N>::value; };
// threads per line: row pass (pass_tpl) and column pass (col_tpl)
template <typename T, int N> __host__ __device__ constexpr int pass_tpl() { return N / PassE<T, N>::value; }
template <typename T, int N> __host__ __device__ constexpr int col_tpl() { return N / ColE<T, N>::value; }
// Largest spectral layout (ylog) a column pass of length N can address with
// per-register row offsets (all multiples of col_tpl): 2 (rows in fours),
// less for N < 64.
template <typename T, int N> __host__ __device__ constexpr int col_ylog_max() {
  return col_tpl<T, N>() >= 4 ? 2 : col_tpl<T, N>() >= 2 ? 1 : 0;
}

// Compensated FP64 sum of the real parts of column 0 of a column-pass block
// (lines w = 0: threads t*W, registers v[0..E)), returned in thread 0.  Uses
// the line buffer of line 0 (before the forward transform touches it).
template <typename T, typename C, int E, int TPL>
__device__ __forceinline__ double column0_sum(const C* v, int w, int t, C* line0) {
  double* part = reinterpret_cast<double*>(line0);  // TPL doubles fit in N complex values
  if (w == 0) {
    double s = 0, c = 0;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const double y = (double)v[i].x - c;
      const double u = s + y;
      c = (u - s) - y;
      s = u;
    }
    part[t] = s;
  }
  __syncthreads();
  double tot = 0;
  if (threadIdx.x < 32) {
    double c = 0;
    for (int k = threadIdx.x; k < TPL; k += 32) {
      const double y = part[k] - c;
      const double u = tot + y;
      c = (u - tot) - y;
      tot = u;
    }
    for (int off = 16; off > 0; off /= 2) tot += __shfl_xor_sync(0xffffffffu, tot, off);
  }
  __syncthreads();
  return tot;
}

// The same sum for the batched form, where a block's W lines run over the
// columns of several slots: every line holding column 0 of its slot (`mine`,
// uniform along the line) sums its E values per thread, then the line's
// thread t = 0 (which owns position 0) adds the TPL partials, compensated.
// Returned in that thread; every thread of the block must call this.
template <typename T, typename C, int E, int TPL>
__device__ __forceinline__ double column0_sum_lines(const C* v, int w, int t, bool mine, C* sm) {
  double* part = reinterpret_cast<double*>(sm);  // W*TPL doubles fit in the W lines
  if (mine) {
    double s = 0, c = 0;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const double y = (double)v[i].x - c;
      const double u = s + y;
      c = (u - s) - y;
      s = u;
    }
    part[w * TPL + t] = s;
  }
  __syncthreads();
  double tot = 0;
  if (mine && t == 0) {
    double c = 0;
    for (int k = 0; k < TPL; ++k) {
      const double y = part[w * TPL + k] - c;
      const double u = tot + y;
      c = (u - tot) - y;
      tot = u;
    }
  }
  __syncthreads();
  return tot;
}

// Stepper stage combination at one spectral element o (FourierFlows RK4;
// Cox-Matthews ETDRK4 with coefficient planes E - 1, E2 - 1, zeta, alpha,
// beta, gamma at cf[o + e*plane]: E = exp(L dt) and E2 = exp(L dt / 2) are
// held as expm1 values and applied as s + (E - 1) s, which keeps the
// relative accuracy of the small decay 1 - E of the slowly damped modes in
// an FP32 table -- rounding E itself near 1 to FP32 misstates that decay by
// up to several percent, an error that grows linearly with the steps).  Nh = the RHS transform N(stage input) here;
// returns the next stage input (or the new state after stage 4) and updates
// the state arrays S (sol), SI (RK4 stage input / ETDRK4 d = E2 a - zeta N(sol)),
// AC (accumulator).  RK4 stores only when `store` (batched slots); Lf() gives
// the linear operator at o.
// The operand of a stage combination the column pass fetches ahead into
// shared memory (cp.async, before the forward transform): 1 = S, 2 = SI,
// 3 = AC, 0 = none -- the first state operand each mode reads.
__host__ __device__ constexpr int early_operand(int mode) {
  return (mode == COL_RK4_1 || mode == COL_ETD_1 || mode == COL_ETD_2) ? 1
         : (mode == COL_RK4_2 || mode == COL_RK4_3 || mode == COL_RK4_4 || mode == COL_ETD_3) ? 2
         : (mode == COL_ETD_4) ? 3 : 0;
}

// hi + lo += d for a state held as a pair with hi = RN(hi + lo): Knuth's
// two-sum of hi and d, its error added to lo, then renormalised (Dekker's
// fast two-sum), so the pair stays canonical and round-trips through FP64.
template <typename T> __device__ __forceinline__ void add_compensated(T& hi, T& lo, T d) {
  const T t = hi + d;
  const T bp = t - hi;
  const T err = (hi - (t - bp)) + (d - bp);
  const T l = lo + err;
  hi = t + l;
  lo = l - (hi - t);
}

// SLO non-null (FP32 handles): the state is the pair s + s_lo, AC holds only
// the step's increment (not s plus it), and the last stage adds the
// increment to the pair with add_compensated.  Rounding the state to FP32
// then no longer costs half an ulp of s every step: over the 1000 ETDRK4
// steps of the 1024^2 cellular workload that rounding, fed back through the
// FP32 transforms, was most of the FP32 error against the FP64 oracle
// (NumPy emulation: 1.1e-5 with an FP32 state, 2.0e-6 with an FP64 one).
template <typename T, int MODE, int PF = 0, bool PS = false, typename C, typename LF>
__device__ __forceinline__ C stage_combine(const C Nh, int o, C* __restrict__ S, C* __restrict__ SI,
                                           C* __restrict__ AC, const T* __restrict__ cf,
                                           size_t plane, T dt, bool store, LF&& Lf,
                                           const T* __restrict__ filt = nullptr, C pre = C(),
                                           C* __restrict__ SLO = nullptr, C pre_s = C()) {
  // PS: the state at o was fetched ahead too (compensated last stage): pre_s
  // PF != 0: operand early_operand(MODE) was fetched ahead; its value is `pre`
  auto ldS = [&]() { return PF == 1 ? pre : S[o]; };
  auto ldSI = [&]() { return PF == 2 ? pre : SI[o]; };
  auto ldAC = [&]() { return PF == 3 ? pre : AC[o]; };
  const bool comp = SLO != nullptr;
  // the new state from d (last stage): s + d as a compensated pair, or d
  // itself (AC carried s), then the filter
  auto finish = [&](C d) -> C {
    C hi;
    if (comp) {
      hi = PS ? pre_s : S[o];
      C lo = SLO[o];
      add_compensated(hi.x, lo.x, d.x);
      add_compensated(hi.y, lo.y, d.y);
      if (filt) {
        // scale both parts, then renormalise (fast two-sum) so the pair stays canonical
        const T f = filt[o];
        C h, l;
        h.x = hi.x * f; h.y = hi.y * f;
        l.x = lo.x * f; l.y = lo.y * f;
        hi.x = h.x + l.x; hi.y = h.y + l.y;
        lo.x = l.x - (hi.x - h.x); lo.y = l.y - (hi.y - h.y);
      }
      if (store) SLO[o] = lo;
    } else {
      hi = d;
      if (filt) { const T f = filt[o]; hi.x *= f; hi.y *= f; }
    }
    if (store) S[o] = hi;
    return hi;
  };
  C x;
  if (MODE == COL_RK4_1) {
    const T L = Lf();
    const C s = ldS();
    C k; k.x = L * s.x + Nh.x; k.y = L * s.y + Nh.y;
    C ac;
    if (comp) { ac.x = (dt / 6) * k.x; ac.y = (dt / 6) * k.y; }
    else { ac.x = s.x + (dt / 6) * k.x; ac.y = s.y + (dt / 6) * k.y; }
    x.x = s.x + (dt / 2) * k.x; x.y = s.y + (dt / 2) * k.y;
    if (store) { AC[o] = ac; SI[o] = x; }
  } else if (MODE == COL_RK4_2 || MODE == COL_RK4_3) {
    const T L = Lf();
    const C si = ldSI(), s = ldS();
    C ac = ldAC();
    C k; k.x = L * si.x + Nh.x; k.y = L * si.y + Nh.y;
    ac.x += (dt / 3) * k.x; ac.y += (dt / 3) * k.y;
    const T h = (MODE == COL_RK4_2) ? dt / 2 : dt;
    x.x = s.x + h * k.x; x.y = s.y + h * k.y;
    if (store) { AC[o] = ac; SI[o] = x; }
  } else if (MODE == COL_RK4_4) {
    const T L = Lf();
    const C si = ldSI(), ac = ldAC();
    C k; k.x = L * si.x + Nh.x; k.y = L * si.y + Nh.y;
    C d; d.x = ac.x + (dt / 6) * k.x; d.y = ac.y + (dt / 6) * k.y;
    x = finish(d);
  } else if (MODE == COL_ETD_1) {
    // a = E2 s + zeta N(s) is the next input; stage 3's
    // c = E2 a + zeta (2 N(b) - N(s)) = d + 2 zeta N(b) needs only
    // d = E2 a - zeta N(s), stored in SI in place of a and N(s)
    const T Em = cf[o], E2m = cf[o + plane], ze = cf[o + 2 * plane], al = cf[o + 3 * plane];
    const C s = ldS();
    C ac;
    if (comp) { ac.x = Em * s.x + al * Nh.x; ac.y = Em * s.y + al * Nh.y; }
    else { ac.x = (s.x + Em * s.x) + al * Nh.x; ac.y = (s.y + Em * s.y) + al * Nh.y; }
    AC[o] = ac;
    x.x = (s.x + E2m * s.x) + ze * Nh.x; x.y = (s.y + E2m * s.y) + ze * Nh.y;
    C d; d.x = (x.x + E2m * x.x) - ze * Nh.x; d.y = (x.y + E2m * x.y) - ze * Nh.y;
    SI[o] = d;
  } else if (MODE == COL_ETD_2) {
    const T E2m = cf[o + plane], ze = cf[o + 2 * plane], be = cf[o + 4 * plane];
    const C s = ldS();
    C ac = ldAC();
    ac.x += 2 * be * Nh.x; ac.y += 2 * be * Nh.y;
    AC[o] = ac;
    x.x = (s.x + E2m * s.x) + ze * Nh.x; x.y = (s.y + E2m * s.y) + ze * Nh.y;
  } else if (MODE == COL_ETD_3) {
    const T ze = cf[o + 2 * plane], be = cf[o + 4 * plane];
    const C d = ldSI();
    C ac = ldAC();
    ac.x += 2 * be * Nh.x; ac.y += 2 * be * Nh.y;
    AC[o] = ac;
    x.x = d.x + 2 * ze * Nh.x; x.y = d.y + 2 * ze * Nh.y;
  } else {  // COL_ETD_4
    const T ga = cf[o + 5 * plane];
    const C ac = ldAC();
    C d; d.x = ac.x + ga * Nh.x; d.y = ac.y + ga * Nh.y;
    x = finish(d);
  }
  return x;
}

// The stage combination of the (0,0[,0]) mode in FP64 (FP32 handles): q =
// {s, stage input (ETDRK4: d), acc, unused} of one solve, kc = {L, E, E2, zeta, alpha, beta,
// gamma} at that mode, Nd = N there.  Returns the next stage input (the new
// state after stage 4).  Same formulas as stage_combine.
template <int MODE>
__device__ __forceinline__ double k0_combine(double* q, const double* kc, double dd, double Nd) {
  double xd = q[0];
  if (MODE == COL_RK4_1) {
    const double k = kc[0] * q[0] + Nd;
    q[2] = q[0] + dd / 6 * k; xd = q[0] + dd / 2 * k; q[1] = xd;
  } else if (MODE == COL_RK4_2 || MODE == COL_RK4_3) {
    const double k = kc[0] * q[1] + Nd;
    q[2] += dd / 3 * k; xd = q[0] + (MODE == COL_RK4_2 ? dd / 2 : dd) * k; q[1] = xd;
  } else if (MODE == COL_RK4_4) {
    const double k = kc[0] * q[1] + Nd;
    xd = q[2] + dd / 6 * k; q[0] = xd;
  } else if (MODE == COL_ETD_1) {
    q[2] = kc[1] * q[0] + kc[4] * Nd; xd = kc[2] * q[0] + kc[3] * Nd; q[1] = kc[2] * xd - kc[3] * Nd;
  } else if (MODE == COL_ETD_2) {
    q[2] += 2 * kc[5] * Nd; xd = kc[2] * q[0] + kc[3] * Nd;
  } else if (MODE == COL_ETD_3) {
    q[2] += 2 * kc[5] * Nd; xd = q[1] + 2 * kc[3] * Nd;
  } else if (MODE == COL_ETD_4) {
    xd = q[2] + kc[6] * Nd; q[0] = xd;
  }
  return xd;  // COL_FWD_STORE: the seeded state
}

// Body of one column-pass block (tile = column tile index, blk = block of
// fields).  BATCHED: flat columns run over the slots of a bucket, each
// thread carries its own slot; the linear operator and dt come from the
// slot's parameters, and inactive slots are not written.
template <typename T, int N, int MODE, bool BATCHED, int CSTRIDE = 0>
__device__ __forceinline__ void col_body(const ColArgs<T>& a, int tile, int blk, unsigned char* smem_raw) {
  typedef typename cplx_of<T>::type C;
  static_assert(!BATCHED || MODE < COL_ETD_1 || MODE >= COL_FWD_N, "the batched form runs RK4");
  constexpr int E = ColE<T, N>::value;
  constexpr int TPL = N / E;
  constexpr int LS = line_stride(N);
  constexpr int RF0 = FirstRadix<N, -1, E>::value;  // forward input pattern
  constexpr int RF = LastRadix<N, -1, E>::value;    // forward output pattern
  constexpr int RI = FirstRadix<N, +1, E>::value;   // inverse input pattern (== RF)
  constexpr int RO = LastRadix<N, +1, E>::value;    // inverse output pattern
  static_assert(RF == RI, "forward-last and inverse-first radices must match");
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int W = blockDim.x / TPL;
  const int w = threadIdx.x % W, t = threadIdx.x / W;
  int col = tile * W + w;
  // CSTRIDE != 0: the row pitch known at compile time (square grids), so
  // the per-register offsets below become immediate offsets of the loads
  const int stride = CSTRIDE ? CSTRIDE : a.stride;
  size_t boff = (size_t)blk * (size_t)a.bstride;
  bool store = true;
  T dt = a.dt;
  int slot = 0;
  if (BATCHED) {
    int k = col / a.slot_cols;
    col -= k * a.slot_cols;
    store = k < a.nslots;
    if (!store) k = a.nslots - 1;  // keep loads in bounds; nothing is written
    slot = a.slot_list[k];
    store = store && a.slots[slot].active;
    dt = a.slots[slot].dt;
    boff = (size_t)slot * (size_t)a.bstride;
  }
  // table plane: compile-time too for the stage modes of a square 2D grid
  constexpr bool STAGE = MODE >= COL_RK4_1 && MODE <= COL_ETD_4;
  const size_t plane = (CSTRIDE && STAGE) ? (size_t)N * CSTRIDE : (size_t)a.tplane;
  const size_t toff = a.tab_per_block ? (size_t)blk * plane : 0;
  C* line = sm + w * LS;
  C* park = sm + W * LS;  // slot i of this thread: park[i*blockDim + tid]
  const int nthr = blockDim.x;
  // this thread's offset inside one field: element (row t, column col) of
  // the layout (spec_index); every register's row offset below is a multiple
  // of TPL >= 2^ylog (the launcher checks), so it adds (offset * stride)
  const int yl = a.ylog;
  const int tb = (((t >> yl) * stride + col) << yl) + (t & ((1 << yl) - 1));
  // register order of the private fields (SpecMap): column groups of 2^PL
  constexpr int PL = sizeof(T) == 4 ? 2 : 1;
  const bool priv = a.priv != 0;
  const int pb = (((col >> PL) * N + t) << PL) + (col & ((1 << PL) - 1));
  // offset of register i for a first/last stage of radix R
#define PTF_OFF(R, i) (tb + (((i) / (R)) * TPL + ((i) % (R)) * (N / (R))) * stride)
  // a private field's register i (last forward stage pattern)
#define PTF_POFF(i) (priv ? pb + (i) * (TPL << PL) : PTF_OFF(RF, i))

  constexpr bool K0MODE = (MODE >= COL_RK4_1 && MODE <= COL_ETD_4) || MODE == COL_FWD_STORE;
  const bool k0blk = !BATCHED && K0MODE && a.k0 != nullptr && tile == 0;  // uniform across the block
  // batched form: a.k0 holds {s, stage input, acc, L(0,0)} per slot of the bucket
  const bool k0bat = BATCHED && K0MODE && a.k0 != nullptr;  // uniform across the block
  double k0N = 0;
  // the combination's first state operand, fetched into this thread's park
  // slots while the forward transform runs (the slots are free until the
  // combination writes the next stage input there)
  // (batched form too: a thread of an inactive slot fetches from a valid
  // slot, in bounds, and writes nothing)
#ifndef PTF_EARLY_OPERAND_BATCHED
#define PTF_EARLY_OPERAND_BATCHED 1
#endif
  constexpr int PF = (PTF_EARLY_OPERAND && (!BATCHED || PTF_EARLY_OPERAND_BATCHED)) ? early_operand(MODE) : 0;
  // the compensated last stage also reads the state: fetched into a second
  // slot array (single-solve form; col_smem_bytes_mode sizes it)
  constexpr bool PS2 = PF != 0 && !BATCHED && col_second_park(MODE);
  C* park2 = park + W * N;
  const bool ps = PS2 && a.slo != nullptr;  // uniform across the block
  if (PF) {
    const C* __restrict__ op = (PF == 1 ? a.s : PF == 2 ? a.si : a.acc) + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) cp_async<sizeof(C)>(park + i * nthr + threadIdx.x, op + PTF_POFF(i));
    if (PS2 && ps) {
      const C* __restrict__ sp = a.s + boff;
#pragma unroll
      for (int i = 0; i < E; ++i) cp_async<sizeof(C)>(park2 + i * nthr + threadIdx.x, sp + PTF_POFF(i));
    }
    cp_async_commit();
  }
  C v[E];
  if (MODE != COL_PROLOGUE && MODE != COL_YINV3) {
    const C* __restrict__ src = a.nxin + boff;
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = src[PTF_OFF(RF0, i)];
    // FP64 k = 0 mode: N(0,0) is the sum of column 0 (the kr = 0 bins of
    // the rows, real), taken here as a compensated FP64 sum instead of from
    // the FP32 transform; it lands in thread 0, which owns position 0.
    if (k0blk && MODE != COL_FWD_STORE) k0N = column0_sum<T, C, E, TPL>(v, w, t, sm);
    if (k0bat && MODE != COL_FWD_STORE) k0N = column0_sum_lines<T, C, E, TPL>(v, w, t, store && col == 0, sm);
    fft_line<N, -1, E>(v, t, line, a.tw);
  }
  // column 0, t = 0: position p = 0 is its register 0
  const bool k0thr = (k0blk && threadIdx.x == 0) || (k0bat && store && col == 0 && t == 0);

  // Stage combination at the positions p = reg_pos<N, RF, E>(t, i); the
  // next stage input is parked (each thread reads back only its own slots,
  // so no barrier is needed).
  // Linear operator: table, or (batched) from the slot's parameters.
  T Lk2 = 0, Lka = 0, Lkb = 0, Lkh = 0;
  int Lnh = 0;
  if (BATCHED) {
    const SlotParams<T>& sp = a.slots[slot];
    const T kr = (T)col * sp.dkx;
    Lk2 = kr * kr; Lka = sp.kappa; Lkb = sp.eta; Lkh = sp.kappah; Lnh = sp.nkappah;
  }
  auto Lval = [&](const T* Lt, int o, int i) -> T {
    if (!BATCHED) return Lt[o];
    const T l = kval<T, N>(reg_pos<N, RF, E>(t, i), a.slots[slot].dky);
    const T l2 = l * l;
    T hyp = 0;
    if (Lkh != 0) { const T K2 = Lk2 + l2; hyp = Lkh; for (int q = 0; q < Lnh; ++q) hyp *= K2; }
    return -(Lka * Lk2 + Lkb * l2 + hyp);
  };
  {
    C* __restrict__ S = a.s + boff;
    C* __restrict__ SI = a.si + boff;
    C* __restrict__ AC = a.acc + boff;
    C* __restrict__ SL = a.slo ? a.slo + boff : nullptr;  // compensated state (FP32)
    const T* __restrict__ Lt = a.Ltab + toff;
    const T* __restrict__ cf = a.coef + 6 * toff;
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int o = PTF_POFF(i);  // the private fields (state, tables)
      const C Nh = v[i];  // forward transform of the RHS at this element
      C x;
      if (MODE == COL_PROLOGUE || MODE == COL_YINV3) {
        x = S[o];
      } else if (MODE == COL_FWD_STORE) {
        x = Nh;
        if (store) {
          S[o] = x;
          if (SL) SL[o] = C();  // a new state: no low part
        }
      } else if (MODE == COL_FWD_N) {
        x = Nh; if (store) a.nout[boff + PTF_OFF(RF, i)] = Nh;  // an intermediate: spectral layout
      } else {
        if (PF && i == 0) cp_async_wait_all();
        auto lf = [&]() { return Lval(Lt, o, i); };
        if (PS2 && ps) {
          x = stage_combine<T, MODE, PF, true>(Nh, o, S, SI, AC, cf, plane, dt, store, lf,
                                               (!BATCHED && a.filt) ? a.filt + toff : nullptr,
                                               park[i * nthr + threadIdx.x], SL, park2[i * nthr + threadIdx.x]);
        } else {
          x = stage_combine<T, MODE, PF>(Nh, o, S, SI, AC, cf, plane, dt, store, lf,
                                         (!BATCHED && a.filt) ? a.filt + toff : nullptr,
                                         PF ? park[i * nthr + threadIdx.x] : C(), SL);
        }
      }
      if (k0thr && i == 0) {
        // the (0,0) mode in FP64: {s, stage input (ETDRK4: d), acc, -} of this solve
        double* q = a.k0 + (size_t)(BATCHED ? slot : blk) * 4;
        const double* kc = a.k0c;
        double dd = a.dt64;
        double kcs[7] = {0, 0, 0, 0, 0, 0, 0};
        if (BATCHED) {  // RK4: only L(0,0) enters, kept in the slot's fourth value; FP64 dt from the slot
          kcs[0] = q[3];
          kc = kcs;
          dd = a.slots[slot].dtd;
        }
        const double Nd = k0N;
        const double xd = k0_combine<MODE>(q, kc, dd, Nd);
        x.x = (T)xd; x.y = 0;
        if (MODE == COL_FWD_STORE || MODE == COL_RK4_4 || MODE == COL_ETD_4) {
          S[o] = x;
          if (SL) SL[o] = C();  // the FP64 mode is exact: no low part
        }
      }
      park[i * nthr + threadIdx.x] = x;
    }
  }
  if (MODE == COL_FWD_N || !a.do_inverse) return;  // uniform across the block

  // A = F^-1(s_next)
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = park[i * nthr + threadIdx.x];
  fft_line<N, +1, E>(v, t, line, a.tw);
  if (store) {
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
    const T k = kval<T, N>(reg_pos<N, RI, E>(t, i), BATCHED ? a.slots[slot].dky : a.dk);
    const C x = park[i * nthr + threadIdx.x];
    v[i].x = -k * x.y;
    v[i].y = k * x.x;
  }
  fft_line<N, +1, E>(v, t, line, a.tw);
  if (store) {
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
#undef PTF_POFF
}

template <typename T, int N, int MODE, int CSTRIDE = 0>
__global__ void __launch_bounds__(ColBounds<T>::threads, ColBounds<T>::blocks) col_pass_kernel(ColArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  col_body<T, N, MODE, false, CSTRIDE>(a, blockIdx.x, blockIdx.y, smem_raw);
}
// Row pitch of a square grid's half spectrum (nx/2 + 1 rounded up to 8).
template <int N> __host__ __device__ constexpr int square_pitch() { return ((N / 2 + 1 + 7) / 8) * 8; }

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
// Shared memory of a row-pass block with P pairs: one FFT line and
// `slots` parking slots per point of each pair (1 in 2D, 2 in 3D).
template <typename T, int NX> __host__ __device__ constexpr size_t row_smem_bytes(int P, int slots) {
  return (size_t)P * (line_stride(NX) + slots * NX) * sizeof(typename cplx_of<T>::type);
}

// exp(i K x_j) on the grid x_j = -L/2 + j L/n for an integer K:
// (-1)^K conj(tw[(K j) mod n]) with tw[m] = exp(-2 pi i m / n).
template <typename C>
__device__ __forceinline__ C grid_expi(const C* __restrict__ tw, int K, int j, int n) {
  // n is a power of two and |K j| < 2^31: the residue of K j mod n is a mask
  const int m = (K * j) & (n - 1);
  const C w = __ldg(tw + m);
  C r;
  r.x = w.x; r.y = -w.y;
  if (K & 1) { r.x = -r.x; r.y = -r.y; }
  return r;
}
// The scaled cellular flow psi = U cos(Kx x + eps sin(omega t)) cos(Ky y) of a
// slot at one row: u = -d(psi)/dy, v = d(psi)/dx, times fscale.
template <typename T> struct CellularRow {
  T cphi, sphi, au, av, sy, cy;
  int Kx;
};
template <typename T, typename C>
__device__ __forceinline__ CellularRow<T> cellular_row(const SlotParams<T>& sp, const C* tw, int yrow, int n,
                                                        T stage_c, T fscale) {
  CellularRow<T> r;
  const int q = stage_c < (T)0.25 ? 0 : stage_c < (T)0.75 ? 1 : 2;  // stage time t + stage_c dt (slot_phases)
  r.cphi = sp.ph_c[q];
  r.sphi = sp.ph_s[q];
  const C ey = grid_expi(tw, sp.Ky, yrow, n);
  r.cy = ey.x; r.sy = ey.y;
  const T kx = (T)sp.Kx * sp.dkx, ky = (T)sp.Ky * sp.dky;
  r.au = fscale * sp.U * ky;    // u =  U ky cos(kx x + phi) sin(ky y)
  r.av = -fscale * sp.U * kx;   // v = -U kx sin(kx x + phi) cos(ky y)
  r.Kx = sp.Kx;
  return r;
}
// The cellular flow at column x of a row pair: r describes row 0, (cy1, sy1)
// is row 1's y factor; the x factor is shared by both rows.
template <typename T, typename C>
__device__ __forceinline__ void cellular_uv2(const CellularRow<T>& r, T cy1, T sy1, const C* tw, int x, int n, T* u0,
                                             T* v0, T* u1, T* v1) {
  const C e = grid_expi(tw, r.Kx, x, n);
  const T ct = e.x * r.cphi - e.y * r.sphi, st = e.y * r.cphi + e.x * r.sphi;
  const T uc = r.au * ct, vs = r.av * st;
  *u0 = uc * r.sy;
  *v0 = vs * r.cy;
  *u1 = uc * sy1;
  *v1 = vs * cy1;
}

// Input of an inverse x transform of two rows at once: Z[k] = H0[k] + i H1[k],
// H_r the Hermitian extension of row r's half spectrum X_r = g Y_r with
// g = i kr (DERIV) or 1, the imaginary parts at the self-conjugate bins
// k = 0, NX/2 dropped (as a c2r transform does).  p, q = Y_0, Y_1 at
// min(k, NX - k).  Re of the result is row 0's field, Im row 1's.
template <bool DERIV, typename T, typename C>
__device__ __forceinline__ C zpair(C p, C q, int k, int NX, T dkx) {
  const int h = NX / 2;
  if (DERIV) {
    const T kr = (T)(k <= h ? k : NX - k) * dkx;
    C a, b;
    a.x = -kr * p.y; a.y = kr * p.x;
    b.x = -kr * q.y; b.y = kr * q.x;
    p = a; q = b;
  }
  C z;
  if (k == 0 || k == h) {
    z.x = p.x; z.y = q.x;
  } else if (k < h) {
    z.x = p.x - q.y; z.y = p.y + q.x;
  } else {  // conj(p) + i conj(q)
    z.x = p.x + q.y; z.y = q.x - p.y;
  }
  return z;
}

// Element `off` of both rows of a pair.  PAIRED: the rows are interleaved
// (spectral layout ylog >= 1), row 1's element follows row 0's, and an FP32
// pair is one 16-byte load.
template <bool PAIRED, typename C>
__device__ __forceinline__ void ld_pair(const C* __restrict__ r0, const C* __restrict__ r1, int off, C& x0, C& x1) {
  if constexpr (PAIRED && sizeof(C) == 8) {
    const float4 q = *reinterpret_cast<const float4*>(r0 + off);
    x0.x = q.x; x0.y = q.y; x1.x = q.z; x1.y = q.w;
  } else {
    x0 = r0[off];
    x1 = r1[off];
  }
}
template <bool PAIRED, typename C>
__device__ __forceinline__ void st_pair(C* r0, C* r1, int off, C x0, C x1) {
  if constexpr (PAIRED && sizeof(C) == 8) {
    *reinterpret_cast<float4*>(r0 + off) = make_float4(x0.x, x0.y, x1.x, x1.y);
  } else {
    r0[off] = x0;
    r1[off] = x1;
  }
}

// Body of one row-pass block (tile = pair tile index, blk = block of fields).
// The rows of a pair are transformed together: one inverse x transform gives
// c_x of both rows (Re, Im), a second c_y (and in 3D a third c_z), and the
// products -(u.grad c) of the two rows form the one forward transform.
// BATCHED: flat pairs run over the slots of a bucket; each thread carries
// its slot, whose flow is an array or the analytic cellular flow.
// PAIRED: the spectral layout interleaves rows (a.ylog >= 1).
template <typename T, int NX, bool BATCHED, bool PAIRED = false>
__device__ __forceinline__ void row_body(const RowArgs<T>& a, int tile, int blk, unsigned char* smem_raw) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = PassE<T, NX>::value;
  constexpr int TPL = NX / E;
  constexpr int LS = line_stride(NX);
  constexpr int RI0 = FirstRadix<NX, +1, E>::value;
  constexpr int RIL = LastRadix<NX, +1, E>::value;   // == E
  constexpr int RF0 = FirstRadix<NX, -1, E>::value;  // == E
  constexpr int RFL = LastRadix<NX, -1, E>::value;
  static_assert(RIL == RF0, "inverse-last and forward-first radices must match");
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int P = blockDim.x / TPL;
  const int pr = threadIdx.x / TPL, t = threadIdx.x % TPL;
  int y0 = 2 * (tile * P + pr);
  long long boff = (long long)blk * a.bstride;
  long long poff = (long long)blk * a.pstride;
  long long foff = (long long)blk * a.fstride;
  bool valid = y0 < a.rows;  // grids are sized exactly; kept for safety
  int slot = 0;
  if (BATCHED) {
    const int pair = y0 / 2, pps = a.rows / 2;
    int k = pair / pps;
    y0 = 2 * (pair - k * pps);
    valid = k < a.nslots;
    if (!valid) k = a.nslots - 1;  // keep loads in bounds; nothing is written
    slot = a.slot_list[k];
    valid = valid && a.slots[slot].active;
    boff = (long long)slot * a.bstride;
    poff = (long long)slot * a.pstride;
    foff = (long long)slot * a.fstride;
  }
  const int pitch = a.pitch;
  const int yl = PAIRED ? a.ylog : 0;
  C* line = sm + pr * LS;
  // this pair's parking slots: park[i*TPL + t] (and park[NX + i*TPL + t] in 3D)
  C* park = sm + P * LS + pr * a.park_slots * NX;
  const int yy0 = (BATCHED || valid) ? y0 : 0;
  // the pair's rows in the spectral layout (row 1 follows row 0 when PAIRED)
  const long long r0 = boff + spec_row_base(yy0, pitch, yl);
  const long long r1 = PAIRED ? r0 + 1 : r0 + pitch;
  const long long q0 = (long long)yy0 * NX, q1 = q0 + NX;
  constexpr int H = NX / 2;
  auto kk_of = [](int k) { return k <= H ? k : NX - k; };

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
    for (int i = 0; i < E; ++i) {
      const int k = reg_pos<NX, RI0, E>(t, i);
      C p, q;
      ld_pair<PAIRED>(a.A + r0, a.A + r1, kk_of(k) << yl, p, q);
      v[i] = zpair<false, T>(p, q, k, NX, a.dkx);
    }
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
      // c_z of both rows: F^-1 of (C0 + i C1, Hermitian-extended) -> park
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int k = reg_pos<NX, RI0, E>(t, i);
        C p, q;
        ld_pair<PAIRED>(a.Cin + r0, a.Cin + r1, kk_of(k) << yl, p, q);
        v[i] = zpair<false, T>(p, q, k, NX, a.dkx);
      }
      fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
      for (int i = 0; i < E; ++i) park[NX + i * TPL + t] = v[i];
      asm volatile("" ::: "memory");
    }
    // c_x of both rows (from i kr A) -> park
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int k = reg_pos<NX, RI0, E>(t, i);
      C p, q;
      ld_pair<PAIRED>(a.A + r0, a.A + r1, kk_of(k) << yl, p, q);
      v[i] = zpair<true, T>(p, q, k, NX, a.dkx);
    }
    fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
    for (int i = 0; i < E; ++i) park[i * TPL + t] = v[i];
    asm volatile("" ::: "memory");
    // c_y of both rows (from B)
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int k = reg_pos<NX, RI0, E>(t, i);
      C p, q;
      ld_pair<PAIRED>(a.B + r0, a.B + r1, kk_of(k) << yl, p, q);
      v[i] = zpair<false, T>(p, q, k, NX, a.dkx);
    }
    fft_line<NX, +1, E>(v, t, line, a.tw);
    // keep the flow loads below from being hoisted into the transform (that
    // holds 4 E more values across it)
    asm volatile("" ::: "memory");
    // the products n = -(u.grad c) of rows y0 (Re) and y1 (Im); the flow is
    // pre-scaled (see the file header)
    const bool analytic = BATCHED && a.slots[slot].flow_kind == FLOW_CELLULAR;
    if (analytic) {
      const CellularRow<T> cr0 = cellular_row<T, C>(a.slots[slot], a.tw, yy0, NX, a.stage_c, a.fscale);
      const C ey1 = grid_expi(a.tw, a.slots[slot].Ky, yy0 + 1, NX);  // row 1's y factor
#pragma unroll
      for (int i = 0; i < E; ++i) {
        T u0, v0, u1, v1;
        cellular_uv2<T, C>(cr0, ey1.x, ey1.y, a.tw, reg_pos<NX, RIL, E>(t, i), NX, &u0, &v0, &u1, &v1);
        const C cx = park[i * TPL + t];
        C w;
        w.x = u0 * cx.x + v0 * v[i].x;
        w.y = u1 * cx.y + v1 * v[i].y;
        v[i] = w;
        if ((i & 3) == 3) asm volatile("" ::: "memory");  // a few elements' loads in flight at a time
      }
    } else {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const int x = reg_pos<NX, RIL, E>(t, i);
        const C cx = park[i * TPL + t];
        T n0 = a.u[foff + q0 + x] * cx.x + a.v[foff + q0 + x] * v[i].x;
        T n1 = a.u[foff + q1 + x] * cx.y + a.v[foff + q1 + x] * v[i].y;
        if (three) {
          const C cz = park[NX + i * TPL + t];
          n0 += a.w[foff + q0 + x] * cz.x;
          n1 += a.w[foff + q1 + x] * cz.y;
        }
        C w;
        w.x = n0;
        w.y = n1;
        v[i] = w;
      }
    }
  }
  // forward x-FFT of n_y0 + i n_y1, separated into the two rows' half
  // spectra: row y0 W[k] + conj(W[n-k]), row y1 -i (W[k] - conj(W[n-k]))
  const T sc = a.scale;
  auto emit = [&](int k, C wk, C wn) {
    C o0, o1;
    o0.x = (wk.x + wn.x) * sc; o0.y = (wk.y - wn.y) * sc;
    o1.x = (wk.y + wn.y) * sc; o1.y = (wn.x - wk.x) * sc;
    st_pair<PAIRED>(a.out + r0, a.out + r1, k << yl, o0, o1);
  };
  if constexpr (MirrorLast<NX, E>::ok) {
    // last stage on mirror-paired butterflies: W[k] and W[n-k] are in this
    // thread's registers (MirrorLast), so no shared-memory round trip
    fft_line_mirror_last<NX, E>(v, t, line, a.tw);
    constexpr int R = MirrorLast<NX, E>::R, B = MirrorLast<NX, E>::B, M = MirrorLast<NX, E>::M;
    if (valid) {
#pragma unroll
      for (int q = 0; q < M; ++q) {
        const int j = t + q * TPL;  // slot q; slot q + M holds B - j (B/2 when j = 0)
#pragma unroll
        for (int r = 0; r < R / 2; ++r) {
          if (q == 0 && t == 0) {
            // butterfly 0 (outputs r B, mirrored within itself) and butterfly B/2
            emit(r * B, v[r], v[(R - r) % R]);
            emit(B / 2 + r * B, v[M * R + r], v[M * R + R - 1 - r]);
          } else {
            emit(j + r * B, v[q * R + r], v[(q + M) * R + R - 1 - r]);
            emit(B - j + r * B, v[(q + M) * R + r], v[q * R + R - 1 - r]);
          }
        }
      }
      if (t == 0) emit(NX / 2, v[R / 2], v[R / 2]);  // k = n/2 = (R/2) B: butterfly 0, output R/2
    }
  } else {
    fft_line<NX, -1, E>(v, t, line, a.tw);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < E; ++i) line[smem_pad(reg_pos<NX, RFL, E>(t, i))] = v[i];
    __syncthreads();
    if (valid) {
      for (int k = t; k <= NX / 2; k += TPL) emit(k, line[smem_pad(k)], line[smem_pad((NX - k) & (NX - 1))]);
    }
  }
}

// ---------------------------------------------------------------------------
// Row pass, 2D RHS, with bulk-copy staging.  At block start one thread issues
// bulk copies (cp.async.bulk) of every row the block needs -- A, B of both
// rows and u, v of both rows, for each of its P pairs -- into shared memory,
// completing on one mbarrier; the transforms then read their inputs from
// shared memory.  Per pair: the line, one parking slot array, 4 spectral rows
// of `pitch` complex values, 4 flow rows of NX reals.
// ---------------------------------------------------------------------------
template <typename T, int NX> __host__ __device__ constexpr size_t row_tma_smem_bytes(int P, int pitch) {
  return (size_t)P * (line_stride(NX) + NX + 4 * pitch) * sizeof(typename cplx_of<T>::type) +
         (size_t)P * 4 * NX * sizeof(T) + 16;
}

template <typename T, int NX>
__global__ void __launch_bounds__(256) row_rhs_tma_kernel(RowArgs<T> a) {
  typedef typename cplx_of<T>::type C;
  constexpr int E = PassE<T, NX>::value;
  constexpr int TPL = NX / E;
  constexpr int LS = line_stride(NX);
  constexpr int RI0 = FirstRadix<NX, +1, E>::value;
  constexpr int RIL = LastRadix<NX, +1, E>::value;
  constexpr int RFL = LastRadix<NX, -1, E>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int P = blockDim.x / TPL;
  const int pr = threadIdx.x / TPL, t = threadIdx.x % TPL;
  const int pitch = a.pitch;
  C* line = sm + pr * LS;
  C* park = sm + P * LS + pr * NX;
  C* rows = sm + P * (LS + NX) + pr * 4 * pitch;  // A0, A1, B0, B1
  T* flows = reinterpret_cast<T*>(sm + P * (LS + NX + 4 * pitch)) + pr * 4 * NX;  // u0, u1, v0, v1
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + row_tma_smem_bytes<T, NX>(P, pitch) - 16);
  const long long boff = (long long)blockIdx.y * a.bstride;
  const long long foff = (long long)blockIdx.y * a.fstride;
  const int y0 = 2 * (blockIdx.x * P + pr);

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t rb = (uint32_t)((((NX / 2 + 1) * sizeof(C)) + 15) / 16 * 16);
    const uint32_t fb = (uint32_t)(NX * sizeof(T));
    mbar_arrive_expect_tx(bar, (uint32_t)P * 4u * (rb + fb));
    for (int q = 0; q < P; ++q) {
      const int yq = 2 * (blockIdx.x * P + q);
      C* rq = sm + P * (LS + NX) + q * 4 * pitch;
      T* fq = reinterpret_cast<T*>(sm + P * (LS + NX + 4 * pitch)) + q * 4 * NX;
      const C* A0 = a.A + boff + (long long)yq * pitch;
      const C* B0 = a.B + boff + (long long)yq * pitch;
      tma_load_1d(rq, A0, rb, bar);
      tma_load_1d(rq + pitch, A0 + pitch, rb, bar);
      tma_load_1d(rq + 2 * pitch, B0, rb, bar);
      tma_load_1d(rq + 3 * pitch, B0 + pitch, rb, bar);
      const T* u0 = a.u + foff + (long long)yq * NX;
      const T* v0 = a.v + foff + (long long)yq * NX;
      tma_load_1d(fq, u0, fb, bar);
      tma_load_1d(fq + NX, u0 + NX, fb, bar);
      tma_load_1d(fq + 2 * NX, v0, fb, bar);
      tma_load_1d(fq + 3 * NX, v0 + NX, fb, bar);
    }
  }
  const bool ok = mbar_wait_bounded(bar, 0, a.err);
  if (!__syncthreads_and(ok)) return;  // uniform: every thread returns

  const C* A0 = rows;
  const C* A1 = rows + pitch;
  const C* B0 = rows + 2 * pitch;
  const C* B1 = rows + 3 * pitch;
  const T* u0 = flows;
  const T* u1 = flows + NX;
  const T* v0 = flows + 2 * NX;
  const T* v1 = flows + 3 * NX;
  C v[E];
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(A0, B0, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
  fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int x = reg_pos<NX, RIL, E>(t, i);
    C pk; pk.x = u0[x] * v[i].x + v0[x] * v[i].y; pk.y = 0;
    park[i * TPL + t] = pk;
  }
  asm volatile("" ::: "memory");
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = zsrc_rhs<T, C>(A1, B1, reg_pos<NX, RI0, E>(t, i), NX, a.dkx);
  fft_line<NX, +1, E>(v, t, line, a.tw);
#pragma unroll
  for (int i = 0; i < E; ++i) {
    const int x = reg_pos<NX, RIL, E>(t, i);
    C w;
    w.x = park[i * TPL + t].x;
    w.y = u1[x] * v[i].x + v1[x] * v[i].y;
    v[i] = w;
  }
  fft_line<NX, -1, E>(v, t, line, a.tw);
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E; ++i) line[smem_pad(reg_pos<NX, RFL, E>(t, i))] = v[i];
  __syncthreads();
  const T sc = a.scale;
  C* out0 = a.out + boff + (long long)y0 * pitch;
  C* out1 = out0 + pitch;
  for (int k = t; k <= NX / 2; k += TPL) {
    const C wk = line[smem_pad(k)];
    const C wn = line[smem_pad((NX - k) & (NX - 1))];
    C o0, o1;
    o0.x = (wk.x + wn.x) * sc; o0.y = (wk.y - wn.y) * sc;
    o1.x = (wk.y + wn.y) * sc; o1.y = (wn.x - wk.x) * sc;
    out0[k] = o0;
    out1[k] = o1;
  }
}

// FP32 row blocks are held to 128 registers (two 256-thread blocks, or eight
// of the default 64 threads, per SM); FP64 takes what it needs.
#ifndef PTF_ROW_MINB_F32
#define PTF_ROW_MINB_F32 2
#endif
template <typename T> struct RowBounds { static constexpr int blocks = 1; };
template <> struct RowBounds<float> { static constexpr int blocks = PTF_ROW_MINB_F32; };
template <typename T, int NX, bool PAIRED = false>
__global__ void __launch_bounds__(256, RowBounds<T>::blocks) row_pass_kernel(RowArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  row_body<T, NX, false, PAIRED>(a, blockIdx.x, blockIdx.y, smem_raw);
}

}  // namespace ptf
