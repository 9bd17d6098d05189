// C ABI of libptf.so: problem handles, coefficient tables and the step
// driver.  The structure follows TracerAdvectionDiffusion.Problem
// (src/traceradvectiondiffusion.jl:165-216): a grid, the linear operator L
// (:511-554), scratch fields (:597-668) and the FourierFlows time stepper
// state; stepping is FourierFlows' stepforward! with the calcN! plugin of
// :756-786 fused into the pass kernels of ptf_passes.cuh.
//
// 2D step (per stage):  row pass (A, B -> Nx); column pass along y (Nx ->
//   stage combination -> A, B).
// 3D step (per stage):  row pass (A, B, C -> P1); y-forward (P1 -> P1);
//   z-pass (P1 -> stage combination -> Z1 in P1, Z2 in P2); y-inverse
//   (Z1, Z2 -> A in P1, B, C in P2).  Every pass reads a line completely
//   before writing it, so these in-place reuses are safe and 3D needs three
//   intermediate fields.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ptf.h"
#include "ptf_internal.h"

using namespace ptf;

namespace {

thread_local std::string g_create_error;

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// cos and sin of 2*pi*m/n by octant symmetry on host libm values (FP64).
void cos_sin_2pi(long long m, long long n, double* c, double* s) {
  m %= n;
  if (m < 0) m += n;
  const long long q = (4 * m) / n;          // quadrant
  long long r = m - q * (n / 4);            // 0 <= r < n/4 (n divisible by 4)
  double c0, s0;
  if (2 * r <= n / 4) {
    const double th = 2.0 * M_PI * ((double)r / (double)n);
    c0 = std::cos(th); s0 = std::sin(th);
  } else {
    const double th = 2.0 * M_PI * ((double)(n / 4 - r) / (double)n);
    c0 = std::sin(th); s0 = std::cos(th);
  }
  switch (q) {
    case 0: *c = c0; *s = s0; break;
    case 1: *c = -s0; *s = c0; break;
    case 2: *c = -c0; *s = -s0; break;
    default: *c = s0; *s = -c0; break;
  }
}

// Kassam-Trefethen contour mean for the ETDRK4 coefficients of one real z = dt*L
// (32 points on a circle of radius 1).  Returns zeta, alpha, beta, gamma / dt.
void etd_phis(double z, double out[4]) {
  const int M = 32;
  std::complex<double> acc[4] = {0, 0, 0, 0};
  for (int j = 0; j < M; ++j) {
    double cc, ss;
    // exp(2*pi*i*(j+1/2)/M) = exp(2*pi*i*(2j+1)/(2M))
    cos_sin_2pi(2 * j + 1, 2 * M, &cc, &ss);
    const std::complex<double> zc(z + cc, ss);
    const std::complex<double> ez = std::exp(zc), ez2 = std::exp(zc / 2.0);
    const std::complex<double> z2 = zc * zc, z3 = z2 * zc;
    acc[0] += (ez2 - 1.0) / zc;
    acc[1] += (-4.0 - zc + ez * (4.0 - 3.0 * zc + z2)) / z3;
    acc[2] += (2.0 + zc + ez * (-2.0 + zc)) / z3;
    acc[3] += (-4.0 - 3.0 * zc - z2 + ez * (4.0 - zc)) / z3;
  }
  for (int k = 0; k < 4; ++k) out[k] = acc[k].real() / M;
}

template <typename F> void parallel_for(long long n, F f) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > 64) nt = 64;
  if (n < 4096) nt = 1;
  std::vector<std::thread> th;
  const long long chunk = (n + nt - 1) / nt;
  for (unsigned i = 0; i < nt; ++i) {
    const long long a = i * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([=] { for (long long k = a; k < b; ++k) f(k); });
  }
  for (auto& t : th) t.join();
}

// Geometry of one column-pass launch: transform length n along a line of
// stride `stride`, ncols flat columns, nblk_y blocks of fields bstride apart.
struct ColGeom {
  int n = 0, stride = 0, ncols = 0, nblk_y = 0, W = 1;
  long long bstride = 0;
  double dk = 0;
  int axis = 0;  // 1 = y, 2 = z
};

}  // namespace

void ptf::set_global_error(const std::string& msg) { g_create_error = msg; }

struct ptf_handle {
  ptf_config cfg;
  int dim = 2, nx = 0, ny = 0, nz = 1;
  int nkr = 0, pitch = 0;
  long long plane = 0;      // spectral elements per solve (nz*ny*pitch)
  long long nphys = 0;      // physical points per solve (nz*ny*nx)
  long long rows = 0;       // x rows per solve (nz*ny)
  bool fp32 = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // device buffers (compute precision)
  void *s = nullptr, *si = nullptr, *acc = nullptr, *n1 = nullptr;
  void *A = nullptr, *B = nullptr, *Nx = nullptr;  // 2D; in 3D A = P1, Nx = P1
  void *C = nullptr;                               // 3D: P2 (Z2 / C)
  void *Ltab = nullptr, *coef = nullptr, *twx = nullptr, *twy = nullptr, *twz = nullptr;
  void *u = nullptr, *v = nullptr, *w = nullptr, *phys = nullptr;
  double* stage = nullptr;  // FP64 staging buffer
  long long stage_elems = 0;
  double t = 0.0;
  long long step = 0;
  bool ab_valid = false, have_c = false, have_flow = false;
  ColGeom gmain, gy3;  // main column pass (y in 2D, z in 3D); 3D y passes
  int rowP = 1;
  long long bytes = 0;
  long long launches = 0;
  std::string err;
  std::vector<void*> allocs;
  // per-pass timing (ptf_profile): CUDA events around each pass launch
  struct ProfRec { int kind; cudaEvent_t e0, e1; double bytes; };
  bool profiling = false;
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> event_pool;
};

namespace {

int fail(ptf_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg; else g_create_error = msg;
  return code;
}
int cuda_fail(ptf_handle* h, cudaError_t e, const char* what) {
  return fail(h, PTF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool dev_alloc(ptf_handle* h, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) { *p = nullptr; cudaGetLastError(); return false; }
  h->allocs.push_back(*p);
  h->bytes += (long long)bytes;
  return cudaMemsetAsync(*p, 0, bytes, h->stream) == cudaSuccess;
}

template <typename T> void fill_twiddles(std::vector<T>& out, int n) {
  out.resize(2 * (size_t)n);
  for (int m = 0; m < n; ++m) {
    double c, s;
    cos_sin_2pi(m, n, &c, &s);
    out[2 * m] = (T)c;
    out[2 * m + 1] = (T)(-s);  // exp(-2 pi i m / n)
  }
}

size_t elem_c(const ptf_handle* h) { return h->fp32 ? sizeof(float2) : sizeof(double2); }
size_t elem_r(const ptf_handle* h) { return h->fp32 ? sizeof(float) : sizeof(double); }

template <typename T> int upload(ptf_handle* h, void* dst, const std::vector<T>& src, const char* what) {
  cudaError_t e = cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, what);
  return PTF_OK;
}

// L (src/traceradvectiondiffusion.jl:538-554) and, for ETDRK4, its six
// coefficient planes, one value per spectral element [nz][ny][pitch].
template <typename T> int upload_tables(ptf_handle* h) {
  const ptf_config& c = h->cfg;
  const int ny = h->ny, nz = h->nz, pitch = h->pitch, nkr = h->nkr;
  const double dkx = 2 * M_PI / c.Lx, dky = 2 * M_PI / c.Ly, dkz = h->dim == 3 ? 2 * M_PI / c.Lz : 0.0;
  const size_t plane = (size_t)h->plane;
  std::vector<double> L(plane, 0.0);
  for (int q = 0; q < nz; ++q) {
    const double m = h->dim == 3 ? (q < nz / 2 ? q : q - nz) * dkz : 0.0;
    for (int j = 0; j < ny; ++j) {
      const double l = (j < ny / 2 ? j : j - ny) * dky;
      for (int k = 0; k < nkr; ++k) {
        const double kr = k * dkx;
        const double krsq = kr * kr + l * l + m * m;
        double hyp = 0.0;
        if (c.kappah != 0.0) hyp = c.kappah * std::pow(krsq, (double)c.nkappah);
        double Lv = -c.kappa * kr * kr - c.eta * l * l - hyp;
        if (h->dim == 3) Lv -= c.iota * m * m;
        L[((size_t)q * ny + j) * pitch + k] = Lv;
      }
    }
  }
  std::vector<T> Lt(plane);
  for (size_t i = 0; i < plane; ++i) Lt[i] = (T)L[i];
  int rc = upload(h, h->Ltab, Lt, "upload L");
  if (rc) return rc;
  if (c.stepper == PTF_ETDRK4) {
    std::vector<T> cf(6 * plane, (T)0);
    const double dt = c.dt;
    // L depends on l and m only through l^2 and m^2: compute rows j <= ny/2,
    // planes q <= nz/2 and mirror.
    const int nq = h->dim == 3 ? nz / 2 + 1 : 1;
    const long long njobs = (long long)nq * (ny / 2 + 1) * nkr;
    parallel_for(njobs, [&](long long idx) {
      const int k = (int)(idx % nkr);
      const int j = (int)((idx / nkr) % (ny / 2 + 1));
      const int q = (int)(idx / ((long long)nkr * (ny / 2 + 1)));
      const double Lv = L[((size_t)q * ny + j) * pitch + k];
      double ph[4];
      etd_phis(dt * Lv, ph);
      const double vals[6] = {std::exp(dt * Lv), std::exp(dt * Lv / 2), dt * ph[0], dt * ph[1], dt * ph[2], dt * ph[3]};
      const int js[2] = {j, (ny - j) % ny};
      const int qs[2] = {q, (nz - q) % nz};
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < (h->dim == 3 ? 2 : 1); ++b)
          for (int e = 0; e < 6; ++e) cf[e * plane + ((size_t)qs[b] * ny + js[a]) * pitch + k] = (T)vals[e];
    });
    rc = upload(h, h->coef, cf, "upload ETDRK4 coefficients");
    if (rc) return rc;
  }
  std::vector<T> tw;
  fill_twiddles(tw, h->nx);
  if ((rc = upload(h, h->twx, tw, "upload twiddles"))) return rc;
  fill_twiddles(tw, h->ny);
  if ((rc = upload(h, h->twy, tw, "upload twiddles"))) return rc;
  if (h->dim == 3) {
    fill_twiddles(tw, h->nz);
    if ((rc = upload(h, h->twz, tw, "upload twiddles"))) return rc;
  }
  return PTF_OK;
}

// ---------------------------------------------------------------------------
// Algorithmic bytes of one pass launch (the minimum HBM traffic of the
// design): M = one complex half-spectrum field of a solve, Tb = one real
// table of that shape, P = one real physical field; tables and the flow are
// shared by the batch and counted once per launch.
// ---------------------------------------------------------------------------
double pass_bytes(const ptf_handle* h, int kind, int mode) {
  const double e = (double)elem_c(h), r = (double)elem_r(h);
  const double ne = (double)h->nz * h->ny * h->nkr;
  const double M = ne * e, Tb = ne * r;
  const double P = (double)h->nphys * r;
  const double B = (double)h->cfg.batch;
  if (kind == 1) {  // row pass
    if (mode == ROW_RHS) return B * 3 * M + 2 * P;
    if (mode == ROW_RHS3) return B * 4 * M + 3 * P;
    return B * (M + P);
  }
  switch (mode) {
    case COL_PROLOGUE: return B * 3 * M;
    case COL_FWD_STORE: return B * 4 * M;
    case COL_FWD_N: return B * 2 * M;
    case COL_YINV3: return B * 5 * M;
    case COL_RK4_1: return B * 6 * M + Tb;
    case COL_RK4_2: case COL_RK4_3: return B * 8 * M + Tb;
    case COL_RK4_4: return B * 6 * M + Tb;
    case COL_ETD_1: return B * 7 * M + 4 * Tb;
    case COL_ETD_2: return B * 6 * M + 3 * Tb;
    case COL_ETD_3: return B * 7 * M + 3 * Tb;
    default: return B * 5 * M + Tb;  // COL_ETD_4
  }
}

cudaEvent_t pool_event(ptf_handle* h) {
  if (!h->event_pool.empty()) { cudaEvent_t e = h->event_pool.back(); h->event_pool.pop_back(); return e; }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
void prof_begin(ptf_handle* h, cudaEvent_t* e0) {
  *e0 = nullptr;
  if (!h->profiling) return;
  *e0 = pool_event(h);
  cudaEventRecord(*e0, h->stream);
}
void prof_end(ptf_handle* h, cudaEvent_t e0, int kind, double bytes) {
  if (!h->profiling || !e0) return;
  cudaEvent_t e1 = pool_event(h);
  cudaEventRecord(e1, h->stream);
  h->prof.push_back({kind, e0, e1, bytes});
}
void prof_clear(ptf_handle* h) {
  for (auto& r : h->prof) { h->event_pool.push_back(r.e0); h->event_pool.push_back(r.e1); }
  h->prof.clear();
}

// ---------------------------------------------------------------------------
// pass launches
// ---------------------------------------------------------------------------
struct ColIO {
  const void* nxin = nullptr;
  void* s = nullptr;     // defaults to the state
  void* A = nullptr;
  void* B = nullptr;
  void* Cout = nullptr;
  const void* z2in = nullptr;
  void* nout = nullptr;
};

template <typename T> int run_col(ptf_handle* h, const ColGeom& g, int mode, const ColIO& io, bool do_inverse) {
  typedef typename cplx_of<T>::type C;
  ColArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.nxin = (const C*)io.nxin;
  a.s = (C*)(io.s ? io.s : h->s);
  a.si = (C*)h->si; a.acc = (C*)h->acc; a.n1 = (C*)h->n1;
  a.A = (C*)io.A; a.B = (C*)io.B; a.Cout = (C*)io.Cout; a.z2in = (const C*)io.z2in; a.nout = (C*)io.nout;
  a.tw = (const C*)(g.axis == 2 ? h->twz : h->twy);
  a.Ltab = (const T*)h->Ltab; a.coef = (const T*)h->coef;
  a.dt = (T)h->cfg.dt;
  a.dk = (T)g.dk;
  a.stride = g.stride; a.mode = mode; a.do_inverse = do_inverse ? 1 : 0;
  a.bstride = g.bstride; a.tplane = h->plane; a.tab_per_block = 0;
  cudaEvent_t e0;
  prof_begin(h, &e0);
  cudaError_t e = launch_col<T>(g.n, a, g.W, g.ncols / g.W, g.nblk_y, h->stream);
  prof_end(h, e0, 0, pass_bytes(h, 0, mode));
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "column pass launch");
  return PTF_OK;
}

template <typename T>
int run_row(ptf_handle* h, int mode, const void* A, const void* B, const void* Cin, void* out, const void* cin,
            void* cout, double scale) {
  typedef typename cplx_of<T>::type C;
  RowArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.A = (const C*)A; a.B = (const C*)B; a.Cin = (const C*)Cin; a.out = (C*)out;
  a.u = (const T*)h->u; a.v = (const T*)h->v; a.w = (const T*)h->w;
  a.cin = (const T*)cin; a.cout = (T*)cout;
  a.tw = (const C*)h->twx;
  a.dkx = (T)(2 * M_PI / h->cfg.Lx);
  a.scale = (T)scale;
  a.rows = (int)h->rows; a.pitch = h->pitch; a.mode = mode;
  a.park_slots = h->dim == 3 ? 2 : 1;
  a.bstride = h->plane; a.pstride = h->nphys; a.fstride = 0;
  const int P = h->rowP;
  const int nby = (int)((h->rows / 2) / P);
  cudaEvent_t e0;
  prof_begin(h, &e0);
  cudaError_t e = launch_row<T>(h->nx, a, P, nby, h->cfg.batch, h->stream);
  prof_end(h, e0, 1, pass_bytes(h, 1, mode));
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "row pass launch");
  return PTF_OK;
}

// Inverse transforms of the state along the column axes: after this, A
// (and B[, C]) hold what the next row pass needs and A is the input of a c2r.
template <typename T> int do_prologue(ptf_handle* h, void* sbuf = nullptr) {
  ColIO io;
  io.s = sbuf;
  int rc;
  if (h->dim == 2) {
    io.A = h->A; io.B = h->B;
    rc = run_col<T>(h, h->gmain, COL_PROLOGUE, io, true);
  } else {
    io.A = h->A; io.B = h->C;  // Z1 -> P1, Z2 -> P2
    rc = run_col<T>(h, h->gmain, COL_PROLOGUE, io, true);
    if (!rc) {
      ColIO y;
      y.s = h->A; y.z2in = h->C; y.A = h->A; y.B = h->B; y.Cout = h->C;
      rc = run_col<T>(h, h->gy3, COL_YINV3, y, true);
    }
  }
  if (rc == PTF_OK && !sbuf) h->ab_valid = true;
  return rc;
}

// One RHS evaluation up to and including the main column pass, whose mode
// (a stage combination, or a plain forward into nout) the caller picks.
template <typename T> int rhs_and_column(ptf_handle* h, int col_mode, void* nout, bool do_inverse) {
  int rc;
  if (h->dim == 2) {
    rc = run_row<T>(h, ROW_RHS, h->A, h->B, nullptr, h->Nx, nullptr, nullptr, 1.0);
    if (rc) return rc;
    ColIO io;
    io.nxin = h->Nx; io.A = h->A; io.B = h->B; io.nout = nout;
    return run_col<T>(h, h->gmain, col_mode, io, do_inverse);
  }
  rc = run_row<T>(h, ROW_RHS3, h->A, h->B, h->C, h->A, nullptr, nullptr, 1.0);
  if (rc) return rc;
  ColIO yf;
  yf.nxin = h->A; yf.nout = h->A;
  rc = run_col<T>(h, h->gy3, COL_FWD_N, yf, false);
  if (rc) return rc;
  ColIO z;
  z.nxin = h->A; z.A = h->A; z.B = h->C; z.nout = nout;
  rc = run_col<T>(h, h->gmain, col_mode, z, do_inverse);
  if (rc || !do_inverse) return rc;
  ColIO y;
  y.s = h->A; y.z2in = h->C; y.A = h->A; y.B = h->B; y.Cout = h->C;
  return run_col<T>(h, h->gy3, COL_YINV3, y, true);
}

template <typename T> int do_steps(ptf_handle* h, long long nsteps) {
  if (!h->ab_valid) { int rc = do_prologue<T>(h); if (rc) return rc; }
  const bool etd = h->cfg.stepper == PTF_ETDRK4;
  for (long long n = 0; n < nsteps; ++n) {
    for (int st = 0; st < 4; ++st) {
      int rc = rhs_and_column<T>(h, (etd ? COL_ETD_1 : COL_RK4_1) + st, nullptr, true);
      if (rc) return rc;
    }
    h->t += h->cfg.dt;
    h->step += 1;
  }
  return PTF_OK;
}

// user physical (double, host or device) -> dst (compute precision), scaled
template <typename T> int phys_in(ptf_handle* h, const double* src, int where, T* dst, long long n, double scale) {
  const double* dsrc = src;
  cudaError_t e;
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(h->stage, src, n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "host to device copy");
    dsrc = h->stage;
  }
  e = launch_real_in<T>(dsrc, dst, n, scale, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "convert");
  if (where == PTF_HOST) {
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  }
  return PTF_OK;
}

template <typename T> int set_c_impl(ptf_handle* h, const double* c, int where) {
  int rc = phys_in<T>(h, c, where, (T*)h->phys, h->nphys * h->cfg.batch, 1.0);
  if (rc) return rc;
  void* nx = h->dim == 2 ? h->Nx : h->A;
  rc = run_row<T>(h, ROW_R2C, nullptr, nullptr, nullptr, nx, h->phys, nullptr, 0.5);
  if (rc) return rc;
  if (h->dim == 3) {
    ColIO yf;
    yf.nxin = h->A; yf.nout = h->A;
    if ((rc = run_col<T>(h, h->gy3, COL_FWD_N, yf, false))) return rc;
  }
  ColIO io;
  io.nxin = nx; io.A = h->A; io.B = h->dim == 2 ? h->B : h->C;
  if ((rc = run_col<T>(h, h->gmain, COL_FWD_STORE, io, true))) return rc;
  if (h->dim == 3) {
    ColIO y;
    y.s = h->A; y.z2in = h->C; y.A = h->A; y.B = h->B; y.Cout = h->C;
    if ((rc = run_col<T>(h, h->gy3, COL_YINV3, y, true))) return rc;
  }
  h->ab_valid = true;
  return PTF_OK;
}

template <typename T> int get_c_impl(ptf_handle* h, double* dst) {
  int rc = PTF_OK;
  if (!h->ab_valid) rc = do_prologue<T>(h);
  if (rc) return rc;
  const double inv = 1.0 / (double)h->nphys;
  rc = run_row<T>(h, ROW_C2R, h->A, nullptr, nullptr, nullptr, nullptr, h->phys, inv);
  if (rc) return rc;
  const long long n = h->nphys * h->cfg.batch;
  cudaError_t e = launch_real_out<T>((const T*)h->phys, dst, n, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "get_c");
  return PTF_OK;
}

template <typename T> int calcN_impl(ptf_handle* h, void* sbuf) {
  int rc = do_prologue<T>(h, sbuf);
  if (!rc) rc = rhs_and_column<T>(h, COL_FWD_N, sbuf, false);
  h->ab_valid = false;
  return rc;
}

int check_where(ptf_handle* h, int32_t where) {
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  return PTF_OK;
}

int spec_in(ptf_handle* h, const double* sol, int32_t where, void* dst) {
  const long long rows = h->rows * h->cfg.batch;
  const long long n = rows * h->nkr;
  const double2* src = (const double2*)sol;
  cudaError_t e;
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(h->stage, sol, n * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "spectral copy");
    src = (const double2*)h->stage;
  }
  e = h->fp32 ? launch_spec_in<float>(src, (float2*)dst, h->nkr, h->pitch, rows, h->stream)
              : launch_spec_in<double>(src, (double2*)dst, h->nkr, h->pitch, rows, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "spectral convert");
  return PTF_OK;
}

int spec_out(ptf_handle* h, const void* src, double* user, int32_t where) {
  const long long rows = h->rows * h->cfg.batch;
  const long long n = rows * h->nkr;
  double2* dst = (where == PTF_HOST) ? (double2*)h->stage : (double2*)user;
  cudaError_t e = h->fp32 ? launch_spec_out<float>((const float2*)src, dst, h->nkr, h->pitch, rows, h->stream)
                          : launch_spec_out<double>((const double2*)src, dst, h->nkr, h->pitch, rows, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "spectral convert");
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(user, h->stage, n * sizeof(double2), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "spectral copy");
  }
  return PTF_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int32_t ptf_abi_version(void) { return PTF_ABI_VERSION; }

void ptf_config_default(ptf_config* c, int32_t dim) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->dim = dim;
  c->nx = c->ny = c->nz = 128;
  c->Lx = c->Ly = c->Lz = 2 * M_PI;
  c->kappa = c->eta = c->iota = 0.1;
  c->kappah = 0.0;
  c->nkappah = 0;
  c->dt = 0.01;
  c->stepper = PTF_RK4;
  c->precision = PTF_FP64;
  c->time_mode = PTF_CLOCK_T;
  c->batch = 1;
}

const char* ptf_last_error(const ptf_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

void ptf_destroy(ptf_handle* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  prof_clear(h);
  for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
  for (void* p : h->allocs) cudaFree(p);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int ptf_create(const ptf_config* cfg, ptf_handle** out) {
  if (!cfg || !out) return fail(nullptr, PTF_ERR_ARG, "ptf_create: null argument");
  *out = nullptr;
  const ptf_config c = *cfg;
  if (c.dim == 1) return fail(nullptr, PTF_ERR_UNSUPPORTED, "1D problems are not built in this library");
  if (c.dim != 2 && c.dim != 3) return fail(nullptr, PTF_ERR_ARG, "dim must be 2 or 3");
  auto okn = [](int n) { return is_pow2(n) && n >= 16 && n <= 4096; };
  if (!okn(c.nx) || !okn(c.ny) || (c.dim == 3 && !okn(c.nz)))
    return fail(nullptr, PTF_ERR_ARG, "nx, ny (and nz) must be powers of two in [16, 4096]");
  if (!(c.Lx > 0) || !(c.Ly > 0) || (c.dim == 3 && !(c.Lz > 0)))
    return fail(nullptr, PTF_ERR_ARG, "domain lengths must be positive");
  if (!(c.dt > 0) || !std::isfinite(c.dt)) return fail(nullptr, PTF_ERR_ARG, "dt must be positive and finite");
  if (c.stepper != PTF_RK4 && c.stepper != PTF_ETDRK4) return fail(nullptr, PTF_ERR_ARG, "stepper must be RK4 or ETDRK4");
  if (c.precision != PTF_FP64 && c.precision != PTF_FP32) return fail(nullptr, PTF_ERR_ARG, "precision must be FP64 or FP32");
  if (c.time_mode != PTF_CLOCK_T && c.time_mode != PTF_STAGE_T) return fail(nullptr, PTF_ERR_ARG, "time_mode must be CLOCK_T or STAGE_T");
  if (c.batch < 1) return fail(nullptr, PTF_ERR_ARG, "batch must be >= 1");
  if (c.nkappah < 0) return fail(nullptr, PTF_ERR_ARG, "nkappah must be >= 0");
  if (!std::isfinite(c.kappa) || !std::isfinite(c.eta) || !std::isfinite(c.iota) || !std::isfinite(c.kappah))
    return fail(nullptr, PTF_ERR_ARG, "diffusivities must be finite");

  ptf_handle* h = new ptf_handle();
  h->cfg = c;
  h->dim = c.dim;
  h->nx = c.nx; h->ny = c.ny; h->nz = c.dim == 3 ? c.nz : 1;
  h->fp32 = c.precision == PTF_FP32;
  h->nkr = c.nx / 2 + 1;
  h->pitch = ((h->nkr + 7) / 8) * 8;
  h->plane = (long long)h->nz * h->ny * h->pitch;
  h->nphys = (long long)h->nz * h->ny * h->nx;
  h->rows = (long long)h->nz * h->ny;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { ptf_destroy(h); return cuda_fail(nullptr, e, "stream create"); }
  h->own_stream = true;
  // launch geometry
  auto lines = [&](int n, bool col, int div) {
    return h->fp32 ? default_lines_per_block<float>(n, col, div) : default_lines_per_block<double>(n, col, div);
  };
  if (h->dim == 2) {
    ColGeom& g = h->gmain;
    g.n = h->ny; g.stride = h->pitch; g.ncols = h->pitch; g.nblk_y = c.batch; g.bstride = h->plane;
    g.dk = 2 * M_PI / c.Ly; g.axis = 1; g.W = lines(h->ny, true, h->pitch);
  } else {
    ColGeom& g = h->gmain;
    g.n = h->nz; g.stride = h->ny * h->pitch; g.ncols = h->ny * h->pitch; g.nblk_y = c.batch;
    g.bstride = h->plane; g.dk = 2 * M_PI / c.Lz; g.axis = 2; g.W = lines(h->nz, true, h->ny * h->pitch);
    ColGeom& y = h->gy3;
    y.n = h->ny; y.stride = h->pitch; y.ncols = h->pitch; y.nblk_y = c.batch * h->nz;
    y.bstride = (long long)h->ny * h->pitch; y.dk = 2 * M_PI / c.Ly; y.axis = 1; y.W = lines(h->ny, true, h->pitch);
  }
  h->rowP = lines(h->nx, false, (int)(h->rows / 2));
  const size_t B = (size_t)c.batch;
  const size_t sc = (size_t)h->plane * B * elem_c(h);
  const size_t sp = (size_t)h->nphys * B * elem_r(h);
  bool ok = true;
  ok = ok && dev_alloc(h, &h->s, sc) && dev_alloc(h, &h->si, sc) && dev_alloc(h, &h->acc, sc);
  if (c.stepper == PTF_ETDRK4) ok = ok && dev_alloc(h, &h->n1, sc);
  ok = ok && dev_alloc(h, &h->A, sc) && dev_alloc(h, &h->B, sc);
  if (h->dim == 2) ok = ok && dev_alloc(h, &h->Nx, sc);
  else { ok = ok && dev_alloc(h, &h->C, sc); h->Nx = h->A; }
  ok = ok && dev_alloc(h, &h->Ltab, (size_t)h->plane * elem_r(h));
  if (c.stepper == PTF_ETDRK4) ok = ok && dev_alloc(h, &h->coef, 6 * (size_t)h->plane * elem_r(h));
  ok = ok && dev_alloc(h, &h->twx, (size_t)h->nx * elem_c(h)) && dev_alloc(h, &h->twy, (size_t)h->ny * elem_c(h));
  if (h->dim == 3) ok = ok && dev_alloc(h, &h->twz, (size_t)h->nz * elem_c(h));
  ok = ok && dev_alloc(h, &h->u, (size_t)h->nphys * elem_r(h)) && dev_alloc(h, &h->v, (size_t)h->nphys * elem_r(h));
  if (h->dim == 3) ok = ok && dev_alloc(h, &h->w, (size_t)h->nphys * elem_r(h));
  ok = ok && dev_alloc(h, &h->phys, sp);
  h->stage_elems = std::max<long long>(h->nphys * (long long)B, 2 * h->rows * h->nkr * (long long)B);
  ok = ok && dev_alloc(h, (void**)&h->stage, (size_t)h->stage_elems * sizeof(double));
  if (!ok) {
    const long long held = h->bytes;
    ptf_destroy(h);
    return fail(nullptr, PTF_ERR_MEMORY, "device allocation failed (" + std::to_string(held) + " bytes held)");
  }
  const int rc = h->fp32 ? upload_tables<float>(h) : upload_tables<double>(h);
  if (rc) { std::string m = h->err; ptf_destroy(h); return fail(nullptr, rc, m); }
  *out = h;
  return PTF_OK;
}

int ptf_set_flow_arrays(ptf_handle* h, const double* u, const double* v, const double* w, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!u || !v || (h->dim == 3 && !w)) return fail(h, PTF_ERR_ARG, "u, v (and w in 3D) are required");
  if (check_where(h, where)) return PTF_ERR_ARG;
  // The flow is shared by the batch: nphys values per component.
  const double sc = -1.0 / (2.0 * (double)h->nphys);
  const double* src[3] = {u, v, w};
  void* dst[3] = {h->u, h->v, h->w};
  for (int q = 0; q < h->dim; ++q) {
    const int rc = h->fp32 ? phys_in<float>(h, src[q], where, (float*)dst[q], h->nphys, sc)
                           : phys_in<double>(h, src[q], where, (double*)dst[q], h->nphys, sc);
    if (rc) return rc;
  }
  h->have_flow = true;
  return PTF_OK;
}

int ptf_set_c(ptf_handle* h, const double* c, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!c) return fail(h, PTF_ERR_ARG, "null field");
  if (check_where(h, where)) return PTF_ERR_ARG;
  const int rc = h->fp32 ? set_c_impl<float>(h, c, where) : set_c_impl<double>(h, c, where);
  if (rc) return rc;
  h->have_c = true;
  if (where == PTF_HOST) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "set_c");
  }
  return PTF_OK;
}

int ptf_get_c(ptf_handle* h, double* c, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!c) return fail(h, PTF_ERR_ARG, "null field");
  if (check_where(h, where)) return PTF_ERR_ARG;
  const long long n = h->nphys * h->cfg.batch;
  double* dst = (where == PTF_HOST) ? h->stage : c;
  const int rc = h->fp32 ? get_c_impl<float>(h, dst) : get_c_impl<double>(h, dst);
  if (rc) return rc;
  if (where == PTF_HOST) {
    cudaError_t e = cudaMemcpyAsync(c, h->stage, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "get_c copy");
  }
  return PTF_OK;
}

int ptf_get_sol(ptf_handle* h, double* sol, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol) return fail(h, PTF_ERR_ARG, "null field");
  if (check_where(h, where)) return PTF_ERR_ARG;
  return spec_out(h, h->s, sol, where);
}

int ptf_set_sol(ptf_handle* h, const double* sol, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol) return fail(h, PTF_ERR_ARG, "null field");
  if (check_where(h, where)) return PTF_ERR_ARG;
  int rc = spec_in(h, sol, where, h->s);
  if (rc) return rc;
  h->ab_valid = false;
  h->have_c = true;
  if (where == PTF_HOST) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "set_sol");
  }
  return PTF_OK;
}

int ptf_step(ptf_handle* h, int64_t nsteps) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (nsteps < 0) return fail(h, PTF_ERR_ARG, "nsteps must be >= 0");
  if (!h->have_flow) return fail(h, PTF_ERR_STATE, "no flow set (ptf_set_flow_arrays)");
  if (!h->have_c) return fail(h, PTF_ERR_STATE, "no initial condition (ptf_set_c / ptf_set_sol)");
  return h->fp32 ? do_steps<float>(h, nsteps) : do_steps<double>(h, nsteps);
}

int ptf_calcN(ptf_handle* h, const double* sol, double* N, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol || !N) return fail(h, PTF_ERR_ARG, "null field");
  if (!h->have_flow) return fail(h, PTF_ERR_STATE, "no flow set (ptf_set_flow_arrays)");
  if (check_where(h, where)) return PTF_ERR_ARG;
  // The input goes to a scratch state buffer (acc: free between steps), so
  // the handle's solution is untouched; the intermediates are recomputed by
  // the next step.
  void* sbuf = h->acc;
  int rc = spec_in(h, sol, where, sbuf);
  if (!rc) rc = h->fp32 ? calcN_impl<float>(h, sbuf) : calcN_impl<double>(h, sbuf);
  if (rc) return rc;
  return spec_out(h, sbuf, N, where);
}

int ptf_clock(const ptf_handle* h, double* t, int64_t* step) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (t) *t = h->t;
  if (step) *step = h->step;
  return PTF_OK;
}
int ptf_set_clock(ptf_handle* h, double t, int64_t step) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  h->t = t;
  h->step = step;
  return PTF_OK;
}
int ptf_synchronize(ptf_handle* h) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  return PTF_OK;
}
int ptf_get_stream(const ptf_handle* h, void** stream) {
  if (!h || !stream) return fail(nullptr, PTF_ERR_ARG, "null argument");
  *stream = (void*)h->stream;
  return PTF_OK;
}
int ptf_set_stream(ptf_handle* h, void* stream) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->own_stream = false;
  h->stream = (cudaStream_t)stream;
  return PTF_OK;
}
int ptf_device_bytes(const ptf_handle* h, int64_t* bytes) {
  if (!h || !bytes) return fail(nullptr, PTF_ERR_ARG, "null argument");
  *bytes = h->bytes;
  return PTF_OK;
}

int ptf_profile(ptf_handle* h, int32_t enable) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  prof_clear(h);
  h->profiling = enable != 0;
  return PTF_OK;
}

int ptf_profile_read(ptf_handle* h, int32_t kind, double* total_ms, int64_t* launches, double* bytes) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  double ms = 0.0, by = 0.0;
  int64_t n = 0;
  for (const auto& r : h->prof) {
    if (r.kind != kind) continue;
    float t = 0.f;
    e = cudaEventElapsedTime(&t, r.e0, r.e1);
    if (e != cudaSuccess) return cuda_fail(h, e, "event elapsed time");
    ms += t; by += r.bytes; ++n;
  }
  if (total_ms) *total_ms = ms;
  if (launches) *launches = n;
  if (bytes) *bytes = by;
  return PTF_OK;
}

int ptf_kernel_launches(const ptf_handle* h, int64_t* count) {
  if (!h || !count) return fail(nullptr, PTF_ERR_ARG, "null argument");
  *count = h->launches;
  return PTF_OK;
}

}  // extern "C"
