// C ABI of libptf.so: problem handles, coefficient tables and the step
// driver.  The structure follows TracerAdvectionDiffusion.Problem
// (src/traceradvectiondiffusion.jl:165-216): a grid, the linear operator L
// (:538-554), scratch fields (:652-668) and the FourierFlows time stepper
// state; stepping is FourierFlows' stepforward! with the calcN! plugin of
// :756-786 fused into two kernels per stage (ptf_pass2d.cuh).
#include <cuda_runtime.h>

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

}  // namespace

void ptf::set_global_error(const std::string& msg) { g_create_error = msg; }

struct ptf_handle {
  ptf_config cfg;
  int nkr = 0, pitch = 0;
  long long plane = 0;      // ny*pitch complex elements (2D)
  long long nphys = 0;      // nx*ny reals (2D)
  bool fp32 = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // device buffers (compute precision)
  void *s = nullptr, *si = nullptr, *acc = nullptr, *n1 = nullptr, *A = nullptr, *B = nullptr, *Nx = nullptr;
  void *Ltab = nullptr, *coef = nullptr, *twx = nullptr, *twy = nullptr;
  void *u = nullptr, *v = nullptr, *phys = nullptr;
  double* stage = nullptr;  // FP64 staging buffer
  long long stage_elems = 0;
  double t = 0.0;
  long long step = 0;
  bool ab_valid = false, have_c = false, have_flow = false;
  int colW = 1, rowP = 1;
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

template <typename T> int upload_tables(ptf_handle* h) {
  const ptf_config& c = h->cfg;
  const int nx = c.nx, ny = c.ny, pitch = h->pitch, nkr = h->nkr;
  const double dkx = 2 * M_PI / c.Lx, dky = 2 * M_PI / c.Ly;
  std::vector<double> L((size_t)ny * pitch, 0.0);
  for (int j = 0; j < ny; ++j) {
    const double l = (j < ny / 2 ? j : j - ny) * dky;
    for (int k = 0; k < nkr; ++k) {
      const double kr = k * dkx;
      const double krsq = kr * kr + l * l;
      double hyp = 0.0;
      if (c.kappah != 0.0) hyp = c.kappah * std::pow(krsq, (double)c.nkappah);
      L[(size_t)j * pitch + k] = -c.kappa * kr * kr - c.eta * l * l - hyp;
    }
  }
  std::vector<T> Lt(L.size());
  for (size_t i = 0; i < L.size(); ++i) Lt[i] = (T)L[i];
  cudaError_t e = cudaMemcpyAsync(h->Ltab, Lt.data(), Lt.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "upload L");
  if (c.stepper == PTF_ETDRK4) {
    const long long plane = (long long)ny * pitch;
    std::vector<T> cf(6 * (size_t)plane, (T)0);
    const double dt = c.dt;
    // L depends on l only through l^2: compute rows 0..ny/2 and mirror.
    parallel_for((long long)(ny / 2 + 1) * nkr, [&](long long idx) {
      const int j = (int)(idx / nkr), k = (int)(idx % nkr);
      const double Lv = L[(size_t)j * pitch + k];
      double ph[4];
      etd_phis(dt * Lv, ph);
      const double vals[6] = {std::exp(dt * Lv), std::exp(dt * Lv / 2), dt * ph[0], dt * ph[1], dt * ph[2], dt * ph[3]};
      const int j2 = (ny - j) % ny;
      for (int q = 0; q < 6; ++q) {
        cf[(size_t)q * plane + (size_t)j * pitch + k] = (T)vals[q];
        cf[(size_t)q * plane + (size_t)j2 * pitch + k] = (T)vals[q];
      }
    });
    e = cudaMemcpyAsync(h->coef, cf.data(), cf.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload ETDRK4 coefficients");
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "upload ETDRK4 coefficients");
  }
  std::vector<T> tw;
  fill_twiddles(tw, nx);
  e = cudaMemcpyAsync(h->twx, tw.data(), tw.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "upload twiddles");
  std::vector<T> twy;
  fill_twiddles(twy, ny);
  e = cudaMemcpyAsync(h->twy, twy.data(), twy.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "upload twiddles");
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "upload tables");
  return PTF_OK;
}

// ---------------------------------------------------------------------------
// algorithmic bytes of one pass launch (minimum HBM traffic of the design):
// M = one complex half-spectrum array (ny*(nx/2+1)), Tb = one real table of
// that shape, P = one real physical array (nx*ny); tables and the flow are
// shared by the batch and counted once per launch.
// ---------------------------------------------------------------------------
double pass_bytes(const ptf_handle* h, int kind, int mode) {
  const double e = (double)elem_c(h), r = (double)elem_r(h);
  const double M = (double)h->cfg.ny * h->nkr * e, Tb = (double)h->cfg.ny * h->nkr * r;
  const double P = (double)h->nphys * r;
  const double B = (double)h->cfg.batch;
  if (kind == 1) {  // row pass
    if (mode == ROW_RHS) return B * 3 * M + 2 * P;
    return B * (M + P);
  }
  switch (mode) {
    case COL_PROLOGUE: return B * 3 * M;
    case COL_FWD_STORE: return B * 4 * M;
    case COL_FWD_N: return B * 2 * M;
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
template <typename T> int run_col(ptf_handle* h, int mode, const void* nxin, void* nout, bool do_inverse) {
  typedef typename cplx_of<T>::type C;
  ColArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.nxin = (const C*)nxin;
  a.s = (C*)h->s; a.si = (C*)h->si; a.acc = (C*)h->acc; a.n1 = (C*)h->n1;
  a.A = (C*)h->A; a.B = (C*)h->B; a.nout = (C*)nout;
  a.tw = (const C*)h->twy; a.Ltab = (const T*)h->Ltab; a.coef = (const T*)h->coef;
  a.dt = (T)h->cfg.dt;
  a.dky = (T)(2 * M_PI / h->cfg.Ly);
  a.pitch = h->pitch; a.mode = mode; a.do_inverse = do_inverse ? 1 : 0;
  a.bstride = h->plane; a.tab_per_solve = 0;
  const int W = h->colW;
  const int nbx = h->pitch / W;
  cudaEvent_t e0;
  prof_begin(h, &e0);
  cudaError_t e = launch_col2d<T>(h->cfg.ny, a, W, nbx, h->cfg.batch, h->stream);
  prof_end(h, e0, 0, pass_bytes(h, 0, mode));
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "column pass launch");
  return PTF_OK;
}
template <typename T> int run_row(ptf_handle* h, int mode, const void* A, const void* B, void* out, const void* cin, void* cout, double scale) {
  typedef typename cplx_of<T>::type C;
  RowArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.A = (const C*)A; a.B = (const C*)B; a.out = (C*)out;
  a.u = (const T*)h->u; a.v = (const T*)h->v;
  a.cin = (const T*)cin; a.cout = (T*)cout;
  a.tw = (const C*)h->twx;
  a.dkx = (T)(2 * M_PI / h->cfg.Lx);
  a.scale = (T)scale;
  a.ny = h->cfg.ny; a.pitch = h->pitch; a.mode = mode;
  a.bstride = h->plane; a.pstride = h->nphys; a.fstride = 0;
  const int P = h->rowP;
  const int nby = (h->cfg.ny / 2) / P;
  cudaEvent_t e0;
  prof_begin(h, &e0);
  cudaError_t e = launch_row2d<T>(h->cfg.nx, a, P, nby, h->cfg.batch, h->stream);
  prof_end(h, e0, 1, pass_bytes(h, 1, mode));
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "row pass launch");
  return PTF_OK;
}

template <typename T> int do_prologue(ptf_handle* h) {
  int rc = run_col<T>(h, COL_PROLOGUE, nullptr, nullptr, true);
  if (rc == PTF_OK) h->ab_valid = true;
  return rc;
}

template <typename T> int do_steps(ptf_handle* h, long long nsteps) {
  if (!h->ab_valid) { int rc = do_prologue<T>(h); if (rc) return rc; }
  const bool etd = h->cfg.stepper == PTF_ETDRK4;
  const double norm = 1.0;
  for (long long n = 0; n < nsteps; ++n) {
    for (int st = 0; st < 4; ++st) {
      int rc = run_row<T>(h, ROW_RHS, h->A, h->B, h->Nx, nullptr, nullptr, norm);
      if (rc) return rc;
      rc = run_col<T>(h, (etd ? COL_ETD_1 : COL_RK4_1) + st, h->Nx, nullptr, true);
      if (rc) return rc;
    }
    h->t += h->cfg.dt;
    h->step += 1;
  }
  return PTF_OK;
}

// user physical (double, host or device) -> h->phys (compute precision), scaled
template <typename T> int phys_in(ptf_handle* h, const double* src, int where, T* dst, double scale) {
  const long long n = h->nphys * h->cfg.batch;
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
  if (c.dim != 2) return fail(nullptr, PTF_ERR_UNSUPPORTED, "dim must be 2 (3D handles are created by ptf_create with dim=3 once built)");
  auto okn = [](int n) { return is_pow2(n) && n >= 16 && n <= 4096; };
  if (!okn(c.nx) || !okn(c.ny)) return fail(nullptr, PTF_ERR_ARG, "nx and ny must be powers of two in [16, 4096]");
  if (!(c.Lx > 0) || !(c.Ly > 0)) return fail(nullptr, PTF_ERR_ARG, "domain lengths must be positive");
  if (!(c.dt > 0) || !std::isfinite(c.dt)) return fail(nullptr, PTF_ERR_ARG, "dt must be positive and finite");
  if (c.stepper != PTF_RK4 && c.stepper != PTF_ETDRK4) return fail(nullptr, PTF_ERR_ARG, "stepper must be RK4 or ETDRK4");
  if (c.precision != PTF_FP64 && c.precision != PTF_FP32) return fail(nullptr, PTF_ERR_ARG, "precision must be FP64 or FP32");
  if (c.batch < 1) return fail(nullptr, PTF_ERR_ARG, "batch must be >= 1");
  if (c.nkappah < 0) return fail(nullptr, PTF_ERR_ARG, "nkappah must be >= 0");
  if (!std::isfinite(c.kappa) || !std::isfinite(c.eta) || !std::isfinite(c.kappah))
    return fail(nullptr, PTF_ERR_ARG, "diffusivities must be finite");

  ptf_handle* h = new ptf_handle();
  h->cfg = c;
  h->fp32 = c.precision == PTF_FP32;
  h->nkr = c.nx / 2 + 1;
  h->pitch = ((h->nkr + 7) / 8) * 8;
  h->plane = (long long)c.ny * h->pitch;
  h->nphys = (long long)c.nx * c.ny;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { ptf_destroy(h); return cuda_fail(nullptr, e, "stream create"); }
  h->own_stream = true;
  // launch shapes
  h->colW = h->fp32 ? default_lines_per_block<float>(c.ny, true, h->pitch)
                    : default_lines_per_block<double>(c.ny, true, h->pitch);
  h->rowP = h->fp32 ? default_lines_per_block<float>(c.nx, false, c.ny / 2)
                    : default_lines_per_block<double>(c.nx, false, c.ny / 2);
  const size_t B = (size_t)c.batch;
  const size_t sc = (size_t)h->plane * B * elem_c(h);
  const size_t sp = (size_t)h->nphys * B * elem_r(h);
  bool ok = true;
  ok = ok && dev_alloc(h, &h->s, sc) && dev_alloc(h, &h->si, sc) && dev_alloc(h, &h->acc, sc);
  if (c.stepper == PTF_ETDRK4) ok = ok && dev_alloc(h, &h->n1, sc);
  ok = ok && dev_alloc(h, &h->A, sc) && dev_alloc(h, &h->B, sc) && dev_alloc(h, &h->Nx, sc);
  ok = ok && dev_alloc(h, &h->Ltab, (size_t)h->plane * elem_r(h));
  if (c.stepper == PTF_ETDRK4) ok = ok && dev_alloc(h, &h->coef, 6 * (size_t)h->plane * elem_r(h));
  ok = ok && dev_alloc(h, &h->twx, (size_t)c.nx * elem_c(h)) && dev_alloc(h, &h->twy, (size_t)c.ny * elem_c(h));
  ok = ok && dev_alloc(h, &h->u, (size_t)h->nphys * elem_r(h)) && dev_alloc(h, &h->v, (size_t)h->nphys * elem_r(h));
  ok = ok && dev_alloc(h, &h->phys, sp);
  h->stage_elems = std::max<long long>((long long)h->nphys * (long long)B, 2 * (long long)c.ny * h->nkr * (long long)B);
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
  (void)w;
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!u || !v) return fail(h, PTF_ERR_ARG, "u and v are required for a 2D flow");
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  // flow is shared by the batch: nphys values each
  const double sc = -1.0 / (2.0 * (double)h->cfg.nx * (double)h->cfg.ny);
  const double* src[2] = {u, v};
  void* dst[2] = {h->u, h->v};
  for (int q = 0; q < 2; ++q) {
    const double* d = src[q];
    cudaError_t e;
    if (where == PTF_HOST) {
      e = cudaMemcpyAsync(h->stage, src[q], h->nphys * sizeof(double), cudaMemcpyHostToDevice, h->stream);
      if (e != cudaSuccess) return cuda_fail(h, e, "flow upload");
      d = h->stage;
    }
    e = h->fp32 ? launch_real_in<float>(d, (float*)dst[q], h->nphys, sc, h->stream)
                : launch_real_in<double>(d, (double*)dst[q], h->nphys, sc, h->stream);
    h->launches++;
    if (e != cudaSuccess) return cuda_fail(h, e, "flow convert");
    if (where == PTF_HOST) {
      e = cudaStreamSynchronize(h->stream);
      if (e != cudaSuccess) return cuda_fail(h, e, "flow upload");
    }
  }
  h->have_flow = true;
  return PTF_OK;
}

int ptf_set_c(ptf_handle* h, const double* c, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!c) return fail(h, PTF_ERR_ARG, "null field");
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  int rc;
  if (h->fp32) {
    rc = phys_in<float>(h, c, where, (float*)h->phys, 1.0);
    if (!rc) rc = run_row<float>(h, ROW_R2C, nullptr, nullptr, h->Nx, h->phys, nullptr, 0.5);
    if (!rc) rc = run_col<float>(h, COL_FWD_STORE, h->Nx, nullptr, true);
  } else {
    rc = phys_in<double>(h, c, where, (double*)h->phys, 1.0);
    if (!rc) rc = run_row<double>(h, ROW_R2C, nullptr, nullptr, h->Nx, h->phys, nullptr, 0.5);
    if (!rc) rc = run_col<double>(h, COL_FWD_STORE, h->Nx, nullptr, true);
  }
  if (rc) return rc;
  h->ab_valid = true;
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
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  const long long n = h->nphys * h->cfg.batch;
  const double inv = 1.0 / ((double)h->cfg.nx * (double)h->cfg.ny);
  int rc = PTF_OK;
  double* dst = (where == PTF_HOST) ? h->stage : c;
  cudaError_t e;
  if (h->fp32) {
    if (!h->ab_valid) rc = do_prologue<float>(h);
    if (!rc) rc = run_row<float>(h, ROW_C2R, h->A, nullptr, nullptr, nullptr, h->phys, inv);
    if (rc) return rc;
    e = launch_real_out<float>((const float*)h->phys, dst, n, h->stream);
  } else {
    if (!h->ab_valid) rc = do_prologue<double>(h);
    if (!rc) rc = run_row<double>(h, ROW_C2R, h->A, nullptr, nullptr, nullptr, h->phys, inv);
    if (rc) return rc;
    e = cudaMemcpyAsync(dst, h->phys, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream);
  }
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "get_c");
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(c, h->stage, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "get_c copy");
  }
  return PTF_OK;
}

int ptf_get_sol(ptf_handle* h, double* sol, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol) return fail(h, PTF_ERR_ARG, "null field");
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  const long long rows = (long long)h->cfg.ny * h->cfg.batch;
  const long long n = rows * h->nkr;  // complex
  double2* dst = (where == PTF_HOST) ? (double2*)h->stage : (double2*)sol;
  cudaError_t e = h->fp32 ? launch_spec_out<float>((const float2*)h->s, dst, h->nkr, h->pitch, rows, h->stream)
                          : launch_spec_out<double>((const double2*)h->s, dst, h->nkr, h->pitch, rows, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "get_sol");
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(sol, h->stage, n * sizeof(double2), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "get_sol copy");
  }
  return PTF_OK;
}

int ptf_set_sol(ptf_handle* h, const double* sol, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol) return fail(h, PTF_ERR_ARG, "null field");
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  const long long rows = (long long)h->cfg.ny * h->cfg.batch;
  const long long n = rows * h->nkr;
  const double2* src = (const double2*)sol;
  cudaError_t e;
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(h->stage, sol, n * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "set_sol copy");
    src = (const double2*)h->stage;
  }
  e = h->fp32 ? launch_spec_in<float>(src, (float2*)h->s, h->nkr, h->pitch, rows, h->stream)
              : launch_spec_in<double>(src, (double2*)h->s, h->nkr, h->pitch, rows, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "set_sol");
  h->ab_valid = false;
  h->have_c = true;
  if (where == PTF_HOST) {
    e = cudaStreamSynchronize(h->stream);
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
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  // Work on copies so the handle's state is untouched: sol -> si buffer, N via acc buffer.
  const long long rows = (long long)h->cfg.ny * h->cfg.batch;
  const long long n = rows * h->nkr;
  const double2* src = (const double2*)sol;
  cudaError_t e;
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(h->stage, sol, n * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "calcN copy");
    src = (const double2*)h->stage;
  }
  // Temporarily swap the state pointer so the prologue transforms `sol`.
  void* saved_s = h->s;
  h->s = h->n1 ? h->n1 : h->acc;
  void* sbuf = h->s;
  e = h->fp32 ? launch_spec_in<float>(src, (float2*)sbuf, h->nkr, h->pitch, rows, h->stream)
              : launch_spec_in<double>(src, (double2*)sbuf, h->nkr, h->pitch, rows, h->stream);
  h->launches++;
  int rc = (e == cudaSuccess) ? PTF_OK : cuda_fail(h, e, "calcN convert");
  const bool fp32 = h->fp32;
  if (!rc) rc = fp32 ? run_col<float>(h, COL_PROLOGUE, nullptr, nullptr, true) : run_col<double>(h, COL_PROLOGUE, nullptr, nullptr, true);
  if (!rc) rc = fp32 ? run_row<float>(h, ROW_RHS, h->A, h->B, h->Nx, nullptr, nullptr, 1.0)
                     : run_row<double>(h, ROW_RHS, h->A, h->B, h->Nx, nullptr, nullptr, 1.0);
  if (!rc) rc = fp32 ? run_col<float>(h, COL_FWD_N, h->Nx, sbuf, false) : run_col<double>(h, COL_FWD_N, h->Nx, sbuf, false);
  h->s = saved_s;
  h->ab_valid = false;
  if (rc) return rc;
  double2* dst = (where == PTF_HOST) ? (double2*)h->stage : (double2*)N;
  e = fp32 ? launch_spec_out<float>((const float2*)sbuf, dst, h->nkr, h->pitch, rows, h->stream)
           : launch_spec_out<double>((const double2*)sbuf, dst, h->nkr, h->pitch, rows, h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "calcN out");
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(N, h->stage, n * sizeof(double2), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "calcN copy");
  }
  return PTF_OK;
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
