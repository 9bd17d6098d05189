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
#include <cstddef>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ptf.h"
#include "ptf_internal.h"
#include "ptf_trace.h"

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
  int carve = -1;  // preferred shared-memory carve-out in percent (-1: the CUDA driver's choice)
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
  int ylog = 0;             // spectral layout: rows interleaved in groups of 2^ylog (spec_index)
  int priv = 0;             // 1: state and tables in the main column pass's register order (SpecMap)
  long long plane = 0;      // spectral elements per solve (nz*ny*pitch)
  long long nphys = 0;      // physical points per solve (nz*ny*nx)
  long long rows = 0;       // x rows per solve (nz*ny)
  int bpad = 1;             // solves held on the device: 1D rounds the batch up to pairs
  bool fp32 = false;
  bool etd = false;         // ETDRK4 (plain or filtered)
  bool filtered = false;    // Filtered steppers: the state is multiplied by `filt` after each step
  bool flow_layers = false; // one flow per solve (ptf_set_flow_layers)
  bool flow_tv = false;     // analytic flow re-evaluated at clock.t before each step
  ptf_flow_desc fdesc{};    // the analytic flow (ptf_set_flow_analytic)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // device buffers (compute precision)
  void *s = nullptr, *si = nullptr, *acc = nullptr;
  void* slo = nullptr;  // FP32 handles: the state's low part (compensated state, stage_combine)
  void *A = nullptr, *B = nullptr, *Nx = nullptr;  // 2D; in 3D A = P1, Nx = P1
  void *C = nullptr;                               // 3D: P2 (Z2 / C)
  void *Ltab = nullptr, *coef = nullptr, *twx = nullptr, *twy = nullptr, *twz = nullptr, *filt = nullptr;
  void *ul = nullptr, *vl = nullptr;  // per-solve flows (batch x nphys each)
  double* layerU = nullptr;            // per-solve mean flow added to u (device, batch values)
  void *u = nullptr, *v = nullptr, *w = nullptr, *phys = nullptr;
  double* stage = nullptr;  // FP64 staging buffer
  long long stage_elems = 0;
  double t = 0.0;
  long long step = 0;
  bool ab_valid = false, have_c = false, have_flow = false;
  ColGeom gmain, gy3;  // main column pass (y in 2D, z in 3D); 3D y passes
  int rowP = 1;
  // schedule: solves per group (a step runs all its passes group by group so
  // a group's fields stay in L2), and a CUDA graph of one step
  int* err_dev = nullptr;  // device error flag of bounded waits
  // FP64 k = 0 mode (FP32 handles): per solve {s, stage input (ETDRK4: d), acc, -} of
  // the (0,0[,0]) mode, then 64 sum partials per solve and one sum per
  // solve; k0c = FP64 {L, E, E2, zeta, alpha, beta, gamma} at (0,0[,0])
  bool k0mode = false;
  double* k0 = nullptr;
  double* k0c = nullptr;
  int row_tma = 0;         // 2D RHS row pass with bulk-copy staging (tuning variant)
  int group = 0;           // 0: automatic
  int branches = 1;        // groups run as this many concurrent stream branches
  int use_graph = 1;
  double tuned_ms = 0.0;   // ms per step of the tuned shapes (0: not tuned)
  cudaStream_t side[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[3] = {nullptr, nullptr, nullptr};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_group = -1;
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

// Layouts of a handle's fields: intermediates (A, B, C, Nx) in the
// interleaved spectral layout; the state (s, si, acc) and the tables in the
// main column pass's register order when h->priv (SpecMap).
SpecMap lay_map(const ptf_handle* h) {
  SpecMap m;
  m.pitch = h->pitch;
  m.ylog = h->ylog;
  return m;
}
SpecMap state_map(const ptf_handle* h) {
  SpecMap m = lay_map(h);
  if (!h->priv) return m;
  m.priv = 1;
  m.n = h->gmain.n;
  if (h->fp32) col_line_shape<float>(m.n, &m.tpl, &m.rf);
  else col_line_shape<double>(m.n, &m.tpl, &m.rf);
  m.pl = h->fp32 ? 2 : 1;
  m.ny = h->ny;
  m.three = h->dim == 3;
  return m;
}

template <typename T> int upload(ptf_handle* h, void* dst, const std::vector<T>& src, const char* what) {
  cudaError_t e = cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, what);
  return PTF_OK;
}

// L (src/traceradvectiondiffusion.jl:538-554) and, for ETDRK4, its six
// coefficient planes, one value per spectral element in the layout of the
// state (state_map over the rows q * ny + j).
template <typename T> int upload_tables(ptf_handle* h) {
  const ptf_config& c = h->cfg;
  const int ny = h->ny, nz = h->nz, nkr = h->nkr;
  const SpecMap sm = state_map(h);
  auto at = [&](int q, int j, int k) { return (size_t)spec_map(sm, (long long)q * ny + j, k); };
  const double dkx = 2 * M_PI / c.Lx, dky = h->dim >= 2 ? 2 * M_PI / c.Ly : 0.0, dkz = h->dim == 3 ? 2 * M_PI / c.Lz : 0.0;
  const size_t plane = (size_t)h->plane;
  std::vector<double> L(plane, 0.0);
  for (int q = 0; q < nz; ++q) {
    const double m = h->dim == 3 ? (q < nz / 2 ? q : q - nz) * dkz : 0.0;
    for (int j = 0; j < ny; ++j) {
      const double l = h->dim == 1 ? 0.0 : (j < ny / 2 ? j : j - ny) * dky;
      for (int k = 0; k < nkr; ++k) {
        const double kr = k * dkx;
        const double krsq = kr * kr + l * l + m * m;
        double hyp = 0.0;
        if (c.kappah != 0.0) hyp = c.kappah * std::pow(krsq, (double)c.nkappah);
        double Lv = -c.kappa * kr * kr - c.eta * l * l - hyp;
        if (h->dim == 3) Lv -= c.iota * m * m;
        L[at(q, j, k)] = Lv;
      }
    }
  }
  std::vector<T> Lt(plane);
  for (size_t i = 0; i < plane; ++i) Lt[i] = (T)L[i];
  int rc = upload(h, h->Ltab, Lt, "upload L");
  if (rc) return rc;
  if (h->k0mode) {
    // the (0,0[,0]) mode's operator and ETDRK4 coefficients in FP64
    const double L0 = L[0], dt = c.dt;
    double ph[4];
    etd_phis(dt * L0, ph);
    const std::vector<double> kc = {L0, std::exp(dt * L0), std::exp(dt * L0 / 2), dt * ph[0], dt * ph[1],
                                    dt * ph[2], dt * ph[3], 0.0};
    if ((rc = upload(h, h->k0c, kc, "upload k = 0 coefficients"))) return rc;
  }
  if (h->filtered) {
    // FourierFlows' spectral filter (makefilter: order 4, innerK 0.65,
    // outerK 1, tol 1e-15): K = |(kr dx, l dy, m dz)| / pi; 1 below innerK,
    // exp(-decay (K - innerK)^4) above, decay = -log(tol) / (outerK - innerK)^4
    const double innerK = 0.65, outerK = 1.0, order = 4.0, tol = 1e-15;
    const double decay = -std::log(tol) / std::pow(outerK - innerK, order);
    const double dx = c.Lx / h->nx, dy = h->dim >= 2 ? c.Ly / h->ny : 0.0, dz = h->dim == 3 ? c.Lz / h->nz : 0.0;
    std::vector<T> ft(plane, (T)0);
    for (int q = 0; q < nz; ++q) {
      const double m = h->dim == 3 ? (q < nz / 2 ? q : q - nz) * dkz : 0.0;
      for (int j = 0; j < ny; ++j) {
        const double l = h->dim == 1 ? 0.0 : (j < ny / 2 ? j : j - ny) * dky;
        for (int k = 0; k < nkr; ++k) {
          const double a = k * dkx * dx / M_PI, b = l * dy / M_PI, e = m * dz / M_PI;
          const double K = std::sqrt(a * a + b * b + e * e);
          ft[at(q, j, k)] = (T)(K < innerK ? 1.0 : std::exp(-decay * std::pow(K - innerK, order)));
        }
      }
    }
    if ((rc = upload(h, h->filt, ft, "upload filter"))) return rc;
  }
  if (h->etd) {
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
      const double Lv = L[at(q, j, k)];
      double ph[4];
      etd_phis(dt * Lv, ph);
      // E - 1 and E2 - 1 (expm1): the stage combination applies s + (E - 1) s
      const double vals[6] = {std::expm1(dt * Lv), std::expm1(dt * Lv / 2), dt * ph[0], dt * ph[1], dt * ph[2],
                              dt * ph[3]};
      const int js[2] = {j, (ny - j) % ny};
      const int qs[2] = {q, (nz - q) % nz};
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < (h->dim == 3 ? 2 : 1); ++b)
          for (int e = 0; e < 6; ++e) cf[e * plane + at(qs[b], js[a], k)] = (T)vals[e];
    });
    rc = upload(h, h->coef, cf, "upload ETDRK4 coefficients");
    if (rc) return rc;
  }
  std::vector<T> tw;
  fill_twiddles(tw, h->nx);
  if ((rc = upload(h, h->twx, tw, "upload twiddles"))) return rc;
  if (h->dim >= 2) {
    fill_twiddles(tw, h->ny);
    if ((rc = upload(h, h->twy, tw, "upload twiddles"))) return rc;
  }
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
  if (kind == 2) {  // 1D stage pass: stage input + state traffic, flow
    switch (mode) {
      case COL_FWD_N: return B * 2 * M + P;
      case COL_RK4_1: return B * 3 * M + Tb + P;
      case COL_RK4_2: case COL_RK4_3: return B * 5 * M + Tb + P;
      case COL_RK4_4: return B * 3 * M + Tb + P;
      case COL_ETD_1: return B * 4 * M + 4 * Tb + P;
      case COL_ETD_2: return B * 5 * M + 3 * Tb + P;
      case COL_ETD_3: return B * 5 * M + 2 * Tb + P;
      default: return B * 3 * M + Tb + P;  // COL_ETD_4
    }
  }
  if (kind == 1) {  // row pass
    if (mode == ROW_RHS) return B * 3 * M + 2 * P;
    if (mode == ROW_RHS3) return B * 4 * M + 3 * P;
    return B * (M + P);
  }
  // the compensated state (FP32 2D/3D): the last stage also reads s and its
  // low part and writes the low part; set_c writes the low part (zero)
  const double lo = h->slo ? 1.0 : 0.0;
  switch (mode) {
    case COL_PROLOGUE: return B * 3 * M;
    case COL_FWD_STORE: return B * (4 + lo) * M;
    case COL_FWD_N: return B * 2 * M;
    case COL_YINV3: return B * 5 * M;
    case COL_RK4_1: return B * 6 * M + Tb;
    case COL_RK4_2: case COL_RK4_3: return B * 8 * M + Tb;
    case COL_RK4_4: return B * (6 + 3 * lo) * M + Tb;
    case COL_ETD_1: return B * 6 * M + 4 * Tb;
    case COL_ETD_2: return B * 6 * M + 3 * Tb;
    case COL_ETD_3: return B * 6 * M + 2 * Tb;
    default: return B * (5 + 3 * lo) * M + Tb;  // COL_ETD_4
  }
}

cudaEvent_t pool_event(ptf_handle* h) {
  if (!h->event_pool.empty()) { cudaEvent_t e = h->event_pool.back(); h->event_pool.pop_back(); return e; }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
void prof_begin(ptf_handle* h, cudaEvent_t* e0, cudaStream_t st) {
  *e0 = nullptr;
  if (!h->profiling) return;
  *e0 = pool_event(h);
  cudaEventRecord(*e0, st);
}
void prof_end(ptf_handle* h, cudaEvent_t e0, int kind, double bytes, cudaStream_t st) {
  if (!h->profiling || !e0) return;
  cudaEvent_t e1 = pool_event(h);
  cudaEventRecord(e1, st);
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

// Solves [b0, b0 + nb) of the batch: every per-solve field pointer is
// offset by b0 solves.
struct Group { int b0 = 0, nb = 0; cudaStream_t st = nullptr; };

template <typename C> C* goff(const void* p, const ptf_handle* h, const Group& gr) {
  return p ? (C*)p + (size_t)gr.b0 * (size_t)h->plane : nullptr;
}

template <typename T> int run_col(ptf_handle* h, const ColGeom& g, int mode, const ColIO& io, bool do_inverse,
                                  Group gr = Group()) {
  typedef typename cplx_of<T>::type C;
  if (gr.nb == 0) gr.nb = h->cfg.batch;
  ColArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.nxin = goff<const C>(io.nxin, h, gr);
  a.s = goff<C>(io.s ? io.s : h->s, h, gr);
  a.si = goff<C>(h->si, h, gr); a.acc = goff<C>(h->acc, h, gr);
  // the compensated state belongs to the main pass's own state
  a.slo = (&g == &h->gmain && !io.s) ? goff<C>(h->slo, h, gr) : nullptr;
  a.A = goff<C>(io.A, h, gr); a.B = goff<C>(io.B, h, gr); a.Cout = goff<C>(io.Cout, h, gr);
  a.z2in = goff<const C>(io.z2in, h, gr); a.nout = goff<C>(io.nout, h, gr);
  a.tw = (const C*)(g.axis == 2 ? h->twz : h->twy);
  a.Ltab = (const T*)h->Ltab; a.coef = (const T*)h->coef; a.filt = (const T*)h->filt;
  a.dt = (T)h->cfg.dt;
  a.dk = (T)g.dk;
  a.stride = g.stride; a.mode = mode; a.do_inverse = do_inverse ? 1 : 0;
  // lines along y run over the interleaved rows; the 3D z lines over flat
  // in-plane offsets, which any layout leaves contiguous
  a.ylog = g.axis == 1 ? h->ylog : 0;
  a.priv = (&g == &h->gmain) ? h->priv : 0;  // the state and tables are the main pass's
  a.bstride = g.bstride; a.tplane = h->plane; a.tab_per_block = 0;
  if (h->k0mode && &g == &h->gmain) {
    a.k0 = h->k0 + 4 * (size_t)gr.b0;
    a.k0c = h->k0c;
    a.dt64 = h->cfg.dt;
  }
  const int nblk_y = (int)((long long)g.nblk_y * gr.nb / h->cfg.batch);  // blocks of fields of the group
  cudaStream_t st = gr.st ? gr.st : h->stream;
  cudaEvent_t e0;
  prof_begin(h, &e0, st);
  cudaError_t e = launch_col<T>(g.n, a, g.W, g.ncols / g.W, nblk_y, st, g.carve);
  prof_end(h, e0, 0, pass_bytes(h, 0, mode) * gr.nb / h->cfg.batch, st);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "column pass launch");
  return PTF_OK;
}

template <typename T>
int run_row(ptf_handle* h, int mode, const void* A, const void* B, const void* Cin, void* out, const void* cin,
            void* cout, double scale, Group gr = Group()) {
  typedef typename cplx_of<T>::type C;
  if (gr.nb == 0) gr.nb = h->cfg.batch;
  RowArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.A = goff<const C>(A, h, gr); a.B = goff<const C>(B, h, gr); a.Cin = goff<const C>(Cin, h, gr);
  a.out = goff<C>(out, h, gr);
  a.u = (const T*)h->u; a.v = (const T*)h->v; a.w = (const T*)h->w;
  if (h->flow_layers) {  // one flow per solve: offset by the group, stride per field block
    a.u = (const T*)h->ul + (size_t)gr.b0 * h->nphys;
    a.v = (const T*)h->vl + (size_t)gr.b0 * h->nphys;
  }
  a.cin = cin ? (const T*)cin + (size_t)gr.b0 * h->nphys : nullptr;
  a.cout = cout ? (T*)cout + (size_t)gr.b0 * h->nphys : nullptr;
  a.tw = (const C*)h->twx;
  a.dkx = (T)(2 * M_PI / h->cfg.Lx);
  a.scale = (T)scale;
  a.rows = (int)h->rows; a.pitch = h->pitch; a.mode = mode; a.ylog = h->ylog;
  a.park_slots = h->dim == 3 ? 2 : 1;
  a.err = h->err_dev;
  a.tma = (h->row_tma && h->dim == 2 && mode == ROW_RHS) ? 1 : 0;
  a.bstride = h->plane; a.pstride = h->nphys; a.fstride = h->flow_layers ? h->nphys : 0;
  const int P = h->rowP;
  int nby = (int)((h->rows / 2) / P), nfields = gr.nb;
  if (h->dim == 1) {  // one row per solve: the pairs run over the (padded) batch
    a.rows = h->bpad;
    a.bstride = 0; a.pstride = 0;
    nby = (h->bpad / 2) / P;
    nfields = 1;
  }
  cudaStream_t st = gr.st ? gr.st : h->stream;
  cudaEvent_t e0;
  prof_begin(h, &e0, st);
  cudaError_t e = launch_row<T>(h->nx, a, P, nby, nfields, st);
  prof_end(h, e0, 1, pass_bytes(h, 1, mode) * gr.nb / h->cfg.batch, st);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "row pass launch");
  return PTF_OK;
}

// One 1D stage pass over every solve: stage input xin, next input xout.
template <typename T> int run_line1d(ptf_handle* h, int mode, const void* xin, void* xout) {
  typedef typename cplx_of<T>::type C;
  Line1DArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.xin = (const C*)xin; a.xout = (C*)xout;
  a.s = (C*)h->s; a.si = (C*)h->si; a.acc = (C*)h->acc;
  a.u = (const T*)h->u; a.Ltab = (const T*)h->Ltab; a.coef = (const T*)h->coef; a.tw = (const C*)h->twx;
  a.filt = (const T*)h->filt;
  a.dkx = (T)(2 * M_PI / h->cfg.Lx);
  a.dt = (T)h->cfg.dt;
  a.pitch = h->pitch; a.rows = h->bpad;
  if (h->k0mode && mode != COL_FWD_N) { a.k0 = h->k0; a.k0c = h->k0c; a.dt64 = h->cfg.dt; }
  const int P = h->rowP;
  cudaEvent_t e0;
  prof_begin(h, &e0, h->stream);
  cudaError_t e = launch_line1d<T>(h->nx, mode, a, P, (h->bpad / 2) / P, h->stream);
  prof_end(h, e0, 1, pass_bytes(h, 2, mode), h->stream);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "1D stage pass launch");
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
template <typename T> int rhs_and_column(ptf_handle* h, int col_mode, void* nout, bool do_inverse,
                                         Group gr = Group()) {
  int rc;
  if (h->dim == 2) {
    rc = run_row<T>(h, ROW_RHS, h->A, h->B, nullptr, h->Nx, nullptr, nullptr, 1.0, gr);
    if (rc) return rc;
    ColIO io;
    io.nxin = h->Nx; io.A = h->A; io.B = h->B; io.nout = nout;
    return run_col<T>(h, h->gmain, col_mode, io, do_inverse, gr);
  }
  rc = run_row<T>(h, ROW_RHS3, h->A, h->B, h->C, h->A, nullptr, nullptr, 1.0, gr);
  if (rc) return rc;
  ColIO yf;
  yf.nxin = h->A; yf.nout = h->A;
  rc = run_col<T>(h, h->gy3, COL_FWD_N, yf, false, gr);
  if (rc) return rc;
  ColIO z;
  z.nxin = h->A; z.A = h->A; z.B = h->C; z.nout = nout;
  rc = run_col<T>(h, h->gmain, col_mode, z, do_inverse, gr);
  if (rc || !do_inverse) return rc;
  ColIO y;
  y.s = h->A; y.z2in = h->C; y.A = h->A; y.B = h->B; y.Cout = h->C;
  return run_col<T>(h, h->gy3, COL_YINV3, y, true, gr);
}

// Solves per group: as many as keep a group's per-solve fields within about
// 3/4 of L2 (shared tables and flow take the rest), at least one.
int auto_group(const ptf_handle* h) {
  int dev = 0, l2 = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
  const double per = 7.0 * (double)h->plane * (double)elem_c(h);
  const double shared = (double)h->plane * elem_r(h) * (h->etd ? 7 : 1) +
                        (double)h->nphys * elem_r(h) * h->dim;
  int g = (int)((0.75 * (double)l2 - shared) / per);
  (void)g;
  // Measured on GB300 (16 x 1024^2, FP32): the passes are latency bound and
  // lose more to smaller launches than they gain from L2 residency, so the
  // default is the whole batch per launch; ptf_set_schedule picks groups.
  return (int)h->cfg.batch;
}

// One step: the four stages of every group.  Groups are dealt round-robin to
// `branches` streams (the handle's stream and up to three side streams that
// fork from it and join back), so passes of different groups can run at the
// same time; within a branch the groups follow one another.
template <typename T> int enqueue_step(ptf_handle* h, int group) {
  const bool etd = h->etd;
  if (h->dim == 1) {
    // stage inputs: RK4 s, si, si, si (si updated in place); ETDRK4 s, then
    // a, b, c in A (updated in place)
    int rc;
    if (etd) {
      if ((rc = run_line1d<T>(h, COL_ETD_1, h->s, h->A))) return rc;
      if ((rc = run_line1d<T>(h, COL_ETD_2, h->A, h->A))) return rc;
      if ((rc = run_line1d<T>(h, COL_ETD_3, h->A, h->A))) return rc;
      return run_line1d<T>(h, COL_ETD_4, h->A, nullptr);
    }
    if ((rc = run_line1d<T>(h, COL_RK4_1, h->s, nullptr))) return rc;
    if ((rc = run_line1d<T>(h, COL_RK4_2, h->si, nullptr))) return rc;
    if ((rc = run_line1d<T>(h, COL_RK4_3, h->si, nullptr))) return rc;
    return run_line1d<T>(h, COL_RK4_4, h->si, nullptr);
  }
  const int nbr = std::max(1, std::min(h->branches, 4));
  if (nbr > 1) {
    for (int k = 0; k < nbr - 1; ++k) {
      if (!h->side[k]) {
        cudaError_t e = cudaStreamCreateWithFlags(&h->side[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join[k], cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(h, e, "side stream");
      }
    }
    if (!h->ev_fork) {
      cudaError_t e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_fail(h, e, "fork event");
    }
    cudaEventRecord(h->ev_fork, h->stream);
    for (int k = 0; k < nbr - 1; ++k) cudaStreamWaitEvent(h->side[k], h->ev_fork, 0);
  }
  int gi = 0;
  for (int b0 = 0; b0 < h->cfg.batch; b0 += group, ++gi) {
    Group gr;
    gr.b0 = b0;
    gr.nb = std::min(group, h->cfg.batch - b0);
    const int br = gi % nbr;
    gr.st = br == 0 ? h->stream : h->side[br - 1];
    for (int st = 0; st < 4; ++st) {
      int rc = rhs_and_column<T>(h, (etd ? COL_ETD_1 : COL_RK4_1) + st, nullptr, true, gr);
      if (rc) return rc;
    }
  }
  if (nbr > 1) {
    for (int k = 0; k < nbr - 1; ++k) {
      cudaEventRecord(h->ev_join[k], h->side[k]);
      cudaStreamWaitEvent(h->stream, h->ev_join[k], 0);
    }
  }
  return PTF_OK;
}

void drop_graph(ptf_handle* h);
void drop_graph(ptf_handle* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->graph) cudaGraphDestroy(h->graph);
  h->gexec = nullptr;
  h->graph = nullptr;
  h->graph_group = -1;
}

template <typename T> cudaError_t eval_flow(ptf_handle* h, double t) {
  const double sc = -1.0 / (2.0 * (double)h->nphys);
  const ptf_config& c = h->cfg;
  h->launches++;
  return launch_flow_analytic<T>((T*)h->u, (T*)h->v, (T*)h->w, h->nx, h->ny, h->nz, c.Lx, h->dim >= 2 ? c.Ly : 1.0,
                                 h->dim == 3 ? c.Lz : 1.0, h->fdesc, t, sc, h->stream);
}

template <typename T> int do_steps(ptf_handle* h, long long nsteps) {
  if (!h->ab_valid && h->dim >= 2) { int rc = do_prologue<T>(h); if (rc) return rc; }
  int group = h->group > 0 ? std::min(h->group, (int)h->cfg.batch) : auto_group(h);
  if (h->branches > 1 && h->group == 0) group = (h->cfg.batch + h->branches - 1) / h->branches;
  // Replay a captured step unless per-pass timing is on (it records events
  // between the launches).
  bool graph = h->use_graph && !h->profiling && nsteps > 1;
  if (graph && (!h->gexec || h->graph_group != group)) {
    drop_graph(h);
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(h, e, "graph capture");
    const long long l0 = h->launches;
    const int rc = enqueue_step<T>(h, group);
    e = cudaStreamEndCapture(h->stream, &h->graph);
    h->launches = l0;
    if (rc == PTF_OK && e == cudaSuccess) e = cudaGraphInstantiate(&h->gexec, h->graph, 0);
    if (rc != PTF_OK || e != cudaSuccess) {
      // capture is an optimisation only: step with direct launches instead
      drop_graph(h);
      cudaGetLastError();
      h->use_graph = 0;
      graph = false;
    } else {
      h->graph_group = group;
    }
  }
  const int per_step = h->dim == 1 ? 4 : (int)(((h->cfg.batch + group - 1) / group) * 4 * (h->dim == 3 ? 4 : 2));
  for (long long n = 0; n < nsteps; ++n) {
    if (h->flow_tv) {  // the analytic flow at clock.t, frozen for the step's four stages
      cudaError_t e = eval_flow<T>(h, h->t);
      if (e != cudaSuccess) return cuda_fail(h, e, "flow evaluation");
    }
    if (graph) {
      cudaError_t e = cudaGraphLaunch(h->gexec, h->stream);
      if (e != cudaSuccess) return cuda_fail(h, e, "graph launch");
      h->launches += per_step;
    } else {
      int rc = enqueue_step<T>(h, group);
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

// FP64 k = 0 mode scratch: sum partials and per-solve sums
double* k0_partials(const ptf_handle* h) { return h->k0 + 4 * (size_t)h->bpad; }
double* k0_sums(const ptf_handle* h) { return h->k0 + 68 * (size_t)h->bpad; }

template <typename T> int set_c_impl(ptf_handle* h, const double* c, int where) {
  int rc = phys_in<T>(h, c, where, (T*)h->phys, h->nphys * h->cfg.batch, 1.0);
  if (rc) return rc;
  if (h->k0mode) {
    // s(0,0[,0]) = sum of c, compensated, from the FP64 input
    const double* dsrc = where == PTF_HOST ? h->stage : c;
    cudaError_t e = launch_solve_sums<double>(dsrc, h->nphys, h->cfg.batch, k0_partials(h), h->k0, 4, h->stream);
    h->launches += 2;
    if (e != cudaSuccess) return cuda_fail(h, e, "k = 0 mode sum");
  }
  if (h->dim == 1) {  // sol = rfft(c) of every solve, straight into the state
    rc = run_row<T>(h, ROW_R2C, nullptr, nullptr, nullptr, h->s, h->phys, nullptr, 0.5);
    if (rc) return rc;
    h->ab_valid = true;
    return PTF_OK;
  }
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
  if (!h->ab_valid && h->dim >= 2) rc = do_prologue<T>(h);
  if (rc) return rc;
  const double inv = 1.0 / (double)h->nphys;
  rc = run_row<T>(h, ROW_C2R, h->dim == 1 ? h->s : h->A, nullptr, nullptr, nullptr, nullptr, h->phys, inv);
  if (rc) return rc;
  const long long n = h->nphys * h->cfg.batch;
  cudaError_t e;
  if (h->k0mode) {
    // shift each solve's field so that its sum is the FP64 (0,0[,0]) mode
    e = launch_solve_sums<T>((const T*)h->phys, h->nphys, h->cfg.batch, k0_partials(h), k0_sums(h), 1, h->stream);
    if (e == cudaSuccess)
      e = launch_real_out_shift<T>((const T*)h->phys, dst, h->nphys, h->cfg.batch, h->k0, k0_sums(h), h->stream);
    h->launches += 3;
  } else {
    e = launch_real_out<T>((const T*)h->phys, dst, n, h->stream);
    h->launches++;
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "get_c");
  return PTF_OK;
}

template <typename T> int calcN_impl(ptf_handle* h, void* sbuf) {
  if (h->dim == 1) return run_line1d<T>(h, COL_FWD_N, sbuf, sbuf);  // N replaces the input in place
  int rc = do_prologue<T>(h, sbuf);
  if (!rc) rc = rhs_and_column<T>(h, COL_FWD_N, sbuf, false);
  h->ab_valid = false;
  return rc;
}

int check_where(ptf_handle* h, int32_t where) {
  if (where != PTF_HOST && where != PTF_DEVICE) return fail(h, PTF_ERR_ARG, "where must be PTF_HOST or PTF_DEVICE");
  return PTF_OK;
}

int spec_in(ptf_handle* h, const double* sol, int32_t where, void* dst, const SpecMap& map, void* lo = nullptr) {
  const long long rows = h->rows * h->cfg.batch;
  const long long n = rows * h->nkr;
  const double2* src = (const double2*)sol;
  cudaError_t e;
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(h->stage, sol, n * sizeof(double2), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "spectral copy");
    src = (const double2*)h->stage;
  }
  e = h->fp32 ? launch_spec_in<float>(src, (float2*)dst, h->nkr, h->pitch, rows, h->stream, &map, h->rows, (float2*)lo)
              : launch_spec_in<double>(src, (double2*)dst, h->nkr, h->pitch, rows, h->stream, &map, h->rows);
  h->launches++;
  if (e != cudaSuccess) return cuda_fail(h, e, "spectral convert");
  return PTF_OK;
}

// k0patch: the (0,0[,0]) element of each solve comes from the FP64 k = 0 state
int spec_out(ptf_handle* h, const void* src, double* user, int32_t where, const SpecMap& map, bool k0patch = false,
             const void* lo = nullptr) {
  const long long rows = h->rows * h->cfg.batch;
  const long long n = rows * h->nkr;
  double2* dst = (where == PTF_HOST) ? (double2*)h->stage : (double2*)user;
  cudaError_t e = h->fp32 ? launch_spec_out<float>((const float2*)src, dst, h->nkr, h->pitch, rows, h->stream, &map, h->rows,
                                                   (const float2*)lo)
                          : launch_spec_out<double>((const double2*)src, dst, h->nkr, h->pitch, rows, h->stream, &map, h->rows);
  h->launches++;
  if (e == cudaSuccess && k0patch) {
    e = launch_k0_to_spec(dst, h->rows * h->nkr, h->cfg.batch, h->k0, h->stream);
    h->launches++;
  }
  if (e != cudaSuccess) return cuda_fail(h, e, "spectral convert");
  if (where == PTF_HOST) {
    e = cudaMemcpyAsync(user, h->stage, n * sizeof(double2), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "spectral copy");
  }
  return PTF_OK;
}

// ---------------------------------------------------------------------------
// Launch-shape tuning.  The shapes (columns per column-pass block, row pairs
// per row-pass block, stream branches, the row pass's staged variant) change
// no result, only the time per step, so they are picked by timing whole
// steps on the handle itself, one knob at a time; the state is saved before
// and restored after, so tuning leaves the solve where it was.  Choices are
// cached per (precision, grid, batch, stepper) for the process.
// ---------------------------------------------------------------------------
std::mutex g_tune_mutex;
std::map<std::string, ptf_tuning> g_tune_cache;

std::string tuning_key(const ptf_handle* h) {
  char buf[160];
  std::snprintf(buf, sizeof(buf), "%d:%d:%d:%d:%d:%d:%d:%d", h->fp32 ? 32 : 64, h->dim, h->nx, h->ny, h->nz,
                (int)h->cfg.batch, (int)h->cfg.stepper, h->k0mode ? 1 : 0);
  return buf;
}

ptf_tuning current_tuning(const ptf_handle* h) {
  ptf_tuning t;
  std::memset(&t, 0, sizeof(t));
  t.col_lines = h->gmain.W;
  t.col_lines_y = h->dim == 3 ? h->gy3.W : 0;
  t.row_pairs = h->rowP;
  t.branches = h->branches;
  t.solves_per_group = h->group;
  t.row_staged = h->row_tma;
  t.col_carveout = h->gmain.carve;
  t.ms_per_step = h->tuned_ms;
  return t;
}

bool lines_ok(const ptf_handle* h, int n, bool col, int W, long long divisor) {
  if (W < 1 || (W & (W - 1)) || divisor % W) return false;
  const int mx = h->fp32 ? max_lines_per_block<float>(n, col) : max_lines_per_block<double>(n, col);
  return W <= mx;
}

long long row_pairs_total(const ptf_handle* h) { return h->dim == 1 ? h->bpad / 2 : h->rows / 2; }

int apply_tuning(ptf_handle* h, const ptf_tuning& t) {
  if (h->dim >= 2 && !lines_ok(h, h->gmain.n, true, t.col_lines, h->gmain.ncols))
    return fail(h, PTF_ERR_ARG, "col_lines: a power of two dividing the columns, within the block limit");
  if (h->dim == 3 && !lines_ok(h, h->gy3.n, true, t.col_lines_y, h->gy3.ncols))
    return fail(h, PTF_ERR_ARG, "col_lines_y: a power of two dividing the columns, within the block limit");
  if (!lines_ok(h, h->nx, false, t.row_pairs, row_pairs_total(h)))
    return fail(h, PTF_ERR_ARG, "row_pairs: a power of two dividing the row pairs, within the block limit");
  if (t.branches < 1 || t.branches > 4 || (h->dim == 1 && t.branches != 1))
    return fail(h, PTF_ERR_ARG, "branches must be 1..4 (1 for 1D problems)");
  if (t.solves_per_group < 0) return fail(h, PTF_ERR_ARG, "solves_per_group must be >= 0");
  if (t.row_staged != 0 && t.row_staged != 1) return fail(h, PTF_ERR_ARG, "row_staged must be 0 or 1");
  if (t.col_carveout < -1 || t.col_carveout > 100) return fail(h, PTF_ERR_ARG, "col_carveout must be -1..100");
  if (h->dim >= 2) { h->gmain.W = t.col_lines; h->gmain.carve = t.col_carveout; h->gy3.carve = t.col_carveout; }
  if (h->dim == 3) h->gy3.W = t.col_lines_y;
  h->rowP = t.row_pairs;
  h->branches = t.branches;
  h->group = t.solves_per_group;
  h->row_tma = (h->dim == 2 && h->ylog == 0) ? t.row_staged : 0;
  h->tuned_ms = t.ms_per_step;
  drop_graph(h);
  return PTF_OK;
}

// Device time of `steps` steps (best of two runs, after one untimed step).
template <typename T> int time_steps(ptf_handle* h, int steps, double* ms) {
  int rc = do_steps<T>(h, 1);
  if (rc) return rc;
  cudaEvent_t a = pool_event(h), b = pool_event(h);
  double best = 1e30;
  for (int rep = 0; rep < 2 && !rc; ++rep) {
    cudaEventRecord(a, h->stream);
    if ((rc = do_steps<T>(h, steps))) break;
    cudaEventRecord(b, h->stream);
    cudaError_t e = cudaEventSynchronize(b);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "tuning timer");
    else best = std::min(best, (double)t / steps);
  }
  h->event_pool.push_back(a);
  h->event_pool.push_back(b);
  *ms = best;
  return rc;
}

template <typename T> int autotune_impl(ptf_handle* h, int steps) {
  typedef typename cplx_of<T>::type C;
  const size_t sbytes = (size_t)h->plane * h->bpad * sizeof(C);
  const size_t nparts = h->slo ? 2 : 1;  // the state and, when compensated, its low part
  void* saved = nullptr;
  double* saved_k0 = nullptr;
  if (cudaMalloc(&saved, nparts * sbytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, PTF_ERR_MEMORY, "tuning: state copy");
  }
  if (h->k0mode && cudaMalloc((void**)&saved_k0, 4 * sizeof(double) * h->bpad) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(saved);
    return fail(h, PTF_ERR_MEMORY, "tuning: state copy");
  }
  const double t0 = h->t;
  const long long step0 = h->step;
  cudaError_t e = cudaMemcpyAsync(saved, h->s, sbytes, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess && h->slo)
    e = cudaMemcpyAsync((char*)saved + sbytes, h->slo, sbytes, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess && saved_k0)
    e = cudaMemcpyAsync(saved_k0, h->k0, 4 * sizeof(double) * h->bpad, cudaMemcpyDeviceToDevice, h->stream);
  int rc = e == cudaSuccess ? PTF_OK : cuda_fail(h, e, "tuning: save state");

  ptf_tuning best = current_tuning(h);
  double best_ms = 1e30;
  auto trial = [&](const ptf_tuning& t) -> int {
    int r = apply_tuning(h, t);
    if (r) return r;
    double ms = 0;
    if ((r = time_steps<T>(h, steps, &ms))) return r;
    if (ms < best_ms) { best_ms = ms; best = t; best.ms_per_step = ms; }
    return PTF_OK;
  };
  if (!rc) rc = trial(best);
  // one knob at a time, starting from the best so far
  for (int knob = 0; knob < 5 && !rc; ++knob) {
    std::vector<ptf_tuning> cands;
    for (int v = 1; v <= 64; v *= 2) {
      ptf_tuning t = best;
      if (knob == 0) { if (h->dim < 2 || !lines_ok(h, h->gmain.n, true, v, h->gmain.ncols)) continue; t.col_lines = v; }
      else if (knob == 1) { if (h->dim != 3 || !lines_ok(h, h->gy3.n, true, v, h->gy3.ncols)) continue; t.col_lines_y = v; }
      else if (knob == 2) { if (!lines_ok(h, h->nx, false, v, row_pairs_total(h))) continue; t.row_pairs = v; }
      else if (knob == 3) { if (v > 4 || v > h->cfg.batch || h->dim == 1) continue; t.branches = v; t.solves_per_group = 0; }
      else { if (v > 2 || h->dim != 2 || h->ylog != 0) continue; t.row_staged = v - 1; }
      cands.push_back(t);
    }
    for (const ptf_tuning& t : cands) {
      if (std::memcmp(&t, &best, offsetof(ptf_tuning, ms_per_step)) == 0) continue;
      if ((rc = trial(t))) break;
    }
  }
  if (!rc) rc = apply_tuning(h, best);
  // restore the solve
  e = cudaMemcpyAsync(h->s, saved, sbytes, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess && h->slo)
    e = cudaMemcpyAsync(h->slo, (char*)saved + sbytes, sbytes, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess && saved_k0)
    e = cudaMemcpyAsync(h->k0, saved_k0, 4 * sizeof(double) * h->bpad, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(saved);
  if (saved_k0) cudaFree(saved_k0);
  if (e != cudaSuccess && !rc) rc = cuda_fail(h, e, "tuning: restore state");
  h->t = t0;
  h->step = step0;
  h->ab_valid = false;
  return rc;
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
  c->k0_mode = 1;
}

const char* ptf_last_error(const ptf_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

void ptf_destroy(ptf_handle* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graph(h);
  for (int k = 0; k < 3; ++k) {
    if (h->side[k]) { cudaStreamSynchronize(h->side[k]); cudaStreamDestroy(h->side[k]); }
    if (h->ev_join[k]) cudaEventDestroy(h->ev_join[k]);
  }
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
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
  if (c.dim < 1 || c.dim > 3) return fail(nullptr, PTF_ERR_ARG, "dim must be 1, 2 or 3");
  auto okn = [](int n) { return is_pow2(n) && n >= 16 && n <= 4096; };
  if (!okn(c.nx) || (c.dim >= 2 && !okn(c.ny)) || (c.dim == 3 && !okn(c.nz)))
    return fail(nullptr, PTF_ERR_ARG, "nx (ny, nz) must be powers of two in [16, 4096]");
  if (!(c.Lx > 0) || (c.dim >= 2 && !(c.Ly > 0)) || (c.dim == 3 && !(c.Lz > 0)))
    return fail(nullptr, PTF_ERR_ARG, "domain lengths must be positive");
  if (!(c.dt > 0) || !std::isfinite(c.dt)) return fail(nullptr, PTF_ERR_ARG, "dt must be positive and finite");
  if (c.stepper < PTF_RK4 || c.stepper > PTF_FILTERED_ETDRK4)
    return fail(nullptr, PTF_ERR_ARG, "stepper must be RK4, ETDRK4, FilteredRK4 or FilteredETDRK4");
  if (c.precision != PTF_FP64 && c.precision != PTF_FP32) return fail(nullptr, PTF_ERR_ARG, "precision must be FP64 or FP32");
  if (c.time_mode != PTF_CLOCK_T && c.time_mode != PTF_STAGE_T) return fail(nullptr, PTF_ERR_ARG, "time_mode must be CLOCK_T or STAGE_T");
  if (c.batch < 1) return fail(nullptr, PTF_ERR_ARG, "batch must be >= 1");
  if (c.nkappah < 0) return fail(nullptr, PTF_ERR_ARG, "nkappah must be >= 0");
  if (c.k0_mode != 0 && c.k0_mode != 1) return fail(nullptr, PTF_ERR_ARG, "k0_mode must be 0 or 1");
  if (!std::isfinite(c.kappa) || !std::isfinite(c.eta) || !std::isfinite(c.iota) || !std::isfinite(c.kappah))
    return fail(nullptr, PTF_ERR_ARG, "diffusivities must be finite");

  ptf_handle* h = new ptf_handle();
  h->cfg = c;
  h->dim = c.dim;
  h->nx = c.nx; h->ny = c.dim >= 2 ? c.ny : 1; h->nz = c.dim == 3 ? c.nz : 1;
  h->bpad = c.dim == 1 ? c.batch + (c.batch & 1) : c.batch;
  h->fp32 = c.precision == PTF_FP32;
  h->etd = c.stepper == PTF_ETDRK4 || c.stepper == PTF_FILTERED_ETDRK4;
  h->filtered = c.stepper == PTF_FILTERED_RK4 || c.stepper == PTF_FILTERED_ETDRK4;
  h->k0mode = h->fp32 && c.k0_mode == 1;
  h->nkr = c.nx / 2 + 1;
  h->pitch = ((h->nkr + 7) / 8) * 8;
  h->plane = (long long)h->nz * h->ny * h->pitch;
  h->nphys = (long long)h->nz * h->ny * h->nx;
  h->rows = (long long)h->nz * h->ny;
  // spectral layout: rows in groups of four where the y lines allow (1D: plain).
  // PTF_SPEC_YLOG (0..2) caps it, for comparing layouts.
  if (h->dim >= 2) {
    h->ylog = h->fp32 ? col_ylog_limit<float>(h->ny) : col_ylog_limit<double>(h->ny);
    if (const char* ev = std::getenv("PTF_SPEC_YLOG")) {
      const int cap = std::atoi(ev);
      if (cap >= 0 && cap < h->ylog) h->ylog = cap;
    }
    // the state and tables in the main pass's register order (PTF_SPEC_PRIV=0: off)
    const char* ev = std::getenv("PTF_SPEC_PRIV");
    h->priv = (ev && std::atoi(ev) == 0) ? 0 : 1;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { ptf_destroy(h); return cuda_fail(nullptr, e, "stream create"); }
  h->own_stream = true;
  // launch geometry
  auto lines = [&](int n, bool col, int div) {
    return h->fp32 ? default_lines_per_block<float>(n, col, div) : default_lines_per_block<double>(n, col, div);
  };
  if (h->dim == 1) {
    // no column passes
  } else if (h->dim == 2) {
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
  h->rowP = lines(h->nx, false, (int)(h->dim == 1 ? h->bpad / 2 : h->rows / 2));
  // two concurrent stream branches for batches (measured +4% on 16 x 1024^2)
  h->branches = (c.batch >= 2 && h->dim >= 2) ? 2 : 1;
  const size_t B = (size_t)h->bpad;
  const size_t sc = (size_t)h->plane * B * elem_c(h);
  const size_t sp = (size_t)h->nphys * B * elem_r(h);
  bool ok = true;
  ok = ok && dev_alloc(h, &h->s, sc) && dev_alloc(h, &h->si, sc) && dev_alloc(h, &h->acc, sc);
  if (h->fp32 && h->dim >= 2) ok = ok && dev_alloc(h, &h->slo, sc);
  ok = ok && dev_alloc(h, &h->A, sc);
  if (h->dim >= 2) ok = ok && dev_alloc(h, &h->B, sc);
  if (h->dim == 2) ok = ok && dev_alloc(h, &h->Nx, sc);
  else if (h->dim == 3) { ok = ok && dev_alloc(h, &h->C, sc); h->Nx = h->A; }
  ok = ok && dev_alloc(h, &h->Ltab, (size_t)h->plane * elem_r(h));
  if (h->etd) ok = ok && dev_alloc(h, &h->coef, 6 * (size_t)h->plane * elem_r(h));
  if (h->filtered) ok = ok && dev_alloc(h, &h->filt, (size_t)h->plane * elem_r(h));
  ok = ok && dev_alloc(h, &h->twx, (size_t)h->nx * elem_c(h));
  if (h->dim >= 2) ok = ok && dev_alloc(h, &h->twy, (size_t)h->ny * elem_c(h));
  if (h->dim == 3) ok = ok && dev_alloc(h, &h->twz, (size_t)h->nz * elem_c(h));
  ok = ok && dev_alloc(h, &h->u, (size_t)h->nphys * elem_r(h));
  if (h->dim >= 2) ok = ok && dev_alloc(h, &h->v, (size_t)h->nphys * elem_r(h));
  if (h->dim == 3) ok = ok && dev_alloc(h, &h->w, (size_t)h->nphys * elem_r(h));
  ok = ok && dev_alloc(h, &h->phys, sp);
  h->stage_elems = std::max<long long>(h->nphys * (long long)B, 2 * h->rows * h->nkr * (long long)B);
  ok = ok && dev_alloc(h, (void**)&h->stage, (size_t)h->stage_elems * sizeof(double));
  ok = ok && dev_alloc(h, (void**)&h->err_dev, sizeof(int));
  if (h->k0mode)
    ok = ok && dev_alloc(h, (void**)&h->k0, 69 * B * sizeof(double)) && dev_alloc(h, (void**)&h->k0c, 8 * sizeof(double));
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
  if (!u || (h->dim >= 2 && !v) || (h->dim == 3 && !w))
    return fail(h, PTF_ERR_ARG, "u (v in 2D/3D, w in 3D) are required");
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
  h->flow_layers = false;
  h->flow_tv = false;
  h->have_flow = true;
  return PTF_OK;
}

int ptf_set_flow_analytic(ptf_handle* h, const ptf_flow_desc* d) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!d) return fail(h, PTF_ERR_ARG, "null flow description");
  if (d->kind == PTF_FLOW_CELLULAR) {
    if (h->dim != 2) return fail(h, PTF_ERR_ARG, "the cellular flow is 2D");
  } else if (d->kind == PTF_FLOW_ABC) {
    if (h->dim != 3) return fail(h, PTF_ERR_ARG, "the ABC flow is 3D");
  } else {
    return fail(h, PTF_ERR_ARG, "flow kind must be PTF_FLOW_CELLULAR or PTF_FLOW_ABC");
  }
  const double vals[6] = {d->U, d->eps, d->omega, d->A, d->B, d->C};
  for (double x : vals)
    if (!std::isfinite(x)) return fail(h, PTF_ERR_ARG, "flow parameters must be finite");
  h->fdesc = *d;
  h->flow_layers = false;
  h->flow_tv = d->kind == PTF_FLOW_CELLULAR && d->eps != 0.0 && d->omega != 0.0;
  cudaError_t e = h->fp32 ? eval_flow<float>(h, h->t) : eval_flow<double>(h, h->t);
  if (e != cudaSuccess) return cuda_fail(h, e, "flow evaluation");
  h->have_flow = true;
  return PTF_OK;
}

int ptf_set_flow_layers(ptf_handle* h, const double* u, const double* v, const double* U, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (h->dim != 2) return fail(h, PTF_ERR_UNSUPPORTED, "layered flows are 2D (MultiLayerQG)");
  if (!u || !v) return fail(h, PTF_ERR_ARG, "u and v are required");
  if (check_where(h, where)) return PTF_ERR_ARG;
  const long long B = h->cfg.batch, n = h->nphys * B;
  if (!h->ul) {
    const size_t bytes = (size_t)n * elem_r(h);
    if (!dev_alloc(h, &h->ul, bytes) || !dev_alloc(h, &h->vl, bytes) ||
        !dev_alloc(h, (void**)&h->layerU, (size_t)B * sizeof(double)))
      return fail(h, PTF_ERR_MEMORY, "device allocation failed (layer flows)");
  }
  std::vector<double> Uh((size_t)B, 0.0);
  if (U) Uh.assign(U, U + B);
  cudaError_t e = cudaMemcpyAsync(h->layerU, Uh.data(), (size_t)B * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "layer mean flows");
  // the flow is pre-scaled by -1/(2 nx ny) like ptf_set_flow_arrays
  const double sc = -1.0 / (2.0 * (double)h->nphys);
  const double* src[2] = {u, v};
  void* dst[2] = {h->ul, h->vl};
  for (int q = 0; q < 2; ++q) {
    const double* dsrc = src[q];
    if (where == PTF_HOST) {
      e = cudaMemcpyAsync(h->stage, src[q], (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
      if (e != cudaSuccess) return cuda_fail(h, e, "host to device copy");
      dsrc = h->stage;
    }
    e = h->fp32 ? launch_layers_in<float>(dsrc, (float*)dst[q], h->nphys, (int)B, q == 0 ? h->layerU : nullptr, sc, h->stream)
                : launch_layers_in<double>(dsrc, (double*)dst[q], h->nphys, (int)B, q == 0 ? h->layerU : nullptr, sc, h->stream);
    h->launches++;
    if (e != cudaSuccess) return cuda_fail(h, e, "convert");
    if (where == PTF_HOST) {
      e = cudaStreamSynchronize(h->stream);
      if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
    }
  }
  h->flow_layers = true;
  h->flow_tv = false;
  h->have_flow = true;
  return PTF_OK;
}

int ptf_set_c(ptf_handle* h, const double* c, int32_t where) {
  ptf::TraceRange tr("ptf_set_c");
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
  ptf::TraceRange tr("ptf_get_c");
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
  return spec_out(h, h->s, sol, where, state_map(h), h->k0mode, h->slo);  // s + its low part, exact in FP64
}

int ptf_set_sol(ptf_handle* h, const double* sol, int32_t where) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol) return fail(h, PTF_ERR_ARG, "null field");
  if (check_where(h, where)) return PTF_ERR_ARG;
  int rc = spec_in(h, sol, where, h->s, state_map(h), h->slo);  // split into s and its low part
  if (rc) return rc;
  if (h->k0mode) {
    const double2* src = where == PTF_HOST ? (const double2*)h->stage : (const double2*)sol;
    cudaError_t e = launch_k0_from_spec(src, h->rows * h->nkr, h->cfg.batch, h->k0, h->stream);
    h->launches++;
    if (e != cudaSuccess) return cuda_fail(h, e, "k = 0 mode seed");
  }
  h->ab_valid = false;
  h->have_c = true;
  if (where == PTF_HOST) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "set_sol");
  }
  return PTF_OK;
}

int ptf_step(ptf_handle* h, int64_t nsteps) {
  ptf::TraceRange tr("ptf_step");
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (nsteps < 0) return fail(h, PTF_ERR_ARG, "nsteps must be >= 0");
  if (!h->have_flow) return fail(h, PTF_ERR_STATE, "no flow set (ptf_set_flow_arrays)");
  if (!h->have_c) return fail(h, PTF_ERR_STATE, "no initial condition (ptf_set_c / ptf_set_sol)");
  return h->fp32 ? do_steps<float>(h, nsteps) : do_steps<double>(h, nsteps);
}

int ptf_calcN(ptf_handle* h, const double* sol, double* N, int32_t where) {
  ptf::TraceRange tr("ptf_calcN");
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (!sol || !N) return fail(h, PTF_ERR_ARG, "null field");
  if (!h->have_flow) return fail(h, PTF_ERR_STATE, "no flow set (ptf_set_flow_arrays)");
  if (check_where(h, where)) return PTF_ERR_ARG;
  // The input goes to a scratch state buffer (acc: free between steps), so
  // the handle's solution is untouched; the intermediates are recomputed by
  // the next step.
  void* sbuf = h->acc;
  if (h->flow_tv) {  // calcN! evaluates a time-varying flow at clock.t
    cudaError_t e = h->fp32 ? eval_flow<float>(h, h->t) : eval_flow<double>(h, h->t);
    if (e != cudaSuccess) return cuda_fail(h, e, "flow evaluation");
  }
  int rc = spec_in(h, sol, where, sbuf, state_map(h));  // read as a state by the prologue
  if (!rc) rc = h->fp32 ? calcN_impl<float>(h, sbuf) : calcN_impl<double>(h, sbuf);
  if (rc) return rc;
  return spec_out(h, sbuf, N, where, lay_map(h));  // the forward pass writes an intermediate
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
  int err = 0;
  e = cudaMemcpy(&err, h->err_dev, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(h, e, "error flag");
  if (err) return fail(h, PTF_ERR_CUDA, "a kernel gave up waiting for its bulk copies (bounded wait ran out)");
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
  drop_graph(h);
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

int ptf_set_schedule(ptf_handle* h, int32_t solves_per_group, int32_t branches, int32_t use_graph) {
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (solves_per_group < 0) return fail(h, PTF_ERR_ARG, "solves_per_group must be >= 0 (0: automatic)");
  if (branches < 1 || branches > 4) return fail(h, PTF_ERR_ARG, "branches must be 1..4");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  h->group = solves_per_group;
  h->branches = branches;
  h->use_graph = use_graph ? 1 : 0;
  drop_graph(h);
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

int ptf_get_tuning(const ptf_handle* h, ptf_tuning* out) {
  if (!h || !out) return fail(nullptr, PTF_ERR_ARG, "null argument");
  *out = current_tuning(h);
  return PTF_OK;
}

int ptf_set_tuning(ptf_handle* h, const ptf_tuning* t) {
  if (!h || !t) return fail(nullptr, PTF_ERR_ARG, "null argument");
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "synchronize");
  return apply_tuning(h, *t);
}

int ptf_autotune(ptf_handle* h, int32_t trial_steps, int32_t flags) {
  ptf::TraceRange tr("ptf_autotune");
  if (!h) return fail(nullptr, PTF_ERR_ARG, "null handle");
  if (trial_steps < 1 || trial_steps > 1000) return fail(h, PTF_ERR_ARG, "trial_steps must be in 1..1000");
  if (!h->have_flow) return fail(h, PTF_ERR_STATE, "no flow set (ptf_set_flow_arrays)");
  if (h->profiling) return fail(h, PTF_ERR_STATE, "per-pass timing is on (ptf_profile)");
  const std::string key = tuning_key(h);
  if (!(flags & PTF_TUNE_FORCE)) {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) return apply_tuning(h, it->second);
  }
  const int rc = h->fp32 ? autotune_impl<float>(h, trial_steps) : autotune_impl<double>(h, trial_steps);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_tune_mutex);
  g_tune_cache[key] = current_tuning(h);
  return PTF_OK;
}

}  // extern "C"
