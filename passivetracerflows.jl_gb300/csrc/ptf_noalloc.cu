// ptf_calcN2d_noalloc: the 2D FP64 advective term without any device
// allocation.
//
// Who needs this: a host that owns every byte of device memory through its
// own pool and does not let a library call cudaMalloc/cudaFree behind its
// back (a Julia process whose CUDA.jl pool holds the device budget is one),
// and a time-critical loop that cannot pay the device-wide synchronisation
// that cudaFree (and often cudaMalloc) imposes.  Such a caller passes its own
// input and output buffers; the intermediates live in the fixed scratch array
// below instead of in a handle.
//
// The scratch is a file-scope __device__ array of PTF_NOALLOC_SCRATCH_BYTES.
// Every GPU that loads this library holds it until the process exits.  Host
// code cannot use the array's name as a device address, so the first call on
// each device looks the address up with cudaGetSymbolAddress (that device
// current) and uploads the FFT twiddle tables into it with a synchronous
// copy; make that first call before any stream capture.  All calls share the
// one array and it keeps the last call's contents: calls that overlap on the
// GPU (different streams, or different host threads) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ptf.h"
#include "ptf_internal.h"

using namespace ptf;

namespace {

constexpr size_t kScratchBytes = PTF_NOALLOC_SCRATCH_BYTES;
// Twiddle tables for every supported length 16..4096 sit at the start of the
// scratch: length n starts at complex offset n - 16 (sum of smaller lengths).
constexpr size_t kTwiddleElems = 4096 * 2 - 16;
constexpr size_t kTwiddleBytes = kTwiddleElems * sizeof(double2);

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_base[kMaxDevices] = {nullptr};
// Failures are reported through ptf_last_error(NULL).
int fail(int code, const std::string& m) { set_global_error(m); return code; }

void host_twiddles(std::vector<double2>& all) {
  all.assign(kTwiddleElems, make_double2(0, 0));
  for (int n = 16; n <= 4096; n *= 2) {
    double2* t = all.data() + (n - 16);
    for (int m = 0; m < n; ++m) {
      // exp(-2 pi i m / n) by octant symmetry of host libm values
      const long long q = (4LL * m) / n, r = m - q * (n / 4);
      double c0, s0;
      if (2 * r <= n / 4) { const double th = 2.0 * M_PI * ((double)r / n); c0 = std::cos(th); s0 = std::sin(th); }
      else { const double th = 2.0 * M_PI * ((double)(n / 4 - r) / n); c0 = std::sin(th); s0 = std::cos(th); }
      double c, s;
      switch (q) { case 0: c = c0; s = s0; break; case 1: c = -s0; s = c0; break;
                   case 2: c = -c0; s = -s0; break; default: c = s0; s = -c0; break; }
      t[m] = make_double2(c, -s);
    }
  }
}

// Once per device, with that device current.
int setup_device(int dev, unsigned char** base) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= kMaxDevices) return fail(PTF_ERR_UNSUPPORTED, "device ordinal out of range");
  if (!g_base[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return fail(PTF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    std::vector<double2> tw;
    host_twiddles(tw);
    e = cudaMemcpy(p, tw.data(), kTwiddleBytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("twiddle upload: ") + cudaGetErrorString(e));
    g_base[dev] = p;
  }
  *base = (unsigned char*)g_base[dev];
  return PTF_OK;
}

inline bool pow2_in_range(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Scratch bytes a grid needs: twiddles, four pitched spectral fields, two flow fields.
size_t scratch_need(int nx, int ny) {
  const size_t pitch = ((size_t)(nx / 2 + 1) + 7) / 8 * 8;
  const size_t spec = align256((size_t)ny * pitch * sizeof(double2));
  const size_t phys = align256((size_t)nx * ny * sizeof(double));
  return align256(kTwiddleBytes) + 4 * spec + 2 * phys;
}

}  // namespace

extern "C" {

int ptf_calcN2d_noalloc(int32_t nx, int32_t ny, double Lx, double Ly, const double* sol, const double* u,
                        const double* v, double* N, void* stream) {
  if (!pow2_in_range(nx) || !pow2_in_range(ny)) return fail(PTF_ERR_ARG, "nx and ny must be powers of two in [16, 4096]");
  if (!(Lx > 0) || !(Ly > 0)) return fail(PTF_ERR_ARG, "domain lengths must be positive");
  if (!sol || !u || !v || !N) return fail(PTF_ERR_ARG, "null device pointer");
  const size_t need = scratch_need(nx, ny);
  if (need > kScratchBytes)
    return fail(PTF_ERR_MEMORY, "grid needs " + std::to_string(need) + " scratch bytes; the fixed scratch holds " +
                                    std::to_string(kScratchBytes) + " (e.g. 512x512 fits, 1024x1024 does not)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  unsigned char* base = nullptr;
  int rc = setup_device(dev, &base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int nkr = nx / 2 + 1;
  const int pitch = (nkr + 7) / 8 * 8;
  const size_t spec = align256((size_t)ny * pitch * sizeof(double2));
  const size_t phys = align256((size_t)nx * ny * sizeof(double));
  const double2* twx = (const double2*)base + (nx - 16);
  const double2* twy = (const double2*)base + (ny - 16);
  unsigned char* p = base + align256(kTwiddleBytes);
  double2* S = (double2*)p;  p += spec;   // sol in the pitched layout, then N
  double2* A = (double2*)p;  p += spec;
  double2* B = (double2*)p;  p += spec;
  double2* NX = (double2*)p; p += spec;
  double* U = (double*)p;    p += phys;   // flow scaled by -1/(2 nx ny)
  double* V = (double*)p;
  // Nx pad columns are never written by the row pass: start them at zero.
  e = cudaMemsetAsync(NX, 0, spec, st);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e));
  e = launch_spec_in<double>((const double2*)sol, S, nkr, pitch, ny, st);
  if (e == cudaSuccess) e = launch_real_in<double>(u, U, (long long)nx * ny, -1.0 / (2.0 * nx * ny), st);
  if (e == cudaSuccess) e = launch_real_in<double>(v, V, (long long)nx * ny, -1.0 / (2.0 * nx * ny), st);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("input conversion: ") + cudaGetErrorString(e));

  const int W = default_lines_per_block<double>(ny, true, pitch);
  const int P = default_lines_per_block<double>(nx, false, ny / 2);

  ColArgs<double> ca;
  std::memset(&ca, 0, sizeof(ca));
  ca.s = S; ca.A = A; ca.B = B; ca.tw = twy;
  ca.dk = 2 * M_PI / Ly;
  ca.stride = pitch; ca.mode = COL_PROLOGUE; ca.do_inverse = 1;
  ca.tplane = (long long)ny * pitch;
  e = launch_col<double>(ny, ca, W, pitch / W, 1, st);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("column pass: ") + cudaGetErrorString(e));
  RowArgs<double> ra;
  std::memset(&ra, 0, sizeof(ra));
  ra.A = A; ra.B = B; ra.out = NX; ra.u = U; ra.v = V; ra.tw = twx;
  ra.dkx = 2 * M_PI / Lx; ra.scale = 1.0;
  ra.rows = ny; ra.pitch = pitch; ra.mode = ROW_RHS; ra.park_slots = 1;
  e = launch_row<double>(nx, ra, P, (ny / 2) / P, 1, st);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("row pass: ") + cudaGetErrorString(e));
  ColArgs<double> cf;
  std::memset(&cf, 0, sizeof(cf));
  cf.nxin = NX; cf.nout = S; cf.tw = twy;
  cf.dk = 2 * M_PI / Ly;
  cf.stride = pitch; cf.mode = COL_FWD_N; cf.do_inverse = 0;
  cf.tplane = (long long)ny * pitch;
  e = launch_col<double>(ny, cf, W, pitch / W, 1, st);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("column pass: ") + cudaGetErrorString(e));
  e = launch_spec_out<double>(S, (double2*)N, nkr, pitch, ny, st);
  if (e != cudaSuccess) return fail(PTF_ERR_CUDA, std::string("output conversion: ") + cudaGetErrorString(e));
  return PTF_OK;
}

}  // extern "C"
