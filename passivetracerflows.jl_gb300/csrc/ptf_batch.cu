// Batched form: many independent square 2D solves of different sizes stepped
// together on one GPU.
//
// Solves of the same size share a bucket (fixed number of slots, one set of
// fields per slot).  The work of an RK4 stage over every bucket is a list of
// items -- the row-pass tiles of every bucket, then the column-pass tiles.
// By default a stage is a row launch and a column launch, one block per
// item.  With cfg.persistent it is ONE launch of a persistent kernel
// (batch_stage_kernel): blocks take items from an atomic counter and a
// column tile of bucket b starts once all row tiles of b are done (a
// per-bucket completion counter; the wait is bounded and sets an error flag
// if it ever runs out; items are handed out in order, so every row tile a
// column tile waits for is already running on a resident block, and the
// wait always ends).  After the four stages a clock
// kernel advances each active solve's t and step and retires solves that
// reached their own step count (their fields are no longer written).  One
// step is captured once in a CUDA graph and replayed.
//
// Per-slot parameters give each solve its own kappa, dt, clock and flow: an
// array (steady) or the analytic cellular flow re-evaluated at clock.t
// (PTF_CLOCK_T, as the reference) or at each stage time (PTF_STAGE_T).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/ptf.h"
#include "ptf_batch_kern.cuh"
#include "ptf_trace.h"

using namespace ptf;

namespace ptf {

template <typename T> __global__ void batch_clock_kernel(SlotParams<T>* slots, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SlotParams<T>& s = slots[i];
  if (!s.active) return;
  s.t += s.dtd;
  s.step += 1;
  if (s.step >= s.nsteps) s.active = 0;
  else if (s.flow_kind == FLOW_CELLULAR) slot_phases(s);
}
// The flow phases of one slot after its parameters were uploaded.
template <typename T> __global__ void batch_phase_kernel(SlotParams<T>* slot) {
  if (slot->flow_kind == FLOW_CELLULAR) slot_phases(*slot);
}

#define PTF_EXTERN_STAGE(T, M)                                                                              \
  extern template cudaError_t launch_batch_stage<T, M>(const BatchPlan<T>*, unsigned int*, int*, T, int, size_t, \
                                                       cudaStream_t);                                          \
  extern template cudaError_t setup_batch_stage<T, M>(size_t, int*);
#define PTF_EXTERN_ITEMS(T, M)                                                                           \
  extern template cudaError_t launch_batch_cols<T, M>(const BatchPlan<T>*, int, size_t, cudaStream_t); \
  extern template cudaError_t setup_batch_items<T, M>(size_t);
PTF_EXTERN_ITEMS(float, COL_RK4_1) PTF_EXTERN_ITEMS(float, COL_RK4_2) PTF_EXTERN_ITEMS(float, COL_RK4_3)
PTF_EXTERN_ITEMS(float, COL_RK4_4) PTF_EXTERN_ITEMS(double, COL_RK4_1) PTF_EXTERN_ITEMS(double, COL_RK4_2)
PTF_EXTERN_ITEMS(double, COL_RK4_3) PTF_EXTERN_ITEMS(double, COL_RK4_4)
#undef PTF_EXTERN_ITEMS
extern template cudaError_t launch_batch_rows<float>(const BatchPlan<float>*, float, int, size_t, cudaStream_t);
extern template cudaError_t launch_batch_rows<double>(const BatchPlan<double>*, double, int, size_t, cudaStream_t);
PTF_EXTERN_STAGE(float, COL_RK4_1) PTF_EXTERN_STAGE(float, COL_RK4_2) PTF_EXTERN_STAGE(float, COL_RK4_3)
PTF_EXTERN_STAGE(float, COL_RK4_4) PTF_EXTERN_STAGE(double, COL_RK4_1) PTF_EXTERN_STAGE(double, COL_RK4_2)
PTF_EXTERN_STAGE(double, COL_RK4_3) PTF_EXTERN_STAGE(double, COL_RK4_4)
#undef PTF_EXTERN_STAGE

}  // namespace ptf

namespace {

struct Bucket {
  int n = 0, pitch = 0, cap = 0;
  double L = 0;
  void *s = nullptr, *si = nullptr, *acc = nullptr, *A = nullptr, *B = nullptr, *Nx = nullptr;
  void *u = nullptr, *v = nullptr, *phys = nullptr, *tw = nullptr;
  void* slo = nullptr;             // FP32: the state's low part (compensated state, stage_combine)
  int slot_base = 0;               // first entry of the bucket in the slot parameter array
  std::vector<long long> owner;    // solve id per slot, -1 when free
  int W = 1, P = 1;                // single-slot launch shapes (admission, readback)
  size_t bytes = 0;                // device bytes of the bucket's fields
  std::vector<void*> allocs;       // the bucket's own device allocations
  size_t alloc_bytes = 0;          // their total
  bool dead = false;               // released (its slot range stays reserved for a new bucket)
  int span = 0;                    // slots of the parameter table reserved for this entry (>= cap)
};

struct SolveRef {
  int bucket, slot;
  ptf_solve_desc desc;
};

}  // namespace

struct ptf_batch {
  ptf_batch_config cfg;
  bool fp32 = false;
  cudaStream_t stream = nullptr;
  std::vector<Bucket> buckets;
  std::vector<void*> allocs;
  size_t bytes = 0;
  // slot parameters (global index = bucket.slot_base + slot)
  int slot_cap = 0, slot_used = 0;
  void* slots_dev = nullptr;
  std::vector<unsigned char> slots_host;
  void* slot_list_dev = nullptr;  // per-bucket active-slot lists, concatenated
  void* plan_dev = nullptr;
  // FP64 k = 0 mode (FP32 batches): per slot {s, stage input, acc, L(0,0)},
  // then 64 sum partials and one sum for readback
  bool k0mode = false;
  double* k0 = nullptr;
  double k0_seed[3] = {0, 0, 0};  // host source of the seed copy (kept alive until it completes)
  unsigned int* ctr = nullptr;
  int* err = nullptr;
  double* stage = nullptr;
  size_t stage_elems = 0;
  std::map<long long, SolveRef> solves;
  long long next_id = 1;
  bool plan_dirty = true;
  long long bucket_gen = 0, plan_gen = -1;  // bumped when a bucket's buffers change
  unsigned long long spin_limit = 0;         // persistent kernel's bounded wait (0: default)
  unsigned int wait_extra = 0;               // test hook: row items a column item waits for beyond the real ones
  int plan_total = 0, plan_row_total = 0;
  std::vector<int> plan_lists;      // active slots per bucket of the current plan
  std::vector<int> plan_buckets;
  int grid = 0;
  size_t smem = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long long launches = 0;
  std::string error;
};

namespace {

int bfail(ptf_batch* b, int code, const std::string& m) {
  if (b) b->error = m; else set_global_error(m);
  return code;
}
int bcuda(ptf_batch* b, cudaError_t e, const char* what) {
  return bfail(b, PTF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
size_t ec(const ptf_batch* b) { return b->fp32 ? sizeof(float2) : sizeof(double2); }
size_t er(const ptf_batch* b) { return b->fp32 ? sizeof(float) : sizeof(double); }
size_t slot_param_bytes(const ptf_batch* b) { return b->fp32 ? sizeof(SlotParams<float>) : sizeof(SlotParams<double>); }

bool balloc(ptf_batch* b, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) { *p = nullptr; cudaGetLastError(); return false; }
  b->allocs.push_back(*p);
  b->bytes += bytes;
  return cudaMemsetAsync(*p, 0, bytes, b->stream) == cudaSuccess;
}

bool bucket_alloc(ptf_batch* b, Bucket& k, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) != cudaSuccess) { *p = nullptr; cudaGetLastError(); return false; }
  k.allocs.push_back(*p);
  k.alloc_bytes += bytes;
  b->bytes += bytes;
  return cudaMemsetAsync(*p, 0, bytes, b->stream) == cudaSuccess;
}

void free_bucket(ptf_batch* b, Bucket& k) {
  cudaStreamSynchronize(b->stream);
  for (void* p : k.allocs) cudaFree(p);
  k.allocs.clear();
  b->bytes -= std::min(b->bytes, k.alloc_bytes);
  k.alloc_bytes = 0;
  k.s = k.si = k.acc = k.A = k.B = k.Nx = k.u = k.v = k.phys = k.tw = k.slo = nullptr;
  k.dead = true;
  k.n = 0;
  b->bucket_gen++;
  b->plan_dirty = true;
}

// Under a memory budget, release the buckets that hold no solve (their slot
// ranges stay reserved and are reused by later buckets that fit in them).
void reclaim_empty_buckets(ptf_batch* b) {
  for (Bucket& k : b->buckets) {
    if (k.dead) continue;
    bool empty = true;
    for (long long o : k.owner) if (o >= 0) { empty = false; break; }
    if (empty) free_bucket(b, k);
  }
}

size_t per_slot_bytes(const ptf_batch* b, int n) {
  const int pitch = ((n / 2 + 1) + 7) / 8 * 8;
  return (b->fp32 ? 7 : 6) * (size_t)n * pitch * ec(b) + 3 * (size_t)n * n * er(b);
}

void host_twiddles_d(std::vector<double>& out, int n) {
  out.resize(2 * (size_t)n);
  for (int m = 0; m < n; ++m) {
    const long long q = (4LL * m) / n, r = m - q * (n / 4);
    double c0, s0;
    if (2 * r <= n / 4) { const double th = 2.0 * M_PI * ((double)r / n); c0 = std::cos(th); s0 = std::sin(th); }
    else { const double th = 2.0 * M_PI * ((double)(n / 4 - r) / n); c0 = std::sin(th); s0 = std::cos(th); }
    double c, s;
    switch (q) { case 0: c = c0; s = s0; break; case 1: c = -s0; s = c0; break;
                 case 2: c = -c0; s = -s0; break; default: c = s0; s = -c0; break; }
    out[2 * m] = c;
    out[2 * m + 1] = -s;
  }
}

int default_cap(const ptf_batch* b, int n) {
  if (b->cfg.slots_per_bucket > 0) return b->cfg.slots_per_bucket;
  // about 1 GB of fields per bucket, between 4 and 256 slots
  const size_t ps = per_slot_bytes(b, n);
  long long c = (long long)((1ull << 30) / ps);
  return (int)std::max(4LL, std::min(256LL, c));
}

int new_bucket(ptf_batch* b, int n, double L) {
  Bucket k;
  k.n = n;
  k.L = L;
  k.pitch = ((n / 2 + 1) + 7) / 8 * 8;
  int cap = default_cap(b, n);
  const size_t ps = per_slot_bytes(b, n);
  if (b->cfg.memory_budget > 0) {
    long long left = b->cfg.memory_budget - (long long)b->bytes;
    if (left < (long long)ps) {  // empty buckets of other sizes may hold the room
      reclaim_empty_buckets(b);
      left = b->cfg.memory_budget - (long long)b->bytes;
    }
    const long long fit = left > 0 ? left / (long long)ps : 0;
    if (fit < 1) return -1;
    cap = (int)std::min<long long>(cap, fit);
  }
  // a released entry whose slot range is large enough, else a new entry
  int reuse = -1;
  for (size_t i = 0; i < b->buckets.size(); ++i)
    if (b->buckets[i].dead && b->buckets[i].span >= 1 && (reuse < 0 || b->buckets[i].span > b->buckets[reuse].span))
      reuse = (int)i;
  if (reuse >= 0) {
    cap = std::min(cap, b->buckets[reuse].span);
  } else {
    if ((int)b->buckets.size() >= kMaxBuckets) return -1;
    if (b->slot_used + cap > b->slot_cap) cap = b->slot_cap - b->slot_used;
  }
  if (cap < 1) return -1;
  k.cap = cap;
  const size_t sc = (size_t)cap * n * k.pitch * ec(b), sp = (size_t)cap * n * n * er(b);
  bool ok = bucket_alloc(b, k, &k.s, sc) && bucket_alloc(b, k, &k.si, sc) && bucket_alloc(b, k, &k.acc, sc) &&
            bucket_alloc(b, k, &k.A, sc) && bucket_alloc(b, k, &k.B, sc) && bucket_alloc(b, k, &k.Nx, sc) &&
            bucket_alloc(b, k, &k.u, sp) && bucket_alloc(b, k, &k.v, sp) && bucket_alloc(b, k, &k.phys, sp) &&
            bucket_alloc(b, k, &k.tw, (size_t)n * ec(b)) && (!b->fp32 || bucket_alloc(b, k, &k.slo, sc));
  if (!ok) {
    cudaStreamSynchronize(b->stream);
    for (void* p : k.allocs) cudaFree(p);
    b->bytes -= std::min(b->bytes, k.alloc_bytes);
    return -2;
  }
  std::vector<double> tw;
  host_twiddles_d(tw, n);
  cudaError_t e;
  if (b->fp32) {
    std::vector<float> tf(tw.begin(), tw.end());
    e = cudaMemcpyAsync(k.tw, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  } else {
    e = cudaMemcpyAsync(k.tw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  }
  if (e != cudaSuccess) {
    cudaStreamSynchronize(b->stream);
    for (void* p : k.allocs) cudaFree(p);
    b->bytes -= std::min(b->bytes, k.alloc_bytes);
    return -2;
  }
  k.owner.assign(cap, -1);
  k.bytes = ps * cap;
  k.W = b->fp32 ? default_lines_per_block<float>(n, true, k.pitch) : default_lines_per_block<double>(n, true, k.pitch);
  k.P = b->fp32 ? default_lines_per_block<float>(n, false, n / 2) : default_lines_per_block<double>(n, false, n / 2);
  b->bucket_gen++;
  b->plan_dirty = true;
  if (reuse >= 0) {
    Bucket& old = b->buckets[reuse];
    k.slot_base = old.slot_base;
    k.span = old.span;  // slots of the range beyond the new capacity stay inactive
    old = k;
    return reuse;
  }
  k.slot_base = b->slot_used;
  k.span = cap;
  b->slot_used += cap;
  b->buckets.push_back(k);
  return (int)b->buckets.size() - 1;
}

template <typename T> SlotParams<T>& host_slot(ptf_batch* b, int g) {
  return reinterpret_cast<SlotParams<T>*>(b->slots_host.data())[g];
}

template <typename T> int upload_slot(ptf_batch* b, int g) {
  cudaError_t e = cudaMemcpyAsync((SlotParams<T>*)b->slots_dev + g, &host_slot<T>(b, g), sizeof(SlotParams<T>),
                                  cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "slot upload");
  return PTF_OK;
}
// One slot's device parameters back into the host copy.
template <typename T> int download_slot(ptf_batch* b, int g) {
  cudaError_t e = cudaMemcpyAsync(&host_slot<T>(b, g), (SlotParams<T>*)b->slots_dev + g, sizeof(SlotParams<T>),
                                  cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "slot download");
  return PTF_OK;
}
template <typename T> int download_slots(ptf_batch* b) {
  cudaError_t e = cudaMemcpyAsync(b->slots_host.data(), b->slots_dev, (size_t)b->slot_used * sizeof(SlotParams<T>),
                                  cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "slot download");
  return PTF_OK;
}

// Single-slot pass launches (admission and readback) on the regular kernels.
template <typename T> ColArgs<T> slot_col(ptf_batch* b, const Bucket& k, int slot, int mode) {
  typedef typename cplx_of<T>::type C;
  ColArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  const size_t off = (size_t)slot * k.n * k.pitch;
  a.s = (C*)k.s + off; a.si = (C*)k.si + off; a.acc = (C*)k.acc + off;
  a.slo = k.slo ? (C*)k.slo + off : nullptr;
  a.A = (C*)k.A + off; a.B = (C*)k.B + off; a.nxin = (C*)k.Nx + off;
  a.tw = (const C*)k.tw;
  a.stride = k.pitch; a.mode = mode; a.do_inverse = 1;
  a.ylog = kBatchYlog; a.priv = 1;  // the single-handle layouts (spec_index, SpecMap)
  a.bstride = (long long)k.n * k.pitch; a.tplane = a.bstride;
  (void)b;
  return a;
}
template <typename T> RowArgs<T> slot_row(ptf_batch* b, const Bucket& k, int slot, int mode) {
  typedef typename cplx_of<T>::type C;
  RowArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  const size_t off = (size_t)slot * k.n * k.pitch, poff = (size_t)slot * k.n * k.n;
  a.A = (const C*)k.A + off; a.out = (C*)k.Nx + off;
  a.cin = (const T*)k.phys + poff; a.cout = (T*)k.phys + poff;
  a.tw = (const C*)k.tw;
  a.rows = k.n; a.pitch = k.pitch; a.mode = mode; a.park_slots = 1; a.ylog = kBatchYlog;
  a.bstride = (long long)k.n * k.pitch; a.pstride = (long long)k.n * k.n;
  (void)b;
  return a;
}

template <typename T> int admit(ptf_batch* b, Bucket& k, int slot, const ptf_solve_desc& d, const double* c0,
                                const double* u, const double* v, long long id) {
  const long long np = (long long)k.n * k.n;
  const size_t poff = (size_t)slot * np;
  cudaError_t e = cudaMemcpyAsync(b->stage, c0, np * sizeof(double), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = launch_real_in<T>(b->stage, (T*)k.phys + poff, np, 1.0, b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "admission copy");
  if (b->k0mode) {
    // the slot's (0,0) mode in FP64: s = sum of c0 (compensated, from the FP64
    // input), stage input and accumulator 0, and L(0,0) (non-zero only for
    // hyperdiffusion of order 0, which damps every mode alike)
    double* q = b->k0 + 4 * (size_t)(k.slot_base + slot);
    e = launch_solve_sums<double>(b->stage, np, 1, b->k0 + 4 * (size_t)b->slot_cap, q, 4, b->stream);
    b->k0_seed[0] = 0.0;
    b->k0_seed[1] = 0.0;
    b->k0_seed[2] = d.nkappah == 0 ? -d.kappah : 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(q + 1, b->k0_seed, 3 * sizeof(double), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "k = 0 mode seed");
    b->launches += 2;
  }
  RowArgs<T> r = slot_row<T>(b, k, slot, ROW_R2C);
  r.scale = (T)0.5;
  e = launch_row<T>(k.n, r, k.P, (k.n / 2) / k.P, 1, b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "admission row pass");
  ColArgs<T> c = slot_col<T>(b, k, slot, COL_FWD_STORE);
  c.dk = (T)(2 * M_PI / d.L);
  e = launch_col<T>(k.n, c, k.W, k.pitch / k.W, 1, b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "admission column pass");
  b->launches += 3;
  if (d.flow_kind == PTF_FLOW_ARRAYS) {
    const double sc = -1.0 / (2.0 * (double)np);
    const double* src[2] = {u, v};
    void* dst[2] = {k.u, k.v};
    for (int q = 0; q < 2; ++q) {
      e = cudaMemcpyAsync(b->stage, src[q], np * sizeof(double), cudaMemcpyHostToDevice, b->stream);
      if (e == cudaSuccess) e = launch_real_in<T>(b->stage, (T*)dst[q] + poff, np, sc, b->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
      if (e != cudaSuccess) return bcuda(b, e, "flow upload");
      b->launches++;
    }
  }
  const int g = k.slot_base + slot;
  SlotParams<T>& sp = host_slot<T>(b, g);
  std::memset(&sp, 0, sizeof(sp));
  sp.t = 0.0; sp.dtd = d.dt; sp.step = 0; sp.nsteps = d.nsteps;
  sp.kappa = (T)d.kappa; sp.eta = (T)d.eta; sp.kappah = (T)d.kappah; sp.nkappah = d.nkappah;
  sp.dt = (T)d.dt;
  sp.dkx = sp.dky = (T)(2 * M_PI / d.L);
  sp.U = (T)d.U; sp.eps = (T)d.eps; sp.omega = (T)d.omega; sp.Kx = d.Kx; sp.Ky = d.Ky;
  sp.flow_kind = d.flow_kind == PTF_FLOW_CELLULAR ? FLOW_CELLULAR : FLOW_ARRAYS;
  sp.time_mode = d.time_mode == PTF_STAGE_T ? 1 : 0;
  sp.active = d.nsteps > 0 ? 1 : 0;
  k.owner[slot] = id;
  b->plan_dirty = true;
  int rc = upload_slot<T>(b, g);
  if (rc) return rc;
  batch_phase_kernel<T><<<1, 1, 0, b->stream>>>((SlotParams<T>*)b->slots_dev + g);
  b->launches++;
  e = cudaStreamSynchronize(b->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return bcuda(b, e, "slot phases");
  return download_slot<T>(b, g);
}

// Rebuild the work plan over the slots that are still active.
template <typename T> int build_plan(ptf_batch* b) {
  typedef typename cplx_of<T>::type C;
  if (!b->plan_dirty) return PTF_OK;
  int rc = download_slots<T>(b);
  if (rc) return rc;
  BatchPlan<T> plan;
  std::memset(&plan, 0, sizeof(plan));
  std::vector<int> lists;
  std::vector<int> list_off;
  int nb = 0;
  for (size_t bi = 0; bi < b->buckets.size(); ++bi) {
    const Bucket& k = b->buckets[bi];
    std::vector<int> act;
    for (int s = 0; s < k.cap; ++s)
      if (k.owner[s] >= 0 && host_slot<T>(b, k.slot_base + s).active) act.push_back(s);
    if (act.empty()) continue;
    list_off.push_back((int)lists.size());
    lists.push_back(-1 - (int)bi);  // bucket marker keeps plans of different buckets distinct
    lists.insert(lists.end(), act.begin(), act.end());
    BucketPlan<T>& bp = plan.b[nb];
    bp.n = k.n;
    const int tplN = b->fp32 ? 0 : 0;
    (void)tplN;
    ColArgs<T>& c = bp.col;
    c.s = (C*)k.s; c.si = (C*)k.si; c.acc = (C*)k.acc; c.A = (C*)k.A; c.B = (C*)k.B; c.nxin = (const C*)k.Nx;
    c.slo = (C*)k.slo;
    c.tw = (const C*)k.tw;
    c.stride = k.pitch; c.do_inverse = 1;
    c.ylog = kBatchYlog; c.priv = 1;
    c.bstride = (long long)k.n * k.pitch; c.tplane = c.bstride;
    c.slots = (const SlotParams<T>*)b->slots_dev + k.slot_base;
    c.k0 = b->k0mode ? b->k0 + 4 * (size_t)k.slot_base : nullptr;
    c.nslots = (int)act.size();
    c.slot_cols = k.pitch;
    RowArgs<T>& r = bp.row;
    r.A = (const C*)k.A; r.B = (const C*)k.B; r.out = (C*)k.Nx;
    r.u = (const T*)k.u; r.v = (const T*)k.v;
    r.tw = (const C*)k.tw;
    r.dkx = (T)0;  // set below from the bucket's first solve (square, same L per bucket)
    r.scale = (T)1;
    r.rows = k.n; r.pitch = k.pitch; r.mode = ROW_RHS; r.park_slots = 1; r.ylog = kBatchYlog;
    r.bstride = c.bstride; r.pstride = (long long)k.n * k.n; r.fstride = r.pstride;
    r.slots = c.slots;
    r.nslots = c.nslots;
    r.fscale = (T)(-1.0 / (2.0 * (double)k.n * k.n));
    const SlotParams<T>& s0 = host_slot<T>(b, k.slot_base + act[0]);
    r.dkx = s0.dkx;
    int tpl = 1, ctpl = 1;
    switch (k.n) {
#define PTF_CASE(n) case n: tpl = pass_tpl<T, n>(); ctpl = col_tpl<T, n>(); break;
      PTF_BATCH_SIZES(PTF_CASE)
#undef PTF_CASE
      default: return bfail(b, PTF_ERR_UNSUPPORTED, "grid size not built for the batched form");
    }
    const int lines = kBatchThreads / tpl, clines = kBatchThreads / ctpl;
    bp.row_items = (int)(((long long)c.nslots * (k.n / 2) + lines - 1) / lines);
    bp.col_items = (int)(((long long)c.nslots * k.pitch + clines - 1) / clines);
    ++nb;
  }
  std::vector<int> pbk;
  for (size_t bi = 0; bi < b->buckets.size(); ++bi) pbk.push_back(b->buckets[bi].cap);
  if (b->gexec && lists == b->plan_lists && pbk == b->plan_buckets && b->plan_gen == b->bucket_gen) {
    b->plan_dirty = false;  // same active set: keep the plan and the captured step
    return PTF_OK;
  }
  b->plan_lists = lists;
  b->plan_buckets = pbk;
  b->plan_gen = b->bucket_gen;
  plan.nb = nb;
  plan.spin_limit = b->spin_limit;
  plan.wait_extra = b->wait_extra;
  int off = 0;
  for (int i = 0; i < nb; ++i) { plan.b[i].row_begin = off; off += plan.b[i].row_items; }
  plan.row_total = off;
  for (int i = 0; i < nb; ++i) { plan.b[i].col_begin = off; off += plan.b[i].col_items; }
  plan.total = off;
  // slot lists
  if (!lists.empty()) {
    if (b->slot_list_dev == nullptr) {
      if (!balloc(b, &b->slot_list_dev, (size_t)b->slot_cap * sizeof(int))) return bfail(b, PTF_ERR_MEMORY, "slot list");
    }
    cudaError_t e = cudaMemcpyAsync(b->slot_list_dev, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return bcuda(b, e, "slot list upload");
    for (int i = 0; i < nb; ++i) {
      plan.b[i].col.slot_list = (const int*)b->slot_list_dev + list_off[i] + 1;  // skip the marker
      plan.b[i].row.slot_list = plan.b[i].col.slot_list;
    }
  }
  cudaError_t e = cudaMemcpyAsync(b->plan_dev, &plan, sizeof(plan), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "plan upload");
  b->plan_total = plan.total;
  b->plan_row_total = plan.row_total;
  b->plan_dirty = false;
  if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  return PTF_OK;
}

template <typename T> cudaError_t enqueue_step(ptf_batch* b) {
  const T cs[4] = {(T)0, (T)0.5, (T)0.5, (T)1};
  const BatchPlan<T>* plan = (const BatchPlan<T>*)b->plan_dev;
  if (!b->cfg.persistent) {
    const int rows = b->plan_row_total, cols = b->plan_total - b->plan_row_total;
    for (int st = 0; st < 4; ++st) {
      cudaError_t e = rows > 0 ? launch_batch_rows<T>(plan, cs[st], rows, b->smem, b->stream) : cudaSuccess;
      if (e == cudaSuccess && cols > 0) {
        switch (st) {
          case 0: e = launch_batch_cols<T, COL_RK4_1>(plan, cols, b->smem, b->stream); break;
          case 1: e = launch_batch_cols<T, COL_RK4_2>(plan, cols, b->smem, b->stream); break;
          case 2: e = launch_batch_cols<T, COL_RK4_3>(plan, cols, b->smem, b->stream); break;
          default: e = launch_batch_cols<T, COL_RK4_4>(plan, cols, b->smem, b->stream); break;
        }
      }
      if (e != cudaSuccess) return e;
    }
    batch_clock_kernel<T><<<(b->slot_used + 255) / 256, 256, 0, b->stream>>>((SlotParams<T>*)b->slots_dev, b->slot_used);
    return cudaGetLastError();
  }
  for (int st = 0; st < 4; ++st) {
    cudaError_t e = cudaMemsetAsync(b->ctr, 0, (kMaxBuckets + 1) * sizeof(unsigned int), b->stream);
    if (e != cudaSuccess) return e;
    switch (st) {
      case 0: e = launch_batch_stage<T, COL_RK4_1>(plan, b->ctr, b->err, cs[0], b->grid, b->smem, b->stream); break;
      case 1: e = launch_batch_stage<T, COL_RK4_2>(plan, b->ctr, b->err, cs[1], b->grid, b->smem, b->stream); break;
      case 2: e = launch_batch_stage<T, COL_RK4_3>(plan, b->ctr, b->err, cs[2], b->grid, b->smem, b->stream); break;
      default: e = launch_batch_stage<T, COL_RK4_4>(plan, b->ctr, b->err, cs[3], b->grid, b->smem, b->stream); break;
    }
    if (e != cudaSuccess) return e;
  }
  batch_clock_kernel<T><<<(b->slot_used + 255) / 256, 256, 0, b->stream>>>((SlotParams<T>*)b->slots_dev, b->slot_used);
  return cudaGetLastError();
}

template <typename T> int setup_kernels(ptf_batch* b) {
  b->smem = batch_smem_bytes<T>();
  cudaError_t e;
  int occ = 1 << 30;
  for (int st = 0; st < 4; ++st) {
    int o = 0;
    switch (st) {
      case 0: e = setup_batch_stage<T, COL_RK4_1>(b->smem, &o); break;
      case 1: e = setup_batch_stage<T, COL_RK4_2>(b->smem, &o); break;
      case 2: e = setup_batch_stage<T, COL_RK4_3>(b->smem, &o); break;
      default: e = setup_batch_stage<T, COL_RK4_4>(b->smem, &o); break;
    }
    if (e != cudaSuccess) return bcuda(b, e, "batched kernel set-up");
    occ = std::min(occ, o);
    switch (st) {
      case 0: e = setup_batch_items<T, COL_RK4_1>(b->smem); break;
      case 1: e = setup_batch_items<T, COL_RK4_2>(b->smem); break;
      case 2: e = setup_batch_items<T, COL_RK4_3>(b->smem); break;
      default: e = setup_batch_items<T, COL_RK4_4>(b->smem); break;
    }
    if (e != cudaSuccess) return bcuda(b, e, "batched kernel set-up");
  }
  if (occ < 1) return bfail(b, PTF_ERR_UNSUPPORTED, "batched kernel does not fit on an SM");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->grid = sms * occ;
  return PTF_OK;
}

template <typename T> int step_impl(ptf_batch* b, long long nsteps) {
  int rc = build_plan<T>(b);
  if (rc) return rc;
  if (b->plan_total == 0 || nsteps == 0) return PTF_OK;
  cudaError_t e;
  if (b->cfg.use_graph) {
    if (!b->gexec) {
      e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return bcuda(b, e, "graph capture");
      cudaError_t e2 = enqueue_step<T>(b);
      e = cudaStreamEndCapture(b->stream, &b->graph);
      if (e2 != cudaSuccess) return bcuda(b, e2, "graph capture launch");
      if (e != cudaSuccess) return bcuda(b, e, "graph capture end");
      e = cudaGraphInstantiate(&b->gexec, b->graph, 0);
      if (e != cudaSuccess) return bcuda(b, e, "graph instantiate");
    }
    for (long long i = 0; i < nsteps; ++i) {
      e = cudaGraphLaunch(b->gexec, b->stream);
      if (e != cudaSuccess) return bcuda(b, e, "graph launch");
    }
  } else {
    for (long long i = 0; i < nsteps; ++i) {
      e = enqueue_step<T>(b);
      if (e != cudaSuccess) return bcuda(b, e, "step launch");
    }
  }
  // kernels per step: 4 stage launches (persistent) or up to 4 x (rows + columns), then the clock kernel
  const long long per_step = b->cfg.persistent ? 5 : 4 * ((b->plan_row_total > 0) + (b->plan_total > b->plan_row_total)) + 1;
  b->launches += per_step * nsteps;
  // solves that finished are retired from the plan at the next call
  b->plan_dirty = true;
  return PTF_OK;
}

template <typename T> int get_c_impl(ptf_batch* b, const Bucket& k, int slot, double* c) {
  const long long np = (long long)k.n * k.n;
  RowArgs<T> r = slot_row<T>(b, k, slot, ROW_C2R);
  r.scale = (T)(1.0 / (double)np);
  cudaError_t e = launch_row<T>(k.n, r, k.P, (k.n / 2) / k.P, 1, b->stream);
  const T* phys = (const T*)k.phys + (size_t)slot * np;
  if (b->k0mode) {
    // shift the field so that its sum is the slot's FP64 (0,0) mode
    double* part = b->k0 + 4 * (size_t)b->slot_cap;
    if (e == cudaSuccess) e = launch_solve_sums<T>(phys, np, 1, part, part + 64, 1, b->stream);
    if (e == cudaSuccess)
      e = launch_real_out_shift<T>(phys, b->stage, np, 1, b->k0 + 4 * (size_t)(k.slot_base + slot), part + 64, b->stream);
    b->launches += 2;
  } else if (e == cudaSuccess) {
    e = launch_real_out<T>(phys, b->stage, np, b->stream);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(c, b->stage, np * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "batched readback");
  b->launches += 2;
  return PTF_OK;
}

int validate(ptf_batch* b, const ptf_solve_desc* d) {
  if (!d) return bfail(b, PTF_ERR_ARG, "null solve description");
  if (d->dim != 2) return bfail(b, PTF_ERR_ARG, "the batched form takes 2D solves");
  const int n = d->n;
  if (!(n == 64 || n == 128 || n == 256 || n == 512 || n == 1024))
    return bfail(b, PTF_ERR_ARG, "batched solves are square 2D grids with n in {64, 128, 256, 512, 1024}");
  if (!(d->L > 0)) return bfail(b, PTF_ERR_ARG, "domain length must be positive");
  if (!(d->dt > 0) || !std::isfinite(d->dt)) return bfail(b, PTF_ERR_ARG, "dt must be positive and finite");
  if (d->nsteps < 0) return bfail(b, PTF_ERR_ARG, "nsteps must be >= 0");
  if (d->nkappah < 0) return bfail(b, PTF_ERR_ARG, "nkappah must be >= 0");
  if (d->flow_kind != PTF_FLOW_ARRAYS && d->flow_kind != PTF_FLOW_CELLULAR) return bfail(b, PTF_ERR_ARG, "unknown flow kind");
  if (d->time_mode != PTF_CLOCK_T && d->time_mode != PTF_STAGE_T) return bfail(b, PTF_ERR_ARG, "unknown time mode");
  return PTF_OK;
}

}  // namespace

int64_t ptf::batch_fixed_bytes(const ptf_batch* b) {
  int64_t bytes = (int64_t)b->bytes;
  for (const Bucket& k : b->buckets) bytes -= (int64_t)k.alloc_bytes;
  return bytes;
}
int64_t ptf::batch_slot_bytes(const ptf_batch* b, int n) {
  return (int64_t)per_slot_bytes(b, n) + (int64_t)n * (int64_t)ec(b);  // fields of one slot + the bucket's twiddles
}

extern "C" {

void ptf_batch_config_default(ptf_batch_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->precision = PTF_FP32;
  c->memory_budget = 0;
  c->slots_per_bucket = 0;
  c->use_graph = 1;
  c->max_slots = 4096;
  c->k0_mode = 1;
}

void ptf_solve_desc_default(ptf_solve_desc* d) {
  if (!d) return;
  std::memset(d, 0, sizeof(*d));
  d->dim = 2;
  d->n = 128;
  d->L = 2 * M_PI;
  d->kappa = d->eta = 0.1;
  d->dt = 0.01;
  d->nsteps = 1;
  d->flow_kind = PTF_FLOW_ARRAYS;
  d->time_mode = PTF_CLOCK_T;
  d->U = 1.0;
  d->Kx = d->Ky = 1;
}

int ptf_batch_create(const ptf_batch_config* cfg, ptf_batch** out) {
  if (!cfg || !out) return bfail(nullptr, PTF_ERR_ARG, "ptf_batch_create: null argument");
  *out = nullptr;
  if (cfg->precision != PTF_FP32 && cfg->precision != PTF_FP64) return bfail(nullptr, PTF_ERR_ARG, "precision must be FP64 or FP32");
  if (cfg->memory_budget < 0 || cfg->slots_per_bucket < 0 || cfg->max_slots < 1)
    return bfail(nullptr, PTF_ERR_ARG, "invalid batch limits");
  if (cfg->k0_mode != 0 && cfg->k0_mode != 1) return bfail(nullptr, PTF_ERR_ARG, "k0_mode must be 0 or 1");
  ptf_batch* b = new ptf_batch();
  b->cfg = *cfg;
  b->fp32 = cfg->precision == PTF_FP32;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete b; return bcuda(nullptr, e, "stream create"); }
  b->slot_cap = cfg->max_slots;
  b->slots_host.assign((size_t)b->slot_cap * slot_param_bytes(b), 0);
  bool ok = balloc(b, &b->slots_dev, (size_t)b->slot_cap * slot_param_bytes(b)) &&
            balloc(b, &b->plan_dev, b->fp32 ? sizeof(BatchPlan<float>) : sizeof(BatchPlan<double>)) &&
            balloc(b, (void**)&b->ctr, (kMaxBuckets + 1) * sizeof(unsigned int)) &&
            balloc(b, (void**)&b->err, sizeof(int));
  b->stage_elems = (size_t)1024 * 1024;
  ok = ok && balloc(b, (void**)&b->stage, b->stage_elems * sizeof(double));
  b->k0mode = b->fp32 && cfg->k0_mode == 1;
  if (b->k0mode) ok = ok && balloc(b, (void**)&b->k0, (4 * (size_t)b->slot_cap + 65) * sizeof(double));
  if (!ok) { ptf_batch_destroy(b); return bfail(nullptr, PTF_ERR_MEMORY, "batch allocation failed"); }
  const int rc = b->fp32 ? setup_kernels<float>(b) : setup_kernels<double>(b);
  if (rc) { std::string m = b->error; ptf_batch_destroy(b); return bfail(nullptr, rc, m); }
  *out = b;
  return PTF_OK;
}

void ptf_batch_destroy(ptf_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (Bucket& k : b->buckets)
    for (void* p : k.allocs) cudaFree(p);
  for (void* p : b->allocs) cudaFree(p);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char* ptf_batch_last_error(const ptf_batch* b) { return b ? b->error.c_str() : ptf_last_error(nullptr); }

int ptf_batch_can_admit(ptf_batch* b, const ptf_solve_desc* d) {
  if (!b) return 0;
  if (validate(b, d)) return 0;
  for (const Bucket& k : b->buckets)
    if (k.n == d->n && k.L == d->L)
      for (long long o : k.owner)
        if (o < 0) return 1;
  const size_t ps = per_slot_bytes(b, d->n);
  size_t reclaimable = 0;
  bool dead_entry = false;
  for (const Bucket& k : b->buckets) {
    if (k.dead) { dead_entry = true; continue; }
    bool empty = true;
    for (long long o : k.owner) if (o >= 0) { empty = false; break; }
    if (empty) reclaimable += k.alloc_bytes;
  }
  if (!dead_entry && ((int)b->buckets.size() >= kMaxBuckets || b->slot_used >= b->slot_cap)) return 0;
  if (b->cfg.memory_budget > 0 && (long long)(b->bytes - reclaimable + ps) > b->cfg.memory_budget) return 0;
  return 1;
}

int ptf_batch_add(ptf_batch* b, const ptf_solve_desc* d, const double* c0, const double* u, const double* v,
                  int64_t* id) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  int rc = validate(b, d);
  if (rc) return rc;
  if (!c0) return bfail(b, PTF_ERR_ARG, "initial condition required");
  if (d->flow_kind == PTF_FLOW_ARRAYS && (!u || !v)) return bfail(b, PTF_ERR_ARG, "u and v required for an array flow");
  // a free slot in a bucket of this size, else a new bucket
  int bi = -1, slot = -1;
  for (size_t i = 0; i < b->buckets.size() && bi < 0; ++i) {
    if (b->buckets[i].n != d->n || b->buckets[i].L != d->L) continue;
    for (int s = 0; s < b->buckets[i].cap; ++s)
      if (b->buckets[i].owner[s] < 0) { bi = (int)i; slot = s; break; }
  }
  if (bi < 0) {
    bi = new_bucket(b, d->n, d->L);
    if (bi == -2) return bfail(b, PTF_ERR_MEMORY, "device allocation failed");
    if (bi < 0) return bfail(b, PTF_ERR_MEMORY, "the memory budget or slot table has no room for this solve");
    slot = 0;
  }
  const long long sid = b->next_id++;
  Bucket& k = b->buckets[bi];
  rc = b->fp32 ? admit<float>(b, k, slot, *d, c0, u, v, sid) : admit<double>(b, k, slot, *d, c0, u, v, sid);
  if (rc) { k.owner[slot] = -1; return rc; }
  b->solves[sid] = SolveRef{bi, slot, *d};
  if (id) *id = sid;
  return PTF_OK;
}

int ptf_batch_step(ptf_batch* b, int64_t nsteps) {
  ptf::TraceRange tr("ptf_batch_step");
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  if (nsteps < 0) return bfail(b, PTF_ERR_ARG, "nsteps must be >= 0");
  return b->fp32 ? step_impl<float>(b, nsteps) : step_impl<double>(b, nsteps);
}

int ptf_batch_synchronize(ptf_batch* b) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "synchronize");
  int err = 0;
  e = cudaMemcpy(&err, b->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return bcuda(b, e, "error flag");
  if (err) return bfail(b, PTF_ERR_CUDA, "a batched stage gave up waiting for its row pass (work-list fault)");
  return PTF_OK;
}

int ptf_batch_status(ptf_batch* b, int64_t id, int64_t* step, double* t, int32_t* active) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  auto it = b->solves.find(id);
  if (it == b->solves.end()) return bfail(b, PTF_ERR_ARG, "unknown solve id");
  int rc = ptf_batch_synchronize(b);
  if (rc) return rc;
  const Bucket& k = b->buckets[it->second.bucket];
  const int g = k.slot_base + it->second.slot;
  if (b->fp32) {
    SlotParams<float> sp;
    if (cudaMemcpy(&sp, (SlotParams<float>*)b->slots_dev + g, sizeof(sp), cudaMemcpyDeviceToHost) != cudaSuccess)
      return bfail(b, PTF_ERR_CUDA, "status read");
    if (step) *step = sp.step;
    if (t) *t = sp.t;
    if (active) *active = sp.active;
  } else {
    SlotParams<double> sp;
    if (cudaMemcpy(&sp, (SlotParams<double>*)b->slots_dev + g, sizeof(sp), cudaMemcpyDeviceToHost) != cudaSuccess)
      return bfail(b, PTF_ERR_CUDA, "status read");
    if (step) *step = sp.step;
    if (t) *t = sp.t;
    if (active) *active = sp.active;
  }
  return PTF_OK;
}

int ptf_batch_get_c(ptf_batch* b, int64_t id, double* c) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  if (!c) return bfail(b, PTF_ERR_ARG, "null field");
  auto it = b->solves.find(id);
  if (it == b->solves.end()) return bfail(b, PTF_ERR_ARG, "unknown solve id");
  const Bucket& k = b->buckets[it->second.bucket];
  return b->fp32 ? get_c_impl<float>(b, k, it->second.slot, c) : get_c_impl<double>(b, k, it->second.slot, c);
}

int ptf_batch_remove(ptf_batch* b, int64_t id) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  auto it = b->solves.find(id);
  if (it == b->solves.end()) return bfail(b, PTF_ERR_ARG, "unknown solve id");
  Bucket& k = b->buckets[it->second.bucket];
  const int g = k.slot_base + it->second.slot;
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "synchronize");
  // deactivate on the device, then free the slot
  const int zero = 0;
  const size_t off = b->fp32 ? offsetof(SlotParams<float>, active) : offsetof(SlotParams<double>, active);
  e = cudaMemcpy((unsigned char*)b->slots_dev + (size_t)g * slot_param_bytes(b) + off, &zero, sizeof(int),
                 cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bcuda(b, e, "slot release");
  k.owner[it->second.slot] = -1;
  b->solves.erase(it);
  b->plan_dirty = true;
  return PTF_OK;
}

int ptf_batch_info(ptf_batch* b, int64_t* device_bytes, int64_t* solves, int64_t* launches) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  if (device_bytes) *device_bytes = (int64_t)b->bytes;
  if (solves) *solves = (int64_t)b->solves.size();
  if (launches) *launches = b->launches;
  return PTF_OK;
}

int ptf_batch_inject_wait_timeout(ptf_batch* b, int32_t extra_row_items, int64_t spin_limit) {
  if (!b) return bfail(nullptr, PTF_ERR_ARG, "null batch");
  if (extra_row_items < 0 || spin_limit < 0) return bfail(b, PTF_ERR_ARG, "extra_row_items and spin_limit must be >= 0");
  if (!b->cfg.persistent) return bfail(b, PTF_ERR_STATE, "the bounded wait exists in the persistent form only");
  b->wait_extra = (unsigned)extra_row_items;
  b->spin_limit = (unsigned long long)spin_limit;
  b->plan_dirty = true;
  b->bucket_gen++;  // rebuild the plan and the captured step with the new wait
  return PTF_OK;
}

int ptf_batch_get_stream(const ptf_batch* b, void** stream) {
  if (!b || !stream) return bfail(nullptr, PTF_ERR_ARG, "null argument");
  *stream = (void*)b->stream;
  return PTF_OK;
}

}  // extern "C"
