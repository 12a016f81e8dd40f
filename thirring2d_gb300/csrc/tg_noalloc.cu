// tg_noalloc.cu -- a CG solve on M^dagger M that allocates nothing.
//
// Some callers cannot call cudaMalloc: programs whose device memory is fully
// budgeted at start-up (a framework's caching allocator already holds the
// free memory), and programs that must not stall: cudaMalloc and cudaFree can
// synchronize the whole device and so stall every other stream.  For them,
// tg_cg_noalloc() solves M^dagger M x = b (the FP64 solver of tg_cg /
// fmdm_invert_cg, hmc.c:341-404) with every work vector in one file-scope
// device array of fixed size, for lattices of at most kNoAllocMaxSites sites.
// The caller passes the gauge field, the source and the solution buffer.
#include <mutex>

#include "tg_launch.h"

namespace tg {
int record_error(int code, const char* msg);  // tg_capi.cu: message for tg_last_error()
}

using namespace tg;

namespace {

// Largest lattice the fixed scratch serves: 16384 sites (128 x 128).
constexpr int kNoAllocMaxSites = 16384;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kVec64 = align_up(sizeof(double2) * kNoAllocMaxSites);
constexpr size_t kVec32 = align_up(sizeof(float2) * kNoAllocMaxSites);
constexpr size_t kPartials = align_up(sizeof(double) * (kNoAllocMaxSites / kBlock + 64));
constexpr size_t kStateBytes = align_up(sizeof(CgState));
constexpr size_t kCounterBytes = align_up(sizeof(unsigned));
// Wt, Wx, r, p0, p1, Mp (FP64) + Wt32, Wx32 (FP32 links the link kernel also
// writes) + block partials + solver state + reduction counter: about 1.9 MB.
constexpr size_t kScratchBytes = 6 * kVec64 + 2 * kVec32 + kPartials + kStateBytes + kCounterBytes;

}  // namespace

// The scratch.  Every GPU that loads the library holds it until the process
// exits.  All calls share it and it keeps the last call's contents, so calls
// that overlap on the GPU (different streams, or threads without ordering
// between their calls) race on it.
static __device__ __align__(256) unsigned char g_cg_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {};

// Device address of the scratch on the current device.  In host code the name
// g_cg_scratch is only a host-side stand-in, so the address is looked up once
// per device, with that device current, and kept.
int scratch_base(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_error(TG_E_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return record_error(TG_E_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_base[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_cg_scratch);
    if (e != cudaSuccess) return record_error(TG_E_CUDA, cudaGetErrorString(e));
    g_base[dev] = (unsigned char*)p;
  }
  *out = g_base[dev];
  return TG_OK;
}

int ck(cudaError_t e) { return e == cudaSuccess ? TG_OK : record_error(TG_E_CUDA, cudaGetErrorString(e)); }

}  // namespace

extern "C" int tg_cg_noalloc(const tg_lattice_params* p, const tg_cg_params* cp, const void* A_dev,
                             const void* b_dev, void* x_dev, tg_cg_result* res, void* stream) {
  if (!p || !cp || !A_dev || !b_dev || !x_dev) return record_error(TG_E_ARG, "tg_cg_noalloc: null argument");
  if (p->nt < 2 || p->nx < 2) return record_error(TG_E_ARG, "tg_cg_noalloc: lattice sides must be >= 2");
  if ((long long)p->nt * p->nx > kNoAllocMaxSites)
    return record_error(TG_E_ARG, "tg_cg_noalloc: lattice larger than its fixed scratch (at most 16384 sites)");
  auto bc_ok = [](int b) { return b == 1 || b == -1 || b == 0; };
  if (!bc_ok(p->bc_t) || !bc_ok(p->bc_x)) return record_error(TG_E_ARG, "tg_cg_noalloc: bad boundary condition");
  if (cp->precision != TG_PREC_FP64) return record_error(TG_E_ARG, "tg_cg_noalloc: only the FP64 solver");
  if (cp->maxiter <= 0 || !(cp->rel_tol >= 0) || !(cp->abs_tol2 >= 0))
    return record_error(TG_E_ARG, "tg_cg_noalloc: bad CG parameters");
  cudaStream_t s = (cudaStream_t)stream;
  // An error left by an earlier, unrelated runtime call on this thread would
  // otherwise surface at this function's first launch check: clear it here.
  (void)cudaGetLastError();
  // The solve copies its state to the host and synchronizes the stream every
  // few iterations, which a stream under capture cannot do (and the sync
  // would invalidate the caller's capture): refuse before enqueueing anything.
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(s, &cs);
  if (ce != cudaSuccess) {
    (void)cudaGetLastError();
    return record_error(TG_E_ARG, "tg_cg_noalloc: cannot run while a stream capture is in progress");
  }
  if (cs != cudaStreamCaptureStatusNone)
    return record_error(TG_E_ARG, "tg_cg_noalloc: cannot run on a stream that is being captured");
  unsigned char* base = nullptr;
  int rc = scratch_base(&base);
  if (rc != TG_OK) return rc;

  Geo g{};
  g.nt = p->nt;
  g.nx = p->nx;
  g.V = p->nt * p->nx;
  g.inv_nx = 1.0f / (float)p->nx;
  g.march = (p->nx % 32 == 0) && (p->nt % kMarchT == 0);
  g.grid = nblocks(g.V);
  g.mgrid = g.grid;
  // carve the scratch
  size_t off = 0;
  auto take = [&](size_t bytes) { unsigned char* q = base + off; off += bytes; return q; };
  double2* Wt = (double2*)take(kVec64);
  double2* Wx = (double2*)take(kVec64);
  CgBufs64 w;
  w.r = (double2*)take(kVec64);
  w.p[0] = (double2*)take(kVec64);
  w.p[1] = (double2*)take(kVec64);
  w.Mp = (double2*)take(kVec64);
  float2* Wt32 = (float2*)take(kVec32);
  float2* Wx32 = (float2*)take(kVec32);
  Red red;
  red.partials = (double*)take(kPartials);
  CgState* st = (CgState*)take(kStateBytes);
  red.counter = (unsigned*)take(kCounterBytes);

  const double ep = exp(p->mu), em = exp(-p->mu);
  OpK<double> km{p->m, ep, -em, p->mu == 0.0}, kd{p->m, -em, ep, p->mu == 0.0};
  Links lk{Wt, Wx, Wt32, Wx32};
  // the reduction counter must start at 0; everything else is written before it is read
  if ((rc = ck(cudaMemsetAsync(red.counter, 0, sizeof(unsigned), s))) != TG_OK) return rc;
  link_phase_fixed(s, g, p->bc_t, p->bc_x, (const double2*)A_dev, Wt, Wx, Wt32, Wx32);
  cg64_init_fixed(s, g, (const double2*)b_dev, (double2*)x_dev, w, st, red, cp->rel_tol, cp->abs_tol2, cp->maxiter);
  if ((rc = ck(cudaGetLastError())) != TG_OK) return rc;
  CgState hs;
  const int chunk = 16;  // even: p ends in its first buffer
  const long max_chunks = (long)cp->maxiter / chunk + 2;
  for (long c = 0;; c++) {
    if ((rc = ck(cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s))) != TG_OK) return rc;
    if ((rc = ck(cudaStreamSynchronize(s))) != TG_OK) return rc;
    if (hs.done) break;
    if (c >= max_chunks) return record_error(TG_E_NOCONV, "tg_cg_noalloc: CG loop did not terminate");
    for (int j = 0; j < chunk; j++) cg64_iter_fixed(s, g, km, kd, lk, (double2*)x_dev, w, j & 1, st, red);
    if ((rc = ck(cudaGetLastError())) != TG_OK) return rc;
  }
  if (res) {
    res->iterations = hs.iter;
    res->status = hs.status;
    res->reliable_updates = 0;
    res->rr = hs.rr;
    res->rr0 = hs.rr0;
  }
  switch (hs.status) {
    case TG_OK: return TG_OK;
    case TG_E_NOCONV: return record_error(TG_E_NOCONV, "CG reached its iteration cap");
    case TG_E_DIVERGED: return record_error(TG_E_DIVERGED, "Cannot invert fermion matrix (|r|^2/|r0|^2 > 1e10)");
    default: return record_error(TG_E_NAN, "NaN in the CG recurrence");
  }
}
