// tg_capi.cu -- host side of the Thirring2D GB300 library: lattice context,
// reference RNG stream, CG and trajectory scheduling (CUDA graphs with
// conditional WHILE/IF nodes, or eager launches with host polling), and the
// C ABI declared in include/thirring_gpu.h.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "tg_batch.h"
#include "tg_launch.h"

using namespace tg;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define TG_CK(call)                                                                                    \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess)                                                                             \
      return fail(TG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " (" __FILE__ ":" + \
                                 std::to_string(__LINE__) + ")");                                      \
  } while (0)

#define TG_TRY(expr)          \
  do {                        \
    int rc_ = (expr);         \
    if (rc_ != TG_OK) return rc_; \
  } while (0)

constexpr int kMaxPf = 8;
constexpr int kMaxLog = 4096;

// ---------------------------------------------------------------------------
// The reference's random stream: MT19937 (Matsumoto & Nishimura 1998) seeded
// by the Knuth 69069 recurrence from an odd seed, each block of 624 tempered
// words handed out last-first as y * 2^-32 (mersenne_inline.c:73-128,
// mersenne.h:11).  Box-Muller pairs as hmc.c:423-426.
// ---------------------------------------------------------------------------
struct RefStream {
  uint32_t w[624];
  double out[624];
  int avail = 0;

  void seed(long s) {
    if (s % 2 == 0) s++;
    w[0] = (uint32_t)(s & 0xffffffffL);
    for (int i = 1; i < 624; i++) w[i] = 69069u * w[i - 1];
    avail = 0;
  }
  void twist() {
    for (int i = 0; i < 624; i++) {
      uint32_t y = (w[i] & 0x80000000u) | (w[i + 1 < 624 ? i + 1 : 0] & 0x7fffffffu);
      uint32_t n = w[i + 397 < 624 ? i + 397 : i + 397 - 624] ^ (y >> 1);
      w[i] = (y & 1u) ? n ^ 0x9908b0dfu : n;
    }
    for (int i = 0; i < 624; i++) {
      uint32_t y = w[i];
      y ^= y >> 11;
      y ^= (y << 7) & 0x9d2c5680u;
      y ^= (y << 15) & 0xefc60000u;
      y ^= y >> 18;
      out[i] = (double)y * (1.0 / 4294967296.0);
    }
    avail = 624;
  }
  double next() {
    if (avail == 0) twist();
    return out[--avail];
  }
  void gauss_pairs(long n, double* dst) {  // dst[2n]
    for (long k = 0; k < n; k++) {
      double u1 = next(), u2 = next();
      double r = sqrt(-2 * log(u1));
      dst[2 * k] = r * cos(2 * M_PI * u2);
      dst[2 * k + 1] = r * sin(2 * M_PI * u2);
    }
  }
};

struct GraphEntry {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

}  // namespace

struct tg_lattice {
  tg_lattice_params P{};
  Geo g{};
  int V = 0;
  int version = 0;  // bumped when couplings change (invalidates graphs)
  cudaStream_t stream = nullptr, cap2 = nullptr, cap3 = nullptr;

  double2 *A = nullptr, *Anew = nullptr, *Wt = nullptr, *Wx = nullptr;
  double2 *Wt1 = nullptr, *Wx1 = nullptr;  // W / m (unit-mass FP64 CG)
  float2 *Wt32 = nullptr, *Wx32 = nullptr;
  double2 *mom = nullptr, *noise = nullptr, *chi = nullptr, *Mchi = nullptr, *vin = nullptr, *vout = nullptr;
  double2 *eta = nullptr, *phi = nullptr;  // [npf_alloc][V]
  double* unif = nullptr;                  // [4V] uniforms of one pure-gauge sweep (allocated on first use)
  int* mask = nullptr;                     // masked real operator: occupation mask and 6 real vectors
  double* rv[6] = {};                      // in/b, out/x, r, p, tmp, Ap (allocated on first use)
  int npf_alloc = 0;
  CgBufs64 w64{};
  CgBufsMixed wmx{};
  CgState* st = nullptr;
  CgLog* log = nullptr;
  TrajStats* ts = nullptr;
  Red red{};
  unsigned* bar = nullptr;      // persistent solver: barrier words [kBarWords]
  double* pcg_part = nullptr;   // and its partial sums [4 * kPcgMaxGrid]

  double* h_stage = nullptr;  // pinned, 2*V*kMaxPf doubles... sized at create
  size_t h_stage_len = 0;
  CgState* h_st = nullptr;
  TrajStats* h_ts = nullptr;
  CgLog* h_log = nullptr;

  RefStream mt;
  bool mt_seeded = false;
  std::map<std::string, GraphEntry> graphs;
  std::vector<cudaEvent_t> ev;
  double l2_bytes = 0;  // the device's L2 size
};

namespace {

// NVTX range for the lifetime of a scope: the host side of an entry point or
// a trajectory phase, for Nsight timelines (no cost without a tool attached).
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

OpK<double> op_k(const tg_lattice* L, int dagger) {
  double ep = exp(L->P.mu), em = exp(-L->P.mu);
  OpK<double> k;
  k.m = L->P.m;
  if (!dagger) { k.cf = ep; k.cb = -em; }
  else { k.cf = -em; k.cb = ep; }
  k.mu0 = L->P.mu == 0.0;
  return k;
}
OpK<float> op_k32(const tg_lattice* L, int dagger) {
  OpK<double> k = op_k(L, dagger);
  OpK<float> f;
  f.m = (float)k.m; f.cf = (float)k.cf; f.cb = (float)k.cb; f.mu0 = k.mu0;
  return f;
}
// TG_SOLVER_DEFAULT: the persistent solver (one cooperative launch per solve),
// measured faster than two launches per iteration on the 1024^2 trajectory:
// FP64 1.416 vs 1.342, mixed 5.56 vs 4.33 trajectories/s
constexpr bool kDefaultPersistent = true;

// The FP64 CG runs in unit-mass form (links W / m) whenever 1/m is a finite
// nonzero number; m = 0 keeps the plain form.
bool unit_mass(const tg_lattice* L) {
  const double m = L->P.m;
  return m != 0.0 && std::isfinite(1.0 / m) && std::isfinite(1.0 / (m * m)) && 1.0 / (m * m) != 0.0;
}
Links links(const tg_lattice* L) {
  Links lk{L->Wt, L->Wx, L->Wt32, L->Wx32};
  if (unit_mass(L)) {
    lk.Wt1 = L->Wt1;
    lk.Wx1 = L->Wx1;
    lk.inv_m2 = 1.0 / (L->P.m * L->P.m);
  }
  return lk;
}
LinkOut link_out(const tg_lattice* L) {
  LinkOut o{L->Wt, L->Wx, L->Wt32, L->Wx32};
  if (unit_mass(L)) {
    o.Wt1 = L->Wt1;
    o.Wx1 = L->Wx1;
    o.inv_m = 1.0 / L->P.m;
  }
  return o;
}

bool env_graph_enabled() {
  const char* e = getenv("TG_GRAPH");
  return !(e && e[0] == '0');
}

template <typename T> int dmalloc(T** p, size_t n) {
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) return fail(TG_E_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return TG_OK;
}

int ensure_pf(tg_lattice* L, int npf) {
  if (npf <= L->npf_alloc) return TG_OK;
  if (npf > kMaxPf) return fail(TG_E_ARG, "npf > 8");
  TG_CK(cudaStreamSynchronize(L->stream));
  if (L->eta) cudaFree(L->eta);
  if (L->phi) cudaFree(L->phi);
  L->eta = L->phi = nullptr;
  TG_TRY(dmalloc(&L->eta, (size_t)npf * L->V));
  TG_TRY(dmalloc(&L->phi, (size_t)npf * L->V));
  L->npf_alloc = npf;
  for (auto& kv : L->graphs) {  // graphs hold the old pointers
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  L->graphs.clear();
  return TG_OK;
}

int ensure_events(tg_lattice* L, size_t n) {
  while (L->ev.size() < n) {
    cudaEvent_t e;
    TG_CK(cudaEventCreate(&e));
    L->ev.push_back(e);
  }
  return TG_OK;
}

int check_cg_params(const tg_cg_params* cp) {
  if (!cp) return fail(TG_E_ARG, "null CG parameters");
  if (cp->maxiter <= 0) return fail(TG_E_ARG, "maxiter must be positive");
  if (cp->precision != TG_PREC_FP64 && cp->precision != TG_PREC_MIXED) return fail(TG_E_ARG, "bad precision");
  if (cp->precision == TG_PREC_MIXED && cp->ru_interval <= 0) return fail(TG_E_ARG, "ru_interval must be positive");
  if (cp->solver < TG_SOLVER_DEFAULT || cp->solver > TG_SOLVER_PERSISTENT) return fail(TG_E_ARG, "bad solver");
  if (!(cp->rel_tol >= 0) || !(cp->abs_tol2 >= 0)) return fail(TG_E_ARG, "tolerances must be >= 0");
  return TG_OK;
}

// Add a conditional node after the current capture dependencies of `s` and
// return its body graph; the capture continues after the node.
int add_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                    cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t gr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  TG_CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &gr, &deps, nullptr, &nd));
  if (cs != cudaStreamCaptureStatusActive) return fail(TG_E_CUDA, "stream is not capturing");
  // cudaGraphNodeParams has no usable default constructor in C++; zero it as bytes
  alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(raw);
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  TG_CK(cudaGraphAddNode(&node, gr, deps, nullptr, nd, &np));
  TG_CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  *body = np.conditional.phGraph_out[0];
  return TG_OK;
}

int capture_graph_of(cudaStream_t s, cudaGraph_t* gr) {
  cudaStreamCaptureStatus cs;
  TG_CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, gr, nullptr, nullptr, nullptr));
  return TG_OK;
}

// Enqueue one CG solve of M^dag M x = b on stream s.  graph = true: s is
// capturing and the iteration loop becomes a conditional WHILE node (no host
// involvement at run time).  graph = false: iterations are launched in
// chunks and the host polls the device `done` flag between chunks.
bool use_persistent(const tg_cg_params& cp) {
  if (cp.solver == TG_SOLVER_PERSISTENT) return true;
  if (cp.solver == TG_SOLVER_LAUNCHES) return false;
  const char* e = getenv("TG_SOLVER");  // default: TG_SOLVER=persistent|launches overrides
  if (e && strcmp(e, "persistent") == 0) return true;
  if (e && strcmp(e, "launches") == 0) return false;
  return kDefaultPersistent;
}

// The mixed persistent solve on column-march lattices whose FP32 CG working set
// (r, w, s, p, x and the two links: 56 B per site) is more than 1.5 times the
// L2 runs the single-reduction CG (k_pcgcg: one grid sum and one fused
// M^dag M pass per iteration); smaller lattices, whose vectors stay in L2 and
// where the fused pass's halo recomputation costs more latency than the second
// sum, run the two-sum CG (k_pcgmx).  Measured on GB300 (us per iteration,
// fused / two-sum): 1024^2 30.3 / 21.7, 1536^2 58.1 / 58.6, 2048^2 93.8 / 102.5.
// TG_MIXED_CG=twosum|onesum overrides.
bool use_single_reduction(const tg_lattice* L) {
  if (!L->g.march) return false;
  const char* e = getenv("TG_MIXED_CG");
  if (e && strcmp(e, "twosum") == 0) return false;
  if (e && strcmp(e, "onesum") == 0) return true;
  return 56.0 * (double)L->V > 1.5 * (double)L->l2_bytes;
}

// The whole solve as one cooperative launch (tg_pcg.cu); the barrier's
// arrival count is cleared first, so a solve that timed out leaves no trace.
int enqueue_pcg(tg_lattice* L, cudaStream_t s, const tg_cg_params& cp, const double2* b, double2* x, int log_index) {
  const Links lk = links(L);
  const GridBar bar{L->bar, reinterpret_cast<unsigned long long*>(L->bar + 2)};
  TG_CK(cudaMemsetAsync(L->bar, 0, kBarWords * sizeof(unsigned), s));
  cudaError_t e;
  if (cp.precision == TG_PREC_MIXED) {
    PcgMxArgs a{};
    a.g = L->g;
    a.km32 = op_k32(L, 0);
    a.kd32 = op_k32(L, 1);
    a.km = op_k(L, 0);
    a.kd = op_k(L, 1);
    a.Wt32 = lk.Wt32;
    a.Wx32 = lk.Wx32;
    a.Wt = lk.Wt;
    a.Wx = lk.Wx;
    a.b = b;
    a.x = x;
    a.tmp = L->wmx.tmp64;
    a.xs = L->wmx.xs;
    a.r = L->wmx.rs;
    a.p0 = L->wmx.ps[0];
    a.p1 = L->wmx.ps[1];
    a.Mp = L->wmx.Mps;
    a.st = L->st;
    a.log = L->log;
    a.log_index = log_index;
    a.part = L->pcg_part;
    a.bar = bar;
    a.rel_tol = cp.rel_tol;
    a.abs_tol2 = cp.abs_tol2;
    a.maxiter = cp.maxiter;
    a.ru_interval = cp.ru_interval;
    if (use_single_reduction(L)) {
      a.w0 = L->wmx.Mps;
      a.s0 = L->wmx.ss;
      e = pcgcg(s, L->P.mu == 0.0, a);
    } else {
      e = pcgmx(s, L->P.mu == 0.0, a);
    }
  } else {
    Pcg64Args a{};
    a.g = L->g;
    a.km = op_k(L, 0);
    a.kd = op_k(L, 1);
    const bool unit = lk.Wt1 != nullptr;
    a.Wt = unit ? lk.Wt1 : lk.Wt;
    a.Wx = unit ? lk.Wx1 : lk.Wx;
    a.inv_m2 = unit ? lk.inv_m2 : 0.0;
    a.b = b;
    a.x = x;
    a.r = L->w64.r;
    a.p0 = L->w64.p[0];
    a.p1 = L->w64.p[1];
    a.Mp = L->w64.Mp;
    a.st = L->st;
    a.log = L->log;
    a.log_index = log_index;
    a.part = L->pcg_part;
    a.bar = bar;
    a.rel_tol = cp.rel_tol;
    a.abs_tol2 = cp.abs_tol2;
    a.maxiter = cp.maxiter;
    e = pcg64(s, L->P.mu == 0.0, a);
  }
  if (e != cudaSuccess) return fail(TG_E_CUDA, std::string("persistent CG launch: ") + cudaGetErrorString(e));
  return TG_OK;
}

int enqueue_cg(tg_lattice* L, cudaStream_t s, const tg_cg_params& cp, const double2* b, double2* x, int log_index,
               bool graph) {
  if (use_persistent(cp)) return enqueue_pcg(L, s, cp, b, x, log_index);
  const Geo& g = L->g;
  const bool mixed = cp.precision == TG_PREC_MIXED;
  OpK<double> km = op_k(L, 0), kd = op_k(L, 1);
  OpK<float> km32 = op_k32(L, 0), kd32 = op_k32(L, 1);
  Links lk = links(L);
  if (graph) {
    cudaGraph_t top;
    TG_TRY(capture_graph_of(s, &top));
    cudaGraphConditionalHandle hloop;
    TG_CK(cudaGraphConditionalHandleCreate(&hloop, top, 0, 0));
    Cond c0{hloop, 0, 1};
    if (mixed)
      cgmx_init(s, g, b, x, L->wmx, L->st, L->log, L->red, cp.rel_tol, cp.abs_tol2, cp.maxiter, cp.ru_interval, log_index,
                c0);
    else
      cg64_init(s, g, b, x, L->w64, L->st, L->log, L->red, cp.rel_tol, cp.abs_tol2, cp.maxiter, log_index, c0);
    TG_CK(cudaGetLastError());
    cudaGraph_t body;
    TG_TRY(add_conditional(s, hloop, cudaGraphCondTypeWhile, &body));
    // the body holds two iterations (p alternates between its two buffers);
    // the kernels of the second are no-ops once the first has converged
    TG_CK(cudaStreamBeginCaptureToGraph(L->cap2, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    for (int half = 0; half < 2; half++) {
      if (!mixed) {
        cg64_iter(L->cap2, g, km, kd, lk, x, L->w64, half, L->st, L->log, L->red, c0);
      } else {
        cudaGraphConditionalHandle hru;
        TG_CK(cudaGraphConditionalHandleCreate(&hru, body, 0, 0));
        Cond c1{hloop, hru, 1};
        cgmx_iter(L->cap2, g, km32, kd32, lk, L->wmx, half, L->st, L->red, c1);
        cudaGraph_t ifbody;
        TG_TRY(add_conditional(L->cap2, hru, cudaGraphCondTypeIf, &ifbody));
        TG_CK(cudaStreamBeginCaptureToGraph(L->cap3, ifbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        cgmx_reliable(L->cap3, g, km, kd, lk, b, x, L->wmx, L->st, L->log, L->red, c1);
        TG_CK(cudaGetLastError());
        cudaGraph_t tmp;
        TG_CK(cudaStreamEndCapture(L->cap3, &tmp));
      }
    }
    TG_CK(cudaGetLastError());
    cudaGraph_t tmp;
    TG_CK(cudaStreamEndCapture(L->cap2, &tmp));
    return TG_OK;
  }
  Cond none{0, 0, 0};
  if (mixed)
    cgmx_init(s, g, b, x, L->wmx, L->st, L->log, L->red, cp.rel_tol, cp.abs_tol2, cp.maxiter, cp.ru_interval, log_index,
              none);
  else
    cg64_init(s, g, b, x, L->w64, L->st, L->log, L->red, cp.rel_tol, cp.abs_tol2, cp.maxiter, log_index, none);
  TG_CK(cudaGetLastError());
  const int chunk = 16;
  long max_chunks = (long)cp.maxiter / chunk + 2;
  for (long c = 0; c < max_chunks; c++) {
    TG_CK(cudaMemcpyAsync(L->h_st, L->st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    TG_CK(cudaStreamSynchronize(s));
    if (L->h_st->done) return TG_OK;
    for (int j = 0; j < chunk; j++) {  // chunk is even: p ends in buffer 0 again
      const int half = j & 1;
      if (!mixed) {
        cg64_iter(s, g, km, kd, lk, x, L->w64, half, L->st, L->log, L->red, none);
      } else {
        cgmx_iter(s, g, km32, kd32, lk, L->wmx, half, L->st, L->red, none);
        cgmx_reliable(s, g, km, kd, lk, b, x, L->wmx, L->st, L->log, L->red, none);
      }
    }
    TG_CK(cudaGetLastError());
  }
  TG_CK(cudaMemcpyAsync(L->h_st, L->st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  TG_CK(cudaStreamSynchronize(s));
  if (!L->h_st->done) return fail(TG_E_NOCONV, "CG loop did not terminate");
  return TG_OK;
}

// Run `fn(stream, graph)` either as a cached CUDA graph (key) or eagerly.
template <typename F> int run_maybe_graph(tg_lattice* L, const std::string& key, bool use_graph, F fn) {
  if (!use_graph) return fn(L->stream, false);
  auto it = L->graphs.find(key);
  if (it == L->graphs.end()) {
    GraphEntry ge;
    TG_CK(cudaStreamBeginCapture(L->stream, cudaStreamCaptureModeThreadLocal));
    int rc = fn(L->stream, true);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(L->stream, &gr);
    if (rc != TG_OK) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    if (e != cudaSuccess) return fail(TG_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    ge.graph = gr;
    TG_CK(cudaGraphInstantiate(&ge.exec, gr, 0));
    it = L->graphs.emplace(key, ge).first;
  }
  TG_CK(cudaGraphLaunch(it->second.exec, L->stream));
  return TG_OK;
}

std::string cg_key(const tg_cg_params& cp) {
  char buf[160];
  snprintf(buf, sizeof buf, "%.17g/%.17g/%d/%d/%d/%d", cp.rel_tol, cp.abs_tol2, cp.maxiter, cp.precision,
           cp.ru_interval, use_persistent(cp) ? 1 : 0);
  return buf;
}

int read_cg_result(tg_lattice* L, tg_cg_result* res) {
  TG_CK(cudaMemcpyAsync(L->h_st, L->st, sizeof(CgState), cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  if (res) {
    res->iterations = L->h_st->iter;
    res->status = L->h_st->status;
    res->reliable_updates = L->h_st->n_ru;
    res->rr = L->h_st->rr;
    res->rr0 = L->h_st->rr0;
  }
  return TG_OK;
}

// Solve on device vectors b -> x (both double2[V]) with the lattice's links.
int solve_dev(tg_lattice* L, const tg_cg_params& cp, const double2* b, double2* x, tg_cg_result* res) {
  std::string key = "cg:" + cg_key(cp) + ":" + std::to_string((uintptr_t)b) + ":" + std::to_string((uintptr_t)x) +
                    ":" + std::to_string(L->version);
  TG_TRY(run_maybe_graph(L, key, env_graph_enabled(),
                         [&](cudaStream_t s, bool graph) { return enqueue_cg(L, s, cp, b, x, -1, graph); }));
  TG_TRY(read_cg_result(L, res));
  return TG_OK;
}

// A finished solve that did not converge is reported as the call's status
// (the outputs are still written), with a message for tg_last_error().
int solver_status(int status) {
  switch (status) {
    case TG_OK: return TG_OK;
    case TG_E_NOCONV: return fail(TG_E_NOCONV, "CG reached its iteration cap");
    case TG_E_DIVERGED: return fail(TG_E_DIVERGED, "Cannot invert fermion matrix (|r|^2/|r0|^2 > 1e10)");
    case TG_E_NAN: return fail(TG_E_NAN, "NaN in the CG recurrence");
    case TG_E_TIMEOUT: return fail(TG_E_TIMEOUT, "persistent CG: a grid barrier waited past its limit");
    default: return fail(status, "solver error");
  }
}

int upload(tg_lattice* L, void* dst, const double* src, size_t ndouble) {
  if (ndouble > L->h_stage_len) return fail(TG_E_ARG, "field larger than staging buffer");
  memcpy(L->h_stage, src, ndouble * sizeof(double));
  TG_CK(cudaMemcpyAsync(dst, L->h_stage, ndouble * sizeof(double), cudaMemcpyHostToDevice, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));  // staging buffer is reused
  return TG_OK;
}
int download(tg_lattice* L, double* dst, const void* src, size_t ndouble) {
  if (ndouble > L->h_stage_len) return fail(TG_E_ARG, "field larger than staging buffer");
  TG_CK(cudaMemcpyAsync(L->h_stage, src, ndouble * sizeof(double), cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  memcpy(dst, L->h_stage, ndouble * sizeof(double));
  return TG_OK;
}

// ---------------------------------------------------------------------------
// One trajectory (hmc.c:671-746) on the device.  The random fields are in
// L->eta[0..npf), L->mom, L->noise and L->ts->u already, or are drawn here
// from Philox (rng == TG_RNG_PHILOX).
// ---------------------------------------------------------------------------
int enqueue_trajectory(tg_lattice* L, cudaStream_t s, const tg_hmc_params& p, bool graph) {
  const Geo& g = L->g;
  const int V = L->V;
  const bool use_noise = p.stochastic_term != 0;
  OpK<double> km = op_k(L, 0), kd = op_k(L, 1);
  const double ep = exp(L->P.mu), em = exp(-L->P.mu);
  TrajStats* ts = L->ts;
  int solve = 0;
  auto rec = [&](int i) -> int {
    TG_CK(cudaEventRecordWithFlags(L->ev[i], s, graph ? cudaEventRecordExternal : cudaEventRecordDefault));
    return TG_OK;
  };
  auto cg = [&](const double2* b, double2* x) -> int {
    TG_TRY(rec(2 * solve));
    TG_TRY(enqueue_cg(L, s, p.cg, b, x, solve, graph));
    TG_TRY(rec(2 * solve + 1));
    solve++;
    return TG_OK;
  };
  {  // heatbath and start actions
    Range range("heatbath");
    if (p.rng == TG_RNG_PHILOX) {
      for (int k = 0; k < p.npf; k++) philox_gauss(s, g, p.seed, ts, (unsigned)k, L->eta + (size_t)k * V);
      philox_gauss(s, g, p.seed, ts, 16u, L->mom);
      if (use_noise) philox_gauss(s, g, p.seed, ts, 17u, L->noise);
      philox_uniform(s, p.seed, ts, 18u);
    }
    link_phase(s, g, L->P.bc_t, L->P.bc_x, L->A, link_out(L));
    // start: S_pf = |eta|^2 exactly (phi = M^dag eta), hmc.c:418-436
    TG_CK(cudaMemsetAsync(&ts->Spf0, 0, sizeof(double), s));
    for (int k = 0; k < p.npf; k++) {
      norm2(s, g, L->eta + (size_t)k * V, &ts->Spf0, 1, L->red);
      dslash64(s, g, kd, 1, L->eta + (size_t)k * V, L->phi + (size_t)k * V, L->Wt, L->Wx);
    }
    norm2(s, g, L->mom, &ts->Smom0, 0, L->red);
    gauge_action(s, g, L->A, kNf / L->P.g, &ts->Sg0, L->red);
    if (use_noise) md_action(s, g, kd, L->noise, L->Wt, L->Wx, &ts->Smd0, L->red);
    else TG_CK(cudaMemsetAsync(&ts->Smd0, 0, sizeof(double), s));
    TG_CK(cudaMemcpyAsync(L->Anew, L->A, (size_t)V * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  }
  // leapfrog, hmc.c:708-716; the two half steps between MD steps share a launch
  const double eps = p.tau / p.nsteps;
  const double c = 2.0 * (p.tau * 0.5 / p.nsteps);
  const double gfac = eps * kNf / L->P.g;
  for (int i = 0; i < p.nsteps; i++) {
    Range step("md_step");
    gauge_step(s, g, L->P.bc_t, L->P.bc_x, L->Anew, L->mom, c, i == 0 ? 1 : 2, link_out(L));
    if (p.npf == 0)
      momentum_update(s, g, L->P.bc_t, L->P.bc_x, ep, em, L->Anew, L->Wt, L->Wx, nullptr, nullptr, L->noise, L->mom, eps, gfac,
                      1 | (use_noise ? 2 : 0));
    for (int k = 0; k < p.npf; k++) {
      TG_TRY(cg(L->phi + (size_t)k * V, L->chi));
      dslash64(s, g, km, 0, L->chi, L->Mchi, L->Wt, L->Wx);
      int flags = (k == 0 ? 1 : 0) | ((k == p.npf - 1 && use_noise) ? 2 : 0);
      momentum_update(s, g, L->P.bc_t, L->P.bc_x, ep, em, L->Anew, L->Wt, L->Wx, L->chi, L->Mchi, L->noise, L->mom, eps, gfac, flags);
    }
  }
  Range end("end_actions");
  gauge_step(s, g, L->P.bc_t, L->P.bc_x, L->Anew, L->mom, c, 1, link_out(L));
  // end actions, hmc.c:719-726
  TG_CK(cudaMemsetAsync(&ts->Spf1, 0, sizeof(double), s));
  for (int k = 0; k < p.npf; k++) {
    TG_TRY(cg(L->phi + (size_t)k * V, L->chi));
    redot(s, g, L->phi + (size_t)k * V, L->chi, &ts->Spf1, 1, L->red);
  }
  norm2(s, g, L->mom, &ts->Smom1, 0, L->red);
  gauge_action(s, g, L->Anew, kNf / L->P.g, &ts->Sg1, L->red);
  if (use_noise) md_action(s, g, kd, L->noise, L->Wt, L->Wx, &ts->Smd1, L->red);
  else TG_CK(cudaMemsetAsync(&ts->Smd1, 0, sizeof(double), s));
  finish_trajectory(s, ts);
  accept_copy(s, g, ts, L->A, L->Anew);
  link_phase(s, g, L->P.bc_t, L->P.bc_x, L->A, link_out(L));
  TG_CK(cudaGetLastError());
  return TG_OK;
}

int check_hmc_params(const tg_hmc_params* p) {
  if (!p) return fail(TG_E_ARG, "null HMC parameters");
  if (p->nsteps <= 0 || !(p->tau > 0)) return fail(TG_E_ARG, "nsteps and tau must be positive");
  if (p->npf < 0 || p->npf > kMaxPf) return fail(TG_E_ARG, "npf must be in [0, 8]");
  if ((p->nsteps + 1) * (p->npf > 0 ? p->npf : 1) > kMaxLog) return fail(TG_E_ARG, "too many CG solves");
  return check_cg_params(&p->cg);
}

int run_trajectory(tg_lattice* L, const tg_hmc_params& p, tg_traj_result* r) {
  Range range("tg_trajectory");
  TG_TRY(ensure_pf(L, p.npf > 0 ? p.npf : 1));
  const int nsolves = (p.nsteps + 1) * p.npf;
  TG_TRY(ensure_events(L, 2 * (size_t)nsolves + 2));
  char buf[256];
  snprintf(buf, sizeof buf, "traj:%d/%.17g/%d/%d/%d/%llu/%d:", p.nsteps, p.tau, p.npf, p.stochastic_term, p.rng,
           (unsigned long long)p.seed, L->version);
  std::string key = buf + cg_key(p.cg);
  bool use_graph = p.use_graph && env_graph_enabled();
  TG_TRY(run_maybe_graph(L, key, use_graph, [&](cudaStream_t s, bool graph) {
    return enqueue_trajectory(L, s, p, graph);
  }));
  TG_CK(cudaMemcpyAsync(L->h_ts, L->ts, sizeof(TrajStats), cudaMemcpyDeviceToHost, L->stream));
  if (nsolves > 0)
    TG_CK(cudaMemcpyAsync(L->h_log, L->log, sizeof(CgLog) * nsolves, cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  if (r) {
    const TrajStats& t = *L->h_ts;
    memset(r, 0, sizeof(*r));
    r->dH = t.dH;
    r->Sg0 = t.Sg0; r->Spf0 = t.Spf0; r->Smd0 = t.Smd0; r->Smom0 = t.Smom0;
    r->Sg1 = t.Sg1; r->Spf1 = t.Spf1; r->Smd1 = t.Smd1; r->Smom1 = t.Smom1;
    r->u_accept = t.u;
    r->accepted = t.accepted;
    r->cg_solves = nsolves;
    double ms = 0;
    for (int i = 0; i < nsolves; i++) {
      const CgLog& l = L->h_log[i];
      r->cg_iterations += l.iter;
      if (l.iter > r->cg_max_iterations) r->cg_max_iterations = l.iter;
      r->reliable_updates += l.n_ru;
      if (l.status > r->status) r->status = l.status;
      float e = 0;
      if (cudaEventElapsedTime(&e, L->ev[2 * i], L->ev[2 * i + 1]) == cudaSuccess) ms += e;
    }
    r->cg_ms = ms;
    return solver_status(r->status);
  }
  return TG_OK;
}

}  // namespace

namespace tg {
// error recording for entry points defined in other translation units
int record_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace tg

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* tg_last_error(void) { return g_err.c_str(); }
const char* tg_version(void) { return "thirring2d_gb300 0.1 (sm_103a)"; }

int tg_grid_barrier_check(int device, int phantom_blocks, int* status) {
  if (!status || phantom_blocks < 0) return fail(TG_E_ARG, "bad argument");
  TG_CK(cudaSetDevice(device));
  unsigned* count = nullptr;
  int* st = nullptr;
  TG_TRY(dmalloc(&count, 1));
  if (dmalloc(&st, 1) != TG_OK) {
    cudaFree(count);
    return TG_E_ALLOC;
  }
  cudaError_t e = cudaMemset(count, 0, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(st, 0xff, sizeof(int));
  // 2^16 polls: tens of milliseconds before a barrier that cannot complete gives up
  if (e == cudaSuccess) e = barrier_check(0, count, (unsigned)phantom_blocks, 1LL << 16, st);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(status, st, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(count);
  cudaFree(st);
  if (e != cudaSuccess) return fail(TG_E_CUDA, std::string("barrier check: ") + cudaGetErrorString(e));
  return TG_OK;
}

int tg_stage_faults(int device, unsigned* count) {
  if (!count) return fail(TG_E_ARG, "null argument");
  TG_CK(cudaSetDevice(device));
  *count = stage_faults();
  if (*count == 0xffffffffu) return fail(TG_E_CUDA, "cannot read the stage fault counter");
  return TG_OK;
}

int tg_measure_fp64_peak(int device, double* tflops) {
  if (!tflops) return fail(TG_E_ARG, "null argument");
  TG_CK(cudaSetDevice(device));
  int sms = 0;
  TG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int iters = 4096;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double* sink = nullptr;
  int rc = TG_OK;
  double best = 0;  // FMA/s
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess || cudaMalloc(&sink, sizeof(double)) != cudaSuccess) {
    rc = fail(TG_E_CUDA, "fp64 peak setup failed");
  } else {
    // 2, 4 and 8 blocks of 256 threads per SM; the best rate of 3 timed launches each
    for (int bps = 2; bps <= 8 && rc == TG_OK; bps *= 2) {
      const int grid = bps * sms;
      dfma_peak(st, grid, iters, sink);  // warm-up
      for (int rep = 0; rep < 3 && rc == TG_OK; rep++) {
        float ms = 0;
        if (cudaEventRecord(e0, st) != cudaSuccess) rc = TG_E_CUDA;
        dfma_peak(st, grid, iters, sink);
        if (rc == TG_OK && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                            cudaGetLastError() != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
          rc = TG_E_CUDA;
        const double rate = (double)grid * 256 * 32 * iters / (ms * 1e-3);
        if (rc == TG_OK && ms > 0 && rate > best) best = rate;
      }
    }
    if (rc != TG_OK) fail(TG_E_CUDA, "fp64 peak kernel failed");
  }
  if (sink) cudaFree(sink);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (rc != TG_OK) return rc;
  *tflops = 2.0 * best / 1e12;
  return TG_OK;
}

int tg_create(const tg_lattice_params* p, tg_lattice** out) {
  if (!p || !out) return fail(TG_E_ARG, "null argument");
  *out = nullptr;
  if (p->nt < 2 || p->nx < 2) return fail(TG_E_ARG, "lattice sides must be >= 2");
  long long V = (long long)p->nt * p->nx;
  if (V >= (1LL << 24)) return fail(TG_E_ARG, "volume must be below 2^24 sites");
  auto bc_ok = [](int b) { return b == 1 || b == -1 || b == 0; };
  if (!bc_ok(p->bc_t) || !bc_ok(p->bc_x)) return fail(TG_E_ARG, "boundary conditions must be -1, 0 or 1");
  if (!(p->g > 0)) return fail(TG_E_ARG, "g must be positive");
  TG_CK(cudaSetDevice(p->device));
  tg_lattice* L = new tg_lattice();
  L->P = *p;
  L->V = (int)V;
  L->g.nt = p->nt;
  L->g.nx = p->nx;
  L->g.V = (int)V;
  L->g.inv_nx = 1.0f / (float)p->nx;
  {
    int sms = 0, l2 = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess || sms <= 0) sms = 1;
    if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, p->device) != cudaSuccess || l2 <= 0) l2 = 128 << 20;
    L->l2_bytes = (double)l2;
    // 8 resident 256-thread blocks per SM at <= 32 registers per thread
    int cap = 8 * sms;
    L->g.grid = nblocks((int)V) < cap ? nblocks((int)V) : cap;
    const char* e = getenv("TG_MARCH");
    L->g.march = (p->nx % 32 == 0) && (p->nt % kMarchT == 0) && !(e && e[0] == '0');
    int items = L->g.march ? (p->nx / 32) * (p->nt / kMarchT) : 0;
    int mg = (items + kBlock / 32 - 1) / (kBlock / 32);
    L->g.mgrid = L->g.march ? (mg < cap ? mg : cap) : L->g.grid;
  }
  auto bail = [&](int rc) { tg_destroy(L); return rc; };
  if (cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&L->cap2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&L->cap3, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(TG_E_CUDA, "stream creation failed"));
  size_t n = (size_t)V;
  int rc = TG_OK;
  double2** d2[] = {&L->A, &L->Anew, &L->Wt, &L->Wx, &L->Wt1, &L->Wx1, &L->mom, &L->noise, &L->chi, &L->Mchi, &L->vin, &L->vout,
                    &L->w64.r, &L->w64.p[0], &L->w64.p[1], &L->w64.Mp, &L->wmx.tmp64};
  for (auto pp : d2)
    if ((rc = dmalloc(pp, n)) != TG_OK) return bail(rc);
  float2** f2[] = {&L->Wt32, &L->Wx32, &L->wmx.xs, &L->wmx.rs, &L->wmx.ps[0], &L->wmx.ps[1], &L->wmx.Mps,
                   &L->wmx.ss};
  for (auto pp : f2)
    if ((rc = dmalloc(pp, n)) != TG_OK) return bail(rc);
  if ((rc = dmalloc(&L->st, 1)) != TG_OK || (rc = dmalloc(&L->log, kMaxLog)) != TG_OK ||
      (rc = dmalloc(&L->ts, 1)) != TG_OK || (rc = dmalloc(&L->red.partials, (size_t)nblocks((int)V) + 32)) != TG_OK ||
      (rc = dmalloc(&L->red.counter, 1)) != TG_OK || (rc = dmalloc(&L->bar, kBarWords)) != TG_OK ||
      (rc = dmalloc(&L->pcg_part, 4 * (size_t)kPcgMaxGrid)) != TG_OK)
    return bail(rc);
  if ((rc = ensure_pf(L, 1)) != TG_OK) return bail(rc);
  L->h_stage_len = (size_t)(kMaxPf + 2) * 2 * n;  // npf eta fields + momenta + noise
  if (cudaMallocHost((void**)&L->h_stage, L->h_stage_len * sizeof(double)) != cudaSuccess ||
      cudaMallocHost((void**)&L->h_st, sizeof(CgState)) != cudaSuccess ||
      cudaMallocHost((void**)&L->h_ts, sizeof(TrajStats)) != cudaSuccess ||
      cudaMallocHost((void**)&L->h_log, sizeof(CgLog) * kMaxLog) != cudaSuccess)
    return bail(fail(TG_E_ALLOC, "pinned host allocation failed"));
  if (cudaMemsetAsync(L->A, 0, n * sizeof(double2), L->stream) != cudaSuccess ||
      cudaMemsetAsync(L->noise, 0, n * sizeof(double2), L->stream) != cudaSuccess ||
      cudaMemsetAsync(L->red.counter, 0, sizeof(unsigned), L->stream) != cudaSuccess ||
      cudaMemsetAsync(L->bar, 0, kBarWords * sizeof(unsigned), L->stream) != cudaSuccess ||
      cudaMemsetAsync(L->ts, 0, sizeof(TrajStats), L->stream) != cudaSuccess ||
      cudaMemsetAsync(L->st, 0, sizeof(CgState), L->stream) != cudaSuccess)
    return bail(fail(TG_E_CUDA, "initial memset failed"));
  link_phase(L->stream, L->g, p->bc_t, p->bc_x, L->A, link_out(L));
  if (cudaStreamSynchronize(L->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(TG_E_CUDA, "initialisation kernels failed"));
  L->mt.seed(0);
  *out = L;
  return TG_OK;
}

int tg_destroy(tg_lattice* L) {
  if (!L) return TG_OK;
  cudaSetDevice(L->P.device);
  if (L->stream) cudaStreamSynchronize(L->stream);
  for (auto& kv : L->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  for (auto e : L->ev) cudaEventDestroy(e);
  void* dev[] = {L->A, L->Anew, L->Wt, L->Wx, L->Wt1, L->Wx1, L->mom, L->noise, L->chi, L->Mchi, L->vin, L->vout, L->w64.r,
                 L->w64.p[0], L->w64.p[1], L->w64.Mp, L->wmx.tmp64, L->Wt32, L->Wx32, L->wmx.xs, L->wmx.rs,
                 L->wmx.ps[0], L->wmx.ps[1], L->wmx.Mps, L->wmx.ss,
                 L->st, L->log, L->ts, L->red.partials, L->red.counter, L->bar, L->pcg_part, L->eta, L->phi, L->unif, L->mask,
                 L->rv[0], L->rv[1], L->rv[2], L->rv[3], L->rv[4], L->rv[5]};
  for (void* d : dev)
    if (d) cudaFree(d);
  void* hst[] = {L->h_stage, L->h_st, L->h_ts, L->h_log};
  for (void* h : hst)
    if (h) cudaFreeHost(h);
  if (L->stream) cudaStreamDestroy(L->stream);
  if (L->cap2) cudaStreamDestroy(L->cap2);
  if (L->cap3) cudaStreamDestroy(L->cap3);
  delete L;
  return TG_OK;
}

int tg_set_couplings(tg_lattice* L, double m, double g, double mu) {
  if (!L) return fail(TG_E_ARG, "null lattice");
  if (!(g > 0)) return fail(TG_E_ARG, "g must be positive");
  L->P.m = m;
  L->P.g = g;
  L->P.mu = mu;
  L->version++;
  link_phase(L->stream, L->g, L->P.bc_t, L->P.bc_x, L->A, link_out(L));  // W / m follows m
  TG_CK(cudaGetLastError());
  return TG_OK;
}

int tg_get_params(const tg_lattice* L, tg_lattice_params* p) {
  if (!L || !p) return fail(TG_E_ARG, "null argument");
  *p = L->P;
  return TG_OK;
}

int tg_synchronize(tg_lattice* L) {
  if (!L) return fail(TG_E_ARG, "null lattice");
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}

void* tg_stream(tg_lattice* L) { return L ? (void*)L->stream : nullptr; }

int tg_set_gauge(tg_lattice* L, const double* A) {
  if (!L || !A) return fail(TG_E_ARG, "null argument");
  TG_TRY(upload(L, L->A, A, 2 * (size_t)L->V));
  link_phase(L->stream, L->g, L->P.bc_t, L->P.bc_x, L->A, link_out(L));
  TG_CK(cudaGetLastError());
  return TG_OK;
}

int tg_set_gauge_dev(tg_lattice* L, const void* A_dev) {
  if (!L || !A_dev) return fail(TG_E_ARG, "null argument");
  TG_CK(cudaMemcpyAsync(L->A, A_dev, (size_t)L->V * sizeof(double2), cudaMemcpyDeviceToDevice, L->stream));
  link_phase(L->stream, L->g, L->P.bc_t, L->P.bc_x, L->A, link_out(L));
  TG_CK(cudaGetLastError());
  return TG_OK;
}

int tg_get_gauge(tg_lattice* L, double* A) {
  if (!L || !A) return fail(TG_E_ARG, "null argument");
  return download(L, A, L->A, 2 * (size_t)L->V);
}

int tg_apply(tg_lattice* L, const double* in, double* out, int dagger) {
  if (!L || !in || !out) return fail(TG_E_ARG, "null argument");
  TG_TRY(upload(L, L->vin, in, 2 * (size_t)L->V));
  dslash64(L->stream, L->g, op_k(L, dagger), dagger, L->vin, L->vout, L->Wt, L->Wx);
  TG_CK(cudaGetLastError());
  return download(L, out, L->vout, 2 * (size_t)L->V);
}

int tg_apply_dev(tg_lattice* L, const void* in, void* out, int dagger, int precision) {
  if (!L || !in || !out) return fail(TG_E_ARG, "null argument");
  if (precision == TG_PREC_FP64)
    dslash64(L->stream, L->g, op_k(L, dagger), dagger, (const double2*)in, (double2*)out, L->Wt, L->Wx);
  else if (precision == TG_PREC_MIXED)
    dslash32(L->stream, L->g, op_k32(L, dagger), dagger, (const float2*)in, (float2*)out, L->Wt32, L->Wx32);
  else
    return fail(TG_E_ARG, "bad precision");
  TG_CK(cudaGetLastError());
  return TG_OK;
}

int tg_time_apply(tg_lattice* L, int n, int dagger, int precision, double* ms_per_apply) {
  if (!L || n <= 0 || !ms_per_apply) return fail(TG_E_ARG, "bad argument");
  TG_TRY(ensure_events(L, 2));
  cudaEvent_t e0 = L->ev[0], e1 = L->ev[1];
  TG_CK(cudaEventRecord(e0, L->stream));
  for (int i = 0; i < n; i++) {
    // ping-pong between two buffers so every apply reads the previous output
    if (precision == TG_PREC_FP64) {
      const double2* in = (i & 1) ? L->vout : L->vin;
      double2* out = (i & 1) ? L->vin : L->vout;
      dslash64(L->stream, L->g, op_k(L, dagger), dagger, in, out, L->Wt, L->Wx);
    } else {
      const float2* in = (i & 1) ? L->wmx.Mps : L->wmx.ps[0];
      float2* out = (i & 1) ? L->wmx.ps[0] : L->wmx.Mps;
      dslash32(L->stream, L->g, op_k32(L, dagger), dagger, in, out, L->Wt32, L->Wx32);
    }
  }
  TG_CK(cudaEventRecord(e1, L->stream));
  TG_CK(cudaEventSynchronize(e1));
  TG_CK(cudaGetLastError());
  float ms = 0;
  TG_CK(cudaEventElapsedTime(&ms, e0, e1));
  *ms_per_apply = ms / n;
  return TG_OK;
}

int tg_cg(tg_lattice* L, const tg_cg_params* cp, const double* b, double* x, tg_cg_result* res) {
  Range range("tg_cg");
  if (!L || !b || !x) return fail(TG_E_ARG, "null argument");
  TG_TRY(check_cg_params(cp));
  TG_TRY(upload(L, L->vin, b, 2 * (size_t)L->V));
  tg_cg_result r{};
  TG_TRY(solve_dev(L, *cp, L->vin, L->vout, &r));
  if (res) *res = r;
  TG_TRY(download(L, x, L->vout, 2 * (size_t)L->V));
  return solver_status(r.status);
}

int tg_cg_dev(tg_lattice* L, const tg_cg_params* cp, const void* b_dev, void* x_dev, tg_cg_result* res) {
  if (!L || !b_dev || !x_dev) return fail(TG_E_ARG, "null argument");
  TG_TRY(check_cg_params(cp));
  tg_cg_result r{};
  TG_TRY(solve_dev(L, *cp, (const double2*)b_dev, (double2*)x_dev, &r));
  if (res) *res = r;
  return solver_status(r.status);
}

int tg_gauge_action(tg_lattice* L, double* S) {
  if (!L || !S) return fail(TG_E_ARG, "null argument");
  gauge_action(L->stream, L->g, L->A, kNf / L->P.g, &L->ts->Sg0, L->red);
  TG_CK(cudaGetLastError());
  TG_CK(cudaMemcpyAsync(S, &L->ts->Sg0, sizeof(double), cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}

int tg_pseudofermion_action(tg_lattice* L, const tg_cg_params* cp, const double* phi, double* S,
                            tg_cg_result* res) {
  if (!L || !phi || !S) return fail(TG_E_ARG, "null argument");
  TG_TRY(check_cg_params(cp));
  TG_TRY(upload(L, L->vin, phi, 2 * (size_t)L->V));
  tg_cg_result r{};
  TG_TRY(solve_dev(L, *cp, L->vin, L->vout, &r));
  if (res) *res = r;
  redot(L->stream, L->g, L->vin, L->vout, &L->ts->Spf1, 0, L->red);
  TG_CK(cudaGetLastError());
  TG_CK(cudaMemcpyAsync(S, &L->ts->Spf1, sizeof(double), cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  return solver_status(r.status);
}

int tg_md_action(tg_lattice* L, const double* n, double* S) {
  if (!L || !n || !S) return fail(TG_E_ARG, "null argument");
  TG_TRY(upload(L, L->vin, n, 2 * (size_t)L->V));
  md_action(L->stream, L->g, op_k(L, 1), L->vin, L->Wt, L->Wx, &L->ts->Smd0, L->red);
  TG_CK(cudaGetLastError());
  TG_CK(cudaMemcpyAsync(S, &L->ts->Smd0, sizeof(double), cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}

int tg_force(tg_lattice* L, int npf, const double* chi, const double* noise, double* F) {
  if (!L || !F || npf < 0 || (npf > 0 && !chi)) return fail(TG_E_ARG, "bad argument");
  const size_t V = (size_t)L->V;
  const double ep = exp(L->P.mu), em = exp(-L->P.mu);
  TG_CK(cudaMemsetAsync(L->vout, 0, V * sizeof(double2), L->stream));  // F accumulates in vout
  if (noise) TG_TRY(upload(L, L->noise, noise, 2 * V));
  if (npf == 0)
    force_field(L->stream, L->g, L->P.bc_t, L->P.bc_x, ep, em, L->A, L->Wt, L->Wx, nullptr, nullptr, L->noise, L->vout, kNf / L->P.g,
                1 | (noise ? 2 : 0));
  for (int k = 0; k < npf; k++) {
    TG_TRY(upload(L, L->chi, chi + 2 * V * k, 2 * V));
    dslash64(L->stream, L->g, op_k(L, 0), 0, L->chi, L->Mchi, L->Wt, L->Wx);
    int flags = (k == 0 ? 1 : 0) | ((k == npf - 1 && noise) ? 2 : 0);
    force_field(L->stream, L->g, L->P.bc_t, L->P.bc_x, ep, em, L->A, L->Wt, L->Wx, L->chi, L->Mchi, L->noise, L->vout, kNf / L->P.g,
                flags);
  }
  TG_CK(cudaGetLastError());
  return download(L, F, L->vout, 2 * V);
}

int tg_pf_force(tg_lattice* L, const tg_cg_params* cp, int npf, const double* phi, double* F, tg_cg_result* res) {
  if (!L || !F || npf <= 0 || npf > kMaxPf || !phi) return fail(TG_E_ARG, "bad argument");
  TG_TRY(check_cg_params(cp));
  const size_t V = (size_t)L->V;
  TG_TRY(ensure_pf(L, npf));
  const double ep = exp(L->P.mu), em = exp(-L->P.mu);
  TG_TRY(upload(L, L->phi, phi, 2 * V * npf));
  TG_CK(cudaMemsetAsync(L->vout, 0, V * sizeof(double2), L->stream));  // F accumulates in vout
  tg_cg_result acc{};
  for (int k = 0; k < npf; k++) {
    tg_cg_result r{};
    TG_TRY(solve_dev(L, *cp, L->phi + V * k, L->chi, &r));
    acc.iterations += r.iterations;
    acc.reliable_updates += r.reliable_updates;
    if (r.status > acc.status) acc.status = r.status;
    acc.rr = r.rr;
    acc.rr0 = r.rr0;
    dslash64(L->stream, L->g, op_k(L, 0), 0, L->chi, L->Mchi, L->Wt, L->Wx);
    force_field(L->stream, L->g, L->P.bc_t, L->P.bc_x, ep, em, L->A, L->Wt, L->Wx, L->chi, L->Mchi, nullptr, L->vout, 0.0, 0);
  }
  TG_CK(cudaGetLastError());
  if (res) *res = acc;
  TG_TRY(download(L, F, L->vout, 2 * V));
  return solver_status(acc.status);
}

int tg_momentum_step(tg_lattice* L, const tg_cg_params* cp, double* mom, int npf, const double* phi,
                     const double* noise, double eps, tg_cg_result* res) {
  if (!L || !mom || npf < 0 || npf > kMaxPf || (npf > 0 && !phi)) return fail(TG_E_ARG, "bad argument");
  TG_TRY(check_cg_params(cp));
  const size_t V = (size_t)L->V;
  TG_TRY(ensure_pf(L, npf > 0 ? npf : 1));
  const double ep = exp(L->P.mu), em = exp(-L->P.mu);
  const double gfac = eps * kNf / L->P.g;
  TG_TRY(upload(L, L->mom, mom, 2 * V));
  if (noise) TG_TRY(upload(L, L->noise, noise, 2 * V));
  if (npf > 0) TG_TRY(upload(L, L->phi, phi, 2 * V * npf));
  tg_cg_result acc{};
  if (npf == 0)
    momentum_update(L->stream, L->g, L->P.bc_t, L->P.bc_x, ep, em, L->A, L->Wt, L->Wx, nullptr, nullptr, L->noise, L->mom, eps, gfac,
                    1 | (noise ? 2 : 0));
  for (int k = 0; k < npf; k++) {
    tg_cg_result r{};
    TG_TRY(solve_dev(L, *cp, L->phi + V * k, L->chi, &r));
    acc.iterations += r.iterations;
    acc.reliable_updates += r.reliable_updates;
    if (r.status > acc.status) acc.status = r.status;
    acc.rr = r.rr;
    acc.rr0 = r.rr0;
    dslash64(L->stream, L->g, op_k(L, 0), 0, L->chi, L->Mchi, L->Wt, L->Wx);
    int flags = (k == 0 ? 1 : 0) | ((k == npf - 1 && noise) ? 2 : 0);
    momentum_update(L->stream, L->g, L->P.bc_t, L->P.bc_x, ep, em, L->A, L->Wt, L->Wx, L->chi, L->Mchi, L->noise, L->mom, eps, gfac,
                    flags);
  }
  TG_CK(cudaGetLastError());
  if (res) *res = acc;
  TG_TRY(download(L, mom, L->mom, 2 * V));
  return solver_status(acc.status);
}

int tg_gauge_step(tg_lattice* L, const double* mom, double eps) {
  if (!L || !mom) return fail(TG_E_ARG, "null argument");
  TG_TRY(upload(L, L->mom, mom, 2 * (size_t)L->V));
  gauge_step(L->stream, L->g, L->P.bc_t, L->P.bc_x, L->A, L->mom, 2.0 * eps, 1, link_out(L));
  TG_CK(cudaGetLastError());
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}

int tg_mt_seed(tg_lattice* L, long seed, long warmup) {
  if (!L || warmup < 0) return fail(TG_E_ARG, "bad argument");
  L->mt.seed(seed);
  for (long i = 0; i < warmup; i++) L->mt.next();
  L->mt_seeded = true;
  return TG_OK;
}

// ---- checkpoint -------------------------------------------------------------
// Layout (little-endian, as the host stores it): a fixed header, the MT
// stream's words, its pending outputs, then A.  Offsets in bytes.
namespace {
constexpr char kCkptMagic[8] = {'T', 'G', 'C', 'K', 'P', 'T', '0', '1'};
struct CkptHeader {                 // 72 bytes
  char magic[8];
  int32_t version, nt, nx, bc_t, bc_x, mt_avail, mt_seeded, pad_;
  double m, g, mu;
  uint64_t traj;                    // Philox trajectory counter
};
size_t ckpt_bytes(const tg_lattice* L) {
  return sizeof(CkptHeader) + 624 * sizeof(uint32_t) + 624 * sizeof(double) + 2 * (size_t)L->V * sizeof(double);
}
}  // namespace

size_t tg_checkpoint_size(const tg_lattice* L) { return L ? ckpt_bytes(L) : 0; }

int tg_checkpoint_save(tg_lattice* L, void* buf, size_t size) {
  if (!L || !buf) return fail(TG_E_ARG, "null argument");
  if (size < ckpt_bytes(L)) return fail(TG_E_ARG, "checkpoint buffer too small");
  CkptHeader h{};
  memcpy(h.magic, kCkptMagic, 8);
  h.version = 1;
  h.nt = L->P.nt;
  h.nx = L->P.nx;
  h.bc_t = L->P.bc_t;
  h.bc_x = L->P.bc_x;
  h.mt_avail = L->mt.avail;
  h.mt_seeded = L->mt_seeded ? 1 : 0;
  h.m = L->P.m;
  h.g = L->P.g;
  h.mu = L->P.mu;
  unsigned long long tr = 0;
  TG_CK(cudaMemcpyAsync(&tr, &L->ts->traj, sizeof tr, cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  h.traj = tr;
  unsigned char* q = static_cast<unsigned char*>(buf);
  memcpy(q, &h, sizeof h);
  q += sizeof h;
  memcpy(q, L->mt.w, sizeof L->mt.w);
  q += sizeof L->mt.w;
  memcpy(q, L->mt.out, sizeof L->mt.out);
  q += sizeof L->mt.out;
  TG_TRY(download(L, reinterpret_cast<double*>(q), L->A, 2 * (size_t)L->V));
  return TG_OK;
}

int tg_checkpoint_load(tg_lattice* L, const void* buf, size_t size) {
  if (!L || !buf) return fail(TG_E_ARG, "null argument");
  CkptHeader h;
  if (size < sizeof h) return fail(TG_E_ARG, "not a checkpoint");
  memcpy(&h, buf, sizeof h);
  if (memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) return fail(TG_E_ARG, "not a checkpoint");
  if (h.nt != L->P.nt || h.nx != L->P.nx || h.bc_t != L->P.bc_t || h.bc_x != L->P.bc_x)
    return fail(TG_E_ARG, "checkpoint of another lattice (size or boundary conditions)");
  if (size < ckpt_bytes(L)) return fail(TG_E_ARG, "checkpoint truncated");
  if (h.mt_avail < 0 || h.mt_avail > 624) return fail(TG_E_ARG, "corrupt checkpoint (MT state)");
  const unsigned char* q = static_cast<const unsigned char*>(buf) + sizeof h;
  TG_TRY(tg_set_couplings(L, h.m, h.g, h.mu));
  memcpy(L->mt.w, q, sizeof L->mt.w);
  q += sizeof L->mt.w;
  memcpy(L->mt.out, q, sizeof L->mt.out);
  q += sizeof L->mt.out;
  L->mt.avail = h.mt_avail;
  L->mt_seeded = h.mt_seeded != 0;
  TG_TRY(tg_set_gauge(L, reinterpret_cast<const double*>(q)));
  const unsigned long long tr = h.traj;
  TG_CK(cudaMemcpyAsync(&L->ts->traj, &tr, sizeof tr, cudaMemcpyHostToDevice, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}

int tg_mt_uniforms(tg_lattice* L, double* out, long n) {
  if (!L || (!out && n > 0) || n < 0) return fail(TG_E_ARG, "bad argument");
  for (long i = 0; i < n; i++) out[i] = L->mt.next();
  return TG_OK;
}

int tg_puregauge_ext(tg_lattice* L, const double* u, int sweeps) {
  if (!L || sweeps < 0 || (sweeps > 0 && !u)) return fail(TG_E_ARG, "bad argument");
  const size_t nl = 2 * (size_t)L->V;
  if (!L->unif) TG_TRY(dmalloc(&L->unif, 2 * nl));
  for (int sw = 0; sw < sweeps; sw++) {
    // the 2 uniforms of each of the 2V links of one sweep
    TG_TRY(upload(L, L->unif, u + 2 * nl * sw, 2 * nl));
    puregauge(L->stream, L->g, (double*)L->A, L->unif, -kNf / L->P.g);
    TG_CK(cudaGetLastError());
  }
  link_phase(L->stream, L->g, L->P.bc_t, L->P.bc_x, L->A, link_out(L));
  TG_CK(cudaGetLastError());
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}

int tg_puregauge_sweeps(tg_lattice* L, int sweeps) {
  if (!L || sweeps < 0) return fail(TG_E_ARG, "bad argument");
  const size_t nl = 2 * (size_t)L->V;
  std::vector<double> u(2 * nl);
  for (int sw = 0; sw < sweeps; sw++) {
    for (size_t k = 0; k < 2 * nl; k++) u[k] = L->mt.next();
    TG_TRY(tg_puregauge_ext(L, u.data(), 1));
  }
  return TG_OK;
}

// ---- measurements (hmc.c:794-842) and the masked real operator (vec_ops.c) ----
namespace {
int ensure_real(tg_lattice* L) {
  if (L->mask) return TG_OK;
  TG_TRY(dmalloc(&L->mask, (size_t)L->V));
  for (int k = 0; k < 6; k++) TG_TRY(dmalloc(&L->rv[k], (size_t)L->V));
  return TG_OK;
}
int read_scalar(tg_lattice* L, const double* d, double* h) {
  TG_CK(cudaMemcpyAsync(h, d, sizeof(double), cudaMemcpyDeviceToHost, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  return TG_OK;
}
int upload_mask(tg_lattice* L, const int* mask) {
  TG_CK(cudaMemcpyAsync(L->mask, mask, sizeof(int) * L->V, cudaMemcpyHostToDevice, L->stream));
  return TG_OK;
}
}  // namespace

int tg_magnetisation(tg_lattice* L, double* M) {
  if (!L || !M) return fail(TG_E_ARG, "null argument");
  sum_links(L->stream, L->g, L->A, &L->ts->Sg0, L->red);
  TG_CK(cudaGetLastError());
  double s = 0;
  TG_TRY(read_scalar(L, &L->ts->Sg0, &s));
  *M = s / L->V;
  return TG_OK;
}

int tg_fermion_phase(tg_lattice* L, int sources, const double* noise, double* phase) {
  if (!L || !phase || sources <= 0) return fail(TG_E_ARG, "bad argument");
  const size_t V = (size_t)L->V;
  std::vector<double> draw;
  if (!noise) {  // the reference's stream: V Gaussian pairs per source (hmc.c:802)
    draw.resize(2 * V);
  }
  TG_CK(cudaMemsetAsync(&L->ts->Smd1, 0, sizeof(double), L->stream));
  for (int k = 0; k < sources; k++) {
    const double* src = noise ? noise + 2 * V * k : nullptr;
    if (!noise) {
      L->mt.gauss_pairs((long)V, draw.data());
      src = draw.data();
    }
    TG_TRY(upload(L, L->vin, src, 2 * V));
    dslash64(L->stream, L->g, op_k(L, 1), 1, L->vin, L->vout, L->Wt, L->Wx);
    imdot(L->stream, L->g, L->vin, L->vout, &L->ts->Smd1, 1, L->red);
    TG_CK(cudaGetLastError());
  }
  double s = 0;
  TG_TRY(read_scalar(L, &L->ts->Smd1, &s));
  *phase = s / sources;
  return TG_OK;
}

int tg_chiral_condensate(tg_lattice* L, const tg_cg_params* cp, int sources, unsigned long long seed, double* pbp,
                         double* err) {
  if (!L || !pbp || sources <= 0) return fail(TG_E_ARG, "bad argument");
  TG_TRY(check_cg_params(cp));
  std::vector<double> vals(sources);
  for (int k = 0; k < sources; k++) {
    philox_gauss(L->stream, L->g, seed, L->ts, 64u + (unsigned)k, L->vin);    // eta
    dslash64(L->stream, L->g, op_k(L, 1), 1, L->vin, L->Mchi, L->Wt, L->Wx);  // M^dag eta
    TG_CK(cudaGetLastError());
    tg_cg_result r{};
    TG_TRY(solve_dev(L, *cp, L->Mchi, L->chi, &r));                         // M^-1 eta
    if (r.status != TG_OK) return solver_status(r.status);
    redot(L->stream, L->g, L->vin, L->chi, &L->ts->Smd1, 0, L->red);
    TG_CK(cudaGetLastError());
    TG_TRY(read_scalar(L, &L->ts->Smd1, &vals[k]));
    vals[k] /= 2.0 * L->V;  // E[eta eta^dag] = 2 for complex Gaussian noise of unit-variance parts
  }
  double mean = 0;
  for (double v : vals) mean += v;
  mean /= sources;
  double var = 0;
  for (double v : vals) var += (v - mean) * (v - mean);
  *pbp = mean;
  if (err) *err = sources > 1 ? sqrt(var / (sources - 1) / sources) : 0.0;
  return TG_OK;
}

int tg_fm_apply(tg_lattice* L, const int* mask, const double* in, double* out, int transpose) {
  if (!L || !mask || !in || !out) return fail(TG_E_ARG, "null argument");
  TG_TRY(ensure_real(L));
  TG_TRY(upload_mask(L, mask));
  TG_TRY(upload(L, L->rv[0], in, (size_t)L->V));
  fm_apply(L->stream, L->g, L->P.m, L->P.mu, L->P.bc_t, L->P.bc_x, L->mask, L->rv[0], L->rv[1], transpose);
  TG_CK(cudaGetLastError());
  return download(L, out, L->rv[1], (size_t)L->V);
}

int tg_cg_mdm_masked(tg_lattice* L, const tg_cg_params* cp, const int* mask, const double* b, double* x,
                     tg_cg_result* res) {
  if (!L || !mask || !b || !x) return fail(TG_E_ARG, "null argument");
  TG_TRY(check_cg_params(cp));
  TG_TRY(ensure_real(L));
  TG_TRY(upload_mask(L, mask));
  TG_TRY(upload(L, L->rv[0], b, (size_t)L->V));
  rcg_init(L->stream, L->g, L->rv[0], L->rv[1], L->rv[2], L->rv[3], cp->rel_tol, cp->abs_tol2, cp->maxiter, L->st,
           L->red);
  TG_CK(cudaGetLastError());
  const int chunk = 16;
  const long max_chunks = (long)cp->maxiter / chunk + 2;
  for (long c = 0;; c++) {
    TG_CK(cudaMemcpyAsync(L->h_st, L->st, sizeof(CgState), cudaMemcpyDeviceToHost, L->stream));
    TG_CK(cudaStreamSynchronize(L->stream));
    if (L->h_st->done) break;
    if (c >= max_chunks) return fail(TG_E_NOCONV, "CG loop did not terminate");
    for (int j = 0; j < chunk; j++)
      rcg_iter(L->stream, L->g, L->P.m, L->P.mu, L->P.bc_t, L->P.bc_x, L->mask, L->rv[1], L->rv[2], L->rv[3],
               L->rv[4], L->rv[5], L->st, L->red);
    TG_CK(cudaGetLastError());
  }
  if (res) {
    res->iterations = L->h_st->iter;
    res->status = L->h_st->status;
    res->reliable_updates = 0;
    res->rr = L->h_st->rr;
    res->rr0 = L->h_st->rr0;
  }
  TG_TRY(download(L, x, L->rv[1], (size_t)L->V));
  return solver_status(L->h_st->status);
}

int tg_fm_propagator(tg_lattice* L, const tg_cg_params* cp, const int* mask, double* Dinv, tg_cg_result* res) {
  if (!L || !Dinv) return fail(TG_E_ARG, "null argument");
  TG_TRY(check_cg_params(cp));
  if (L->P.nx % 2 != 0) return fail(TG_E_ARG, "the propagator matrix needs an even nx");
  if (L->V > 16384) return fail(TG_E_ARG, "the propagator matrix is for lattices of at most 16384 sites");
  TG_TRY(ensure_real(L));
  const int V = L->V;
  if (mask) {
    TG_TRY(upload_mask(L, mask));
  } else {
    TG_CK(cudaMemsetAsync(L->mask, 0, sizeof(int) * V, L->stream));
  }
  const size_t nD = (size_t)V * V / 2;
  // sources per launch: their CG vectors (5 V doubles each) within 1 GiB
  const size_t per_src = 5 * (size_t)V;
  int nb = (int)std::min<size_t>((size_t)V, std::max<size_t>(1, ((size_t)1 << 27) / per_src));
  double *dD = nullptr, *scratch = nullptr;
  int* stats = nullptr;
  TG_TRY(dmalloc(&dD, nD));
  int rc = dmalloc(&scratch, per_src * nb);
  if (rc == TG_OK) rc = dmalloc(&stats, 2);
  if (rc == TG_OK && cudaMemsetAsync(stats, 0, 2 * sizeof(int), L->stream) != cudaSuccess)
    rc = fail(TG_E_CUDA, "memset failed");
  if (rc == TG_OK) {
    PropArgs a{};
    a.g = L->g;
    a.m = L->P.m;
    a.ep = exp(L->P.mu);
    a.em = exp(-L->P.mu);
    a.bc_t = L->P.bc_t;
    a.bc_x = L->P.bc_x;
    a.mask = L->mask;
    a.scratch = scratch;
    a.Dinv = dD;
    a.abs_tol2 = cp->abs_tol2;
    a.rel_tol = cp->rel_tol;
    a.maxiter = cp->maxiter;
    a.max_iter = stats;
    a.worst = stats + 1;
    for (int src0 = 0; src0 < V && rc == TG_OK; src0 += nb) {
      a.src0 = src0;
      prop_cg(L->stream, std::min(nb, V - src0), a);
      if (cudaGetLastError() != cudaSuccess) rc = fail(TG_E_CUDA, "propagator kernel launch failed");
    }
  }
  int h[2] = {0, 0};
  if (rc == TG_OK && (cudaMemcpyAsync(Dinv, dD, nD * sizeof(double), cudaMemcpyDeviceToHost, L->stream) != cudaSuccess ||
                      cudaMemcpyAsync(h, stats, sizeof h, cudaMemcpyDeviceToHost, L->stream) != cudaSuccess ||
                      cudaStreamSynchronize(L->stream) != cudaSuccess))
    rc = fail(TG_E_CUDA, "propagator matrix failed");
  cudaFree(dD);
  if (scratch) cudaFree(scratch);
  if (stats) cudaFree(stats);
  if (rc != TG_OK) return rc;
  if (res) {
    res->iterations = h[0];
    res->status = h[1];
    res->reliable_updates = 0;
    res->rr = 0;
    res->rr0 = 0;
  }
  return solver_status(h[1]);
}

int tg_dense_M(tg_lattice* L, double* Md) {
  if (!L || !Md) return fail(TG_E_ARG, "null argument");
  if (L->V > 4096) return fail(TG_E_ARG, "dense M only for lattices of at most 4096 sites");
  const size_t n = (size_t)L->V * L->V;
  double2* d = nullptr;
  TG_TRY(dmalloc(&d, n));
  dense_M(L->stream, L->g, op_k(L, 0), L->Wt, L->Wx, d);
  cudaError_t e1 = cudaGetLastError();
  cudaError_t e2 = cudaMemcpyAsync(Md, d, n * sizeof(double2), cudaMemcpyDeviceToHost, L->stream);
  cudaError_t e3 = cudaStreamSynchronize(L->stream);
  cudaFree(d);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) return fail(TG_E_CUDA, "dense M failed");
  return TG_OK;
}

int tg_log_det(tg_lattice* L, int nconf, const double* A, double* logabs, double* phase) {
  if (!L || nconf <= 0 || !logabs || !phase) return fail(TG_E_ARG, "bad argument");
  if (L->V > 1024) return fail(TG_E_ARG, "determinant only for lattices of at most 1024 sites");
  const size_t V = (size_t)L->V, n = V * V;
  double2* mats = nullptr;
  double* out = nullptr;
  TG_TRY(dmalloc(&mats, n * nconf));
  if (dmalloc(&out, 2 * (size_t)nconf) != TG_OK) { cudaFree(mats); return TG_E_ALLOC; }
  int rc = TG_OK;
  std::vector<double> h(2 * (size_t)nconf);
  for (int c = 0; c < nconf && rc == TG_OK; c++) {
    if (A) rc = tg_set_gauge(L, A + 2 * V * c);
    if (rc == TG_OK) dense_M(L->stream, L->g, op_k(L, 0), L->Wt, L->Wx, mats + n * c);
  }
  if (rc == TG_OK) {
    lu_logdet(L->stream, (int)V, nconf, mats, out);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(h.data(), out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, L->stream) != cudaSuccess ||
        cudaStreamSynchronize(L->stream) != cudaSuccess)
      rc = fail(TG_E_CUDA, "determinant kernel failed");
  }
  cudaFree(mats);
  cudaFree(out);
  if (rc != TG_OK) return rc;
  for (int c = 0; c < nconf; c++) {
    logabs[c] = h[2 * c];
    phase[c] = h[2 * c + 1];
  }
  return TG_OK;
}

int tg_trajectory(tg_lattice* L, const tg_hmc_params* p, tg_traj_result* r) {
  if (!L) return fail(TG_E_ARG, "null lattice");
  TG_TRY(check_hmc_params(p));
  if (p->rng == TG_RNG_PHILOX) return run_trajectory(L, *p, r);
  if (p->rng != TG_RNG_MT) return fail(TG_E_ARG, "tg_trajectory needs TG_RNG_MT or TG_RNG_PHILOX");
  // the reference's order: pseudofermion pairs, momentum pairs, noise pairs
  // (hmc.c:695-698), then the accept uniform (hmc.c:738)
  const size_t V = (size_t)L->V;
  TG_TRY(ensure_pf(L, p->npf > 0 ? p->npf : 1));
  double* h = L->h_stage;
  size_t off = 0;
  size_t n_eta = 2 * V * p->npf;
  L->mt.gauss_pairs((long)V * p->npf, h);
  off += n_eta;
  L->mt.gauss_pairs((long)V, h + off);
  off += 2 * V;
  if (p->stochastic_term) L->mt.gauss_pairs((long)V, h + off);
  double u = L->mt.next();
  if (n_eta) TG_CK(cudaMemcpyAsync(L->eta, h, n_eta * sizeof(double), cudaMemcpyHostToDevice, L->stream));
  TG_CK(cudaMemcpyAsync(L->mom, h + n_eta, 2 * V * sizeof(double), cudaMemcpyHostToDevice, L->stream));
  if (p->stochastic_term)
    TG_CK(cudaMemcpyAsync(L->noise, h + n_eta + 2 * V, 2 * V * sizeof(double), cudaMemcpyHostToDevice, L->stream));
  L->h_ts->u = u;
  TG_CK(cudaMemcpyAsync(&L->ts->u, &L->h_ts->u, sizeof(double), cudaMemcpyHostToDevice, L->stream));
  TG_CK(cudaStreamSynchronize(L->stream));
  return run_trajectory(L, *p, r);
}

int tg_trajectory_ext(tg_lattice* L, const tg_hmc_params* p, const double* eta, const double* mom,
                      const double* noise, double u_accept, tg_traj_result* r) {
  if (!L || !mom || (p && p->npf > 0 && !eta) || (p && p->stochastic_term && !noise))
    return fail(TG_E_ARG, "null argument");
  TG_TRY(check_hmc_params(p));
  const size_t V = (size_t)L->V;
  TG_TRY(ensure_pf(L, p->npf > 0 ? p->npf : 1));
  if (p->npf > 0) TG_TRY(upload(L, L->eta, eta, 2 * V * p->npf));
  TG_TRY(upload(L, L->mom, mom, 2 * V));
  if (p->stochastic_term) TG_TRY(upload(L, L->noise, noise, 2 * V));
  L->h_ts->u = u_accept;
  TG_CK(cudaMemcpyAsync(&L->ts->u, &L->h_ts->u, sizeof(double), cudaMemcpyHostToDevice, L->stream));
  tg_hmc_params q = *p;
  q.rng = TG_RNG_EXTERNAL;
  return run_trajectory(L, q, r);
}

}  // extern "C"

// ===========================================================================
// Batched chains
// ===========================================================================
struct tg_batch {
  int device = 0;
  int n = 0;
  long long total = 0;
  std::vector<tg_chain_params> P;
  std::vector<long long> off;
  std::vector<int> order;  // the work queue: chains by estimated cost, largest first
  cudaStream_t stream = nullptr;
  cudaStream_t filler = nullptr;               // the filler blocks' stream (batch_filler_launch)
  cudaEvent_t fork = nullptr, join = nullptr;  // ordering it into `stream` (also under graph capture)
  // instances with pairs: the queue's first pair_top chains (estimated cost
  // above twice an SM's share of the batch) run on 4-block clusters
  int pair_top = 0;
  BatchChain* d_chains = nullptr;
  int* d_order = nullptr;
  ChainResult* d_res = nullptr;
  ChainResult* h_res = nullptr;
  unsigned long long* d_queue = nullptr;
  BatchFields F{};
  int sms = 1;
  int tuned_cfg = 1;  // index into kBatchCfgs
  std::map<std::string, GraphEntry> graphs;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace {

// kernel instance for p.block: 0 the tuned one; a block size the first
// one-block-per-chain instance with that size; an instance id as
// tg_batch_autotune reports it that instance
int batch_cfg(const tg_batch* B, const tg_batch_params& p) {
  if (p.block <= 0) return B->tuned_cfg;
  for (int c = 0; c < kBatchNumCfgs; c++)
    if (batch_cfg_id(kBatchCfgs[c]) == p.block) return c;
  for (int c = 0; c < kBatchNumCfgs; c++)
    if (kBatchCfgs[c].block == p.block) return c;
  return -1;
}

int batch_launch(tg_batch* B, const tg_batch_params& p, int cfg, cudaStream_t s) {
  if (cfg < 0 || cfg >= kBatchNumCfgs) return fail(TG_E_ARG, "unknown batch kernel instance");
  if (batch_teams(cfg, B->sms) <= 0) return fail(TG_E_CUDA, "batch kernel instance cannot launch on this GPU");
  BatchTraj t;
  t.nsteps = p.nsteps;
  t.tau = p.tau;
  t.stochastic_term = p.stochastic_term;
  t.cg = BatchCg{p.cg.rel_tol, p.cg.abs_tol2, p.cg.maxiter, p.cg.precision, p.cg.ru_interval};
  t.from_back = 0;
  // cluster instances with solo_sites: single blocks from the first queued chain that small
  t.solo_from = B->n;
  if (kBatchCfgs[cfg].cluster > 1 && kBatchCfgs[cfg].solo_sites > 0)
    for (int q = 0; q < B->n; q++)
      if ((long long)B->P[B->order[q]].nt * B->P[B->order[q]].nx <= kBatchCfgs[cfg].solo_sites) {
        t.solo_from = q;
        break;
      }
  t.pair_end = t.solo_from;
  if (kBatchCfgs[cfg].pairs) t.solo_from = std::min(B->pair_top, t.pair_end);
  TG_CK(cudaMemsetAsync(B->d_queue, 0, sizeof(unsigned long long), s));
  // filler blocks on the SMs the clusters leave idle, on a stream forked from s
  // after the queue's reset and joined back into s; launched after the cluster
  // kernel, whose clusters should take their SMs first
  const int fill = (t.pair_end < B->n) ? batch_filler_blocks(cfg, B->sms) : 0;
  if (fill > 0) TG_CK(cudaEventRecord(B->fork, s));
  batch_trajectory(s, cfg, B->sms, B->d_chains, B->d_order, B->n, B->F, t, B->d_res, B->d_queue);
  TG_CK(cudaGetLastError());
  if (fill > 0) {
    BatchTraj tf = t;
    tf.solo_from = t.pair_end;  // the filler draws one-block chains only
    TG_CK(cudaStreamWaitEvent(B->filler, B->fork, 0));
    batch_filler_launch(B->filler, cfg, fill, B->d_chains, B->d_order, B->n, B->F, tf, B->d_res, B->d_queue);
    TG_CK(cudaGetLastError());
    TG_CK(cudaEventRecord(B->join, B->filler));
    TG_CK(cudaStreamWaitEvent(s, B->join, 0));
  }
  return TG_OK;
}

int batch_run(tg_batch* B, const tg_batch_params& p, int cfg, double* ms) {
  char buf[256];
  snprintf(buf, sizeof buf, "b%d/%d/%.17g/%d/", cfg, p.nsteps, p.tau, p.stochastic_term);
  std::string key = buf + cg_key(p.cg);
  TG_CK(cudaEventRecord(B->e0, B->stream));
  if (p.use_graph && env_graph_enabled()) {
    auto it = B->graphs.find(key);
    if (it == B->graphs.end()) {
      GraphEntry ge;
      TG_CK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
      int rc = batch_launch(B, p, cfg, B->stream);
      cudaGraph_t gr = nullptr;
      cudaError_t e = cudaStreamEndCapture(B->stream, &gr);
      if (rc != TG_OK) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
      }
      if (e != cudaSuccess) return fail(TG_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
      ge.graph = gr;
      TG_CK(cudaGraphInstantiate(&ge.exec, gr, 0));
      it = B->graphs.emplace(key, ge).first;
    }
    TG_CK(cudaGraphLaunch(it->second.exec, B->stream));
  } else {
    TG_TRY(batch_launch(B, p, cfg, B->stream));
  }
  TG_CK(cudaEventRecord(B->e1, B->stream));
  TG_CK(cudaMemcpyAsync(B->h_res, B->d_res, sizeof(ChainResult) * B->n, cudaMemcpyDeviceToHost, B->stream));
  TG_CK(cudaStreamSynchronize(B->stream));
  float f = 0;
  TG_CK(cudaEventElapsedTime(&f, B->e0, B->e1));
  if (ms) *ms = f;
  return TG_OK;
}

int check_batch_params(const tg_batch_params* p) {
  if (!p) return fail(TG_E_ARG, "null batch parameters");
  if (p->nsteps <= 0 || !(p->tau > 0)) return fail(TG_E_ARG, "nsteps and tau must be positive");
  bool known = p->block == 0;
  for (int c = 0; c < kBatchNumCfgs && !known; c++)
    known = p->block == kBatchCfgs[c].block || p->block == batch_cfg_id(kBatchCfgs[c]);
  if (!known) return fail(TG_E_ARG, "block must be 0, a block size (128, 256, 384, 512) or an instance id");
  return check_cg_params(&p->cg);
}

}  // namespace

extern "C" {

int tg_batch_create(const tg_chain_params* chains, int nchains, int device, tg_batch** out) {
  if (!chains || nchains <= 0 || !out) return fail(TG_E_ARG, "bad argument");
  *out = nullptr;
  TG_CK(cudaSetDevice(device));
  tg_batch* B = new tg_batch();
  auto bail = [&](int rc) { tg_batch_destroy(B); return rc; };
  B->device = device;
  B->n = nchains;
  B->P.assign(chains, chains + nchains);
  std::vector<BatchChain> hc(nchains);
  long long total = 0;
  for (int i = 0; i < nchains; i++) {
    const tg_chain_params& c = chains[i];
    auto bc_ok = [](int b) { return b == 1 || b == -1 || b == 0; };
    if (c.nt < 2 || c.nx < 2 || (long long)c.nt * c.nx >= (1LL << 24) || !bc_ok(c.bc_t) || !bc_ok(c.bc_x) ||
        !(c.g > 0))
      return bail(fail(TG_E_ARG, "invalid chain " + std::to_string(i)));
    BatchChain& b = hc[i];
    memset(&b, 0, sizeof b);
    b.geo.nt = c.nt;
    b.geo.nx = c.nx;
    b.geo.V = c.nt * c.nx;
    b.geo.inv_nx = 1.0f / (float)c.nx;
    b.m = c.m;
    b.g = c.g;
    b.mu = c.mu;
    b.bc_t = c.bc_t;
    b.bc_x = c.bc_x;
    b.seed = c.seed;
    b.off = total;
    B->off.push_back(total);
    total += b.geo.V;
  }
  B->total = total;
  // largest estimated cost first: sites x 1/m (CG iterations grow like 1/m)
  std::vector<int> order(nchains);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    double ca = (double)hc[a].geo.V / std::max(fabs(hc[a].m), 1e-3);
    double cb = (double)hc[b].geo.V / std::max(fabs(hc[b].m), 1e-3);
    return ca > cb;
  });
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&B->filler, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&B->e0) != cudaSuccess || cudaEventCreate(&B->e1) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&B->join, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(TG_E_CUDA, "stream/event creation failed"));
  cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, device);
  if (B->sms <= 0) B->sms = 1;
  int rc;
  double2** d2[] = {&B->F.A, &B->F.An, &B->F.mom, &B->F.phi, &B->F.noise, &B->F.x, &B->F.Mx, &B->F.tmp,
                    &B->F.Wt, &B->F.Wx, &B->F.r64, &B->F.p64, &B->F.p64b, &B->F.Mp64};
  for (auto pp : d2)
    if ((rc = dmalloc(pp, (size_t)total)) != TG_OK) return bail(rc);
  float2** f2[] = {&B->F.Wt32, &B->F.Wx32, &B->F.xs, &B->F.rs, &B->F.ps, &B->F.ps2, &B->F.Mps};
  for (auto pp : f2)
    if ((rc = dmalloc(pp, (size_t)total)) != TG_OK) return bail(rc);
  if ((rc = dmalloc(&B->d_chains, nchains)) != TG_OK || (rc = dmalloc(&B->d_order, nchains)) != TG_OK ||
      (rc = dmalloc(&B->d_res, nchains)) != TG_OK || (rc = dmalloc(&B->d_queue, 1)) != TG_OK)
    return bail(rc);
  if (cudaMallocHost((void**)&B->h_res, sizeof(ChainResult) * nchains) != cudaSuccess)
    return bail(fail(TG_E_ALLOC, "pinned allocation failed"));
  B->order = order;
  {
    auto cost = [&](int c) { return (double)hc[c].geo.V / std::max(fabs(hc[c].m), 1e-3); };
    double w = 0;
    for (int c = 0; c < nchains; c++) w += cost(c);
    const double share = w / B->sms;
    int top = 0;
    while (top < nchains && cost(order[top]) > 2.0 * share) top++;
    B->pair_top = top;
  }
  if (cudaMemcpyAsync(B->d_chains, hc.data(), sizeof(BatchChain) * nchains, cudaMemcpyHostToDevice, B->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(B->d_order, order.data(), sizeof(int) * nchains, cudaMemcpyHostToDevice, B->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(B->d_res, 0, sizeof(ChainResult) * nchains, B->stream) != cudaSuccess ||
      cudaMemsetAsync(B->F.A, 0, sizeof(double2) * total, B->stream) != cudaSuccess ||
      cudaMemsetAsync(B->F.noise, 0, sizeof(double2) * total, B->stream) != cudaSuccess ||
      cudaStreamSynchronize(B->stream) != cudaSuccess)
    return bail(fail(TG_E_CUDA, "batch initialisation failed"));
  *out = B;
  return TG_OK;
}

int tg_batch_destroy(tg_batch* B) {
  if (!B) return TG_OK;
  cudaSetDevice(B->device);
  if (B->stream) cudaStreamSynchronize(B->stream);
  for (auto& kv : B->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  void* dev[] = {B->F.A, B->F.An, B->F.mom, B->F.phi, B->F.noise, B->F.x, B->F.Mx, B->F.tmp, B->F.Wt, B->F.Wx,
                 B->F.r64, B->F.p64, B->F.p64b, B->F.Mp64, B->F.Wt32, B->F.Wx32, B->F.xs, B->F.rs, B->F.ps,
                 B->F.ps2, B->F.Mps,
                 B->d_chains, B->d_order, B->d_res, B->d_queue};
  for (void* d : dev)
    if (d) cudaFree(d);
  if (B->h_res) cudaFreeHost(B->h_res);
  if (B->e0) cudaEventDestroy(B->e0);
  if (B->e1) cudaEventDestroy(B->e1);
  if (B->fork) cudaEventDestroy(B->fork);
  if (B->join) cudaEventDestroy(B->join);
  if (B->filler) cudaStreamDestroy(B->filler);
  if (B->stream) cudaStreamDestroy(B->stream);
  delete B;
  return TG_OK;
}

int tg_batch_size(const tg_batch* B, int* nchains, long long* total_sites) {
  if (!B) return fail(TG_E_ARG, "null batch");
  if (nchains) *nchains = B->n;
  if (total_sites) *total_sites = B->total;
  return TG_OK;
}

int tg_batch_set_gauge(tg_batch* B, int chain, const double* A) {
  if (!B || !A || chain < 0 || chain >= B->n) return fail(TG_E_ARG, "bad argument");
  size_t V = (size_t)B->P[chain].nt * B->P[chain].nx;
  TG_CK(cudaMemcpyAsync(B->F.A + B->off[chain], A, V * sizeof(double2), cudaMemcpyHostToDevice, B->stream));
  TG_CK(cudaStreamSynchronize(B->stream));
  return TG_OK;
}

int tg_batch_get_gauge(tg_batch* B, int chain, double* A) {
  if (!B || !A || chain < 0 || chain >= B->n) return fail(TG_E_ARG, "bad argument");
  size_t V = (size_t)B->P[chain].nt * B->P[chain].nx;
  TG_CK(cudaMemcpyAsync(A, B->F.A + B->off[chain], V * sizeof(double2), cudaMemcpyDeviceToHost, B->stream));
  TG_CK(cudaStreamSynchronize(B->stream));
  return TG_OK;
}

// ---- batch checkpoint --------------------------------------------------------
namespace {
constexpr char kBatchCkptMagic[8] = {'T', 'G', 'B', 'A', 'T', 'C', 'H', '1'};
struct BatchCkptHeader {  // 24 bytes
  char magic[8];
  int32_t version, nchains;
  int64_t total_sites;
};
struct BatchCkptChain {  // 56 bytes
  int32_t nt, nx, bc_t, bc_x;
  double m, g, mu;
  uint64_t seed, traj;  // traj: the chain's Philox trajectory counter
};
size_t batch_ckpt_bytes(const tg_batch* B) {
  return sizeof(BatchCkptHeader) + (size_t)B->n * sizeof(BatchCkptChain) + 2 * (size_t)B->total * sizeof(double);
}
int batch_download_results(tg_batch* B) {
  TG_CK(cudaMemcpyAsync(B->h_res, B->d_res, sizeof(ChainResult) * B->n, cudaMemcpyDeviceToHost, B->stream));
  TG_CK(cudaStreamSynchronize(B->stream));
  return TG_OK;
}
}  // namespace

size_t tg_batch_checkpoint_size(const tg_batch* B) { return B ? batch_ckpt_bytes(B) : 0; }

int tg_batch_checkpoint_save(tg_batch* B, void* buf, size_t size) {
  if (!B || !buf) return fail(TG_E_ARG, "null argument");
  if (size < batch_ckpt_bytes(B)) return fail(TG_E_ARG, "checkpoint buffer too small");
  TG_CK(cudaSetDevice(B->device));
  TG_TRY(batch_download_results(B));
  unsigned char* q = static_cast<unsigned char*>(buf);
  BatchCkptHeader h{};
  memcpy(h.magic, kBatchCkptMagic, 8);
  h.version = 1;
  h.nchains = B->n;
  h.total_sites = B->total;
  memcpy(q, &h, sizeof h);
  q += sizeof h;
  for (int i = 0; i < B->n; i++) {
    const tg_chain_params& c = B->P[i];
    BatchCkptChain e{c.nt, c.nx, c.bc_t, c.bc_x, c.m, c.g, c.mu, c.seed, B->h_res[i].traj};
    memcpy(q, &e, sizeof e);
    q += sizeof e;
  }
  TG_CK(cudaMemcpyAsync(q, B->F.A, sizeof(double2) * B->total, cudaMemcpyDeviceToHost, B->stream));
  TG_CK(cudaStreamSynchronize(B->stream));
  return TG_OK;
}

int tg_batch_checkpoint_load(tg_batch* B, const void* buf, size_t size) {
  if (!B || !buf) return fail(TG_E_ARG, "null argument");
  BatchCkptHeader h;
  if (size < sizeof h) return fail(TG_E_ARG, "not a batch checkpoint");
  memcpy(&h, buf, sizeof h);
  if (memcmp(h.magic, kBatchCkptMagic, 8) != 0 || h.version != 1) return fail(TG_E_ARG, "not a batch checkpoint");
  if (h.nchains != B->n || h.total_sites != B->total || size < batch_ckpt_bytes(B))
    return fail(TG_E_ARG, "checkpoint of another batch (chain count or size)");
  const unsigned char* q = static_cast<const unsigned char*>(buf) + sizeof h;
  std::vector<uint64_t> traj(B->n);
  for (int i = 0; i < B->n; i++) {
    BatchCkptChain e;
    memcpy(&e, q + i * sizeof e, sizeof e);
    const tg_chain_params& c = B->P[i];
    if (e.nt != c.nt || e.nx != c.nx || e.bc_t != c.bc_t || e.bc_x != c.bc_x || e.m != c.m || e.g != c.g ||
        e.mu != c.mu || e.seed != c.seed)
      return fail(TG_E_ARG, "checkpoint of another batch (chain " + std::to_string(i) + " differs)");
    traj[i] = e.traj;
  }
  q += (size_t)B->n * sizeof(BatchCkptChain);
  TG_CK(cudaSetDevice(B->device));
  TG_TRY(batch_download_results(B));
  for (int i = 0; i < B->n; i++) B->h_res[i].traj = traj[i];
  TG_CK(cudaMemcpyAsync(B->d_res, B->h_res, sizeof(ChainResult) * B->n, cudaMemcpyHostToDevice, B->stream));
  TG_CK(cudaMemcpyAsync(B->F.A, q, sizeof(double2) * B->total, cudaMemcpyHostToDevice, B->stream));
  TG_CK(cudaStreamSynchronize(B->stream));
  return TG_OK;
}

int tg_batch_trajectory(tg_batch* B, const tg_batch_params* p, tg_traj_result* results) {
  Range range("tg_batch_trajectory");
  if (!B) return fail(TG_E_ARG, "null batch");
  TG_TRY(check_batch_params(p));
  TG_CK(cudaSetDevice(B->device));
  double ms = 0;
  TG_TRY(batch_run(B, *p, batch_cfg(B, *p), &ms));
  int worst = TG_OK;
  for (int i = 0; i < B->n; i++) {
    const ChainResult& c = B->h_res[i];
    worst = std::max(worst, c.status);
    if (!results) continue;
    tg_traj_result& r = results[i];
    memset(&r, 0, sizeof r);
    r.dH = c.dH;
    r.Sg0 = c.Sg0; r.Spf0 = c.Spf0; r.Smd0 = c.Smd0; r.Smom0 = c.Smom0;
    r.Sg1 = c.Sg1; r.Spf1 = c.Spf1; r.Smd1 = c.Smd1; r.Smom1 = c.Smom1;
    r.u_accept = c.u;
    r.accepted = c.accepted;
    r.status = c.status;
    r.cg_solves = c.solves;
    r.cg_iterations = c.cg_iterations;
    r.cg_max_iterations = c.cg_max_iterations;
    r.reliable_updates = c.reliable_updates;
    r.cg_ms = ms;
  }
  return solver_status(worst);
}

int tg_batch_autotune(tg_batch* B, const tg_batch_params* p, int* best_block, double* best_ms) {
  if (!B) return fail(TG_E_ARG, "null batch");
  TG_TRY(check_batch_params(p));
  TG_CK(cudaSetDevice(B->device));
  // save the chains' state (gauge fields and trajectory counters)
  double2* A0 = nullptr;
  ChainResult* R0 = nullptr;
  TG_TRY(dmalloc(&A0, (size_t)B->total));
  if (dmalloc(&R0, (size_t)B->n) != TG_OK) { cudaFree(A0); return TG_E_ALLOC; }
  auto cleanup = [&]() { cudaFree(A0); cudaFree(R0); };
  if (cudaMemcpyAsync(A0, B->F.A, sizeof(double2) * B->total, cudaMemcpyDeviceToDevice, B->stream) != cudaSuccess ||
      cudaMemcpyAsync(R0, B->d_res, sizeof(ChainResult) * B->n, cudaMemcpyDeviceToDevice, B->stream) != cudaSuccess) {
    cleanup();
    return fail(TG_E_CUDA, "autotune state copy failed");
  }
  int best = -1;
  double bms = 1e300;
  for (int c = 0; c < kBatchNumCfgs; c++) {
    if (batch_teams(c, B->sms) <= 0) continue;
    double ms = 0;
    tg_batch_params q = *p;
    q.use_graph = 0;
    int rc = batch_run(B, q, c, &ms);
    if (rc == TG_OK && ms < bms) { bms = ms; best = c; }
    if (cudaMemcpyAsync(B->F.A, A0, sizeof(double2) * B->total, cudaMemcpyDeviceToDevice, B->stream) != cudaSuccess ||
        cudaMemcpyAsync(B->d_res, R0, sizeof(ChainResult) * B->n, cudaMemcpyDeviceToDevice, B->stream) !=
            cudaSuccess) {
      cleanup();
      return fail(TG_E_CUDA, "autotune state restore failed");
    }
  }
  cudaStreamSynchronize(B->stream);
  cleanup();
  if (best < 0) return fail(TG_E_CUDA, "no kernel instance could run the batch");
  B->tuned_cfg = best;
  if (best_block) *best_block = batch_cfg_id(kBatchCfgs[best]);
  if (best_ms) *best_ms = bms;
  return TG_OK;
}

}  // extern "C"
