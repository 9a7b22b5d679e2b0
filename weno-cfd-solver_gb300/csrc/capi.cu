// C ABI (include/weno_gb300.h): argument checks, workspace layout, dispatch to
// the launchers of the exact / fast translation units, and the device-resident
// SSP-RK3 solver.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/weno_gb300.h"
#include "ctx_id.h"
#include <nvtx3/nvToolsExt.h>

#include "df64.cuh"
#include "errors.h"
#include "launch_api.h"
#include "step_ctl.h"

using namespace weno;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(WENO_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define WENO_CK(...)                                           \
  do {                                                         \
    cudaError_t e_ = (__VA_ARGS__);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #__VA_ARGS__); \
  } while (0)

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
inline int64_t align_elems(int64_t x) { return (x + 63) / 64 * 64; }  // 256 B for f32, 512 B for f64

// Workspace of the residual pipeline for an (m, n) array: pass-1 planes
// (reused by both directions) and the face planes of x and y.
struct ResidualLayout {
  int64_t m, n, P1, FX, FY;
  int nf;
  size_t es;
  size_t off_pl, off_pr, off_fx, off_fy, total;
  ResidualLayout(int64_t m_, int64_t n_, bool force_hlle, size_t es_) : m(m_), n(n_), es(es_) {
    P1 = align_elems(std::max((m - 5) * n, m * (n - 5)));
    FX = align_elems(std::max<int64_t>((m - 5) * (n - 6), 0));
    FY = align_elems(std::max<int64_t>((m - 6) * (n - 5), 0));
    nf = force_hlle ? 4 : 9;
    off_pl = 0;
    off_pr = off_pl + align_up(4 * P1 * es, 256);
    off_fx = off_pr + align_up(4 * P1 * es, 256);
    off_fy = off_fx + align_up(nf * FX * es, 256);
    total = off_fy + align_up(nf * FY * es, 256);
  }
};

inline void* at(void* base, size_t off) { return static_cast<char*>(base) + off; }

// One residual evaluation: u -> F_x, F_y -> L (dense out) or an RK stage.
struct TimingHook {
  void* solver = nullptr;
  cudaError_t (*mark)(void*, int, bool) = nullptr;
  cudaError_t operator()(int cls, bool start) const { return mark ? mark(solver, cls, start) : cudaSuccess; }
};
enum { HC_PASS1_X = 2, HC_PASS2_X, HC_BLEND, HC_PASS1_Y, HC_PASS2_Y, HC_RESIDUAL };

template <class T, bool FAST>
cudaError_t residual_pipeline(HostView u, int64_t m, int64_t n, const ResidualLayout& Lo, void* ws, double gamma,
                              double dx, bool force_hlle, double jp_lo, double jp_hi, bool cons, int stage, void* out,
                              HostPlanes Qn, HostPlanes Qs, HostPlanes Qo, const StepCtl* ctl, cudaStream_t st,
                              TimingHook tm = TimingHook(), double weps = 1e-12) {
  using Lx = Launch<T, FAST>;
  const int kind = force_hlle ? 1 : 2;
  T* fx = static_cast<T*>(at(ws, Lo.off_fx));
  T* fy = static_cast<T*>(at(ws, Lo.off_fy));
  cudaError_t e;
  // x sweep
  HostPlanes PL{at(ws, Lo.off_pl), Lo.P1, n}, PR{at(ws, Lo.off_pr), Lo.P1, n};
#define WENO_TIMED(cls, call)                              \
  do {                                                     \
    if ((e = tm(cls, true)) != cudaSuccess) return e;      \
    if ((e = (call)) != cudaSuccess) return e;             \
    if ((e = tm(cls, false)) != cudaSuccess) return e;     \
  } while (0)
  WENO_TIMED(HC_PASS1_X, Lx::pass1(u, m - 5, n, gamma, false, !cons, PL, PR, weps, st));
  WENO_TIMED(HC_PASS2_X, Lx::pass2(PL, PR, m - 5, n - 6, gamma, false, kind, fx, fx + 4 * Lo.FX, fx + 8 * Lo.FX,
                                   nullptr, Lo.FX, n - 6, weps, st));
  if (!force_hlle) {
    HostPlanes C{fx, Lo.FX, n - 6}, E{fx + 4 * Lo.FX, Lo.FX, n - 6}, P{fx + 8 * Lo.FX, Lo.FX, n - 6};
    WENO_TIMED(HC_BLEND, Lx::blend(C, E, P, m - 5, n - 6, jp_lo, jp_hi, nullptr, st));
  }
  // y sweep
  PL.ld = n - 5;
  PR.ld = n - 5;
  WENO_TIMED(HC_PASS1_Y, Lx::pass1(u, m, n - 5, gamma, true, !cons, PL, PR, weps, st));
  WENO_TIMED(HC_PASS2_Y, Lx::pass2(PL, PR, m - 6, n - 5, gamma, true, kind, fy, fy + 4 * Lo.FY, fy + 8 * Lo.FY,
                                   nullptr, Lo.FY, n - 5, weps, st));
  if (!force_hlle) {
    HostPlanes C{fy, Lo.FY, n - 5}, E{fy + 4 * Lo.FY, Lo.FY, n - 5}, P{fy + 8 * Lo.FY, Lo.FY, n - 5};
    WENO_TIMED(HC_BLEND, Lx::blend(C, E, P, m - 6, n - 5, jp_lo, jp_hi, nullptr, st));
  }
  HostPlanes Fx{fx, Lo.FX, n - 6}, Fy{fy, Lo.FY, n - 5};
  WENO_TIMED(HC_RESIDUAL, Lx::residual(Fx, Fy, m - 6, n - 6, dx, stage, out, Qn, Qs, Qo, ctl, st));
#undef WENO_TIMED
  return cudaSuccess;
}

cudaError_t residual_dispatch(int mode, HostView u, int64_t m, int64_t n, const ResidualLayout& Lo, void* ws,
                              double gamma, double dx, bool force_hlle, double jp_lo, double jp_hi, bool cons,
                              void* out, cudaStream_t st) {
  HostPlanes none{nullptr, 0, 0};
  if (mode == WENO_FAST)
    return residual_pipeline<double, true>(u, m, n, Lo, ws, gamma, dx, force_hlle, jp_lo, jp_hi, cons, 0, out, none,
                                           none, none, nullptr, st);
  return residual_pipeline<double, false>(u, m, n, Lo, ws, gamma, dx, force_hlle, jp_lo, jp_hi, cons, 0, out, none,
                                          none, none, nullptr, st);
}

bool debug_nan_fill() {
  const char* v = std::getenv("WENO_DEBUG_NAN_FILL");
  return v && v[0] && v[0] != '0';
}

int check_mode(int mode) {
  if (mode != WENO_EXACT && mode != WENO_FAST) return fail(WENO_ERR_ARG, "mode must be WENO_EXACT or WENO_FAST");
  return WENO_OK;
}

int check_array(const void* p, int64_t m, int64_t n, int64_t c, const char* what) {
  if (m < 0 || n < 0) return fail(WENO_ERR_SHAPE, "%s: negative extent", what);
  if (c < 4) return fail(WENO_ERR_SHAPE, "%s: needs at least 4 channels, got %lld", what, (long long)c);
  if (!p && m * n > 0) return fail(WENO_ERR_ARG, "%s: null pointer", what);
  return WENO_OK;
}

}  // namespace

namespace weno {
int set_last_error(int code, const char* msg) {
  g_err = msg;
  return code;
}
}  // namespace weno

extern "C" {

const char* weno_last_error(void) { return g_err.c_str(); }

int weno_abi_version(void) { return 2; }

int weno_flux(const double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double gamma,
              int ydir, int mode, double* out, void* stream) {
  int rc;
  if ((rc = check_array(q, m, n, c, "flux")) || (rc = check_mode(mode))) return rc;
  HostView v{q, s0, s1, s2};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  WENO_CK(mode == WENO_FAST ? Launch<double, true>::flux(v, m, n, gamma, ydir != 0, out, st)
                            : Launch<double, false>::flux(v, m, n, gamma, ydir != 0, out, st));
  return WENO_OK;
}

int weno_con2primi(const double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2,
                   double gamma, int mode, double* p, double* a, double* rho, double* u, double* v, double* h,
                   void* stream) {
  int rc;
  if ((rc = check_array(q, m, n, c, "con2primi")) || (rc = check_mode(mode))) return rc;
  HostView vw{q, s0, s1, s2};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  WENO_CK(mode == WENO_FAST ? Launch<double, true>::con2primi(vw, m, n, gamma, p, a, rho, u, v, h, st)
                            : Launch<double, false>::con2primi(vw, m, n, gamma, p, a, rho, u, v, h, st));
  return WENO_OK;
}

size_t weno_reconstruct_workspace(int64_t m, int64_t n, int ydir) {
  (void)ydir;
  if (m < 6 || n < 6) return 0;
  const int64_t P1 = align_elems(std::max((m - 5) * n, m * (n - 5)));
  return 2 * align_up(4 * P1 * sizeof(double), 256);
}

int weno_reconstruct(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2,
                     double gamma, int ydir, int cons, int mode, double* q_l, double* f_l, double* q_r, double* f_r,
                     void* ws, size_t ws_bytes, void* stream) {
  int rc;
  if ((rc = check_array(u, m, n, c, "reconstruct")) || (rc = check_mode(mode))) return rc;
  if (m < 6 || n < 6) return fail(WENO_ERR_SHAPE, "reconstruct: needs m, n >= 6 (6-cell stencil), got (%lld, %lld)",
                                  (long long)m, (long long)n);
  const size_t need = weno_reconstruct_workspace(m, n, ydir);
  if (!ws || ws_bytes < need) return fail(WENO_ERR_WORKSPACE, "reconstruct: workspace of %zu bytes needed", need);
  const int64_t P1 = align_elems(std::max((m - 5) * n, m * (n - 5)));
  const int64_t r1 = ydir ? m : m - 5, c1 = ydir ? n - 5 : n;
  const int64_t r2 = ydir ? m - 6 : m - 5, c2 = ydir ? n - 5 : n - 6;
  HostPlanes PL{ws, P1, c1}, PR{at(ws, align_up(4 * P1 * sizeof(double), 256)), P1, c1};
  HostView v{u, s0, s1, s2};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (mode == WENO_FAST) {
    WENO_CK((Launch<double, true>::pass1(v, r1, c1, gamma, ydir != 0, cons == 0, PL, PR, 1e-12, st)));
    WENO_CK((Launch<double, true>::pass2(PL, PR, r2, c2, gamma, ydir != 0, 0, q_l, f_l, q_r, f_r, 0, 0, 1e-12, st)));
  } else {
    WENO_CK((Launch<double, false>::pass1(v, r1, c1, gamma, ydir != 0, cons == 0, PL, PR, 1e-12, st)));
    WENO_CK((Launch<double, false>::pass2(PL, PR, r2, c2, gamma, ydir != 0, 0, q_l, f_l, q_r, f_r, 0, 0, 1e-12,
                                          st)));
  }
  return WENO_OK;
}

size_t weno_riemann_workspace(int64_t m, int64_t n, int kind) {
  if (kind != WENO_BLEND || m <= 0 || n <= 0) return 0;
  return align_up(9 * align_elems(m * n) * sizeof(double), 256);
}

int weno_riemann(const double* q_l, const double* f_l, const double* q_r, const double* f_r, int64_t m, int64_t n,
                 double gamma, int ydir, int kind, double jp_lo, double jp_hi, int mode, double* out, void* ws,
                 size_t ws_bytes, void* stream) {
  int rc;
  if ((rc = check_mode(mode))) return rc;
  if (kind < WENO_HLLC || kind > WENO_BLEND) return fail(WENO_ERR_ARG, "riemann: unknown solver kind %d", kind);
  if (m < 0 || n < 0) return fail(WENO_ERR_SHAPE, "riemann: negative extent");
  if (kind == WENO_BLEND && (m < 2 || n < 2))
    return fail(WENO_ERR_SHAPE, "riemann: the shock sensor needs a face array of at least 2 x 2, got (%lld, %lld)",
                (long long)m, (long long)n);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (kind != WENO_BLEND) {
    WENO_CK(mode == WENO_FAST
                ? Launch<double, true>::riemann(q_l, f_l, q_r, f_r, m, n, gamma, ydir != 0, kind, out, nullptr,
                                                nullptr, nullptr, 0, 0, st)
                : Launch<double, false>::riemann(q_l, f_l, q_r, f_r, m, n, gamma, ydir != 0, kind, out, nullptr,
                                                 nullptr, nullptr, 0, 0, st));
    return WENO_OK;
  }
  const size_t need = weno_riemann_workspace(m, n, kind);
  if (!ws || ws_bytes < need) return fail(WENO_ERR_WORKSPACE, "riemann: workspace of %zu bytes needed", need);
  const int64_t ps = align_elems(m * n);
  double* w = static_cast<double*>(ws);
  HostPlanes C{w, ps, n}, E{w + 4 * ps, ps, n}, P{w + 8 * ps, ps, n};
  if (mode == WENO_FAST) {
    WENO_CK((Launch<double, true>::riemann(q_l, f_l, q_r, f_r, m, n, gamma, ydir != 0, 2, nullptr, C.p, E.p, P.p, ps,
                                          n, st)));
    WENO_CK((Launch<double, true>::blend(C, E, P, m, n, jp_lo, jp_hi, out, st)));
  } else {
    WENO_CK((Launch<double, false>::riemann(q_l, f_l, q_r, f_r, m, n, gamma, ydir != 0, 2, nullptr, C.p, E.p, P.p,
                                           ps, n, st)));
    WENO_CK((Launch<double, false>::blend(C, E, P, m, n, jp_lo, jp_hi, out, st)));
  }
  return WENO_OK;
}

size_t weno_l_local_workspace(int64_t m, int64_t n, int force_hlle) {
  if (m < 6 || n < 6) return 0;
  return ResidualLayout(m, n, force_hlle != 0, sizeof(double)).total;
}

int weno_l_local(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double dx,
                 double gamma, int force_hlle, double jp_lo, double jp_hi, int cons, int mode, double* out, void* ws,
                 size_t ws_bytes, void* stream) {
  int rc;
  if ((rc = check_array(u, m, n, c, "l_local")) || (rc = check_mode(mode))) return rc;
  if (m < 6 || n < 6)
    return fail(WENO_ERR_SHAPE, "l_local: needs at least 6 x 6 cells (3 ghost cells per side), got (%lld, %lld)",
                (long long)m, (long long)n);
  if (!force_hlle && (m < 8 || n < 8))
    return fail(WENO_ERR_SHAPE, "l_local: the HLLC/HLLE blend's shock sensor needs at least 8 x 8 cells, got "
                "(%lld, %lld)", (long long)m, (long long)n);
  ResidualLayout Lo(m, n, force_hlle != 0, sizeof(double));
  if (!ws || ws_bytes < Lo.total) return fail(WENO_ERR_WORKSPACE, "l_local: workspace of %zu bytes needed", Lo.total);
  HostView v{u, s0, s1, s2};
  WENO_CK(residual_dispatch(mode, v, m, n, Lo, ws, gamma, dx, force_hlle != 0, jp_lo, jp_hi, cons != 0, out,
                            static_cast<cudaStream_t>(stream)));
  return WENO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Host-memory residual (one cached buffer set per device, serialised).
// ---------------------------------------------------------------------------
namespace {

struct HostCache {
  void* d_in = nullptr;
  size_t in_bytes = 0;
  void* d_out = nullptr;
  size_t out_bytes = 0;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  cudaStream_t st = nullptr;
  unsigned long long ctx = 0;  // context that owns the buffers and the stream
};
std::mutex g_host_mu;
std::map<int, HostCache> g_host_cache;

cudaError_t grow(void** p, size_t* have, size_t need) {
  if (*have >= need) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  cudaError_t e = cudaMalloc(p, std::max<size_t>(need, 256));
  if (e == cudaSuccess) *have = need;
  return e;
}

}  // namespace

extern "C" int weno_l_local_host(const double* u, int64_t m, int64_t n, int64_t c, double dx, double gamma,
                                 int force_hlle, double jp_lo, double jp_hi, int cons, int mode, double* out) {
  int rc;
  if ((rc = check_array(u, m, n, c, "l_local_host")) || (rc = check_mode(mode))) return rc;
  if (m < 6 || n < 6) return fail(WENO_ERR_SHAPE, "l_local_host: needs at least 6 x 6 cells, got (%lld, %lld)",
                                  (long long)m, (long long)n);
  if (!force_hlle && (m < 8 || n < 8))
    return fail(WENO_ERR_SHAPE, "l_local_host: the shock sensor needs at least 8 x 8 cells");
  int dev = 0;
  WENO_CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_host_mu);
  HostCache& hc = g_host_cache[dev];
  // buffers of a context that has since been destroyed (cudaDeviceReset) are
  // dropped, not freed: they went with it
  const unsigned long long ctx = weno::current_context_id();
  if (hc.st && ctx != 0 && hc.ctx != 0 && ctx != hc.ctx) hc = HostCache();
  if (!hc.st) {
    WENO_CK(cudaStreamCreateWithFlags(&hc.st, cudaStreamNonBlocking));
    hc.ctx = weno::current_context_id();
  }
  const size_t in_bytes = (size_t)(m * n * c) * sizeof(double);
  const size_t out_bytes = (size_t)((m - 6) * (n - 6) * 4) * sizeof(double);
  ResidualLayout Lo(m, n, force_hlle != 0, sizeof(double));
  WENO_CK(grow(&hc.d_in, &hc.in_bytes, in_bytes));
  WENO_CK(grow(&hc.d_out, &hc.out_bytes, out_bytes));
  WENO_CK(grow(&hc.ws, &hc.ws_bytes, Lo.total));
  WENO_CK(cudaMemcpyAsync(hc.d_in, u, in_bytes, cudaMemcpyHostToDevice, hc.st));
  HostView v{hc.d_in, n * c, c, 1};
  WENO_CK(residual_dispatch(mode, v, m, n, Lo, hc.ws, gamma, dx, force_hlle != 0, jp_lo, jp_hi, cons != 0, hc.d_out,
                            hc.st));
  if (out_bytes) WENO_CK(cudaMemcpyAsync(out, hc.d_out, out_bytes, cudaMemcpyDeviceToHost, hc.st));
  WENO_CK(cudaStreamSynchronize(hc.st));
  return WENO_OK;
}

// ---------------------------------------------------------------------------
// Device-resident solver
// ---------------------------------------------------------------------------
struct weno_solver {
  int device = 0;
  cudaStream_t stream = nullptr;
  int prec = 64, mode = WENO_EXACT;
  bool cons = false, force_hlle = true;
  double jp_lo = 0, jp_hi = 0, cfl = 0.5, dx = 1, gamma = 1.4, weps = 1e-12;
  int bc_kind = WENO_BC_TRANSMISSIVE;
  int64_t bound = 0;
  double post8[8] = {0};
  int64_t nx = 0, ny = 0, M = 0, N = 0, PS = 0;
  size_t es = 8;
  void* q = nullptr;   // current state, 4 planes
  void* q1 = nullptr;  // stage-1 state
  void* q2 = nullptr;  // stage-2 state
  void* ws = nullptr;
  ResidualLayout* layout = nullptr;
  StepCtl* ctl = nullptr;
  StepCtl* ctl_host = nullptr;  // pinned
  double* staging = nullptr;    // (M, N, 8) doubles for the host and export paths
  cudaGraphExec_t graph = nullptr;
  int sm_count = 152;
  int launches = 0;
  bool own_stream = false;
  // Per-kernel-class CUDA-event timing (non-graph runs with timing enabled).
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, size_t>> ev_marks;  // (class, index of the start event)
};

namespace {

HostPlanes state_planes(weno_solver* s, void* base) { return HostPlanes{base, s->PS, s->N}; }

// Kernel classes of the timing report.
enum { TC_CFL = 0, TC_BC, TC_PASS1_X, TC_PASS2_X, TC_BLEND, TC_PASS1_Y, TC_PASS2_Y, TC_RESIDUAL, TC_COUNT };

cudaError_t mark(weno_solver* s, int cls, bool start) {
  if (!s || !s->timing) return cudaSuccess;
  if (s->ev_used == s->ev_pool.size()) {
    cudaEvent_t e;
    cudaError_t err = cudaEventCreate(&e);
    if (err) return err;
    s->ev_pool.push_back(e);
  }
  const size_t idx = s->ev_used++;
  if (start) s->ev_marks.push_back({cls, idx});
  return cudaEventRecord(s->ev_pool[idx], s->stream);
}
HostView state_view(weno_solver* s, void* base) { return HostView{base, s->N, 1, s->PS}; }

template <class T, bool FAST>
cudaError_t bc_state(weno_solver* s, void* base) {
  if (s->bc_kind == WENO_BC_DMR)
    return Launch<T, FAST>::bc_dmr(state_view(s, base), 4, s->nx, s->ny, s->bound, s->post8, s->ctl, s->stream);
  return Launch<T, FAST>::bc_transmissive(state_view(s, base), 4, s->M, s->N, s->ctl, s->stream);
}

template <class T, bool FAST>
cudaError_t enqueue_step_t(weno_solver* s, int* launches) {
  cudaError_t e;
  int nl = 0;
  const cudaStream_t st = s->stream;
  HostPlanes Q = state_planes(s, s->q), Q1 = state_planes(s, s->q1), Q2 = state_planes(s, s->q2);
  TimingHook tm;
  if (s->timing) {
    tm.solver = s;
    tm.mark = [](void* p, int cls, bool start) { return mark(static_cast<weno_solver*>(p), cls, start); };
  }
  if ((e = tm(TC_CFL, true))) return e;
  if ((e = Launch<T, FAST>::cfl_max(state_view(s, s->q), false, s->nx, s->ny, s->gamma, s->ctl, s->sm_count, st)))
    return e;
  if ((e = launch_dt(s->ctl, st))) return e;
  if ((e = tm(TC_CFL, false))) return e;
  nl += 2;
  if (s->bc_kind == WENO_BC_TRANSMISSIVE) {
    if ((e = tm(TC_BC, true))) return e;
    if ((e = bc_state<T, FAST>(s, s->q))) return e;
    if ((e = tm(TC_BC, false))) return e;
    nl += 1;
  }
  const int per_residual = s->force_hlle ? 5 : 7;
  struct StageIO {
    void* in;
    HostPlanes qs, qo;
  } stages[3] = {{s->q, Q, Q1}, {s->q1, Q1, Q2}, {s->q2, Q2, Q}};
  static const char* const kStageName[3] = {"weno RK3 stage 1", "weno RK3 stage 2", "weno RK3 stage 3"};
  for (int k = 0; k < 3; ++k) {
    // host-side NVTX range around the stage's launches (visible to profilers when
    // the step is enqueued directly; a captured graph carries no ranges)
    nvtxRangePushA(kStageName[k]);
    e = residual_pipeline<T, FAST>(state_view(s, stages[k].in), s->M, s->N, *s->layout, s->ws, s->gamma, s->dx,
                                   s->force_hlle, s->jp_lo, s->jp_hi, s->cons, k + 1, nullptr, Q, stages[k].qs,
                                   stages[k].qo, s->ctl, st, tm, s->weps);
    if (!e && !(e = tm(TC_BC, true)) && !(e = bc_state<T, FAST>(s, stages[k].qo.p))) e = tm(TC_BC, false);
    nvtxRangePop();
    if (e) return e;
    nl += per_residual + 1;
  }
  if ((e = launch_step_end(s->ctl, st))) return e;
  nl += 1;
  if (launches) *launches = nl;
  return cudaSuccess;
}

cudaError_t enqueue_step(weno_solver* s, int* launches) {
  if (s->prec == 32) return enqueue_step_t<float, true>(s, launches);
  if (s->prec == 48) return enqueue_step_t<df64, true>(s, launches);
  if (s->mode == WENO_FAST) return enqueue_step_t<double, true>(s, launches);
  return enqueue_step_t<double, false>(s, launches);
}

void solver_free(weno_solver* s) {
  if (!s) return;
  for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  cudaFree(s->q);
  cudaFree(s->q1);
  cudaFree(s->q2);
  cudaFree(s->ws);
  cudaFree(s->ctl);
  cudaFree(s->staging);
  if (s->ctl_host) cudaFreeHost(s->ctl_host);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s->layout;
  delete s;
}

}  // namespace

extern "C" {

int weno_solver_create(weno_solver** out, int64_t nx, int64_t ny, double dx, double gamma, int precision, int mode,
                       int cons, int force_hlle, double jp_lo, double jp_hi, double cfl, double weno_eps, int bc_kind,
                       int64_t bound, const double* post8, void* stream) {
  if (!out) return fail(WENO_ERR_ARG, "solver_create: null handle pointer");
  *out = nullptr;
  if (nx < 3 || ny < 3) return fail(WENO_ERR_SHAPE, "solver_create: nx, ny >= 3 required, got (%lld, %lld)",
                                    (long long)nx, (long long)ny);
  if (!force_hlle && (nx < 2 || ny < 2)) return fail(WENO_ERR_SHAPE, "solver_create: grid too small for the sensor");
  if (precision != 64 && precision != 32 && precision != 48)
    return fail(WENO_ERR_ARG, "solver_create: precision must be 64, 48 (double-float) or 32");
  int rc;
  if ((rc = check_mode(mode))) return rc;
  if (bc_kind != WENO_BC_TRANSMISSIVE && bc_kind != WENO_BC_DMR)
    return fail(WENO_ERR_ARG, "solver_create: unknown boundary kind %d", bc_kind);
  if (bc_kind == WENO_BC_DMR && !post8) return fail(WENO_ERR_ARG, "solver_create: DMR boundary needs post8");
  weno_solver* s = new weno_solver();
  s->prec = precision;
  s->mode = precision != 64 ? WENO_FAST : mode;
  s->cons = cons != 0;
  s->force_hlle = force_hlle != 0;
  s->jp_lo = jp_lo;
  s->jp_hi = jp_hi;
  s->cfl = cfl;
  s->weps = weno_eps > 0.0 ? weno_eps : 1e-12;
  s->dx = dx;
  s->gamma = gamma;
  s->bc_kind = bc_kind;
  s->bound = bound;
  if (post8) std::memcpy(s->post8, post8, sizeof(s->post8));
  s->nx = nx;
  s->ny = ny;
  s->M = nx + 6;
  s->N = ny + 6;
  s->es = precision == 32 ? 4 : 8;
  s->PS = align_elems(s->M * s->N);
  s->stream = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  auto bail = [&](cudaError_t err, const char* where) {
    solver_free(s);
    return cuda_fail(err, where);
  };
  // Graph capture needs a stream other than the legacy default stream.
  if (!s->stream) {
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking))) return bail(e, "cudaStreamCreate");
    s->own_stream = true;
  }
  if ((e = cudaGetDevice(&s->device))) return bail(e, "cudaGetDevice");
  if ((e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device)))
    return bail(e, "cudaDeviceGetAttribute");
  const size_t state_bytes = (size_t)(4 * s->PS) * s->es;
  s->layout = new ResidualLayout(s->M, s->N, s->force_hlle, s->es);
  if ((e = cudaMalloc(&s->q, state_bytes))) return bail(e, "cudaMalloc(state)");
  if ((e = cudaMalloc(&s->q1, state_bytes))) return bail(e, "cudaMalloc(stage 1)");
  if ((e = cudaMalloc(&s->q2, state_bytes))) return bail(e, "cudaMalloc(stage 2)");
  if ((e = cudaMalloc(&s->ws, s->layout->total))) return bail(e, "cudaMalloc(workspace)");
  if ((e = cudaMalloc(&s->ctl, sizeof(StepCtl)))) return bail(e, "cudaMalloc(control)");
  if ((e = cudaMallocHost(&s->ctl_host, sizeof(StepCtl)))) return bail(e, "cudaMallocHost(control)");
  std::memset(s->ctl_host, 0, sizeof(StepCtl));
  s->ctl_host->cfl_dx = cfl * dx;
  s->ctl_host->t_final = -1.0;
  if ((e = cudaMemcpyAsync(s->ctl, s->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, s->stream)))
    return bail(e, "cudaMemcpyAsync(control)");
  // WENO_DEBUG_NAN_FILL=1 fills the state, stage and workspace buffers with a
  // NaN bit pattern instead of zeros, so that any read of data the step did not
  // write (a missed ghost cell, a stale stage) shows up as NaN in the results.
  const int fill = debug_nan_fill() ? 0xFF : 0;
  if ((e = cudaMemsetAsync(s->q, fill, state_bytes, s->stream))) return bail(e, "cudaMemsetAsync");
  if ((e = cudaMemsetAsync(s->q1, fill, state_bytes, s->stream))) return bail(e, "cudaMemsetAsync");
  if ((e = cudaMemsetAsync(s->q2, fill, state_bytes, s->stream))) return bail(e, "cudaMemsetAsync");
  if (fill && (e = cudaMemsetAsync(s->ws, fill, s->layout->total, s->stream))) return bail(e, "cudaMemsetAsync");
  if ((e = cudaStreamSynchronize(s->stream))) return bail(e, "cudaStreamSynchronize");
  *out = s;
  return WENO_OK;
}

int weno_solver_destroy(weno_solver* s) {
  if (!s) return WENO_OK;
  cudaStreamSynchronize(s->stream);
  solver_free(s);
  return WENO_OK;
}

int weno_solver_set_state(weno_solver* s, const double* q, int64_t c, int64_t s0, int64_t s1, int64_t s2) {
  if (!s || !q) return fail(WENO_ERR_ARG, "solver_set_state: null argument");
  if (c < 4) return fail(WENO_ERR_SHAPE, "solver_set_state: needs at least 4 channels");
  HostView v{q, s0, s1, s2};
  HostPlanes Q = state_planes(s, s->q);
  if (s->prec == 32) WENO_CK((Launch<float, true>::import_planes(v, s->M, s->N, Q, s->stream)));
  else if (s->prec == 48) WENO_CK((Launch<df64, true>::import_planes(v, s->M, s->N, Q, s->stream)));
  else WENO_CK((Launch<double, false>::import_planes(v, s->M, s->N, Q, s->stream)));
  // Fresh clock; with primitive channels present the first dt comes from them.
  std::memset(s->ctl_host, 0, sizeof(StepCtl));
  s->ctl_host->cfl_dx = s->cfl * s->dx;
  s->ctl_host->t_final = -1.0;
  s->ctl_host->active = 1;
  WENO_CK(cudaMemcpyAsync(s->ctl, s->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, s->stream));
  if (c >= 8) {
    WENO_CK((Launch<double, false>::cfl_max(v, true, s->nx, s->ny, s->gamma, s->ctl, s->sm_count, s->stream)));
    const int one = 1;
    WENO_CK(cudaMemcpyAsync(&s->ctl->cmax_preset, &one, sizeof(int), cudaMemcpyHostToDevice, s->stream));
  }
  WENO_CK(cudaStreamSynchronize(s->stream));
  return WENO_OK;
}

int weno_solver_set_state_host(weno_solver* s, const double* q, int64_t c) {
  if (!s || !q) return fail(WENO_ERR_ARG, "solver_set_state_host: null argument");
  if (c < 4 || c > 8) return fail(WENO_ERR_SHAPE, "solver_set_state_host: 4..8 channels supported");
  if (!s->staging) WENO_CK(cudaMalloc(&s->staging, (size_t)(s->M * s->N * 8) * sizeof(double)));
  WENO_CK(cudaMemcpyAsync(s->staging, q, (size_t)(s->M * s->N * c) * sizeof(double), cudaMemcpyHostToDevice,
                          s->stream));
  return weno_solver_set_state(s, s->staging, c, s->N * c, c, 1);
}

int weno_solver_run(weno_solver* s, int64_t nsteps, double t_final, int use_graph) {
  if (!s) return fail(WENO_ERR_ARG, "solver_run: null handle");
  if (nsteps < 0) return fail(WENO_ERR_ARG, "solver_run: negative step count");
  WENO_CK(launch_run_begin(s->ctl, t_final, (long long)nsteps, s->stream));
  if (use_graph && !s->graph && nsteps > 0) {
    cudaGraph_t g = nullptr;
    WENO_CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_step(s, &s->launches);
    cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
    if (e) return cuda_fail(e, "enqueue_step (capture)");
    if (e2) return cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e) return cuda_fail(e, "cudaGraphInstantiate");
  }
  for (int64_t k = 0; k < nsteps; ++k) {
    if (use_graph) WENO_CK(cudaGraphLaunch(s->graph, s->stream));
    else {
      cudaError_t e = enqueue_step(s, &s->launches);
      if (e) return cuda_fail(e, "enqueue_step");
    }
  }
  return WENO_OK;
}

int weno_solver_get_state(weno_solver* s, double* out) {
  if (!s || !out) return fail(WENO_ERR_ARG, "solver_get_state: null argument");
  HostPlanes Q = state_planes(s, s->q);
  if (s->prec == 32) WENO_CK((Launch<float, true>::export_aos8(Q, s->M, s->N, s->gamma, out, s->stream)));
  else if (s->prec == 48) WENO_CK((Launch<df64, true>::export_aos8(Q, s->M, s->N, s->gamma, out, s->stream)));
  else if (s->mode == WENO_FAST) WENO_CK((Launch<double, true>::export_aos8(Q, s->M, s->N, s->gamma, out, s->stream)));
  else WENO_CK((Launch<double, false>::export_aos8(Q, s->M, s->N, s->gamma, out, s->stream)));
  if (s->bc_kind == WENO_BC_DMR) {
    HostView v{out, s->N * 8, 8, 1};
    WENO_CK((Launch<double, false>::bc_dmr(v, 8, s->nx, s->ny, s->bound, s->post8, nullptr, s->stream)));
  }
  return WENO_OK;
}

int weno_solver_get_state_host(weno_solver* s, double* out) {
  if (!s || !out) return fail(WENO_ERR_ARG, "solver_get_state_host: null argument");
  if (!s->staging) WENO_CK(cudaMalloc(&s->staging, (size_t)(s->M * s->N * 8) * sizeof(double)));
  int rc = weno_solver_get_state(s, s->staging);
  if (rc) return rc;
  WENO_CK(cudaMemcpyAsync(out, s->staging, (size_t)(s->M * s->N * 8) * sizeof(double), cudaMemcpyDeviceToHost,
                          s->stream));
  WENO_CK(cudaStreamSynchronize(s->stream));
  return WENO_OK;
}

int weno_solver_info(weno_solver* s, double* t, int64_t* steps, int* status) {
  if (!s) return fail(WENO_ERR_ARG, "solver_info: null handle");
  WENO_CK(cudaMemcpyAsync(s->ctl_host, s->ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, s->stream));
  WENO_CK(cudaStreamSynchronize(s->stream));
  if (t) *t = s->ctl_host->t;
  if (steps) *steps = s->ctl_host->steps;
  if (status) *status = s->ctl_host->status;
  return WENO_OK;
}

int weno_solver_totals(weno_solver* s, double* out4) {
  if (!s || !out4) return fail(WENO_ERR_ARG, "solver_totals: null argument");
  double* d = nullptr;
  if (!s->staging) WENO_CK(cudaMalloc(&s->staging, (size_t)(s->M * s->N * 8) * sizeof(double)));
  d = s->staging;  // the first four doubles of the staging buffer
  const HostView v = state_view(s, s->q);
  if (s->prec == 32) WENO_CK((Launch<float, true>::totals(v, s->nx, s->ny, d, s->sm_count, s->stream)));
  else if (s->prec == 48) WENO_CK((Launch<df64, true>::totals(v, s->nx, s->ny, d, s->sm_count, s->stream)));
  else WENO_CK((Launch<double, false>::totals(v, s->nx, s->ny, d, s->sm_count, s->stream)));
  WENO_CK(cudaMemcpyAsync(out4, d, 4 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  WENO_CK(cudaStreamSynchronize(s->stream));
  return WENO_OK;
}

int weno_solver_enable_timing(weno_solver* s, int on) {
  if (!s) return fail(WENO_ERR_ARG, "solver_enable_timing: null handle");
  WENO_CK(cudaStreamSynchronize(s->stream));
  s->timing = on != 0;
  s->ev_used = 0;
  s->ev_marks.clear();
  return WENO_OK;
}

int weno_solver_timing_report(weno_solver* s, double* ms, int64_t* launches, int nclasses) {
  if (!s || !ms || !launches) return fail(WENO_ERR_ARG, "solver_timing_report: null argument");
  WENO_CK(cudaStreamSynchronize(s->stream));
  for (int c = 0; c < nclasses; ++c) {
    ms[c] = 0.0;
    launches[c] = 0;
  }
  for (const auto& mk : s->ev_marks) {
    float t = 0.f;
    WENO_CK(cudaEventElapsedTime(&t, s->ev_pool[mk.second], s->ev_pool[mk.second + 1]));
    if (mk.first < nclasses) {
      ms[mk.first] += t;
      launches[mk.first] += 1;
    }
  }
  return WENO_OK;
}

int weno_solver_launches_per_step(weno_solver* s) {
  if (!s) return 0;
  if (!s->launches) {
    // Count without enqueuing: the structure is fixed by the configuration.
    const int per_residual = s->force_hlle ? 5 : 7;
    s->launches = 2 + (s->bc_kind == WENO_BC_TRANSMISSIVE ? 1 : 0) + 3 * (per_residual + 1) + 1;
  }
  return s->launches;
}

}  // extern "C"
