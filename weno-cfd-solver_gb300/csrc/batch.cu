// C ABI of the batched solver (include/weno_gb300.h, weno_batch_*).
//
// A batch owns one packed pool per RK buffer (state, stage 1, stage 2) of a
// fixed capacity, carved from one allocation, a table of solve descriptors,
// per-solve clocks and TMA tensor maps, and a tile list.  Solves join
// (weno_batch_add) and leave (weno_batch_remove) between runs; the pool is
// first-fit allocated on the host.  The device-side tables
// keep their addresses for the batch's lifetime, so a captured step graph stays
// valid while membership changes; the tile count is the only launch argument
// that changes, and a change re-captures the graph.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

#define WENO_TU_NS batch_host
#include "../../include/weno_gb300.h"
#include "batch_api.h"
#include "batch_kernels.cuh"
#include "errors.h"
#include "launch_api.h"

using namespace weno;

namespace {

int bfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return set_last_error(code, buf);
}

#define WB_CK(...)                                                                      \
  do {                                                                                  \
    cudaError_t e_ = (__VA_ARGS__);                                                     \
    if (e_ != cudaSuccess) return bfail(WENO_ERR_CUDA, "%s: %s", #__VA_ARGS__, cudaGetErrorString(e_)); \
  } while (0)

inline long long align64(long long x) { return (x + 63) / 64 * 64; }

// cuTensorMapEncodeTiled, fetched once through the runtime (no link against libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

}  // namespace

struct weno_batch {
  int prec = 32, mode = WENO_FAST;
  bool chr = false, blend = false;
  double gamma = 1.4, jp_lo = 0.2, jp_hi = 1.0, cfl = 0.5, weps = 1e-12;
  int cfg = 1;
  int max_solves = 0;
  long long capacity = 0;  // elements per pool
  size_t es = 4;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sm_count = 152;
  int occ = 1;  // resident CTAs per SM of the stage kernel
  void* pool_base = nullptr;  // the three pools, `capacity` elements apart
  void* pool[3] = {nullptr, nullptr, nullptr};
  CUtensorMap* d_tmaps = nullptr;  // one per slot: (column, row, plane, pool) of that solve
  std::vector<CUtensorMap> h_tmaps;
  SolveDesc* d_solves = nullptr;
  SolveCtl* d_ctl = nullptr;
  std::vector<SolveDesc> h_solves;
  std::vector<bool> used;
  SolveCtl* h_ctl = nullptr;  // pinned
  // tiles
  int4* d_tiles = nullptr;
  int tile_cap = 0;
  int ntiles = 0;
  bool tiles_dirty = true;
  int4* h_tiles = nullptr;  // pinned, tile_cap entries
  int4* d_add_tiles = nullptr;
  int add_tile_cap = 0;
  // free list: offset -> length (elements)
  std::map<long long, long long> free_list;
  // staged configuration: the face workspace pool (elements) and its free list
  void* ws_base = nullptr;
  long long ws_capacity = 0;
  std::map<long long, long long> ws_free;
  std::vector<long long> ws_off, ws_len;  // per slot
  cudaGraphExec_t graph = nullptr;
  int graph_ntiles = -1;
  // test hook (weno_batch_debug_skip_copy): tile whose staging copy is not issued,
  // the bounded wait of every staging copy, and a fixed stage grid (0: occupancy)
  int skip_tile = -1;
  unsigned long long wait_ns = 1000000000ull;  // 1 s
  int fixed_grid = 0;
};

namespace {

template <class T, bool FAST>
cudaError_t enqueue_batch_step(weno_batch* b) {
  using BL = BatchLaunch<T, FAST>;
  // The fused kernel keeps a persistent grid (its tiles stage through shared
  // memory sized for the resident CTAs); the staged kernels launch one CTA per
  // tile, so their CTAs are short and the block scheduler can interleave the
  // CTAs of other streams (a higher-priority FP32 batch) between them.
  const int grid = b->fixed_grid > 0 ? b->fixed_grid
                   : (b->cfg == kStagedConfig ? b->ntiles : std::min(b->ntiles, b->sm_count * b->occ));
  cudaError_t e;
  if ((e = BL::clock(b->d_ctl, b->max_solves, 0, b->stream))) return e;
  if (b->cfg == kStagedConfig) {
    for (int s = 1; s <= 3; ++s) {
      void* qo = b->pool[s == 1 ? 1 : (s == 2 ? 2 : 0)];
      if ((e = BL::staged(b->chr, b->blend, b->d_solves, b->d_ctl, b->d_tiles, b->ntiles, grid, b->pool[s - 1],
                          b->pool[0], qo, b->ws_base, s, b->gamma, b->jp_lo, b->jp_hi, b->weps, b->stream)))
        return e;
    }
    return BL::clock(b->d_ctl, b->max_solves, 1, b->stream);
  }
  for (int s = 1; s <= 3; ++s) {
    // stage s reads pool s-1 (q, q1, q2) through the tensor maps
    void* qo = b->pool[s == 1 ? 1 : (s == 2 ? 2 : 0)];
    if ((e = BL::stage(b->cfg, b->chr, b->blend, b->d_solves, b->d_ctl, b->d_tiles, b->ntiles, grid, b->d_tmaps,
                       b->pool[0], qo, s, b->gamma, b->jp_lo, b->jp_hi, b->weps, b->skip_tile, b->wait_ns,
                       b->stream)))
      return e;
  }
  return BL::clock(b->d_ctl, b->max_solves, 1, b->stream);
}

cudaError_t enqueue_step(weno_batch* b) {
  if (b->prec == 32) return enqueue_batch_step<float, true>(b);
  if (b->mode == WENO_FAST) return enqueue_batch_step<double, true>(b);
  return enqueue_batch_step<double, false>(b);
}

int tiles_of(const weno_batch* b, int slot, std::vector<int4>& out) {
  const SolveDesc& d = b->h_solves[slot];
  const int tx = kTileTX[b->cfg], ty = kTileTY[b->cfg];
  int n = 0;
  for (int i0 = 0; i0 < d.nx; i0 += tx)
    for (int j0 = 0; j0 < d.ny; j0 += ty) {
      out.push_back(make_int4(slot, i0, j0, 0));
      ++n;
    }
  return n;
}

int rebuild_tiles(weno_batch* b) {
  std::vector<int4> all;
  for (int s = 0; s < b->max_solves; ++s)
    if (b->used[s]) tiles_of(b, s, all);
  const int n = (int)all.size();
  if (n > b->tile_cap) {
    int cap = std::max(n, 2 * b->tile_cap);
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaFree(b->d_tiles);
    cudaFreeHost(b->h_tiles);
    b->d_tiles = nullptr;
    b->h_tiles = nullptr;
    WB_CK(cudaMalloc(&b->d_tiles, sizeof(int4) * cap));
    WB_CK(cudaMallocHost(&b->h_tiles, sizeof(int4) * cap));
    b->tile_cap = cap;
  }
  if (n) {
    // The previous upload may still be read by a queued copy: wait for the stream.
    WB_CK(cudaStreamSynchronize(b->stream));
    std::memcpy(b->h_tiles, all.data(), sizeof(int4) * n);
    WB_CK(cudaMemcpyAsync(b->d_tiles, b->h_tiles, sizeof(int4) * n, cudaMemcpyHostToDevice, b->stream));
  }
  b->ntiles = n;
  b->tiles_dirty = false;
  return WENO_OK;
}

long long fl_alloc(std::map<long long, long long>& fl, long long len) {
  len = align64(len);
  for (auto it = fl.begin(); it != fl.end(); ++it) {
    if (it->second >= len) {
      const long long off = it->first, rest = it->second - len;
      fl.erase(it);
      if (rest > 0) fl[off + len] = rest;
      return off;
    }
  }
  return -1;
}

void fl_free(std::map<long long, long long>& fl, long long off, long long len) {
  len = align64(len);
  auto it = fl.emplace(off, len).first;
  auto next = std::next(it);
  if (next != fl.end() && it->first + it->second == next->first) {
    it->second += next->second;
    fl.erase(next);
  }
  if (it != fl.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == it->first) {
      prev->second += it->second;
      fl.erase(it);
    }
  }
}

long long pool_alloc(weno_batch* b, long long len) { return fl_alloc(b->free_list, len); }
void pool_free(weno_batch* b, long long off, long long len) { fl_free(b->free_list, off, len); }

// Face workspace of one solve in the staged configuration (element counts; see
// k_staged_pass1): fills the layout fields of `d` with offsets relative to the
// solve's block and returns the block's length.
long long staged_layout(SolveDesc& d, int lq, int nf) {
  auto up = [lq](long long x) { return (x + lq - 1) / lq * lq; };
  const long long nx = d.nx, ny = d.ny;
  d.l_p1x = (int)up(ny + 4);
  d.l_p1y = (int)up(ny + 1);
  d.s_p1x = align64((nx + 1) * d.l_p1x);
  d.s_p1y = align64((nx + 4) * d.l_p1y);
  d.s_fx = align64((nx + 1) * d.ld);
  d.s_fy = align64(nx * d.l_p1y);
  d.w_p1x = 0;
  d.w_p1y = 8 * d.s_p1x;
  d.w_fx = d.w_p1y + 8 * d.s_p1y;
  d.w_fy = d.w_fx + nf * d.s_fx;
  return d.w_fy + nf * d.s_fy;
}

// Workspace elements reserved per pool cell in the staged configuration: the
// face arrays of a solve take about 16 + 2 NF values per cell, more for small
// grids (halo rows and columns, 64-element plane alignment).
constexpr double kStagedWsPerCellMargin = 1.25;
inline long long staged_ws_capacity(long long pool_cells, int max_solves, int nf) {
  return align64((long long)(kStagedWsPerCellMargin * (16 + 2 * nf) * (double)pool_cells) +
                 (long long)max_solves * (16 + 2 * nf) * 128);
}

// Installs a host-encoded tensor map (passed by value) at `dst` in global
// memory and releases it to the tensormap proxy; the stage kernel acquires it.
__global__ void k_install_tensormap(CUtensorMap* dst, const __grid_constant__ CUtensorMap src) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint4* s = reinterpret_cast<const uint4*>(&src);
  uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
  for (int k = 0; k < (int)(sizeof(CUtensorMap) / sizeof(uint4)); ++k) d[k] = s[k];
  tma::tensormap_release(dst);
}

// Import a padded (nx+6, ny+6, c) array into a solve's interior planes.
template <class T>
__global__ void k_import_interior(const double* q, long long s0, long long s1, long long s2, int nx, int ny, T* dst,
                                  long long ps, int ld) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ld) return;
  const double* c = q + (long long)(i + 3) * s0 + (long long)(j + 3) * s1;
#pragma unroll
  for (int k = 0; k < 4; ++k) dst[k * ps + (long long)i * ld + j] = j < ny ? (T)c[k * s2] : T(0);
}

// Export a solve as the driver's (nx+6, ny+6, 8) array: ghost cells from the
// boundary rule, then the primitive sync (utils.rs:9-35) on every cell.
template <class T>
__global__ void k_export_solve(const SolveDesc* solves, int slot, const T* pool, double gamma, double* out) {
  const SolveDesc d = solves[slot];
  const int J = blockIdx.x * blockDim.x + threadIdx.x;
  const int I = blockIdx.y * blockDim.y + threadIdx.y;
  const int M = d.nx + 6, N = d.ny + 6;
  if (I >= M || J >= N) return;
  const GhostSrc g = resolve_cell(d, I, J);
  double* o = out + ((long long)I * N + J) * 8;
  if (g.post) {
    // The inflow state carries its own primitive channels (unitest.py:215).
    for (int k = 0; k < 4; ++k) o[k] = (double)(T)d.post[k];
    for (int k = 4; k < 8; ++k) o[k] = d.post[k];
    return;
  }
  double q[4];
  {
    const long long o = d.off + (long long)g.i * d.ld + g.j;
    for (int k = 0; k < 4; ++k) q[k] = (double)pool[o + k * d.ps];
    if (g.flip2) q[2] = -q[2];
  }
  const double rho = fmax(q[0], 1e-12);
  const double u = q[1] / rho, v = q[2] / rho;
  const double p = fmax((gamma - 1.0) * (q[3] - 0.5 * rho * (u * u + v * v)), 1e-12);
  o[0] = q[0]; o[1] = q[1]; o[2] = q[2]; o[3] = q[3];
  o[4] = rho; o[5] = u; o[6] = v; o[7] = p;
}

void batch_free(weno_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->pool_base);
  cudaFree(b->ws_base);
  cudaFree(b->d_tmaps);
  cudaFree(b->d_solves);
  cudaFree(b->d_ctl);
  cudaFree(b->d_tiles);
  cudaFree(b->d_add_tiles);
  if (b->h_ctl) cudaFreeHost(b->h_ctl);
  if (b->h_tiles) cudaFreeHost(b->h_tiles);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // namespace

extern "C" {

int weno_batch_tile_config_count(void) { return kNumTileConfigs; }

int weno_batch_create(weno_batch** out, int64_t pool_cells, int max_solves, int precision, int mode, int cons,
                      int force_hlle, double gamma, double jp_lo, double jp_hi, double cfl, double weno_eps,
                      int tile_config, void* stream) {
  if (!out) return bfail(WENO_ERR_ARG, "batch_create: null handle pointer");
  *out = nullptr;
  if (pool_cells <= 0 || max_solves <= 0) return bfail(WENO_ERR_ARG, "batch_create: empty pool");
  if (precision != 32 && precision != 64) return bfail(WENO_ERR_ARG, "batch_create: precision must be 32 or 64");
  if (mode != WENO_EXACT && mode != WENO_FAST) return bfail(WENO_ERR_ARG, "batch_create: bad mode");
  if (tile_config < 0 || tile_config >= kNumTileConfigs)
    return bfail(WENO_ERR_ARG, "batch_create: tile_config must be in [0, %d)", kNumTileConfigs);
  weno_batch* b = new weno_batch();
  b->prec = precision;
  b->mode = precision == 32 ? WENO_FAST : mode;
  b->chr = cons == 0;
  b->blend = force_hlle == 0;
  b->gamma = gamma;
  b->jp_lo = jp_lo;
  b->jp_hi = jp_hi;
  b->cfl = cfl;
  b->weps = weno_eps > 0.0 ? weno_eps : 1e-12;
  b->cfg = tile_config;
  b->max_solves = max_solves;
  b->es = precision == 32 ? 4 : 8;
  b->capacity = align64(4 * pool_cells);
  b->stream = static_cast<cudaStream_t>(stream);
  auto bail = [&](cudaError_t e, const char* w) {
    batch_free(b);
    return bfail(WENO_ERR_CUDA, "%s: %s", w, cudaGetErrorString(e));
  };
  cudaError_t e;
  if (!b->stream) {
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking))) return bail(e, "cudaStreamCreate");
    b->own_stream = true;
  }
  int dev = 0;
  if ((e = cudaGetDevice(&dev))) return bail(e, "cudaGetDevice");
  if ((e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev))) return bail(e, "attr");
  if (b->cfg == kStagedConfig) {
    b->occ = 8;  // grid of the staged kernels: up to 8 CTAs of 256 threads per SM walk the tile list
  } else {
    const size_t smem = precision == 32 ? BatchLaunch<float, true>::smem_bytes(b->cfg, b->blend)
                        : (b->mode == WENO_FAST ? BatchLaunch<double, true>::smem_bytes(b->cfg, b->blend)
                                                : BatchLaunch<double, false>::smem_bytes(b->cfg, b->blend));
    if (!smem) {
      batch_free(b);
      return bfail(WENO_ERR_ARG, "batch_create: tile configuration %d does not fit in shared memory", tile_config);
    }
    b->occ = std::max(1, precision == 32 ? BatchLaunch<float, true>::ctas_per_sm(b->cfg, b->chr, b->blend)
                         : (b->mode == WENO_FAST ? BatchLaunch<double, true>::ctas_per_sm(b->cfg, b->chr, b->blend)
                                                 : BatchLaunch<double, false>::ctas_per_sm(b->cfg, b->chr, b->blend)));
  }
  if (!encode_tiled()) {
    batch_free(b);
    return bfail(WENO_ERR_CUDA, "batch_create: cuTensorMapEncodeTiled is not available from the driver");
  }
  if ((e = cudaMalloc(&b->pool_base, 3 * (size_t)b->capacity * b->es))) return bail(e, "cudaMalloc(pool)");
  {
    // WENO_DEBUG_NAN_FILL=1: pools start as a NaN bit pattern, so a tile load or
    // a store outside a solve's written cells shows up as NaN in its results.
    const char* v = std::getenv("WENO_DEBUG_NAN_FILL");
    if (v && v[0] && v[0] != '0' &&
        (e = cudaMemsetAsync(b->pool_base, 0xFF, 3 * (size_t)b->capacity * b->es, b->stream)))
      return bail(e, "cudaMemsetAsync(pool)");
  }
  for (int k = 0; k < 3; ++k) b->pool[k] = static_cast<char*>(b->pool_base) + (size_t)k * b->capacity * b->es;
  b->ws_off.assign(max_solves, -1);
  b->ws_len.assign(max_solves, 0);
  if (b->cfg == kStagedConfig) {
    b->ws_capacity = staged_ws_capacity(pool_cells, max_solves, b->blend ? 9 : 4);
    if ((e = cudaMalloc(&b->ws_base, (size_t)b->ws_capacity * b->es))) return bail(e, "cudaMalloc(workspace)");
    const char* v = std::getenv("WENO_DEBUG_NAN_FILL");
    if (v && v[0] && v[0] != '0' && (e = cudaMemsetAsync(b->ws_base, 0xFF, (size_t)b->ws_capacity * b->es, b->stream)))
      return bail(e, "cudaMemsetAsync(workspace)");
    b->ws_free[0] = b->ws_capacity;
  }
  if ((e = cudaMalloc(&b->d_tmaps, sizeof(CUtensorMap) * max_solves))) return bail(e, "cudaMalloc(tensor maps)");
  b->h_tmaps.assign(max_solves, CUtensorMap{});
  if ((e = cudaMalloc(&b->d_solves, sizeof(SolveDesc) * max_solves))) return bail(e, "cudaMalloc(solves)");
  if ((e = cudaMalloc(&b->d_ctl, sizeof(SolveCtl) * max_solves))) return bail(e, "cudaMalloc(ctl)");
  if ((e = cudaMallocHost(&b->h_ctl, sizeof(SolveCtl) * max_solves))) return bail(e, "cudaMallocHost(ctl)");
  std::memset(b->h_ctl, 0, sizeof(SolveCtl) * max_solves);
  if ((e = cudaMemcpyAsync(b->d_ctl, b->h_ctl, sizeof(SolveCtl) * max_solves, cudaMemcpyHostToDevice, b->stream)))
    return bail(e, "cudaMemcpy(ctl)");
  b->h_solves.assign(max_solves, SolveDesc{});
  b->used.assign(max_solves, false);
  b->free_list[0] = b->capacity;
  if ((e = cudaStreamSynchronize(b->stream))) return bail(e, "sync");
  *out = b;
  return WENO_OK;
}

int weno_batch_destroy(weno_batch* b) {
  if (!b) return WENO_OK;
  cudaStreamSynchronize(b->stream);
  batch_free(b);
  return WENO_OK;
}

int weno_batch_add(weno_batch* b, int64_t nx, int64_t ny, double dx, int bc_kind, int64_t bound, const double* post8,
                   double t_end, int64_t max_steps, double cfl, const double* q, int64_t c, int64_t s0, int64_t s1,
                   int64_t s2, int* slot_out) {
  if (!b || !q || !slot_out) return bfail(WENO_ERR_ARG, "batch_add: null argument");
  if (nx < 3 || ny < 3) return bfail(WENO_ERR_SHAPE, "batch_add: nx, ny >= 3 required");
  if (b->blend && (nx < 2 || ny < 2)) return bfail(WENO_ERR_SHAPE, "batch_add: grid too small for the sensor");
  if (c < 4) return bfail(WENO_ERR_SHAPE, "batch_add: needs at least 4 channels");
  if (bc_kind != WENO_BC_TRANSMISSIVE && bc_kind != WENO_BC_DMR) return bfail(WENO_ERR_ARG, "batch_add: bad bc");
  if (bc_kind == WENO_BC_DMR && !post8) return bfail(WENO_ERR_ARG, "batch_add: DMR boundary needs post8");
  int slot = -1;
  for (int s = 0; s < b->max_solves; ++s)
    if (!b->used[s]) {
      slot = s;
      break;
    }
  if (slot < 0) return bfail(WENO_ERR_WORKSPACE, "batch_add: all %d solve slots are in use", b->max_solves);
  const int lq = (int)(16 / b->es);  // row pitch quantum: 16 bytes
  const long long ld = (ny + lq - 1) / lq * lq;
  const long long ps = align64(nx * ld);
  const long long off = pool_alloc(b, 4 * ps);
  if (off < 0) return bfail(WENO_ERR_WORKSPACE, "batch_add: pool full (%lld cells requested)", (long long)(nx * ny));
  // Tensor map of this solve over all three pools: dims (column, row, plane, pool).
  {
    unsigned bc = 0, br = 0;
    if (b->prec == 32) BatchLaunch<float, true>::box(b->cfg, b->blend, &bc, &br);
    else BatchLaunch<double, true>::box(b->cfg, b->blend, &bc, &br);
    const cuuint64_t dims[4] = {(cuuint64_t)ny, (cuuint64_t)nx, 4, 3};
    const cuuint64_t strides[3] = {(cuuint64_t)(ld * b->es), (cuuint64_t)(ps * b->es),
                                   (cuuint64_t)(b->capacity * b->es)};
    const cuuint32_t box[4] = {bc, br, 4, 1};
    const cuuint32_t elem[4] = {1, 1, 1, 1};
    void* base = static_cast<char*>(b->pool_base) + (size_t)off * b->es;
    const CUresult r = encode_tiled()(&b->h_tmaps[slot],
                                      b->prec == 32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                                      4, base, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      pool_free(b, off, 4 * ps);
      return bfail(WENO_ERR_CUDA, "batch_add: cuTensorMapEncodeTiled failed (%d)", (int)r);
    }
  }
  SolveDesc d{};
  d.off = off;
  d.ps = ps;
  d.nx = (int)nx;
  d.ny = (int)ny;
  d.ld = (int)ld;
  d.bc = bc_kind;
  d.bound = (int)bound;
  d.dx = dx;
  if (post8)
    for (int k = 0; k < 8; ++k) d.post[k] = post8[k];
  if (b->cfg == kStagedConfig) {
    const long long len = staged_layout(d, lq, b->blend ? 9 : 4);
    const long long woff = fl_alloc(b->ws_free, len);
    if (woff < 0) {
      pool_free(b, off, 4 * ps);
      return bfail(WENO_ERR_WORKSPACE, "batch_add: face workspace full (%lld elements requested)", len);
    }
    d.w_p1x += woff;
    d.w_p1y += woff;
    d.w_fx += woff;
    d.w_fy += woff;
    b->ws_off[slot] = woff;
    b->ws_len[slot] = len;
  }
  b->h_solves[slot] = d;
  b->used[slot] = true;
  WB_CK(cudaMemcpyAsync(b->d_solves + slot, &b->h_solves[slot], sizeof(SolveDesc), cudaMemcpyHostToDevice, b->stream));
  k_install_tensormap<<<1, 32, 0, b->stream>>>(b->d_tmaps + slot, b->h_tmaps[slot]);
  WB_CK(cudaGetLastError());
  // interior state (the row padding is zeroed)
  const dim3 blk(32, 4);
  const dim3 grd((unsigned)((ld + 31) / 32), (unsigned)((nx + 3) / 4));
  if (b->prec == 32)
    k_import_interior<float><<<grd, blk, 0, b->stream>>>(q, s0, s1, s2, (int)nx, (int)ny,
                                                        static_cast<float*>(b->pool[0]) + off, ps, (int)ld);
  else
    k_import_interior<double><<<grd, blk, 0, b->stream>>>(q, s0, s1, s2, (int)nx, (int)ny,
                                                         static_cast<double*>(b->pool[0]) + off, ps, (int)ld);
  WB_CK(cudaGetLastError());
  // clock
  SolveCtl& cc = b->h_ctl[slot];
  WB_CK(cudaStreamSynchronize(b->stream));
  std::memset(&cc, 0, sizeof(SolveCtl));
  cc.t_end = t_end;
  cc.cfl_dx = (cfl > 0.0 ? cfl : b->cfl) * dx;
  cc.active = 1;
  cc.max_steps = max_steps > 0 ? max_steps : (1ll << 62);
  WB_CK(cudaMemcpyAsync(b->d_ctl + slot, &cc, sizeof(SolveCtl), cudaMemcpyHostToDevice, b->stream));
  // first dt: wave speed of the initial state over this solve's tiles
  std::vector<int4> mine;
  const int n = tiles_of(b, slot, mine);
  if (n > b->add_tile_cap) {
    cudaFree(b->d_add_tiles);
    b->d_add_tiles = nullptr;
    WB_CK(cudaMalloc(&b->d_add_tiles, sizeof(int4) * n));
    b->add_tile_cap = n;
  }
  WB_CK(cudaMemcpy(b->d_add_tiles, mine.data(), sizeof(int4) * n, cudaMemcpyHostToDevice));
  const int grid = std::min(n, b->sm_count * 8);
  if (b->prec == 32)
    WB_CK(BatchLaunch<float, true>::cfl(b->cfg, b->d_solves, b->d_ctl, b->d_add_tiles, n, grid, b->pool[0], b->gamma,
                                        b->stream));
  else if (b->mode == WENO_FAST)
    WB_CK(BatchLaunch<double, true>::cfl(b->cfg, b->d_solves, b->d_ctl, b->d_add_tiles, n, grid, b->pool[0],
                                         b->gamma, b->stream));
  else
    WB_CK(BatchLaunch<double, false>::cfl(b->cfg, b->d_solves, b->d_ctl, b->d_add_tiles, n, grid, b->pool[0],
                                          b->gamma, b->stream));
  WB_CK(cudaStreamSynchronize(b->stream));
  b->tiles_dirty = true;
  *slot_out = slot;
  return WENO_OK;
}

int weno_batch_remove(weno_batch* b, int slot) {
  if (!b || slot < 0 || slot >= b->max_solves || !b->used[slot]) return bfail(WENO_ERR_ARG, "batch_remove: bad slot");
  WB_CK(cudaStreamSynchronize(b->stream));
  pool_free(b, b->h_solves[slot].off, 4 * b->h_solves[slot].ps);
  if (b->ws_off[slot] >= 0) {
    fl_free(b->ws_free, b->ws_off[slot], b->ws_len[slot]);
    b->ws_off[slot] = -1;
  }
  b->used[slot] = false;
  SolveCtl zero{};
  WB_CK(cudaMemcpy(b->d_ctl + slot, &zero, sizeof(SolveCtl), cudaMemcpyHostToDevice));
  b->tiles_dirty = true;
  return WENO_OK;
}

int weno_batch_run(weno_batch* b, int64_t nsteps, int use_graph) {
  if (!b) return bfail(WENO_ERR_ARG, "batch_run: null handle");
  if (b->tiles_dirty) {
    int rc = rebuild_tiles(b);
    if (rc) return rc;
  }
  if (b->ntiles == 0 || nsteps <= 0) return WENO_OK;
  if (use_graph && (!b->graph || b->graph_ntiles != b->ntiles)) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    WB_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_step(b);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e) return bfail(WENO_ERR_CUDA, "batch step (capture): %s", cudaGetErrorString(e));
    if (e2) return bfail(WENO_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e2));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e) return bfail(WENO_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    b->graph_ntiles = b->ntiles;
  }
  for (int64_t k = 0; k < nsteps; ++k) {
    if (use_graph) WB_CK(cudaGraphLaunch(b->graph, b->stream));
    else WB_CK(enqueue_step(b));
  }
  return WENO_OK;
}

int weno_batch_get_state(weno_batch* b, int slot, double* out) {
  if (!b || !out || slot < 0 || slot >= b->max_solves || !b->used[slot])
    return bfail(WENO_ERR_ARG, "batch_get_state: bad argument");
  const SolveDesc& d = b->h_solves[slot];
  const dim3 blk(32, 4);
  const dim3 grd((unsigned)((d.ny + 6 + 31) / 32), (unsigned)((d.nx + 6 + 3) / 4));
  if (b->prec == 32)
    k_export_solve<float><<<grd, blk, 0, b->stream>>>(b->d_solves, slot, static_cast<const float*>(b->pool[0]),
                                                      b->gamma, out);
  else
    k_export_solve<double><<<grd, blk, 0, b->stream>>>(b->d_solves, slot, static_cast<const double*>(b->pool[0]),
                                                       b->gamma, out);
  WB_CK(cudaGetLastError());
  WB_CK(cudaStreamSynchronize(b->stream));
  return WENO_OK;
}

int weno_batch_info(weno_batch* b, int slot, double* t, int64_t* steps, int* active, int* status) {
  if (!b || slot < 0 || slot >= b->max_solves) return bfail(WENO_ERR_ARG, "batch_info: bad slot");
  WB_CK(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(SolveCtl) * b->max_solves, cudaMemcpyDeviceToHost, b->stream));
  WB_CK(cudaStreamSynchronize(b->stream));
  const SolveCtl& c = b->h_ctl[slot];
  if (t) *t = c.t;
  if (steps) *steps = c.steps;
  if (active) *active = b->used[slot] ? c.active : 0;
  if (status) *status = (c.status & 4) ? WENO_ERR_CUDA : (c.status ? WENO_ERR_NUMERIC : WENO_OK);
  return WENO_OK;
}

int weno_batch_poll(weno_batch* b, int* active, double* t, int64_t* steps) {
  if (!b) return bfail(WENO_ERR_ARG, "batch_poll: null handle");
  WB_CK(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(SolveCtl) * b->max_solves, cudaMemcpyDeviceToHost, b->stream));
  WB_CK(cudaStreamSynchronize(b->stream));
  for (int s = 0; s < b->max_solves; ++s) {
    if (active) active[s] = b->used[s] ? b->h_ctl[s].active : 0;
    if (t) t[s] = b->h_ctl[s].t;
    if (steps) steps[s] = b->h_ctl[s].steps;
  }
  return WENO_OK;
}

double weno_batch_bytes_per_cell(int precision, int force_hlle, int tile_config) {
  const double es = precision == 32 ? 4.0 : 8.0;
  double values = 12.0;  // three RK pools of four conserved planes
  if (tile_config == kStagedConfig) values += kStagedWsPerCellMargin * (16 + 2 * (force_hlle ? 4 : 9));
  return values * es;
}

int weno_batch_debug_skip_copy(weno_batch* b, int tile, int64_t wait_ns, int grid) {
  if (!b) return bfail(WENO_ERR_ARG, "batch_debug_skip_copy: null handle");
  if (tile >= 0 && (wait_ns <= 0 || grid < 0)) return bfail(WENO_ERR_ARG, "batch_debug_skip_copy: bad argument");
  WB_CK(cudaStreamSynchronize(b->stream));
  b->skip_tile = tile >= 0 ? tile : -1;
  b->wait_ns = tile >= 0 ? (unsigned long long)wait_ns : 1000000000ull;
  b->fixed_grid = tile >= 0 ? grid : 0;
  b->graph_ntiles = -1;  // launch arguments changed: re-capture the step graph
  return WENO_OK;
}

int weno_batch_stats(weno_batch* b, int64_t* ntiles, int64_t* free_cells, int* launches_per_step) {
  if (!b) return bfail(WENO_ERR_ARG, "batch_stats: null handle");
  if (b->tiles_dirty) {
    int rc = rebuild_tiles(b);
    if (rc) return rc;
  }
  long long fr = 0;
  for (auto& kv : b->free_list) fr += kv.second;
  if (ntiles) *ntiles = b->ntiles;
  if (free_cells) *free_cells = fr / 4;
  if (launches_per_step) *launches_per_step = 5;
  return WENO_OK;
}

}  // extern "C"
