// Shared state of the engine's translation units: error reporting, launch counting,
// device allocations and the per-grid state behind the C ABI's opaque handles.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cfdgpu.h"
#include "plain_kernels.cuh"
#include "setup.hpp"

namespace cfdg {

extern thread_local std::string t_error;  // last error message of the calling thread
extern std::atomic<uint64_t> g_launches;   // kernels enqueued by this library (graph launches count their nodes)
inline void count(uint64_t k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

inline double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

inline int fail(int code, const std::string& msg) {
  t_error = msg;
  return code;
}

#define CU(expr)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("CUDA: ") + #expr + ": " + cudaGetErrorString(e_)); \
  } while (0)

inline int grid_blocks(long long n) {
  long long b = (n + BLOCK - 1) / BLOCK;
  return (int)std::max(1LL, std::min<long long>(b, MAX_BLOCKS));
}

}  // namespace cfdg

struct cfdg_context {
  int device = 0;
  uint64_t budget = 0;
  std::atomic<uint64_t> used{0};
  // Grids keep their context alive: destroy() only marks it, the last grid frees it.
  std::mutex mu;
  int grids = 0;
  bool destroyed = false;
};

namespace cfdg {

// Device allocation owned by a grid, counted against the context's budget.
struct Arena {
  cfdg_context* ctx = nullptr;
  std::vector<void*> ptrs;
  uint64_t bytes = 0;
  template <class T>
  int alloc(T** p, size_t n) {
    size_t b = std::max<size_t>(n, 1) * sizeof(T);
    if (ctx->used.load() + b > ctx->budget) return fail(CFDG_ERR_ADMISSION, "the grid does not fit the context's HBM budget");
    CU(cudaMalloc((void**)p, b));
    ptrs.push_back(*p);
    bytes += b;
    ctx->used += b;
    return 0;
  }
  template <class T>
  int upload(T** p, const std::vector<T>& v, cudaStream_t s) {
    if (int e = alloc(p, v.size())) return e;
    if (!v.empty()) CU(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return 0;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    if (ctx) ctx->used -= bytes;
    ptrs.clear();
    bytes = 0;
  }
};

struct DevCsr {
  int* off = nullptr;
  int* col = nullptr;
  double* val = nullptr;
  int rows = 0;
};
inline int upload_csr(Arena& A, const Csr& c, DevCsr& d, cudaStream_t s) {
  d.rows = c.rows();
  if (int e = A.upload(&d.off, c.off, s)) return e;
  if (int e = A.upload(&d.col, c.col, s)) return e;
  if (!c.val.empty() || c.col.empty())
    if (int e = A.upload(&d.val, c.val, s)) return e;
  return 0;
}

struct DevSchedule {
  int* order = nullptr;
  std::vector<int32_t> start;
  int* d_start = nullptr;  // device copy of start (the cooperative coarse kernel walks it)
};

struct DevIc0 {
  Arena arena;
  ~DevIc0() { arena.release(); }
  DevCsr lower, upper;
  double* diag = nullptr;
  double *lx = nullptr, *ly = nullptr, *lz = nullptr;  // structured grids: per-cell lower coefficients
  DevSchedule fwd, bwd;
};

struct DevLevel {
  int n = 0;
  DevCsr a;
  double* diag = nullptr;
  DevSchedule fwd, bwd;
  DevCsr groups, prolong, restrict_;
  int ngroups = 0;
  bool terminal = false;
  int nblocks = 0;
  int* d_ioff = nullptr;
  int* d_idx = nullptr;
  long long* d_foff = nullptr;
  double* d_fac = nullptr;
  double *rhs = nullptr, *x = nullptr, *res = nullptr;
  // Anisotropic levels: the block smoother (setup.hpp LineBlocks) and its scratch.
  bool lines = false;
  int llen = 0, lbw = 0, lcount = 0;
  int *lnodes = nullptr, *looff = nullptr, *locol = nullptr;
  double *loval = nullptr, *lfac = nullptr, *lscr = nullptr;
  DevSchedule lfwd, lbwd;
};

struct DevHierarchy {
  Arena arena;
  ~DevHierarchy() { arena.release(); }
  bool masked = false;
  bool full0 = false;  // level 0 kept in full-grid layout and swept by the wavefront kernel
  int nfluid = 0;
  int* fluid_idx = nullptr;
  std::vector<DevLevel> levels;
  std::vector<uint64_t> level_cells, level_nonzeros;
  // Levels 1 .. L-1 as one cooperative kernel's descriptors (engine.cu PLev), and its grid
  // (0: not co-resident, the level-by-level launches are used instead).
  void* d_plev = nullptr;
  int coop_blocks = 0;
  bool cluster = false;  // the coarse kernel runs as one thread-block cluster (engine.cu)
  // Block-smoothed (anisotropic) hierarchies: d_plev starts at level 0 and the whole cycle
  // is the cooperative launch.
  bool coop0 = false;
};

}  // namespace cfdg

using namespace cfdg;

struct cfdg_grid {
  cfdg_context* ctx = nullptr;
  std::mutex mu;        // serialises solves on this grid
  std::mutex stats_mu;  // guards the stats copy (readable from a poll callback)
  std::string stats_json;
  HostGrid h;
  int preconditioner = 0, precision = 0;
  cudaStream_t stream = nullptr;  // where work is enqueued (the grid's own stream or the caller's)
  cudaStream_t own = nullptr;     // the grid's own stream; graphs are captured on it
  bool capturing = false;
  Arena arena;  // topology, weights, vectors, scalars
  GridDev g{};
  bool uniform = false;
  uint8_t* d_fluid = nullptr;
  uint16_t* d_flags = nullptr;
  uint8_t* d_kind = nullptr;
  int *d_lo = nullptr, *d_hi = nullptr;
  double *d_area = nullptr, *d_dist = nullptr, *d_fw = nullptr;
  DevCsr comp_groups;  // closed components of the grid
  int ncomp_groups = 0;
  double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *ap = nullptr, *bc = nullptr, *b = nullptr,
         *terms = nullptr, *u = nullptr, *pp = nullptr;
  double* partials = nullptr;
  Scalars* S = nullptr;
  Scalars* hS = nullptr;  // pinned mirror
  std::unique_ptr<DevIc0> ic0;
  std::unique_ptr<DevHierarchy> mg;
  std::unique_ptr<Signature> signature;
  cudaGraphExec_t chunk = nullptr;  // 8 PCG iterations
  int chunk_kind = -1;
  size_t chunk_nodes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool structured = false;  // no periodic axis: pipelined wavefront sweeps on the fine level
  int tiles_j = 0, tiles_k = 0;
  int* wave_sync = nullptr;  // ticket, abort, per-tile progress of one sweep
  int* wave_err = nullptr;   // set when a wavefront wait gave up
  long long wave_spin_limit = WAVE_SPIN_LIMIT;  // cfdg_debug_wave_stall
  int wave_hold_tile = -1;
  std::shared_ptr<cfdg::Hierarchy> host_mg;  // the hierarchy as uploaded (level 0 re-indexed when full0)
  // Mixed form on grids without solid cells: the aggregation hierarchy it runs on (level 0
  // re-indexed to the full grid), built on first use; null until then and for masked grids.
  std::shared_ptr<cfdg::Hierarchy> host_mg_mx;
  std::shared_ptr<void> mixed;               // the mixed-precision form's device state (mixed.cu)
  std::shared_ptr<struct cfdg_batch> solo;   // a one-grid batch for cfdg_project in the mixed form
  // Face coefficients change only through cfdg_grid_update_faces, which bumps
  // faces_version; the hierarchy's signature is re-compared only after a change.
  uint64_t faces_version = 0;
  // Mixed form: V-cycle sweeps before and after the coarse correction on level 0 and on
  // the coarse levels (cfdg_grid_set_cycle); a batch takes them from its grids.
  int mx_nu0 = 2, mx_nuc = 2;
  float mx_alpha = 1.8f;  // mixed form: coarse-correction scale on aggregation hierarchies
  // Mixed form: tile shape of the staged level-0 half sweeps (cfdg_grid_set_sweep_tile):
  // rows per shared-memory stage (8, 16, 32) and stages in flight per block (2..8); 0 and 0
  // choose from the row length when a batch is packed.
  int mx_sweep_rows = 0, mx_sweep_stages = 0;
  // Mixed form: first coarse level laid out as the 2x2x2 bin grid where the hierarchy
  // allows it (cfdg_grid_set_coarse_layout); 0 keeps the aggregates' colour order.
  int mx_bins = 1;
  // Laminar time stepping (cfdg_grid_set_flow / cfdg_step_device): the case flow and the
  // stage buffers (cell velocities, the two stage velocities, the stage pressure).
  bool has_flow = false;
  int flow_bnd[3] = {0, 0, 0};
  double flow_size[3] = {0, 0, 0}, flow_vel[3] = {0, 0, 0}, flow_nu = 0, flow_acc[3] = {0, 0, 0};
  double *st_cu = nullptr, *st_v = nullptr, *st_v2 = nullptr, *st_p1 = nullptr;
  double* sc_part = nullptr;  // scalar transport rates: two stages of per-block partials, then three rates
  int sc_muscl = 0;           // scalar transport advection: 0 linear upwind, 1 MUSCL (cfdg_grid_set_advection)
  double* st_sc = nullptr;  // scalar transport: the SSPRK2 stage (N)
  // Receptors (cfdg_receptors_set): CSR of cells and weights, in receptor order.
  int32_t rc_n = 0, rc_cap_n = 0;
  int64_t rc_cap_entries = 0;
  int64_t* rc_off = nullptr;
  int32_t* rc_cell = nullptr;
  double* rc_w = nullptr;
  // Scalar transport on a uniform grid: per axis and transporting kind (interior, inlet,
  // outlet) the one face area and distance, bit for bit (refresh_weights).
  bool sc_uniform = false;
  bool sc_used[3][3] = {};
  double sc_area[3][3] = {}, sc_dist[3][3] = {};
  uint64_t sig_version = ~0ull;
};

struct cfdg_batch;

namespace cfdg {
// engine.cu helpers used by the mixed form (the grid's lock is held by the caller).
int prepare_multigrid(cfdg_grid* G);                     // builds or reuses the hierarchy
int mixed_host_hierarchy(cfdg_grid* G, std::shared_ptr<Hierarchy>& out);  // the mixed form's host hierarchy
int plain_compat_center(cfdg_grid* G, cudaStream_t s);  // E031 check of G->b, then G->bc = centred b
void plain_center(cfdg_grid* G, double* x, cudaStream_t s);
}  // namespace cfdg

// mixed.cu
cfdg_batch* cfdg_mixed_new(cfdg_context* ctx);
void cfdg_mixed_delete(cfdg_batch* B);
void cfdg_mixed_set_stream(cfdg_batch* B, cudaStream_t s);
int cfdg_mixed_add_case(cfdg_batch* B, cfdg_grid* G);
int cfdg_mixed_pack(cfdg_batch* B);
int cfdg_mixed_project(cfdg_batch* B, double* const* d_u, double* const* d_p, const double* dt, double tol,
                       uint64_t max_iter, cfdg_poll_fn poll, void* poll_ctx, cfdg_info* infos, int32_t* codes);
