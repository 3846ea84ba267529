// Test harness (tests only): builds the engine's host-side multigrid hierarchy
// (cfd-craft_gb300/csrc/setup.cpp, compiled with it by the test fixture) from a grid's
// arrays and exports its levels, so the CPU tests compare the engine's setup with the
// oracle without a GPU.
#include <algorithm>
#include <cstdint>
#include <memory>
#include <string>

#include "setup.hpp"

using namespace cfdg;

static std::unique_ptr<Hierarchy> g_h;
static std::unique_ptr<HostGrid> g_grid;
static std::string g_err;

extern "C" {

int32_t hh_build(const int32_t* n, const double* dx, double volume, const int32_t* periodic, int64_t nf,
                 const uint8_t* fluid, const uint8_t* kind, const int64_t* lo, const int64_t* hi, const double* area,
                 const double* dist, const int32_t* comp, int32_t ncomp, const uint8_t* anchored) {
  HostGrid h;
  for (int a = 0; a < 3; ++a) {
    h.n[a] = n[a];
    h.dx[a] = dx[a];
    h.periodic[a] = periodic[a];
  }
  h.volume = volume;
  h.cells = (int64_t)n[0] * n[1] * n[2];
  h.faces = nf;
  h.fluid.assign(fluid, fluid + h.cells);
  h.face_kind.assign(kind, kind + nf);
  h.face_lo.resize(nf);
  h.face_hi.resize(nf);
  for (int64_t f = 0; f < nf; ++f) {
    h.face_lo[f] = (int32_t)lo[f];
    h.face_hi[f] = (int32_t)hi[f];
  }
  h.face_area.assign(area, area + nf);
  h.face_distance.assign(dist, dist + nf);
  h.component.assign(comp, comp + h.cells);
  h.n_components = ncomp;
  h.anchored.assign(anchored, anchored + ncomp);
  g_err = check_layout(h);
  if (!g_err.empty()) return -1;
  g_grid = std::make_unique<HostGrid>(h);
  g_h = std::make_unique<Hierarchy>();
  Poller poll;
  return build_hierarchy(h, poll, *g_h);
}

int32_t hh_levels() { return g_h ? (int32_t)g_h->levels.size() : 0; }
int32_t hh_masked() { return g_h && g_h->masked ? 1 : 0; }

// Level `l` as a dense n x n matrix (diagonal plus off-diagonal entries); returns n.
int64_t hh_level_dense(int32_t l, double* dense) {
  const MgLevel& M = g_h->levels[l];
  const int64_t n = M.n;
  if (dense) {
    std::fill(dense, dense + n * n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
      dense[i * n + i] = M.diag[i];
      for (int32_t k = M.a.off[i]; k < M.a.off[i + 1]; ++k) dense[i * n + M.a.col[k]] += M.a.val[k];
    }
  }
  return n;
}

// Block smoother of level `l`: out = {length, bandwidth, blocks, forward dependency levels};
// returns 0 when the level has none.
int32_t hh_level_lines(int32_t l, int32_t* out) {
  const MgLevel& M = g_h->levels[l];
  if (M.lines.empty()) return 0;
  const LineBlocks& B = M.lines[0];
  out[0] = B.length;
  out[1] = B.bandwidth;
  out[2] = B.count();
  out[3] = B.fwd.levels();
  return 1;
}

// IC(0) of the grid last passed to hh_build (build_ic0) applied to r, in the order of
// pressure.rs:223-241 (forward substitution by rows, then the backward scatter).
int32_t hh_ic0_apply(const double* r, double* z) {
  if (!g_grid) return -1;
  Ic0 f;
  build_ic0(*g_grid, f);
  const int64_t n = g_grid->cells;
  for (int64_t i = 0; i < n; ++i) {
    double v = r[i];
    for (int32_t k = f.lower.off[i]; k < f.lower.off[i + 1]; ++k) v -= f.lower.val[k] * z[f.lower.col[k]];
    z[i] = v / f.diag[i];
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    const double v = z[i] / f.diag[i];
    z[i] = v;
    for (int32_t k = f.lower.off[i]; k < f.lower.off[i + 1]; ++k) z[f.lower.col[k]] -= f.lower.val[k] * v;
  }
  return 0;
}

}  // extern "C"
