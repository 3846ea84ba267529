// Host-side setup of the pressure engine (see setup.hpp). Compiled with
// -ffp-contract=off: every sum and product is evaluated as written, in the
// reference's order, so factors and coarse operators match it bit for bit.
#include "setup.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>

#include "../../include/cfdgpu.h"

namespace cfdg {

int Poller::check() const {
  if (!fn) return 0;
  int r = fn(ctx);
  if (r == 1) return CFDG_CANCELLED;
  if (r == 2) return CFDG_WALL_TIME;
  return 0;
}

std::string check_layout(HostGrid& g) {
  int64_t total = 0;
  for (int a = 0; a < 3; ++a) {
    if (g.n[a] < 1) return "cell counts must be positive";
    g.face_offset[a] = total;
    for (int d = 0; d < 3; ++d) g.face_dims[a][d] = g.n[d];
    if (!g.periodic[a]) g.face_dims[a][a] += 1;
    total += g.face_dims[a][0] * g.face_dims[a][1] * g.face_dims[a][2];
  }
  if (total != g.faces) return "face count does not match the staggered layout";
  if (g.cells != (int64_t)g.n[0] * g.n[1] * g.n[2]) return "cell count mismatch";
  if (g.cells >= (int64_t)1 << 31) return "more than 2^31 cells";
  // Each face's lo/hi must be the structural neighbour (wrapped on a periodic
  // axis) when that cell is fluid, else -1 (grid.rs:352-370); interior iff both.
  for (int a = 0; a < 3; ++a) {
    const int64_t* fd = g.face_dims[a];
    int64_t f = g.face_offset[a];
    for (int64_t k = 0; k < fd[2]; ++k)
      for (int64_t j = 0; j < fd[1]; ++j)
        for (int64_t i = 0; i < fd[0]; ++i, ++f) {
          int64_t q[3] = {i, j, k};
          int64_t t = q[a];
          int64_t lo0 = -1, hi0 = -1;
          if (t > 0) {
            int64_t p[3] = {i, j, k};
            p[a] -= 1;
            lo0 = g.cell(p[0], p[1], p[2]);
          } else if (g.periodic[a]) {
            int64_t p[3] = {i, j, k};
            p[a] = g.n[a] - 1;
            lo0 = g.cell(p[0], p[1], p[2]);
          }
          if (t < g.n[a]) hi0 = g.cell(i, j, k);
          int64_t lo = (lo0 >= 0 && g.fluid[lo0]) ? lo0 : -1;
          int64_t hi = (hi0 >= 0 && g.fluid[hi0]) ? hi0 : -1;
          if (g.face_lo[f] != lo || g.face_hi[f] != hi) return "face lo/hi do not match the mask";
          bool interior = lo >= 0 && hi >= 0;
          if (interior != (g.face_kind[f] == INTERIOR)) return "face kind does not match lo/hi";
          if (g.face_kind[f] == OUTLET && (lo >= 0) == (hi >= 0)) return "outlet face without exactly one cell";
          if (g.face_kind[f] > BLOCKED) return "unknown face kind";
        }
  }
  for (int64_t c = 0; c < g.cells; ++c) {
    int32_t id = g.component[c];
    if (g.fluid[c] ? (id < 0 || id >= g.n_components) : id != -1) return "component ids do not match the mask";
  }
  return "";
}

Schedule schedule(const Csr& pattern, bool backward) {
  int32_t n = pattern.rows();
  std::vector<int32_t> lev(n, 0);
  int32_t top = 0;
  for (int32_t s = 0; s < n; ++s) {
    int32_t i = backward ? n - 1 - s : s;
    int32_t l = 0;
    for (int32_t k = pattern.off[i]; k < pattern.off[i + 1]; ++k) {
      int32_t j = pattern.col[k];
      if (backward ? j > i : j < i) l = std::max(l, lev[j] + 1);
    }
    lev[i] = l;
    top = std::max(top, l);
  }
  Schedule out;
  out.start.assign(n ? top + 2 : 1, 0);
  for (int32_t i = 0; i < n; ++i) out.start[lev[i] + 1] += 1;
  for (size_t l = 1; l < out.start.size(); ++l) out.start[l] += out.start[l - 1];
  out.order.assign(n, 0);
  std::vector<int32_t> fill(out.start.begin(), out.start.end() - 1);
  for (int32_t i = 0; i < n; ++i) out.order[fill[lev[i]]++] = i;
  return out;
}

// ------------------------------------------------------------------ IC(0)
void build_ic0(const HostGrid& g, Ic0& out) {
  const int64_t N = g.cells;
  // A row of the factor has at most six columns (six faces); periodic
  // duplicates of one neighbour merge into one entry (pressure.rs:147-156).
  std::vector<int32_t> cols(N * 6);
  std::vector<double> vals(N * 6);
  std::vector<uint8_t> cnt(N, 0);
  std::vector<double> diag(N, 0.0);
  for (int64_t f = 0; f < g.faces; ++f) {
    double w = g.weight(f);
    if (g.face_kind[f] == INTERIOR) {
      int32_t i = g.face_lo[f], j = g.face_hi[f];
      if (i == j) continue;  // a one-cell periodic axis joins a cell to itself
      diag[i] += w;
      diag[j] += w;
      int32_t row = std::max(i, j), col = std::min(i, j);
      int32_t* rc = &cols[row * 6];
      double* rv = &vals[row * 6];
      int e = 0;
      while (e < cnt[row] && rc[e] != col) ++e;
      if (e < cnt[row]) {
        rv[e] -= w;
      } else {
        rc[e] = col;
        rv[e] = -w;
        cnt[row] += 1;
      }
    } else if (g.face_kind[f] == OUTLET) {
      diag[g.face_lo[f] >= 0 ? g.face_lo[f] : g.face_hi[f]] += w;
    }
  }
  double maxdiag = 1.0;
  for (double d : diag) maxdiag = std::fmax(maxdiag, d);
  out.lower.off.assign(N + 1, 0);
  for (int64_t r = 0; r < N; ++r) {
    int32_t* rc = &cols[r * 6];
    double* rv = &vals[r * 6];
    // Insertion sort by column, carrying the values (pressure.rs:166-187).
    for (int e = 1; e < cnt[r]; ++e) {
      int32_t c = rc[e];
      double v = rv[e];
      int at = e;
      for (; at > 0 && rc[at - 1] > c; --at) {
        rc[at] = rc[at - 1];
        rv[at] = rv[at - 1];
      }
      rc[at] = c;
      rv[at] = v;
    }
    out.lower.off[r + 1] = out.lower.off[r] + cnt[r];
  }
  // Numeric factorisation in row order (pressure.rs:191-215).
  for (int64_t r = 0; r < N; ++r) {
    int32_t* rc = &cols[r * 6];
    double* rv = &vals[r * 6];
    for (int e = 0; e < cnt[r]; ++e) {
      int32_t c = rc[e];
      const int32_t* oc = &cols[(int64_t)c * 6];
      const double* ov = &vals[(int64_t)c * 6];
      double dot = 0.0;
      int other = 0;
      for (int prev = 0; prev < e; ++prev) {
        int32_t k = rc[prev];
        while (other < cnt[c] && oc[other] < k) ++other;
        if (other < cnt[c] && oc[other] == k) dot += rv[prev] * ov[other];
      }
      rv[e] = (rv[e] - dot) / diag[c];
    }
    double squared = -0.0;
    for (int e = 0; e < cnt[r]; ++e) squared += rv[e] * rv[e];
    diag[r] = std::sqrt(std::fmax(diag[r] + 1e-6 * maxdiag - squared, 1e-12 * maxdiag));
  }
  int64_t nnz = out.lower.off[N];
  out.lower.col.resize(nnz);
  out.lower.val.resize(nnz);
  for (int64_t r = 0; r < N; ++r)
    for (int e = 0; e < cnt[r]; ++e) {
      out.lower.col[out.lower.off[r] + e] = cols[r * 6 + e];
      out.lower.val[out.lower.off[r] + e] = vals[r * 6 + e];
    }
  out.diag = std::move(diag);
  // Transpose: column c lists the rows i > c holding it, descending.
  out.upper.off.assign(N + 1, 0);
  for (int64_t k = 0; k < nnz; ++k) out.upper.off[out.lower.col[k] + 1] += 1;
  for (int64_t c = 0; c < N; ++c) out.upper.off[c + 1] += out.upper.off[c];
  out.upper.col.resize(nnz);
  out.upper.val.resize(nnz);
  std::vector<int32_t> fill(out.upper.off.begin(), out.upper.off.end() - 1);
  for (int64_t r = N; r-- > 0;)
    for (int32_t k = out.lower.off[r]; k < out.lower.off[r + 1]; ++k) {
      int32_t c = out.lower.col[k];
      out.upper.col[fill[c]] = (int32_t)r;
      out.upper.val[fill[c]] = out.lower.val[k];
      fill[c] += 1;
    }
  // Symmetric pattern for the schedules.
  Csr pattern;
  pattern.off.assign(N + 1, 0);
  for (int64_t r = 0; r < N; ++r)
    pattern.off[r + 1] = pattern.off[r] + (out.lower.off[r + 1] - out.lower.off[r]) + (out.upper.off[r + 1] - out.upper.off[r]);
  pattern.col.resize(pattern.off[N]);
  for (int64_t r = 0; r < N; ++r) {
    int32_t at = pattern.off[r];
    for (int32_t k = out.lower.off[r]; k < out.lower.off[r + 1]; ++k) pattern.col[at++] = out.lower.col[k];
    for (int32_t k = out.upper.off[r]; k < out.upper.off[r + 1]; ++k) pattern.col[at++] = out.upper.col[k];
  }
  out.fwd = schedule(pattern, false);
  out.bwd = schedule(pattern, true);
}

// ------------------------------------------------------------------ multigrid
struct Edge {
  int32_t i, j;
  double w;
};

// multigrid.rs:233-262: rows filled in edge order, diagonal = anchors + weights.
static void matrix_build(const std::vector<Edge>& edges, const std::vector<double>& anchors, Csr& a,
                         std::vector<double>& diag) {
  int32_t n = (int32_t)anchors.size();
  a.off.assign(n + 1, 0);
  for (auto& e : edges) {
    a.off[e.i + 1] += 1;
    a.off[e.j + 1] += 1;
  }
  for (int32_t i = 0; i < n; ++i) a.off[i + 1] += a.off[i];
  a.col.assign(a.off[n], 0);
  a.val.assign(a.off[n], 0.0);
  std::vector<int32_t> next(a.off.begin(), a.off.end() - 1);
  diag = anchors;
  for (auto& e : edges) {
    int32_t pairs[2][2] = {{e.i, e.j}, {e.j, e.i}};
    for (auto& p : pairs) {
      diag[p[0]] += e.w;
      a.col[next[p[0]]] = p[1];
      a.val[next[p[0]]] = -e.w;
      next[p[0]] += 1;
    }
  }
}

// Dense lower Cholesky of the rows `idx` (masked.rs:21-51, multigrid.rs:468-500).
static int dense_cholesky(const Csr& a, const std::vector<double>& diag, const std::vector<int32_t>& idx,
                          std::vector<double>& l) {
  size_t n = idx.size();
  std::map<int32_t, size_t> local;
  for (size_t j = 0; j < n; ++j) local[idx[j]] = j;
  l.assign(n * n, 0.0);
  for (size_t i = 0; i < n; ++i) {
    int32_t row = idx[i];
    l[i * n + i] = diag[row];
    for (int32_t at = a.off[row]; at < a.off[row + 1]; ++at) {
      auto it = local.find(a.col[at]);
      if (it != local.end()) l[i * n + it->second] += a.val[at];
    }
  }
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j <= i; ++j) {
      double v = l[i * n + j];
      for (size_t k = 0; k < j; ++k) v -= l[i * n + k] * l[j * n + k];
      if (i == j) {
        if (!std::isfinite(v) || v <= 0.0) return CFDG_E035;
        l[i * n + j] = std::sqrt(v);
      } else {
        l[i * n + j] = v / l[j * n + j];
      }
    }
  return 0;
}

static Csr groups_of(const std::vector<std::vector<int32_t>>& lists) {
  Csr c;
  c.off.push_back(0);
  for (auto& l : lists) {
    c.col.insert(c.col.end(), l.begin(), l.end());
    c.off.push_back((int32_t)c.col.size());
  }
  return c;
}

static void finish_terminal(MgLevel& lev, const std::vector<std::vector<int32_t>>& blocks,
                            const std::vector<std::vector<double>>& factors) {
  lev.direct_idx = groups_of(blocks);
  lev.direct_off.clear();
  lev.direct_factor.clear();
  for (auto& f : factors) {
    lev.direct_off.push_back((int64_t)lev.direct_factor.size());
    lev.direct_factor.insert(lev.direct_factor.end(), f.begin(), f.end());
  }
  lev.direct_off.push_back((int64_t)lev.direct_factor.size());
}

// Coarse transfer of a piecewise-constant aggregation: P[i] = e_parent(i).
static void aggregation_transfer(const std::vector<int32_t>& parent, int32_t nc, MgLevel& lev) {
  int32_t n = (int32_t)parent.size();
  lev.prolong.off.resize(n + 1);
  lev.prolong.col.resize(n);
  lev.prolong.val.assign(n, 1.0);
  for (int32_t i = 0; i <= n; ++i) lev.prolong.off[i] = i;
  for (int32_t i = 0; i < n; ++i) lev.prolong.col[i] = parent[i];
  lev.restrict.off.assign(nc + 1, 0);
  for (int32_t i = 0; i < n; ++i) lev.restrict.off[parent[i] + 1] += 1;
  for (int32_t j = 0; j < nc; ++j) lev.restrict.off[j + 1] += lev.restrict.off[j];
  lev.restrict.col.resize(n);
  lev.restrict.val.assign(n, 1.0);
  std::vector<int32_t> fill(lev.restrict.off.begin(), lev.restrict.off.end() - 1);
  for (int32_t i = 0; i < n; ++i) lev.restrict.col[fill[parent[i]]++] = i;
}

typedef std::array<int32_t, 3> C3;

// masked.rs:181-291
static int build_masked(const HostGrid& g, const Poller& poll, Hierarchy& h) {
  h.masked = true;
  std::vector<int32_t> compact(g.cells, -1);
  for (int64_t c = 0; c < g.cells; ++c)
    if (g.fluid[c]) {
      compact[c] = (int32_t)h.fluid_indices.size();
      h.fluid_indices.push_back((int32_t)c);
    }
  std::vector<C3> coords;
  coords.reserve(h.fluid_indices.size());
  for (int32_t c : h.fluid_indices)
    coords.push_back({c % g.n[0], c / g.n[0] % g.n[1], c / (g.n[0] * g.n[1])});
  std::vector<double> anchors(coords.size(), 0.0);
  std::vector<Edge> edges;
  for (int64_t f = 0; f < g.faces; ++f) {
    double w = g.weight(f);
    if (g.face_kind[f] == INTERIOR && g.face_lo[f] != g.face_hi[f])
      edges.push_back({compact[g.face_lo[f]], compact[g.face_hi[f]], w});
    else if (g.face_kind[f] == OUTLET)
      anchors[compact[g.face_lo[f] >= 0 ? g.face_lo[f] : g.face_hi[f]]] += w;
  }
  for (;;) {
    if (int c = poll.check()) return c;
    MgLevel lev;
    lev.n = (int32_t)coords.size();
    matrix_build(edges, anchors, lev.a, lev.diag);
    // Components by breadth-first search over the matrix rows (masked.rs:90-126).
    std::vector<std::vector<int32_t>> regions;
    std::vector<uint8_t> fixed;
    {
      std::vector<uint8_t> seen(lev.n, 0);
      for (int32_t s = 0; s < lev.n; ++s) {
        if (s % 1024 == 0)
          if (int c = poll.check()) return c;
        if (seen[s]) continue;
        seen[s] = 1;
        std::deque<int32_t> queue{s};
        std::vector<int32_t> cells;
        bool anchored = false;
        while (!queue.empty()) {
          int32_t i = queue.front();
          queue.pop_front();
          if (cells.size() % 1024 == 0)
            if (int c = poll.check()) return c;
          cells.push_back(i);
          anchored |= anchors[i] > 0.0;
          for (int32_t k = lev.a.off[i]; k < lev.a.off[i + 1]; ++k) {
            int32_t j = lev.a.col[k];
            if (!seen[j]) {
              seen[j] = 1;
              queue.push_back(j);
            }
          }
        }
        regions.push_back(std::move(cells));
        fixed.push_back(anchored);
      }
    }
    std::vector<std::vector<int32_t>> closed;
    bool small = true;
    for (size_t r = 0; r < regions.size(); ++r) {
      if (!fixed[r]) closed.push_back(regions[r]);
      small &= regions[r].size() <= 32;
    }
    lev.groups = groups_of(closed);
    if (small) {
      std::vector<std::vector<int32_t>> blocks;
      std::vector<std::vector<double>> factors;
      for (size_t r = 0; r < regions.size(); ++r) {
        std::vector<int32_t> idx(regions[r].begin() + (fixed[r] ? 0 : 1), regions[r].end());
        std::vector<double> l;
        if (int e = dense_cholesky(lev.a, lev.diag, idx, l)) return e;
        blocks.push_back(std::move(idx));
        factors.push_back(std::move(l));
      }
      finish_terminal(lev, blocks, factors);
      for (auto& p : coords) lev.parity.push_back((uint8_t)((p[0] + p[1] + p[2]) & 1));
      h.levels.push_back(std::move(lev));
      break;
    }
    // Connected aggregates within 2x2x2 bins, in discovery order (masked.rs:127-156).
    std::vector<int32_t> parent(lev.n, -1);
    std::vector<C3> coarse;
    for (int32_t s = 0; s < lev.n; ++s) {
      if (s % 1024 == 0)
        if (int c = poll.check()) return c;
      if (parent[s] >= 0) continue;
      C3 bin = {coords[s][0] / 2, coords[s][1] / 2, coords[s][2] / 2};
      int32_t id = (int32_t)coarse.size();
      coarse.push_back(bin);
      parent[s] = id;
      std::deque<int32_t> queue{s};
      while (!queue.empty()) {
        int32_t i = queue.front();
        queue.pop_front();
        for (int32_t k = lev.a.off[i]; k < lev.a.off[i + 1]; ++k) {
          int32_t j = lev.a.col[k];
          if (parent[j] < 0 && coords[j][0] / 2 == bin[0] && coords[j][1] / 2 == bin[1] && coords[j][2] / 2 == bin[2]) {
            parent[j] = id;
            queue.push_back(j);
          }
        }
      }
    }
    if ((int32_t)coarse.size() == lev.n) {
      bool all_zero = true;
      for (auto& p : coords) {
        p = {p[0] / 2, p[1] / 2, p[2] / 2};
        all_zero &= p[0] == 0 && p[1] == 0 && p[2] == 0;
      }
      if (all_zero) return CFDG_E035;
      continue;
    }
    int32_t nc = (int32_t)coarse.size();
    // Coarse edges: weights summed per aggregate pair in edge order, emitted in
    // pair order (the BTreeMap of masked.rs:239-249), via a stable sort.
    struct Keyed {
      int64_t key;
      double w;
    };
    std::vector<Keyed> keyed;
    keyed.reserve(edges.size());
    for (auto& e : edges) {
      int32_t a = parent[e.i], b = parent[e.j];
      if (a != b) keyed.push_back({(int64_t)std::min(a, b) * nc + std::max(a, b), e.w});
    }
    std::stable_sort(keyed.begin(), keyed.end(), [](const Keyed& x, const Keyed& y) { return x.key < y.key; });
    std::vector<Edge> next;
    for (size_t s = 0; s < keyed.size();) {
      double sum = 0.0;
      size_t t = s;
      for (; t < keyed.size() && keyed[t].key == keyed[s].key; ++t) sum += keyed[t].w;
      next.push_back({(int32_t)(keyed[s].key / nc), (int32_t)(keyed[s].key % nc), sum});
      s = t;
    }
    std::vector<double> ac(nc, 0.0);
    for (size_t i = 0; i < anchors.size(); ++i) ac[parent[i]] += anchors[i];
    aggregation_transfer(parent, nc, lev);
    for (auto& p : coords) lev.parity.push_back((uint8_t)((p[0] + p[1] + p[2]) & 1));
    h.levels.push_back(std::move(lev));
    edges = std::move(next);
    anchors = std::move(ac);
    coords = std::move(coarse);
  }
  return 0;
}

// multigrid.rs:296-320
static std::vector<std::pair<int32_t, double>> axis_weights(double x, const std::vector<double>& centers, bool periodic,
                                                            double extent) {
  int32_t n = (int32_t)centers.size();
  if (n == 1) return {{0, 1.0}};
  int32_t hi = (int32_t)(std::partition_point(centers.begin(), centers.end(), [&](double v) { return v < x; }) -
                         centers.begin());
  int32_t lo_i, hi_i;
  double left, right;
  if (hi == 0) {
    if (!periodic) return {{0, 1.0}};
    lo_i = n - 1, hi_i = 0, left = centers[n - 1] - extent, right = centers[0];
  } else if (hi == n) {
    if (!periodic) return {{n - 1, 1.0}};
    lo_i = n - 1, hi_i = 0, left = centers[n - 1], right = centers[0] + extent;
  } else {
    lo_i = hi - 1, hi_i = hi, left = centers[hi - 1], right = centers[hi];
  }
  double t = (x - left) / (right - left);
  std::vector<std::pair<int32_t, double>> out;
  if (1.0 - t != 0.0) out.push_back({lo_i, 1.0 - t});
  if (t != 0.0) out.push_back({hi_i, t});
  return out;
}

static std::vector<int> line_axes(const int32_t n[3], const double dx[3]) {
  double w[3];
  for (int a = 0; a < 3; ++a) {
    w[a] = 1.0 / (dx[a] * dx[a]);
    if (!std::isfinite(w[a]) || w[a] <= 0.0) return {};
  }
  double lo = INFINITY, hi = 0.0;
  for (int a = 0; a < 3; ++a) {
    if (n[a] > 2) lo = std::fmin(lo, w[a]);
    hi = std::fmax(hi, w[a]);
  }
  if (hi / lo <= 25.0) return {};
  std::vector<int> out;
  for (int a = 0; a < 3; ++a)
    if (w[a] >= hi / 4.0) out.push_back(a);
  return out;
}

// multigrid/line.rs:39-150 BlockSmoother::build: node order (a periodic axis folded to
// 0, n-1, 1, n-2, ...), bandwidth from the entries, outside-block rows, banded Cholesky per
// block with reciprocal diagonals; CFD-E036 on a non-positive pivot. The block-level
// dependency schedules are the engine's (blocks that share an outside entry).
static int build_lines(const Csr& a, const std::vector<double>& diag, const int32_t n[3], const std::vector<int>& axes,
                       const bool periodic[3], const Poller& poll, LineBlocks& out) {
  const int32_t count = (int32_t)diag.size();
  out.axes.assign(axes.begin(), axes.end());
  int32_t length = 1;
  for (int ax : axes) length *= n[ax];
  out.length = length;
  out.nodes.clear();
  out.nodes.reserve(count);
  for (int32_t i = 0; i < count; ++i) {
    int32_t q[3] = {i % n[0], i / n[0] % n[1], i / (n[0] * n[1])};
    bool skip = false;
    for (int ax : axes) skip |= q[ax] != 0;
    if (skip) continue;
    for (int32_t at = 0; at < length; ++at) {
      int32_t remainder = at;
      for (int ax : axes) {
        const int32_t v = remainder % n[ax];
        remainder /= n[ax];
        q[ax] = !periodic[ax] ? v : (v % 2 == 0 ? v / 2 : n[ax] - 1 - v / 2);
      }
      out.nodes.push_back((q[2] * n[1] + q[1]) * n[0] + q[0]);
    }
  }
  std::vector<int32_t> position(count, 0);
  for (int32_t at = 0; at < (int32_t)out.nodes.size(); ++at) position[out.nodes[at]] = at;
  int32_t bw = 0;
  for (int32_t i = 0; i < count; ++i)
    for (int32_t k = a.off[i]; k < a.off[i + 1]; ++k) {
      const int32_t pi = position[i], pj = position[a.col[k]];
      if (pi / length == pj / length) bw = std::max(bw, pi > pj ? pi - pj : pj - pi);
    }
  out.bandwidth = bw;
  const int64_t stride = bw + 1;
  out.outside.off.assign(1, 0);
  out.outside.col.clear();
  out.outside.val.clear();
  for (int32_t at = 0; at < (int32_t)out.nodes.size(); ++at) {
    const int32_t cell = out.nodes[at];
    for (int32_t k = a.off[cell]; k < a.off[cell + 1]; ++k)
      if (position[a.col[k]] / length != at / length) {
        out.outside.col.push_back(a.col[k]);
        out.outside.val.push_back(a.val[k]);
      }
    out.outside.off.push_back((int32_t)out.outside.col.size());
  }
  std::vector<double>& f = out.factor;
  f.assign((size_t)count * stride, 0.0);
  for (int32_t at = 0; at < (int32_t)out.nodes.size(); ++at) {
    const int32_t cell = out.nodes[at];
    f[at * stride] = diag[cell];
    for (int32_t k = a.off[cell]; k < a.off[cell + 1]; ++k) {
      const int32_t col = position[a.col[k]];
      if (col / length == at / length && col < at) f[at * stride + at - col] += a.val[k];
    }
  }
  for (int32_t line = 0; line < count / length; ++line) {
    if (line % 128 == 0)
      if (int c = poll.check()) return c;
    const int64_t base = (int64_t)line * length * stride;
    for (int32_t i = 0; i < length; ++i)
      for (int32_t j = std::max(0, i - bw); j <= i; ++j) {
        const int64_t row = base + i * stride, other = base + j * stride;
        double value = f[row + i - j];
        for (int32_t k = std::max(0, i - bw); k < j; ++k) value -= f[row + i - k] * f[other + j - k];
        if (i == j) {
          if (!std::isfinite(value) || value <= 0.0) return CFDG_E036;
          f[row] = std::sqrt(value);
        } else {
          f[row + i - j] = value / f[other];
        }
      }
  }
  for (int32_t row = 0; row < count; ++row) f[row * stride] = 1.0 / f[row * stride];
  // Block dependency pattern: block b reads the cells of the blocks its outside entries name.
  const int32_t nb = count / length;
  std::vector<std::vector<int32_t>> adj(nb);
  for (int32_t at = 0; at < (int32_t)out.nodes.size(); ++at)
    for (int32_t k = out.outside.off[at]; k < out.outside.off[at + 1]; ++k)
      adj[at / length].push_back(position[out.outside.col[k]] / length);
  Csr pattern;
  pattern.off.assign(1, 0);
  for (auto& v : adj) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    pattern.col.insert(pattern.col.end(), v.begin(), v.end());
    pattern.off.push_back((int32_t)pattern.col.size());
  }
  out.fwd = schedule(pattern, false);
  out.bwd = schedule(pattern, true);
  return 0;
}

// multigrid.rs:530-645 (tensor-linear P, Galerkin coarse operators), with the line/plane
// block smoothers and semicoarsening of anisotropic grids (:573-607).
static int build_unmasked(const HostGrid& g, const Poller& poll, Hierarchy& h) {
  h.masked = false;
  const std::vector<int> axes = line_axes(g.n, g.dx);
  int32_t n[3] = {g.n[0], g.n[1], g.n[2]};
  std::vector<double> centers[3];
  for (int a = 0; a < 3; ++a)
    for (int32_t i = 0; i < n[a]; ++i) centers[a].push_back((double)i + 0.5);
  double extent[3] = {(double)n[0], (double)n[1], (double)n[2]};
  bool periodic[3] = {false, false, false};
  for (int a = 0; a < 3; ++a) {
    // multigrid.rs:544-548: an interior face at coordinate 0 of its axis
    int64_t f = g.face_offset[a];
    const int64_t* fd = g.face_dims[a];
    for (int64_t k = 0; k < fd[2] && !periodic[a]; ++k)
      for (int64_t j = 0; j < fd[1] && !periodic[a]; ++j)
        for (int64_t i = 0; i < fd[0]; ++i, ++f) {
          int64_t q[3] = {i, j, k};
          if (q[a] == 0 && g.face_kind[f] == INTERIOR) {
            periodic[a] = true;
            break;
          }
        }
  }
  bool anchored = g.anchored[0] != 0;
  std::vector<double> anchors(g.cells, 0.0);
  std::vector<Edge> edges;
  for (int64_t f = 0; f < g.faces; ++f) {
    double w = g.weight(f);
    if (g.face_kind[f] == INTERIOR) edges.push_back({g.face_lo[f], g.face_hi[f], w});
    else if (g.face_kind[f] == OUTLET) anchors[g.face_lo[f] >= 0 ? g.face_lo[f] : g.face_hi[f]] += w;
  }
  for (;;) {
    if (int c = poll.check()) return c;
    MgLevel lev;
    lev.n = (int32_t)anchors.size();
    h.level_dims.push_back({n[0], n[1], n[2]});
    matrix_build(edges, anchors, lev.a, lev.diag);
    if (!anchored) {
      std::vector<int32_t> all(lev.n);
      for (int32_t i = 0; i < lev.n; ++i) all[i] = i;
      lev.groups = groups_of({all});
    } else {
      lev.groups = groups_of({});
    }
    if (lev.n <= 32) {
      std::vector<int32_t> idx;
      for (int32_t i = anchored ? 0 : 1; i < lev.n; ++i) idx.push_back(i);
      std::vector<double> l;
      if (int e = dense_cholesky(lev.a, lev.diag, idx, l)) return e;
      finish_terminal(lev, {idx}, {l});
      h.levels.push_back(std::move(lev));
      break;
    }
    // Which axes coarsen: all with more than two cells, or on anisotropic grids only the
    // stiff ones until they are down to two cells (multigrid.rs:575-581).
    bool coarsen[3] = {n[0] > 2, n[1] > 2, n[2] > 2};
    if (!axes.empty()) {
      bool stiff_can_coarsen = false;
      for (int a : axes) stiff_can_coarsen |= n[a] > 2;
      for (int a = 0; a < 3; ++a) {
        const bool in_axes = std::find(axes.begin(), axes.end(), a) != axes.end();
        coarsen[a] = n[a] > 2 && (!stiff_can_coarsen || in_axes);
      }
      // :584-599: one plane block over all stiff axes when it holds at most 16 cells,
      // else lines along the stiff axis of smallest spacing (the first of equals).
      std::vector<int> group;
      int32_t plane = 1;
      for (int a : axes) plane *= n[a];
      if (axes.size() > 1 && plane <= 16) {
        group = axes;
      } else {
        int best = axes[0];
        for (int a : axes)
          if (g.dx[a] < g.dx[best]) best = a;
        group = {best};
      }
      LineBlocks lb;
      if (int e = build_lines(lev.a, lev.diag, n, group, periodic, poll, lb)) return e;
      lev.lines.push_back(std::move(lb));
    }
    // Tensor-linear interpolation (multigrid.rs:330-371).
    std::vector<double> coarse[3];
    std::vector<std::vector<std::pair<int32_t, double>>> wts[3];
    for (int a = 0; a < 3; ++a) {
      size_t step = coarsen[a] ? 2 : 1;
      for (size_t s = 0; s < centers[a].size(); s += step) {
        size_t e = std::min(s + step, centers[a].size());
        double sum = -0.0;
        for (size_t q = s; q < e; ++q) sum += centers[a][q];
        coarse[a].push_back(sum / (double)(e - s));
      }
      for (double x : centers[a]) wts[a].push_back(axis_weights(x, coarse[a], periodic[a], extent[a]));
    }
    int32_t nc[3] = {(int32_t)coarse[0].size(), (int32_t)coarse[1].size(), (int32_t)coarse[2].size()};
    Csr& P = lev.prolong;
    P.off.assign(1, 0);
    std::vector<std::pair<int32_t, double>> row;
    for (int32_t i = 0; i < lev.n; ++i) {
      int32_t q[3] = {i % n[0], i / n[0] % n[1], i / (n[0] * n[1])};
      row.clear();
      for (auto& zz : wts[2][q[2]])
        for (auto& yy : wts[1][q[1]])
          for (auto& xx : wts[0][q[0]])
            row.push_back({(zz.first * nc[1] + yy.first) * nc[0] + xx.first, xx.second * yy.second * zz.second});
      std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
      for (auto& e : row) {
        P.col.push_back(e.first);
        P.val.push_back(e.second);
      }
      P.off.push_back((int32_t)P.col.size());
    }
    int32_t ncells = nc[0] * nc[1] * nc[2];
    // Restriction = P^T, gathered per coarse row in ascending fine order.
    Csr& R = lev.restrict;
    R.off.assign(ncells + 1, 0);
    for (int32_t c : P.col) R.off[c + 1] += 1;
    for (int32_t j = 0; j < ncells; ++j) R.off[j + 1] += R.off[j];
    R.col.resize(P.col.size());
    R.val.resize(P.col.size());
    {
      std::vector<int32_t> fill(R.off.begin(), R.off.end() - 1);
      for (int32_t i = 0; i < lev.n; ++i)
        for (int32_t k = P.off[i]; k < P.off[i + 1]; ++k) {
          R.col[fill[P.col[k]]] = i;
          R.val[fill[P.col[k]]] = P.val[k];
          fill[P.col[k]] += 1;
        }
    }
    // Galerkin coarse operator from edge energies (multigrid.rs:379-429).
    std::map<std::pair<int32_t, int32_t>, double> off;
    std::vector<std::pair<int32_t, double>> delta;
    for (auto& e : edges) {
      delta.clear();
      int32_t a = P.off[e.i], ae = P.off[e.i + 1], b = P.off[e.j], be = P.off[e.j + 1];
      while (a < ae || b < be) {
        int32_t ca = a < ae ? P.col[a] : INT32_MAX, cb = b < be ? P.col[b] : INT32_MAX;
        int32_t col;
        double v;
        if (ca == cb) col = ca, v = P.val[a] - P.val[b], ++a, ++b;
        else if (ca < cb) col = ca, v = P.val[a], ++a;
        else col = cb, v = -P.val[b], ++b;
        if (v != 0.0) delta.push_back({col, v});
      }
      for (size_t s = 0; s < delta.size(); ++s)
        for (size_t t = s + 1; t < delta.size(); ++t)
          off.emplace(std::make_pair(delta[s].first, delta[t].first), 0.0).first->second +=
              e.w * delta[s].second * delta[t].second;
    }
    std::vector<double> ca(ncells, 0.0);
    for (int32_t i = 0; i < lev.n; ++i) {
      double w = anchors[i];
      if (w == 0.0) continue;
      for (int32_t s = P.off[i]; s < P.off[i + 1]; ++s) {
        ca[P.col[s]] += w * P.val[s];
        for (int32_t t = s + 1; t < P.off[i + 1]; ++t)
          off.emplace(std::make_pair(P.col[s], P.col[t]), 0.0).first->second += w * P.val[s] * P.val[t];
      }
    }
    std::vector<Edge> next;
    for (auto& kv : off)
      if (kv.second != 0.0) next.push_back({kv.first.first, kv.first.second, -kv.second});
    h.levels.push_back(std::move(lev));
    edges = std::move(next);
    anchors = std::move(ca);
    for (int a = 0; a < 3; ++a) {
      centers[a] = coarse[a];
      n[a] = nc[a];
    }
  }
  return 0;
}

static void finish_hierarchy(Hierarchy& h) {
  for (auto& l : h.levels) {
    Csr pattern = l.a;
    l.fwd = schedule(pattern, false);
    l.bwd = schedule(pattern, true);
    h.level_cells.push_back((uint64_t)l.n);
    h.level_nonzeros.push_back((uint64_t)l.a.val.size() + (uint64_t)l.n);
  }
}

int build_hierarchy(const HostGrid& g, const Poller& poll, Hierarchy& h) {
  if (g.n_components == 0) return CFDG_E034;
  bool any_solid = false;
  for (auto v : g.fluid) any_solid |= v == 0;
  int e = (any_solid || g.n_components != 1) ? build_masked(g, poll, h) : build_unmasked(g, poll, h);
  if (e) return e;
  finish_hierarchy(h);
  return 0;
}

int build_aggregation_hierarchy(const HostGrid& g, const Poller& poll, Hierarchy& h) {
  if (g.n_components == 0) return CFDG_E034;
  if (int e = build_masked(g, poll, h)) return e;
  finish_hierarchy(h);
  return 0;
}

bool Signature::operator==(const Signature& o) const {
  for (int a = 0; a < 3; ++a)
    if (n[a] != o.n[a] || spacing[a] != o.spacing[a]) return false;
  return anchored == o.anchored && fluid == o.fluid && kind == o.kind && lo == o.lo && hi == o.hi && wbits == o.wbits;
}

int signature_of(const HostGrid& g, Signature& s) {
  if (g.n_components == 0) return CFDG_E034;
  for (int a = 0; a < 3; ++a) {
    s.n[a] = g.n[a];
    std::memcpy(&s.spacing[a], &g.dx[a], 8);
  }
  s.anchored = g.anchored;
  s.fluid = g.fluid;
  s.kind.clear(), s.lo.clear(), s.hi.clear(), s.wbits.clear();
  for (int64_t f = 0; f < g.faces; ++f) {
    uint8_t k = g.face_kind[f];
    if (k != INTERIOR && k != OUTLET) continue;
    double w = g.weight(f);
    if (!std::isfinite(w) || w <= 0.0) return CFDG_E034;
    uint64_t bits;
    std::memcpy(&bits, &w, 8);
    s.kind.push_back(k == INTERIOR ? 1 : 2);
    s.lo.push_back(g.face_lo[f]);
    s.hi.push_back(g.face_hi[f]);
    s.wbits.push_back(bits);
  }
  return 0;
}

}  // namespace cfdg
