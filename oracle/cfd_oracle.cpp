// CPU oracle for the CFD-craft pressure projection.
//
// TEST INFRASTRUCTURE ONLY. This file is the parity checker and the timed CPU
// baseline. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
// reference legs load it; the GPU engine never links, calls or falls back to it.
//
// It restates, in plain C++17 compiled with -O2 -ffp-contract=off (Rust never
// contracts a*b+c into an FMA, so neither may this), the reference algorithms of
// crates/cfd-craft (CFD-craft 0.2.0) in their natural orders:
//   grid.rs:246-464      Grid::build (box masks, faces, cell_faces, BFS components)
//   grid.rs:612-691      divergence / gradient / enforce_velocity
//   case.rs:345-365      Flow::vector;  case.rs:438-446 Block::contains
//   geometry.rs:118-150  box raster (cell centre rule min <= c < max)
//   pressure.rs:118-241  IC(0) Factor::build / apply
//   pressure.rs:246-312  Operator (compact, face order) and public apply
//   pressure.rs:316-325  center_nullspaces
//   pressure.rs:342-436  solve_scaled (PCG, true-residual gate, E031/E032/E033)
//   pressure.rs:440-502  projection_rhs / project
//   multigrid.rs:24-726  unmasked geometric multigrid (Galerkin, V(2,2), dense Cholesky,
//                        semicoarsening of anisotropic grids)
//   multigrid/line.rs:26-201    line/plane block smoothers (banded Cholesky block GS)
//   multigrid/masked.rs:16-342  masked aggregation multigrid
//   flow.rs:426-525, solver.rs:671-732,879-960  laminar momentum RHS and SSPRK2 step
//   transport.rs:651-723, solver.rs:808-855     linear-upwind scalar step and budgets
// Parity is pinned by the reference's published known answers (iteration counts,
// residuals) and by its unit-test identities, re-run in tests/.
//
// Floating-point sums that Rust writes with Iterator::sum start from -0.0 (the
// identity of f64 addition used by Rust >= 1.81); explicit `let mut s = 0.0`
// accumulators start from +0.0. Both are kept as written in the reference.

#include <algorithm>
#include <array>
#include <tuple>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace oracle {

static const size_t NONE = SIZE_MAX;

enum Boundary { B_PERIODIC = 0, B_OPEN = 1, B_WALL = 2, B_SLIP = 3, B_GROUND_OPEN_TOP = 4 };
enum FlowKind { F_PRESCRIBED = 0, F_LAMINAR = 1, F_RANS = 2 };
enum FaceKind { K_INTERIOR = 0, K_WALL = 1, K_SLIP = 2, K_INLET = 3, K_OUTLET = 4, K_BLOCKED = 5 };

// Return codes shared with the GPU engine's C ABI.
enum Code {
  OK = 0, E031 = 31, E032 = 32, E033 = 33, E034 = 34, E035 = 35, E036 = 36,
  CANCELLED = 100, WALL_TIME = 101, UNSUPPORTED = 299
};

struct Flow {
  int kind = F_LAMINAR;
  double velocity[3] = {0, 0, 0};
  double speed = 0, ref_height = 1, roughness = 0.1, direction_deg = 0;
  // case.rs:345-365
  void vector(double z, double out[3]) const {
    if (kind != F_RANS) {
      for (int a = 0; a < 3; ++a) out[a] = velocity[a];
      return;
    }
    double u = speed * std::log((std::max(z, 0.0) + roughness) / roughness) /
               std::log((ref_height + roughness) / roughness);
    double t = direction_deg * (M_PI / 180.0);  // f64::to_radians
    out[0] = -u * std::sin(t);
    out[1] = -u * std::cos(t);
    out[2] = 0.0;
  }
};

struct Face {
  int axis;
  size_t coord[3];
  double center[3];
  size_t lo, hi;  // NONE when absent
  int kind;
  double area, distance;
};

struct Info {
  uint64_t iterations = 0;
  double relative_residual = 0;
  uint64_t work_units = 0, operator_applications = 0, preconditioner_applications = 0,
           true_residual_checks = 0;
  uint64_t hierarchy_builds = 0, hierarchy_levels = 0, hierarchy_cells = 0,
           hierarchy_nonzeros = 0, cycles = 0, smoothing_cell_updates = 0,
           residual_cell_updates = 0, restriction_cell_updates = 0,
           prolongation_cell_updates = 0, coarse_solves = 0;
  // Block (line/plane) smoothing of anisotropic levels (multigrid.rs:103-114, 677-718).
  uint64_t block_smoothing_cell_updates = 0, block_solves = 0, block_level_cell_visits = 0;
};

typedef int (*PollFn)(void*);
struct Control {
  PollFn poll = nullptr;
  void* ctx = nullptr;
  uint64_t polls = 0;
  int check() {
    ++polls;
    if (!poll) return OK;
    int r = poll(ctx);
    if (r == 1) return CANCELLED;
    if (r == 2) return WALL_TIME;
    return OK;
  }
};

static inline double rsum_init() { return -0.0; }  // Iterator::sum identity

// ---------------------------------------------------------------- multigrid data
typedef std::tuple<size_t, size_t, double> Edge;

// multigrid.rs:225-288
struct Matrix {
  std::vector<size_t> offsets, columns;
  std::vector<double> values, diagonal;
  static Matrix build(const std::vector<Edge>& edges, const std::vector<double>& anchors) {
    Matrix m;
    size_t n = anchors.size();
    m.offsets.assign(n + 1, 0);
    for (auto& e : edges) {
      m.offsets[std::get<0>(e) + 1] += 1;
      m.offsets[std::get<1>(e) + 1] += 1;
    }
    for (size_t i = 0; i < n; ++i) m.offsets[i + 1] += m.offsets[i];
    m.columns.assign(m.offsets[n], 0);
    m.values.assign(m.offsets[n], 0.0);
    std::vector<size_t> next(m.offsets.begin(), m.offsets.begin() + n);
    m.diagonal = anchors;
    for (auto& e : edges) {
      size_t i = std::get<0>(e), j = std::get<1>(e);
      double w = std::get<2>(e);
      size_t rc[2][2] = {{i, j}, {j, i}};
      for (auto& p : rc) {
        size_t row = p[0], col = p[1];
        m.diagonal[row] += w;
        size_t at = next[row];
        m.columns[at] = col;
        m.values[at] = -w;
        next[row] += 1;
      }
    }
    return m;
  }
  void product(const double* x, double* y, size_t n) const {
    for (size_t i = 0; i < n; ++i) {
      double value = diagonal[i] * x[i];
      for (size_t at = offsets[i]; at < offsets[i + 1]; ++at) value += values[at] * x[columns[at]];
      y[i] = value;
    }
  }
  void sweep(const double* rhs, double* x, size_t n, bool backward) const {
    for (size_t at = 0; at < n; ++at) {
      size_t i = backward ? n - 1 - at : at;
      double value = rhs[i];
      for (size_t e = offsets[i]; e < offsets[i + 1]; ++e) value -= values[e] * x[columns[e]];
      x[i] = value / diagonal[i];
    }
  }
};

// multigrid.rs:290-433
struct Transfer {
  std::vector<size_t> offsets, columns;
  std::vector<double> weights;
};

static std::vector<std::pair<size_t, double>> axis_weights(double x, const std::vector<double>& centers,
                                                           bool periodic, double extent) {
  size_t n = centers.size();
  if (n == 1) return {{0, 1.0}};
  size_t hi = std::partition_point(centers.begin(), centers.end(), [&](double v) { return v < x; }) -
              centers.begin();
  size_t lo_i, hi_i;
  double left, right;
  if (hi == 0) {
    if (!periodic) return {{0, 1.0}};
    lo_i = n - 1; hi_i = 0; left = centers[n - 1] - extent; right = centers[0];
  } else if (hi == n) {
    if (!periodic) return {{n - 1, 1.0}};
    lo_i = n - 1; hi_i = 0; left = centers[n - 1]; right = centers[0] + extent;
  } else {
    lo_i = hi - 1; hi_i = hi; left = centers[hi - 1]; right = centers[hi];
  }
  double t = (x - left) / (right - left);
  std::vector<std::pair<size_t, double>> out;
  if (1.0 - t != 0.0) out.push_back({lo_i, 1.0 - t});
  if (t != 0.0) out.push_back({hi_i, t});
  return out;
}

static size_t index3(const size_t n[3], size_t i, size_t j, size_t k) { return (k * n[1] + j) * n[0] + i; }

static Transfer transfer_build(const size_t n[3], const std::vector<double> centers[3],
                               const bool periodic[3], const double extent[3], const bool coarsen[3],
                               std::vector<double> coarse[3]) {
  for (int a = 0; a < 3; ++a) {
    coarse[a].clear();
    size_t step = coarsen[a] ? 2 : 1;
    for (size_t s = 0; s < centers[a].size(); s += step) {
      size_t e = std::min(s + step, centers[a].size());
      double sum = rsum_init();
      for (size_t q = s; q < e; ++q) sum += centers[a][q];
      coarse[a].push_back(sum / (double)(e - s));
    }
  }
  size_t nc[3] = {coarse[0].size(), coarse[1].size(), coarse[2].size()};
  std::vector<std::vector<std::pair<size_t, double>>> w[3];
  for (int a = 0; a < 3; ++a)
    for (double x : centers[a]) w[a].push_back(axis_weights(x, coarse[a], periodic[a], extent[a]));
  Transfer p;
  p.offsets.push_back(0);
  std::vector<std::pair<size_t, double>> row;
  size_t count = n[0] * n[1] * n[2];
  for (size_t i = 0; i < count; ++i) {
    size_t q[3] = {i % n[0], i / n[0] % n[1], i / (n[0] * n[1])};
    row.clear();
    for (auto& zz : w[2][q[2]])
      for (auto& yy : w[1][q[1]])
        for (auto& xx : w[0][q[0]])
          row.push_back({index3(nc, xx.first, yy.first, zz.first), xx.second * yy.second * zz.second});
    std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (auto& e : row) {
      p.columns.push_back(e.first);
      p.weights.push_back(e.second);
    }
    p.offsets.push_back(p.columns.size());
  }
  return p;
}

// multigrid.rs:379-429 (Galerkin P^T A P from edge energies, ordered map)
static void galerkin(const Transfer& t, const std::vector<Edge>& edges, const std::vector<double>& anchors,
                     size_t nc, std::vector<Edge>& out_edges, std::vector<double>& out_anchors) {
  std::map<std::pair<size_t, size_t>, double> off;
  std::vector<std::pair<size_t, double>> delta;
  for (auto& e : edges) {
    size_t i = std::get<0>(e), j = std::get<1>(e);
    double w = std::get<2>(e);
    delta.clear();
    size_t a = t.offsets[i], ae = t.offsets[i + 1], b = t.offsets[j], be = t.offsets[j + 1];
    while (a < ae || b < be) {
      size_t ca = a < ae ? t.columns[a] : SIZE_MAX;
      size_t cb = b < be ? t.columns[b] : SIZE_MAX;
      size_t col;
      double value;
      if (ca == cb) {
        col = ca; value = t.weights[a] - t.weights[b]; ++a; ++b;
      } else if (ca < cb) {
        col = ca; value = t.weights[a]; ++a;
      } else {
        col = cb; value = -t.weights[b]; ++b;
      }
      if (value != 0.0) delta.push_back({col, value});
    }
    for (size_t at = 0; at < delta.size(); ++at)
      for (size_t bt = at + 1; bt < delta.size(); ++bt) {
        auto it = off.emplace(std::make_pair(delta[at].first, delta[bt].first), 0.0).first;
        it->second += w * delta[at].second * delta[bt].second;
      }
  }
  out_anchors.assign(nc, 0.0);
  for (size_t i = 0; i < anchors.size(); ++i) {
    double w = anchors[i];
    if (w == 0.0) continue;
    delta.clear();
    for (size_t at = t.offsets[i]; at < t.offsets[i + 1]; ++at) delta.push_back({t.columns[at], t.weights[at]});
    for (size_t at = 0; at < delta.size(); ++at) {
      out_anchors[delta[at].first] += w * delta[at].second;
      for (size_t bt = at + 1; bt < delta.size(); ++bt) {
        auto it = off.emplace(std::make_pair(delta[at].first, delta[bt].first), 0.0).first;
        it->second += w * delta[at].second * delta[bt].second;
      }
    }
  }
  out_edges.clear();
  for (auto& kv : off)
    if (kv.second != 0.0) out_edges.push_back(Edge(kv.first.first, kv.first.second, -kv.second));
}

static void center_plain(double* x, size_t n, bool anchored) {
  if (anchored) return;
  double s = rsum_init();
  for (size_t i = 0; i < n; ++i) s += x[i];
  double mean = s / (double)n;
  for (size_t i = 0; i < n; ++i) x[i] -= mean;
}

// multigrid.rs:434-521
// multigrid/line.rs:26-201: exact line (or small plane) solves for block Gauss-Seidel.
// The blocks are the cells sharing their coordinates off `axes`; a periodic axis is folded
// (0, n-1, 1, n-2, ...) so its cycle has a narrow band. Each block holds a banded Cholesky
// factor with the diagonal replaced by its reciprocal; outside-block entries are kept as
// rows of (column, value) in block order.
struct BlockSmoother {
  std::vector<int> axes;
  size_t length = 0, bandwidth = 0;
  std::vector<size_t> nodes, outside_offsets, outside_columns;
  std::vector<double> outside_values, factor, scratch;

  int build(const Matrix& m, const size_t n[3], const std::vector<int>& ax, const bool periodic[3], Control& control) {
    axes = ax;
    const size_t count = m.diagonal.size();
    length = 1;
    for (int a : axes) length *= n[a];
    nodes.clear();
    nodes.reserve(count);
    for (size_t i = 0; i < count; ++i) {
      size_t q[3] = {i % n[0], i / n[0] % n[1], i / (n[0] * n[1])};
      bool skip = false;
      for (int a : axes) skip |= q[a] != 0;
      if (skip) continue;
      for (size_t at = 0; at < length; ++at) {
        size_t remainder = at;
        for (int axis : axes) {
          const size_t v = remainder % n[axis];
          remainder /= n[axis];
          q[axis] = !periodic[axis] ? v : (v % 2 == 0 ? v / 2 : n[axis] - 1 - v / 2);
        }
        nodes.push_back((q[2] * n[1] + q[1]) * n[0] + q[0]);
      }
    }
    std::vector<size_t> position(count, 0);
    for (size_t at = 0; at < nodes.size(); ++at) position[nodes[at]] = at;
    bandwidth = 0;
    for (size_t i = 0; i < count; ++i) {
      const size_t pi = position[i];
      for (size_t at = m.offsets[i]; at < m.offsets[i + 1]; ++at) {
        const size_t pj = position[m.columns[at]];
        if (pi / length == pj / length) bandwidth = std::max(bandwidth, pi > pj ? pi - pj : pj - pi);
      }
    }
    const size_t stride = bandwidth + 1;
    outside_offsets.assign(1, 0);
    outside_columns.clear();
    outside_values.clear();
    for (size_t at = 0; at < nodes.size(); ++at) {
      const size_t cell = nodes[at];
      for (size_t e = m.offsets[cell]; e < m.offsets[cell + 1]; ++e) {
        const size_t col = m.columns[e];
        if (position[col] / length != at / length) {
          outside_columns.push_back(col);
          outside_values.push_back(m.values[e]);
        }
      }
      outside_offsets.push_back(outside_columns.size());
    }
    factor.assign(count * stride, 0.0);
    for (size_t at = 0; at < nodes.size(); ++at) {
      const size_t cell = nodes[at];
      factor[at * stride] = m.diagonal[cell];
      for (size_t e = m.offsets[cell]; e < m.offsets[cell + 1]; ++e) {
        const size_t col = position[m.columns[e]];
        if (col / length == at / length && col < at) factor[at * stride + at - col] += m.values[e];
      }
    }
    for (size_t line = 0; line < count / length; ++line) {
      if (line % 128 == 0) {
        int c = control.check();
        if (c) return c;
      }
      const size_t base = line * length * stride;
      for (size_t i = 0; i < length; ++i)
        for (size_t j = i > bandwidth ? i - bandwidth : 0; j <= i; ++j) {
          const size_t row = base + i * stride, other = base + j * stride;
          double value = factor[row + i - j];
          for (size_t k = i > bandwidth ? i - bandwidth : 0; k < j; ++k)
            value -= factor[row + i - k] * factor[other + j - k];
          if (i == j) {
            if (!std::isfinite(value) || value <= 0.0) return E036;
            factor[row] = std::sqrt(value);
          } else {
            factor[row + i - j] = value / factor[other];
          }
        }
    }
    for (size_t row = 0; row < count; ++row) factor[row * stride] = 1.0 / factor[row * stride];
    scratch.assign(length, 0.0);
    return OK;
  }

  // line.rs:155-190
  void sweep(const double* rhs, double* x, bool backward) {
    const size_t count = nodes.size() / length, stride = bandwidth + 1;
    for (size_t at = 0; at < count; ++at) {
      const size_t line = backward ? count - 1 - at : at;
      const size_t start = line * length, base = start * stride;
      for (size_t i = 0; i < length; ++i) {
        double value = rhs[nodes[start + i]];
        for (size_t e = outside_offsets[start + i]; e < outside_offsets[start + i + 1]; ++e)
          value -= outside_values[e] * x[outside_columns[e]];
        scratch[i] = value;
      }
      for (size_t i = 0; i < length; ++i) {
        const size_t row = base + i * stride;
        double value = scratch[i];
        for (size_t j = i > bandwidth ? i - bandwidth : 0; j < i; ++j) value -= factor[row + i - j] * scratch[j];
        scratch[i] = value * factor[row];
      }
      for (size_t i = length; i-- > 0;) {
        double value = scratch[i];
        for (size_t j = i + 1; j < std::min(length, i + bandwidth + 1); ++j)
          value -= factor[base + j * stride + j - i] * scratch[j];
        scratch[i] = value * factor[base + i * stride];
      }
      for (size_t i = 0; i < length; ++i) x[nodes[start + i]] = scratch[i];
    }
  }
};

struct Level {
  Matrix matrix;
  Transfer transfer;
  std::vector<BlockSmoother> lines;  // anisotropic levels: replaces the point sweeps
  size_t dims[3] = {0, 0, 0};        // cells per axis of this level
  std::vector<double> rhs, x, residual, cholesky;
  bool anchored = true;
  bool terminal = false;
  int factor() {
    size_t skip = anchored ? 0 : 1;
    size_t n = x.size() - skip;
    std::vector<double> l(n * n, 0.0);
    for (size_t row = skip; row < x.size(); ++row) {
      size_t i = row - skip;
      l[i * n + i] = matrix.diagonal[row];
      for (size_t at = matrix.offsets[row]; at < matrix.offsets[row + 1]; ++at) {
        size_t col = matrix.columns[at];
        if (col >= skip) l[i * n + col - skip] += matrix.values[at];
      }
    }
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j <= i; ++j) {
        double value = l[i * n + j];
        for (size_t k = 0; k < j; ++k) value -= l[i * n + k] * l[j * n + k];
        if (i == j) {
          if (!std::isfinite(value) || value <= 0.0) return E035;
          l[i * n + j] = std::sqrt(value);
        } else {
          l[i * n + j] = value / l[j * n + j];
        }
      }
    cholesky = l;
    return OK;
  }
  void direct() {
    size_t skip = anchored ? 0 : 1;
    size_t n = x.size() - skip;
    std::fill(x.begin(), x.end(), 0.0);
    for (size_t i = 0; i < n; ++i) {
      double value = rhs[i + skip];
      for (size_t j = 0; j < i; ++j) value -= cholesky[i * n + j] * x[j + skip];
      x[i + skip] = value / cholesky[i * n + i];
    }
    for (size_t ii = n; ii-- > 0;) {
      double value = x[ii + skip];
      for (size_t j = ii + 1; j < n; ++j) value -= cholesky[j * n + ii] * x[j + skip];
      x[ii + skip] = value / cholesky[ii * n + ii];
    }
    center_plain(x.data(), x.size(), anchored);
  }
};

// masked.rs:15-70
struct Direct {
  std::vector<size_t> indices;
  std::vector<double> factor;
  int build(const Matrix& a, const std::vector<size_t>& component, bool anchored) {
    indices.assign(component.begin() + (anchored ? 0 : 1), component.end());
    size_t n = indices.size();
    std::map<size_t, size_t> local;
    for (size_t j = 0; j < n; ++j) local[indices[j]] = j;
    factor.assign(n * n, 0.0);
    for (size_t i = 0; i < n; ++i) {
      size_t row = indices[i];
      factor[i * n + i] = a.diagonal[row];
      for (size_t at = a.offsets[row]; at < a.offsets[row + 1]; ++at) {
        auto it = local.find(a.columns[at]);
        if (it != local.end()) factor[i * n + it->second] += a.values[at];
      }
    }
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j <= i; ++j) {
        double v = factor[i * n + j];
        for (size_t k = 0; k < j; ++k) v -= factor[i * n + k] * factor[j * n + k];
        if (i == j) {
          if (!std::isfinite(v) || v <= 0.0) return E035;
          factor[i * n + j] = std::sqrt(v);
        } else {
          factor[i * n + j] = v / factor[j * n + j];
        }
      }
    return OK;
  }
  void solve(const double* rhs, double* x) const {
    size_t n = indices.size();
    for (size_t i = 0; i < n; ++i) {
      size_t row = indices[i];
      double v = rhs[row];
      for (size_t j = 0; j < i; ++j) v -= factor[i * n + j] * x[indices[j]];
      x[row] = v / factor[i * n + i];
    }
    for (size_t i = n; i-- > 0;) {
      size_t row = indices[i];
      double v = x[row];
      for (size_t j = i + 1; j < n; ++j) v -= factor[j * n + i] * x[indices[j]];
      x[row] = v / factor[i * n + i];
    }
  }
};

static void center_components(double* x, const std::vector<std::vector<size_t>>& closed) {
  for (auto& cells : closed) {
    double s = rsum_init();
    for (size_t i : cells) s += x[i];
    double mean = s / (double)cells.size();
    for (size_t i : cells) x[i] -= mean;
  }
}

struct MaskedLevel {
  Matrix a;
  std::vector<size_t> parent;
  std::vector<std::vector<size_t>> closed;
  std::vector<double> rhs, x, residual;
  std::vector<Direct> direct;
  // masked.rs:158-172
  void sweep(bool backward) {
    size_t n = x.size();
    for (size_t at = 0; at < n; ++at) {
      size_t i = backward ? n - 1 - at : at;
      if (a.diagonal[i] == 0.0) {
        x[i] = 0.0;
        continue;
      }
      double v = rhs[i];
      for (size_t k = a.offsets[i]; k < a.offsets[i + 1]; ++k) v -= a.values[k] * x[a.columns[k]];
      x[i] = v / a.diagonal[i];
    }
  }
};

// ---------------------------------------------------------------- grid
struct Grid;
struct Hierarchy;
struct Factor {
  std::vector<size_t> row_offsets, columns;
  std::vector<double> lower, diagonal;
};

struct SigFace {
  uint8_t kind;
  size_t lo, hi;
  uint64_t wbits;
  bool operator==(const SigFace& o) const { return kind == o.kind && lo == o.lo && hi == o.hi && wbits == o.wbits; }
};
struct Signature {
  size_t n[3];
  std::vector<uint8_t> anchored, fluid;
  uint64_t spacing[3];
  std::vector<SigFace> faces;
};

struct Hierarchy {
  std::vector<Level> levels;                 // unmasked
  bool masked = false;
  std::vector<MaskedLevel> mlevels;          // masked
  std::vector<size_t> fluid_indices;
  std::vector<uint64_t> level_cells, level_nonzeros;
};

struct Grid {
  size_t n[3];
  double dx[3];
  double size_m[3];  // the case's domain size (ghost_values' boundary test)
  double volume;
  double viscosity = 1.5e-5;            // laminar kinematic viscosity (case flow)
  double acceleration[3] = {0, 0, 0};   // laminar body acceleration (case flow)
  int boundary[3];
  Flow flow;
  int preconditioner = 0;  // 0 ic0, 1 multigrid
  std::vector<uint8_t> fluid;
  std::vector<Face> faces;
  std::vector<std::array<size_t, 6>> cell_faces;  // [axis*2 + side]
  std::vector<size_t> component;
  std::vector<std::vector<size_t>> components;
  std::vector<uint8_t> anchored;
  size_t face_dims[3][3];
  size_t offsets[3];
  std::unique_ptr<Factor> factor;        // OnceLock: built by the first IC(0) solve
  std::unique_ptr<Hierarchy> hierarchy;  // rebuilt when the signature changes
  std::unique_ptr<Signature> signature;
  size_t count() const { return fluid.size(); }
};

static inline double face_weight(const Grid& g, const Face& f) { return f.area / (f.distance * g.volume); }

struct BoxDesc { double min[3], max[3]; };

// grid.rs:246-464 (boxes only: geometry.rs raster with the centre rule)
static int grid_build(Grid& g, const size_t n[3], const double size_m[3], const int boundary[3],
                      const Flow& flow, const std::vector<BoxDesc>& boxes, std::string& err) {
  for (int a = 0; a < 3; ++a) {
    g.n[a] = n[a];
    g.dx[a] = size_m[a] / (double)n[a];
    g.size_m[a] = size_m[a];
    g.boundary[a] = boundary[a];
  }
  g.flow = flow;
  g.volume = ((1.0 * g.dx[0]) * g.dx[1]) * g.dx[2];  // dx.iter().product()
  size_t count = n[0] * n[1] * n[2];
  g.fluid.assign(count, 1);
  g.cell_faces.assign(count, {NONE, NONE, NONE, NONE, NONE, NONE});
  g.component.assign(count, NONE);
  for (size_t bi = 0; bi < boxes.size(); ++bi) {
    const BoxDesc& b = boxes[bi];
    size_t lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      // geometry.rs:122-128 partition points of the centre rule
      size_t first = 0, end = 0;
      {
        size_t l = 0, h = n[a];
        while (l < h) {
          size_t mid = l + (h - l) / 2;
          double c = ((double)mid + 0.5) * g.dx[a];
          if (c < b.min[a] || std::isnan(b.min[a])) l = mid + 1; else h = mid;
        }
        first = l;
      }
      {
        size_t l = 0, h = n[a];
        while (l < h) {
          size_t mid = l + (h - l) / 2;
          double c = ((double)mid + 0.5) * g.dx[a];
          if (c < b.max[a]) l = mid + 1; else h = mid;
        }
        end = l;
      }
      lo[a] = first;
      hi[a] = std::max(end, first);
    }
    size_t cells = 0;
    for (size_t k = lo[2]; k < hi[2]; ++k)
      for (size_t j = lo[1]; j < hi[1]; ++j)
        for (size_t i = lo[0]; i < hi[0]; ++i) {
          g.fluid[index3(n, i, j, k)] = 0;
          ++cells;
        }
    if (cells == 0) {
      err = "CFD-E028: geometry[" + std::to_string(bi) + "] (box) contains no cell center";
      return 28;
    }
  }
  bool any = false;
  for (auto v : g.fluid) any |= v != 0;
  if (!any) {
    err = "CFD-E030: geometry contains no fluid cells";
    return 30;
  }
  for (int a = 0; a < 3; ++a) {
    g.offsets[a] = g.faces.size();
    for (int d = 0; d < 3; ++d) g.face_dims[a][d] = n[d];
    bool periodic = boundary[a] == B_PERIODIC;
    if (!periodic) g.face_dims[a][a] += 1;
    const size_t* dims = g.face_dims[a];
    for (size_t k = 0; k < dims[2]; ++k)
      for (size_t j = 0; j < dims[1]; ++j)
        for (size_t i = 0; i < dims[0]; ++i) {
          size_t q[3] = {i, j, k};
          size_t t = q[a];
          size_t lo0 = NONE, hi0 = NONE;
          if (t > 0) {
            size_t p[3] = {q[0], q[1], q[2]};
            p[a] -= 1;
            lo0 = index3(n, p[0], p[1], p[2]);
          } else if (periodic) {
            size_t p[3] = {q[0], q[1], q[2]};
            p[a] = n[a] - 1;
            lo0 = index3(n, p[0], p[1], p[2]);
          }
          if (t < n[a]) hi0 = index3(n, q[0], q[1], q[2]);
          size_t lo = (lo0 != NONE && g.fluid[lo0]) ? lo0 : NONE;
          size_t hi = (hi0 != NONE && g.fluid[hi0]) ? hi0 : NONE;
          double center[3];
          for (int d = 0; d < 3; ++d) center[d] = ((double)q[d] + (d == a ? 0.0 : 0.5)) * g.dx[d];
          int kind;
          if (lo != NONE && hi != NONE) kind = K_INTERIOR;
          else if (lo == NONE && hi == NONE) kind = K_BLOCKED;
          else if (lo0 != NONE && hi0 != NONE) kind = K_WALL;
          else {
            switch (boundary[a]) {
              case B_WALL: kind = K_WALL; break;
              case B_SLIP: kind = K_SLIP; break;
              case B_GROUND_OPEN_TOP: kind = t == 0 ? K_WALL : K_SLIP; break;
              case B_OPEN: {
                double normal = t == 0 ? -1.0 : 1.0;
                double vec[3];
                flow.vector(center[2], vec);
                double v = vec[a] * normal;
                kind = v < -1e-12 ? K_INLET : (v > 1e-12 ? K_OUTLET : K_SLIP);
                break;
              }
              default: kind = K_BLOCKED;
            }
          }
          size_t f = g.faces.size();
          if (lo != NONE) g.cell_faces[lo][a * 2 + 1] = f;
          if (hi != NONE) g.cell_faces[hi][a * 2 + 0] = f;
          Face face;
          face.axis = a;
          for (int d = 0; d < 3; ++d) {
            face.coord[d] = q[d];
            face.center[d] = center[d];
          }
          face.lo = lo;
          face.hi = hi;
          face.kind = kind;
          face.area = g.volume / g.dx[a];
          face.distance = kind == K_INTERIOR ? g.dx[a] : 0.5 * g.dx[a];
          g.faces.push_back(face);
        }
  }
  for (size_t start = 0; start < count; ++start) {
    if (!g.fluid[start] || g.component[start] != NONE) continue;
    size_t id = g.components.size();
    std::vector<size_t> members;
    std::deque<size_t> queue{start};
    g.component[start] = id;
    bool anchored = false;
    while (!queue.empty()) {
      size_t i = queue.front();
      queue.pop_front();
      members.push_back(i);
      for (int s = 0; s < 6; ++s) {
        const Face& f = g.faces[g.cell_faces[i][s]];
        anchored |= f.kind == K_OUTLET;
        if (f.kind != K_INTERIOR) continue;
        size_t j = f.lo == i ? f.hi : f.lo;
        if (g.component[j] == NONE) {
          g.component[j] = id;
          queue.push_back(j);
        }
      }
    }
    g.components.push_back(std::move(members));
    g.anchored.push_back(anchored ? 1 : 0);
  }
  return OK;
}

// ---------------------------------------------------------------- pressure.rs
// pressure.rs:118-222
static std::unique_ptr<Factor> factor_build(const Grid& g) {
  size_t N = g.count();
  auto F = std::make_unique<Factor>();
  std::vector<size_t>& row_offsets = F->row_offsets;
  row_offsets.assign(N + 1, 0);
  for (auto& f : g.faces)
    if (f.kind == K_INTERIOR && f.lo != f.hi) row_offsets[std::max(f.lo, f.hi) + 1] += 1;
  for (size_t row = 0; row < N; ++row) row_offsets[row + 1] += row_offsets[row];
  size_t capacity = row_offsets[N];
  std::vector<size_t>& columns = F->columns;
  std::vector<double>& lower = F->lower;
  columns.assign(capacity, 0);
  lower.assign(capacity, 0.0);
  std::vector<size_t> counts(N, 0);
  std::vector<double> diag(N, 0.0);
  for (auto& f : g.faces) {
    double w = face_weight(g, f);
    if (f.kind == K_INTERIOR) {
      if (f.lo == f.hi) continue;
      size_t i = f.lo, j = f.hi;
      diag[i] += w;
      diag[j] += w;
      size_t row = i > j ? i : j, col = i > j ? j : i;
      size_t start = row_offsets[row], end = start + counts[row];
      size_t found = NONE;
      for (size_t k = start; k < end; ++k)
        if (columns[k] == col) { found = k; break; }
      if (found != NONE) {
        lower[found] -= w;
      } else {
        columns[end] = col;
        lower[end] = -w;
        counts[row] += 1;
      }
    } else if (f.kind == K_OUTLET) {
      diag[f.lo != NONE ? f.lo : f.hi] += w;
    }
  }
  size_t write = 0, read = 0;
  for (size_t row = 0; row < N; ++row) {
    size_t next = row_offsets[row + 1];
    size_t end = read + counts[row];
    for (size_t offset = read + 1; offset < end; ++offset) {
      size_t column = columns[offset];
      double value = lower[offset];
      size_t at = offset;
      while (at > read && columns[at - 1] > column) {
        columns[at] = columns[at - 1];
        lower[at] = lower[at - 1];
        at -= 1;
      }
      columns[at] = column;
      lower[at] = value;
    }
    row_offsets[row] = write;
    for (size_t offset = read; offset < end; ++offset) {
      columns[write] = columns[offset];
      lower[write] = lower[offset];
      write += 1;
    }
    read = next;
  }
  row_offsets[N] = write;
  columns.resize(write);
  lower.resize(write);
  double maxdiag = 1.0;
  for (double d : diag) maxdiag = std::fmax(maxdiag, d);
  for (size_t row = 0; row < N; ++row) {
    size_t start = row_offsets[row], end = row_offsets[row + 1];
    for (size_t offset = start; offset < end; ++offset) {
      size_t col = columns[offset];
      double dot = 0.0;
      size_t other = row_offsets[col], other_end = row_offsets[col + 1];
      for (size_t previous = start; previous < offset; ++previous) {
        size_t k = columns[previous];
        while (other < other_end && columns[other] < k) other += 1;
        if (other < other_end && columns[other] == k) dot += lower[previous] * lower[other];
      }
      lower[offset] = (lower[offset] - dot) / diag[col];
    }
    double squared = rsum_init();
    for (size_t o = start; o < end; ++o) squared += lower[o] * lower[o];
    diag[row] = std::sqrt(std::fmax(diag[row] + 1e-6 * maxdiag - squared, 1e-12 * maxdiag));
  }
  F->diagonal = diag;
  return F;
}

// pressure.rs:223-241
static void factor_apply(const Factor& F, const double* r, double* z, size_t N) {
  for (size_t i = 0; i < N; ++i) {
    double value = r[i];
    for (size_t k = F.row_offsets[i]; k < F.row_offsets[i + 1]; ++k) value -= F.lower[k] * z[F.columns[k]];
    z[i] = value / F.diagonal[i];
  }
  for (size_t i = N; i-- > 0;) {
    double value = z[i] / F.diagonal[i];
    z[i] = value;
    for (size_t k = F.row_offsets[i]; k < F.row_offsets[i + 1]; ++k) z[F.columns[k]] -= F.lower[k] * value;
  }
}

// pressure.rs:246-286: entries in face order, interior and outlet interleaved
struct Entry { bool interior; size_t lo, hi; double w; };
struct Operator {
  std::vector<Entry> entries;
  static Operator build(const Grid& g) {
    Operator op;
    op.entries.reserve(g.faces.size());
    for (auto& f : g.faces) {
      double w = face_weight(g, f);
      if (f.kind == K_INTERIOR) op.entries.push_back({true, f.lo, f.hi, w});
      else if (f.kind == K_OUTLET) op.entries.push_back({false, f.lo != NONE ? f.lo : f.hi, 0, w});
    }
    return op;
  }
  void apply(const double* x, double* y, size_t N) const {
    std::fill(y, y + N, 0.0);
    for (auto& e : entries) {
      if (e.interior) {
        double d = e.w * (x[e.lo] - x[e.hi]);
        y[e.lo] += d;
        y[e.hi] -= d;
      } else {
        y[e.lo] += e.w * x[e.lo];
      }
    }
  }
};

// pressure.rs:293-312
static void public_apply(const Grid& g, const double* x, double* y) {
  std::fill(y, y + g.count(), 0.0);
  for (auto& f : g.faces) {
    double w = face_weight(g, f);
    if (f.kind == K_INTERIOR) {
      double d = w * (x[f.lo] - x[f.hi]);
      y[f.lo] += d;
      y[f.hi] -= d;
    } else if (f.kind == K_OUTLET) {
      size_t i = f.lo != NONE ? f.lo : f.hi;
      y[i] += w * x[i];
    }
  }
}

// pressure.rs:316-325
static void center_nullspaces(const Grid& g, double* x) {
  for (size_t id = 0; id < g.components.size(); ++id) {
    if (g.anchored[id]) continue;
    const auto& m = g.components[id];
    double s = rsum_init();
    for (size_t i : m) s += x[i];
    double mean = s / (double)m.size();
    for (size_t i : m) x[i] -= mean;
  }
}

// ---------------------------------------------------------------- multigrid build
static std::vector<int> line_axes(const size_t n[3], const double dx[3]) {
  double w[3];
  for (int a = 0; a < 3; ++a) w[a] = 1.0 / (dx[a] * dx[a]);
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(w[a]) || w[a] <= 0.0) return {};
  double minimum = INFINITY;
  for (int a = 0; a < 3; ++a)
    if (n[a] > 2) minimum = std::fmin(minimum, w[a]);
  double maximum = 0.0;
  for (int a = 0; a < 3; ++a) maximum = std::fmax(maximum, w[a]);
  if (maximum / minimum <= 25.0) return {};
  std::vector<int> out;
  for (int a = 0; a < 3; ++a)
    if (w[a] >= maximum / 4.0) out.push_back(a);
  return out;
}

// masked.rs:90-126
static int mcomponents(const Matrix& a, const std::vector<double>& anchors, Control& control,
                       std::vector<std::vector<size_t>>& result, std::vector<uint8_t>& anchored) {
  std::vector<uint8_t> seen(anchors.size(), 0);
  for (size_t start = 0; start < seen.size(); ++start) {
    if (start % 1024 == 0) {
      int c = control.check();
      if (c) return c;
    }
    if (seen[start]) continue;
    seen[start] = 1;
    std::deque<size_t> queue{start};
    std::vector<size_t> cells;
    bool fixed = false;
    while (!queue.empty()) {
      size_t i = queue.front();
      queue.pop_front();
      if (cells.size() % 1024 == 0) {
        int c = control.check();
        if (c) return c;
      }
      cells.push_back(i);
      fixed |= anchors[i] > 0.0;
      for (size_t k = a.offsets[i]; k < a.offsets[i + 1]; ++k) {
        size_t j = a.columns[k];
        if (!seen[j]) {
          seen[j] = 1;
          queue.push_back(j);
        }
      }
    }
    result.push_back(std::move(cells));
    anchored.push_back(fixed ? 1 : 0);
  }
  return OK;
}

typedef std::array<size_t, 3> C3;
// masked.rs:127-156
static int maggregate(const Matrix& a, const std::vector<C3>& coords, Control& control,
                      std::vector<size_t>& parent, std::vector<C3>& coarse) {
  std::vector<C3> bins(coords.size());
  for (size_t i = 0; i < coords.size(); ++i) bins[i] = {coords[i][0] / 2, coords[i][1] / 2, coords[i][2] / 2};
  parent.assign(coords.size(), NONE);
  coarse.clear();
  for (size_t start = 0; start < parent.size(); ++start) {
    if (start % 1024 == 0) {
      int c = control.check();
      if (c) return c;
    }
    if (parent[start] != NONE) continue;
    size_t id = coarse.size();
    coarse.push_back(bins[start]);
    parent[start] = id;
    std::deque<size_t> queue{start};
    while (!queue.empty()) {
      size_t i = queue.front();
      queue.pop_front();
      for (size_t k = a.offsets[i]; k < a.offsets[i + 1]; ++k) {
        size_t j = a.columns[k];
        if (parent[j] == NONE && bins[j] == bins[start]) {
          parent[j] = id;
          queue.push_back(j);
        }
      }
    }
  }
  return OK;
}

// masked.rs:181-291
static int masked_build(const Grid& g, Control& control, Hierarchy& h) {
  h.masked = true;
  size_t N = g.count();
  std::vector<size_t> compact(N, NONE);
  for (size_t i = 0; i < N; ++i)
    if (g.fluid[i]) {
      compact[i] = h.fluid_indices.size();
      h.fluid_indices.push_back(i);
    }
  std::vector<C3> coords;
  for (size_t i : h.fluid_indices) coords.push_back({i % g.n[0], i / g.n[0] % g.n[1], i / (g.n[0] * g.n[1])});
  std::vector<double> anchors(coords.size(), 0.0);
  std::vector<Edge> edges;
  for (auto& f : g.faces) {
    double w = face_weight(g, f);
    if (f.kind == K_INTERIOR && f.lo != f.hi) edges.push_back(Edge(compact[f.lo], compact[f.hi], w));
    else if (f.kind == K_OUTLET) anchors[compact[f.lo != NONE ? f.lo : f.hi]] += w;
  }
  for (;;) {
    int c = control.check();
    if (c) return c;
    MaskedLevel level;
    level.a = Matrix::build(edges, anchors);
    std::vector<std::vector<size_t>> regions;
    std::vector<uint8_t> anchored;
    c = mcomponents(level.a, anchors, control, regions, anchored);
    if (c) return c;
    for (size_t r = 0; r < regions.size(); ++r)
      if (!anchored[r]) level.closed.push_back(regions[r]);
    size_t n = coords.size();
    level.rhs.assign(n, 0.0);
    level.x.assign(n, 0.0);
    level.residual.assign(n, 0.0);
    bool small = true;
    for (auto& r : regions) small &= r.size() <= 32;
    if (small) {
      for (size_t r = 0; r < regions.size(); ++r) {
        Direct d;
        int e = d.build(level.a, regions[r], anchored[r] != 0);
        if (e) return e;
        level.direct.push_back(std::move(d));
      }
      h.mlevels.push_back(std::move(level));
      break;
    }
    std::vector<size_t> parent;
    std::vector<C3> coarse;
    c = maggregate(level.a, coords, control, parent, coarse);
    if (c) return c;
    if (coarse.size() == n) {
      bool all0 = true;
      for (auto& p : coords) {
        p = {p[0] / 2, p[1] / 2, p[2] / 2};
        all0 &= p[0] == 0 && p[1] == 0 && p[2] == 0;
      }
      if (all0) return E035;
      continue;
    }
    std::map<std::pair<size_t, size_t>, double> sums;
    for (auto& e : edges) {
      size_t i = parent[std::get<0>(e)], j = parent[std::get<1>(e)];
      if (i != j) sums[{std::min(i, j), std::max(i, j)}] += std::get<2>(e);
    }
    edges.clear();
    for (auto& kv : sums) edges.push_back(Edge(kv.first.first, kv.first.second, kv.second));
    std::vector<double> ac(coarse.size(), 0.0);
    for (size_t i = 0; i < anchors.size(); ++i) ac[parent[i]] += anchors[i];
    anchors = ac;
    coords = coarse;
    level.parent = parent;
    h.mlevels.push_back(std::move(level));
  }
  for (auto& l : h.mlevels) {
    h.level_cells.push_back(l.x.size());
    h.level_nonzeros.push_back(l.a.values.size() + l.x.size());
  }
  return OK;
}

// multigrid.rs:530-645, with the line/plane block smoothers of anisotropic grids (:573-607)
static int hierarchy_build(const Grid& g, Control& control, Hierarchy& h) {
  bool any_solid = false;
  for (auto v : g.fluid) any_solid |= !v;
  if (any_solid || g.components.size() != 1) return masked_build(g, control, h);
  size_t n[3] = {g.n[0], g.n[1], g.n[2]};
  const std::vector<int> axes = line_axes(g.n, g.dx);
  std::vector<double> centers[3];
  for (int a = 0; a < 3; ++a)
    for (size_t i = 0; i < n[a]; ++i) centers[a].push_back((double)i + 0.5);
  double extent[3] = {(double)n[0], (double)n[1], (double)n[2]};
  bool periodic[3];
  for (int a = 0; a < 3; ++a) {
    periodic[a] = false;
    for (auto& f : g.faces)
      if (f.axis == a && f.coord[a] == 0 && f.kind == K_INTERIOR) { periodic[a] = true; break; }
  }
  bool anchored = g.anchored[0] != 0;
  std::vector<double> anchors(g.count(), 0.0);
  std::vector<Edge> edges;
  for (auto& f : g.faces) {
    double w = face_weight(g, f);
    if (f.kind == K_INTERIOR) edges.push_back(Edge(f.lo, f.hi, w));
    else if (f.kind == K_OUTLET) anchors[f.lo != NONE ? f.lo : f.hi] += w;
  }
  for (;;) {
    int c = control.check();
    if (c) return c;
    Level level;
    level.matrix = Matrix::build(edges, anchors);
    level.anchored = anchored;
    for (int a = 0; a < 3; ++a) level.dims[a] = n[a];
    size_t cnt = anchors.size();
    level.rhs.assign(cnt, 0.0);
    level.x.assign(cnt, 0.0);
    level.residual.assign(cnt, 0.0);
    if (cnt <= 32) {
      level.terminal = true;
      int e = level.factor();
      if (e) return e;
      h.levels.push_back(std::move(level));
      break;
    }
    bool coarsen[3] = {n[0] > 2, n[1] > 2, n[2] > 2};
    if (!axes.empty()) {
      // Weak-axis modes are kept until the stiff directions have collapsed (:575-581).
      bool stiff_can_coarsen = false;
      for (int a : axes) stiff_can_coarsen |= n[a] > 2;
      for (int a = 0; a < 3; ++a) {
        const bool in_axes = std::find(axes.begin(), axes.end(), a) != axes.end();
        coarsen[a] = n[a] > 2 && (!stiff_can_coarsen || in_axes);
      }
    }
    std::vector<double> coarse[3];
    level.transfer = transfer_build(n, centers, periodic, extent, coarsen, coarse);
    // :584-599: one plane block over all stiff axes when it holds at most 16 cells, else
    // lines along the stiff axis of smallest spacing (the first of equals).
    std::vector<std::vector<int>> groups;
    if (!axes.empty()) {
      size_t plane = 1;
      for (int a : axes) plane *= n[a];
      if (axes.size() > 1 && plane <= 16) {
        groups.push_back(axes);
      } else {
        int best = axes[0];
        for (int a : axes)
          if (g.dx[a] < g.dx[best]) best = a;
        groups.push_back({best});
      }
    }
    for (auto& grp : groups) {
      BlockSmoother b;
      int e = b.build(level.matrix, n, grp, periodic, control);
      if (e) return e;
      level.lines.push_back(std::move(b));
    }
    for (int a = 0; a < 3; ++a) n[a] = coarse[a].size();
    std::vector<Edge> ce;
    std::vector<double> ca;
    galerkin(level.transfer, edges, anchors, n[0] * n[1] * n[2], ce, ca);
    edges = ce;
    for (int a = 0; a < 3; ++a) centers[a] = coarse[a];
    h.levels.push_back(std::move(level));
    anchors = ca;
  }
  for (auto& l : h.levels) {
    h.level_cells.push_back(l.x.size());
    h.level_nonzeros.push_back(l.matrix.values.size() + l.x.size());
  }
  return OK;
}

// multigrid.rs:667-726
static void cycle(std::vector<Level>& levels, size_t at, Info& w) {
  Level& level = levels[at];
  center_plain(level.rhs.data(), level.rhs.size(), level.anchored);
  if (at + 1 == levels.size()) {
    level.direct();
    w.coarse_solves += 1;
    return;
  }
  size_t n = level.x.size();
  std::fill(level.x.begin(), level.x.end(), 0.0);
  const int sweeps = level.lines.empty() ? 2 : 1;
  if (!level.lines.empty()) w.block_level_cell_visits += n;
  for (int pass = 0; pass < sweeps; ++pass) {
    if (level.lines.empty()) {
      level.matrix.sweep(level.rhs.data(), level.x.data(), n, false);
    } else {
      BlockSmoother& b = level.lines[pass % level.lines.size()];
      b.sweep(level.rhs.data(), level.x.data(), false);
      w.block_solves += b.nodes.size() / b.length;
      w.block_smoothing_cell_updates += n;
    }
  }
  center_plain(level.x.data(), n, level.anchored);
  level.matrix.product(level.x.data(), level.residual.data(), n);
  for (size_t i = 0; i < n; ++i) level.residual[i] = level.rhs[i] - level.residual[i];
  center_plain(level.residual.data(), n, level.anchored);
  Level& next = levels[at + 1];
  std::fill(next.rhs.begin(), next.rhs.end(), 0.0);
  for (size_t i = 0; i < n; ++i) {
    double r = level.residual[i];
    for (size_t k = level.transfer.offsets[i]; k < level.transfer.offsets[i + 1]; ++k)
      next.rhs[level.transfer.columns[k]] += level.transfer.weights[k] * r;
  }
  cycle(levels, at + 1, w);
  for (size_t i = 0; i < n; ++i) {
    double s = rsum_init();
    for (size_t k = level.transfer.offsets[i]; k < level.transfer.offsets[i + 1]; ++k)
      s += level.transfer.weights[k] * next.x[level.transfer.columns[k]];
    level.x[i] += s;
  }
  for (int pass = 0; pass < sweeps; ++pass) {
    if (level.lines.empty()) {
      level.matrix.sweep(level.rhs.data(), level.x.data(), n, true);
    } else {
      BlockSmoother& b = level.lines[(sweeps - 1 - pass) % level.lines.size()];
      b.sweep(level.rhs.data(), level.x.data(), true);
      w.block_solves += b.nodes.size() / b.length;
      w.block_smoothing_cell_updates += n;
    }
  }
  center_plain(level.x.data(), n, level.anchored);
  w.smoothing_cell_updates += 2 * sweeps * n;
  w.residual_cell_updates += n;
  w.restriction_cell_updates += n;
  w.prolongation_cell_updates += n;
}

// masked.rs:304-342
static void mcycle(std::vector<MaskedLevel>& levels, size_t at, Info& w) {
  MaskedLevel& level = levels[at];
  center_components(level.rhs.data(), level.closed);
  std::fill(level.x.begin(), level.x.end(), 0.0);
  if (at + 1 == levels.size()) {
    for (auto& d : level.direct) d.solve(level.rhs.data(), level.x.data());
    center_components(level.x.data(), level.closed);
    w.coarse_solves += 1;
    return;
  }
  size_t n = level.x.size();
  for (int s = 0; s < 2; ++s) level.sweep(false);
  center_components(level.x.data(), level.closed);
  level.a.product(level.x.data(), level.residual.data(), n);
  for (size_t i = 0; i < n; ++i) level.residual[i] = level.rhs[i] - level.residual[i];
  center_components(level.residual.data(), level.closed);
  MaskedLevel& next = levels[at + 1];
  std::fill(next.rhs.begin(), next.rhs.end(), 0.0);
  for (size_t i = 0; i < n; ++i) next.rhs[level.parent[i]] += level.residual[i];
  mcycle(levels, at + 1, w);
  for (size_t i = 0; i < n; ++i) level.x[i] += next.x[level.parent[i]];
  for (int s = 0; s < 2; ++s) level.sweep(true);
  center_components(level.x.data(), level.closed);
  w.smoothing_cell_updates += 4 * n;
  w.residual_cell_updates += n;
  w.restriction_cell_updates += n;
  w.prolongation_cell_updates += n;
}

static void hierarchy_apply(Hierarchy& h, const double* rhs, double* z, size_t N, Info& w) {
  if (h.masked) {
    auto& l0 = h.mlevels[0];
    for (size_t j = 0; j < h.fluid_indices.size(); ++j) l0.rhs[j] = rhs[h.fluid_indices[j]];
    mcycle(h.mlevels, 0, w);
    std::fill(z, z + N, 0.0);
    for (size_t j = 0; j < h.fluid_indices.size(); ++j) z[h.fluid_indices[j]] = l0.x[j];
  } else {
    std::copy(rhs, rhs + N, h.levels[0].rhs.begin());
    cycle(h.levels, 0, w);
    std::copy(h.levels[0].x.begin(), h.levels[0].x.end(), z);
  }
  w.cycles += 1;
}

// multigrid.rs:158-222
static int signature_of(const Grid& g, Signature& s) {
  if (g.components.empty()) return E034;
  for (int a = 0; a < 3; ++a) {
    s.n[a] = g.n[a];
    std::memcpy(&s.spacing[a], &g.dx[a], 8);
  }
  s.anchored = g.anchored;
  s.fluid = g.fluid;
  s.faces.clear();
  for (auto& f : g.faces) {
    uint8_t kind;
    if (f.kind == K_INTERIOR) kind = 1;
    else if (f.kind == K_OUTLET) kind = 2;
    else continue;
    double w = face_weight(g, f);
    if (!std::isfinite(w) || w <= 0.0) return E034;
    uint64_t bits;
    std::memcpy(&bits, &w, 8);
    s.faces.push_back({kind, f.lo, f.hi, bits});
  }
  return OK;
}
static bool signature_matches(const Signature& a, const Signature& b) {
  for (int d = 0; d < 3; ++d)
    if (a.n[d] != b.n[d] || a.spacing[d] != b.spacing[d]) return false;
  return a.anchored == b.anchored && a.fluid == b.fluid && a.faces == b.faces;
}

// pressure.rs:55-97 (returns the hierarchy to apply, building or reusing it)
static int prepare_multigrid(Grid& g, Control& control, Info& info) {
  int c = control.check();
  if (c) return c;
  if (g.components.empty()) return E034;
  Signature s;
  bool built = !g.hierarchy || !g.signature;
  if (!built) {
    Signature cur;
    int e = signature_of(g, cur);
    if (e) built = true;
    else built = !signature_matches(*g.signature, cur);
  }
  if (built) {
    int e = signature_of(g, s);
    if (e) return e;
    info.hierarchy_builds = 1;
    auto h = std::make_unique<Hierarchy>();
    e = hierarchy_build(g, control, *h);
    if (e) return e;
    g.hierarchy = std::move(h);
    g.signature = std::make_unique<Signature>(std::move(s));
  }
  info.hierarchy_levels = g.hierarchy->level_cells.size();
  uint64_t cells = 0, nz = 0;
  for (auto v : g.hierarchy->level_cells) cells += v;
  for (auto v : g.hierarchy->level_nonzeros) nz += v;
  info.hierarchy_cells = cells;
  info.hierarchy_nonzeros = nz;
  return OK;
}

static double dotv(const std::vector<double>& x, const std::vector<double>& y) {
  double s = rsum_init();
  for (size_t i = 0; i < x.size(); ++i) s += x[i] * y[i];
  return s;
}

// pressure.rs:342-436
static int solve_scaled(Grid& g, const double* b, const double* scale_terms, double tol, uint64_t max,
                        Control& control, std::vector<double>& x, Info& info) {
  size_t N = g.count();
  for (size_t id = 0; id < g.components.size(); ++id) {
    if (g.anchored[id]) continue;
    double sum = rsum_init(), scale = rsum_init();
    for (size_t i : g.components[id]) sum += b[i];
    for (size_t i : g.components[id]) scale += std::fmax(std::fabs(b[i]), scale_terms ? scale_terms[i] : 0.0);
    if (std::fabs(sum) > 1e-9 * scale) return E031;
  }
  bool mg = g.preconditioner == 1;
  if (mg) {
    int c = prepare_multigrid(g, control, info);
    if (c) return c;
  } else if (!g.factor) {
    g.factor = factor_build(g);
  }
  auto precondition = [&](const std::vector<double>& r, std::vector<double>& z) {
    if (mg) hierarchy_apply(*g.hierarchy, r.data(), z.data(), N, info);
    else factor_apply(*g.factor, r.data(), z.data(), N);
    info.preconditioner_applications += 1;
  };
  x.assign(N, 0.0);
  std::vector<double> r(b, b + N);
  center_nullspaces(g, r.data());
  std::vector<double> compatible_b = r;
  double norm = std::sqrt(dotv(r, r));
  if (norm < 1e-24) {
    info.iterations = 0;
    info.relative_residual = 0.0;
    return OK;
  }
  std::vector<double> z(N, 0.0);
  precondition(r, z);
  center_nullspaces(g, z.data());
  std::vector<double> p = z;
  double rz = dotv(r, z);
  std::vector<double> ap(N, 0.0);
  Operator op = Operator::build(g);
  for (uint64_t it = 0; it < max; ++it) {
    if (it % 8 == 0) {
      int c = control.check();
      if (c) return c;
    }
    info.work_units += 1;
    op.apply(p.data(), ap.data(), N);
    info.operator_applications += 1;
    double denom = dotv(p, ap);
    if (denom <= 0.0 || !std::isfinite(denom)) return E032;
    double alpha = rz / denom;
    for (size_t i = 0; i < N; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * ap[i];
    }
    double rel = std::sqrt(dotv(r, r)) / norm;
    if (rel <= tol) {
      public_apply(g, x.data(), ap.data());
      info.operator_applications += 1;
      info.true_residual_checks += 1;
      double s = rsum_init();
      for (size_t i = 0; i < N; ++i) {
        double d = ap[i] - compatible_b[i];
        s += d * d;
      }
      double true_rel = std::sqrt(s) / norm;
      if (true_rel <= tol * 10.0 + 1e-12) {
        center_nullspaces(g, x.data());
        info.iterations = it + 1;
        info.relative_residual = true_rel;
        return OK;
      }
    }
    precondition(r, z);
    center_nullspaces(g, z.data());
    double next = dotv(r, z);
    double beta = next / rz;
    for (size_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
    rz = next;
  }
  return E033;
}

// pressure.rs:440-459
static void projection_rhs(const Grid& g, const double* u, double dt, double* b, double* terms) {
  for (size_t i = 0; i < g.count(); ++i) {
    b[i] = -0.0;
    terms[i] = 0.0;
    if (!g.fluid[i]) continue;
    double divergence = 0.0, scale = 0.0;
    for (int a = 0; a < 3; ++a) {
      size_t lo = g.cell_faces[i][a * 2], hi = g.cell_faces[i][a * 2 + 1];
      divergence += (u[hi] - u[lo]) / g.dx[a];
      scale += (std::fabs(u[lo]) + std::fabs(u[hi])) / g.dx[a];
    }
    b[i] = -divergence / dt;
    terms[i] = scale / dt;
  }
}

// pressure.rs:469-502
static int project(Grid& g, double* u, double* p, double dt, double tol, uint64_t max, Control& control,
                   Info& info) {
  size_t N = g.count();
  std::vector<double> b(N), terms(N), correction;
  projection_rhs(g, u, dt, b.data(), terms.data());
  int c = solve_scaled(g, b.data(), terms.data(), tol, max, control, correction, info);
  if (c) return c;
  for (size_t fi = 0; fi < g.faces.size(); ++fi) {
    const Face& f = g.faces[fi];
    double d;
    if (f.kind == K_INTERIOR) d = (correction[f.hi] - correction[f.lo]) / f.distance;
    else if (f.kind == K_OUTLET) d = f.lo != NONE ? -correction[f.lo] / f.distance : correction[f.hi] / f.distance;
    else d = 0.0;
    u[fi] -= dt * d;
  }
  for (size_t i = 0; i < N; ++i) p[i] += correction[i];
  center_nullspaces(g, p);
  return OK;
}

}  // namespace oracle

// ---------------------------------------------------------------- C ABI for ctypes
using namespace oracle;

extern "C" {

typedef struct {
  int32_t n[3];
  double size_m[3];
  int32_t boundary[3];     // 0 periodic, 1 open, 2 wall, 3 slip, 4 ground_open_top
  int32_t flow_kind;       // 0 prescribed_uniform, 1 laminar, 2 neutral_rans
  double velocity[3];
  double speed_m_s, reference_height_m, roughness_m, direction_deg_from;
  int32_t n_boxes;
  const double* boxes;     // n_boxes * 6: min xyz, max xyz
  int32_t preconditioner;  // 0 ic0, 1 multigrid
} ora_case;

typedef struct {
  uint64_t iterations;
  double relative_residual;
  uint64_t work_units, operator_applications, preconditioner_applications, true_residual_checks;
  uint64_t hierarchy_builds, hierarchy_levels, hierarchy_cells, hierarchy_nonzeros, cycles,
      smoothing_cell_updates, residual_cell_updates, restriction_cell_updates,
      prolongation_cell_updates, coarse_solves;
  uint64_t polls;
  uint64_t block_smoothing_cell_updates, block_solves, block_level_cell_visits;
} ora_info;

static void fill_info(const Info& in, uint64_t polls, ora_info* out) {
  if (!out) return;
  out->iterations = in.iterations;
  out->relative_residual = in.relative_residual;
  out->work_units = in.work_units;
  out->operator_applications = in.operator_applications;
  out->preconditioner_applications = in.preconditioner_applications;
  out->true_residual_checks = in.true_residual_checks;
  out->hierarchy_builds = in.hierarchy_builds;
  out->hierarchy_levels = in.hierarchy_levels;
  out->hierarchy_cells = in.hierarchy_cells;
  out->hierarchy_nonzeros = in.hierarchy_nonzeros;
  out->cycles = in.cycles;
  out->smoothing_cell_updates = in.smoothing_cell_updates;
  out->residual_cell_updates = in.residual_cell_updates;
  out->restriction_cell_updates = in.restriction_cell_updates;
  out->prolongation_cell_updates = in.prolongation_cell_updates;
  out->coarse_solves = in.coarse_solves;
  out->polls = polls;
  out->block_smoothing_cell_updates = in.block_smoothing_cell_updates;
  out->block_solves = in.block_solves;
  out->block_level_cell_visits = in.block_level_cell_visits;
}

void* ora_grid_build(const ora_case* c, char* err, size_t cap) {
  auto g = new Grid();
  size_t n[3] = {(size_t)c->n[0], (size_t)c->n[1], (size_t)c->n[2]};
  Flow flow;
  flow.kind = c->flow_kind;
  for (int a = 0; a < 3; ++a) flow.velocity[a] = c->velocity[a];
  flow.speed = c->speed_m_s;
  flow.ref_height = c->reference_height_m;
  flow.roughness = c->roughness_m;
  flow.direction_deg = c->direction_deg_from;
  std::vector<BoxDesc> boxes(c->n_boxes);
  for (int b = 0; b < c->n_boxes; ++b)
    for (int a = 0; a < 3; ++a) {
      boxes[b].min[a] = c->boxes[b * 6 + a];
      boxes[b].max[a] = c->boxes[b * 6 + 3 + a];
    }
  int bnd[3] = {c->boundary[0], c->boundary[1], c->boundary[2]};
  std::string e;
  int code = grid_build(*g, n, c->size_m, bnd, flow, boxes, e);
  if (code) {
    if (err && cap) snprintf(err, cap, "%s", e.c_str());
    delete g;
    return nullptr;
  }
  g->preconditioner = c->preconditioner;
  return g;
}
void ora_grid_free(void* g) { delete (Grid*)g; }
void ora_grid_set_preconditioner(void* g, int32_t p) { ((Grid*)g)->preconditioner = p; }
void ora_grid_counts(void* gp, int64_t* cells, int64_t* faces, int64_t* components) {
  Grid* g = (Grid*)gp;
  *cells = (int64_t)g->count();
  *faces = (int64_t)g->faces.size();
  *components = (int64_t)g->components.size();
}
// Exports the grid's products. Absent lo/hi and solid cell_faces are -1.
void ora_grid_export(void* gp, uint8_t* fluid, uint8_t* face_kind, int64_t* face_lo, int64_t* face_hi,
                     double* face_area, double* face_distance, int32_t* component, uint8_t* anchored,
                     int64_t* cell_faces, double* face_center, uint8_t* face_axis) {
  Grid* g = (Grid*)gp;
  size_t N = g->count(), F = g->faces.size();
  for (size_t i = 0; i < N; ++i) {
    if (fluid) fluid[i] = g->fluid[i];
    if (component) component[i] = g->component[i] == NONE ? -1 : (int32_t)g->component[i];
    if (cell_faces)
      for (int s = 0; s < 6; ++s) cell_faces[i * 6 + s] = g->cell_faces[i][s] == NONE ? -1 : (int64_t)g->cell_faces[i][s];
  }
  for (size_t f = 0; f < F; ++f) {
    const Face& x = g->faces[f];
    if (face_kind) face_kind[f] = (uint8_t)x.kind;
    if (face_lo) face_lo[f] = x.lo == NONE ? -1 : (int64_t)x.lo;
    if (face_hi) face_hi[f] = x.hi == NONE ? -1 : (int64_t)x.hi;
    if (face_area) face_area[f] = x.area;
    if (face_distance) face_distance[f] = x.distance;
    if (face_axis) face_axis[f] = (uint8_t)x.axis;
    if (face_center)
      for (int d = 0; d < 3; ++d) face_center[f * 3 + d] = x.center[d];
  }
  if (anchored)
    for (size_t c = 0; c < g->anchored.size(); ++c) anchored[c] = g->anchored[c];
}
void ora_grid_set_faces(void* gp, const double* area, const double* distance) {
  Grid* g = (Grid*)gp;
  for (size_t f = 0; f < g->faces.size(); ++f) {
    if (area) g->faces[f].area = area[f];
    if (distance) g->faces[f].distance = distance[f];
  }
}
int32_t ora_project(void* gp, double* u, double* p, double dt, double tol, uint64_t max, int (*poll)(void*),
                    void* ctx, ora_info* out) {
  Control control;
  control.poll = poll;
  control.ctx = ctx;
  Info info;
  Grid* g = (Grid*)gp;
  // Transactional: work on copies, commit on success (pressure.rs:468).
  std::vector<double> uu(u, u + g->faces.size()), pp(p, p + g->count());
  int c = project(*g, uu.data(), pp.data(), dt, tol, max, control, info);
  fill_info(info, control.polls, out);
  if (c) return c;
  std::copy(uu.begin(), uu.end(), u);
  std::copy(pp.begin(), pp.end(), p);
  return OK;
}
int32_t ora_solve_scaled(void* gp, const double* b, const double* terms, double tol, uint64_t max,
                         int (*poll)(void*), void* ctx, double* x, ora_info* out) {
  Control control;
  control.poll = poll;
  control.ctx = ctx;
  Info info;
  std::vector<double> xx;
  int c = solve_scaled(*(Grid*)gp, b, terms, tol, max, control, xx, info);
  fill_info(info, control.polls, out);
  if (c) return c;
  std::copy(xx.begin(), xx.end(), x);
  return OK;
}
void ora_apply(void* gp, const double* x, double* y) { public_apply(*(Grid*)gp, x, y); }
void ora_operator_apply(void* gp, const double* x, double* y) {
  Grid* g = (Grid*)gp;
  Operator::build(*g).apply(x, y, g->count());
}
void ora_center_nullspaces(void* gp, double* x) { center_nullspaces(*(Grid*)gp, x); }
void ora_projection_rhs(void* gp, const double* u, double dt, double* b, double* terms) {
  projection_rhs(*(Grid*)gp, u, dt, b, terms);
}
// grid.rs:612-627 (Iterator::sum over the three axes)
void ora_divergence(void* gp, const double* u, double* out) {
  Grid* g = (Grid*)gp;
  for (size_t i = 0; i < g->count(); ++i) {
    if (!g->fluid[i]) { out[i] = 0.0; continue; }
    double s = -0.0;
    for (int a = 0; a < 3; ++a) s += (u[g->cell_faces[i][a * 2 + 1]] - u[g->cell_faces[i][a * 2]]) / g->dx[a];
    out[i] = s;
  }
}
// grid.rs:650-665
void ora_gradient(void* gp, const double* p, double* out) {
  Grid* g = (Grid*)gp;
  for (size_t f = 0; f < g->faces.size(); ++f) {
    const Face& x = g->faces[f];
    if (x.kind == K_INTERIOR) out[f] = (p[x.hi] - p[x.lo]) / x.distance;
    else if (x.kind == K_OUTLET) out[f] = x.lo != NONE ? -p[x.lo] / x.distance : p[x.hi] / x.distance;
    else out[f] = 0.0;
  }
}
}  // extern "C" (momentum below is C++)

// ---------------------------------------------------------------- laminar momentum (next row)
// grid.rs:593-607 face_at: the axis-a face at position q; periodic axes wrap.
static size_t face_at(const Grid& g, int a, long q[3]) {
  for (int d = 0; d < 3; ++d) {
    if (g.boundary[d] == B_PERIODIC) {
      long n = (long)g.n[d];
      q[d] = ((q[d] % n) + n) % n;
    } else if (q[d] < 0 || q[d] >= (long)g.face_dims[a][d]) {
      return NONE;
    }
  }
  return g.offsets[a] + ((size_t)q[2] * g.face_dims[a][1] + (size_t)q[1]) * g.face_dims[a][0] + (size_t)q[0];
}

// flow.rs:66-154 ghost_values for laminar flow without moving walls: slip and outflow
// mirror the face value, an inflowing open side reflects about the inflow, walls and
// buildings reflect about zero.
static double ghost_value(const Grid& g, const Face& f, int d, int side, double value) {
  const bool at_domain = side < 0 ? f.center[d] < g.dx[d] : f.center[d] > g.size_m[d] - g.dx[d];
  const int bc = g.boundary[d];
  if (at_domain && bc == B_SLIP) return value;
  if (at_domain && bc == B_OPEN) {
    double v[3];
    g.flow.vector(f.center[2], v);
    const double speed = v[d] * (double)side;
    if (speed < -1e-12) {
      const double inflow = v[f.axis];
      return 2.0 * inflow - value;
    }
    return value;
  }
  const double target = 0.0;
  return 2.0 * target - value;
}

// flow.rs:156-180 sample
static double sample(const Grid& g, size_t fi, int d, int side, size_t nb, const double* u) {
  const Face& f = g.faces[fi];
  if (nb != NONE) {
    const int k = g.faces[nb].kind;
    if ((k == K_WALL || k == K_BLOCKED) && d != f.axis) return ghost_value(g, f, d, side, u[fi]);
    return u[nb];
  }
  if (d == f.axis) return u[fi];
  return ghost_value(g, f, d, side, u[fi]);
}

// flow.rs:426-525 momentum_rhs, laminar flow with the default donor-cell advection and no
// vegetation: zero on faces without an equation.
static int momentum_rhs(const Grid& g, const double* u, double* out) {
  if (g.flow.kind == F_RANS) return UNSUPPORTED;
  const size_t N = g.count();
  // grid.rs:631-645 cell_velocity
  std::vector<std::array<double, 3>> cu(N);
  for (size_t i = 0; i < N; ++i)
    for (int a = 0; a < 3; ++a)
      cu[i][a] = g.fluid[i] ? 0.5 * (u[g.cell_faces[i][a * 2]] + u[g.cell_faces[i][a * 2 + 1]]) : 0.0;
  const double nu = g.viscosity;
  for (size_t fi = 0; fi < g.faces.size(); ++fi) {
    const Face& f = g.faces[fi];
    if (f.kind != K_INTERIOR && f.kind != K_OUTLET) {
      out[fi] = 0.0;
      continue;
    }
    double velocity[3];
    for (int a = 0; a < 3; ++a) {
      if (f.lo != NONE && f.hi != NONE) velocity[a] = 0.5 * (cu[f.lo][a] + cu[f.hi][a]);
      else if (f.lo != NONE) velocity[a] = cu[f.lo][a];
      else if (f.hi != NONE) velocity[a] = cu[f.hi][a];
      else velocity[a] = 0.0;
    }
    double rhs = 0.0;
    for (int d = 0; d < 3; ++d) {
      long ql[3] = {(long)f.coord[0], (long)f.coord[1], (long)f.coord[2]};
      long qh[3] = {(long)f.coord[0], (long)f.coord[1], (long)f.coord[2]};
      ql[d] -= 1;
      qh[d] += 1;
      const size_t lo_face = face_at(g, f.axis, ql), hi_face = face_at(g, f.axis, qh);
      const double lo = sample(g, fi, d, -1, lo_face, u);
      const double hi = sample(g, fi, d, 1, hi_face, u);
      rhs = rhs - velocity[d] * (velocity[d] >= 0.0 ? (u[fi] - lo) / g.dx[d] : (hi - u[fi]) / g.dx[d]);
      const double mu = nu + 0.0;
      const double mu_lo = mu, mu_hi = mu;
      rhs = rhs + (mu_hi * (hi - u[fi]) - mu_lo * (u[fi] - lo)) / (g.dx[d] * g.dx[d]);
    }
    rhs = rhs + g.acceleration[f.axis];
    rhs = rhs + (f.lo != NONE && f.hi != NONE ? 0.5 * (0.0 + 0.0) : 0.0);  // the RANS cross term, zero
    out[fi] = rhs;
  }
  return OK;
}

static void enforce_velocity(const Grid& g, double* u) {
  for (size_t f = 0; f < g.faces.size(); ++f) {
    const Face& x = g.faces[f];
    if (x.kind == K_WALL || x.kind == K_SLIP || x.kind == K_BLOCKED) u[f] = 0.0;
    else if (x.kind == K_INLET) {
      double v[3];
      g.flow.vector(x.center[2], v);
      u[f] = v[x.axis];
    }
  }
}

// solver.rs:671-732 flow_euler (explicit algorithm, no vegetation drag).
static int flow_euler(Grid& g, const double* u, const double* p, double dt, double tol, uint64_t max,
                      std::vector<double>& v, std::vector<double>& pp, uint64_t& iterations) {
  const size_t F = g.faces.size();
  std::vector<double> rhs(F), grad(F);
  if (int c = momentum_rhs(g, u, rhs.data())) return c;
  for (size_t f = 0; f < F; ++f) {
    const Face& x = g.faces[f];
    if (x.kind == K_INTERIOR) grad[f] = (p[x.hi] - p[x.lo]) / x.distance;
    else if (x.kind == K_OUTLET) grad[f] = x.lo != NONE ? -p[x.lo] / x.distance : p[x.hi] / x.distance;
    else grad[f] = 0.0;
  }
  v.resize(F);
  for (size_t f = 0; f < F; ++f) v[f] = u[f] + dt * (rhs[f] - grad[f]);
  enforce_velocity(g, v.data());
  pp.assign(p, p + g.count());
  Control control;
  Info info;
  if (int c = project(g, v.data(), pp.data(), dt, tol, max, control, info)) return c;
  iterations += info.iterations;
  enforce_velocity(g, v.data());
  return OK;
}

// transport.rs:510-516 minmod: 0 when a b <= 0, else signum(a) min(|a|, |b|) (a is
// nonzero then, so f64::signum is +-1, or NaN for a NaN).
static double minmod(double a, double b) {
  if (a * b <= 0.0) return 0.0;
  const double signum = std::isnan(a) ? a : (std::signbit(a) ? -1.0 : 1.0);
  return signum * std::fmin(std::fabs(a), std::fabs(b));
}
// transport.rs:502-509: the cell across cell i's face on axis a, side 0 (lo) or 1 (hi),
// when that face is interior.
static size_t neighbor(const Grid& g, size_t i, int a, int side) {
  const Face& f = g.faces[g.cell_faces[i][a * 2 + side]];
  if (f.kind != K_INTERIOR) return NONE;
  return side == 0 ? f.lo : f.hi;
}
// transport.rs:517-526: the monotonized-central slope of c at cell i along axis a.
static double slope(const Grid& g, const double* c, size_t i, int a) {
  const size_t jl = neighbor(g, i, a, 0), jh = neighbor(g, i, a, 1);
  const double lo = jl != NONE ? c[jl] : c[i];
  const double hi = jh != NONE ? c[jh] : c[i];
  return minmod(0.5 * (hi - lo), minmod(2.0 * (c[i] - lo), 2.0 * (hi - c[i])));
}

// transport.rs:656-723 rhs_into with linear upwind or MUSCL (`muscl`: the donor value plus
// or minus half the limited slope of the upwind cell along the face's axis) and a zero inlet
// concentration (solver.rs:823-832 passes |_| 0.0), in face order.
// Also returns the emission rate (the source densities summed, times the volume) and the
// open-boundary inflow and outflow rates (transport.rs:717-723).
static void scalar_rhs(const Grid& g, const double* c, const double* u, const double* d, const double* source,
                       double* v, double rates[3], bool muscl = false) {
  const size_t N = g.count();
  double inflow = 0.0, outflow = 0.0;
  for (size_t i = 0; i < N; ++i) v[i] = source[i];
  for (size_t fi = 0; fi < g.faces.size(); ++fi) {
    const Face& f = g.faces[fi];
    if (f.kind != K_INTERIOR && f.kind != K_INLET && f.kind != K_OUTLET) continue;
    const double cl = f.lo != NONE ? c[f.lo] : 0.0;
    const double cr = f.hi != NONE ? c[f.hi] : 0.0;
    double donor;
    if (u[fi] >= 0.0) donor = f.lo != NONE ? cl + (muscl ? 0.5 * slope(g, c, f.lo, f.axis) : 0.0) : cl;
    else donor = f.hi != NONE ? cr - (muscl ? 0.5 * slope(g, c, f.hi, f.axis) : 0.0) : cr;
    double diffusivity;
    if (f.lo != NONE && f.hi != NONE) diffusivity = 0.5 * (d[f.lo] + d[f.hi]);
    else if (f.lo != NONE) diffusivity = d[f.lo];
    else if (f.hi != NONE) diffusivity = d[f.hi];
    else diffusivity = 0.0;
    const double diff = f.kind == K_OUTLET ? 0.0 : diffusivity * (cl - cr) / f.distance;
    const double flux = (u[fi] * donor + diff) * f.area;
    const double per_volume = flux / g.volume;
    if (f.lo != NONE) v[f.lo] = v[f.lo] - per_volume;
    if (f.hi != NONE) v[f.hi] = v[f.hi] + per_volume;
    if (f.lo == NONE || f.hi == NONE) {
      const double outward = f.lo != NONE ? flux : -flux;
      outflow += std::fmax(outward, 0.0);
      inflow += std::fmax(-outward, 0.0);
    }
  }
  double s = rsum_init();
  for (size_t i = 0; i < N; ++i) s += source[i];
  rates[0] = s * g.volume;
  rates[1] = inflow;
  rates[2] = outflow;
}

extern "C" {

// solver.rs:808-855 advance_scalar: one SSPRK2 step of a constituent in place (no particle
// terms).
// `budget` (nullable): emitted, inflow and outflow masses in kg, incremented as
// solver.rs:851-853 does.
// muscl: Advection::Muscl (transport.rs:670-694), else linear upwind.
void ora_scalar_step_adv(void* gp, double* c, const double* u, const double* d, const double* source, double dt,
                         double* budget, int32_t muscl) {
  const Grid& g = *(Grid*)gp;
  const size_t N = g.count();
  std::vector<double> r1(N), stage(N), r2(N);
  double a[3], b[3];
  scalar_rhs(g, c, u, d, source, r1.data(), a, muscl != 0);
  for (size_t i = 0; i < N; ++i) stage[i] = c[i] + dt * r1[i];
  scalar_rhs(g, stage.data(), u, d, source, r2.data(), b, muscl != 0);
  for (size_t i = 0; i < N; ++i) c[i] = 0.5 * (c[i] + stage[i] + dt * r2[i]);
  if (budget)
    for (int k = 0; k < 3; ++k) budget[k] += 0.5 * dt * (a[k] + b[k]);
}
void ora_scalar_step(void* gp, double* c, const double* u, const double* d, const double* source, double dt,
                     double* budget) {
  ora_scalar_step_adv(gp, c, u, d, source, dt, budget, 0);
}

// transport.rs:651-699 rhs_into's returned rates of the field c: emitted (source sum times
// the cell volume), inflow and outflow over the domain-boundary faces, in kg/s.
void ora_scalar_rates(void* gp, const double* c, const double* u, const double* d, const double* source,
                      double* rates, int32_t muscl) {
  const Grid& g = *(Grid*)gp;
  std::vector<double> r(g.count());
  scalar_rhs(g, c, u, d, source, r.data(), rates, muscl != 0);
}

// Laminar flow terms the projection does not need (case flow: viscosity_m2_s, acceleration_m_s2).
void ora_grid_set_flow_terms(void* gp, double viscosity, const double* acceleration) {
  Grid* g = (Grid*)gp;
  g->viscosity = viscosity;
  for (int a = 0; a < 3; ++a) g->acceleration[a] = acceleration ? acceleration[a] : 0.0;
}
int32_t ora_momentum_rhs(void* gp, const double* u, double* out) { return momentum_rhs(*(Grid*)gp, u, out); }
// solver.rs:879-960: one SSPRK2 step of the laminar flow, a projection per stage, in place.
int32_t ora_step(void* gp, double* u, double* p, double dt, double tol, uint64_t max, uint64_t* iterations) {
  Grid& g = *(Grid*)gp;
  const size_t F = g.faces.size();
  std::vector<double> v, p1, v2, p2;
  uint64_t it = 0;
  if (int c = flow_euler(g, u, p, dt, tol, max, v, p1, it)) return c;
  if (int c = flow_euler(g, v.data(), p1.data(), dt, tol, max, v2, p2, it)) return c;
  for (size_t f = 0; f < F; ++f) u[f] = 0.5 * (u[f] + v2[f]);
  std::copy(p2.begin(), p2.end(), p);
  enforce_velocity(g, u);
  if (iterations) *iterations = it;
  return OK;
}

// grid.rs:683-691
void ora_enforce_velocity(void* gp, double* u) {
  Grid* g = (Grid*)gp;
  for (size_t f = 0; f < g->faces.size(); ++f) {
    const Face& x = g->faces[f];
    if (x.kind == K_WALL || x.kind == K_SLIP || x.kind == K_BLOCKED) u[f] = 0.0;
    else if (x.kind == K_INLET) {
      double v[3];
      g->flow.vector(x.center[2], v);
      u[f] = v[x.axis];
    }
  }
}
// Applies the IC(0) preconditioner of the grid (building the cached factor).
void ora_ic0_apply(void* gp, const double* r, double* z) {
  Grid* g = (Grid*)gp;
  if (!g->factor) g->factor = factor_build(*g);
  factor_apply(*g->factor, r, z, g->count());
}
// Exports the IC(0) factor diagonal (N) and, for each row, its CSR lower entries.
int64_t ora_ic0_nnz(void* gp) {
  Grid* g = (Grid*)gp;
  if (!g->factor) g->factor = factor_build(*g);
  return (int64_t)g->factor->lower.size();
}
void ora_ic0_export(void* gp, int64_t* row_offsets, int64_t* columns, double* lower, double* diagonal) {
  Grid* g = (Grid*)gp;
  if (!g->factor) g->factor = factor_build(*g);
  const Factor& F = *g->factor;
  for (size_t i = 0; i < F.row_offsets.size(); ++i) row_offsets[i] = (int64_t)F.row_offsets[i];
  for (size_t i = 0; i < F.columns.size(); ++i) {
    columns[i] = (int64_t)F.columns[i];
    lower[i] = F.lower[i];
  }
  for (size_t i = 0; i < F.diagonal.size(); ++i) diagonal[i] = F.diagonal[i];
}
// One multigrid V-cycle application (builds or reuses the hierarchy).
int32_t ora_mg_apply(void* gp, const double* r, double* z, ora_info* out) {
  Grid* g = (Grid*)gp;
  Control control;
  Info info;
  int c = prepare_multigrid(*g, control, info);
  if (c) return c;
  hierarchy_apply(*g->hierarchy, r, z, g->count(), info);
  fill_info(info, control.polls, out);
  return OK;
}
// Unmasked hierarchy export of one level: its dims and the dense matrix (n*n, row major;
// dense may be null to query the dims). Returns n, or -1 when absent.
int64_t ora_mg_level_dense(void* gp, int32_t level, int64_t* dims, double* dense) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy || g->hierarchy->masked || level < 0 || level >= (int32_t)g->hierarchy->levels.size()) return -1;
  const Level& L = g->hierarchy->levels[level];
  const size_t n = L.matrix.diagonal.size();
  for (int a = 0; a < 3; ++a) dims[a] = (int64_t)L.dims[a];
  if (dense) {
    std::fill(dense, dense + n * n, 0.0);
    for (size_t i = 0; i < n; ++i) {
      dense[i * n + i] = L.matrix.diagonal[i];
      for (size_t k = L.matrix.offsets[i]; k < L.matrix.offsets[i + 1]; ++k)
        dense[i * n + L.matrix.columns[k]] += L.matrix.values[k];
    }
  }
  return (int64_t)n;
}
// The prolongation of an unmasked level to the next one as a dense n x nc matrix (row
// major; dense may be null to query nc). Returns nc, or -1 when absent.
int64_t ora_mg_transfer_dense(void* gp, int32_t level, double* dense) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy || g->hierarchy->masked || level < 0 || level + 1 >= (int32_t)g->hierarchy->levels.size())
    return -1;
  const Level& L = g->hierarchy->levels[level];
  const size_t n = L.matrix.diagonal.size();
  const size_t nc = g->hierarchy->levels[level + 1].matrix.diagonal.size();
  if (dense) {
    std::fill(dense, dense + n * nc, 0.0);
    for (size_t i = 0; i < n; ++i)
      for (size_t k = L.transfer.offsets[i]; k < L.transfer.offsets[i + 1]; ++k)
        dense[i * nc + L.transfer.columns[k]] += L.transfer.weights[k];
  }
  return (int64_t)nc;
}
// multigrid/line.rs: a block smoother over the axes in `axes_mask` (bit a = axis a, in
// axis order) with the periodic flags `periodic_mask`, built on an unmasked level's matrix
// and swept once over x in place. Returns 0, or E036 / -1.
int32_t ora_block_sweep(void* gp, int32_t level, int32_t axes_mask, int32_t periodic_mask, int32_t backward,
                        const double* rhs, double* x) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy || g->hierarchy->masked || level < 0 || level >= (int32_t)g->hierarchy->levels.size()) return -1;
  const Level& L = g->hierarchy->levels[level];
  std::vector<int> axes;
  for (int a = 0; a < 3; ++a)
    if (axes_mask & (1 << a)) axes.push_back(a);
  bool periodic[3];
  for (int a = 0; a < 3; ++a) periodic[a] = (periodic_mask >> a) & 1;
  Control control;
  BlockSmoother b;
  if (int e = b.build(L.matrix, L.dims, axes, periodic, control)) return e;
  if (x) b.sweep(rhs, x, backward != 0);
  return x ? OK : -(int32_t)b.bandwidth - 1000;  // without x: the half-bandwidth, encoded
}
// Level sizes of the current hierarchy; returns the level count (0 before the first build).
int32_t ora_mg_levels(void* gp, uint64_t* cells, uint64_t* nonzeros, int32_t cap) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy) return 0;
  int32_t L = (int32_t)g->hierarchy->level_cells.size();
  for (int32_t i = 0; i < L && i < cap; ++i) {
    cells[i] = g->hierarchy->level_cells[i];
    nonzeros[i] = g->hierarchy->level_nonzeros[i];
  }
  return L;
}
// Cell dimensions per level of an unmasked hierarchy (MultigridStats::level_dimensions,
// multigrid.rs:561-563,611): dims[3*i + a]. Returns the level count, 0 for a masked
// hierarchy (its aggregates have no dimensions, masked.rs:261-262) or before a build.
int32_t ora_mg_dims(void* gp, int64_t* dims, int32_t cap) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy || g->hierarchy->masked) return 0;
  int32_t L = (int32_t)g->hierarchy->levels.size();
  for (int32_t i = 0; i < L && i < cap; ++i)
    for (int a = 0; a < 3; ++a) dims[3 * i + a] = (int64_t)g->hierarchy->levels[i].dims[a];
  return L;
}
// The block smoothers of the hierarchy (MultigridStats::block_smoothers, multigrid.rs:
// 612-616; BlockSmootherStats, line.rs:200-209 without the storage bytes): per smoother
// out[5*s ..] = level, axes bit mask, unknowns per block, block count, half-bandwidth.
// Returns the number of smoothers.
int32_t ora_mg_blocks(void* gp, int64_t* out, int32_t cap) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy || g->hierarchy->masked) return 0;
  int32_t s = 0;
  for (size_t l = 0; l < g->hierarchy->levels.size(); ++l)
    for (const BlockSmoother& b : g->hierarchy->levels[l].lines) {
      if (s < cap) {
        int64_t mask = 0;
        for (int a : b.axes) mask |= 1 << a;
        int64_t* o = out + 5 * s;
        o[0] = (int64_t)l, o[1] = mask, o[2] = (int64_t)b.length;
        o[3] = (int64_t)(b.nodes.size() / b.length), o[4] = (int64_t)b.bandwidth;
      }
      ++s;
    }
  return s;
}
// Masked hierarchy export of one level: parent map (cells of this level -> next), the CSR
// matrix, and the diagonal. Returns the number of rows, or -1 when absent.
int64_t ora_mg_masked_level(void* gp, int32_t level, int64_t* parent, int64_t* offsets, int64_t* columns,
                            double* values, double* diagonal, int64_t* nnz) {
  Grid* g = (Grid*)gp;
  if (!g->hierarchy || !g->hierarchy->masked || level < 0 || level >= (int32_t)g->hierarchy->mlevels.size())
    return -1;
  const MaskedLevel& l = g->hierarchy->mlevels[level];
  size_t n = l.x.size();
  if (nnz) *nnz = (int64_t)l.a.values.size();
  if (parent)
    for (size_t i = 0; i < l.parent.size(); ++i) parent[i] = (int64_t)l.parent[i];
  if (offsets)
    for (size_t i = 0; i <= n; ++i) offsets[i] = (int64_t)l.a.offsets[i];
  if (columns)
    for (size_t i = 0; i < l.a.columns.size(); ++i) columns[i] = (int64_t)l.a.columns[i];
  if (values)
    for (size_t i = 0; i < l.a.values.size(); ++i) values[i] = l.a.values[i];
  if (diagonal)
    for (size_t i = 0; i < n; ++i) diagonal[i] = l.a.diagonal[i];
  return (int64_t)n;
}

}  // extern "C"
