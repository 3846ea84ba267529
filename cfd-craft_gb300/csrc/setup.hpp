// Host-side setup of the pressure engine: the IC(0) factor, level schedules and
// the multigrid hierarchy, built once per grid (or per signature) and uploaded.
// Everything here is plain C++ compiled without FMA contraction, so the numbers
// it produces are bit-identical to the reference's (crates/cfd-craft, Rust).
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace cfdg {

enum FaceKind : uint8_t { INTERIOR = 0, WALL = 1, SLIP = 2, INLET = 3, OUTLET = 4, BLOCKED = 5 };

// The caller's grid (cfdg_grid_desc), copied.
struct HostGrid {
  int32_t n[3];
  double dx[3];
  double volume;
  int32_t periodic[3];
  int64_t cells, faces;
  std::vector<uint8_t> fluid, face_kind;
  std::vector<int32_t> face_lo, face_hi;  // -1 for none
  std::vector<double> face_area, face_distance;
  std::vector<int32_t> component;
  std::vector<uint8_t> anchored;
  int32_t n_components;
  int64_t face_offset[3];
  int64_t face_dims[3][3];
  // Pressure weight of face f: area / (distance * volume) (pressure.rs:257).
  double weight(int64_t f) const { return face_area[f] / (face_distance[f] * volume); }
  int64_t cell(int64_t i, int64_t j, int64_t k) const { return (k * n[1] + j) * n[0] + i; }
};

// Validates the face arrays against the structured layout and fills face_offset/face_dims.
// Returns an empty string when consistent.
std::string check_layout(HostGrid& g);

struct Csr {
  std::vector<int32_t> off;  // rows + 1
  std::vector<int32_t> col;
  std::vector<double> val;
  int32_t rows() const { return off.empty() ? 0 : (int32_t)off.size() - 1; }
};

// Rows grouped by dependency level: the rows of level l are order[start[l] .. start[l+1]).
struct Schedule {
  std::vector<int32_t> order;
  std::vector<int32_t> start;
  int32_t levels() const { return start.empty() ? 0 : (int32_t)start.size() - 1; }
};
// Level schedule of a lexicographic sweep over a structurally symmetric pattern:
// forward, row i waits for its columns j < i; backward, for its columns j > i.
Schedule schedule(const Csr& pattern, bool backward);

// IC(0) of the shifted pressure matrix (pressure.rs:118-222): lower rows sorted by
// column, plus the transpose used by the backward substitution as a gather (for
// column c, the rows i > c that hold c, in descending i: the order in which the
// reference's backward scatter updates z[c], pressure.rs:233-240).
struct Ic0 {
  Csr lower;
  std::vector<double> diag;
  Csr upper;  // row c: columns i (rows of `lower` that contain c), descending
  Schedule fwd, bwd;
};
void build_ic0(const HostGrid& g, Ic0& out);

// Cooperative cancellation during setup (pressure.rs:69, masked.rs:99-111).
struct Poller {
  int (*fn)(void*) = nullptr;
  void* ctx = nullptr;
  int check() const;  // 0, or CFDG_CANCELLED / CFDG_WALL_TIME
};

// The line (or small plane) block smoother of an anisotropic level (multigrid/line.rs:
// 26-150): block b is nodes[b*length .. (b+1)*length); `outside` holds, per node position,
// the level's entries whose column lies in another block (value, column); `factor` holds
// each block's banded Cholesky factor (stride bandwidth+1, entry [pos*stride + d] = L(pos,
// pos-d)) with the diagonal replaced by its reciprocal. fwd/bwd: the blocks grouped by
// dependency level for a forward / backward block Gauss-Seidel sweep.
struct LineBlocks {
  int32_t length = 0, bandwidth = 0;
  std::vector<int32_t> axes;
  std::vector<int32_t> nodes;
  Csr outside;
  std::vector<double> factor;
  Schedule fwd, bwd;
  int32_t count() const { return length ? (int32_t)(nodes.size() / length) : 0; }
};

// One level of the symmetric V(2,2) cycle (multigrid.rs:667-726, masked.rs:304-342), or
// V(1,1) with block smoothers on anisotropic grids.
struct MgLevel {
  int32_t n = 0;
  Csr a;  // off-diagonal entries in the reference's row order (multigrid.rs:233-262)
  std::vector<double> diag;
  Schedule fwd, bwd;
  Csr groups;    // closed groups centred at this level: members per group
  Csr prolong;   // fine row -> (coarse column, weight), columns ascending
  Csr restrict;  // coarse row -> (fine child, weight), children ascending
  // Masked levels: parity of the node's bin coordinates. Aggregates are connected sets
  // inside one bin, so neighbouring nodes sit in face-adjacent bins and the parity is
  // a two-colouring of the level's graph (used by the parallel smoothers).
  std::vector<uint8_t> parity;
  // Anisotropic unmasked levels: the block smoothers, used in turn by the cycle's sweeps
  // (one sweep each way, multigrid.rs:676-718); empty for point Gauss-Seidel.
  std::vector<LineBlocks> lines;
  // Terminal level: dense lower Cholesky blocks (masked.rs:16-70, multigrid.rs:468-520).
  Csr direct_idx;                   // block -> solved indices
  std::vector<int64_t> direct_off;  // block -> offset of its n*n factor in direct_factor
  std::vector<double> direct_factor;
};

struct Hierarchy {
  bool masked = false;
  std::vector<int32_t> fluid_indices;  // compact index -> cell (masked); empty = identity
  std::vector<MgLevel> levels;
  std::vector<uint64_t> level_cells, level_nonzeros;
  // Cells per axis of each level of an unmasked hierarchy (multigrid.rs:561-563); empty
  // for masked hierarchies, whose aggregates have no dimensions (masked.rs:261-262).
  std::vector<std::array<int32_t, 3>> level_dims;
};

// multigrid.rs:530-645 / masked.rs:181-291. Returns 0 or a CFDG_* code.
int build_hierarchy(const HostGrid& g, const Poller& poll, Hierarchy& h);
// The aggregation (masked.rs) hierarchy whether or not the grid has solid cells: the
// mixed form's hierarchy on grids the reference coarsens geometrically.
int build_aggregation_hierarchy(const HostGrid& g, const Poller& poll, Hierarchy& h);

// The exact signature a hierarchy was built from (multigrid.rs:158-222).
struct Signature {
  int32_t n[3];
  uint64_t spacing[3];
  std::vector<uint8_t> anchored, fluid;
  std::vector<uint8_t> kind;
  std::vector<int32_t> lo, hi;
  std::vector<uint64_t> wbits;
  bool operator==(const Signature& o) const;
};
// Returns 0, or CFDG_E034 for an empty pressure space or a non-finite/non-positive weight.
int signature_of(const HostGrid& g, Signature& s);

}  // namespace cfdg
