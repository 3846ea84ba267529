// Mixed-precision, batched form of the pressure projection.
//
// Per case: the FP64 projection right-hand side b and its compatible (gauge-centred)
// part b_c, then an outer FP64 defect-correction loop. Each outer step recomputes
// r = b_c - A x with the exact FP64 operator (the reference's face order, with
// rounded-as-written products: the true residual of pressure.rs:403-415) and stops
// once |r|/|b_c| <= tol; otherwise it solves A e = r/|r| approximately with an inner
// FP32 PCG (vectors, operator and the multigrid V-cycle in FP32; dot products carried
// as compensated FP32 pairs, alpha/beta in FP64) and adds |r| e to x.
//
// The V-cycle keeps the reference hierarchy (multigrid.rs / masked.rs: same aggregates,
// Galerkin coarse operators, transfers and per-component gauges) but smooths with
// parallel orderings: red-black Gauss-Seidel on the structured fine level (level-0 FP32
// arrays in a colour-split row layout), two-colour Gauss-Seidel by bin parity on the
// aggregation levels, l1-Jacobi on levels needing more than 8 colours, colours reversed
// on the way up so the cycle stays symmetric; the coarse corrections of aggregation
// hierarchies are scaled by the grid's over-correction factor. Sweep counts and the
// factor are per grid (cfdg_grid_set_cycle / cfdg_grid_set_coarse_scale). The coarsest
// level is solved in FP64 with the inverses of the reference's dense Cholesky factors.
//
// Batching: the fine-level kernels are persistent and run over a device work-list of
// row tiles (8 rows, one warp per row) drawn from all active cases; all coarse levels of
// all cases run in one cooperative kernel (grid-wide phases for large levels, one block
// per case for small ones). A per-case state machine (outer step -> inner start -> inner
// iterations -> outer step ... -> done) lets a fixed kernel sequence serve every case,
// so the whole iteration is captured once as a CUDA graph and replayed in chunks; the
// server (continuous batching) admits and finishes requests between chunks.
#include <cooperative_groups.h>
#include <cuda.h>  // CUtensorMap (the encoder is fetched from the driver at run time)
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "state.hpp"

namespace cg = cooperative_groups;

namespace cfdg {
namespace mx {

constexpr int TILE = 256;       // fine cells per block
constexpr int FTILE = 1024;     // faces per block (velocity correction)
constexpr int CS = 16;          // CTAs per cluster (non-portable size, opted in at pack time)
constexpr int CT = 1024;        // threads per cluster CTA
constexpr int MAXL = 16;        // coarse levels per case
constexpr int CHUNK_IT = 8;     // iterations per captured graph launch (batched projections)
constexpr int SERVER_CHUNK_IT = 4;  // the same for servers: requests join and leave at chunk ends

enum State : int { OUTER = 0, SCALE = 1, START = 2, RUN = 3, DONE = 4, FAIL = 5, IDLE = 6 };

struct MState {
  double norm, rz, alpha, beta, scale, true_rel, tol, inner_tol;
  double rr;
  int state, error, inner_it, total_it, outer, max_it, max_inner, has_e;
  unsigned counter;
  int pad;
};

struct FineCase {
  int n[3];
  int N;
  int uniform;
  float w32[3], wo32[3];
  double w64[3], wo64[3];
  long long face_off[3];
  int fdim[3][3];
  double dx[3];
  long long F;
  int tile0, ntiles;     // cell tiles of this case in the work-list
  int ftile0, nftiles;   // face tiles
  const uint16_t* flags;
  const uint8_t* fluid;
  const double* fw64;    // per-face FP64 weights (the grid's)
  const double* diag64;  // the level-0 diagonal in FP64 (the grid's hierarchy, full-grid cells)
  const float* fw32;     // per-face FP32 weights (non-uniform grids)
  // Level-0 FP32 arrays use the colour-split row layout (slot lay(r, colour, nxh, i>>1)).
  const float* diag0;    // level-0 diagonal, 0 for solid cells
  const float* idiag0;   // its reciprocal, 0 where the diagonal is 0
  const uint16_t* flags0;  // face flags
  int nxh, N2;           // slots per colour and row (ceil(nx/2)); slots in all (2 * rows * nxh)
  // TMA descriptors of the level-0 arrays viewed as [rows][2 colours][nxh] (k_rb_tma):
  // rhs0, idiag0, flags0, x0 with boxes of RT rows, x0 with RT + 2 rows; null when the
  // case does not take the staged path (non-uniform weights or nxh not a multiple of 8).
  const CUtensorMap* tmaps;
  // FP64 outer vectors (the grid's buffers, natural cell order)
  double *x64, *r64, *bc, *b, *terms;
  // FP32 inner vectors (split layout; padding slots stay zero)
  float *e, *r32, *p, *q, *x0, *rhs0, *res0;
  double* partials;  // ntiles doubles
  // level-0 closed groups (full indices) for the gauge
  int ngroups;
  // No closed groups on level 0: the residual before restriction is taken on colour 0
  // only (colour 1's is zero up to rounding after the last pre-smoothing half sweep), its
  // colour-1 slots stay zero and the restriction gathers colour-0 children only.
  int resc0;
  int wbc;  // the grid has no closed components: k_rhs writes b_c (= b) itself
  // Level 1 laid out as the bin grid (bin1): aggregate of bin (I, J, K) in row
  // colour*h1 + (K*nb1[1] + J)*nbh1 + (I>>1), colour = (I+J+K)&1, nbh1 = ceil(nb1[0]/2),
  // h1 = nb1[1]*nb1[2]*nbh1; empty bins are empty rows. Valid where every 2x2x2 bin holds at
  // most one aggregate and prolongation is by injection; the residual of the colour-0
  // children is then formed inside the restriction and the parent of a cell is its bin.
  int bin1, nbh1, h1, pad_bin1;
  int nb1[3], pad_nb1;
  const int *goff, *gmem;
  // transfers level 0 <-> 1
  int n1;
  const int *r_off, *r_child;  // level-1 rows gather level-0 children
  const float* r_w;
  const int *p_off, *p_col;    // level-0 rows (full layout) from level-1
  const float* p_w;
  const int* pinj;             // injection prolongation (aggregation): level-1 parent per slot, -1 none
  float pscale;                // the coarse-correction scale of the injection path
  float *rhs1, *x1;
  // projection I/O for this solve
  double* u;
  double* pfield;
  double dt;
  double rdt;  // RN(1/dt) for div_rdt, 0 when dt lies outside [2^-60, 2^60]
  const uint8_t* fkind;
  const int *flo, *fhi;
  const double* fdist;
};
static_assert(sizeof(FineCase) % 8 == 0, "FineCase is copied to shared memory in 8-byte words");

struct CLev {
  int n, terminal, ncolors, ngroups;
  // Smoother: 0 multicolour Gauss-Seidel, 1 l1-Jacobi (levels whose graph needs many
  // colours: the wide Galerkin stencils of linear-interpolation hierarchies).
  // res0: a two-colour Gauss-Seidel level without closed groups. The residual is taken on
  // colour 0 only: after the last (colour-1) half sweep before it, colour 1's residual is
  // zero up to rounding, so those rows keep res = 0 (the cycle is unchanged in exact
  // arithmetic and stays symmetric).
  int jacobi, res0;
  const float* il1;  // l1-Jacobi: 1 / (diag + sum |a_ij|), 0 where diag is 0
  float* x2;         // l1-Jacobi: the second iterate of a sweep pair
  const int *off, *col;
  const float *val, *diag;
  const int* coff;  // colour c owns rows coff[c] .. coff[c+1]-1
  const int *ell_off, *ell_w;  // per colour: start of its ELL block and its width
  const int* ell_col;          // column-major ELL per colour (padding points at the row itself)
  const float* ell_val;        // entries, 0 in padding
  const float* idiag;          // 1/diag, 0 where diag is 0
  const int *goff, *gmem;
  const int *roff, *rchild;  // restriction to the next level
  const float* rw;
  const int *poff, *pcol;    // prolongation from the next level
  const float* pw;
  float *rhs, *x, *res;
  int nblocks;
  const int *ioff, *idx;
  const long long* foff;
  const double* fac;
  // Level 1 of a bin1 grid whose rows all fit the bin stencil: per row its ELL entries in
  // order as 7-bit codes (bits 7a..7a+2 the neighbour direction x-lo, x-hi, y-lo, y-hi,
  // z-lo, z-hi, 7 for padding; bits 7a+3..7a+6 an index into svt, the level's distinct
  // entry values), so a sweep computes its columns instead of loading them. Null: ELL.
  const unsigned long long* scode;
  const float* svt;
  int snb1y, snbh;  // bins per column (nb1[1]) and per colour of a bin row (nbh1)
};

static_assert(sizeof(CLev) % 8 == 0, "CLev is copied to shared memory in 8-byte words");

struct CCase {
  int nl;  // levels 1 .. nl (lv[0] is level 1)
  CLev lv[MAXL];
  double* gpart;  // group partials, max groups * CS
};

__device__ __forceinline__ bool in_state(const MState& S, int a, int b = -1) {
  return S.state == a || S.state == b;
}

__device__ __forceinline__ double bsum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;
}

// Reductions of the fine-level kernels. Every warp stores its sum in the case's partials
// (slot = tile * RT + warp, no block barrier); a block counts a case's tiles once per run
// of consecutive tiles of that case, and the block that completes a case sums the
// partials in slot order (the same bits whatever the grid size) and applies the case's
// scalar update.
__device__ __forceinline__ void tile_partial(double v, const FineCase& F, int lt, double* sh, int& seg_n) {
  (void)sh;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) F.partials[lt * (TILE / 32) + (threadIdx.x >> 5)] = v;
  ++seg_n;
}

// The same from a compensated FP32 pair per thread (hi, lo): the warp's pairs are summed
// with TwoSum in FP32 and converted to FP64 once per warp (the FP64 pipe is narrow).
__device__ __forceinline__ void tile_partial2(float hi, float lo, const FineCase& F, int lt, int& seg_n) {
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_down_sync(0xffffffffu, hi, o), l2 = __shfl_down_sync(0xffffffffu, lo, o);
    const float s = hi + h2, bb = s - hi;
    lo += l2 + ((hi - (s - bb)) + (h2 - bb));
    hi = s;
  }
  if ((threadIdx.x & 31) == 0) F.partials[lt * (TILE / 32) + (threadIdx.x >> 5)] = (double)hi + (double)lo;
  ++seg_n;
}

struct Seg {
  int ci = -1, n = 0;  // case of the current run of tiles, tiles with a stored partial
};

template <class Fin>
__device__ __forceinline__ void close_seg(const FineCase* FC, MState* ST, Seg& g, double* sh, Fin fin) {
  if (g.n == 0) return;
  __shared__ bool last;
  __syncthreads();  // every warp's partials of the run are stored
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ST[g.ci].counter, (unsigned)g.n) + (unsigned)g.n == (unsigned)FC[g.ci].ntiles;
  }
  __syncthreads();
  g.n = 0;
  if (!last) return;
  __threadfence();
  const int nt = FC[g.ci].ntiles * (TILE / 32);
  const double* part = FC[g.ci].partials;
  double a = 0.0;
  for (int k = threadIdx.x; k < nt; k += blockDim.x) a += __ldcg(&part[k]);
  const double s = bsum(a, sh);
  if (threadIdx.x == 0) {
    ST[g.ci].counter = 0;
    fin(ST[g.ci], s);
  }
}

// Persistent fine-level kernels: block b takes the contiguous tile range
// [b*per, (b+1)*per) of the work-list (neighbouring rows stay in one block's cache).
// A tile whose case is not in the kernel's state: skip the rest of that case's tiles in
// this block's range (a case's tiles are consecutive in every list, in tile order), so
// idle cases cost one state read per block instead of one per tile.
#define SKIP_CASE(T_, TEST_)                \
  {                                         \
    const MState& S_ = ST[(T_).x];          \
    if (!(TEST_)) {                         \
      ti += FC[(T_).x].ntiles - 1 - (T_).y; \
      continue;                             \
    }                                       \
  }

#define TILE_RANGE                                   \
  const int n_ = *count;                             \
  const int per_ = (n_ + gridDim.x - 1) / gridDim.x; \
  const int t0_ = blockIdx.x * per_, t1_ = min(n_, t0_ + per_);

// The fine-level kernels that take groups of tiles: up to PG consecutive tiles of one case
// per step of a block's loop, so the fixed cost of a tile (its work-list entry, the case's
// state and descriptor) is paid once per group and a warp's loads of several rows are in
// flight together. tile_run: the length of the run of consecutive tiles of t's case that
// starts at list entry ti (at most PG, inside the block's range).
constexpr int PG = 4;
__device__ __forceinline__ int tile_run(const int2* tiles, int ti, int t1, int2 t) {
  int2 u[PG - 1];
#pragma unroll
  for (int m = 1; m < PG; ++m) u[m - 1] = ti + m < t1 ? tiles[ti + m] : make_int2(-1, 0);
  int n = 1;
#pragma unroll
  for (int m = 1; m < PG; ++m)
    if (n == m && u[m - 1].x == t.x && u[m - 1].y == t.y + m) n = m + 1;
  return n;
}

// 1/y when y is a positive power of two whose reciprocal is a normal number, else 0. A
// product with it is the quotient by y bit for bit (the same real value, rounded the same
// way): FP64 division is ~20x dearer than a product on this part.
__device__ __forceinline__ double exact_recip(double y) {
  const long long b = __double_as_longlong(y);
  const int e = (int)((b >> 52) & 0x7ff);
  if ((b & (long long)0x800fffffffffffffull) != 0 || e < 1 || e > 2045) return 0.0;
  return __longlong_as_double((long long)(2046 - e) << 52);
}

// x / y rounded to nearest from ry = RN(1/y), by Markstein's correction step (P. Markstein,
// IBM J. Res. Dev. 34(1), 1990; restated as a theorem in Muller et al., Handbook of
// Floating-Point Arithmetic): q = RN(x ry) lies within one ulp of x/y, rem = x - q y is
// exact under one FMA, and RN(q + rem ry) is RN(x/y) when nothing underflows or overflows.
// With y in [2^-60, 2^60] (else ry = 0) and |x| in [2^-900, 2^900] every intermediate stays
// normal; zeros, subnormals, NaN, infinities and x outside that range take the division.
__device__ __forceinline__ double div_rdt(double x, double y, double ry) {
  const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  if (ry == 0.0 || e < 123 || e > 1923) return __ddiv_rn(x, y);
  const double q = __dmul_rn(x, ry);
  const double rem = __fma_rn(-q, y, x);
  return __fma_rn(rem, ry, q);
}

// The host side of div_rdt: RN(1/dt), or 0 outside the range the device step assumes.
inline double rdt_of(double dt) {
  return (dt >= 0x1p-60 && dt <= 0x1p60) ? 1.0 / dt : 0.0;
}

__device__ __forceinline__ long long fidx(const FineCase& F, int a, int i, int j, int k) {
  return F.face_off[a] + ((long long)k * F.fdim[a][1] + j) * F.fdim[a][0] + i;
}

// w * d for a weight w = 2^k (k from pow2_k, else 99): the exponent field of d moved by k
// when d and the product are normal (the exact product, so the same bits), else the FP64
// product. Moves the uniform grids' weight products off the FP64 pipe.
__device__ __forceinline__ int pow2_k(double w) {
  const long long b = __double_as_longlong(w);
  const int e = (int)((b >> 52) & 0x7ff);
  return ((b & (long long)0x800fffffffffffffull) == 0 && e >= 1 && e <= 2046) ? e - 1023 : 99;
}
__device__ __forceinline__ double mulw(double w, int k, double d) {
  if (k != 99) {
    const long long b = __double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    const int r = e + k;
    if (e != 0 && e != 0x7ff && r >= 1 && r <= 2046) return __longlong_as_double(b + ((long long)k << 52));
    if ((b & 0x7fffffffffffffffLL) == 0) return d;
  }
  return __dmul_rn(w, d);
}
// x / y bit for bit: for y a power of two the exponent field of x moved (mulw), else the
// division.
__device__ __forceinline__ double div_p2(double x, double y) {
  const double r = exact_recip(y);
  return r != 0.0 ? mulw(r, pow2_k(r), x) : __ddiv_rn(x, y);
}

// FP64 operator with every product and sum rounded as written, in the reference's
// face order (non-periodic grid): bit-identical to pressure::apply.
__device__ __forceinline__ double op64r(const FineCase& F, const double* __restrict__ x, int c, int i, int j, int k,
                                        unsigned fl) {
  if (!(fl & 0x0fffu)) return 0.0;
  const int q[3] = {i, j, k};
  const int stride[3] = {1, F.n[0], F.n[0] * F.n[1]};
  const double xc = x[c];
  double y = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const unsigned lin = (fl >> (2 * a)) & 1u, uin = (fl >> (2 * a + 1)) & 1u;
    const unsigned lout = (fl >> (6 + 2 * a)) & 1u, uout = (fl >> (7 + 2 * a)) & 1u;
    if (!(lin | uin | lout | uout)) continue;
    double wl, wu;
    int kl = 99, ku = 99;
    if (F.uniform) {
      wl = lout ? F.wo64[a] : F.w64[a];
      wu = uout ? F.wo64[a] : F.w64[a];
      kl = pow2_k(wl);
      ku = pow2_k(wu);
    } else {
      int p[3] = {q[0], q[1], q[2]};
      wl = F.fw64[fidx(F, a, p[0], p[1], p[2])];
      p[a] += 1;
      wu = F.fw64[fidx(F, a, p[0], p[1], p[2])];
    }
    if (lin) y = __dsub_rn(y, mulw(wl, kl, __dsub_rn(x[c - stride[a]], xc)));
    else if (lout) y = __dadd_rn(y, mulw(wl, kl, xc));
    if (uin) y = __dadd_rn(y, mulw(wu, ku, __dsub_rn(xc, x[c + stride[a]])));
    else if (uout) y = __dadd_rn(y, mulw(wu, ku, xc));
  }
  return y;
}

// ----------------------------------------------------------------- fine-level kernels
// Fine-level kernels run over row tiles: tile (case, rt) holds the x-rows
// [rt*RT, rt*RT + RT) of that case's grid, i.e. the cells [rt*RT*nx, (rt*RT+RT)*nx).
// Stencil kernels give each warp one row (no index divisions per cell); element-wise
// kernels stride the tile's cells. Reductions keep one partial per row tile.
constexpr int RT = TILE / 32;  // rows per tile: one warp per row

#define FINE_PROLOGUE(STATE_TEST)                                                     \
  MState& S = ST[t.x];                                                                \
  if (!(STATE_TEST)) return;                                                          \
  __shared__ __align__(16) FineCase sF;                                               \
  if (cached_ != t.x) { /* block-uniform: copy the case descriptor */                 \
    __syncthreads(); /* the previous tile's readers of sF are done */                 \
    const long long* src_ = reinterpret_cast<const long long*>(&FC[t.x]);             \
    long long* dst_ = reinterpret_cast<long long*>(&sF);                              \
    for (int w_ = threadIdx.x; w_ < (int)(sizeof(FineCase) / 8); w_ += blockDim.x)     \
      dst_[w_] = src_[w_];                                                            \
    cached_ = t.x;                                                                    \
    __syncthreads();                                                                  \
  }                                                                                   \
  const FineCase& F = sF;                                                             \
  const int lt = t.y;                                                                 \
  const int nx_ = F.n[0];                                                             \
  const int cb = lt * RT * nx_;                                                       \
  const int ce = min(F.N, cb + RT * nx_);                                             \
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;                         \
  const int nxh_ = F.nxh;                                                             \
  const int sb = lt * RT * 2 * nxh_;                                                  \
  const int se = min(F.N2, sb + RT * 2 * nxh_);                                       \
  (void)cb;                                                                           \
  (void)ce;                                                                           \
  (void)sb;                                                                           \
  (void)se;                                                                           \
  (void)warp;                                                                         \
  (void)lane;

// The row of this warp: returns false when the tile has fewer rows.
__device__ __forceinline__ bool warp_row(const FineCase& F, int lt, int warp, int& j, int& k, int& rowbase) {
  const int r = lt * RT + warp;
  if (r >= F.n[1] * F.n[2]) return false;
  j = r % F.n[1];
  k = r / F.n[1];
  rowbase = r * F.n[0];
  return true;
}

// FP32 error-free transformations: a running sum (hi, lo) of exact products keeps
// about twice the FP32 significand, so a thread's few terms convert to FP64 once.
// Four consecutive slots (16-byte aligned): the level-0 arrays start on 256-byte
// boundaries and a row tile's slots on multiples of four.
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
// Compensated running sum (hi, lo) += v (Knuth's TwoSum).
__device__ __forceinline__ void dd_add(float v, float& hi, float& lo) {
  const float s = hi + v;
  const float bb = s - hi;
  lo += (hi - (s - bb)) + (v - bb);
  hi = s;
}
// Sum of the outlet-face weights of a cell whose outlet bits (x-lo ... z-hi) are ob.
template <class FC>
__device__ __forceinline__ float outlet_sum(const FC& F, unsigned ob) {
  float w = 0.0f;
#pragma unroll
  for (int f = 0; f < 6; ++f)
    if (ob & (1u << f)) w += F.wo32[f >> 1];
  return w;
}
__device__ __forceinline__ void dd_add_prod(float a, float b, float& hi, float& lo) {
  const float p = a * b;
  const float pe = fmaf(a, b, -p);
  const float s = hi + p;
  const float bb = s - hi;
  const float se = (hi - (s - bb)) + (p - bb);
  hi = s;
  lo += se + pe;
}

// Level-0 FP32 layout. Row r = k*ny + j keeps its colour-0 cells ((i+j+k) even) in the
// slots [2r*nxh, 2r*nxh + nxh) and its colour-1 cells in the next nxh slots, cell i in
// slot i>>1 (nxh = ceil(nx/2); an odd nx leaves one zero padding slot in one half). A
// red-black half sweep then reads and writes one contiguous half-row per row, and every
// neighbour of a cell has the other colour: the x-neighbours sit in the same row's other
// half at slots (i-1)>>1 and (i+1)>>1, the y- and z-neighbours at slot i>>1 of the other
// half of rows r-1, r+1, r-ny and r+ny.
__host__ __device__ __forceinline__ int lay(int r, int col, int nxh, int s) { return (2 * r + col) * nxh + s; }

// Offsets of the six neighbours of cell i (slot s) whose other-colour half-row starts at
// oth: x-lo, x-hi, y-lo, y-hi, z-lo, z-hi (only those with a face bit are read).
struct Nbr {
  int o[6];
  __device__ __forceinline__ Nbr(int oth, int i, int s, int sy, int sz) {
    o[0] = oth + ((i - 1) >> 1);
    o[1] = oth + ((i + 1) >> 1);
    o[2] = oth + s - sy;
    o[3] = oth + s + sy;
    o[4] = oth + s - sz;
    o[5] = oth + s + sz;
  }
};

// The neighbours of the two cells in slots s2 and s2+1 (s2 even, nxh even) of one
// colour half-row, loaded as float2 before any is used: the other half of the same row
// (plus the edge slot s2-1 or s2+2) and of rows r-1, r+1, r-ny, r+ny. Rows outside the
// grid are replaced by the same row (their faces are absent, so the values are unused).
struct Pair {
  float2 xo, yl, yh, zl, zh;
  float xe;
  __device__ __forceinline__ void load(const float* __restrict__ x, int oth, int s2, int par, int nxh, int sy,
                                       int sz, bool hy0, bool hy1, bool hz0, bool hz1) {
    xo = *reinterpret_cast<const float2*>(x + oth + s2);
    yl = *reinterpret_cast<const float2*>(x + (hy0 ? oth - sy : oth) + s2);
    yh = *reinterpret_cast<const float2*>(x + (hy1 ? oth + sy : oth) + s2);
    zl = *reinterpret_cast<const float2*>(x + (hz0 ? oth - sz : oth) + s2);
    zh = *reinterpret_cast<const float2*>(x + (hz1 ? oth + sz : oth) + s2);
    const int e = par ? s2 + 2 : s2 - 1;
    xe = (e >= 0 && e < nxh) ? x[oth + e] : 0.0f;
  }
  // Neighbour values of cell h (0: slot s2, 1: slot s2+1) in face order.
  __device__ __forceinline__ void of(int h, int par, float nb[6]) const {
    if (h == 0) {
      nb[0] = par ? xo.x : xe;
      nb[1] = par ? xo.y : xo.x;
      nb[2] = yl.x, nb[3] = yh.x, nb[4] = zl.x, nb[5] = zh.x;
    } else {
      nb[0] = par ? xo.y : xo.x;
      nb[1] = par ? xe : xo.y;
      nb[2] = yl.y, nb[3] = yh.y, nb[4] = zl.y, nb[5] = zh.y;
    }
  }
};

// FP32 operator at cell (i, j, k) in the split layout: sum over interior faces of
// w (x_c - x_n), plus w x_c on outlet faces, faces in x-lo, x-hi, y-lo, ... order.
__device__ __forceinline__ float op32s(const FineCase& F, const float* __restrict__ x, int own, const Nbr& nb, int i,
                                       int j, int k, unsigned fl) {
  if (!(fl & 0x0fffu)) return 0.0f;
  const int q[3] = {i, j, k};
  const float xc = x[own];
  float y = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const unsigned ib = 1u << (2 * a + side), ob = 1u << (6 + 2 * a + side);
      if (!(fl & (ib | ob))) continue;
      float w;
      if (F.uniform) {
        w = (fl & ib) ? F.w32[a] : F.wo32[a];
      } else {
        int p[3] = {q[0], q[1], q[2]};
        p[a] += side;
        w = F.fw32[fidx(F, a, p[0], p[1], p[2])];
      }
      if (fl & ib) y = fmaf(w, xc - x[nb.o[2 * a + side]], y);
      else y = fmaf(w, xc, y);
    }
  return y;
}

// Sum over interior faces of w x_n in face order, starting from v (Gauss-Seidel update
// and residual of the level-0 matrix, whose off-diagonal entries are -w).
__device__ __forceinline__ float nbsum32(const FineCase& F, const float* __restrict__ x, const Nbr& nb, int i, int j,
                                         int k, unsigned fl, float v, float sign) {
  if (F.uniform) {
#pragma unroll
    for (int f = 0; f < 6; ++f)
      if (fl & (1u << f)) v = fmaf(sign * F.w32[f >> 1], x[nb.o[f]], v);
  } else {
    const int q[3] = {i, j, k};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        if (!(fl & (1u << (2 * a + side)))) continue;
        int pp[3] = {q[0], q[1], q[2]};
        pp[a] += side;
        v = fmaf(sign * F.fw32[fidx(F, a, pp[0], pp[1], pp[2])], x[nb.o[2 * a + side]], v);
      }
  }
  return v;
}

struct FinOp {
  __device__ void operator()(MState& S, double pq) const {
    if (!(pq > 0.0) || !isfinite(pq)) {
      S.state = FAIL;
      S.error = CFDG_E032;
    } else {
      S.alpha = S.rz / pq;
    }
  }
};

// A: q = A32 p, alpha = rz / (p.q) (E032 when not positive).
__device__ __forceinline__ void b_op(const FineCase* FC, MState* ST, const int2 t, int& cached_, double* sh,
                                    int& seg_n) {
  FINE_PROLOGUE(S.state == RUN)
  float hi = 0.0f, lo = 0.0f;
  int j, k, rb;
  if (warp_row(F, lt, warp, j, k, rb) && F.uniform && !(nxh_ & 1)) {
    const int r = lt * RT + warp, sy = 2 * nxh_, sz = sy * F.n[1];
    const bool hy0 = j > 0, hy1 = j + 1 < F.n[1], hz0 = k > 0, hz1 = k + 1 < F.n[2];
    for (int col = 0; col < 2; ++col) {
      const int par = (j + k + col) & 1;
      const int own = lay(r, col, nxh_, 0), oth = lay(r, col ^ 1, nxh_, 0);
      for (int s2 = 2 * lane; s2 < nxh_; s2 += 64) {
        const float2 pc = *reinterpret_cast<const float2*>(F.p + own + s2);
        const unsigned fl2 = *reinterpret_cast<const unsigned*>(F.flags0 + own + s2);
        Pair P;
        P.load(F.p, oth, s2, par, nxh_, sy, sz, hy0, hy1, hz0, hz1);
        float nb[6];
        float2 y = make_float2(0.0f, 0.0f);
        // Interior faces in face order, each through a selected weight (0 where the face
        // is not interior) instead of a branch; the rare outlet faces after them.
        P.of(0, par, nb);
#pragma unroll
        for (int f = 0; f < 6; ++f) y.x = fmaf((fl2 & (1u << f)) ? F.w32[f >> 1] : 0.0f, pc.x - nb[f], y.x);
        if (fl2 & 0xfc0u) y.x = fmaf(outlet_sum(F, fl2 >> 6), pc.x, y.x);
        P.of(1, par, nb);
#pragma unroll
        for (int f = 0; f < 6; ++f) y.y = fmaf((fl2 & (1u << (16 + f))) ? F.w32[f >> 1] : 0.0f, pc.y - nb[f], y.y);
        if (fl2 & 0xfc00000u) y.y = fmaf(outlet_sum(F, fl2 >> 22), pc.y, y.y);
        *reinterpret_cast<float2*>(F.q + own + s2) = y;
        // p.q: the pair's two products in one FMA, then a compensated running sum.
        dd_add(fmaf(pc.x, y.x, pc.y * y.y), hi, lo);
      }
    }
  } else if (warp_row(F, lt, warp, j, k, rb)) {
    const int r = lt * RT + warp, sy = 2 * nxh_, sz = sy * F.n[1];
    for (int col = 0; col < 2; ++col) {
      const int par = (j + k + col) & 1;
      const int own = lay(r, col, nxh_, 0), oth = lay(r, col ^ 1, nxh_, 0);
      for (int s = lane; s < nxh_; s += 32) {
        const int i = 2 * s + par;
        if (i >= nx_) break;
        const float v = op32s(F, F.p, own + s, Nbr(oth, i, s, sy, sz), i, j, k, F.flags0[own + s]);
        F.q[own + s] = v;
        dd_add_prod(F.p[own + s], v, hi, lo);
      }
    }
  }
  tile_partial2(hi, lo, F, lt, seg_n);
}
__global__ void __launch_bounds__(TILE, 5) k_op(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  __shared__ double sh[32];
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  Seg g;
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == RUN)
    if (t.x != g.ci) {
      close_seg(FC, ST, g, sh, FinOp());
      g.ci = t.x;
    }
    b_op(FC, ST, t, cached_, sh, g.n);
  }
  close_seg(FC, ST, g, sh, FinOp());
}

struct FinUpdate {
  __device__ void operator()(MState& S, double rr) const {
    S.inner_it += 1;
    S.total_it += 1;
    S.has_e = 1;
    if (sqrt(rr) <= S.inner_tol || S.inner_it >= S.max_inner || S.total_it >= S.max_it) S.state = OUTER;
  }
};

// B: e += alpha p, r -= alpha q; |r| decides the end of the inner solve.
// The slot ranges of the n tiles lt .. lt+n-1 hold one float4 per thread each (row
// tiles of at most 4 * TILE slots, 16-byte aligned): the group path of the element-wise
// kernels, every operand of the group loaded before any result is stored. Otherwise the
// tiles run one at a time.
__device__ __forceinline__ bool group4(const FineCase& F, int sb, int nxh) {
  return !(sb & 3) && !(F.N2 & 3) && RT * 2 * nxh <= 4 * TILE;
}

// B: e += alpha p, r -= alpha q; |r| decides the end of the inner solve. One reduction
// partial per tile, as in the one-tile path, so the bits do not depend on the grouping.
__device__ __forceinline__ void b_update(const FineCase* FC, MState* ST, const int2 t, int n, int& cached_,
                                         int& seg_n) {
  FINE_PROLOGUE(S.state == RUN)
  const float alpha = (float)S.alpha;
  const int T = RT * 2 * nxh_;
  if (group4(F, sb, nxh_)) {
    float4 e[PG], p[PG], q[PG], r[PG];
    bool ok[PG];
#pragma unroll
    for (int m = 0; m < PG; ++m) {
      const int c = sb + m * T + 4 * threadIdx.x;
      ok[m] = m < n && 4 * (int)threadIdx.x < T && c < F.N2;
      if (ok[m]) e[m] = ld4(F.e + c), p[m] = ld4(F.p + c), q[m] = ld4(F.q + c), r[m] = ld4(F.r32 + c);
    }
#pragma unroll
    for (int m = 0; m < PG; ++m) {
      if (m >= n) break;
      float hi = 0.0f, lo = 0.0f;
      if (ok[m]) {
        const int c = sb + m * T + 4 * threadIdx.x;
        float4 ev = e[m], rv = r[m];
        const float4 pv = p[m], qv = q[m];
        ev.x = fmaf(alpha, pv.x, ev.x), ev.y = fmaf(alpha, pv.y, ev.y), ev.z = fmaf(alpha, pv.z, ev.z);
        ev.w = fmaf(alpha, pv.w, ev.w);
        rv.x = fmaf(-alpha, qv.x, rv.x), rv.y = fmaf(-alpha, qv.y, rv.y), rv.z = fmaf(-alpha, qv.z, rv.z);
        rv.w = fmaf(-alpha, qv.w, rv.w);
        st4(F.e + c, ev);
        st4(F.r32 + c, rv);
        dd_add(fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, rv.w * rv.w))), hi, lo);
      }
      tile_partial2(hi, lo, F, lt + m, seg_n);
    }
    return;
  }
  for (int m = 0; m < n; ++m) {
    const int b0 = sb + m * T, b1 = min(F.N2, b0 + T);
    float hi = 0.0f, lo = 0.0f;
    if (!((b0 | b1) & 3)) {
      for (int c = b0 + 4 * threadIdx.x; c < b1; c += 4 * TILE) {
        float4 e = ld4(F.e + c);
        const float4 p = ld4(F.p + c), q = ld4(F.q + c);
        float4 r = ld4(F.r32 + c);
        e.x = fmaf(alpha, p.x, e.x), e.y = fmaf(alpha, p.y, e.y), e.z = fmaf(alpha, p.z, e.z), e.w = fmaf(alpha, p.w, e.w);
        r.x = fmaf(-alpha, q.x, r.x), r.y = fmaf(-alpha, q.y, r.y), r.z = fmaf(-alpha, q.z, r.z);
        r.w = fmaf(-alpha, q.w, r.w);
        st4(F.e + c, e);
        st4(F.r32 + c, r);
        dd_add(fmaf(r.x, r.x, fmaf(r.y, r.y, fmaf(r.z, r.z, r.w * r.w))), hi, lo);
      }
    } else {
      for (int c = b0 + threadIdx.x; c < b1; c += TILE) {
        F.e[c] = fmaf(alpha, F.p[c], F.e[c]);
        const float r = fmaf(-alpha, F.q[c], F.r32[c]);
        F.r32[c] = r;
        dd_add_prod(r, r, hi, lo);
      }
    }
    tile_partial2(hi, lo, F, lt + m, seg_n);
  }
}
__global__ void __launch_bounds__(TILE) k_update(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  __shared__ double sh[32];
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  Seg g;
  for (int ti = t0_; ti < t1_;) {
    const int2 t = tiles[ti];
    if (ST[t.x].state != RUN) {  // the rest of this case's tiles in the range
      ti += FC[t.x].ntiles - t.y;
      continue;
    }
    if (t.x != g.ci) {
      close_seg(FC, ST, g, sh, FinUpdate());
      g.ci = t.x;
    }
    const int n = tile_run(tiles, ti, t1_, t);
    b_update(FC, ST, t, n, cached_, g.n);
    ti += n;
  }
  close_seg(FC, ST, g, sh, FinUpdate());
}

// C1: x += |r| e (the residual is formed by k_outer_resid once every block has updated x).
__device__ __forceinline__ void b_outer(const FineCase* FC, MState* ST, const int2 t, int& cached_) {
  FINE_PROLOGUE(S.state == OUTER)
  if (!S.has_e) return;
  const double scale = S.scale;
  int j, k, rb;
  if (!warp_row(F, lt, warp, j, k, rb)) return;
  const int r = lt * RT + warp, rp = (j + k) & 1;
  for (int i = lane; i < nx_; i += 32)
    F.x64[rb + i] = F.x64[rb + i] + scale * (double)F.e[lay(r, (i + rp) & 1, nxh_, i >> 1)];
}
__global__ void __launch_bounds__(TILE) k_outer(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == OUTER)
    b_outer(FC, ST, t, cached_);
  }
}

struct FinOuterResid {
  __device__ void operator()(MState& S, double rr) const {
    double nr = sqrt(rr);
    S.true_rel = nr / S.norm;
    if (S.true_rel <= S.tol) {
      S.state = DONE;
    } else if (S.total_it >= S.max_it) {
      S.state = FAIL;
      S.error = CFDG_E033;
    } else {
      S.scale = nr;
      S.outer += 1;
      S.state = SCALE;
    }
  }
};

// r = b_c - A x in FP64; the true residual decides convergence.
__device__ __forceinline__ void b_outer_resid(const FineCase* FC, MState* ST, const int2 t, int& cached_, double* sh,
                                    int& seg_n) {
  FINE_PROLOGUE(S.state == OUTER)
  double acc = 0.0;
  int j, k, rb;
  if (!S.has_e) {
    // First outer step: x = 0 exactly, so A x = 0 and r = b_c bit for bit.
    for (int c = cb + threadIdx.x; c < ce; c += TILE) {
      const double v = F.bc[c];
      F.r64[c] = v;
      acc = __fma_rn(v, v, acc);
    }
  } else if (warp_row(F, lt, warp, j, k, rb)) {
    // One warp per row, several cells per lane: the cells' FP64 chains are independent.
    const double* __restrict__ x = F.x64;
    const double* __restrict__ bc = F.bc;
    const uint16_t* __restrict__ fl = F.flags;
    double* __restrict__ r = F.r64;
    if (F.uniform) {
      // A x as diag x minus the interior neighbours through one FMA each (nine FP64
      // operations per cell against the fourteen of the reference's rounding order): on
      // this part the FP64 pipe bounds the kernel. The rounding differs from
      // pressure::apply's by a few ulps of diag |x|, far below the 1e-8 test.
      const int sy = F.n[0], sz = F.n[0] * F.n[1];
      const double mw[3] = {-F.w64[0], -F.w64[1], -F.w64[2]};
      const double* __restrict__ d64 = F.diag64;
#pragma unroll 4
      for (int i = lane; i < nx_; i += 32) {
        const int c = rb + i;
        const unsigned f = fl[c];
        double y = 0.0;
        if (f & 0x0fffu) {
          y = d64[c] * x[c];
          if (f & 1u) y = __fma_rn(mw[0], x[c - 1], y);
          if (f & 2u) y = __fma_rn(mw[0], x[c + 1], y);
          if (f & 4u) y = __fma_rn(mw[1], x[c - sy], y);
          if (f & 8u) y = __fma_rn(mw[1], x[c + sy], y);
          if (f & 16u) y = __fma_rn(mw[2], x[c - sz], y);
          if (f & 32u) y = __fma_rn(mw[2], x[c + sz], y);
        }
        const double v = __dsub_rn(bc[c], y);
        r[c] = v;
        acc = __fma_rn(v, v, acc);
      }
    } else {
#pragma unroll 4
      for (int i = lane; i < nx_; i += 32) {
        const int c = rb + i;
        const double v = __dsub_rn(bc[c], op64r(F, x, c, i, j, k, fl[c]));
        r[c] = v;
        acc = __fma_rn(v, v, acc);
      }
    }
  }
  tile_partial(acc, F, lt, sh, seg_n);
}
__global__ void __launch_bounds__(TILE) k_outer_resid(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  __shared__ double sh[32];
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  Seg g;
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == OUTER)
    if (t.x != g.ci) {
      close_seg(FC, ST, g, sh, FinOuterResid());
      g.ci = t.x;
    }
    b_outer_resid(FC, ST, t, cached_, sh, g.n);
  }
  close_seg(FC, ST, g, sh, FinOuterResid());
}

// C2: r32 = r / |r|, e = 0.
__device__ __forceinline__ void b_scale(const FineCase* FC, MState* ST, const int2 t, int& cached_) {
  FINE_PROLOGUE(S.state == SCALE)
  // r / |r| in FP32: the residual converted, then scaled in FP32 (one FP64-pipe
  // conversion per cell; the inner solve only needs its direction to FP32 precision),
  // while |r| keeps the converted entries normal; else the FP64 product.
  const double inv = 1.0 / S.scale;
  const bool fp32 = S.scale > 1e-25 && S.scale < 1e25;
  const float inv32 = (float)inv;
  for (int c = sb + threadIdx.x; c < se; c += TILE) F.e[c] = 0.0f;
  int j, k, rb;
  if (!warp_row(F, lt, warp, j, k, rb)) return;
  const int r = lt * RT + warp, rp = (j + k) & 1;
  for (int i = lane; i < nx_; i += 32)
    F.r32[lay(r, (i + rp) & 1, nxh_, i >> 1)] =
        fp32 ? __double2float_rn(F.r64[rb + i]) * inv32 : (float)(F.r64[rb + i] * inv);
}
__global__ void __launch_bounds__(TILE) k_scale(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == SCALE)
    b_scale(FC, ST, t, cached_);
  }
}

__global__ void k_start_state(MState* ST, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && ST[i].state == SCALE) {
    ST[i].state = START;
    ST[i].inner_it = 0;
  }
}

struct FinRz {
  __device__ void operator()(MState& S, double rz) const {
    if (S.state == START) {
      S.beta = 0.0;
      S.state = RUN;
    } else {
      S.beta = rz / S.rz;
    }
    S.rz = rz;
  }
};

// F: rz' = r.z; START: rz = rz', p = z (beta = 0) -> RUN; RUN: beta = rz'/rz.
__device__ __forceinline__ void b_rz(const FineCase* FC, MState* ST, const int2 t, int n, int& cached_, int& seg_n) {
  FINE_PROLOGUE(S.state == RUN || S.state == START)
  const int T = RT * 2 * nxh_;
  if (group4(F, sb, nxh_)) {
    float4 r[PG], z[PG];
    bool ok[PG];
#pragma unroll
    for (int m = 0; m < PG; ++m) {
      const int c = sb + m * T + 4 * threadIdx.x;
      ok[m] = m < n && 4 * (int)threadIdx.x < T && c < F.N2;
      if (ok[m]) r[m] = ld4(F.r32 + c), z[m] = ld4(F.x0 + c);
    }
#pragma unroll
    for (int m = 0; m < PG; ++m) {
      if (m >= n) break;
      float hi = 0.0f, lo = 0.0f;
      if (ok[m]) dd_add(fmaf(r[m].x, z[m].x, fmaf(r[m].y, z[m].y, fmaf(r[m].z, z[m].z, r[m].w * z[m].w))), hi, lo);
      tile_partial2(hi, lo, F, lt + m, seg_n);
    }
    return;
  }
  for (int m = 0; m < n; ++m) {
    const int b0 = sb + m * T, b1 = min(F.N2, b0 + T);
    float hi = 0.0f, lo = 0.0f;
    if (!((b0 | b1) & 3)) {
      for (int c = b0 + 4 * threadIdx.x; c < b1; c += 4 * TILE) {
        const float4 r = ld4(F.r32 + c), z = ld4(F.x0 + c);
        dd_add(fmaf(r.x, z.x, fmaf(r.y, z.y, fmaf(r.z, z.z, r.w * z.w))), hi, lo);
      }
    } else {
      for (int c = b0 + threadIdx.x; c < b1; c += TILE) dd_add_prod(F.r32[c], F.x0[c], hi, lo);
    }
    tile_partial2(hi, lo, F, lt + m, seg_n);
  }
}
__global__ void __launch_bounds__(TILE) k_rz(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  __shared__ double sh[32];
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  Seg g;
  for (int ti = t0_; ti < t1_;) {
    const int2 t = tiles[ti];
    if (!in_state(ST[t.x], RUN, START)) {  // the rest of this case's tiles in the range
      ti += FC[t.x].ntiles - t.y;
      continue;
    }
    if (t.x != g.ci) {
      close_seg(FC, ST, g, sh, FinRz());
      g.ci = t.x;
    }
    const int n = tile_run(tiles, ti, t1_, t);
    b_rz(FC, ST, t, n, cached_, g.n);
    ti += n;
  }
  close_seg(FC, ST, g, sh, FinRz());
}

// G: p = z + beta p (z is the V-cycle's level-0 solution x0).
__device__ __forceinline__ void b_p(const FineCase* FC, MState* ST, const int2 t, int n, int& cached_) {
  FINE_PROLOGUE(S.state == RUN)
  const float beta = (float)S.beta;
  const bool copy = S.beta == 0.0;
  const int T = RT * 2 * nxh_;
  if (group4(F, sb, nxh_)) {
    float4 p[PG], z[PG];
    bool ok[PG];
#pragma unroll
    for (int m = 0; m < PG; ++m) {
      const int c = sb + m * T + 4 * threadIdx.x;
      ok[m] = m < n && 4 * (int)threadIdx.x < T && c < F.N2;
      if (ok[m]) {
        z[m] = ld4(F.x0 + c);
        if (!copy) p[m] = ld4(F.p + c);
      }
    }
#pragma unroll
    for (int m = 0; m < PG; ++m)
      if (ok[m]) {
        float4 v = z[m];
        if (!copy) {
          v.x = fmaf(beta, p[m].x, z[m].x), v.y = fmaf(beta, p[m].y, z[m].y);
          v.z = fmaf(beta, p[m].z, z[m].z), v.w = fmaf(beta, p[m].w, z[m].w);
        }
        st4(F.p + sb + m * T + 4 * threadIdx.x, v);
      }
    return;
  }
  const int se_g = min(F.N2, sb + n * T);
  if (!((sb | se_g) & 3)) {
    for (int c = sb + 4 * threadIdx.x; c < se_g; c += 4 * TILE) {
      if (copy) {
        st4(F.p + c, ld4(F.x0 + c));
      } else {
        float4 p = ld4(F.p + c);
        const float4 z = ld4(F.x0 + c);
        p.x = fmaf(beta, p.x, z.x), p.y = fmaf(beta, p.y, z.y), p.z = fmaf(beta, p.z, z.z), p.w = fmaf(beta, p.w, z.w);
        st4(F.p + c, p);
      }
    }
  } else if (copy) {
    for (int c = sb + threadIdx.x; c < se_g; c += TILE) F.p[c] = F.x0[c];
  } else {
    for (int c = sb + threadIdx.x; c < se_g; c += TILE) F.p[c] = fmaf(beta, F.p[c], F.x0[c]);
  }
}
__global__ void __launch_bounds__(TILE) k_p(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_;) {
    const int2 t = tiles[ti];
    if (ST[t.x].state != RUN) {  // the rest of this case's tiles in the range
      ti += FC[t.x].ntiles - t.y;
      continue;
    }
    const int n = tile_run(tiles, ti, t1_, t);
    b_p(FC, ST, t, n, cached_);
    ti += n;
  }
}

// ----------------------------------------------------------------- V-cycle, level 0
// rhs0 = r32 (only when level 0 has closed groups; otherwise rhs0 is r32 itself).
__device__ __forceinline__ void b_v_rhs(const FineCase* FC, MState* ST, const int2 t, int& cached_) {
  FINE_PROLOGUE(S.state == RUN || S.state == START)
  if (F.rhs0 == F.r32) return;
  for (int c = sb + threadIdx.x; c < se; c += TILE) F.rhs0[c] = F.r32[c];
}
__global__ void __launch_bounds__(TILE) k_v_rhs(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == RUN || S_.state == START)
    b_v_rhs(FC, ST, t, cached_);
  }
}

// Red-black Gauss-Seidel half sweep on level 0: cells with (i+j+k)%2 == color, the
// contiguous colour half of the warp's row in the split layout.
// first: x is taken as zero (the cycle's initial guess). Cells outside the operator
// (solid, sealed singletons) are kept at zero.
__device__ __forceinline__ void b_rb(const FineCase* FC, MState* ST, const int2 t, int& cached_, int color, int first) {
  FINE_PROLOGUE(S.state == RUN || S.state == START)
  int j, k, rb;
  if (!warp_row(F, lt, warp, j, k, rb)) return;
  const int r = lt * RT + warp, sy = 2 * nxh_, sz = sy * F.n[1];
  const int par = (j + k + color) & 1;
  const int own = lay(r, color, nxh_, 0), oth = lay(r, color ^ 1, nxh_, 0);
  float* __restrict__ x = F.x0;
  if (F.uniform && !(nxh_ & 1)) {
    const bool hy0 = j > 0, hy1 = j + 1 < F.n[1], hz0 = k > 0, hz1 = k + 1 < F.n[2];
    const bool skip = first && color == 0;
    for (int s2 = 2 * lane; s2 < nxh_; s2 += 64) {
      const float2 id = *reinterpret_cast<const float2*>(F.idiag0 + own + s2);
      float2 v = *reinterpret_cast<const float2*>(F.rhs0 + own + s2);
      const unsigned fl2 = *reinterpret_cast<const unsigned*>(F.flags0 + own + s2);
      if (!skip) {
        Pair P;
        P.load(x, oth, s2, par, nxh_, sy, sz, hy0, hy1, hz0, hz1);
        float nb[6];
        P.of(0, par, nb);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if (fl2 & (1u << f)) v.x = fmaf(F.w32[f >> 1], nb[f], v.x);
        P.of(1, par, nb);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if (fl2 & (1u << (16 + f))) v.y = fmaf(F.w32[f >> 1], nb[f], v.y);
      }
      float2 out;
      out.x = id.x == 0.0f ? 0.0f : v.x * id.x;
      out.y = id.y == 0.0f ? 0.0f : v.y * id.y;
      *reinterpret_cast<float2*>(x + own + s2) = out;
    }
    return;
  }
  for (int s = lane; s < nxh_; s += 32) {
    const int i = 2 * s + par;
    if (i >= nx_) break;
    const float id = F.idiag0[own + s];
    if (id == 0.0f) {
      x[own + s] = 0.0f;
      continue;
    }
    float v = F.rhs0[own + s];
    if (!(first && color == 0)) v = nbsum32(F, x, Nbr(oth, i, s, sy, sz), i, j, k, F.flags0[own + s], v, 1.0f);
    x[own + s] = v * id;
  }
}
__global__ void __launch_bounds__(TILE, 5)
    k_rb(const FineCase* FC, MState* ST, const int2* tiles, const int* count, int color, int first) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == RUN || S_.state == START)
    b_rb(FC, ST, t, cached_, color, first);
  }
}

// ----------------------------------------------------------------- staged red-black half sweep
// The same half sweep as k_rb (uniform weights, nxh a multiple of 8), with every operand
// brought into shared memory by the tensor memory accelerator. A stage holds SR rows of
// one case (SR = 8, 16 or 32: one to four consecutive work-list tiles); its operands are six
// 3-D tensor copies ([rows][colour][nxh] views of the split layout): the own colour's rhs,
// 1/diag and flags of the SR rows, and the other colour's x of rows r0-1 .. r0+SR (y
// neighbours and the rows themselves) and of the SR rows one z-layer below and above.
// Rows outside the grid arrive as zeros (their faces are absent). A producer warp keeps
// NS stages in flight, each completed by an mbarrier transaction count; the RT consumer
// warps sweep a stage (warp w takes rows w, w + RT, ...) and release it through a second
// mbarrier. Results are bit-identical to k_rb: the same operands in the same fmaf order.
// The stage height and depth are the sweep's tile shape (cfdg_grid_set_sweep_tile).
constexpr int RB_MAX_NS = 8;    // stages per block at most
constexpr int RB_HEIGHTS = 3;   // stage heights 8, 16, 32 rows (tensor maps per height)

struct RbOff {
  int rhs, id, fl, xy, zl, zh, stage;
};
// Byte offsets inside one stage of sr rows for a row length of hmax slots (a multiple of
// 16, so every region starts on a 128-byte boundary).
__host__ __device__ __forceinline__ RbOff rb_offsets(int hmax, int sr) {
  RbOff o;
  o.rhs = 0;
  o.id = o.rhs + sr * 4 * hmax;
  o.fl = o.id + sr * 4 * hmax;
  o.xy = o.fl + sr * 2 * hmax;
  o.zl = o.xy + (sr + 2) * 4 * hmax;
  o.zh = o.zl + sr * 4 * hmax;
  o.stage = o.zh + sr * 4 * hmax;
  return o;
}
__host__ __device__ __forceinline__ int rb_height_index(int sr) { return sr == 8 ? 0 : (sr == 16 ? 1 : 2); }
constexpr long long RB_WAIT_CYCLES = 2000000000LL;  // a stage's wait gives up after ~1 s of SM clock

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for a stage's barrier for at most RB_WAIT_CYCLES SM cycles; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > RB_WAIT_CYCLES) return false;
  return true;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// What a consumer warp needs of a stage, written by the producer beside the data.
struct RbHead {
  float* x0;
  float w[3];
  int r0, nrows, ny, h, ci, pad;  // first row, valid rows (-1: end of the block's range)
};
constexpr int RB_THREADS = TILE + 32;  // RT consumer warps and one producer warp

__global__ void __launch_bounds__(RB_THREADS, 3) k_rb_tma(const FineCase* FC, MState* ST, const int2* tiles,
                                                          const int* count, int color, int first, int hmax, int sr,
                                                          int ns) {
  extern __shared__ __align__(128) unsigned char rb_dyn[];
  // Stage base on a 128-byte boundary (the launch adds 128 bytes of slack).
  unsigned char* const rb_smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(rb_dyn) + 127) & ~(uintptr_t)127);
  __shared__ __align__(8) uint64_t full[RB_MAX_NS], empty[RB_MAX_NS];
  __shared__ RbHead head[RB_MAX_NS];
  TILE_RANGE
  const RbOff O = rb_offsets(hmax, sr);
  const bool skipx = first && color == 0;  // x = 0: the sweep reads no neighbour
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int st = 0; st < ns; ++st) {
      mbar_init(&full[st], 1);    // the producer's arrival (with the copies' byte count)
      mbar_init(&empty[st], RT);  // one arrival per consumer warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (warp == RT) {
    // Producer warp: walks the block's tile range 32 entries at a time, keeps the current
    // case's descriptor in registers, skips the tiles of cases that are not running, joins
    // up to sr / RT consecutive tiles of one case into a stage and fills each stage as soon
    // as the consumers have released it.
    int cur = -1, st = 0;
    bool active = false;
    const CUtensorMap* tm = nullptr;
    RbHead hd{};
    int rows_all = 0, run_y = 0, run_n = 0;
    const int group = sr / RT, hi = rb_height_index(sr) * 5;
    unsigned ephase = (1u << RB_MAX_NS) - 1;  // a fresh stage counts as released
    bool dead = false;
    // Issues the open run of tiles into the next released stage; false when the wait gave up.
    auto flush = [&]() -> bool {
      if (run_n == 0) return true;
      int ok = 0;
      if (lane == 0) ok = mbar_wait_bounded(&empty[st], (ephase >> st) & 1u);
      if (!__shfl_sync(0xffffffffu, ok, 0)) return false;
      ephase ^= 1u << st;
      if (lane == 0) {
        const int r0 = run_y * RT, h = hd.h, oc = color ^ 1;
        hd.r0 = r0;
        hd.nrows = min(run_n * RT, rows_all - r0);
        head[st] = hd;
        unsigned char* b = rb_smem + st * O.stage;
        const unsigned bytes = sr * h * 8u + (skipx ? 0u : sr * h * 2u + (3 * sr + 2) * h * 4u);
        mbar_expect_tx(&full[st], bytes);
        tma_load_3d(b + O.rhs, &tm[hi + 0], 0, color, r0, &full[st]);
        tma_load_3d(b + O.id, &tm[hi + 1], 0, color, r0, &full[st]);
        if (!skipx) {
          tma_load_3d(b + O.fl, &tm[hi + 2], 0, color, r0, &full[st]);
          tma_load_3d(b + O.xy, &tm[hi + 4], 0, oc, r0 - 1, &full[st]);
          tma_load_3d(b + O.zl, &tm[hi + 3], 0, oc, r0 - hd.ny, &full[st]);
          tma_load_3d(b + O.zh, &tm[hi + 3], 0, oc, r0 + hd.ny, &full[st]);
        }
      }
      __syncwarp();
      st = st + 1 == ns ? 0 : st + 1;
      run_n = 0;
      return true;
    };
    for (int base = t0_; base < t1_ && !dead; base += 32) {
      const int2 mine = base + lane < t1_ ? tiles[base + lane] : make_int2(-1, 0);
      const int nq = min(32, t1_ - base);
      for (int q = 0; q < nq; ++q) {
        const int tx = __shfl_sync(0xffffffffu, mine.x, q), ty = __shfl_sync(0xffffffffu, mine.y, q);
        if (tx != cur) {
          if (!flush()) {
            dead = true;
            break;
          }
          cur = tx;
          const int state = ST[tx].state;
          active = state == RUN || state == START;
          const FineCase& F = FC[tx];
          tm = F.tmaps;
          hd.x0 = F.x0;
          hd.w[0] = F.w32[0], hd.w[1] = F.w32[1], hd.w[2] = F.w32[2];
          hd.ny = F.n[1], hd.h = F.nxh, hd.ci = tx;
          rows_all = F.n[1] * F.n[2];
        }
        if (!active) continue;
        if (run_n > 0 && ty != run_y + run_n && !flush()) {
          dead = true;
          break;
        }
        if (run_n == 0) run_y = ty;
        if (++run_n == group && !flush()) {
          dead = true;
          break;
        }
      }
    }
    if (!dead && flush()) {
      // End of the range: an empty stage in the next released slot.
      if (lane == 0 && mbar_wait_bounded(&empty[st], (ephase >> st) & 1u)) {
        head[st].nrows = -1;
        mbar_arrive(&full[st]);
      }
      return;
    }
    // The consumers never released a stage: fail the case at hand and stop feeding; the
    // consumers' own bounded waits end their loop.
    if (lane == 0 && cur >= 0) {
      ST[cur].error = CFDG_ERR_TIMEOUT;
      ST[cur].state = FAIL;
    }
    return;
  }
  // Consumer warps: warp w sweeps rows w, w + RT, ... of each stage, then releases it.
  unsigned fphase = 0;  // bit st: parity of the phase stage st completes next
  int last_ci = -1;
  for (int st = 0;; st = st + 1 == ns ? 0 : st + 1) {
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(&full[st], (fphase >> st) & 1u))) {
      // Never filled: fail the case last swept (if any), give the copies that may still be
      // in flight a bounded wait, and leave.
      if (lane == 0 && last_ci >= 0) {
        ST[last_ci].error = CFDG_ERR_TIMEOUT;
        ST[last_ci].state = FAIL;
      }
      mbar_wait_bounded(&full[st], (fphase >> st) & 1u);
      return;
    }
    fphase ^= 1u << st;
    const RbHead hd = head[st];
    if (hd.nrows < 0) return;  // every stage before it was swept; nothing is in flight
    last_ci = hd.ci;
    const int h = hd.h;
    const unsigned char* b = rb_smem + st * O.stage;
    for (int lr = warp; lr < hd.nrows; lr += RT) {
      const int r = hd.r0 + lr;
      const int par = (r % hd.ny + r / hd.ny + color) & 1;
      const float* srhs = reinterpret_cast<const float*>(b + O.rhs) + lr * h;
      const float* sid = reinterpret_cast<const float*>(b + O.id) + lr * h;
      const uint16_t* sfl = reinterpret_cast<const uint16_t*>(b + O.fl) + lr * h;
      const float* sxo = reinterpret_cast<const float*>(b + O.xy) + (lr + 1) * h;
      const float* szl = reinterpret_cast<const float*>(b + O.zl) + lr * h;
      const float* szh = reinterpret_cast<const float*>(b + O.zh) + lr * h;
      float* __restrict__ x = hd.x0 + lay(r, color, h, 0);
      for (int s2 = 2 * lane; s2 < h; s2 += 64) {
        const float2 id = *reinterpret_cast<const float2*>(sid + s2);
        float2 v = *reinterpret_cast<const float2*>(srhs + s2);
        if (!skipx) {
          const unsigned fl2 = *reinterpret_cast<const unsigned*>(sfl + s2);
          Pair P;
          P.xo = *reinterpret_cast<const float2*>(sxo + s2);
          P.yl = *reinterpret_cast<const float2*>(sxo - h + s2);
          P.yh = *reinterpret_cast<const float2*>(sxo + h + s2);
          P.zl = *reinterpret_cast<const float2*>(szl + s2);
          P.zh = *reinterpret_cast<const float2*>(szh + s2);
          const int e = par ? s2 + 2 : s2 - 1;
          P.xe = (e >= 0 && e < h) ? sxo[e] : 0.0f;
          float nb[6];
          P.of(0, par, nb);
#pragma unroll
          for (int f = 0; f < 6; ++f)
            if (fl2 & (1u << f)) v.x = fmaf(hd.w[f >> 1], nb[f], v.x);
          P.of(1, par, nb);
#pragma unroll
          for (int f = 0; f < 6; ++f)
            if (fl2 & (1u << (16 + f))) v.y = fmaf(hd.w[f >> 1], nb[f], v.y);
        }
        float2 out;
        out.x = id.x == 0.0f ? 0.0f : v.x * id.x;
        out.y = id.y == 0.0f ? 0.0f : v.y * id.y;
        *reinterpret_cast<float2*>(x + s2) = out;
      }
    }
    __syncwarp();
    if (lane == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // this warp's reads before the stage's next fill
      mbar_arrive(&empty[st]);
    }
  }
}

// acc + sum over k in [b, e) of w[k] v[idx[k]], in k order, with four entries' index and
// value loads in flight at a time (the transfers' rows are chains of dependent loads).
__device__ __forceinline__ float gather_sum(const int* __restrict__ idx, const float* __restrict__ w,
                                            const float* __restrict__ v, int b, int e, float acc) {
  int k = b;
  for (; k + 4 <= e; k += 4) {
    const int i0 = idx[k], i1 = idx[k + 1], i2 = idx[k + 2], i3 = idx[k + 3];
    const float w0 = w[k], w1 = w[k + 1], w2 = w[k + 2], w3 = w[k + 3];
    const float x0 = __ldcg(&v[i0]), x1 = __ldcg(&v[i1]), x2 = __ldcg(&v[i2]), x3 = __ldcg(&v[i3]);
    acc = fmaf(w0, x0, acc);
    acc = fmaf(w1, x1, acc);
    acc = fmaf(w2, x2, acc);
    acc = fmaf(w3, x3, acc);
  }
  for (; k < e; ++k) acc = fmaf(w[k], __ldcg(&v[idx[k]]), acc);
  return acc;
}

// res0 = rhs0 - A0 x0 (A0 = diag - sum w on interior faces).
__device__ __forceinline__ void b_v_resid(const FineCase* FC, MState* ST, const int2 t, int& cached_) {
  FINE_PROLOGUE(S.state == RUN || S.state == START)
  int j, k, rb;
  if (!warp_row(F, lt, warp, j, k, rb)) return;
  const int r = lt * RT + warp, sy = 2 * nxh_, sz = sy * F.n[1];
  const float* __restrict__ x = F.x0;
  if (F.uniform && !(nxh_ & 1)) {
    const bool hy0 = j > 0, hy1 = j + 1 < F.n[1], hz0 = k > 0, hz1 = k + 1 < F.n[2];
    for (int col = 0; col < (F.resc0 ? 1 : 2); ++col) {
      const int par = (j + k + col) & 1;
      const int own = lay(r, col, nxh_, 0), oth = lay(r, col ^ 1, nxh_, 0);
      for (int s2 = 2 * lane; s2 < nxh_; s2 += 64) {
        const float2 d = *reinterpret_cast<const float2*>(F.diag0 + own + s2);
        const float2 xc = *reinterpret_cast<const float2*>(x + own + s2);
        const float2 rh = *reinterpret_cast<const float2*>(F.rhs0 + own + s2);
        const unsigned fl2 = *reinterpret_cast<const unsigned*>(F.flags0 + own + s2);
        Pair P;
        P.load(x, oth, s2, par, nxh_, sy, sz, hy0, hy1, hz0, hz1);
        float nb[6];
        float va = d.x * xc.x, vb = d.y * xc.y;
        P.of(0, par, nb);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if (fl2 & (1u << f)) va = fmaf(-F.w32[f >> 1], nb[f], va);
        P.of(1, par, nb);
#pragma unroll
        for (int f = 0; f < 6; ++f)
          if (fl2 & (1u << (16 + f))) vb = fmaf(-F.w32[f >> 1], nb[f], vb);
        float2 out;
        out.x = d.x == 0.0f ? 0.0f : rh.x - va;
        out.y = d.y == 0.0f ? 0.0f : rh.y - vb;
        *reinterpret_cast<float2*>(F.res0 + own + s2) = out;
      }
    }
    return;
  }
  for (int col = 0; col < (F.resc0 ? 1 : 2); ++col) {
    const int par = (j + k + col) & 1;
    const int own = lay(r, col, nxh_, 0), oth = lay(r, col ^ 1, nxh_, 0);
    for (int s = lane; s < nxh_; s += 32) {
      const int i = 2 * s + par;
      if (i >= nx_) break;
      const float d = F.diag0[own + s];
      if (d == 0.0f) {
        F.res0[own + s] = 0.0f;
        continue;
      }
      const float v = nbsum32(F, x, Nbr(oth, i, s, sy, sz), i, j, k, F.flags0[own + s], d * x[own + s], -1.0f);
      F.res0[own + s] = F.rhs0[own + s] - v;
    }
  }
}
__global__ void __launch_bounds__(TILE) k_v_resid(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == RUN || S_.state == START)
    b_v_resid(FC, ST, t, cached_);
  }
}

// bin1 restriction, thread q of the case's 2*h1: bin row R = q / (2 nbh1) (J = R mod nb1[1],
// K = R / nb1[1]), bin I = q mod (2 nbh1), so consecutive threads take consecutive bins of a
// row and every level-1 row is written once (I >= nb1[0]: an empty row). Its right-hand
// side is the sum, in cell order, of the level-0 residuals of the bin's colour-0 cells (one
// per fine row: i = 2I + ((j+k)&1), slot I of the row's colour-0 half). The residual holds
// +0 on solid cells and padding slots, and a running sum that starts at +0 never becomes
// -0, so adding them changes no bit: the sum equals the index lists' over the members.
__device__ __forceinline__ void bin_restrict(const FineCase& F, int q) {
  const int nbh = F.nbh1, R = q / (2 * nbh), I = q - R * 2 * nbh;
  const int J = R % F.nb1[1], K = R / F.nb1[1];
  float acc = 0.0f;
  if (I < F.nb1[0]) {
    const int ny = F.n[1], nz = F.n[2], nxh = F.nxh;
    float v[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {  // (dk, dj) in cell order; the loads first, then the sum
      const int k = 2 * K + (c >> 1), j = 2 * J + (c & 1);
      v[c] = (k < nz && j < ny) ? __ldcg(&F.res0[lay(k * ny + j, 0, nxh, I)]) : 0.0f;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) acc = fmaf(1.0f, v[c], acc);
  }
  F.rhs1[((I + J + K) & 1) * F.h1 + R * nbh + (I >> 1)] = acc;
}

// rhs1 = R res0: level-1 rows gather their level-0 children. Tiles index level-1 rows.
__global__ void __launch_bounds__(TILE) k_v_restrict(const FineCase* FC, MState* ST, const int2* tiles1,
                                                     const int* count) {
  const int n = *count;
  for (int ti = blockIdx.x; ti < n; ti += gridDim.x) {
    const int2 t = tiles1[ti];
    const FineCase& F = FC[t.x];
    const MState& S = ST[t.x];
    if (!(S.state == RUN || S.state == START)) continue;
    const int j = t.y * TILE + threadIdx.x;
    if (j >= F.n1) continue;
    if (F.bin1) {
      bin_restrict(F, j);
      continue;
    }
    float v = 0.0f;
    v = gather_sum(F.r_child, F.r_w, F.res0, F.r_off[j], F.r_off[j + 1], v);
    F.rhs1[j] = v;
  }
}

// x0 += P x1 on the colour-0 slots only (the prolongation's rows are the split layout's
// slots; padding rows are empty): the first post-smoothing half sweep (colour 1) rewrites
// every colour-1 slot without reading it, so their coarse correction would be dead work.
// One call covers the n tiles lt .. lt+n-1 of the case.
__device__ __forceinline__ void b_v_prolong(const FineCase* FC, MState* ST, const int2 t, int n, int& cached_) {
  FINE_PROLOGUE(S.state == RUN || S.state == START)
  const int rows = F.n[1] * F.n[2];
  if (F.bin1 && nxh_ <= 64) {
    // One warp per row of each tile; the parent of the cell in colour-0 slot s
    // (i = 2s + par) is bin (s, j/2, k/2). Every load of the group before any store.
    // Solid cells take a correction too: no interior face reads them and the last
    // post-smoothing half sweep (colour 0) sets them to zero.
    const int ny = F.n[1], h1 = F.h1, nb1y = F.nb1[1], nbh = F.nbh1;
    const float* __restrict__ x1 = F.x1;
    float* __restrict__ x0 = F.x0;
    const float a = F.pscale;
    int idx[PG][2];
    float v1[PG][2], v0[PG][2];
#pragma unroll
    for (int m = 0; m < PG; ++m) {
      const int r = (lt + m) * RT + warp;
      const bool rowok = m < n && r < rows;
      const int j = r % ny, k = r / ny;
      const int par = (j + k) & 1, jk = (j >> 1) + (k >> 1), base1 = ((k >> 1) * nb1y + (j >> 1)) * nbh;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int sl = lane + 32 * q;
        const bool ok = rowok && sl < nxh_ && 2 * sl + par < nx_;
        idx[m][q] = ok ? lay(r, 0, nxh_, sl) : -1;
        v1[m][q] = ok ? x1[((sl + jk) & 1) * h1 + base1 + (sl >> 1)] : 0.0f;
        v0[m][q] = ok ? x0[idx[m][q]] : 0.0f;
      }
    }
#pragma unroll
    for (int m = 0; m < PG; ++m)
#pragma unroll
      for (int q = 0; q < 2; ++q)
        if (idx[m][q] >= 0) x0[idx[m][q]] = fmaf(a, v1[m][q], v0[m][q]);
    return;
  }
  for (int mt = 0; mt < n; ++mt) {
    const int ltm = lt + mt;
    const int rows_t = min(RT, rows - ltm * RT);
    if (F.bin1) {  // rows longer than 64 slots per colour: one row per warp and tile
      int j, k, rb;
      if (!warp_row(F, ltm, warp, j, k, rb)) continue;
      const int par = (j + k) & 1, jk = (j >> 1) + (k >> 1), h1 = F.h1;
      const int base1 = ((k >> 1) * F.nb1[1] + (j >> 1)) * F.nbh1;
      float* __restrict__ x = F.x0 + lay(ltm * RT + warp, 0, nxh_, 0);
      const float* __restrict__ x1 = F.x1;
      const float a = F.pscale;
      for (int sl = lane; sl < nxh_; sl += 32)
        if (2 * sl + par < nx_) x[sl] = fmaf(a, x1[((sl + jk) & 1) * h1 + base1 + (sl >> 1)], x[sl]);
      continue;
    }
    if (F.pinj) {  // x0 += x1[parent]: the same value as the weight-1 row below
      for (int m = threadIdx.x; m < rows_t * nxh_; m += TILE) {
        const int c = lay(ltm * RT + m / nxh_, 0, nxh_, m % nxh_);
        const int q = F.pinj[c];
        if (q >= 0) F.x0[c] = fmaf(F.pscale, F.x1[q], F.x0[c]);
      }
      continue;
    }
    for (int m = threadIdx.x; m < rows_t * nxh_; m += TILE) {
      const int c = lay(ltm * RT + m / nxh_, 0, nxh_, m % nxh_);
      const int b = F.p_off[c], e = F.p_off[c + 1];
      if (b == e) continue;
      // The linear-interpolation rows (up to 8 entries) in entry order, four gathers in
      // flight at a time (gather_sum keeps the order of the fmaf chain).
      const float sum = gather_sum(F.p_col, F.p_w, F.x1, b, e, 0.0f);
      F.x0[c] += sum;
    }
  }
}
__global__ void __launch_bounds__(TILE) k_v_prolong(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_;) {
    const int2 t = tiles[ti];
    if (!in_state(ST[t.x], RUN, START)) {  // the rest of this case's tiles in the range
      ti += FC[t.x].ntiles - t.y;
      continue;
    }
    const int n = tile_run(tiles, ti, t1_, t);
    b_v_prolong(FC, ST, t, n, cached_);
    ti += n;
  }
}

// Gauge of level-0 closed groups: one block per (case, group); members strided.
// which: 0 rhs0, 1 x0, 2 res0.
__global__ void k_center0(const FineCase* FC, MState* ST, const int2* gtab, const int* count, int which) {
  __shared__ double sh[32];
  __shared__ float mean;
  const int n = *count;
  for (int ti = blockIdx.x; ti < n; ti += gridDim.x) {
    const int2 t = gtab[ti];
    const FineCase& F = FC[t.x];
    const MState& S = ST[t.x];
    if (!(S.state == RUN || S.state == START)) continue;
    float* v = which == 0 ? F.rhs0 : (which == 1 ? F.x0 : F.res0);
    const int b = F.goff[t.y], e = F.goff[t.y + 1];
    double acc = 0.0;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) acc += v[F.gmem[k]];
    double s = bsum(acc, sh);
    if (threadIdx.x == 0) mean = (float)(s / (double)(e - b));
    __syncthreads();
    const float m = mean;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) v[F.gmem[k]] -= m;
    __syncthreads();
  }
}

// Gauss-Seidel rows of one colour, RPI consecutive rows of the colour block per work item:
// every row's entries are loaded before any row is stored (rows of one colour never read
// each other), entries are summed in ELL order as every other path does. skipx: the first
// colour of the cycle's first sweep, whose neighbours are all zero, takes x = rhs / diag
// (the same bits as summing the zero products).
constexpr int RPI = 4;
// Entry a of a bin-stencil row (CLev::scode): its column (padding: the row `self`) and
// value. ob: the row's slot in the other colour's half (same bin row, same slot); par:
// the parity of the row's bin index along x.
__device__ __forceinline__ void bin_entry(const CLev& L, unsigned long long cw, int a, int ob, int par, int self,
                                          int& col, float& val) {
  const unsigned e = (unsigned)(cw >> (7 * a)) & 127u;
  const int dir = (int)(e & 7u), nbh = L.snbh, nz = L.snb1y * L.snbh;
  const int off = dir == 0 ? par - 1 : dir == 1 ? par : dir == 2 ? -nbh : dir == 3 ? nbh : dir == 4 ? -nz : nz;
  col = dir == 7 ? self : ob + off;
  val = dir == 7 ? 0.0f : __ldg(&L.svt[e >> 3]);
}
constexpr unsigned long long BIN_PAD = 0x3870e1c387ull;  // direction 7 (padding) in all six entries
static_assert(((BIN_PAD >> 35) & 127u) == 7u && (BIN_PAD >> 42) == 0, "six padding codes");

__device__ __forceinline__ void gs_rows(const CLev& L, int color, int k, bool skipx) {
  const int c0 = L.coff[color];
  const int nrow = L.coff[color + 1] - c0;
  const int q = RPI * k;
  if (q >= nrow) return;
  float v[RPI], d[RPI];
#pragma unroll
  for (int r = 0; r < RPI; ++r) {
    const bool ok = q + r < nrow;
    v[r] = ok ? __ldcg(&L.rhs[c0 + q + r]) : 0.0f;
    d[r] = ok ? L.idiag[c0 + q + r] : 0.0f;
  }
  if (!skipx && L.scode) {
    // Bin stencil: the codes of the item's rows (one bin row: nbh is a multiple of RPI),
    // then every entry's column computed and all gathers issued; the same entries, values
    // and fmaf order as the ELL rows below.
    const int nbh = L.snbh, R = q / nbh;
    const int par = (color + R % L.snb1y + R / L.snb1y) & 1;
    const int ob = (1 - color) * L.coff[1] + R * nbh + (q - R * nbh);
    const int w = L.ell_w[color];
    unsigned long long cw[RPI];
#pragma unroll
    for (int r = 0; r < RPI; ++r) cw[r] = q + r < nrow ? __ldg(&L.scode[c0 + q + r]) : BIN_PAD;
#pragma unroll
    for (int a = 0; a < 6; ++a)
      if (a < w) {
        float xv[RPI], wv[RPI];
#pragma unroll
        for (int r = 0; r < RPI; ++r) {
          int col;
          bin_entry(L, cw[r], a, ob + r, par, q + r < nrow ? c0 + q + r : c0 + q, col, wv[r]);
          xv[r] = __ldcg(&L.x[col]);
        }
#pragma unroll
        for (int r = 0; r < RPI; ++r) v[r] = fmaf(-wv[r], xv[r], v[r]);
      }
  } else if (!skipx) {
    const int base = L.ell_off[color], w = L.ell_w[color];
    const int* ec = L.ell_col + base + q;
    const float* ev = L.ell_val + base + q;
    // Software-pipelined: entry a+1's columns and values load while entry a's x gathers.
    int col[RPI];
    float wv[RPI];
#pragma unroll
    for (int r = 0; r < RPI; ++r) {
      const bool ok = q + r < nrow && w > 0;
      col[r] = ok ? ec[r] : c0 + q;
      wv[r] = ok ? ev[r] : 0.0f;
    }
#pragma unroll 1
    for (int a = 0; a < w; ++a) {
      float xv[RPI];
#pragma unroll
      for (int r = 0; r < RPI; ++r) xv[r] = __ldcg(&L.x[col[r]]);
      float wc[RPI];
#pragma unroll
      for (int r = 0; r < RPI; ++r) wc[r] = wv[r];
      if (a + 1 < w) {
#pragma unroll
        for (int r = 0; r < RPI; ++r) {
          const bool ok = q + r < nrow;
          col[r] = ok ? ec[(a + 1) * nrow + r] : c0 + q;
          wv[r] = ok ? ev[(a + 1) * nrow + r] : 0.0f;
        }
      }
#pragma unroll
      for (int r = 0; r < RPI; ++r) v[r] = fmaf(-wc[r], xv[r], v[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < RPI; ++r)
    if (q + r < nrow) L.x[c0 + q + r] = v[r] * d[r];
}

// The residual of a res0 level on colour 0, RPI rows per item through the colour's ELL
// block: res = rhs - (diag x + sum a x) with the entries in ELL order.
__device__ __forceinline__ void res0_rows(const CLev& L, int k) {
  const int nrow = L.coff[1];  // colour 0 owns rows 0 .. coff[1]-1
  const int q = RPI * k;
  if (q >= nrow) return;
  float v[RPI];
#pragma unroll
  for (int r = 0; r < RPI; ++r) v[r] = q + r < nrow ? L.diag[q + r] * __ldcg(&L.x[q + r]) : 0.0f;
  if (L.scode) {  // bin stencil (gs_rows): the same entries in the same order
    const int nbh = L.snbh, R = q / nbh;
    const int par = (R % L.snb1y + R / L.snb1y) & 1;
    const int ob = nrow + R * nbh + (q - R * nbh);
    const int w = L.ell_w[0];
    unsigned long long cw[RPI];
#pragma unroll
    for (int r = 0; r < RPI; ++r) cw[r] = q + r < nrow ? __ldg(&L.scode[q + r]) : BIN_PAD;
#pragma unroll
    for (int a = 0; a < 6; ++a)
      if (a < w) {
        float xv[RPI], wv[RPI];
#pragma unroll
        for (int r = 0; r < RPI; ++r) {
          int col;
          bin_entry(L, cw[r], a, ob + r, par, q + r < nrow ? q + r : q, col, wv[r]);
          xv[r] = __ldcg(&L.x[col]);
        }
#pragma unroll
        for (int r = 0; r < RPI; ++r) v[r] = fmaf(wv[r], xv[r], v[r]);
      }
#pragma unroll
    for (int r = 0; r < RPI; ++r)
      if (q + r < nrow) L.res[q + r] = __ldcg(&L.rhs[q + r]) - v[r];
    return;
  }
  const int base = L.ell_off[0], w = L.ell_w[0];
  const int* ec = L.ell_col + base + q;
  const float* ev = L.ell_val + base + q;
  int col[RPI];
  float wv[RPI];
#pragma unroll
  for (int r = 0; r < RPI; ++r) {
    const bool ok = q + r < nrow && w > 0;
    col[r] = ok ? ec[r] : q;
    wv[r] = ok ? ev[r] : 0.0f;
  }
#pragma unroll 1
  for (int a = 0; a < w; ++a) {
    float xv[RPI];
#pragma unroll
    for (int r = 0; r < RPI; ++r) xv[r] = __ldcg(&L.x[col[r]]);
    float wc[RPI];
#pragma unroll
    for (int r = 0; r < RPI; ++r) wc[r] = wv[r];
    if (a + 1 < w) {
#pragma unroll
      for (int r = 0; r < RPI; ++r) {
        const bool ok = q + r < nrow;
        col[r] = ok ? ec[(a + 1) * nrow + r] : q;
        wv[r] = ok ? ev[(a + 1) * nrow + r] : 0.0f;
      }
    }
#pragma unroll
    for (int r = 0; r < RPI; ++r) v[r] = fmaf(wc[r], xv[r], v[r]);
  }
#pragma unroll
  for (int r = 0; r < RPI; ++r)
    if (q + r < nrow) L.res[q + r] = __ldcg(&L.rhs[q + r]) - v[r];
}

// Rows of a level that the prolongation must update: on Gauss-Seidel levels the last colour
// (the first one the post-smoothing sweeps, backward) is rewritten without being read, so
// its rows (the last colour block) are skipped; l1-Jacobi levels read every row.
__device__ __forceinline__ int prolong_rows(const CLev& L) {
  return L.jacobi ? L.n : L.coff[L.ncolors - 1];
}

// ----------------------------------------------------------------- coarse levels, one cluster per case
__device__ __forceinline__ void csync() { cg::this_cluster().sync(); }

__device__ void c_center(const CLev& L, float* v, double* gpart, double* sh) {
  if (L.ngroups == 0) return;
  const int rank = (int)cg::this_cluster().block_rank();
  const int CSZ = (int)cg::this_cluster().num_blocks();
  for (int g = 0; g < L.ngroups; ++g) {
    const int b = L.goff[g], e = L.goff[g + 1];
    const int len = e - b, seg = (len + CSZ - 1) / CSZ;
    const int sb = b + rank * seg, se = min(e, sb + seg);
    double acc = 0.0;
    for (int k = sb + threadIdx.x; k < se; k += blockDim.x) acc += __ldcg(&v[L.gmem[k]]);
    double s = bsum(acc, sh);
    if (threadIdx.x == 0) gpart[g * CSZ + rank] = s;
  }
  __threadfence();
  csync();
  const int tid = rank * blockDim.x + threadIdx.x, nth = CSZ * blockDim.x;
  for (int g = 0; g < L.ngroups; ++g) {
    double s = 0.0;
    for (int r = 0; r < CSZ; ++r) s += __ldcg(&gpart[g * CSZ + r]);
    const int b = L.goff[g], e = L.goff[g + 1];
    const float mean = (float)(s / (double)(e - b));
    for (int k = b + tid; k < e; k += nth) v[L.gmem[k]] = __ldcg(&v[L.gmem[k]]) - mean;
  }
  __threadfence();
  csync();
}

__device__ void c_sweep(const CLev& L, bool backward, int pass, bool gs_on) {
  const int rank = (int)cg::this_cluster().block_rank();
  const int tid = rank * blockDim.x + threadIdx.x, nth = (int)cg::this_cluster().num_blocks() * blockDim.x;
  if (!L.jacobi && !gs_on) return;
  if (L.jacobi) {  // l1-Jacobi, x -> x2 (pass 0) -> x (pass 1)
    const float* xin = pass ? L.x2 : L.x;
    float* xout = pass ? L.x : L.x2;
    const int w = L.ell_w[0];
    for (int i = tid; i < L.n; i += nth) {
      float v = 0.0f;
      for (int a = 0; a < w; ++a) v = fmaf(L.ell_val[a * L.n + i], __ldcg(&xin[L.ell_col[a * L.n + i]]), v);
      const float xi = __ldcg(&xin[i]);
      xout[i] = fmaf(L.il1[i], __ldcg(&L.rhs[i]) - fmaf(L.diag[i], xi, v), xi);
    }
    __threadfence();
    csync();
    return;
  }
  for (int cc = 0; cc < L.ncolors; ++cc) {
    const int color = backward ? L.ncolors - 1 - cc : cc;
    const int b = L.coff[color], nrow = L.coff[color + 1] - b;
    const int base = L.ell_off[color], w = L.ell_w[color];
    for (int t = tid; t < nrow; t += nth) {
      const int i = b + t;  // colour blocks are contiguous
      const float id = L.idiag[i];
      float v = __ldcg(&L.rhs[i]);
      for (int a = 0; a < w; ++a) {
        const int e = base + a * nrow + t;
        v = fmaf(-L.ell_val[e], __ldcg(&L.x[L.ell_col[e]]), v);
      }
      L.x[i] = v * id;
    }
    __threadfence();
    csync();
  }
}

// nu: Gauss-Seidel sweeps before and after the coarse correction (l1-Jacobi levels run
// the next even count, so their iterate ends in x).
__global__ void __launch_bounds__(CT) k_coarse(const CCase* cases, const MState* ST, int nu) {
  __shared__ double sh[32];
  const int csz = (int)cg::this_cluster().num_blocks();
  const int ci = blockIdx.x / csz;
  const MState& S = ST[ci];
  if (!(S.state == RUN || S.state == START)) return;  // uniform over the cluster
  const CCase& C = cases[ci];
  const int rank = (int)cg::this_cluster().block_rank();
  const int tid = rank * blockDim.x + threadIdx.x, nth = csz * blockDim.x;
  int l = 0;
  for (; l < C.nl; ++l) {
    const CLev& L = C.lv[l];
    c_center(L, L.rhs, C.gpart, sh);
    for (int i = tid; i < L.n; i += nth) L.x[i] = 0.0f;
    __threadfence();
    csync();
    if (L.terminal) {
      // x_idx = (L L^T)^-1 rhs_idx in FP64 (the block inverses formed on the host).
      for (int q = tid; q < L.nblocks * 32; q += nth) {
        const int bk = q >> 5, ln = q & 31;
        const int* ix = L.idx + L.ioff[bk];
        const int n = L.ioff[bk + 1] - L.ioff[bk];
        if (ln >= n) continue;
        const double* m = L.fac + L.foff[bk];
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc = fma(m[ln * n + j], (double)__ldcg(&L.rhs[ix[j]]), acc);
        L.x[ix[ln]] = (float)acc;
      }
      __threadfence();
      csync();
      c_center(L, L.x, C.gpart, sh);
      break;
    }
    for (int sw = 0; sw < nu + (nu & 1); ++sw) c_sweep(L, false, sw & 1, sw < nu);
    c_center(L, L.x, C.gpart, sh);
    if (L.res0) {
      for (int k = tid; k < (L.coff[1] + RPI - 1) / RPI; k += nth) res0_rows(L, k);
    } else {
      for (int i = tid; i < L.n; i += nth) {
        float v = L.diag[i] * __ldcg(&L.x[i]);
        v = gather_sum(L.col, L.val, L.x, L.off[i], L.off[i + 1], v);
        L.res[i] = __ldcg(&L.rhs[i]) - v;
      }
    }
    __threadfence();
    csync();
    c_center(L, L.res, C.gpart, sh);
    const CLev& N = C.lv[l + 1];
    for (int j = tid; j < N.n; j += nth) {
      float v = 0.0f;
      v = gather_sum(L.rchild, L.rw, L.res, L.roff[j], L.roff[j + 1], v);
      N.rhs[j] = v;
    }
    __threadfence();
    csync();
  }
  for (int m = min(l, C.nl - 1) - 1; m >= 0; --m) {
    const CLev& L = C.lv[m];
    const CLev& N = C.lv[m + 1];
    for (int i = tid; i < prolong_rows(L); i += nth) {
      float s = 0.0f;
      s = gather_sum(L.pcol, L.pw, N.x, L.poff[i], L.poff[i + 1], s);
      L.x[i] = __ldcg(&L.x[i]) + s;
    }
    __threadfence();
    csync();
    for (int sw = 0; sw < nu + (nu & 1); ++sw) c_sweep(L, true, sw & 1, sw < nu);
    c_center(L, L.x, C.gpart, sh);
  }
}

// ----------------------------------------------------------------- coarse levels, whole grid
// All coarse levels of every case in one cooperative launch: each phase of the cycle
// spreads the rows of all cases over the whole grid (a global index space of per-case
// row ranges) and the phases are separated by grid-wide barriers.
constexpr int MAXC = 32;  // colours per level
constexpr long long BLK_WORK = 24576;  // rows + stencil entries a single block smooths (block-local levels)

struct CoarseTab {
  int nc, nlev;
  int nu;  // sweeps before and after the coarse correction
  int lb;  // first level (lv index) that every case runs inside one block
  int maxc[MAXL];
  int anyg[MAXL];
  const int* rows;   // [nlev][nc+1] prefix over cases of the rows of level l
  const int* term;   // [nlev][nc+1] terminal blocks at level l
  const int* fwd;    // [nlev][MAXC][nc+1] rows of colour c (non-terminal levels)
  const int* bwd;    // [nlev][MAXC][nc+1] rows of colour C_case-1-c
  const int* next;   // [nlev][nc+1] rows of level l+1 (restriction targets; non-terminal at l)
  const int* live;   // [nlev][nc+1] rows of level l when non-terminal (prolongation)
  const int* res;    // [nlev][nc+1] residual work items: rows, or 8 lanes per row (l1-Jacobi levels)
  const int* grp;    // [nlev][nc+1] closed groups at level l
};

__device__ __forceinline__ int find_case(const int* off, int nc, int t) {
  int lo = 0, hi = nc;  // off[lo] <= t < off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&off[mid]) <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// The case of global item t, remembering the last case's range (a thread's items
// advance by the grid size, so consecutive ones usually share a case).
struct CaseCursor {
  int ci = -1, lo = 0, hi = 0;
};
__device__ __forceinline__ int case_at(const int* off, int nc, int t, CaseCursor& cur) {
  if (t >= cur.lo && t < cur.hi) return cur.ci;
  cur.ci = find_case(off, nc, t);
  cur.lo = __ldg(&off[cur.ci]);
  cur.hi = __ldg(&off[cur.ci + 1]);
  return cur.ci;
}

__device__ __forceinline__ bool active(const MState* ST, int ci) {
  const int st = ST[ci].state;
  return st == RUN || st == START;
}

// The descriptors of the current level (sl[0..nc)) and of the next (sl[nc..2nc)) are
// copied into shared memory at each level, so the phases read them without global
// round trips.
__device__ void load_levels(const CCase* cases, int nc, int l, int nlev_max, CLev* sl) {
  __syncthreads();
  const int words = (int)(sizeof(CLev) / 8);
  for (int w = threadIdx.x; w < 2 * nc * words; w += blockDim.x) {
    const int which = w / (nc * words), rem = w % (nc * words);
    const int ci = rem / words, k = rem % words;
    const int lev = l + which;
    long long v = 0;
    if (lev < nlev_max) v = reinterpret_cast<const long long*>(&cases[ci].lv[lev])[k];
    reinterpret_cast<long long*>(&sl[which * nc + ci])[k] = v;
  }
  __syncthreads();
}

// Subtracts each closed group's mean, one CTA per (case, group) pair.
__device__ void g_center(const CLev* sl, const MState* ST, const CoarseTab& T, int l, int which, double* sh,
                         cg::grid_group& grid) {
  const int* off = T.grp + l * (T.nc + 1);
  const int total = __ldg(&off[T.nc]);
  __shared__ float mean;
  for (int t = blockIdx.x; t < total; t += gridDim.x) {
    const int ci = find_case(off, T.nc, t);
    if (!active(ST, ci)) continue;
    const CLev& L = sl[ci];
    float* v = which == 0 ? L.rhs : (which == 1 ? L.x : L.res);
    const int g = t - off[ci];
    const int b = L.goff[g], e = L.goff[g + 1];
    double acc = 0.0;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) acc += __ldcg(&v[L.gmem[k]]);
    double s = bsum(acc, sh);
    if (threadIdx.x == 0) mean = (float)(s / (double)(e - b));
    __syncthreads();
    const float m = mean;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) v[L.gmem[k]] = __ldcg(&v[L.gmem[k]]) - m;
    __syncthreads();
  }
  grid.sync();
}

__device__ void g_sweep(const CLev* sl, const MState* ST, const CoarseTab& T, int l, bool backward, int pass,
                        bool gs_on, bool first, cg::grid_group& grid) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int cc = 0; cc < T.maxc[l]; ++cc) {
    const int* off = (backward ? T.bwd : T.fwd) + (l * MAXC + cc) * (T.nc + 1);
    const int total = __ldg(&off[T.nc]);
    CaseCursor cur;
    bool on = false;
    for (int t = gt; t < total; t += nth) {
      const int prev = cur.ci;
      const int ci = case_at(off, T.nc, t, cur);
      if (ci != prev) on = active(ST, ci);
      if (!on) continue;
      const CLev& L = sl[ci];
      const int k = t - cur.lo;
      if (!L.jacobi && !gs_on) continue;
      if (L.jacobi) {
        // One sweep x_out = x_in + (rhs - A x_in) / (diag + sum |a_ij|); eight lanes per
        // row (the ranges of such cases start at multiples of eight), x -> x2 -> x.
        const int i = k >> 3, sub = k & 7;
        const float* xin = pass ? L.x2 : L.x;
        float* xout = pass ? L.x : L.x2;
        const int w = L.ell_w[0];
        const int* ec = L.ell_col + i;
        const float* ev = L.ell_val + i;
        float v = 0.0f;
        for (int a = sub; a < w; a += 8) v = fmaf(ev[a * L.n], __ldcg(&xin[ec[a * L.n]]), v);
        const unsigned mask = 0xffu << (threadIdx.x & 24);
        v += __shfl_xor_sync(mask, v, 4, 8);
        v += __shfl_xor_sync(mask, v, 2, 8);
        v += __shfl_xor_sync(mask, v, 1, 8);
        if (sub == 0) {
          const float xi = __ldcg(&xin[i]);
          xout[i] = fmaf(L.il1[i], __ldcg(&L.rhs[i]) - fmaf(L.diag[i], xi, v), xi);
        }
        continue;
      }
      gs_rows(L, backward ? L.ncolors - 1 - cc : cc, k, first && !backward && cc == 0);
    }
    grid.sync();
  }
}

// ----------------------------------------------------------------- block-local coarse levels
// The small coarse levels of one case, smoothed by one block with block barriers. Every
// row sees the same operations in the same order as in the grid-wide phases, so a case
// gives the same bits whichever levels run block-locally.
__device__ void blk_center(const CLev& L, float* v, double* sh) {
  __shared__ float mean;
  for (int g = 0; g < L.ngroups; ++g) {
    const int b = L.goff[g], e = L.goff[g + 1];
    double acc = 0.0;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) acc += __ldcg(&v[L.gmem[k]]);
    const double s = bsum(acc, sh);
    if (threadIdx.x == 0) mean = (float)(s / (double)(e - b));
    __syncthreads();
    const float m = mean;
    for (int k = b + threadIdx.x; k < e; k += blockDim.x) v[L.gmem[k]] = __ldcg(&v[L.gmem[k]]) - m;
    __syncthreads();
  }
}

__device__ void blk_sweep(const CLev& L, bool backward, int pass, bool gs_on, bool first) {
  if (L.jacobi) {
    const float* xin = pass ? L.x2 : L.x;
    float* xout = pass ? L.x : L.x2;
    const int w = L.ell_w[0];
    // Eight lanes per row, as in the grid-wide phase.
    for (int k = threadIdx.x; k < 8 * L.n; k += blockDim.x) {
      const int i = k >> 3, sub = k & 7;
      float v = 0.0f;
      for (int a = sub; a < w; a += 8) v = fmaf(L.ell_val[a * L.n + i], __ldcg(&xin[L.ell_col[a * L.n + i]]), v);
      const unsigned mask = 0xffu << (threadIdx.x & 24);
      v += __shfl_xor_sync(mask, v, 4, 8);
      v += __shfl_xor_sync(mask, v, 2, 8);
      v += __shfl_xor_sync(mask, v, 1, 8);
      if (sub == 0) {
        const float xi = __ldcg(&xin[i]);
        xout[i] = fmaf(L.il1[i], __ldcg(&L.rhs[i]) - fmaf(L.diag[i], xi, v), xi);
      }
    }
    __syncthreads();
    return;
  }
  if (!gs_on) return;
  for (int cc = 0; cc < L.ncolors; ++cc) {
    const int color = backward ? L.ncolors - 1 - cc : cc;
    const int items = (L.coff[color + 1] - L.coff[color] + RPI - 1) / RPI;
    for (int k = threadIdx.x; k < items; k += blockDim.x) gs_rows(L, color, k, first && !backward && cc == 0);
    __syncthreads();
  }
}

// Terminal level: x_idx = (L L^T)^-1 rhs_idx in FP64, one warp per block (as the grid-wide phase).
__device__ __forceinline__ void terminal_block(const CLev& L, int bk, int ln) {
  const int* ix = L.idx + L.ioff[bk];
  const int n = L.ioff[bk + 1] - L.ioff[bk];
  const double* m = L.fac + L.foff[bk];
  const double rj = ln < n ? (double)__ldcg(&L.rhs[ix[ln]]) : 0.0;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  for (int j = 0; j < n; j += 4) {
    const double r0 = __shfl_sync(0xffffffffu, rj, j);
    const double r1 = __shfl_sync(0xffffffffu, rj, j + 1 < 32 ? j + 1 : 31);
    const double r2 = __shfl_sync(0xffffffffu, rj, j + 2 < 32 ? j + 2 : 31);
    const double r3 = __shfl_sync(0xffffffffu, rj, j + 3 < 32 ? j + 3 : 31);
    if (ln < n) {
      a0 = fma(m[ln * n + j], r0, a0);
      if (j + 1 < n) a1 = fma(m[ln * n + j + 1], r1, a1);
      if (j + 2 < n) a2 = fma(m[ln * n + j + 2], r2, a2);
      if (j + 3 < n) a3 = fma(m[ln * n + j + 3], r3, a3);
    }
  }
  if (ln < n) L.x[ix[ln]] = (float)((a0 + a1) + (a2 + a3));
}

// Levels l0 .. of case C, down to the terminal level and back up to l0.
__device__ void blk_cycle(const CCase& C, int l0, int nu, double* sh) {
  int l = l0;
  for (; l < C.nl; ++l) {
    const CLev& L = C.lv[l];
    blk_center(L, L.rhs, sh);
    for (int i = threadIdx.x; i < L.n; i += blockDim.x) L.x[i] = 0.0f;
    __syncthreads();
    if (L.terminal) {
      for (int t = threadIdx.x >> 5; t < L.nblocks; t += blockDim.x >> 5) terminal_block(L, t, threadIdx.x & 31);
      __syncthreads();
      blk_center(L, L.x, sh);
      break;
    }
    for (int sw = 0; sw < nu + (nu & 1); ++sw) blk_sweep(L, false, sw & 1, sw < nu, sw == 0);
    blk_center(L, L.x, sh);
    const int nres = L.res0 ? (L.coff[1] + RPI - 1) / RPI : (L.jacobi ? 8 : 1) * L.n;
    for (int k = threadIdx.x; k < nres; k += blockDim.x) {
      if (L.res0) {
        res0_rows(L, k);
      } else if (L.jacobi) {
        const int i = k >> 3, sub = k & 7;
        float v = 0.0f;
        for (int a = L.off[i] + sub; a < L.off[i + 1]; a += 8) v = fmaf(L.val[a], __ldcg(&L.x[L.col[a]]), v);
        const unsigned mask = 0xffu << (threadIdx.x & 24);
        v += __shfl_xor_sync(mask, v, 4, 8);
        v += __shfl_xor_sync(mask, v, 2, 8);
        v += __shfl_xor_sync(mask, v, 1, 8);
        if (sub == 0) L.res[i] = __ldcg(&L.rhs[i]) - fmaf(L.diag[i], __ldcg(&L.x[i]), v);
      } else {
        const int i = k;
        float v = L.diag[i] * __ldcg(&L.x[i]);
        v = gather_sum(L.col, L.val, L.x, L.off[i], L.off[i + 1], v);
        L.res[i] = __ldcg(&L.rhs[i]) - v;
      }
    }
    __syncthreads();
    blk_center(L, L.res, sh);
    const CLev& N = C.lv[l + 1];
    for (int j = threadIdx.x; j < N.n; j += blockDim.x) {
      float v = 0.0f;
      v = gather_sum(L.rchild, L.rw, L.res, L.roff[j], L.roff[j + 1], v);
      N.rhs[j] = v;
    }
    __syncthreads();
  }
  for (int m = min(l, C.nl - 1) - 1; m >= l0; --m) {
    const CLev& L = C.lv[m];
    const CLev& N = C.lv[m + 1];
    for (int i = threadIdx.x; i < prolong_rows(L); i += blockDim.x) {
      float s = 0.0f;
      s = gather_sum(L.pcol, L.pw, N.x, L.poff[i], L.poff[i + 1], s);
      L.x[i] = __ldcg(&L.x[i]) + s;
    }
    __syncthreads();
    for (int sw = 0; sw < nu + (nu & 1); ++sw) blk_sweep(L, true, sw & 1, sw < nu, false);
    blk_center(L, L.x, sh);
  }
}

__global__ void __launch_bounds__(512, 2) k_coarse_all(const CCase* cases, const MState* ST, const CoarseTab* Tp) {
  const CoarseTab T = *Tp;
  __shared__ double sh[32];
  extern __shared__ __align__(16) unsigned char smem[];
  CLev* sl = reinterpret_cast<CLev*>(smem);
  cg::grid_group grid = cg::this_grid();
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  const int nc = T.nc;
  const int gl = min(T.nlev, T.lb);  // levels 0 .. gl-1 grid-wide
  for (int l = 0; l < gl; ++l) {
    load_levels(cases, nc, l, MAXL, sl);
    if (T.anyg[l]) g_center(sl, ST, T, l, 0, sh, grid);
    {
      const int* off = T.rows + l * (nc + 1);
      CaseCursor cur;
      bool on = false;
      for (int t = gt; t < __ldg(&off[nc]); t += nth) {
        const int prev = cur.ci;
        const int ci = case_at(off, nc, t, cur);
        if (ci != prev) on = active(ST, ci);
        if (on) sl[ci].x[t - cur.lo] = 0.0f;
      }
    }
    grid.sync();
    if (__ldg(&T.term[l * (nc + 1) + nc]) > 0) {  // the same for every block
      // Terminal levels: x_idx = (L L^T)^-1 rhs_idx in FP64, one warp per block.
      const int* off = T.term + l * (nc + 1);
      const int wp = gt >> 5, nw = nth >> 5, ln = threadIdx.x & 31;
      for (int t = wp; t < __ldg(&off[nc]); t += nw) {
        const int ci = find_case(off, nc, t);
        if (!active(ST, ci)) continue;
        terminal_block(sl[ci], t - __ldg(&off[ci]), ln);
      }
      grid.sync();
    }
    for (int sw = 0; sw < T.nu + (T.nu & 1); ++sw) g_sweep(sl, ST, T, l, false, sw & 1, sw < T.nu, sw == 0, grid);
    if (T.anyg[l]) g_center(sl, ST, T, l, 1, sh, grid);
    {
      const int* off = T.res + l * (nc + 1);
      CaseCursor cur;
      bool on = false;
      for (int t = gt; t < __ldg(&off[nc]); t += nth) {
        const int prev = cur.ci;
        const int ci = case_at(off, nc, t, cur);
        if (ci != prev) on = active(ST, ci);
        if (!on) continue;
        const CLev& L = sl[ci];
        const int k = t - cur.lo;
        if (L.res0) {
          res0_rows(L, k);
          continue;
        }
        if (L.jacobi) {  // eight lanes per (wide) row
          const int i = k >> 3, sub = k & 7;
          float v = 0.0f;
          for (int a = L.off[i] + sub; a < L.off[i + 1]; a += 8) v = fmaf(L.val[a], __ldcg(&L.x[L.col[a]]), v);
          const unsigned mask = 0xffu << (threadIdx.x & 24);
          v += __shfl_xor_sync(mask, v, 4, 8);
          v += __shfl_xor_sync(mask, v, 2, 8);
          v += __shfl_xor_sync(mask, v, 1, 8);
          if (sub == 0) L.res[i] = __ldcg(&L.rhs[i]) - fmaf(L.diag[i], __ldcg(&L.x[i]), v);
          continue;
        }
        if (k >= L.n) continue;
        const int i = k;
        float v = L.diag[i] * __ldcg(&L.x[i]);
        v = gather_sum(L.col, L.val, L.x, L.off[i], L.off[i + 1], v);
        L.res[i] = __ldcg(&L.rhs[i]) - v;
      }
    }
    grid.sync();
    if (T.anyg[l]) g_center(sl, ST, T, l, 2, sh, grid);
    {
      const int* off = T.next + l * (nc + 1);
      CaseCursor cur;
      bool on = false;
      for (int t = gt; t < __ldg(&off[nc]); t += nth) {
        const int prev = cur.ci;
        const int ci = case_at(off, nc, t, cur);
        if (ci != prev) on = active(ST, ci);
        if (!on) continue;
        const CLev& L = sl[ci];
        const CLev& N = sl[nc + ci];
        const int j = t - cur.lo;
        float v = 0.0f;
        v = gather_sum(L.rchild, L.rw, L.res, L.roff[j], L.roff[j + 1], v);
        N.rhs[j] = v;
      }
    }
    grid.sync();
  }
  if (gl < T.nlev) {
    // The remaining levels of every case inside one block each.
    for (int ci = blockIdx.x; ci < nc; ci += gridDim.x)
      if (active(ST, ci) && cases[ci].nl > gl) blk_cycle(cases[ci], gl, T.nu, sh);
    __threadfence();
    grid.sync();
  }
  for (int l = min(T.nlev - 2, gl - 1); l >= 0; --l) {
    load_levels(cases, nc, l, MAXL, sl);
    {
      const int* off = T.live + l * (nc + 1);
      CaseCursor cur;
      bool on = false;
      for (int t = gt; t < __ldg(&off[nc]); t += nth) {
        const int prev = cur.ci;
        const int ci = case_at(off, nc, t, cur);
        if (ci != prev) on = active(ST, ci);
        if (!on) continue;
        const CLev& L = sl[ci];
        const CLev& N = sl[nc + ci];
        const int i = t - cur.lo;
        float s = 0.0f;
        s = gather_sum(L.pcol, L.pw, N.x, L.poff[i], L.poff[i + 1], s);
        L.x[i] = __ldcg(&L.x[i]) + s;
      }
    }
    grid.sync();
    for (int sw = 0; sw < T.nu + (T.nu & 1); ++sw) g_sweep(sl, ST, T, l, true, sw & 1, sw < T.nu, false, grid);
    if (T.anyg[l]) g_center(sl, ST, T, l, 1, sh, grid);
  }
}

// ----------------------------------------------------------------- prologue / epilogue (FP64)
// b = -div(u)/dt, terms (pressure.rs:440-459), rounded as written.
__device__ __forceinline__ void b_rhs(const FineCase* FC, MState* ST, const int2 t, int& cached_) {
  FINE_PROLOGUE(S.state == IDLE)
  int j, k, rb;
  if (!warp_row(F, lt, warp, j, k, rb)) return;
  for (int i = lane; i < nx_; i += 32) {
    const int c = rb + i;
    if (!F.fluid[c]) {
      F.b[c] = -0.0;
      if (F.wbc) F.bc[c] = -0.0;
      F.terms[c] = 0.0;
      continue;
    }
    const int q[3] = {i, j, k};
    // The round-off scale only serves the compatibility check of closed components.
    const bool closed = F.ngroups > 0;
    double div = 0.0, scale = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      int p[3] = {q[0], q[1], q[2]};
      const double ul = F.u[fidx(F, a, p[0], p[1], p[2])];
      p[a] += 1;
      const double uu = F.u[fidx(F, a, p[0], p[1], p[2])];
      div = __dadd_rn(div, div_p2(__dsub_rn(uu, ul), F.dx[a]));
      if (closed) scale = __dadd_rn(scale, div_p2(__dadd_rn(fabs(ul), fabs(uu)), F.dx[a]));
    }
    const double bv = div_rdt(-div, F.dt, F.rdt);
    F.b[c] = bv;
    if (F.wbc) F.bc[c] = bv;  // no closed components: b_c is b (no gauge)
    F.terms[c] = closed ? div_rdt(scale, F.dt, F.rdt) : 0.0;
  }
}
__global__ void __launch_bounds__(TILE) k_rhs(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == IDLE)
    b_rhs(FC, ST, t, cached_);
  }
}

struct FinNorm {
  __device__ void operator()(MState& S, double bb) const {
    S.norm = sqrt(bb);
    S.has_e = 0;
    S.scale = 0.0;
    S.state = S.norm < 1e-24 ? DONE : OUTER;
  }
};

// |b_c| (after the host-side gauge of closed components); x = 0.
__device__ __forceinline__ void b_norm(const FineCase* FC, MState* ST, const int2 t, int& cached_, double* sh,
                                    int& seg_n) {
  FINE_PROLOGUE(S.state == IDLE)
  double acc = 0.0;
  for (int c = cb + threadIdx.x; c < ce; c += TILE) {
    const double v = F.bc[c];
    acc = __fma_rn(v, v, acc);
    F.x64[c] = 0.0;
  }
  for (int c = sb + threadIdx.x; c < se; c += TILE) F.e[c] = 0.0f;
  tile_partial(acc, F, lt, sh, seg_n);
}
__global__ void __launch_bounds__(TILE) k_norm(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  __shared__ double sh[32];
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  Seg g;
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == IDLE)
    if (t.x != g.ci) {
      close_seg(FC, ST, g, sh, FinNorm());
      g.ci = t.x;
    }
    b_norm(FC, ST, t, cached_, sh, g.n);
  }
  close_seg(FC, ST, g, sh, FinNorm());
}

// Face correction u -= dt grad(x) (pressure.rs:481-496), face tiles.
__global__ void k_correct(const FineCase* FC, const MState* ST, const int2* ftiles, const int* count) {
  const int n = *count;
  for (int ti = blockIdx.x; ti < n; ti += gridDim.x) {
    const int2 t = ftiles[ti];
    const FineCase& F = FC[t.x];
    if (ST[t.x].state != DONE) continue;
    const long long f0 = (long long)t.y * FTILE + threadIdx.x;
    for (int r = 0; r < FTILE / 256; ++r) {
      const long long ff = f0 + r * 256;
      if (ff >= F.F) break;
      double d;
      const uint8_t k = F.fkind[ff];
      if (k == INTERIOR) d = div_p2(__dsub_rn(F.x64[F.fhi[ff]], F.x64[F.flo[ff]]), F.fdist[ff]);
      else if (k == OUTLET) d = F.flo[ff] >= 0 ? div_p2(-F.x64[F.flo[ff]], F.fdist[ff]) : div_p2(F.x64[F.fhi[ff]], F.fdist[ff]);
      else d = 0.0;
      F.u[ff] = __fma_rn(-F.dt, d, F.u[ff]);  // one rounding (the FP64 pipe bounds this kernel)
    }
  }
}

__device__ __forceinline__ void b_addp(const FineCase* FC, MState* ST, const int2 t, int& cached_) {
  FINE_PROLOGUE(S.state == DONE)
  for (int c = cb + threadIdx.x; c < ce; c += TILE) F.pfield[c] = __dadd_rn(F.pfield[c], F.x64[c]);
}
__global__ void __launch_bounds__(TILE) k_addp(const FineCase* FC, MState* ST, const int2* tiles, const int* count) {
  TILE_RANGE
  int cached_ = -1;  // case whose descriptor is in shared memory
  for (int ti = t0_; ti < t1_; ++ti) {
    const int2 t = tiles[ti];
    SKIP_CASE(t, S_.state == DONE)
    b_addp(FC, ST, t, cached_);
  }
}

// ----------------------------------------------------------------- host side
void greedy_colors(const Csr& a, int n, std::vector<int32_t>& coff, std::vector<int32_t>& rows, int& ncolors) {
  std::vector<int> color(n, -1);
  ncolors = 0;
  std::vector<char> used;
  for (int i = 0; i < n; ++i) {
    used.assign(ncolors + 1, 0);
    for (int k = a.off[i]; k < a.off[i + 1]; ++k) {
      int j = a.col[k];
      if (j != i && color[j] >= 0) used[color[j]] = 1;
    }
    int c = 0;
    while (c < ncolors && used[c]) ++c;
    color[i] = c;
    ncolors = std::max(ncolors, c + 1);
  }
  coff.assign(ncolors + 1, 0);
  for (int i = 0; i < n; ++i) coff[color[i] + 1] += 1;
  for (int c = 0; c < ncolors; ++c) coff[c + 1] += coff[c];
  rows.assign(n, 0);
  std::vector<int32_t> fill(coff.begin(), coff.end() - 1);
  for (int i = 0; i < n; ++i) rows[fill[color[i]]++] = i;
}

// Two colours from a level's bin parity when it colours the graph properly (masked
// hierarchies); false otherwise (the caller falls back to the greedy colouring).
bool parity_colors(const Csr& a, const std::vector<uint8_t>& parity, int n, std::vector<int32_t>& coff,
                   std::vector<int32_t>& rows, int& ncolors) {
  if ((int)parity.size() != n) return false;
  for (int i = 0; i < n; ++i)
    for (int k = a.off[i]; k < a.off[i + 1]; ++k)
      if (a.col[k] != i && parity[a.col[k]] == parity[i]) return false;
  coff.assign(3, 0);
  for (int i = 0; i < n; ++i) coff[parity[i] + 1] += 1;
  coff[2] += coff[1];
  rows.assign(n, 0);
  int fill[2] = {0, coff[1]};
  for (int i = 0; i < n; ++i) rows[fill[parity[i]]++] = i;
  ncolors = coff[1] > 0 && coff[2] > coff[1] ? 2 : 1;
  if (ncolors == 1) coff.resize(2), coff[1] = n;
  return true;
}

template <class T>
std::vector<float> to_f32(const std::vector<T>& v) {
  return std::vector<float>(v.begin(), v.end());
}

struct CaseState {
  cfdg_grid* G = nullptr;
  uint64_t version = 0;  // the grid's faces_version this state was built from
  Arena arena;
  FineCase F{};
  CCase C{};
  std::vector<std::vector<int32_t>> colors;  // per coarse level: colour offsets (host copy)
  struct LevelStats {
    long long rows, nnz, ell, groups, blocks;
    int colors, jacobi;
    int stencil = 0;  // swept through bin-stencil codes
  };
  std::vector<LevelStats> stats;  // per coarse level (diagnostics)
  int ngroups0 = 0;
  ~CaseState() { arena.release(); }
};

// Row r of `a` becomes row prow[r] (entry order kept), columns c become pcol[c]; an
// empty map is the identity.
// Rows moved to prow[r] (of nout rows, -1: a's row count; rows no r maps to stay empty),
// columns renamed by pcol; every row keeps its entries in their order.
Csr permute_csr(const Csr& a, const std::vector<int32_t>& prow, const std::vector<int32_t>& pcol, int nout = -1) {
  Csr out;
  const int n = a.rows();
  const int m = nout < 0 ? n : nout;
  out.off.assign(m + 1, 0);
  for (int r = 0; r < n; ++r) out.off[(prow.empty() ? r : prow[r]) + 1] = a.off[r + 1] - a.off[r];
  for (int r = 0; r < m; ++r) out.off[r + 1] += out.off[r];
  out.col.resize(a.col.size());
  if (!a.val.empty()) out.val.resize(a.val.size());
  for (int r = 0; r < n; ++r) {
    int dst = out.off[prow.empty() ? r : prow[r]];
    for (int k = a.off[r]; k < a.off[r + 1]; ++k, ++dst) {
      out.col[dst] = pcol.empty() ? a.col[k] : pcol[a.col[k]];
      if (!a.val.empty()) out.val[dst] = a.val[k];
    }
  }
  return out;
}

// cuTensorMapEncodeTiled, fetched from the driver (the library links only the runtime).
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled tensor_map_encoder() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// A split-layout level-0 array as a 3-D tensor [rows][2 colours][nxh] (x fastest), read in
// boxes of one colour's half-rows of `box_rows` consecutive rows. The row length in bytes
// must be a multiple of 16 (nxh a multiple of 8 for 16-bit flags).
bool encode_split(CUtensorMap& m, const void* base, bool u16, int nxh, int rows, int box_rows) {
  EncodeTiled enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t es = u16 ? 2 : 4;
  const cuuint64_t dims[3] = {(cuuint64_t)nxh, 2, (cuuint64_t)rows};
  const cuuint64_t strides[2] = {(cuuint64_t)nxh * es, 2 * (cuuint64_t)nxh * es};
  const cuuint32_t box[3] = {(cuuint32_t)nxh, 1, (cuuint32_t)box_rows};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(&m, u16 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims,
             strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Builds the FP32 device copy of a grid's hierarchy for the mixed form (cached on the grid).
// Each coarse level is renumbered so that the rows of every smoother colour are
// contiguous (colour c owns rows [coff[c], coff[c+1])): sweeps then read the right-hand
// side, 1/diag and x of consecutive rows without an index list.
int build_case(cfdg_grid* G, CaseState& cs) {
  std::shared_ptr<Hierarchy> Hp;
  if (int e = mixed_host_hierarchy(G, Hp)) return e;
  const Hierarchy& H = *Hp;
  // Coarse corrections of an aggregation (masked) hierarchy are scaled by the grid's
  // over-correction factor (cfdg_grid_set_coarse_scale): the piecewise-constant
  // prolongation under-corrects smooth errors, and the scaled correction stays symmetric
  // (restriction unchanged) and positive definite for factors below 2.
  const float alpha = H.masked ? G->mx_alpha : 1.0f;
  HostGrid& h = G->h;
  cudaStream_t s = G->stream;
  Arena& A = cs.arena;
  A.ctx = G->ctx;
  FineCase& F = cs.F;
  for (int a = 0; a < 3; ++a) {
    F.n[a] = h.n[a];
    F.w32[a] = (float)G->g.w_in[a];
    F.wo32[a] = (float)G->g.w_out[a];
    F.w64[a] = G->g.w_in[a];
    F.wo64[a] = G->g.w_out[a];
    F.face_off[a] = h.face_offset[a];
    for (int d = 0; d < 3; ++d) F.fdim[a][d] = (int)h.face_dims[a][d];
    F.dx[a] = h.dx[a];
  }
  F.N = (int)h.cells;
  F.F = h.faces;
  F.uniform = G->uniform ? 1 : 0;
  F.flags = G->d_flags;
  F.fluid = G->d_fluid;
  F.fw64 = G->d_fw;
  F.diag64 = G->mg->levels[0].diag;
  F.fkind = G->d_kind;
  F.flo = G->d_lo;
  F.fhi = G->d_hi;
  F.fdist = G->d_dist;
  F.x64 = G->x;
  F.r64 = G->r;
  F.bc = G->bc;
  F.b = G->b;
  F.terms = G->terms;
  if (!G->uniform) {
    std::vector<float> w32(h.faces);
    for (int64_t f = 0; f < h.faces; ++f) w32[f] = (float)h.weight(f);
    float* d;
    if (int e = A.upload(&d, w32, s)) return e;
    F.fw32 = d;
  }
  const MgLevel& M0 = H.levels[0];
  if (!M0.lines.empty())
    return fail(CFDG_ERR_UNSUPPORTED,
                "mixed form: the line/plane block smoothers of anisotropic grids run in the plain form only");
  if ((int64_t)M0.diag.size() != (int64_t)h.cells)
    return fail(CFDG_ERR_UNSUPPORTED, "mixed form: level 0 must cover every cell");
  // The split layout of the level-0 FP32 arrays (slot of each cell, cell of each slot).
  const int nx = h.n[0], ny = h.n[1], rows = h.n[1] * h.n[2];
  F.nxh = (nx + 1) / 2;
  F.N2 = 2 * rows * F.nxh;
  std::vector<int32_t> slot(F.N), cell_of(F.N2, -1);
  for (int r = 0; r < rows; ++r) {
    const int rp = (r % ny + r / ny) & 1;
    for (int i = 0; i < nx; ++i) {
      const int c = r * nx + i, sl = lay(r, (i + rp) & 1, F.nxh, i >> 1);
      slot[c] = sl;
      cell_of[sl] = c;
    }
  }
  {
    std::vector<uint16_t> fl(F.N), fl2(F.N2, 0);
    CU(cudaMemcpyAsync(fl.data(), G->d_flags, sizeof(uint16_t) * F.N, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    std::vector<float> d32(F.N2, 0.0f), i32(F.N2, 0.0f);
    for (int c = 0; c < F.N; ++c) {
      const float d = (float)M0.diag[c];
      d32[slot[c]] = d;
      i32[slot[c]] = d == 0.0f ? 0.0f : 1.0f / d;
      fl2[slot[c]] = fl[c];
    }
    float *d, *id;
    uint16_t* f2;
    if (int e = A.upload(&d, d32, s)) return e;
    if (int e = A.upload(&id, i32, s)) return e;
    if (int e = A.upload(&f2, fl2, s)) return e;
    F.diag0 = d;
    F.idiag0 = id;
    F.flags0 = f2;
  }
  float** fv[] = {&F.e, &F.r32, &F.p, &F.q, &F.x0, &F.res0};
  for (float** v : fv) {
    if (int e = A.alloc(v, F.N2)) return e;
    CU(cudaMemsetAsync(*v, 0, sizeof(float) * F.N2, s));  // padding slots stay zero
  }
  // The cycle's right-hand side is the inner residual itself unless level 0 has
  // closed groups, whose gauge it would modify in place.
  if (M0.groups.rows() > 0) {
    if (int e = A.alloc(&F.rhs0, F.N2)) return e;
    CU(cudaMemsetAsync(F.rhs0, 0, sizeof(float) * F.N2, s));
  } else {
    F.rhs0 = F.r32;
  }
  // Tensor maps of the staged half sweep (k_rb_tma): uniform weights, whole 16-byte rows.
  F.tmaps = nullptr;
  if (F.uniform && F.nxh % 8 == 0 && F.nxh <= 256) {
    // Per stage height (8, 16, 32 rows): rhs0, idiag0, flags0 and x0 in boxes of that
    // height, x0 in boxes of two rows more.
    std::vector<CUtensorMap> maps(5 * RB_HEIGHTS);
    const int rows_all = h.n[1] * h.n[2];
    bool ok = true;
    for (int q = 0; q < RB_HEIGHTS && ok; ++q) {
      const int sr = RT << q;
      CUtensorMap* m = maps.data() + 5 * q;
      ok = encode_split(m[0], F.rhs0, false, F.nxh, rows_all, sr) &&
           encode_split(m[1], F.idiag0, false, F.nxh, rows_all, sr) &&
           encode_split(m[2], F.flags0, true, F.nxh, rows_all, sr) &&
           encode_split(m[3], F.x0, false, F.nxh, rows_all, sr) &&
           encode_split(m[4], F.x0, false, F.nxh, rows_all, sr + 2);
    }
    if (ok) {
      CUtensorMap* d = nullptr;
      if (int e = A.upload(&d, maps, s)) return e;
      F.tmaps = d;
    }
  }
  F.ntiles = (h.n[1] * h.n[2] + RT - 1) / RT;  // row tiles (one reduction partial each)
  if (int e = A.alloc(&F.partials, (size_t)F.ntiles * (TILE / 32))) return e;
  cs.ngroups0 = M0.groups.rows();
  F.ngroups = cs.ngroups0;
  F.wbc = G->ncomp_groups == 0 ? 1 : 0;
  if (F.ngroups) {
    int *o, *m;
    std::vector<int32_t> mem(M0.groups.col.size());
    for (size_t q = 0; q < mem.size(); ++q) mem[q] = slot[M0.groups.col[q]];
    if (int e = A.upload(&o, M0.groups.off, s)) return e;
    if (int e = A.upload(&m, mem, s)) return e;
    F.goff = o;
    F.gmem = m;
  }
  // Level 1 as the bin grid (FineCase::bin1) where the grid allows it: an aggregation
  // hierarchy of three or more levels, no closed groups on level 0, uniform weights with
  // whole colour pairs per row, injection prolongation and restriction with weight 1,
  // every aggregate inside one bin and no bin holding two; then the deeper non-terminal
  // levels on the same terms, each from the bins of the level above.
  F.bin1 = 0;
  // Bin levels: level l laid out as the grid of its 2x2x2 bins of level-(l-1) nodes (level
  // 0: the cells) where every level-l aggregate lies in one bin and no bin holds two. Row
  // of bin (I, J, K): colour*h + (K*nb[1] + J)*nbh + (I>>1), colour = (I+J+K)&1.
  struct BinLevel {
    bool on = false;
    int nb[3] = {0, 0, 0}, nbh = 0, h = 0;
    std::vector<int32_t> slot;                 // aggregate -> row
    std::vector<std::array<int32_t, 3>> bin;   // aggregate -> bin coordinates
  };
  std::vector<BinLevel> binl(H.levels.size());
  auto try_bins = [&](int l, const std::vector<std::array<int32_t, 3>>& child_xyz, const int child_n[3]) {
    const MgLevel& Mc = H.levels[l - 1];  // restriction rows: level-l aggregates
    const MgLevel& Ml = H.levels[l];
    BinLevel& B = binl[l];
    for (int a = 0; a < 3; ++a) B.nb[a] = (child_n[a] + 1) / 2;
    B.nbh = (B.nb[0] + 1) / 2;
    B.h = B.nb[1] * B.nb[2] * B.nbh;
    bool ok = Mc.restrict.rows() == Ml.n && (int)Ml.parity.size() == Ml.n;
    std::vector<char> used(2 * (size_t)B.h, 0);
    B.slot.assign(Ml.n, -1);
    B.bin.assign(Ml.n, {0, 0, 0});
    for (int a = 0; a < Ml.n && ok; ++a) {
      int row = -1;
      std::array<int32_t, 3> bb{-1, -1, -1};
      for (int q = Mc.restrict.off[a]; q < Mc.restrict.off[a + 1] && ok; ++q) {
        const std::array<int32_t, 3>& xyz = child_xyz[Mc.restrict.col[q]];
        const std::array<int32_t, 3> b{xyz[0] >> 1, xyz[1] >> 1, xyz[2] >> 1};
        ok = row < 0 || b == bb;
        if (row < 0 && ok) {
          bb = b;
          const int col = (b[0] + b[1] + b[2]) & 1;
          row = col * B.h + (b[2] * B.nb[1] + b[1]) * B.nbh + (b[0] >> 1);
          ok = Ml.parity[a] == col;
        }
      }
      ok = ok && row >= 0 && !used[row];
      if (ok) {
        used[row] = 1;
        B.slot[a] = row;
        B.bin[a] = bb;
      }
    }
    for (int a = 0; a < Ml.n && ok; ++a)
      for (int q = Ml.a.off[a]; q < Ml.a.off[a + 1] && ok; ++q)
        ok = Ml.a.col[q] == a || Ml.parity[Ml.a.col[q]] != Ml.parity[a];
    B.on = ok;
    if (!ok) B.slot.clear(), B.bin.clear();
  };
  if (G->mx_bins && H.masked && M0.groups.rows() == 0 && F.uniform && !(F.nxh & 1) && H.levels.size() >= 3) {
    bool ok = (int64_t)M0.prolong.rows() == (int64_t)F.N;
    for (int c = 0; c < F.N && ok; ++c) {
      const int n = M0.prolong.off[c + 1] - M0.prolong.off[c];
      ok = n == 0 || (n == 1 && M0.prolong.val[M0.prolong.off[c]] == 1.0);
    }
    for (size_t q = 0; q < M0.restrict.val.size() && ok; ++q) ok = M0.restrict.val[q] == 1.0;
    if (ok) {
      std::vector<std::array<int32_t, 3>> cells(F.N);
      for (int c = 0; c < F.N; ++c) cells[c] = {c % nx, (c / nx) % ny, c / (nx * ny)};
      try_bins(1, cells, h.n);
      // Deeper non-terminal levels while the level above is a bin level.
      for (int l = 2; l + 1 < (int)H.levels.size() && binl[l - 1].on; ++l) try_bins(l, binl[l - 1].bin, binl[l - 1].nb);
    }
    if (binl[1].on) {
      F.bin1 = 1;
      for (int a = 0; a < 3; ++a) F.nb1[a] = binl[1].nb[a];
      F.nbh1 = binl[1].nbh;
      F.h1 = binl[1].h;
    }
  }
  // Coarse levels 1 .. L-1: colouring (bin parity, else greedy; l1-Jacobi when more than
  // 8 colours), then every level renumbered colour by colour (level 1 of a bin1 grid by
  // its bin rows).
  CCase& C = cs.C;
  C.nl = (int)H.levels.size() - 1;
  if (C.nl < 1 || C.nl > MAXL) return fail(CFDG_ERR_UNSUPPORTED, "mixed form: unsupported hierarchy depth");
  std::vector<std::vector<int32_t>> perm(C.nl + 2), lcoff(C.nl + 1);
  std::vector<int> lcolors(C.nl + 1, 1), ljacobi(C.nl + 1, 0);
  for (int l = 1; l <= C.nl; ++l) {
    const MgLevel& M = H.levels[l];
    const bool terminal = l == C.nl;
    if (binl[l].on) {
      lcoff[l] = {0, binl[l].h, 2 * binl[l].h};
      lcolors[l] = 2;
      perm[l] = binl[l].slot;
      continue;
    }
    std::vector<int32_t> rows;
    int nco = 1;
    if (terminal) {
      lcoff[l] = {0, M.n};
      rows.resize(M.n);
      for (int i = 0; i < M.n; ++i) rows[i] = i;
    } else {
      if (!parity_colors(M.a, M.parity, M.n, lcoff[l], rows, nco)) greedy_colors(M.a, M.n, lcoff[l], rows, nco);
      if (nco > 8) {
        ljacobi[l] = 1;
        nco = 1;
        lcoff[l] = {0, M.n};
        for (int i = 0; i < M.n; ++i) rows[i] = i;
      }
    }
    lcolors[l] = nco;
    perm[l].assign(M.n, 0);
    for (int k = 0; k < M.n; ++k) perm[l][rows[k]] = k;
  }
  std::vector<MgLevel> PL(C.nl + 1);
  for (int l = 1; l <= C.nl; ++l) {
    const MgLevel& M = H.levels[l];
    MgLevel& Q = PL[l];
    const std::vector<int32_t>& P = perm[l];
    const std::vector<int32_t> none;
    const int nout = binl[l].on ? 2 * binl[l].h : M.n;  // bin rows include empty bins
    Q.n = nout;
    Q.a = permute_csr(M.a, P, P, nout);
    Q.diag.assign(nout, 0.0);
    for (int i = 0; i < M.n; ++i) Q.diag[P[i]] = M.diag[i];
    Q.groups = permute_csr(M.groups, none, P);
    Q.direct_idx = permute_csr(M.direct_idx, none, P);
    Q.direct_off = M.direct_off;
    Q.direct_factor = M.direct_factor;
    if (l < C.nl) {
      Q.restrict = permute_csr(M.restrict, perm[l + 1], P, binl[l + 1].on ? 2 * binl[l + 1].h : -1);
      Q.prolong = permute_csr(M.prolong, P, perm[l + 1], nout);
    }
  }
  {
    // Restriction gathers level-0 slots; the prolongation's rows follow the slots; level
    // 1 in its colour-by-colour numbering.
    Csr R0 = permute_csr(M0.restrict, perm[1], {}, PL[1].n);
    std::vector<int32_t> child(R0.col.size());
    for (size_t q = 0; q < child.size(); ++q) child[q] = slot[R0.col[q]];
    F.resc0 = M0.groups.rows() == 0 ? 1 : 0;
    if (F.resc0) {
      // Colour-0 children only (slot in the first half of its row pair); order kept.
      Csr K;
      std::vector<int32_t> kept;
      K.off.assign(1, 0);
      for (int j = 0; j < R0.rows(); ++j) {
        for (int q = R0.off[j]; q < R0.off[j + 1]; ++q)
          if (((child[q] / F.nxh) & 1) == 0) {
            kept.push_back(child[q]);
            K.val.push_back(R0.val[q]);
          }
        K.off.push_back((int32_t)kept.size());
      }
      R0.off = std::move(K.off);
      R0.val = std::move(K.val);
      child = std::move(kept);
    }
    std::vector<int32_t> poff(F.N2 + 1, 0), pcol;
    std::vector<float> pw32;
    pcol.reserve(M0.prolong.col.size());
    pw32.reserve(M0.prolong.col.size());
    for (int sl = 0; sl < F.N2; ++sl) {
      const int c = cell_of[sl];
      if (c >= 0)
        for (int q = M0.prolong.off[c]; q < M0.prolong.off[c + 1]; ++q) {
          pcol.push_back(perm[1][M0.prolong.col[q]]);
          pw32.push_back((float)M0.prolong.val[q]);
        }
      poff[sl + 1] = (int32_t)pcol.size();
    }
    // Aggregation hierarchies prolong by injection (one weight-1 entry per row): keep the
    // parent per slot only.
    bool inj = true;
    for (int sl = 0; sl < F.N2 && inj; ++sl) {
      const int n = poff[sl + 1] - poff[sl];
      inj = n == 0 || (n == 1 && pw32[poff[sl]] == 1.0f);
    }
    F.pscale = alpha;
    for (auto& w : pw32) w *= alpha;
    if (inj) {
      std::vector<int32_t> par(F.N2, -1);
      for (int sl = 0; sl < F.N2; ++sl)
        if (poff[sl + 1] > poff[sl]) par[sl] = pcol[poff[sl]];
      int* pp;
      if (int e = A.upload(&pp, par, s)) return e;
      F.pinj = pp;
    }
    int *o, *c, *po, *pc;
    float *w, *pw;
    if (int e = A.upload(&o, R0.off, s)) return e;
    if (int e = A.upload(&c, child, s)) return e;
    if (int e = A.upload(&w, to_f32(R0.val), s)) return e;
    if (int e = A.upload(&po, poff, s)) return e;
    if (int e = A.upload(&pc, pcol, s)) return e;
    if (int e = A.upload(&pw, pw32, s)) return e;
    F.r_off = o, F.r_child = c, F.r_w = w, F.p_off = po, F.p_col = pc, F.p_w = pw;
  }
  int maxg = 1;
  for (int l = 1; l <= C.nl; ++l) {
    const MgLevel& M = PL[l];
    CLev& L = C.lv[l - 1];
    L.n = M.n;
    L.terminal = l == C.nl;
    L.ngroups = M.groups.rows();
    maxg = std::max(maxg, L.ngroups);
    int *o, *c;
    float *v, *d;
    if (int e = A.upload(&o, M.a.off, s)) return e;
    if (int e = A.upload(&c, M.a.col, s)) return e;
    if (int e = A.upload(&v, to_f32(M.a.val), s)) return e;
    if (int e = A.upload(&d, to_f32(M.diag), s)) return e;
    L.off = o, L.col = c, L.val = v, L.diag = d;
    std::vector<int32_t> coff = lcoff[l], rows(M.n);
    for (int i = 0; i < M.n; ++i) rows[i] = i;  // colour c owns rows coff[c] .. coff[c+1]-1
    L.ncolors = lcolors[l];
    // A level whose graph needs many colours (the wide stencils of linear-interpolation
    // coarse operators) is smoothed by l1-Jacobi instead: one phase per sweep.
    L.jacobi = ljacobi[l];
    if (L.jacobi) {
      std::vector<float> il1(M.n, 0.0f);
      for (int i = 0; i < M.n; ++i) {
        double sum = std::fabs(M.diag[i]);
        for (int k = M.a.off[i]; k < M.a.off[i + 1]; ++k) sum += std::fabs(M.a.val[k]);
        il1[i] = M.diag[i] == 0.0 ? 0.0f : (float)(1.0 / sum);
      }
      float *pl, *x2;
      if (int e = A.upload(&pl, il1, s)) return e;
      if (int e = A.alloc(&x2, M.n)) return e;
      L.il1 = pl;
      L.x2 = x2;
    }
    cs.colors.push_back(coff);
    int* co;
    if (int e = A.upload(&co, coff, s)) return e;
    L.coff = co;
    {
      // Column-major ELL per colour: entry a of the colour's t-th row at base + a*nrow + t.
      std::vector<int32_t> eoff(L.ncolors), ew(L.ncolors), ecol;
      std::vector<float> eval, idg(M.n);
      for (int i = 0; i < M.n; ++i) idg[i] = M.diag[i] == 0.0 ? 0.0f : 1.0f / (float)M.diag[i];
      for (int c = 0; c < L.ncolors; ++c) {
        int nrow = coff[c + 1] - coff[c], w = 0;
        for (int t = 0; t < nrow; ++t) {
          int r = rows[coff[c] + t];
          w = std::max(w, M.a.off[r + 1] - M.a.off[r]);
        }
        eoff[c] = (int32_t)ecol.size();
        ew[c] = w;
        ecol.resize(ecol.size() + (size_t)w * nrow);
        eval.resize(eval.size() + (size_t)w * nrow);
        for (int t = 0; t < nrow; ++t) {
          int r = rows[coff[c] + t];
          int len = M.a.off[r + 1] - M.a.off[r];
          for (int a = 0; a < w; ++a) {
            size_t e = (size_t)eoff[c] + (size_t)a * nrow + t;
            ecol[e] = a < len ? M.a.col[M.a.off[r] + a] : r;
            eval[e] = a < len ? (float)M.a.val[M.a.off[r] + a] : 0.0f;
          }
        }
      }
      int *eo, *ewp, *ec;
      float *ev, *idp;
      if (int e = A.upload(&eo, eoff, s)) return e;
      if (int e = A.upload(&ewp, ew, s)) return e;
      if (int e = A.upload(&ec, ecol, s)) return e;
      if (int e = A.upload(&ev, eval, s)) return e;
      if (int e = A.upload(&idp, idg, s)) return e;
      L.ell_off = eo, L.ell_w = ewp, L.ell_col = ec, L.ell_val = ev, L.idiag = idp;
      cs.stats.push_back({M.n, (long long)M.a.col.size(), (long long)ecol.size(), M.groups.rows(),
                          L.terminal ? M.direct_idx.rows() : 0, L.ncolors, L.jacobi});
      // The bin stencil of a bin level (CLev::scode): every ELL entry of every row is one of
      // the row's six bin neighbours or padding, at most six per row, at most 16 distinct
      // values, and a bin row's slots per colour a multiple of the rows per sweep item.
      L.scode = nullptr;
      L.svt = nullptr;
      if (binl[l].on && !L.jacobi && L.ncolors == 2 && binl[l].nbh % RPI == 0 && ew[0] <= 6 && ew[1] <= 6) {
        const int nbh = binl[l].nbh, nb1y = binl[l].nb[1], h1 = binl[l].h;
        std::vector<unsigned long long> code(M.n, 0);
        std::vector<float> vt;
        bool ok = true;
        for (int c = 0; c < 2 && ok; ++c) {
          const int nrow = coff[c + 1] - coff[c];
          for (int t = 0; t < nrow && ok; ++t) {
            const int row = coff[c] + t, R = t / nbh, m = t % nbh;
            const int par = (c + R % nb1y + R / nb1y) & 1;
            const int other = (1 - c) * h1 + R * nbh + m;
            const int offs[6] = {par - 1, par, -nbh, nbh, -nb1y * nbh, nb1y * nbh};
            unsigned long long cw = 0;
            for (int a = 0; a < ew[c] && ok; ++a) {
              const size_t e = (size_t)eoff[c] + (size_t)a * nrow + t;
              int dir = 7, vi = 0;
              if (!(ecol[e] == row && eval[e] == 0.0f)) {
                dir = -1;
                for (int d2 = 0; d2 < 6; ++d2)
                  if (ecol[e] == other + offs[d2]) dir = d2;
                ok = dir >= 0;
                if (ok) {
                  vi = (int)(std::find(vt.begin(), vt.end(), eval[e]) - vt.begin());
                  if (vi == (int)vt.size()) vt.push_back(eval[e]);
                  ok = vi < 16;
                }
              }
              cw |= (unsigned long long)(dir | (vi << 3)) << (7 * a);
            }
            code[row] = cw;
          }
        }
        if (ok) {
          unsigned long long* dc;
          float* dv;
          if (int e = A.upload(&dc, code, s)) return e;
          if (int e = A.upload(&dv, vt, s)) return e;
          L.scode = dc;
          L.svt = dv;
          L.snb1y = nb1y;
          L.snbh = nbh;
          cs.stats.back().stencil = 1;
        }
      }
    }
    if (L.ngroups) {
      int *go, *gm;
      if (int e = A.upload(&go, M.groups.off, s)) return e;
      if (int e = A.upload(&gm, M.groups.col, s)) return e;
      L.goff = go, L.gmem = gm;
    }
    float *rhs, *x, *res;
    if (int e = A.alloc(&rhs, L.n)) return e;
    if (int e = A.alloc(&x, L.n)) return e;
    if (int e = A.alloc(&res, L.n)) return e;
    CU(cudaMemsetAsync(rhs, 0, sizeof(float) * L.n, s));
    CU(cudaMemsetAsync(x, 0, sizeof(float) * L.n, s));
    CU(cudaMemsetAsync(res, 0, sizeof(float) * L.n, s));  // colour-1 rows of res0 levels stay zero
    L.rhs = rhs, L.x = x, L.res = res;
    L.res0 = !L.terminal && !L.jacobi && L.ncolors == 2 && L.ngroups == 0 ? 1 : 0;
    if (L.terminal) {
      L.nblocks = M.direct_idx.rows();
      int *io, *ix;
      long long* fo;
      double* fa;
      std::vector<long long> foff(M.direct_off.begin(), M.direct_off.end());
      if (int e = A.upload(&io, M.direct_idx.off, s)) return e;
      if (int e = A.upload(&ix, M.direct_idx.col, s)) return e;
      if (int e = A.upload(&fo, foff, s)) return e;
      // The coarsest solve as an FP64 mat-vec with (L L^T)^-1 of each block, formed on
      // the host from the reference's Cholesky factor: one warp per block, no FP64
      // dependency chain of substitution steps.
      std::vector<double> inv(M.direct_factor.size());
      for (int b = 0; b < L.nblocks; ++b) {
        const int n = M.direct_idx.off[b + 1] - M.direct_idx.off[b];
        const double* f = M.direct_factor.data() + M.direct_off[b];
        double* out = inv.data() + M.direct_off[b];
        std::vector<double> y(n);
        for (int col = 0; col < n; ++col) {
          for (int i = 0; i < n; ++i) {
            double v = i == col ? 1.0 : 0.0;
            for (int j = 0; j < i; ++j) v -= f[i * n + j] * y[j];
            y[i] = v / f[i * n + i];
          }
          for (int i = n - 1; i >= 0; --i) {
            double v = y[i];
            for (int j = i + 1; j < n; ++j) v -= f[j * n + i] * y[j];
            y[i] = v / f[i * n + i];
          }
          for (int i = 0; i < n; ++i) out[i * n + col] = y[i];
        }
      }
      if (int e = A.upload(&fa, inv, s)) return e;
      L.ioff = io, L.idx = ix, L.foff = fo, L.fac = fa;
      for (int b = 0; b < L.nblocks; ++b)
        if (M.direct_idx.off[b + 1] - M.direct_idx.off[b] > 32)
          return fail(CFDG_ERR_UNSUPPORTED, "mixed form: coarse block larger than 32");
    } else {
      int *ro, *rc, *po, *pc;
      float *rw, *pw;
      Csr R = M.restrict;
      if (L.res0) {
        // Colour-1 residuals stay zero on this level: gather colour-0 children only.
        Csr K;
        K.off.assign(1, 0);
        for (int j = 0; j < R.rows(); ++j) {
          for (int q = R.off[j]; q < R.off[j + 1]; ++q)
            if (R.col[q] < coff[1]) {
              K.col.push_back(R.col[q]);
              K.val.push_back(R.val[q]);
            }
          K.off.push_back((int32_t)K.col.size());
        }
        R = std::move(K);
      }
      if (int e = A.upload(&ro, R.off, s)) return e;
      if (int e = A.upload(&rc, R.col, s)) return e;
      if (int e = A.upload(&rw, to_f32(R.val), s)) return e;
      if (int e = A.upload(&po, M.prolong.off, s)) return e;
      if (int e = A.upload(&pc, M.prolong.col, s)) return e;
      std::vector<float> pw32 = to_f32(M.prolong.val);
      for (auto& w : pw32) w *= alpha;
      if (int e = A.upload(&pw, pw32, s)) return e;
      L.roff = ro, L.rchild = rc, L.rw = rw, L.poff = po, L.pcol = pc, L.pw = pw;
    }
  }
  if (int e = A.alloc(&C.gpart, (size_t)maxg * CS)) return e;
  F.n1 = C.lv[0].n;
  F.rhs1 = C.lv[0].rhs;
  F.x1 = C.lv[0].x;
  CU(cudaStreamSynchronize(s));
  return 0;
}

}  // namespace mx
}  // namespace cfdg

using namespace cfdg;
using namespace cfdg::mx;

// Work-lists of the persistent fine-level kernels: the row tiles, level-1 row tiles,
// face tiles and level-0 group entries of the cases a list covers. Kernels loop over
// the first counts[k] entries, so the lists change between graph replays without
// touching the graph.
struct WorkLists {
  int2 *tiles = nullptr, *tiles1 = nullptr, *ftiles = nullptr, *gtab = nullptr;
  int* counts = nullptr;  // [4]
  int* pos = nullptr;     // [4][cases]: where a case's items start in each list, -1 when absent
};

// Builds work-lists on the device from the case-contiguous master lists: item e of case
// c goes to pos[k][c] + (e - moff[k][c]) when the case is in the list.
struct ListBuild {
  const int2* m[4];
  int2* out[4];
  int total[4];
  const int* moff;  // [4][nc+1]
  const int* pos;   // [4][nc]
  int nc;
};
__global__ void k_build_lists(ListBuild L) {
  const int stride = gridDim.x * blockDim.x;
  for (int k = 0; k < 4; ++k)
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < L.total[k]; e += stride) {
      const int2 t = L.m[k][e];
      const int p = L.pos[k * L.nc + t.x];
      if (p >= 0) L.out[k][p + e - L.moff[k * (L.nc + 1) + t.x]] = t;
    }
}

// A set of grids solved together in the mixed form.
struct cfdg_batch {
  cfdg_context* ctx = nullptr;
  std::vector<cfdg_grid*> grids;
  std::vector<std::shared_ptr<CaseState>> cases;
  Arena arena;
  cudaStream_t stream = nullptr, own = nullptr;
  FineCase* d_fc = nullptr;
  CCase* d_cc = nullptr;
  MState* d_st = nullptr;
  MState* h_st = nullptr;
  std::vector<FineCase> h_fc;
  // All work items of all cases (host), and three device lists: the graph's (run),
  // the prologue's and the epilogue's.
  std::vector<int2> tiles, tiles1, ftiles, gtab;
  WorkLists run, pro, epi;
  int g_fine = 1, g_1 = 1, g_f = 1, g_g = 1;  // work items per list: caps on the persistent grids
  bool any_groups = false;
  bool any_bin1 = false;  // some case has its level 1 as the bin grid
  // Coarse-level phase tables (device), refilled for each active set.
  CoarseTab h_tab{};
  CoarseTab* d_tab = nullptr;
  int* tab_buf = nullptr;
  int nlev_all = 0;
  int coop_blocks = 0;
  bool coop = true;
  // Staged half sweeps (k_rb_tma): every case has its tensor maps; the largest row length
  // (rounded up to 16 slots), the dynamic shared memory and the persistent grid.
  bool rb_tma = false;
  int rb_hmax = 0, rb_grid = 1, rb_sr = RT, rb_ns = 3;
  int rb_sr_req = 0, rb_ns_req = 0;  // the grids' setting (0, 0: automatic)
  size_t rb_smem = 0;
  int csize = CS;
  std::vector<char> active;
  cudaGraphExec_t chunk = nullptr;
  size_t chunk_nodes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // V-cycle sweeps before and after the coarse correction on level 0 and on the coarse
  // levels (from the grids' settings), and iterations per graph chunk.
  int nu0 = 2, nuc = 2, chunk_it = CHUNK_IT;
  // Device copies of the master lists and their per-case offsets [4][nc+1].
  int2 *m_tiles = nullptr, *m_tiles1 = nullptr, *m_ftiles = nullptr, *m_gtab = nullptr;
  int* d_moff = nullptr;
  std::vector<int> moff;
  // Pinned staging ring: host->device copies that return without waiting for the stream.
  struct Stage {
    void* h = nullptr;
    size_t cap = 0;
    cudaEvent_t ev = nullptr;
    bool pending = false;
  };
  std::vector<Stage> ring = std::vector<Stage>(16);
  size_t ring_next = 0;
  ~cfdg_batch() {
    if (chunk) cudaGraphExecDestroy(chunk);
    arena.release();
    if (h_st) cudaFreeHost(h_st);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    for (auto& r : ring) {
      if (r.pending) cudaEventSynchronize(r.ev);
      if (r.h) cudaFreeHost(r.h);
      if (r.ev) cudaEventDestroy(r.ev);
    }
    if (own) cudaStreamDestroy(own);
  }
};

namespace {

// Persistent grids: every block resident at once (the SM count times the kernel's
// occupancy), and no more blocks than work items.
int resident_grid(const void* fn, int threads) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({dev, fn});
  if (it != cache.end()) return it->second;
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0) != cudaSuccess || per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return cache[{dev, fn}] = std::max(1, sms) * per;
}
template <class K>
int grid_of(K kernel, int threads, int items) {
  return std::max(1, std::min(items, resident_grid((const void*)kernel, threads)));
}
// Copies `bytes` from host memory to the device through a pinned staging slot, so the
// call returns without waiting for the work queued on `s` (the slot is reused once the
// copy that last used it has completed).
int staged_h2d(cfdg_batch* B, void* d_dst, const void* h_src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return 0;
  cfdg_batch::Stage& st = B->ring[B->ring_next];
  B->ring_next = (B->ring_next + 1) % B->ring.size();
  if (st.pending) CU(cudaEventSynchronize(st.ev));
  st.pending = false;
  if (!st.ev) CU(cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming));
  if (st.cap < bytes) {
    if (st.h) CU(cudaFreeHost(st.h));
    st.h = nullptr;
    st.cap = 0;
    CU(cudaMallocHost(&st.h, bytes));
    st.cap = bytes;
  }
  std::memcpy(st.h, h_src, bytes);
  CU(cudaMemcpyAsync(d_dst, st.h, bytes, cudaMemcpyHostToDevice, s));
  CU(cudaEventRecord(st.ev, s));
  st.pending = true;
  return 0;
}

// Points work-list W at the cases marked in `on`: the host computes where each case's
// items go, one kernel gathers them from the master lists (no host pass over the items,
// no wait for the stream).
int fill_lists(cfdg_batch* B, WorkLists& W, const std::vector<char>& on, cudaStream_t s) {
  const int nc = (int)B->cases.size();
  static thread_local std::vector<int> pos;
  pos.assign(4 * nc + 4, -1);
  int counts[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < nc; ++c) {
      if (!on[c]) continue;
      const int n = B->moff[k * (nc + 1) + c + 1] - B->moff[k * (nc + 1) + c];
      pos[k * nc + c] = counts[k];
      counts[k] += n;
    }
  for (int k = 0; k < 4; ++k) pos[4 * nc + k] = counts[k];
  if (int e = staged_h2d(B, W.pos, pos.data(), sizeof(int) * 4 * nc, s)) return e;
  if (int e = staged_h2d(B, W.counts, pos.data() + 4 * nc, sizeof(int) * 4, s)) return e;
  ListBuild L;
  const int2* m[4] = {B->m_tiles, B->m_tiles1, B->m_ftiles, B->m_gtab};
  int2* out[4] = {W.tiles, W.tiles1, W.ftiles, W.gtab};
  int most = 0;
  for (int k = 0; k < 4; ++k) {
    L.m[k] = m[k];
    L.out[k] = out[k];
    L.total[k] = B->moff[k * (nc + 1) + nc];
    most = std::max(most, L.total[k]);
  }
  L.moff = B->d_moff;
  L.pos = W.pos;
  L.nc = nc;
  if (most > 0) {
    k_build_lists<<<grid_of(k_build_lists, 256, (most + 255) / 256), 256, 0, s>>>(L);
    count();
  }
  CU(cudaGetLastError());
  return 0;
}

// Coarse phase tables for the active cases (inactive ones contribute no rows).
int fill_tab(cfdg_batch* B, const std::vector<char>& on, cudaStream_t s) {
  const int nc = (int)B->cases.size(), nlev = B->nlev_all, w = nc + 1;
  CoarseTab& T = B->h_tab;
  static thread_local std::vector<int32_t> buf;
  const size_t words = (size_t)nlev * w * (6 + 2 * MAXC);
  buf.assign(words, 0);
  int32_t *rows = buf.data(), *term = rows + nlev * w, *next = term + nlev * w, *live = next + nlev * w,
          *grp = live + nlev * w, *res = grp + nlev * w, *fwd = res + nlev * w, *bwd = fwd + (size_t)nlev * MAXC * w;
  // Sweep and residual ranges are rounded up to multiples of eight, so the eight-lane
  // groups of l1-Jacobi rows never straddle two cases.
  auto r8 = [](int v) { return (v + 7) & ~7; };
  T.nc = nc;
  T.nlev = 0;
  T.nu = B->nuc;
  // Levels on which every active case has at most BLK_WORK rows plus stencil entries run
  // block-locally (one block per case, block barriers) instead of one grid barrier per
  // phase; wide-stencil levels stay grid-wide even when they have few rows.
  T.lb = nlev;
  for (int l = nlev - 1; l >= 0; --l) {
    long long most = 0;
    for (int i = 0; i < nc; ++i)
      if (on[i] && l < B->cases[i]->C.nl) {
        const auto& st = B->cases[i]->stats[l];
        most = std::max(most, st.rows + st.ell);
      }
    if (most > BLK_WORK) break;
    T.lb = l;
  }
  for (int l = 0; l < nlev; ++l) {
    int maxc = 0, anyg = 0;
    auto lev = [&](int i) -> const CLev* {
      return on[i] && l < B->cases[i]->C.nl ? &B->cases[i]->C.lv[l] : nullptr;
    };
    for (int i = 0; i < nc; ++i)
      if (const CLev* L = lev(i)) {
        if (!L->terminal) maxc = std::max(maxc, L->ncolors);
        anyg |= L->ngroups > 0;
        T.nlev = std::max(T.nlev, l + 1);
      }
    T.maxc[l] = maxc;
    T.anyg[l] = anyg;
    for (int i = 0; i < nc; ++i) {
      const CLev* L = lev(i);
      const bool nt = L && !L->terminal;
      rows[l * w + i + 1] = rows[l * w + i] + (L ? L->n : 0);
      term[l * w + i + 1] = term[l * w + i] + (L && L->terminal ? L->nblocks : 0);
      next[l * w + i + 1] = next[l * w + i] + (nt ? B->cases[i]->C.lv[l + 1].n : 0);
      // Prolongation items: every row but the last colour's on Gauss-Seidel levels.
      live[l * w + i + 1] = live[l * w + i] + (nt ? (L->jacobi ? L->n : B->cases[i]->colors[l][L->ncolors - 1]) : 0);
      grp[l * w + i + 1] = grp[l * w + i] + (L ? L->ngroups : 0);
      const auto& cof = B->cases[i]->colors[l];
      const int nres = !nt ? 0 : (L->res0 ? (cof[1] + RPI - 1) / RPI : (L->jacobi ? 8 * L->n : L->n));
      res[l * w + i + 1] = res[l * w + i] + r8(nres);
      for (int c = 0; c < MAXC; ++c) {
        int nf = 0, nb = 0;
        if (nt && L->jacobi) {
          nf = nb = c == 0 ? 8 * L->n : 0;
        } else if (nt && c < L->ncolors) {  // RPI rows per item
          const auto& co = B->cases[i]->colors[l];
          nf = r8((co[c + 1] - co[c] + RPI - 1) / RPI);
          const int cb = L->ncolors - 1 - c;
          nb = r8((co[cb + 1] - co[cb] + RPI - 1) / RPI);
        }
        fwd[(l * MAXC + c) * w + i + 1] = fwd[(l * MAXC + c) * w + i] + nf;
        bwd[(l * MAXC + c) * w + i + 1] = bwd[(l * MAXC + c) * w + i] + nb;
      }
    }
  }
  T.rows = B->tab_buf;
  T.term = T.rows + nlev * w;
  T.next = T.term + nlev * w;
  T.live = T.next + nlev * w;
  T.grp = T.live + nlev * w;
  T.res = T.grp + nlev * w;
  T.fwd = T.res + nlev * w;
  T.bwd = T.fwd + (size_t)nlev * MAXC * w;
  if (int e = staged_h2d(B, B->tab_buf, buf.data(), words * sizeof(int32_t), s)) return e;
  return staged_h2d(B, B->d_tab, &T, sizeof(CoarseTab), s);
}

// The graph's lists and tables cover the cases marked in B->active.
int set_active(cfdg_batch* B, cudaStream_t s) {
  if (int e = fill_lists(B, B->run, B->active, s)) return e;
  return fill_tab(B, B->active, s);
}

void launch_coarse(cfdg_batch* B, cudaStream_t s) {
  if (B->coop) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)B->coop_blocks, 1, 1);
    cfg.blockDim = dim3(512, 1, 1);
    cfg.dynamicSmemBytes = 2 * B->cases.size() * sizeof(CLev);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_coarse_all, (const CCase*)B->d_cc, (const MState*)B->d_st, (const CoarseTab*)B->d_tab);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(B->cases.size() * B->csize), 1, 1);
  cfg.blockDim = dim3(CT, 1, 1);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)B->csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_coarse, (const CCase*)B->d_cc, (const MState*)B->d_st, B->nuc);
}

#define FINE(K, W, ...) \
  K<<<grid_of(K, TILE, B->g_fine), TILE, 0, s>>>(B->d_fc, B->d_st, (W).tiles, (W).counts, ##__VA_ARGS__)

// One red-black half sweep of level 0 over the work-list: the staged kernel when every case
// has its tensor maps, else the register kernel (the same bits either way).
void launch_rb(cfdg_batch* B, const WorkLists& W, int color, int first, cudaStream_t s) {
  if (B->rb_tma)
    k_rb_tma<<<B->rb_grid, RB_THREADS, B->rb_smem, s>>>(B->d_fc, B->d_st, W.tiles, W.counts, color, first,
                                                        B->rb_hmax, B->rb_sr, B->rb_ns);
  else
    FINE(k_rb, W, color, first);
}

void enqueue_vcycle(cfdg_batch* B, cudaStream_t s) {
  const WorkLists& W = B->run;
  if (B->any_groups) {
    FINE(k_v_rhs, W);
    k_center0<<<grid_of(k_center0, 256, B->g_g), 256, 0, s>>>(B->d_fc, B->d_st, W.gtab, W.counts + 3, 0);
  }
  // nu0 forward sweeps: red, black, red, black, ... (the first red starts from x = 0).
  for (int sw = 0; sw < B->nu0; ++sw) {
    launch_rb(B, W, 0, sw == 0 ? 1 : 0, s);
    launch_rb(B, W, 1, 0, s);
  }
  if (B->any_groups) k_center0<<<grid_of(k_center0, 256, B->g_g), 256, 0, s>>>(B->d_fc, B->d_st, W.gtab, W.counts + 3, 1);
  FINE(k_v_resid, W);
  if (B->any_groups) k_center0<<<grid_of(k_center0, 256, B->g_g), 256, 0, s>>>(B->d_fc, B->d_st, W.gtab, W.counts + 3, 2);
  k_v_restrict<<<grid_of(k_v_restrict, TILE, B->g_1), TILE, 0, s>>>(B->d_fc, B->d_st, W.tiles1, W.counts + 1);
  launch_coarse(B, s);
  FINE(k_v_prolong, W);
  // nu0 backward sweeps: black, red, ...
  for (int sw = 0; sw < B->nu0; ++sw) {
    launch_rb(B, W, 1, 0, s);
    launch_rb(B, W, 0, 0, s);
  }
  if (B->any_groups) k_center0<<<grid_of(k_center0, 256, B->g_g), 256, 0, s>>>(B->d_fc, B->d_st, W.gtab, W.counts + 3, 1);
}

// One iteration of the per-case state machine.
void enqueue_iteration(cfdg_batch* B, cudaStream_t s) {
  const WorkLists& W = B->run;
  const int nc = (int)B->cases.size();
  FINE(k_op, W);
  FINE(k_update, W);
  FINE(k_outer, W);
  FINE(k_outer_resid, W);
  FINE(k_scale, W);
  k_start_state<<<(nc + 127) / 128, 128, 0, s>>>(B->d_st, nc);
  enqueue_vcycle(B, s);
  FINE(k_rz, W);
  FINE(k_p, W);
}

int ensure_graph(cfdg_batch* B) {
  if (B->chunk) return 0;
  cudaGraph_t g;
  CU(cudaStreamBeginCapture(B->own, cudaStreamCaptureModeThreadLocal));
  for (int i = 0; i < B->chunk_it; ++i) enqueue_iteration(B, B->own);
  cudaError_t e = cudaStreamEndCapture(B->own, &g);
  if (e != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("mixed capture: ") + cudaGetErrorString(e));
  cudaGraphGetNodes(g, nullptr, &B->chunk_nodes);
  e = cudaGraphInstantiate(&B->chunk, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("mixed graph: ") + cudaGetErrorString(e));
  return 0;
}

// Per-grid FP32 state for the mixed form, built on first use and cached on the grid.
int case_of(cfdg_grid* G, std::shared_ptr<CaseState>& out) {
  if (G->mixed) {
    out = std::static_pointer_cast<CaseState>(G->mixed);
    return 0;
  }
  if (!G->structured || !G->mg || !G->host_mg || !G->mg->full0)
    return fail(CFDG_ERR_UNSUPPORTED, "the mixed form needs a non-periodic grid with a multigrid hierarchy of two or more levels");
  auto cs = std::make_shared<CaseState>();
  cs->G = G;
  cs->version = G->faces_version;
  if (int e = build_case(G, *cs)) return e;
  G->mixed = cs;
  out = cs;
  return 0;
}

MState initial_state(double tol, uint64_t max_iter) {
  MState m;
  std::memset(&m, 0, sizeof(m));
  m.state = IDLE;
  m.tol = tol;
  m.inner_tol = 1e-4;  // per outer step; FP32 reaches it comfortably
  m.max_it = (int)std::min<uint64_t>(max_iter, 1u << 30);
  m.max_inner = 200;
  return m;
}

// Prologue of the cases marked in `on` (their states IDLE): b, terms, the closed
// components' compatibility and gauge, |b_c|. A failed check sets FAIL/E031.
int prologue(cfdg_batch* B, const std::vector<char>& on, cudaStream_t s) {
  if (int e = fill_lists(B, B->pro, on, s)) return e;
  FINE(k_rhs, B->pro);
  count();
  bool groups = false;
  for (size_t i = 0; i < B->cases.size(); ++i) groups |= on[i] && B->grids[i]->ncomp_groups > 0;
  if (groups) CU(cudaStreamSynchronize(s));  // the compatibility check (E031) is decided on the host
  for (size_t i = 0; i < B->cases.size(); ++i) {
    if (!on[i]) continue;
    cfdg_grid* G = B->grids[i];
    if (G->ncomp_groups == 0) continue;  // k_rhs wrote b_c beside b
    int rc = plain_compat_center(G, s);
    if (rc) {
      MState f = initial_state(0, 0);
      f.state = FAIL;
      f.error = rc;
      CU(cudaMemcpyAsync(&B->d_st[i], &f, sizeof(MState), cudaMemcpyHostToDevice, s));
      CU(cudaStreamSynchronize(s));
    }
  }
  FINE(k_norm, B->pro);
  count();
  CU(cudaGetLastError());
  return 0;
}

// Epilogue of the converged cases marked in `on`: gauge of x, u -= dt grad x, p += x,
// gauge of p.
int epilogue(cfdg_batch* B, const std::vector<char>& on, cudaStream_t s) {
  if (int e = fill_lists(B, B->epi, on, s)) return e;
  for (size_t i = 0; i < B->cases.size(); ++i)
    if (on[i] && B->grids[i]->ncomp_groups) plain_center(B->grids[i], B->grids[i]->x, s);
  k_correct<<<grid_of(k_correct, 256, B->g_f), 256, 0, s>>>(B->d_fc, B->d_st, B->epi.ftiles, B->epi.counts + 2);
  FINE(k_addp, B->epi);
  count(2);
  for (size_t i = 0; i < B->cases.size(); ++i)
    if (on[i] && B->grids[i]->ncomp_groups) plain_center(B->grids[i], B->h_fc[i].pfield, s);
  CU(cudaGetLastError());
  return 0;
}

void fill_info(const MState& m, cfdg_info& I) {
  std::memset(&I, 0, sizeof(I));
  I.iterations = (uint64_t)m.total_it;
  I.relative_residual = m.state == DONE ? (m.norm < 1e-24 ? 0.0 : m.true_rel) : 0.0;
  I.work_units = (uint64_t)m.total_it;
  I.operator_applications = (uint64_t)m.total_it + (uint64_t)m.outer + 1;
  I.true_residual_checks = (uint64_t)m.outer + 1;
  I.preconditioner_applications = (uint64_t)m.total_it + (uint64_t)m.outer;
  I.cycles = I.preconditioner_applications;
  I.refinement_steps = (uint64_t)m.outer;
}

}  // namespace

// (Re)packs a batch's device tables after its cases are known.
int cfdg_mixed_pack(cfdg_batch* B) {
  cudaStream_t s = B->own;
  if (B->chunk) cudaGraphExecDestroy(B->chunk);
  B->chunk = nullptr;
  B->arena.release();
  B->arena.ctx = B->ctx;
  B->tiles.clear(), B->tiles1.clear(), B->ftiles.clear(), B->gtab.clear();
  B->h_fc.clear();
  std::vector<CCase> cc;
  const int nc = (int)B->cases.size();
  B->any_groups = false;
  B->any_bin1 = false;
  B->nlev_all = 0;
  for (int i = 0; i < nc; ++i) {
    FineCase F = B->cases[i]->F;
    for (int t = 0; t < F.ntiles; ++t) B->tiles.push_back(make_int2(i, t));
    for (int t = 0; t < (F.n1 + TILE - 1) / TILE; ++t) B->tiles1.push_back(make_int2(i, t));
    F.nftiles = (int)((F.F + FTILE - 1) / FTILE);
    for (int t = 0; t < F.nftiles; ++t) B->ftiles.push_back(make_int2(i, t));
    for (int g = 0; g < F.ngroups; ++g) B->gtab.push_back(make_int2(i, g));
    B->any_groups |= F.ngroups > 0;
    B->any_bin1 |= F.bin1 != 0;
    B->nlev_all = std::max(B->nlev_all, B->cases[i]->C.nl);
    for (int l = 0; l < B->cases[i]->C.nl; ++l)
      if (!B->cases[i]->C.lv[l].terminal && B->cases[i]->C.lv[l].ncolors > MAXC)
        return fail(CFDG_ERR_UNSUPPORTED, "mixed form: too many colours on a coarse level");
    B->h_fc.push_back(F);
    cc.push_back(B->cases[i]->C);
  }
  Arena& A = B->arena;
  for (WorkLists* W : {&B->run, &B->pro, &B->epi}) {
    if (int e = A.alloc(&W->tiles, B->tiles.size())) return e;
    if (int e = A.alloc(&W->tiles1, B->tiles1.size())) return e;
    if (int e = A.alloc(&W->ftiles, B->ftiles.size())) return e;
    if (int e = A.alloc(&W->gtab, B->gtab.size())) return e;
    if (int e = A.alloc(&W->counts, 4)) return e;
    if (int e = A.alloc(&W->pos, 4 * (size_t)nc)) return e;
  }
  // Master lists (case-contiguous) on the device and the offset of each case's items.
  B->moff.assign(4 * (nc + 1), 0);
  {
    const std::vector<int2>* lists[4] = {&B->tiles, &B->tiles1, &B->ftiles, &B->gtab};
    for (int k = 0; k < 4; ++k) {
      int* o = B->moff.data() + k * (nc + 1);
      for (const int2& t : *lists[k]) o[t.x + 1] += 1;
      for (int c = 0; c < nc; ++c) o[c + 1] += o[c];
    }
    if (int e = A.upload(&B->m_tiles, B->tiles, s)) return e;
    if (int e = A.upload(&B->m_tiles1, B->tiles1, s)) return e;
    if (int e = A.upload(&B->m_ftiles, B->ftiles, s)) return e;
    if (int e = A.upload(&B->m_gtab, B->gtab, s)) return e;
    if (int e = A.upload(&B->d_moff, B->moff, s)) return e;
  }
  auto clamp = [](size_t n) { return (int)std::max<size_t>(1, std::min<size_t>(n, 1 << 30)); };
  B->g_fine = clamp(B->tiles.size());
  B->g_1 = clamp(B->tiles1.size());
  B->rb_tma = nc > 0;
  B->rb_hmax = 0;
  for (int i = 0; i < nc; ++i) {
    B->rb_tma = B->rb_tma && B->h_fc[i].tmaps != nullptr;
    B->rb_hmax = std::max(B->rb_hmax, B->h_fc[i].nxh);
  }
  if (B->rb_tma) {
    // The sweep's tile shape comes from the grids (cfdg_grid_set_sweep_tile), like the
    // cycle's sweep counts; fewer stages are used when the requested ones do not fit.
    B->rb_hmax = (B->rb_hmax + 15) / 16 * 16;
    int dev = 0, sms = 0, per = 0, smem_max = 0, smem_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    B->rb_sr = B->rb_sr_req;
    B->rb_ns = B->rb_ns_req;
    if (B->rb_sr == 0) {
      // The automatic shape: two stages of the tallest height whose blocks still fit twice
      // per SM (on the benchmarked mixes the autotuner's choice, 32 x 2, where it fits).
      B->rb_ns = 2;
      B->rb_sr = 8;
      for (int sr : {32, 16}) {
        const size_t need = 2 * (2 * (size_t)rb_offsets(B->rb_hmax, sr).stage + 128 + 2048);
        if (need <= (size_t)smem_sm) {
          B->rb_sr = sr;
          break;
        }
      }
    }
    const size_t stage = (size_t)rb_offsets(B->rb_hmax, B->rb_sr).stage;
    while (B->rb_ns > 1 && (size_t)B->rb_ns * stage + 128 + 1024 > (size_t)smem_max) --B->rb_ns;
    B->rb_smem = (size_t)B->rb_ns * stage + 128;
    cudaFuncSetAttribute(k_rb_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B->rb_smem);
    if (B->rb_ns < 2 ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rb_tma, RB_THREADS, B->rb_smem) != cudaSuccess ||
        per < 1) {
      cudaGetLastError();
      B->rb_tma = false;
    } else {
      B->rb_grid = std::max(1, std::min(B->g_fine, sms * per));
    }
  }
  B->g_f = clamp(B->ftiles.size());
  B->g_g = clamp(B->gtab.size());
  if (int e = A.upload(&B->d_fc, B->h_fc, s)) return e;
  if (int e = A.upload(&B->d_cc, cc, s)) return e;
  if (int e = A.alloc(&B->d_st, nc)) return e;
  std::vector<MState> idle(nc, initial_state(0, 0));
  for (auto& m : idle) m.state = DONE;  // nothing runs before a solve sets its cases
  CU(cudaMemcpyAsync(B->d_st, idle.data(), sizeof(MState) * nc, cudaMemcpyHostToDevice, s));
  if (B->h_st) cudaFreeHost(B->h_st);
  CU(cudaMallocHost((void**)&B->h_st, sizeof(MState) * nc));
  if (int e = A.alloc(&B->tab_buf, (size_t)B->nlev_all * (nc + 1) * (6 + 2 * MAXC) + 1)) return e;
  if (int e = A.alloc(&B->d_tab, 1)) return e;
  B->active.assign(nc, 1);
  if (int e = set_active(B, s)) return e;
  // Grid of the cooperative coarse-level kernel: all blocks co-resident.
  {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t dsm = 2 * (size_t)nc * sizeof(CLev);
    if (dsm > 48 * 1024) cudaFuncSetAttribute(k_coarse_all, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm);
    B->coop = true;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_coarse_all, 512, dsm) != cudaSuccess || per < 1) {
      cudaGetLastError();
      B->coop = false;
    }
    B->coop_blocks = sms * std::max(1, std::min(per, 4));
  }
  if (!B->coop) {
    // One cluster per case: 16 CTAs when that non-portable size is allowed, else 8.
    B->csize = CS;
    if (cudaFuncSetAttribute(k_coarse, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      B->csize = 8;
    }
  }
  CU(cudaStreamSynchronize(s));
  return ensure_graph(B);
}

int cfdg_mixed_add_case(cfdg_batch* B, cfdg_grid* G) {
  std::shared_ptr<CaseState> cs;
  if (int e = case_of(G, cs)) return e;
  if (B->grids.empty()) {
    B->nu0 = G->mx_nu0;
    B->nuc = G->mx_nuc;
    B->rb_sr_req = G->mx_sweep_rows;
    B->rb_ns_req = G->mx_sweep_stages;
  } else if (B->nu0 != G->mx_nu0 || B->nuc != G->mx_nuc) {
    return fail(CFDG_ERR_INVALID, "the grids of a batch must share their V-cycle sweep counts");
  } else if (B->rb_sr_req != G->mx_sweep_rows || B->rb_ns_req != G->mx_sweep_stages) {
    return fail(CFDG_ERR_INVALID, "the grids of a batch must share their sweep tile shape");
  }
  B->grids.push_back(G);
  B->cases.push_back(cs);
  return 0;
}

// Solves the projection of every case of the batch (device u[i], p[i]); codes[i] per case.
int cfdg_mixed_project(cfdg_batch* B, double* const* d_u, double* const* d_p, const double* dt, double tol,
                       uint64_t max_iter, cfdg_poll_fn poll, void* poll_ctx, cfdg_info* infos, int32_t* codes) {
  cudaStream_t s = B->stream;
  const int nc = (int)B->cases.size();
  if (codes)
    for (int i = 0; i < nc; ++i) codes[i] = 0;
  for (int i = 0; i < nc; ++i) {
    B->h_fc[i].u = d_u[i];
    B->h_fc[i].pfield = d_p[i];
    B->h_fc[i].dt = dt[i];
    B->h_fc[i].rdt = rdt_of(dt[i]);
  }
  CU(cudaMemcpyAsync(B->d_fc, B->h_fc.data(), sizeof(FineCase) * nc, cudaMemcpyHostToDevice, s));
  std::vector<MState> st(nc, initial_state(tol, max_iter));
  CU(cudaMemcpyAsync(B->d_st, st.data(), sizeof(MState) * nc, cudaMemcpyHostToDevice, s));
  CU(cudaEventRecord(B->ev0, s));
  std::vector<char> all(nc, 1);
  if (int e = prologue(B, all, s)) return e;
  B->active = all;
  if (int e = set_active(B, s)) return e;
  Poller P;
  P.fn = poll;
  P.ctx = poll_ctx;
  int status = 0;
  uint64_t chunks = 0;
  cudaEvent_t lp0, lp1;
  cudaEventCreate(&lp0);
  cudaEventCreate(&lp1);
  cudaEventRecord(lp0, s);
  for (;;) {
    CU(cudaMemcpyAsync(B->h_st, B->d_st, sizeof(MState) * nc, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    bool all_done = true, shrink = false;
    for (int i = 0; i < nc; ++i) {
      const bool fin = B->h_st[i].state == DONE || B->h_st[i].state == FAIL;
      all_done &= fin;
      if (fin && B->active[i]) {
        B->active[i] = 0;  // finished cases leave the work-lists
        shrink = true;
      }
    }
    if (all_done) break;
    if (int c = P.check()) {
      status = fail(c, c == CFDG_CANCELLED ? "cancelled" : "wall_time_limit");
      break;
    }
    if (shrink)
      if (int e = set_active(B, s)) return e;
    CU(cudaGraphLaunch(B->chunk, s));
    count(B->chunk_nodes);
    chunks += 1;
  }
  cudaEventRecord(lp1, s);
  if (status == 0) {
    std::vector<char> done(nc, 0);
    for (int i = 0; i < nc; ++i) done[i] = B->h_st[i].state == DONE;
    if (int e = epilogue(B, done, s)) return e;
  }
  CU(cudaEventRecord(B->ev1, s));
  CU(cudaEventSynchronize(B->ev1));
  float ms = 0, lms = 0;
  cudaEventElapsedTime(&ms, B->ev0, B->ev1);
  cudaEventElapsedTime(&lms, lp0, lp1);
  cudaEventDestroy(lp0);
  cudaEventDestroy(lp1);
  for (int i = 0; i < nc; ++i) {
    const MState& m = B->h_st[i];
    if (infos) {
      fill_info(m, infos[i]);
      infos[i].device_seconds = ms * 1e-3;
      infos[i].graph_launches = chunks;
      infos[i].loop_seconds = lms * 1e-3;
    }
    if (codes && codes[i] == 0) {
      if (status) codes[i] = status;
      else if (m.state == FAIL) codes[i] = m.error ? m.error : CFDG_E033;
    }
  }
  return status;
}

// ----------------------------------------------------------------- batch lifetime and C ABI
namespace {
// A grid whose faces changed since the batch was packed gets a fresh hierarchy and FP32
// state, and the batch's tables are packed again (the grids' locks are held).
int refresh_batch(cfdg_batch* B) {
  bool stale = false;
  for (size_t i = 0; i < B->cases.size(); ++i) {
    cfdg_grid* G = B->grids[i];
    if (B->cases[i]->version == G->faces_version && G->mixed == B->cases[i]) continue;
    if (int e = prepare_multigrid(G)) return e;
    std::shared_ptr<CaseState> cs;
    if (int e = case_of(G, cs)) return e;
    B->cases[i] = cs;
    stale = true;
  }
  return stale ? cfdg_mixed_pack(B) : 0;
}

std::vector<cfdg_grid*> lock_order(const std::vector<cfdg_grid*>& g) {
  std::vector<cfdg_grid*> v(g);
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
  return v;
}

struct Locks {
  std::vector<std::unique_lock<std::mutex>> held;
  explicit Locks(const std::vector<cfdg_grid*>& grids) {
    for (auto* G : lock_order(grids)) held.emplace_back(G->mu);
  }
};
}  // namespace

cfdg_batch* cfdg_mixed_new(cfdg_context* ctx) {
  auto* B = new cfdg_batch();
  B->ctx = ctx;
  B->arena.ctx = ctx;
  if (cudaStreamCreateWithFlags(&B->own, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&B->ev0) != cudaSuccess ||
      cudaEventCreate(&B->ev1) != cudaSuccess) {
    delete B;
    return nullptr;
  }
  B->stream = B->own;
  return B;
}

void cfdg_mixed_delete(cfdg_batch* B) {
  if (!B) return;
  // The caller's stream may already be gone; the batch's own stream and its last
  // event cover its work.
  if (B->own) cudaStreamSynchronize(B->own);
  if (B->ev1) cudaEventSynchronize(B->ev1);
  delete B;
}

void cfdg_mixed_set_stream(cfdg_batch* B, cudaStream_t s) { B->stream = s ? s : B->own; }

// ----------------------------------------------------------------- serving: continuous batching
// A server keeps a set of resident grids (one slot each) and a queue of projection
// requests. Each progress() round finishes the cases that converged (epilogue, result
// recorded), admits queued requests into free slots up to `max_active` (prologue), points
// the work-lists at the active cases and replays one chunk of the iteration graph, so a
// request that arrives while others run joins them at the next chunk boundary. A grid
// serves its requests in order, one at a time (a time step needs the previous one).
struct cfdg_server {
  cfdg_batch* B = nullptr;
  int max_active = 0;
  struct Req {
    uint64_t ticket;
    int grid;
    double *u, *p;
    double dt, tol;
    uint64_t max_iter;
    int slot;              // host-buffer requests: the grid's device slot (0 or 1), else -1
    double *hu, *hp;       // host-buffer requests: where the results go
  };
  // Host-buffer requests (cfdg_server_submit_host): per grid two device slots holding a
  // request's u and p; the input copy runs on `cin`, the chunk that admits the request
  // waits for it (`ready`), the result copy runs on `cout` after the epilogue, and `drained`
  // marks a slot free again once its results reached host memory.
  struct Slots {
    double *u[2] = {nullptr, nullptr}, *p[2] = {nullptr, nullptr};
    cudaEvent_t ready[2] = {nullptr, nullptr}, drained[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    bool busy[2] = {false, false};  // held by a request whose result copy is not yet issued
    int next = 0;
  };
  std::vector<Slots> slots;
  cudaStream_t cin = nullptr, cout = nullptr;
  struct HostDone {
    int grid, slot;
  };
  std::map<uint64_t, HostDone> copying;  // finished host requests whose results are in flight
  std::deque<Req> queue;
  std::vector<uint64_t> running;  // ticket per case, 0 when idle
  std::vector<Req> running_req;  // the running request per case
  struct Done {
    cfdg_info info;
    int32_t code;
  };
  std::map<uint64_t, Done> results;
  uint64_t next_ticket = 1;
  bool launched = false;
  std::mutex mu;
  // Observability: graph chunks, their device time (events around each launch, read at
  // the next progress), host time inside progress, cases finished and admitted.
  cudaEvent_t ca = nullptr, cb = nullptr, epi = nullptr;
  // Between consecutive chunks: the end of the earlier one (pcb) to the start of the next
  // (ca), i.e. epilogues, prologues and the device waiting on the host.
  cudaEvent_t pcb = nullptr;
  bool timing = false, gap_timing = false;
  double gap_ms = 0.0, work_ms = 0.0;
  uint64_t gaps = 0, last_chunk_round = 0;
  uint64_t chunks = 0, finished = 0, admitted = 0, rounds = 0;
  double chunk_ms = 0.0, host_ms = 0.0;
  ~cfdg_server() {
    if (ca) cudaEventDestroy(ca);
    if (cb) cudaEventDestroy(cb);
    if (pcb) cudaEventDestroy(pcb);
    if (epi) cudaEventDestroy(epi);
    for (auto& g : slots)
      for (int k = 0; k < 2; ++k) {
        if (g.u[k]) cudaFree(g.u[k]);
        if (g.p[k]) cudaFree(g.p[k]);
        if (g.ready[k]) cudaEventDestroy(g.ready[k]);
        if (g.drained[k]) cudaEventDestroy(g.drained[k]);
      }
    if (cin) cudaStreamDestroy(cin);
    if (cout) cudaStreamDestroy(cout);
  }
};

// Checks div_rdt against the correctly rounded division on generated numerators: mode 0
// random significands over the exponents div_rdt takes, mode 1 products RN(y m) (quotients
// next to a double), mode 2 quotients next to the midpoint between two doubles.
__global__ void k_div_check(double y, double ry, unsigned long long seed, long long n, int mode,
                            unsigned long long* bad) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long z = seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(i + 1);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    const unsigned long long mant = z & 0xfffffffffffffull, sign = (z >> 63) << 63;
    const int e = 123 + (int)((z >> 52) % 1801ull);
    double x = __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | mant));
    if (mode > 0) {
      // m near 1 so that x = y m stays within the exponent range for every y in [2^-60, 2^60]
      const double m = __longlong_as_double((long long)(sign | (1023ull << 52) | mant));
      x = mode == 1 ? __dmul_rn(y, m) : __fma_rn(y, m, __dmul_rn(y, __dmul_rn(m, 0x1p-53)));
    }
    const double a = div_rdt(x, y, ry), b = __ddiv_rn(x, y);
    if (__double_as_longlong(a) != __double_as_longlong(b)) atomicAdd(bad, 1ull);
  }
}

extern "C" {

int cfdg_debug_div_check(double y, uint64_t seed, int64_t n, int32_t mode, uint64_t* mismatches) {
  if (n < 1 || mode < 0 || mode > 2 || !mismatches) return fail(CFDG_ERR_INVALID, "invalid arguments");
  unsigned long long* d = nullptr;
  CU(cudaMalloc(&d, sizeof(unsigned long long)));
  CU(cudaMemset(d, 0, sizeof(unsigned long long)));
  k_div_check<<<4 * 152, 256>>>(y, rdt_of(y), seed, n, mode, d);
  const cudaError_t le = cudaGetLastError();
  unsigned long long h = 0;
  const cudaError_t ce = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CU(le);
  CU(ce);
  *mismatches = h;
  return 0;
}

int cfdg_batch_debug_rhs(cfdg_batch* B, int32_t c, double* b, double* terms) {
  if (!B || c < 0 || c >= (int)B->grids.size() || !b || !terms) return fail(CFDG_ERR_INVALID, "invalid arguments");
  CU(cudaSetDevice(B->ctx->device));
  Locks locks(B->grids);
  const FineCase& F = B->h_fc[c];
  if (!F.b) return fail(CFDG_ERR_INVALID, "the batch has not projected yet");
  CU(cudaStreamSynchronize(B->stream));
  CU(cudaMemcpy(b, F.b, sizeof(double) * F.N, cudaMemcpyDeviceToHost));
  CU(cudaMemcpy(terms, F.terms, sizeof(double) * F.N, cudaMemcpyDeviceToHost));
  return 0;
}

int cfdg_batch_create(cfdg_context* ctx, cfdg_grid* const* grids, int32_t n, cfdg_batch** out) {
  if (!ctx || !grids || n < 1 || !out) return fail(CFDG_ERR_INVALID, "invalid batch arguments");
  *out = nullptr;
  CU(cudaSetDevice(ctx->device));
  cfdg_batch* B = cfdg_mixed_new(ctx);
  if (!B) return fail(CFDG_ERR_CUDA, "could not create the batch stream");
  for (int i = 0; i < n; ++i) {
    cfdg_grid* G = grids[i];
    if (!G || G->ctx != ctx) {
      cfdg_mixed_delete(B);
      return fail(CFDG_ERR_INVALID, "every grid of a batch must be open on the batch's context");
    }
    for (int j = 0; j < i; ++j)
      if (grids[j] == G) {
        cfdg_mixed_delete(B);
        return fail(CFDG_ERR_INVALID, "a grid can appear once in a batch");
      }
    std::lock_guard<std::mutex> lk(G->mu);
    if (int e = prepare_multigrid(G)) {
      cfdg_mixed_delete(B);
      return e;
    }
    if (int e = cfdg_mixed_add_case(B, G)) {
      cfdg_mixed_delete(B);
      return e;
    }
  }
  if (int e = cfdg_mixed_pack(B)) {
    cfdg_mixed_delete(B);
    return e;
  }
  *out = B;
  return 0;
}

void cfdg_batch_destroy(cfdg_batch* B) { cfdg_mixed_delete(B); }

int cfdg_batch_set_stream(cfdg_batch* B, void* stream) {
  if (!B) return fail(CFDG_ERR_INVALID, "null batch");
  CU(cudaStreamSynchronize(B->stream));
  cfdg_mixed_set_stream(B, (cudaStream_t)stream);
  return 0;
}

int cfdg_batch_size(const cfdg_batch* B) { return B ? (int)B->cases.size() : 0; }

int64_t cfdg_batch_stats_json(cfdg_batch* B, char* buf, int64_t cap) {
  if (!B) return -(int64_t)fail(CFDG_ERR_INVALID, "null batch");
  Locks locks(B->grids);
  char tmp[256];
  snprintf(tmp, sizeof tmp,
           "{\"coarse_kernel\": \"%s\", \"coarse_blocks\": %d, \"staged_sweeps\": %s, \"sweep_blocks\": %d, "
           "\"sweep_rows\": %d, \"sweep_stages\": %d, \"cases\": [",
           B->coop ? "cooperative" : "cluster", B->coop ? B->coop_blocks : (int)B->cases.size() * B->csize,
           B->rb_tma ? "true" : "false", B->rb_tma ? B->rb_grid : B->g_fine, B->rb_tma ? B->rb_sr : RT,
           B->rb_tma ? B->rb_ns : 0);
  std::string out = tmp;
  for (size_t i = 0; i < B->cases.size(); ++i) {
    const CaseState& cs = *B->cases[i];
    snprintf(tmp, sizeof tmp,
             "%s{\"cells\": %d, \"groups0\": %d, \"level1_bins\": %s, \"level1_stencil\": %s, \"levels\": [",
             i ? ", " : "", cs.F.N, cs.ngroups0, cs.F.bin1 ? "true" : "false",
             cs.C.lv[0].scode ? "true" : "false");
    out += tmp;
    for (size_t l = 0; l < cs.stats.size(); ++l) {
      const auto& v = cs.stats[l];
      snprintf(tmp, sizeof tmp,
               "%s{\"rows\": %lld, \"nnz\": %lld, \"smoother\": \"%s\", \"colors\": %d, \"ell_entries\": %lld, "
               "\"groups\": %lld, \"blocks\": %lld, \"bin_stencil\": %s}",
               l ? ", " : "", v.rows, v.nnz, v.jacobi ? "l1-jacobi" : "gauss-seidel", v.colors, v.ell, v.groups,
               v.blocks, v.stencil ? "true" : "false");
      out += tmp;
    }
    out += "]}";
  }
  out += "]}";
  if (buf && cap > 0) {
    const size_t k = std::min((size_t)cap - 1, out.size());
    memcpy(buf, out.data(), k);
    buf[k] = 0;
  }
  return (int64_t)out.size() + 1;
}

// Algorithmic bytes of one launch of the coarse levels of every case (each logical array
// read or written once per phase): per non-terminal level of n rows, E ELL entries (8 bytes
// each: value and column) and nnz CSR entries, the 2 nu sweeps read the ELL block, the
// right-hand side and 1/diag and write x (8 E + 12 n each); x is zeroed (4 n); the residual
// reads the ELL block of colour 0 with diag, x and rhs and writes res (a res0 level, about
// half: 4 E + 8 n), or the CSR rows (8 nnz + 20 n); the restriction reads res, children and
// weights (12 n) and writes the next level's right-hand side; the prolongation reads the
// injection rows and updates x (20 n). The terminal blocks read their inverse (8 m^2 each).
double coarse_bytes(const cfdg_batch* B) {
  double total = 0.0;
  const double nu = (double)B->nuc;
  for (const auto& cs : B->cases) {
    for (size_t l = 0; l < cs->stats.size(); ++l) {
      const auto& v = cs->stats[l];
      const double n = (double)v.rows, E = (double)v.ell, nnz = (double)v.nnz;
      const bool terminal = (int)l == cs->C.nl - 1;
      if (terminal) {
        total += 8.0 * n + 8.0 * n * 32.0;  // rhs in, x out, up to 32 x 32 inverse entries per row
        continue;
      }
      const bool res0 = cs->C.lv[l].res0 != 0;
      total += 2.0 * nu * (8.0 * E + 12.0 * n) + 4.0 * n;
      total += res0 ? 4.0 * E + 8.0 * n : 8.0 * nnz + 20.0 * n;
      total += 12.0 * n + 4.0 * (l + 1 < cs->stats.size() ? (double)cs->stats[l + 1].rows : 0.0);
      total += 20.0 * n;
    }
  }
  return total;
}

int cfdg_batch_time_kernel(cfdg_batch* B, int32_t which, int32_t reps, double* ms_per_launch,
                           double* algorithmic_bytes) {
  if (!B || reps < 1) return fail(CFDG_ERR_INVALID, "invalid arguments");
  CU(cudaSetDevice(B->ctx->device));
  Locks locks(B->grids);
  const int nc = (int)B->cases.size();
  cudaStream_t s = B->stream;
  if (which == 6)
    for (int i = 0; i < nc; ++i)
      if (B->h_fc[i].u != B->grids[i]->u)
        return fail(CFDG_ERR_INVALID, "time the right-hand side after a host-buffer projection of the batch");
  // Every case in the inner-iteration state, on the vectors of the last solve (the FP64
  // true residual: every case in an outer step with a correction; the right-hand side:
  // every case idle, on the batch's own copy of the last inputs).
  std::vector<MState> saved(nc), run(nc);
  CU(cudaMemcpyAsync(saved.data(), B->d_st, sizeof(MState) * nc, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  for (int i = 0; i < nc; ++i) {
    run[i] = saved[i];
    run[i].state = which == 5 ? OUTER : which == 6 ? IDLE : RUN;
    run[i].has_e = 1;
    run[i].counter = 0;
  }
  CU(cudaMemcpyAsync(B->d_st, run.data(), sizeof(MState) * nc, cudaMemcpyHostToDevice, s));
  B->active.assign(nc, 1);
  if (int e = set_active(B, s)) return e;
  double cells = 0;
  for (auto& F : B->h_fc) cells += F.N;
  double bytes = 0;
  auto launch = [&]() {
    switch (which) {
      case 0:  // one red-black half sweep over every case's fine level
        launch_rb(B, B->run, 1, 0, s);
        break;
      case 4:  // the same half sweep with the register kernel (no staging), for comparison
        FINE(k_rb, B->run, 1, 0);
        break;
      case 1:  // FP32 operator q = A p (with p.q)
        FINE(k_op, B->run);
        break;
      case 2:  // all coarse levels of all cases
        launch_coarse(B, s);
        break;
      case 5:  // FP64 true residual r = b_c - A x with |r|^2
        FINE(k_outer_resid, B->run);
        break;
      case 6:  // FP64 right-hand side b = -div(u)/dt
        FINE(k_rhs, B->run);
        break;
      case 7:  // level-0 residual and its restriction to level 1
        FINE(k_v_resid, B->run);
        k_v_restrict<<<grid_of(k_v_restrict, TILE, B->g_1), TILE, 0, s>>>(B->d_fc, B->d_st, B->run.tiles1,
                                                                          B->run.counts + 1);
        break;
      case 9:  // e += alpha p, r -= alpha q with |r|^2
        FINE(k_update, B->run);
        break;
      case 10:  // r.z
        FINE(k_rz, B->run);
        break;
      case 11:  // p = z + beta p
        FINE(k_p, B->run);
        break;
      case 8:  // level-1 correction prolonged to level 0
        FINE(k_v_prolong, B->run);
        break;
      default:
        enqueue_vcycle(B, s);
        break;
    }
  };
  if (which == 0 || which == 4) bytes = 9.0 * cells;  // half the cells: rhs, 1/diag, u16 flags, x out; the other half's x in
  else if (which == 1) bytes = 10.0 * cells; // p in, u16 flags, q out
  else if (which == 2) bytes = coarse_bytes(B);
  else if (which == 5) bytes = 34.0 * cells;  // x, b_c, diag, r out (FP64), u16 flags
  else if (which == 9) bytes = 24.0 * cells;  // e, p, r, q in; e, r out
  else if (which == 10) bytes = 8.0 * cells;  // r, z in
  else if (which == 11) bytes = 12.0 * cells; // z, p in; p out
  else if (which == 6) {
    for (auto& F : B->h_fc) bytes += 8.0 * (double)F.F + 17.0 * F.N;  // u faces, fluid, b and terms out
  }
  float ms = 0;
  if (which == 5 || which == 6 || which == 9 || which == 10) {
    // These kernels move the cases' states on: restore them before every launch and time
    // the launches alone.
    for (int r = -2; r < reps; ++r) {
      CU(cudaMemcpyAsync(B->d_st, run.data(), sizeof(MState) * nc, cudaMemcpyHostToDevice, s));
      CU(cudaEventRecord(B->ev0, s));
      launch();
      CU(cudaEventRecord(B->ev1, s));
      CU(cudaEventSynchronize(B->ev1));
      float one = 0;
      CU(cudaEventElapsedTime(&one, B->ev0, B->ev1));
      if (r >= 0) ms += one;
    }
  } else {
    launch();
    launch();
    CU(cudaEventRecord(B->ev0, s));
    for (int r = 0; r < reps; ++r) launch();
    CU(cudaEventRecord(B->ev1, s));
    CU(cudaEventSynchronize(B->ev1));
    CU(cudaEventElapsedTime(&ms, B->ev0, B->ev1));
  }
  CU(cudaMemcpyAsync(B->d_st, saved.data(), sizeof(MState) * nc, cudaMemcpyHostToDevice, s));
  CU(cudaStreamSynchronize(s));
  CU(cudaGetLastError());
  if (ms_per_launch) *ms_per_launch = ms / reps;
  if (algorithmic_bytes) *algorithmic_bytes = bytes;
  return 0;
}

int cfdg_batch_project_device(cfdg_batch* B, double* const* d_u, double* const* d_p, const double* dt, double tol,
                              uint64_t max_iter, cfdg_poll_fn poll, void* poll_ctx, cfdg_info* infos, int32_t* codes) {
  if (!B || !d_u || !d_p || !dt) return fail(CFDG_ERR_INVALID, "invalid batch arguments");
  CU(cudaSetDevice(B->ctx->device));
  Locks locks(B->grids);
  if (int e = refresh_batch(B)) return e;
  return cfdg_mixed_project(B, d_u, d_p, dt, tol, max_iter, poll, poll_ctx, infos, codes);
}

int cfdg_batch_project(cfdg_batch* B, double* const* u, double* const* p, const double* dt, double tol,
                       uint64_t max_iter, cfdg_poll_fn poll, void* poll_ctx, cfdg_info* infos, int32_t* codes) {
  if (!B || !u || !p || !dt) return fail(CFDG_ERR_INVALID, "invalid batch arguments");
  CU(cudaSetDevice(B->ctx->device));
  Locks locks(B->grids);
  if (int e = refresh_batch(B)) return e;
  const int nc = (int)B->grids.size();
  std::vector<double*> du(nc), dp(nc);
  cudaStream_t s = B->stream;
  for (int i = 0; i < nc; ++i) {
    cfdg_grid* G = B->grids[i];
    du[i] = G->u;
    dp[i] = G->pp;
    CU(cudaMemcpyAsync(G->u, u[i], G->h.faces * 8, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(G->pp, p[i], G->h.cells * 8, cudaMemcpyHostToDevice, s));
  }
  std::vector<int32_t> local(nc, 0);
  int32_t* cd = codes ? codes : local.data();
  int st = cfdg_mixed_project(B, du.data(), dp.data(), dt, tol, max_iter, poll, poll_ctx, infos, cd);
  if (st) return st;
  for (int i = 0; i < nc; ++i) {
    if (cd[i]) continue;  // transactional: a failed case keeps its inputs
    cfdg_grid* G = B->grids[i];
    CU(cudaMemcpyAsync(u[i], G->u, G->h.faces * 8, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(p[i], G->pp, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  }
  CU(cudaStreamSynchronize(s));
  return 0;
}

// ------------------------------------------------------------------ server
int cfdg_server_create(cfdg_context* ctx, cfdg_grid* const* grids, int32_t n, int32_t max_active,
                       cfdg_server** out) {
  if (!out || max_active < 1) return fail(CFDG_ERR_INVALID, "invalid server arguments");
  *out = nullptr;
  cfdg_batch* B = nullptr;
  if (int e = cfdg_batch_create(ctx, grids, n, &B)) return e;
  auto* S = new cfdg_server();
  S->B = B;
  S->max_active = max_active;
  if (cudaEventCreate(&S->ca) != cudaSuccess || cudaEventCreate(&S->cb) != cudaSuccess ||
      cudaEventCreate(&S->pcb) != cudaSuccess ||
      cudaEventCreateWithFlags(&S->epi, cudaEventDisableTiming) != cudaSuccess) {
    cfdg_batch_destroy(B);
    delete S;
    return fail(CFDG_ERR_CUDA, "could not create the server's events");
  }
  S->running.assign(n, 0);
  S->running_req.assign(n, cfdg_server::Req{});
  B->active.assign(n, 0);
  int e = 0;
  {
    Locks locks(B->grids);
    if (B->chunk) cudaGraphExecDestroy(B->chunk);
    B->chunk = nullptr;
    B->chunk_it = SERVER_CHUNK_IT;
    e = ensure_graph(B);
    if (!e) e = set_active(B, B->stream);
  }
  if (e) {
    cfdg_batch_destroy(B);
    delete S;
    return e;
  }
  *out = S;
  return 0;
}

void cfdg_server_destroy(cfdg_server* S) {
  if (!S) return;
  cfdg_batch_destroy(S->B);
  delete S;
}

int cfdg_server_set_stream(cfdg_server* S, void* stream) {
  if (!S) return fail(CFDG_ERR_INVALID, "null server");
  return cfdg_batch_set_stream(S->B, stream);
}

int cfdg_server_set_chunk(cfdg_server* S, int32_t iterations) {
  if (!S || iterations < 1 || iterations > 64) return fail(CFDG_ERR_INVALID, "chunk iterations must be 1..64");
  std::lock_guard<std::mutex> lk(S->mu);
  cfdg_batch* B = S->B;
  CU(cudaSetDevice(B->ctx->device));
  if (iterations == B->chunk_it) return 0;
  CU(cudaStreamSynchronize(B->stream));
  if (B->chunk) cudaGraphExecDestroy(B->chunk);
  B->chunk = nullptr;
  B->chunk_it = iterations;
  Locks locks(B->grids);
  return ensure_graph(B);
}

int cfdg_server_submit(cfdg_server* S, int32_t grid, double* d_u, double* d_p, double dt, double tol,
                       uint64_t max_iter, uint64_t* ticket) {
  if (!S || grid < 0 || grid >= (int)S->B->grids.size() || !d_u || !d_p || !ticket)
    return fail(CFDG_ERR_INVALID, "invalid submit arguments");
  std::lock_guard<std::mutex> lk(S->mu);
  *ticket = S->next_ticket++;
  S->queue.push_back({*ticket, grid, d_u, d_p, dt, tol, max_iter, -1, nullptr, nullptr});
  return 0;
}

int cfdg_server_submit_host(cfdg_server* S, int32_t grid, const double* u, const double* p, double* u_out,
                            double* p_out, double dt, double tol, uint64_t max_iter, uint64_t* ticket) {
  if (!S || grid < 0 || grid >= (int)S->B->grids.size() || !u || !p || !u_out || !p_out || !ticket)
    return fail(CFDG_ERR_INVALID, "invalid submit arguments");
  std::lock_guard<std::mutex> lk(S->mu);
  cfdg_batch* B = S->B;
  CU(cudaSetDevice(B->ctx->device));
  if (!S->cin) {
    CU(cudaStreamCreateWithFlags(&S->cin, cudaStreamNonBlocking));
    CU(cudaStreamCreateWithFlags(&S->cout, cudaStreamNonBlocking));
  }
  if (S->slots.empty()) S->slots.resize(B->grids.size());
  cfdg_server::Slots& g = S->slots[grid];
  const size_t F = (size_t)B->h_fc[grid].F, N = (size_t)B->h_fc[grid].N;
  const int k = g.next;
  // A grid's requests run one at a time, so two slots let the next input copy overlap the
  // running request; a slot whose results are still being copied out is waited for on the
  // copy stream. A third request before either earlier one has finished has no slot.
  if (g.busy[k])
    return fail(CFDG_ERR_INVALID, "two host requests of this grid are unfinished; collect one before submitting");
  if (!g.u[k]) {
    CU(cudaMalloc(&g.u[k], F * sizeof(double)));
    CU(cudaMalloc(&g.p[k], N * sizeof(double)));
    CU(cudaEventCreateWithFlags(&g.ready[k], cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&g.drained[k], cudaEventDisableTiming));
  }
  if (g.used[k]) CU(cudaStreamWaitEvent(S->cin, g.drained[k], 0));
  CU(cudaMemcpyAsync(g.u[k], u, F * sizeof(double), cudaMemcpyHostToDevice, S->cin));
  CU(cudaMemcpyAsync(g.p[k], p, N * sizeof(double), cudaMemcpyHostToDevice, S->cin));
  CU(cudaEventRecord(g.ready[k], S->cin));
  g.used[k] = true;
  g.busy[k] = true;
  g.next = 1 - k;
  *ticket = S->next_ticket++;
  S->queue.push_back({*ticket, grid, g.u[k], g.p[k], dt, tol, max_iter, k, u_out, p_out});
  return 0;
}

int cfdg_server_progress(cfdg_server* S, int32_t* finished) {
  if (!S) return fail(CFDG_ERR_INVALID, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  cfdg_batch* B = S->B;
  CU(cudaSetDevice(B->ctx->device));
  Locks locks(B->grids);
  cudaStream_t s = B->stream;
  const int nc = (int)B->cases.size();
  int nfin = 0;
  const auto h0 = std::chrono::steady_clock::now();
  struct HostClock {
    cfdg_server* S;
    std::chrono::steady_clock::time_point t0;
    ~HostClock() {
      S->host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  } host_clock{S, h0};
  ++S->rounds;
  // 1. Finish the cases that converged or failed in the last chunk.
  CU(cudaMemcpyAsync(B->h_st, B->d_st, sizeof(MState) * nc, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  const auto w0 = std::chrono::steady_clock::now();
  struct WorkClock {
    cfdg_server* S;
    std::chrono::steady_clock::time_point t0;
    ~WorkClock() {
      S->work_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
  } work_clock{S, w0};
  if (S->timing) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, S->ca, S->cb) == cudaSuccess) S->chunk_ms += ms;
    if (S->gap_timing && cudaEventElapsedTime(&ms, S->pcb, S->ca) == cudaSuccess) {
      S->gap_ms += ms;
      ++S->gaps;
    }
    S->timing = false;
  }
  std::vector<char> done(nc, 0), fin(nc, 0);
  bool changed = false;
  for (int i = 0; i < nc; ++i) {
    if (!S->running[i]) continue;
    const int st = B->h_st[i].state;
    if (st == DONE || st == FAIL) {
      fin[i] = 1;
      done[i] = st == DONE;
    }
  }
  // The epilogue of the converged cases is queued first (it reads their descriptors
  // before an admission below may point them at a new request); their results are
  // published once it has run, after the next chunk is queued.
  bool any_done = false;
  for (int i = 0; i < nc; ++i) any_done |= done[i] != 0;
  if (any_done) {
    if (int e = epilogue(B, done, s)) return e;
    CU(cudaEventRecord(S->epi, s));
  }
  std::vector<std::pair<uint64_t, cfdg_server::Done>> out;
  bool any_host = false;
  for (int i = 0; i < nc; ++i) any_host |= fin[i] && S->running_req[i].slot >= 0;
  if (any_host && !any_done) CU(cudaEventRecord(S->epi, s));  // failed requests: their inputs go back
  for (int i = 0; i < nc; ++i) {
    if (!fin[i]) continue;
    cfdg_server::Done d;
    fill_info(B->h_st[i], d.info);
    d.code = B->h_st[i].state == DONE ? 0 : (B->h_st[i].error ? B->h_st[i].error : CFDG_E033);
    const cfdg_server::Req& rq = S->running_req[i];
    if (rq.slot >= 0) {
      // The results (or, for a failed request, its unchanged inputs) to host memory once
      // the epilogue has run; the ticket reports done when the copy has completed.
      cfdg_server::Slots& g = S->slots[i];
      const size_t F = (size_t)B->h_fc[i].F, N = (size_t)B->h_fc[i].N;
      CU(cudaStreamWaitEvent(S->cout, S->epi, 0));
      CU(cudaMemcpyAsync(rq.hu, g.u[rq.slot], F * sizeof(double), cudaMemcpyDeviceToHost, S->cout));
      CU(cudaMemcpyAsync(rq.hp, g.p[rq.slot], N * sizeof(double), cudaMemcpyDeviceToHost, S->cout));
      CU(cudaEventRecord(g.drained[rq.slot], S->cout));
      g.busy[rq.slot] = false;
      S->copying[S->running[i]] = {i, rq.slot};
    }
    out.push_back({S->running[i], d});
    S->running[i] = 0;
    B->active[i] = 0;
    changed = true;
    ++nfin;
    ++S->finished;
  }
  // 2. Admit queued requests into free slots (in arrival order; one per grid at a time).
  int nactive = 0;
  for (int i = 0; i < nc; ++i) nactive += S->running[i] != 0;
  std::vector<char> admit(nc, 0);
  bool any_admit = false;
  for (auto it = S->queue.begin(); it != S->queue.end() && nactive < S->max_active;) {
    if (S->running[it->grid] || admit[it->grid]) {
      ++it;
      continue;
    }
    const int i = it->grid;
    B->h_fc[i].u = it->u;
    B->h_fc[i].pfield = it->p;
    B->h_fc[i].dt = it->dt;
    B->h_fc[i].rdt = rdt_of(it->dt);
    B->h_st[i] = initial_state(it->tol, it->max_iter);
    S->running[i] = it->ticket;
    S->running_req[i] = *it;
    if (it->slot >= 0) CU(cudaStreamWaitEvent(s, S->slots[i].ready[it->slot], 0));  // its input copy
    ++S->admitted;
    admit[i] = 1;
    any_admit = true;
    B->active[i] = 1;
    ++nactive;
    changed = true;
    it = S->queue.erase(it);
  }
  if (any_admit) {
    // Nothing has run since the states were read, so the other cases' device states
    // equal h_st and whole-array copies are exact.
    if (int e = staged_h2d(B, B->d_fc, B->h_fc.data(), sizeof(FineCase) * nc, s)) return e;
    if (int e = staged_h2d(B, B->d_st, B->h_st, sizeof(MState) * nc, s)) return e;
    if (int e = prologue(B, admit, s)) return e;
  }
  // 3. Point the work-lists at the active cases and run one chunk.
  if (changed)
    if (int e = set_active(B, s)) return e;
  if (nactive > 0) {
    // pcb keeps the previous chunk's end when that chunk ran in the round just before.
    S->gap_timing = S->chunks > 0 && S->last_chunk_round + 1 == S->rounds;
    std::swap(S->cb, S->pcb);
    CU(cudaEventRecord(S->ca, s));
    CU(cudaGraphLaunch(B->chunk, s));
    CU(cudaEventRecord(S->cb, s));
    S->last_chunk_round = S->rounds;
    S->timing = true;
    ++S->chunks;
    count(B->chunk_nodes);
  }
  if (any_done) CU(cudaEventSynchronize(S->epi));
  for (auto& r : out) S->results[r.first] = r.second;
  if (finished) *finished = nfin;
  return 0;
}

int cfdg_server_result(cfdg_server* S, uint64_t ticket, cfdg_info* info, int32_t* code) {
  if (!S) return fail(CFDG_ERR_INVALID, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->results.find(ticket);
  if (it == S->results.end()) return CFDG_PENDING;
  auto hc = S->copying.find(ticket);
  if (hc != S->copying.end()) {  // a host-buffer request: done once its results are in host memory
    const cudaError_t q = cudaEventQuery(S->slots[hc->second.grid].drained[hc->second.slot]);
    if (q == cudaErrorNotReady) return CFDG_PENDING;
    if (q != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("result copy: ") + cudaGetErrorString(q));
    S->copying.erase(hc);
  }
  if (info) *info = it->second.info;
  if (code) *code = it->second.code;
  S->results.erase(it);
  return 0;
}

int64_t cfdg_server_stats_json(cfdg_server* S, char* buf, int64_t cap) {
  if (!S) return -(int64_t)fail(CFDG_ERR_INVALID, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  char tmp[512];
  snprintf(tmp, sizeof tmp,
           "{\"rounds\": %llu, \"chunks\": %llu, \"iterations_per_chunk\": %d, \"chunk_device_ms\": %.3f, "
           "\"progress_host_ms\": %.3f, \"progress_work_ms\": %.3f, \"between_chunks_ms\": %.3f, "
           "\"chunk_pairs\": %llu, \"finished\": %llu, \"admitted\": %llu}",
           (unsigned long long)S->rounds, (unsigned long long)S->chunks, S->B->chunk_it, S->chunk_ms, S->host_ms,
           S->work_ms, S->gap_ms, (unsigned long long)S->gaps, (unsigned long long)S->finished,
           (unsigned long long)S->admitted);
  const std::string out = tmp;
  if (buf && cap > 0) {
    const size_t k = std::min((size_t)cap - 1, out.size());
    memcpy(buf, out.data(), k);
    buf[k] = 0;
  }
  return (int64_t)out.size() + 1;
}

int cfdg_server_pending(cfdg_server* S) {
  if (!S) return 0;
  std::lock_guard<std::mutex> lk(S->mu);
  int n = (int)S->queue.size();
  for (auto t : S->running) n += t != 0;
  return n;
}

}  // extern "C"
