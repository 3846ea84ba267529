// GB300 pressure-projection engine: device kernels of the plain FP64 form and the
// C ABI of include/cfdgpu.h.
//
// Build: nvcc -gencode arch=compute_103a,code=sm_103a -fmad=false (see build.py).
//
// Layout in HBM, per grid (N cells, F faces):
//   flags  u16[N]   interior/outlet bits of the six faces of each cell
//   fw     f64[F]   face weights area/(distance*volume), recomputed when faces change
//   face_kind u8[F], face_lo/face_hi i32[F], face_dist f64[F]   (velocity correction)
//   x r z p ap bc b terms  f64[N]   PCG and projection vectors
//   IC(0): lower CSR (i32 off/col, f64 val), its transpose, diag, level orders
//   multigrid: per level CSR + diag, level orders, transfer CSRs, vectors
// The PCG loop runs as CUDA graphs of 8 iterations; every kernel first reads the
// device Scalars and returns at once when the solve has finished, so the host only
// synchronises between chunks, where it polls the caller's Control.
//
// Also here, on device arrays: laminar SSPRK2 time stepping (momentum right-hand side
// and stage update, cfdg_step_device), linear-upwind scalar transport (k_scalar_pass,
// cfdg_scalar_step_device), receptor sampling (cfdg_receptors_sample), and the
// line/plane block smoothers of anisotropic multigrid hierarchies (line_block, in the
// cooperative V-cycle k_plain_coarse). All of it follows the reference's operation order
// (bit-identical results) under -fmad=false.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/cfdgpu.h"
#include "plain_kernels.cuh"
#include "setup.hpp"
#include "wave.cuh"

using namespace cfdg;

// ============================================================== device helpers

namespace {

__device__ __forceinline__ double block_sum(double v, double* sh) {
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
  return s;  // valid in thread 0
}

// Publishes this block's partial; true in every thread of the block that arrives last.
__device__ __forceinline__ bool arrive(double partial, double* partials, unsigned* counter) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = partial;
    __threadfence();
    unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

// Sum of the partials in a fixed order (thread 0), by the last block.
__device__ __forceinline__ double gather_partials(const double* partials, double* sh, unsigned* counter) {
  __threadfence();
  double v = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) v += __ldcg(&partials[b]);
  double s = block_sum(v, sh);
  if (threadIdx.x == 0) *counter = 0;
  return s;
}

__device__ __forceinline__ long long face_index(const GridDev& g, int a, int q0, int q1, int q2) {
  return g.face_off[a] + ((long long)q2 * g.fdim[a][1] + q1) * g.fdim[a][0] + q0;
}

// (A x)_c in the reference's face order (pressure.rs:273-285, grid.rs:341-429):
// for each axis the lower face, then the upper face, except on a periodic axis
// where the last cell's upper face is the wrap face at coordinate 0, which comes
// first in face order. Interior faces add d = w (x_lo - x_hi) to lo and subtract
// it from hi; outlet faces add w x_c.
template <bool UNIFORM>
__device__ __forceinline__ double op_cell(const GridDev& g, const double* __restrict__ x, int c, int q0, int q1,
                                          int q2, unsigned fl) {
  double y = 0.0;
  const double xc = x[c];
  const int q[3] = {q0, q1, q2};
  const int stride[3] = {1, g.n[0], g.n[0] * g.n[1]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const unsigned lin = (fl >> (2 * a)) & 1u, uin = (fl >> (2 * a + 1)) & 1u;
    const unsigned lout = (fl >> (6 + 2 * a)) & 1u, uout = (fl >> (7 + 2 * a)) & 1u;
    if (!(lin | uin | lout | uout)) continue;
    const int na = g.n[a];
    double wl, wu;
    if (UNIFORM) {
      wl = lout ? g.w_out[a] : g.w_in[a];
      wu = uout ? g.w_out[a] : g.w_in[a];
    } else {
      int p[3] = {q0, q1, q2};
      wl = g.fw[face_index(g, a, p[0], p[1], p[2])];
      p[a] = (g.per[a] && q[a] == na - 1) ? 0 : q[a] + 1;
      wu = g.fw[face_index(g, a, p[0], p[1], p[2])];
    }
    if (g.per[a] && na == 1) {  // one face joining the cell to itself
      if (lin) {
        double d = wl * (xc - xc);
        y = y + d;
        y = y - d;
      }
      continue;
    }
    const int nl = q[a] > 0 ? c - stride[a] : c + (na - 1) * stride[a];
    const int nu = q[a] < na - 1 ? c + stride[a] : c - (na - 1) * stride[a];
    const bool upper_first = g.per[a] && q[a] == na - 1;
    for (int s = 0; s < 2; ++s) {
      const bool upper = (s == 0) == upper_first;
      if (!upper) {
        if (lin) {
          double d = wl * (x[nl] - xc);
          y = y - d;
        } else if (lout) {
          y = y + wl * xc;
        }
      } else {
        if (uin) {
          double d = wu * (xc - x[nu]);
          y = y + d;
        } else if (uout) {
          y = y + wu * xc;
        }
      }
    }
  }
  return y;
}

__device__ __forceinline__ void cell_coords(const GridDev& g, int c, int& q0, int& q1, int& q2) {
  q0 = c % g.n[0];
  int t = c / g.n[0];
  q1 = t % g.n[1];
  q2 = t / g.n[1];
}

// ============================================================== kernels

template <bool UNIFORM>
__global__ void k_apply(GridDev g, const double* __restrict__ x, double* __restrict__ y, int N) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    int q0, q1, q2;
    cell_coords(g, c, q0, q1, q2);
    unsigned fl = g.flags[c];
    y[c] = fl ? op_cell<UNIFORM>(g, x, c, q0, q1, q2, fl) : 0.0;
  }
}

// Iteration start: Ap = A p, denom = p.Ap, alpha = rz/denom (pressure.rs:391-397).
template <bool UNIFORM>
__global__ void k_pcg_op(GridDev g, const double* __restrict__ p, double* __restrict__ ap, int N, double* partials,
                         Scalars* S) {
  __shared__ double sh[32];
  if (S->done) return;
  if (S->it >= S->max_it) {
    if (blockIdx.x == 0 && threadIdx.x == 0) S->done = 3;
    return;
  }
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    int q0, q1, q2;
    cell_coords(g, c, q0, q1, q2);
    unsigned fl = g.flags[c];
    double v = fl ? op_cell<UNIFORM>(g, p, c, q0, q1, q2, fl) : 0.0;
    ap[c] = v;
    acc += p[c] * v;
  }
  double bs = block_sum(acc, sh);
  if (arrive(bs, partials, &S->counter)) {
    double denom = gather_partials(partials, sh, &S->counter);
    if (threadIdx.x == 0) {
      if (!(denom > 0.0) || !isfinite(denom)) {
        S->done = 2;
        S->error = CFDG_E032;
      } else {
        S->alpha = S->rz / denom;
      }
    }
  }
}

// x += alpha p, r -= alpha Ap, rel = |r|/|b_c| (pressure.rs:398-403).
__global__ void k_pcg_xr(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                         const double* __restrict__ ap, int N, double* partials, Scalars* S) {
  __shared__ double sh[32];
  if (S->done) return;
  const double alpha = S->alpha;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    x[i] = x[i] + alpha * p[i];
    double v = r[i] - alpha * ap[i];
    r[i] = v;
    acc += v * v;
  }
  double bs = block_sum(acc, sh);
  if (arrive(bs, partials, &S->counter)) {
    double rr = gather_partials(partials, sh, &S->counter);
    if (threadIdx.x == 0) {
      S->rel = sqrt(rr) / S->norm;
      S->check = S->rel <= S->tol;
    }
  }
}

// The true-residual gate (pressure.rs:403-425): |A x - b_c| / |b_c| <= 10 tol + 1e-12.
template <bool UNIFORM>
__global__ void k_pcg_true(GridDev g, const double* __restrict__ x, const double* __restrict__ bc, int N,
                           double* partials, Scalars* S) {
  __shared__ double sh[32];
  if (S->done || !S->check) return;
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    int q0, q1, q2;
    cell_coords(g, c, q0, q1, q2);
    unsigned fl = g.flags[c];
    double v = fl ? op_cell<UNIFORM>(g, x, c, q0, q1, q2, fl) : 0.0;
    double d = v - bc[c];
    acc += d * d;
  }
  double bs = block_sum(acc, sh);
  if (arrive(bs, partials, &S->counter)) {
    double s = gather_partials(partials, sh, &S->counter);
    if (threadIdx.x == 0) {
      S->true_checks += 1;
      double tr = sqrt(s) / S->norm;
      S->true_rel = tr;
      if (tr <= S->tol * 10.0 + 1e-12) S->done = 1;
    }
  }
}

// Relative residual |A x - b| / |b| with its per-block partial sums in a caller-free
// scratch array (see cfdg_residual_norm_noalloc). Block k sums cells
// [k*NOALLOC_CHUNK, (k+1)*NOALLOC_CHUNK); the last block to finish adds the partials in
// block order and writes the quotient to out[0].
constexpr int NOALLOC_CHUNK = 2048;
constexpr int NOALLOC_MAX_BLOCKS = 8192;  // at most NOALLOC_MAX_BLOCKS * NOALLOC_CHUNK cells
template <bool UNIFORM>
__global__ void k_residual_norm_noalloc(GridDev g, const double* __restrict__ x, const double* __restrict__ b, int N,
                                        double* scratch, double* __restrict__ out) {
  __shared__ double sh[32];
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + 2 * NOALLOC_MAX_BLOCKS);
  const int lo = blockIdx.x * NOALLOC_CHUNK;
  const int hi = min(N, lo + NOALLOC_CHUNK);
  double rr = 0.0, bb = 0.0;
  for (int c = lo + threadIdx.x; c < hi; c += blockDim.x) {
    int q0, q1, q2;
    cell_coords(g, c, q0, q1, q2);
    unsigned fl = g.flags[c];
    double v = fl ? op_cell<UNIFORM>(g, x, c, q0, q1, q2, fl) : 0.0;
    double d = v - b[c];
    rr += d * d;
    bb += b[c] * b[c];
  }
  double s1 = block_sum(rr, sh);
  double s2 = block_sum(bb, sh);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = s1;
    scratch[NOALLOC_MAX_BLOCKS + blockIdx.x] = s2;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a1 = 0.0, a2 = 0.0;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
    a1 += __ldcg(&scratch[k]);
    a2 += __ldcg(&scratch[NOALLOC_MAX_BLOCKS + k]);
  }
  double t1 = block_sum(a1, sh);
  double t2 = block_sum(a2, sh);
  if (threadIdx.x == 0) {
    // |b| < 1e-24: the solve returns x = 0 and LinearInfo::default(), a zero residual
    // (pressure.rs:372-375).
    const double nb = sqrt(t2);
    out[0] = nb < 1e-24 ? 0.0 : sqrt(t1) / nb;
    *counter = 0;
  }
}

// rz' = r.z, beta = rz'/rz, it += 1 (pressure.rs:428-433). init: the first rz.
__global__ void k_pcg_rz(const double* __restrict__ r, const double* __restrict__ z, int N, double* partials,
                         Scalars* S, int init) {
  __shared__ double sh[32];
  if (S->done) return;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) acc += r[i] * z[i];
  double bs = block_sum(acc, sh);
  if (arrive(bs, partials, &S->counter)) {
    double next = gather_partials(partials, sh, &S->counter);
    if (threadIdx.x == 0) {
      if (init) {
        S->rz = next;
      } else {
        S->beta = next / S->rz;
        S->rz = next;
        S->it += 1;
      }
    }
  }
}

__global__ void k_pcg_p(double* __restrict__ p, const double* __restrict__ z, int N, const Scalars* S) {
  if (S->done) return;
  const double beta = S->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) p[i] = z[i] + beta * p[i];
}

// norm = |r|; a zero right-hand side ends the solve with x = 0 (pressure.rs:372-375).
__global__ void k_pcg_norm(const double* __restrict__ r, int N, double* partials, Scalars* S) {
  __shared__ double sh[32];
  if (S->done) return;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) acc += r[i] * r[i];
  double bs = block_sum(acc, sh);
  if (arrive(bs, partials, &S->counter)) {
    double rr = gather_partials(partials, sh, &S->counter);
    if (threadIdx.x == 0) {
      S->norm = sqrt(rr);
      if (S->norm < 1e-24) S->done = 4;
    }
  }
}

__global__ void k_copy(double* __restrict__ dst, const double* __restrict__ src, int N, const Scalars* S) {
  if (S && S->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) dst[i] = src[i];
}
__global__ void k_fill(double* __restrict__ dst, double v, int N, const Scalars* S) {
  if (S && S->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) dst[i] = v;
}

// Gauge: subtract each group's mean from its members (pressure.rs:316-325,
// masked.rs:82-89). One block per group; the sum is a fixed-order tree.
__global__ void k_center(const int* __restrict__ off, const int* __restrict__ members, double* __restrict__ x,
                         const Scalars* S) {
  __shared__ double sh[32];
  __shared__ double mean;
  if (S && S->done) return;
  const int gidx = blockIdx.x;
  const int b = off[gidx], e = off[gidx + 1];
  double acc = 0.0;
  for (int k = b + threadIdx.x; k < e; k += blockDim.x) acc += x[members[k]];
  double s = block_sum(acc, sh);
  if (threadIdx.x == 0) mean = s / (double)(e - b);
  __syncthreads();
  const double m = mean;
  for (int k = b + threadIdx.x; k < e; k += blockDim.x) x[members[k]] = x[members[k]] - m;
}

// Compatibility of the closed components (pressure.rs:351-362): one block per group.
__global__ void k_compat(const int* __restrict__ off, const int* __restrict__ members, const double* __restrict__ b,
                         const double* __restrict__ terms, int use_terms, Scalars* S) {
  __shared__ double sh[32];
  const int gidx = blockIdx.x;
  const int lo = off[gidx], hi = off[gidx + 1];
  double acc = 0.0, sc = 0.0;
  for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
    double v = b[members[k]];
    acc += v;
    sc += fmax(fabs(v), use_terms ? terms[members[k]] : 0.0);
  }
  double s = block_sum(acc, sh);
  double scale = block_sum(sc, sh);
  if (threadIdx.x == 0 && fabs(s) > 1e-9 * scale) {
    S->error = CFDG_E031;
    S->done = 2;
  }
}

// IC(0) forward substitution over one dependency level (pressure.rs:225-232).
__global__ void k_ic0_fwd(const int* __restrict__ order, int begin, int end, const int* __restrict__ off,
                          const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ diag,
                          const double* __restrict__ r, double* __restrict__ z, const Scalars* S) {
  if (S && S->done) return;
  int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int i = order[t];
  double v = r[i];
  for (int k = off[i]; k < off[i + 1]; ++k) v = v - val[k] * z[col[k]];
  z[i] = v / diag[i];
}

// IC(0) backward substitution as a gather over one level (pressure.rs:233-240):
// z_c = (y_c - sum over rows i > c, descending, of l_ic z_i) / d_c.
__global__ void k_ic0_bwd(const int* __restrict__ order, int begin, int end, const int* __restrict__ off,
                          const int* __restrict__ row, const double* __restrict__ val, const double* __restrict__ diag,
                          double* __restrict__ z, const Scalars* S) {
  if (S && S->done) return;
  int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  int c = order[t];
  double v = z[c];
  for (int k = off[c]; k < off[c + 1]; ++k) v = v - val[k] * z[row[k]];
  z[c] = v / diag[c];
}

// Row bodies shared by the level-by-level kernels and the cooperative coarse kernel
// (same operations, same order; L2 loads for vectors another block may have written).
__device__ __forceinline__ void gs_row(int i, const int* __restrict__ off, const int* __restrict__ col,
                                       const double* __restrict__ val, const double* __restrict__ diag,
                                       const double* rhs, double* x) {
  const double d = diag[i];
  if (d == 0.0) {  // an isolated sealed cell: a null pressure space
    x[i] = 0.0;
    return;
  }
  double v = __ldcg(&rhs[i]);
  for (int k = off[i]; k < off[i + 1]; ++k) v = v - val[k] * __ldcg(&x[col[k]]);
  x[i] = v / d;
}
__device__ __forceinline__ void residual_row(int i, const int* __restrict__ off, const int* __restrict__ col,
                                             const double* __restrict__ val, const double* __restrict__ diag,
                                             const double* rhs, const double* x, double* res) {
  double v = diag[i] * __ldcg(&x[i]);
  for (int k = off[i]; k < off[i + 1]; ++k) v = v + val[k] * __ldcg(&x[col[k]]);
  res[i] = __ldcg(&rhs[i]) - v;
}
__device__ __forceinline__ void restrict_row(int j, const int* __restrict__ off, const int* __restrict__ child,
                                             const double* __restrict__ w, const double* res, double* rhs_c) {
  double v = 0.0;
  for (int k = off[j]; k < off[j + 1]; ++k) v = v + w[k] * __ldcg(&res[child[k]]);
  rhs_c[j] = v;
}
__device__ __forceinline__ void prolong_row(int i, const int* __restrict__ off, const int* __restrict__ col,
                                            const double* __restrict__ w, const double* xc, double* x) {
  double s = -0.0;
  for (int k = off[i]; k < off[i + 1]; ++k) s = s + w[k] * __ldcg(&xc[col[k]]);
  x[i] = __ldcg(&x[i]) + s;
}
// Dense Cholesky solve of one terminal block by one thread (masked.rs:52-69).
__device__ __forceinline__ void direct_block(int bk, const int* __restrict__ ioff, const int* __restrict__ idx,
                                             const long long* __restrict__ foff, const double* __restrict__ L,
                                             const double* rhs, double* x) {
  const int* ix = idx + ioff[bk];
  const int n = ioff[bk + 1] - ioff[bk];
  const double* f = L + foff[bk];
  for (int i = 0; i < n; ++i) {
    double v = __ldcg(&rhs[ix[i]]);
    for (int j = 0; j < i; ++j) v = v - f[i * n + j] * __ldcg(&x[ix[j]]);
    x[ix[i]] = v / f[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double v = __ldcg(&x[ix[i]]);
    for (int j = i + 1; j < n; ++j) v = v - f[j * n + i] * __ldcg(&x[ix[j]]);
    x[ix[i]] = v / f[i * n + i];
  }
}
// Gauge of group g by one block: subtract the members' mean (fixed-order tree sum).
__device__ __forceinline__ void center_group(int g, const int* __restrict__ off, const int* __restrict__ members,
                                             double* x, double* sh, double* mean) {
  const int b = off[g], e = off[g + 1];
  double acc = 0.0;
  for (int k = b + threadIdx.x; k < e; k += blockDim.x) acc += __ldcg(&x[members[k]]);
  double s = block_sum(acc, sh);
  if (threadIdx.x == 0) *mean = s / (double)(e - b);
  __syncthreads();
  const double m = *mean;
  for (int k = b + threadIdx.x; k < e; k += blockDim.x) x[members[k]] = __ldcg(&x[members[k]]) - m;
  __syncthreads();
}

// Lexicographic Gauss-Seidel over one level (multigrid.rs:272-281, masked.rs:158-172).
__global__ void k_gs(const int* __restrict__ order, int begin, int end, const int* __restrict__ off,
                     const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ diag,
                     const double* __restrict__ rhs, double* __restrict__ x, const Scalars* S) {
  if (S && S->done) return;
  int t = begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= end) return;
  gs_row(order[t], off, col, val, diag, rhs, x);
}

// res = rhs - A x (multigrid.rs:263-271 then :691-694).
__global__ void k_residual(int n, const int* __restrict__ off, const int* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ diag,
                           const double* __restrict__ rhs, const double* __restrict__ x, double* __restrict__ res,
                           const Scalars* S) {
  if (S && S->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = diag[i] * x[i];
    for (int k = off[i]; k < off[i + 1]; ++k) v = v + val[k] * x[col[k]];
    res[i] = rhs[i] - v;
  }
}

// Level-0 residual on the structured grid: res = rhs - (diag x + sum over the row's
// faces in order x-lo, x-hi, y-lo, y-hi, z-lo, z-hi of (-w) x_nbr) (multigrid.rs:263-271).
template <bool UNIFORM>
__global__ void k_residual_struct(GridDev g, const double* __restrict__ diag, const double* __restrict__ rhs,
                                  const double* __restrict__ x, double* __restrict__ res, int N, const Scalars* S) {
  if (S && S->done) return;
  const int stride[3] = {1, g.n[0], g.n[0] * g.n[1]};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    const unsigned fl = g.flags[c];
    double v = diag[c] * x[c];
    if (fl & 0x3fu) {
      int q[3];
      cell_coords(g, c, q[0], q[1], q[2]);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int side = 0; side < 2; ++side) {
          if (!(fl & (1u << (2 * a + side)))) continue;
          double w;
          if (UNIFORM) {
            w = g.w_in[a];
          } else {
            int p[3] = {q[0], q[1], q[2]};
            p[a] += side;
            w = g.fw[face_index(g, a, p[0], p[1], p[2])];
          }
          v = v - w * x[side ? c + stride[a] : c - stride[a]];
        }
    }
    res[c] = rhs[c] - v;
  }
}

// Coarse rhs = P^T res, per coarse row over its children in ascending order
// (multigrid.rs:696-701, masked.rs:325-328).
__global__ void k_restrict(int nc, const int* __restrict__ off, const int* __restrict__ child,
                           const double* __restrict__ w, const double* __restrict__ res, double* __restrict__ rhs_c,
                           const Scalars* S) {
  if (S && S->done) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nc; j += gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int k = off[j]; k < off[j + 1]; ++k) v = v + w[k] * res[child[k]];
    rhs_c[j] = v;
  }
}

// x += P x_c (multigrid.rs:703-709, masked.rs:330-332).
__global__ void k_prolong(int n, const int* __restrict__ off, const int* __restrict__ col,
                          const double* __restrict__ w, const double* __restrict__ xc, double* __restrict__ x,
                          const Scalars* S) {
  if (S && S->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = -0.0;
    for (int k = off[i]; k < off[i + 1]; ++k) s = s + w[k] * xc[col[k]];
    x[i] = x[i] + s;
  }
}

// Dense Cholesky solves of the terminal level, one thread per block (masked.rs:52-69).
__global__ void k_direct(int nblocks, const int* __restrict__ ioff, const int* __restrict__ idx,
                         const long long* __restrict__ foff, const double* __restrict__ L,
                         const double* __restrict__ rhs, double* __restrict__ x, const Scalars* S) {
  if (S && S->done) return;
  int bk = blockIdx.x * blockDim.x + threadIdx.x;
  if (bk >= nblocks) return;
  const int* ix = idx + ioff[bk];
  const int n = ioff[bk + 1] - ioff[bk];
  const double* f = L + foff[bk];
  for (int i = 0; i < n; ++i) {
    double v = rhs[ix[i]];
    for (int j = 0; j < i; ++j) v = v - f[i * n + j] * x[ix[j]];
    x[ix[i]] = v / f[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double v = x[ix[i]];
    for (int j = i + 1; j < n; ++j) v = v - f[j * n + i] * x[ix[j]];
    x[ix[i]] = v / f[i * n + i];
  }
}

// ----------------------------------------------------------------- coarse levels, one launch
// Levels 1 .. L-1 of the V-cycle in one cooperative kernel: each dependency level of a
// lexicographic sweep, the residual, the restriction, the prolongation and the gauges is
// a phase separated by a grid barrier (level-by-level launches cost a launch each: about
// 1,300 per cycle on a 128x128x64 grid). Levels whose dependency levels have at most one
// block of rows sweep inside block 0 with block barriers. Every row runs the row body of
// the level-by-level kernels, so the bits are the same.
struct PLev {
  int n, terminal, ngroups, nblocks;
  int nfwd, nbwd, blocal, pad_;
  const int *off, *col;
  const double *val, *diag;
  const int *fo, *fs, *bo, *bs;  // sweep orders and dependency-level starts
  const int *goff, *gmem;
  const int *roff, *rcol;        // restriction to the next level (rows of the next level)
  const double* rval;
  const int *poff, *pcol;        // prolongation from the next level
  const double* pval;
  double *rhs, *x, *res;
  const int *ioff, *idx;
  const long long* foff;
  const double* fac;
  // Sweeps each way (2, or 1 with block smoothing) and the block smoother, if any.
  int nsweep, lines, llen, lbw;
  int lnfwd, lnbwd, lblocal, pad2_;
  const int *lnodes, *looff, *locol;
  const double *loval, *lfac;
  double* lscr;
  const int *lfo, *lfs, *lbo, *lbs;
};

namespace cg = cooperative_groups;

// The barrier between the phases of the coarse-level kernel: the whole grid of a cooperative
// launch, or the one thread-block cluster the launch consists of (gridDim.x = cluster size,
// so blockIdx.x is the block's rank in the cluster). Clusters are scheduled as a unit, so
// launches on several streams at once never wait on blocks that are not resident.
struct GridBarrier {
  cg::grid_group g;
  __device__ void sync() { g.sync(); }
};
struct ClusterBarrier {
  __device__ void sync() { cg::this_cluster().sync(); }
};
constexpr int PC_CLUSTER = 8;  // blocks of the plain coarse-level cluster (portable size)

// The banded forward and backward substitutions of one block (multigrid/line.rs:172-185)
// for a half-bandwidth BW: the last BW results stay in registers and the factor entries of
// a row are independent of the chain, so only the multiply-subtract chain is serial. The
// operations and their order are the reference's (bit-identical).
template <int BW>
__device__ __forceinline__ void line_subst(double* s, const double* __restrict__ fac, long long base, int len) {
  constexpr int stride = BW + 1;
  double w[BW + 1];  // w[d]: the result d rows back (forward) or ahead (backward)
#pragma unroll
  for (int d = 0; d <= BW; ++d) w[d] = 0.0;
  for (int i = 0; i < len; ++i) {
    const double* f = fac + base + (long long)i * stride;
    double v = s[i];
#pragma unroll
    for (int d = BW; d >= 1; --d)  // columns i-BW .. i-1, ascending
      if (i - d >= 0) v = v - f[d] * w[d];
    v = v * f[0];
    s[i] = v;
#pragma unroll
    for (int d = BW; d >= 2; --d) w[d] = w[d - 1];
    w[1] = v;
  }
#pragma unroll
  for (int d = 0; d <= BW; ++d) w[d] = 0.0;
  for (int i = len - 1; i >= 0; --i) {
    double v = s[i];
#pragma unroll
    for (int d = 1; d <= BW; ++d)  // columns i+1 .. i+BW, ascending
      if (i + d < len) v = v - fac[base + (long long)(i + d) * stride + d] * w[d];
    v = v * fac[base + (long long)i * stride];
    s[i] = v;
#pragma unroll
    for (int d = BW; d >= 2; --d) w[d] = w[d - 1];
    w[1] = v;
  }
}

// Any half-bandwidth, as line.rs:172-185 writes it.
__device__ __noinline__ void line_subst_any(double* s, const double* __restrict__ fac, long long base, int len, int bw) {
  const long long stride = bw + 1;
  for (int i = 0; i < len; ++i) {
    const long long row = base + i * stride;
    double v = s[i];
    for (int j = max(0, i - bw); j < i; ++j) v = v - fac[row + i - j] * s[j];
    s[i] = v * fac[row];
  }
  for (int i = len - 1; i >= 0; --i) {
    double v = s[i];
    for (int j = i + 1; j < min(len, i + bw + 1); ++j) v = v - fac[base + j * stride + j - i] * s[j];
    s[i] = v * fac[base + i * stride];
  }
}

constexpr int LSCR = 256;  // block lengths up to this keep their scratch in shared memory

// multigrid/line.rs:155-190, one block, by one warp: the lanes gather the right-hand side
// less the outside entries for the block's nodes (each node's entries in the reference's
// order), lane 0 runs the substitutions, the lanes write the block's values to x.
// Bit-identical to the sequential sweep. x and rhs come through L2 (other blocks of the
// launch write them); the scratch is the warp's shared row or the block's global slice.
__device__ __forceinline__ void line_block(int b, const PLev& L, const double* rhs, double* x, int lane,
                                           double* wsh) {
  const int len = L.llen, bw = L.lbw;
  const int start = b * len;
  const long long base = (long long)start * (bw + 1);
  double* scr = len <= LSCR ? wsh : L.lscr + start;
  for (int i = lane; i < len; i += 32) {
    double v = __ldcg(&rhs[L.lnodes[start + i]]);
    for (int e = L.looff[start + i]; e < L.looff[start + i + 1]; ++e) v = v - L.loval[e] * __ldcg(&x[L.locol[e]]);
    scr[i] = v;
  }
  __syncwarp();
  if (lane == 0) {
    switch (bw) {
      case 1: line_subst<1>(scr, L.lfac, base, len); break;
      case 2: line_subst<2>(scr, L.lfac, base, len); break;
      case 3: line_subst<3>(scr, L.lfac, base, len); break;
      case 4: line_subst<4>(scr, L.lfac, base, len); break;
      default: line_subst_any(scr, L.lfac, base, len, bw); break;
    }
  }
  __syncwarp();
  for (int i = lane; i < len; i += 32) x[L.lnodes[start + i]] = scr[i];
  __syncwarp();  // the row is reused by the warp's next block
}

template <class Bar>
__device__ void pc_center(const PLev& L, double* v, double* sh, double* mean, Bar& grid) {
  if (L.ngroups == 0) return;
  for (int g = blockIdx.x; g < L.ngroups; g += gridDim.x) center_group(g, L.goff, L.gmem, v, sh, mean);
  __threadfence();
  grid.sync();
}

// A block Gauss-Seidel sweep over the block dependency levels (blocks of one level share
// no entry, so they run in parallel; the reference's block order is kept where it matters).
template <class Bar>
__device__ void pc_lines(const PLev& L, bool backward, Bar& grid, double* lsh) {
  const int* order = backward ? L.lbo : L.lfo;
  const int* start = backward ? L.lbs : L.lfs;
  const int nlev = backward ? L.lnbwd : L.lnfwd;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double* wsh = lsh + warp * LSCR;
  if (L.lblocal) {
    if (blockIdx.x == 0)
      for (int dl = 0; dl < nlev; ++dl) {
        for (int t = start[dl] + warp; t < start[dl + 1]; t += wpb) line_block(order[t], L, L.rhs, L.x, lane, wsh);
        __threadfence();
        __syncthreads();
      }
    __threadfence();
    grid.sync();
    return;
  }
  const int gw = blockIdx.x * wpb + warp, nw = gridDim.x * wpb;
  for (int dl = 0; dl < nlev; ++dl) {
    for (int t = start[dl] + gw; t < start[dl + 1]; t += nw) line_block(order[t], L, L.rhs, L.x, lane, wsh);
    __threadfence();
    grid.sync();
  }
}

template <class Bar>
__device__ void pc_sweep(const PLev& L, bool backward, Bar& grid, double* lsh) {
  if (L.lines) {
    pc_lines(L, backward, grid, lsh);
    return;
  }
  const int* order = backward ? L.bo : L.fo;
  const int* start = backward ? L.bs : L.fs;
  const int nlev = backward ? L.nbwd : L.nfwd;
  if (L.blocal) {
    if (blockIdx.x == 0)
      for (int dl = 0; dl < nlev; ++dl) {
        for (int t = start[dl] + threadIdx.x; t < start[dl + 1]; t += blockDim.x)
          gs_row(order[t], L.off, L.col, L.val, L.diag, L.rhs, L.x);
        __threadfence();
        __syncthreads();
      }
    __threadfence();
    grid.sync();
    return;
  }
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int dl = 0; dl < nlev; ++dl) {
    for (int t = start[dl] + gt; t < start[dl + 1]; t += nth) gs_row(order[t], L.off, L.col, L.val, L.diag, L.rhs, L.x);
    __threadfence();
    grid.sync();
  }
}

template <class Bar>
__device__ void plain_coarse(const PLev* lv, int nl, const Scalars* S, Bar& grid) {
  if (S && S->done) return;  // read once; nothing in this kernel changes it
  __shared__ double sh[32];
  __shared__ double mean;
  __shared__ double lsh[(BLOCK / 32) * LSCR];  // one scratch row per warp (block smoothers)
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  int l = 0;
  for (; l < nl; ++l) {
    const PLev& L = lv[l];
    pc_center(L, L.rhs, sh, &mean, grid);
    for (int i = gt; i < L.n; i += nth) L.x[i] = 0.0;
    __threadfence();
    grid.sync();
    if (L.terminal) {
      for (int bk = gt; bk < L.nblocks; bk += nth) direct_block(bk, L.ioff, L.idx, L.foff, L.fac, L.rhs, L.x);
      __threadfence();
      grid.sync();
      pc_center(L, L.x, sh, &mean, grid);
      break;
    }
    for (int sw = 0; sw < L.nsweep; ++sw) pc_sweep(L, false, grid, lsh);
    pc_center(L, L.x, sh, &mean, grid);
    for (int i = gt; i < L.n; i += nth) residual_row(i, L.off, L.col, L.val, L.diag, L.rhs, L.x, L.res);
    __threadfence();
    grid.sync();
    pc_center(L, L.res, sh, &mean, grid);
    const PLev& N = lv[l + 1];
    for (int j = gt; j < N.n; j += nth) restrict_row(j, L.roff, L.rcol, L.rval, L.res, N.rhs);
    __threadfence();
    grid.sync();
  }
  for (int m = min(l, nl - 1) - 1; m >= 0; --m) {
    const PLev& L = lv[m];
    const PLev& N = lv[m + 1];
    for (int i = gt; i < L.n; i += nth) prolong_row(i, L.poff, L.pcol, L.pval, N.x, L.x);
    __threadfence();
    grid.sync();
    for (int sw = 0; sw < L.nsweep; ++sw) pc_sweep(L, true, grid, lsh);
    pc_center(L, L.x, sh, &mean, grid);
  }
}

__global__ void __launch_bounds__(BLOCK) k_plain_coarse(const PLev* lv, int nl, const Scalars* S) {
  GridBarrier bar{cg::this_grid()};
  plain_coarse(lv, nl, S, bar);
}
__global__ void __launch_bounds__(BLOCK) k_plain_coarse_cluster(const PLev* lv, int nl, const Scalars* S) {
  ClusterBarrier bar;
  plain_coarse(lv, nl, S, bar);
}

__global__ void k_gather(int n, const int* __restrict__ idx, const double* __restrict__ src, double* __restrict__ dst,
                         const Scalars* S) {
  if (S && S->done) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) dst[j] = src[idx[j]];
}
__global__ void k_scatter(int n, const int* __restrict__ idx, const double* __restrict__ src, double* __restrict__ dst,
                          const Scalars* S) {
  if (S && S->done) return;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) dst[idx[j]] = src[j];
}

// 1/y when y is a positive power of two whose reciprocal is a normal number, else 0. A
// product with it is the quotient by y bit for bit (the same real value, rounded the same
// way); FP64 division is ~20x dearer than a product on this part.
__device__ __forceinline__ double exact_recip(double y) {
  const long long bits = __double_as_longlong(y);
  const int e = (int)((bits >> 52) & 0x7ff);
  if ((bits & (long long)0x800fffffffffffffull) != 0 || e < 1 || e > 2045) return 0.0;
  return __longlong_as_double((long long)(2046 - e) << 52);
}
__device__ __forceinline__ double div_exact(double x, double y) {
  const double r = exact_recip(y);
  return r != 0.0 ? x * r : x / y;
}

// projection_rhs (pressure.rs:440-459): b = -div(u)/dt, terms = sum(|u_lo|+|u_hi|)/dx/dt.
__global__ void k_projection_rhs(GridDev g, const uint8_t* __restrict__ fluid, const double* __restrict__ u, double dt,
                                 double* __restrict__ b, double* __restrict__ terms, int N) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    if (!fluid[c]) {
      b[c] = -0.0;
      terms[c] = 0.0;
      continue;
    }
    int q[3];
    cell_coords(g, c, q[0], q[1], q[2]);
    double div = 0.0, scale = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      int p[3] = {q[0], q[1], q[2]};
      long long fl = face_index(g, a, p[0], p[1], p[2]);
      p[a] = (g.per[a] && q[a] == g.n[a] - 1) ? 0 : q[a] + 1;
      long long fu = face_index(g, a, p[0], p[1], p[2]);
      double ul = u[fl], uu = u[fu];
      div = div + div_exact(uu - ul, g.dx[a]);
      scale = scale + div_exact(fabs(ul) + fabs(uu), g.dx[a]);
    }
    b[c] = -div / dt;
    terms[c] = scale / dt;
  }
}

// u -= dt grad(phi) on interior and outlet faces (pressure.rs:481-496).
__global__ void k_correct_faces(const uint8_t* __restrict__ kind, const int* __restrict__ lo,
                                const int* __restrict__ hi, const double* __restrict__ dist,
                                const double* __restrict__ phi, double dt, double* __restrict__ u, long long F,
                                const Scalars* S) {
  if (S->done != 1 && S->done != 4) return;
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < F; f += (long long)gridDim.x * blockDim.x) {
    double d;
    uint8_t k = kind[f];
    if (k == INTERIOR) d = div_exact(phi[hi[f]] - phi[lo[f]], dist[f]);
    else if (k == OUTLET) d = lo[f] >= 0 ? div_exact(-phi[lo[f]], dist[f]) : div_exact(phi[hi[f]], dist[f]);
    else d = 0.0;
    u[f] = u[f] - dt * d;
  }
}

__global__ void k_add(double* __restrict__ p, const double* __restrict__ q, int N, const Scalars* S) {
  if (S->done != 1 && S->done != 4) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) p[i] = p[i] + q[i];
}

__global__ void k_weights(const double* __restrict__ area, const double* __restrict__ dist, double volume,
                          double* __restrict__ w, long long F) {
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < F; f += (long long)gridDim.x * blockDim.x)
    w[f] = area[f] / (dist[f] * volume);
}

}  // namespace

// ============================================================== host side

namespace cfdg {
thread_local std::string t_error;
std::atomic<uint64_t> g_launches{0};
}  // namespace cfdg

#include "state.hpp"

namespace {

constexpr int CHUNK = 8;

void reset_chunk(cfdg_grid* G) {
  if (G->chunk) cudaGraphExecDestroy(G->chunk);
  G->chunk = nullptr;
  G->chunk_kind = -1;
}

inline void tick(cfdg_grid* G) {
  if (!G->capturing) count();
}

int launch_center(cfdg_grid* G, const DevCsr& groups, int ngroups, double* x, const Scalars* S) {
  if (ngroups == 0) return 0;
  k_center<<<ngroups, BLOCK, 0, G->stream>>>(groups.off, groups.col, x, S); tick(G);
  return 0;
}

WaveArgs wave_args(cfdg_grid* G, const Scalars* S) {
  WaveArgs A{};
  for (int a = 0; a < 3; ++a) {
    A.n[a] = G->h.n[a];
    A.w_in[a] = G->g.w_in[a];
    A.face_off[a] = G->g.face_off[a];
    for (int d = 0; d < 3; ++d) A.fdim[a][d] = G->g.fdim[a][d];
  }
  A.tiles_j = G->tiles_j;
  A.tiles_k = G->tiles_k;
  A.flags = G->d_flags;
  A.uniform = G->uniform ? 1 : 0;
  A.fw = G->d_fw;
  A.sync = G->wave_sync;
  A.error = G->wave_err;
  A.S = S;
  A.spin_limit = G->wave_spin_limit;
  A.hold_tile = G->wave_hold_tile;
  return A;
}

template <int MODE>
void launch_wave(cfdg_grid* G, const WaveArgs& A) {
  cudaMemsetAsync(G->wave_sync, 0, sizeof(int) * (2 + G->tiles_j * G->tiles_k), G->stream);
  k_wave<MODE><<<G->tiles_j * G->tiles_k, WTJ * WTK, 0, G->stream>>>(A);
  tick(G);
}

void launch_sweep_ic0(cfdg_grid* G, const Scalars* S) {
  DevIc0& F = *G->ic0;
  if (G->structured) {
    WaveArgs A = wave_args(G, S);
    A.diag = F.diag;
    A.lx = F.lx;
    A.ly = F.ly;
    A.lz = F.lz;
    A.in = G->r;
    A.x = G->z;
    launch_wave<IC0_FWD>(G, A);
    launch_wave<IC0_BWD>(G, A);
    return;
  }
  for (size_t l = 0; l + 1 < F.fwd.start.size(); ++l) {
    int b = F.fwd.start[l], e = F.fwd.start[l + 1];
    k_ic0_fwd<<<(e - b + BLOCK - 1) / BLOCK, BLOCK, 0, G->stream>>>(F.fwd.order, b, e, F.lower.off, F.lower.col,
                                                                     F.lower.val, F.diag, G->r, G->z, S); tick(G);
  }
  for (size_t l = 0; l + 1 < F.bwd.start.size(); ++l) {
    int b = F.bwd.start[l], e = F.bwd.start[l + 1];
    k_ic0_bwd<<<(e - b + BLOCK - 1) / BLOCK, BLOCK, 0, G->stream>>>(F.bwd.order, b, e, F.upper.off, F.upper.col,
                                                                     F.upper.val, F.diag, G->z, S); tick(G);
  }
}

void launch_gs(cfdg_grid* G, DevLevel& L, bool backward, const Scalars* S, bool full = false) {
  if (full) {
    WaveArgs A = wave_args(G, S);
    A.diag = L.diag;
    A.in = L.rhs;
    A.x = L.x;
    if (backward) launch_wave<GS_BWD>(G, A);
    else launch_wave<GS_FWD>(G, A);
    return;
  }
  const DevSchedule& sc = backward ? L.bwd : L.fwd;
  for (size_t l = 0; l + 1 < sc.start.size(); ++l) {
    int b = sc.start[l], e = sc.start[l + 1];
    k_gs<<<(e - b + BLOCK - 1) / BLOCK, BLOCK, 0, G->stream>>>(sc.order, b, e, L.a.off, L.a.col, L.a.val, L.diag,
                                                                L.rhs, L.x, S); tick(G);
  }
}

// One symmetric V(2,2) cycle, z = M^-1 r (multigrid.rs:656-726, masked.rs:292-342).
void launch_vcycle(cfdg_grid* G, const double* r, double* z, const Scalars* S) {
  DevHierarchy& H = *G->mg;
  cudaStream_t s = G->stream;
  const int N = (int)G->h.cells;
  DevLevel& L0 = H.levels[0];
  if (H.masked && !H.full0) {
    k_gather<<<grid_blocks(H.nfluid), BLOCK, 0, s>>>(H.nfluid, H.fluid_idx, r, L0.rhs, S);
    tick(G);
  } else {
    k_copy<<<grid_blocks(N), BLOCK, 0, s>>>(L0.rhs, r, N, S);
    tick(G);
  }
  const int nl = (int)H.levels.size();
  // Levels 1 .. L-1 in one cooperative launch when available, else level by level.
  const bool coop = (H.coop_blocks > 0 || H.cluster) && nl > 1;
  const int first = H.coop0 ? 0 : 1;  // the first level of the cooperative launch
  for (int l = 0; l < (coop ? first : nl); ++l) {
    DevLevel& L = H.levels[l];
    const bool full = l == 0 && H.full0;
    launch_center(G, L.groups, L.ngroups, L.rhs, S);
    k_fill<<<grid_blocks(L.n), BLOCK, 0, s>>>(L.x, 0.0, L.n, S); tick(G);
    if (L.terminal) {
      if (L.nblocks > 0) {
        k_direct<<<(L.nblocks + 63) / 64, 64, 0, s>>>(L.nblocks, L.d_ioff, L.d_idx, L.d_foff, L.d_fac, L.rhs, L.x, S); tick(G);
      }
      launch_center(G, L.groups, L.ngroups, L.x, S);
      break;
    }
    launch_gs(G, L, false, S, full);
    launch_gs(G, L, false, S, full);
    launch_center(G, L.groups, L.ngroups, L.x, S);
    if (full) {
      if (G->uniform) k_residual_struct<true><<<grid_blocks(L.n), BLOCK, 0, s>>>(G->g, L.diag, L.rhs, L.x, L.res, L.n, S);
      else k_residual_struct<false><<<grid_blocks(L.n), BLOCK, 0, s>>>(G->g, L.diag, L.rhs, L.x, L.res, L.n, S);
      tick(G);
    } else {
      k_residual<<<grid_blocks(L.n), BLOCK, 0, s>>>(L.n, L.a.off, L.a.col, L.a.val, L.diag, L.rhs, L.x, L.res, S); tick(G);
    }
    launch_center(G, L.groups, L.ngroups, L.res, S);
    DevLevel& C = H.levels[l + 1];
    k_restrict<<<grid_blocks(C.n), BLOCK, 0, s>>>(C.n, L.restrict_.off, L.restrict_.col, L.restrict_.val, L.res,
                                                  C.rhs, S); tick(G);
  }
  if (coop) {
    // One cluster of PC_CLUSTER blocks (cluster barriers, about 0.3 us a phase), or the
    // cooperative grid where clusters cannot be launched.
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(BLOCK, 1, 1);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    if (H.cluster) {
      cfg.gridDim = dim3(PC_CLUSTER, 1, 1);
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = PC_CLUSTER;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, k_plain_coarse_cluster, (const PLev*)H.d_plev, nl - first, S);
    } else {
      cfg.gridDim = dim3((unsigned)H.coop_blocks, 1, 1);
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      cudaLaunchKernelEx(&cfg, k_plain_coarse, (const PLev*)H.d_plev, nl - first, S);
    }
    tick(G);
  }
  for (int l = coop ? first - 1 : nl - 2; l >= 0; --l) {
    DevLevel& L = H.levels[l];
    DevLevel& C = H.levels[l + 1];
    const bool full = l == 0 && H.full0;
    k_prolong<<<grid_blocks(L.n), BLOCK, 0, s>>>(L.n, L.prolong.off, L.prolong.col, L.prolong.val, C.x, L.x, S); tick(G);
    launch_gs(G, L, true, S, full);
    launch_gs(G, L, true, S, full);
    launch_center(G, L.groups, L.ngroups, L.x, S);
  }
  if (H.masked && !H.full0) {
    k_fill<<<grid_blocks(N), BLOCK, 0, s>>>(z, 0.0, N, S); tick(G);
    k_scatter<<<grid_blocks(H.nfluid), BLOCK, 0, s>>>(H.nfluid, H.fluid_idx, L0.x, z, S); tick(G);
  } else {
    k_copy<<<grid_blocks(N), BLOCK, 0, s>>>(z, L0.x, N, S); tick(G);
  }
}

// z = M^-1 r with the grid's preconditioner, then the gauge.
void launch_precondition(cfdg_grid* G, const Scalars* S) {
  if (G->preconditioner == CFDG_PRECOND_MULTIGRID) launch_vcycle(G, G->r, G->z, S);
  else launch_sweep_ic0(G, S);
  launch_center(G, G->comp_groups, G->ncomp_groups, G->z, S);
}

template <bool U>
void launch_iteration_t(cfdg_grid* G) {
  const int N = (int)G->h.cells;
  const int nb = grid_blocks(N);
  cudaStream_t s = G->stream;
  k_pcg_op<U><<<nb, BLOCK, 0, s>>>(G->g, G->p, G->ap, N, G->partials, G->S); tick(G);
  k_pcg_xr<<<nb, BLOCK, 0, s>>>(G->x, G->r, G->p, G->ap, N, G->partials, G->S); tick(G);
  k_pcg_true<U><<<nb, BLOCK, 0, s>>>(G->g, G->x, G->bc, N, G->partials, G->S); tick(G);
  launch_precondition(G, G->S);
  k_pcg_rz<<<nb, BLOCK, 0, s>>>(G->r, G->z, N, G->partials, G->S, 0); tick(G);
  k_pcg_p<<<nb, BLOCK, 0, s>>>(G->p, G->z, N, G->S); tick(G);
}
void launch_iteration(cfdg_grid* G) {
  if (G->uniform) launch_iteration_t<true>(G);
  else launch_iteration_t<false>(G);
}

template <bool U>
void launch_apply_t(cfdg_grid* G, const double* x, double* y) {
  const int N = (int)G->h.cells;
  k_apply<U><<<grid_blocks(N), BLOCK, 0, G->stream>>>(G->g, x, y, N); tick(G);
}
void launch_apply(cfdg_grid* G, const double* x, double* y) {
  if (G->uniform) launch_apply_t<true>(G, x, y);
  else launch_apply_t<false>(G, x, y);
}

// Recomputes face weights on the device and decides the uniform fast path.
int refresh_weights(cfdg_grid* G) {
  HostGrid& h = G->h;
  CU(cudaMemcpyAsync(G->d_area, h.face_area.data(), h.faces * 8, cudaMemcpyHostToDevice, G->stream));
  CU(cudaMemcpyAsync(G->d_dist, h.face_distance.data(), h.faces * 8, cudaMemcpyHostToDevice, G->stream));
  k_weights<<<grid_blocks(h.faces), BLOCK, 0, G->stream>>>(G->d_area, G->d_dist, h.volume, G->d_fw, h.faces); tick(G);
  bool uniform = true;
  uint64_t win[3] = {0, 0, 0}, wout[3] = {0, 0, 0};
  bool hin[3] = {false, false, false}, hout[3] = {false, false, false};
  for (int a = 0; a < 3 && uniform; ++a)
    for (int64_t f = h.face_offset[a]; f < h.face_offset[a] + h.face_dims[a][0] * h.face_dims[a][1] * h.face_dims[a][2];
         ++f) {
      uint8_t k = h.face_kind[f];
      if (k != INTERIOR && k != OUTLET) continue;
      double w = h.weight(f);
      uint64_t bits;
      std::memcpy(&bits, &w, 8);
      uint64_t* slot = k == INTERIOR ? &win[a] : &wout[a];
      bool* has = k == INTERIOR ? &hin[a] : &hout[a];
      if (!*has) {
        *slot = bits;
        *has = true;
      } else if (*slot != bits) {
        uniform = false;
        break;
      }
    }
  G->uniform = uniform;
  for (int a = 0; a < 3; ++a) {
    std::memcpy(&G->g.w_in[a], &win[a], 8);
    std::memcpy(&G->g.w_out[a], &wout[a], 8);
  }
  // Scalar transport: area and distance of the transporting faces per axis and kind.
  bool sc_uniform = true;
  uint64_t sa[3][3] = {}, sd[3][3] = {};
  bool sh[3][3] = {};
  for (int a = 0; a < 3 && sc_uniform; ++a)
    for (int64_t f = h.face_offset[a]; f < h.face_offset[a] + h.face_dims[a][0] * h.face_dims[a][1] * h.face_dims[a][2];
         ++f) {
      const uint8_t k = h.face_kind[f];
      if (k != INTERIOR && k != INLET && k != OUTLET) continue;
      const int t = k == INTERIOR ? 0 : (k == INLET ? 1 : 2);
      uint64_t ab, db;
      std::memcpy(&ab, &h.face_area[f], 8);
      std::memcpy(&db, &h.face_distance[f], 8);
      if (!sh[a][t]) {
        sa[a][t] = ab;
        sd[a][t] = db;
        sh[a][t] = true;
      } else if (sa[a][t] != ab || sd[a][t] != db) {
        sc_uniform = false;
        break;
      }
    }
  G->sc_uniform = sc_uniform;
  for (int a = 0; a < 3; ++a)
    for (int t = 0; t < 3; ++t) {
      G->sc_used[a][t] = sh[a][t];
      std::memcpy(&G->sc_area[a][t], &sa[a][t], 8);
      std::memcpy(&G->sc_dist[a][t], &sd[a][t], 8);
    }
  CU(cudaGetLastError());
  return 0;
}

int build_ic0_dev(cfdg_grid* G) {
  Ic0 F;
  build_ic0(G->h, F);
  auto D = std::make_unique<DevIc0>();
  D->arena.ctx = G->ctx;
  cudaStream_t s = G->stream;
  if (int e = upload_csr(D->arena, F.lower, D->lower, s)) return e;
  if (int e = upload_csr(D->arena, F.upper, D->upper, s)) return e;
  if (int e = D->arena.upload(&D->diag, F.diag, s)) return e;
  if (int e = D->arena.upload(&D->fwd.order, F.fwd.order, s)) return e;
  if (int e = D->arena.upload(&D->bwd.order, F.bwd.order, s)) return e;
  D->fwd.start = F.fwd.start;
  D->bwd.start = F.bwd.start;
  if (G->structured) {
    // Each row's lower entries are its (k-1), (j-1), (i-1) neighbours (non-periodic 7-point).
    const int64_t N = G->h.cells, nx = G->h.n[0], nxy = (int64_t)G->h.n[0] * G->h.n[1];
    std::vector<double> lx(N, 0.0), ly(N, 0.0), lz(N, 0.0);
    for (int64_t r = 0; r < N; ++r)
      for (int32_t k = F.lower.off[r]; k < F.lower.off[r + 1]; ++k) {
        int64_t c = F.lower.col[k];
        if (c == r - 1) lx[r] = F.lower.val[k];
        else if (c == r - nx) ly[r] = F.lower.val[k];
        else if (c == r - nxy) lz[r] = F.lower.val[k];
        else return fail(CFDG_ERR_INVALID, "IC(0) factor is not a 7-point lower pattern");
      }
    if (int e = D->arena.upload(&D->lx, lx, s)) return e;
    if (int e = D->arena.upload(&D->ly, ly, s)) return e;
    if (int e = D->arena.upload(&D->lz, lz, s)) return e;
  }
  CU(cudaStreamSynchronize(s));
  G->ic0 = std::move(D);
  return 0;
}

// Device bytes of one level's block smoother as uploaded (nodes, outside rows, banded
// factor, scratch, the two dependency orders).
uint64_t line_device_bytes(const LineBlocks& B) {
  return 4 * (B.nodes.size() + B.outside.off.size() + B.outside.col.size() + B.fwd.order.size() +
              B.fwd.start.size() + B.bwd.order.size() + B.bwd.start.size()) +
         8 * (B.outside.val.size() + B.factor.size() + B.nodes.size());
}

// MultigridStats (multigrid.rs:55-72) as JSON, fields in the reference's order; the empty
// level_dimensions and block_smoothers are omitted as serde skips them. allocated_bytes
// counts the device arrays the hierarchy holds (the storage this engine retains).
std::string stats_json_of(const DevHierarchy& D, const Hierarchy& H) {
  std::string s = "{\"level_cells\":[";
  for (size_t i = 0; i < D.level_cells.size(); ++i) s += (i ? "," : "") + std::to_string(D.level_cells[i]);
  s += "]";
  if (!H.level_dims.empty()) {
    s += ",\"level_dimensions\":[";
    for (size_t i = 0; i < H.level_dims.size(); ++i)
      s += std::string(i ? "," : "") + "[" + std::to_string(H.level_dims[i][0]) + "," +
           std::to_string(H.level_dims[i][1]) + "," + std::to_string(H.level_dims[i][2]) + "]";
    s += "]";
  }
  s += ",\"level_nonzeros\":[";
  for (size_t i = 0; i < D.level_nonzeros.size(); ++i) s += (i ? "," : "") + std::to_string(D.level_nonzeros[i]);
  s += "],\"allocated_bytes\":" + std::to_string(D.arena.bytes);
  std::string blocks;
  for (size_t l = 0; l < H.levels.size(); ++l)
    for (const LineBlocks& B : H.levels[l].lines) {
      blocks += std::string(blocks.empty() ? "" : ",") + "{\"level\":" + std::to_string(l) + ",\"axes\":[";
      for (size_t a = 0; a < B.axes.size(); ++a) blocks += (a ? "," : "") + std::to_string(B.axes[a]);
      blocks += "],\"block_unknowns\":" + std::to_string(B.length) + ",\"block_count\":" +
                std::to_string(B.count()) + ",\"half_bandwidth\":" + std::to_string(B.bandwidth) +
                ",\"allocated_bytes\":" + std::to_string(line_device_bytes(B)) + "}";
    }
  if (!blocks.empty()) s += ",\"block_smoothers\":[" + blocks + "]";
  return s + "}";
}

// Re-indexes level 0 of a host hierarchy from compact fluid numbering to full-grid cells
// (structured grids whose level 0 the device keeps in the full-grid layout).
static void reindex_level0(const cfdg_grid* G, Hierarchy& H) {
  // Re-index level 0 from compact fluid numbering to full-grid cells.
  MgLevel& M = H.levels[0];
  const int32_t N = (int32_t)G->h.cells;
  std::vector<int32_t> full(M.n);
  for (int32_t j = 0; j < M.n; ++j) full[j] = H.masked ? H.fluid_indices[j] : j;
  std::vector<double> diag(N, 0.0);
  for (int32_t j = 0; j < M.n; ++j) diag[full[j]] = M.diag[j];
  M.diag = std::move(diag);
  for (auto& m : M.groups.col) m = full[m];
  for (auto& m : M.restrict.col) m = full[m];
  Csr P;
  P.off.assign(N + 1, 0);
  for (int32_t j = 0; j < M.n; ++j) P.off[full[j] + 1] = M.prolong.off[j + 1] - M.prolong.off[j];
  for (int32_t c = 0; c < N; ++c) P.off[c + 1] += P.off[c];
  P.col.resize(M.prolong.col.size());
  P.val.resize(M.prolong.val.size());
  for (int32_t j = 0; j < M.n; ++j)
    for (int32_t k = 0; k < M.prolong.off[j + 1] - M.prolong.off[j]; ++k) {
      P.col[P.off[full[j]] + k] = M.prolong.col[M.prolong.off[j] + k];
      P.val[P.off[full[j]] + k] = M.prolong.val[M.prolong.off[j] + k];
    }
  M.prolong = std::move(P);
  M.n = N;
  M.a = Csr();  // the wavefront kernel reads the grid's faces
  M.a.off.assign(1, 0);
  M.fwd = Schedule();
  M.bwd = Schedule();
}

// The host hierarchy of the mixed form: the grid's own when it is an aggregation
// hierarchy, else (grids without solid cells, which the reference coarsens geometrically
// with linear interpolation) an aggregation hierarchy of 2x2x2 bins built on first use.
// Its levels are point-smoothed bin grids like those of the grids with buildings, which
// the mixed form's fast paths and coarse-correction scale are made for.
int mixed_host_hierarchy_impl(cfdg_grid* G, std::shared_ptr<Hierarchy>& out) {
  if (!G->host_mg) return fail(CFDG_ERR_INVALID, "mixed form: no multigrid hierarchy");
  if (G->host_mg->masked) {
    out = G->host_mg;
    return 0;
  }
  if (!G->host_mg_mx) {
    Hierarchy H;
    Poller P;
    if (int e = build_aggregation_hierarchy(G->h, P, H)) {
      if (e == CFDG_E035) return fail(e, "CFD-E035: numerics.pressure_preconditioner: multigrid coarse Cholesky lost positive definiteness");
      return fail(e, "mixed form: aggregation hierarchy setup failed");
    }
    if (H.levels.size() > 1) reindex_level0(G, H);
    G->host_mg_mx = std::make_shared<Hierarchy>(std::move(H));
  }
  out = G->host_mg_mx;
  return 0;
}

int build_mg_dev(cfdg_grid* G, const Poller& poll) {
  Hierarchy H;
  if (int e = build_hierarchy(G->h, poll, H)) {
    if (e == CFDG_E034) return fail(e, "CFD-E034: numerics.pressure_preconditioner: multigrid requires fluid cells");
    if (e == CFDG_E035) return fail(e, "CFD-E035: numerics.pressure_preconditioner: multigrid coarse Cholesky lost positive definiteness");
    if (e == CFDG_CANCELLED) return fail(e, "cancelled");
    if (e == CFDG_WALL_TIME) return fail(e, "wall_time_limit");
    if (e == CFDG_E036)
      return fail(e, "CFD-E036: numerics.pressure_preconditioner: multigrid line Cholesky lost positive definiteness");
    return fail(e, "multigrid setup failed");
  }
  auto D = std::make_unique<DevHierarchy>();
  D->arena.ctx = G->ctx;
  cudaStream_t s = G->stream;
  D->masked = H.masked;
  D->nfluid = (int)H.fluid_indices.size();
  if (H.masked)
    if (int e = D->arena.upload(&D->fluid_idx, H.fluid_indices, s)) return e;
  D->levels.resize(H.levels.size());
  const bool lines = !H.levels.empty() && !H.levels[0].lines.empty();
  D->full0 = G->structured && H.levels.size() > 1 && !lines;
  D->coop0 = lines && H.levels.size() > 1;
  if (D->full0) reindex_level0(G, H);
  for (size_t l = 0; l < H.levels.size(); ++l) {
    MgLevel& M = H.levels[l];
    DevLevel& L = D->levels[l];
    L.n = M.n;
    if (int e = upload_csr(D->arena, M.a, L.a, s)) return e;
    if (int e = D->arena.upload(&L.diag, M.diag, s)) return e;
    if (int e = D->arena.upload(&L.fwd.order, M.fwd.order, s)) return e;
    if (int e = D->arena.upload(&L.bwd.order, M.bwd.order, s)) return e;
    L.fwd.start = M.fwd.start;
    L.bwd.start = M.bwd.start;
    if (int e = D->arena.upload(&L.fwd.d_start, M.fwd.start, s)) return e;
    if (int e = D->arena.upload(&L.bwd.d_start, M.bwd.start, s)) return e;
    L.ngroups = M.groups.rows();
    if (L.ngroups)
      if (int e = upload_csr(D->arena, M.groups, L.groups, s)) return e;
    L.terminal = M.direct_idx.rows() > 0 || l + 1 == H.levels.size();
    if (L.terminal) {
      L.nblocks = M.direct_idx.rows();
      if (int e = D->arena.upload(&L.d_ioff, M.direct_idx.off, s)) return e;
      if (int e = D->arena.upload(&L.d_idx, M.direct_idx.col, s)) return e;
      std::vector<long long> foff(M.direct_off.begin(), M.direct_off.end());
      if (int e = D->arena.upload(&L.d_foff, foff, s)) return e;
      if (int e = D->arena.upload(&L.d_fac, M.direct_factor, s)) return e;
    } else {
      if (int e = upload_csr(D->arena, M.prolong, L.prolong, s)) return e;
      if (int e = upload_csr(D->arena, M.restrict, L.restrict_, s)) return e;
    }
    if (int e = D->arena.alloc(&L.rhs, L.n)) return e;
    if (int e = D->arena.alloc(&L.x, L.n)) return e;
    if (int e = D->arena.alloc(&L.res, L.n)) return e;
    if (!M.lines.empty()) {
      const LineBlocks& B = M.lines[0];  // the reference builds one block group per level
      L.lines = true;
      L.llen = B.length;
      L.lbw = B.bandwidth;
      L.lcount = B.count();
      if (int e = D->arena.upload(&L.lnodes, B.nodes, s)) return e;
      if (int e = D->arena.upload(&L.looff, B.outside.off, s)) return e;
      if (int e = D->arena.upload(&L.locol, B.outside.col, s)) return e;
      if (int e = D->arena.upload(&L.loval, B.outside.val, s)) return e;
      if (int e = D->arena.upload(&L.lfac, B.factor, s)) return e;
      if (int e = D->arena.alloc(&L.lscr, B.nodes.size())) return e;
      if (int e = D->arena.upload(&L.lfwd.order, B.fwd.order, s)) return e;
      if (int e = D->arena.upload(&L.lbwd.order, B.bwd.order, s)) return e;
      L.lfwd.start = B.fwd.start;
      L.lbwd.start = B.bwd.start;
      if (int e = D->arena.upload(&L.lfwd.d_start, B.fwd.start, s)) return e;
      if (int e = D->arena.upload(&L.lbwd.d_start, B.bwd.start, s)) return e;
    }
  }
  D->level_cells = H.level_cells;
  D->level_nonzeros = H.level_nonzeros;
  // Levels 1 .. L-1 (0 .. L-1 for block-smoothed hierarchies) for the cooperative kernel,
  // when its grid can be co-resident.
  if (D->levels.size() > 1) {
    std::vector<PLev> pl;
    for (size_t l = D->coop0 ? 0 : 1; l < D->levels.size(); ++l) {
      const DevLevel& L = D->levels[l];
      PLev P{};
      P.n = L.n;
      P.terminal = L.terminal ? 1 : 0;
      P.ngroups = L.ngroups;
      P.nblocks = L.nblocks;
      P.nfwd = (int)L.fwd.start.size() - 1;
      P.nbwd = (int)L.bwd.start.size() - 1;
      int dl_max = 0;
      for (int q = 0; q < P.nfwd; ++q) dl_max = std::max(dl_max, L.fwd.start[q + 1] - L.fwd.start[q]);
      for (int q = 0; q < P.nbwd; ++q) dl_max = std::max(dl_max, L.bwd.start[q + 1] - L.bwd.start[q]);
      P.blocal = dl_max <= BLOCK ? 1 : 0;
      P.off = L.a.off, P.col = L.a.col, P.val = L.a.val, P.diag = L.diag;
      P.fo = L.fwd.order, P.fs = L.fwd.d_start, P.bo = L.bwd.order, P.bs = L.bwd.d_start;
      P.goff = L.groups.off, P.gmem = L.groups.col;
      P.roff = L.restrict_.off, P.rcol = L.restrict_.col, P.rval = L.restrict_.val;
      P.poff = L.prolong.off, P.pcol = L.prolong.col, P.pval = L.prolong.val;
      P.rhs = L.rhs, P.x = L.x, P.res = L.res;
      P.ioff = L.d_ioff, P.idx = L.d_idx, P.foff = L.d_foff, P.fac = L.d_fac;
      P.nsweep = L.lines ? 1 : 2;  // multigrid.rs:676
      P.lines = L.lines ? 1 : 0;
      if (L.lines) {
        P.llen = L.llen, P.lbw = L.lbw;
        P.lnfwd = (int)L.lfwd.start.size() - 1;
        P.lnbwd = (int)L.lbwd.start.size() - 1;
        int lmax = 0;
        for (int q = 0; q < P.lnfwd; ++q) lmax = std::max(lmax, L.lfwd.start[q + 1] - L.lfwd.start[q]);
        for (int q = 0; q < P.lnbwd; ++q) lmax = std::max(lmax, L.lbwd.start[q + 1] - L.lbwd.start[q]);
        P.lblocal = lmax <= BLOCK / 32 ? 1 : 0;  // one warp per block solve
        P.lnodes = L.lnodes, P.looff = L.looff, P.locol = L.locol, P.loval = L.loval, P.lfac = L.lfac;
        P.lscr = L.lscr;
        P.lfo = L.lfwd.order, P.lfs = L.lfwd.d_start, P.lbo = L.lbwd.order, P.lbs = L.lbwd.d_start;
      }
      pl.push_back(P);
    }
    PLev* dp = nullptr;
    if (int e = D->arena.upload(&dp, pl, s)) return e;
    D->d_plev = dp;
    // One block per SM: a dependency level fits in one pass and whole-level phases
    // (residual, transfers) have a few rows per thread.
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_plain_coarse, BLOCK, 0) != cudaSuccess || per < 1) {
      cudaGetLastError();
      per = 0;
    }
    D->coop_blocks = per > 0 ? sms : 0;
    // A cluster of PC_CLUSTER blocks, when one fits an SM group.
    {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(PC_CLUSTER, 1, 1);
      cfg.blockDim = dim3(BLOCK, 1, 1);
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = PC_CLUSTER;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, k_plain_coarse_cluster, &cfg) != cudaSuccess) {
        cudaGetLastError();
        clusters = 0;
      }
      D->cluster = clusters > 0;
    }
    if (D->coop0 && D->coop_blocks == 0 && !D->cluster)
      return fail(CFDG_ERR_UNSUPPORTED, "block-smoothed multigrid needs a co-resident cooperative launch");
  }
  CU(cudaStreamSynchronize(s));
  G->host_mg = std::make_shared<Hierarchy>(std::move(H));
  {
    std::lock_guard<std::mutex> lk(G->stats_mu);
    G->stats_json = stats_json_of(*D, *G->host_mg);
  }
  G->mg = std::move(D);
  return 0;
}

int prepare_mg_impl(cfdg_grid* G, const Poller& poll, cfdg_info* info) {
  if (int c = poll.check()) return fail(c, c == CFDG_CANCELLED ? "cancelled" : "wall_time_limit");
  if (G->h.n_components == 0)
    return fail(CFDG_E034, "CFD-E034: numerics.pressure_preconditioner: multigrid requires fluid cells");
  if (G->mg && G->signature && G->sig_version == G->faces_version) {
    // Faces unchanged since the hierarchy was last checked against them.
    if (info) {
      info->hierarchy_levels = G->mg->level_cells.size();
      for (auto v : G->mg->level_cells) info->hierarchy_cells += v;
      for (auto v : G->mg->level_nonzeros) info->hierarchy_nonzeros += v;
      info->hierarchy_bytes = G->mg->arena.bytes;
    }
    return 0;
  }
  Signature cur;
  int se = signature_of(G->h, cur);
  bool rebuild = !G->mg || !G->signature || se != 0 || !(cur == *G->signature);
  if (rebuild) {
    if (se)
      return fail(CFDG_E034, "CFD-E034: numerics.pressure_preconditioner: multigrid requires finite positive pressure face weights");
    G->mg.reset();
    G->host_mg_mx.reset();
    G->mixed.reset();
    G->solo.reset();
    reset_chunk(G);
    const auto t0 = std::chrono::steady_clock::now();
    if (int e = build_mg_dev(G, poll)) return e;
    G->signature = std::make_unique<Signature>(std::move(cur));
    if (info) {
      info->hierarchy_builds = 1;
      info->multigrid_setup_seconds = seconds_since(t0);
    }
  }
  G->sig_version = G->faces_version;
  if (info) {
    info->hierarchy_levels = G->mg->level_cells.size();
    for (auto v : G->mg->level_cells) info->hierarchy_cells += v;
    for (auto v : G->mg->level_nonzeros) info->hierarchy_nonzeros += v;
    info->hierarchy_bytes = G->mg->arena.bytes;
  }
  return 0;
}

// pressure.rs:55-97: the cached factor, or the hierarchy checked against its signature.
int prepare_preconditioner(cfdg_grid* G, const Poller& poll, cfdg_info* info) {
  if (G->preconditioner == CFDG_PRECOND_MULTIGRID) return prepare_mg_impl(G, poll, info);
  if (!G->ic0) {
    reset_chunk(G);
    const auto t0 = std::chrono::steady_clock::now();
    if (int e = build_ic0_dev(G)) return e;
    if (info) info->factor_setup_seconds = seconds_since(t0);
  }
  return 0;
}

int ensure_chunk(cfdg_grid* G) {
  int kind = G->preconditioner * 2 + (G->uniform ? 1 : 0);
  if (G->chunk && G->chunk_kind == kind) return 0;
  reset_chunk(G);
  cudaGraph_t graph;
  cudaStream_t user = G->stream;
  CU(cudaStreamSynchronize(user));
  G->stream = G->own;
  G->capturing = true;
  cudaError_t ce = cudaStreamBeginCapture(G->stream, cudaStreamCaptureModeThreadLocal);
  if (ce == cudaSuccess) {
    for (int i = 0; i < CHUNK; ++i) launch_iteration(G);
    ce = cudaStreamEndCapture(G->stream, &graph);
  }
  G->stream = user;
  G->capturing = false;
  if (ce != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("CUDA capture: ") + cudaGetErrorString(ce));
  cudaGraphGetNodes(graph, nullptr, &G->chunk_nodes);
  cudaError_t e = cudaGraphInstantiate(&G->chunk, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("CUDA graph: ") + cudaGetErrorString(e));
  G->chunk_kind = kind;
  return 0;
}

int poll_code(int c) { return fail(c, c == CFDG_CANCELLED ? "cancelled" : "wall_time_limit"); }

// The PCG solve of pressure.rs:342-436 on device vectors: G->b (and G->terms when
// use_terms) in, G->x out. Returns 0 or a CFDG code; fills info.
int check_wave(cfdg_grid* G);

int solve_device(cfdg_grid* G, bool use_terms, double tol, uint64_t max_iter, const Poller& poll, cfdg_info* info) {
  const int N = (int)G->h.cells;
  const int nb = grid_blocks(N);
  cudaStream_t s = G->stream;
  cfdg_info local{};
  cfdg_info* inf = info ? info : &local;
  std::memset(inf, 0, sizeof(*inf));
  Scalars init{};
  init.tol = tol;
  init.max_it = (long long)std::min<uint64_t>(max_iter, (uint64_t)1 << 62);
  CU(cudaMemcpyAsync(G->S, &init, sizeof(Scalars), cudaMemcpyHostToDevice, s));
  CU(cudaEventRecord(G->ev0, s));
  // Compatibility of closed components (pressure.rs:351-362).
  if (G->ncomp_groups) {
    k_compat<<<G->ncomp_groups, BLOCK, 0, s>>>(G->comp_groups.off, G->comp_groups.col, G->b, G->terms,
                                               use_terms ? 1 : 0, G->S);
    tick(G);
  }
  CU(cudaMemcpyAsync(G->hS, G->S, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  if (G->hS->done == 2) return fail(CFDG_E031, "CFD-E031: incompatible flux in a closed fluid component");
  if (int e = prepare_preconditioner(G, poll, inf)) return e;
  if (int e = ensure_chunk(G)) return e;
  // Prologue: x = 0, r = centred b, norm, z = M^-1 r, p = z, rz = r.z.
  k_fill<<<nb, BLOCK, 0, s>>>(G->x, 0.0, N, nullptr); tick(G);
  k_copy<<<nb, BLOCK, 0, s>>>(G->r, G->b, N, nullptr); tick(G);
  launch_center(G, G->comp_groups, G->ncomp_groups, G->r, nullptr);
  k_copy<<<nb, BLOCK, 0, s>>>(G->bc, G->r, N, nullptr); tick(G);
  k_pcg_norm<<<nb, BLOCK, 0, s>>>(G->r, N, G->partials, G->S); tick(G);
  launch_precondition(G, G->S);
  k_copy<<<nb, BLOCK, 0, s>>>(G->p, G->z, N, G->S); tick(G);
  k_pcg_rz<<<nb, BLOCK, 0, s>>>(G->r, G->z, N, G->partials, G->S, 1); tick(G);
  CU(cudaGetLastError());
  int status = 0;
  for (;;) {
    CU(cudaMemcpyAsync(G->hS, G->S, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    Scalars st = *G->hS;
    if (st.done) {
      if (st.done == 1) status = 0;
      else if (st.done == 4) status = 0;
      else if (st.done == 2) status = fail(st.error, "CFD-E032: pressure CG lost positive definiteness");
      else status = fail(CFDG_E033, "CFD-E033: pressure iteration limit " + std::to_string(max_iter));
      inf->iterations = st.done == 1 ? (uint64_t)st.it + 1 : 0;
      inf->relative_residual = st.done == 1 ? st.true_rel : 0.0;
      uint64_t loop_ops = st.done == 4 ? 0 : (uint64_t)st.it + (st.done == 3 ? 0 : 1);
      inf->work_units = loop_ops;
      inf->true_residual_checks = (uint64_t)st.true_checks;
      inf->operator_applications = loop_ops + (uint64_t)st.true_checks;
      inf->preconditioner_applications = st.done == 4 ? 0 : 1 + (uint64_t)st.it;
      break;
    }
    if (st.it >= (long long)max_iter) {  // not reached: the op kernel flags done = 3
      status = fail(CFDG_E033, "CFD-E033: pressure iteration limit " + std::to_string(max_iter));
      break;
    }
    if (int c = poll.check()) return poll_code(c);
    CU(cudaGraphLaunch(G->chunk, s));
    count(G->chunk_nodes);
  }
  if (G->preconditioner == CFDG_PRECOND_MULTIGRID && G->mg) {
    uint64_t cyc = inf->preconditioner_applications;
    inf->cycles = cyc;
    uint64_t inner = 0, smooth = 0, bvisits = 0, bsolves = 0;
    for (size_t l = 0; l + 1 < G->mg->levels.size(); ++l) {
      const DevLevel& L = G->mg->levels[l];
      // The hierarchy's unknowns (fluid cells on a masked level 0), not the full-grid
      // layout the device may keep level 0 in (masked.rs:337-341).
      const uint64_t n = G->mg->level_cells[l];
      inner += n;
      smooth += (L.lines ? 2 : 4) * n;  // 2 x sweeps
      if (L.lines) {
        // multigrid.rs:677-718: one block sweep each way, every block solved.
        bvisits += n;
        bsolves += 2 * (uint64_t)L.lcount;
      }
    }
    inf->smoothing_cell_updates = smooth * cyc;
    inf->block_level_cell_visits = bvisits * cyc;
    inf->block_smoothing_cell_updates = 2 * bvisits * cyc;
    inf->block_solves = bsolves * cyc;
    inf->residual_cell_updates = inner * cyc;
    inf->restriction_cell_updates = inner * cyc;
    inf->prolongation_cell_updates = inner * cyc;
    inf->coarse_solves = cyc;
  }
  if (status == 0 && G->hS->done == 1) launch_center(G, G->comp_groups, G->ncomp_groups, G->x, nullptr);
  if (status == 0 && G->hS->done == 4) {
    k_fill<<<nb, BLOCK, 0, s>>>(G->x, 0.0, N, nullptr);
    tick(G);
  }
  CU(cudaEventRecord(G->ev1, s));
  CU(cudaEventSynchronize(G->ev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, G->ev0, G->ev1);
  inf->device_seconds = ms * 1e-3;
  if (int e = check_wave(G)) return e;
  return status;
}

// A wavefront wait that gave up leaves its flag set: report it once and clear it.
int check_wave(cfdg_grid* G) {
  int err = 0;
  CU(cudaMemcpyAsync(&G->hS->counter, G->wave_err, sizeof(int), cudaMemcpyDeviceToHost, G->stream));
  CU(cudaStreamSynchronize(G->stream));
  err = (int)G->hS->counter;
  if (err) {
    CU(cudaMemsetAsync(G->wave_err, 0, sizeof(int), G->stream));
    return fail(CFDG_ERR_TIMEOUT, "a wavefront sweep's bounded wait gave up; results discarded");
  }
  return 0;
}

int project_mixed(cfdg_grid* G, double* d_u, double* d_p, double dt, double tol, uint64_t max_iter,
                  const Poller& poll, cfdg_info* info) {
  cfdg_info local{};
  cfdg_info* inf = info ? info : &local;
  std::memset(inf, 0, sizeof(*inf));
  if (int e = prepare_mg_impl(G, poll, inf)) return e;
  double setup = inf->multigrid_setup_seconds;
  if (!G->solo) {
    const auto t0 = std::chrono::steady_clock::now();
    cfdg_batch* B = cfdg_mixed_new(G->ctx);
    if (!B) return fail(CFDG_ERR_CUDA, "could not create the mixed-form stream");
    std::shared_ptr<cfdg_batch> solo(B, cfdg_mixed_delete);
    if (int e = cfdg_mixed_add_case(B, G)) return e;
    if (int e = cfdg_mixed_pack(B)) return e;
    G->solo = solo;
    setup += seconds_since(t0);
  }
  cfdg_mixed_set_stream(G->solo.get(), G->stream);
  int32_t code = 0;
  uint64_t builds = inf->hierarchy_builds, levels = inf->hierarchy_levels, cells = inf->hierarchy_cells,
           nnz = inf->hierarchy_nonzeros, hbytes = inf->hierarchy_bytes;
  if (int e = cfdg_mixed_project(G->solo.get(), &d_u, &d_p, &dt, tol, max_iter, poll.fn, poll.ctx, inf, &code))
    return e;
  inf->hierarchy_builds = builds, inf->hierarchy_levels = levels, inf->hierarchy_cells = cells;
  inf->hierarchy_nonzeros = nnz;
  inf->hierarchy_bytes = hbytes;
  if (G->host_mg_mx) {  // the solve ran on the aggregation hierarchy: its levels
    inf->hierarchy_levels = G->host_mg_mx->level_cells.size();
    inf->hierarchy_cells = inf->hierarchy_nonzeros = 0;
    for (auto v : G->host_mg_mx->level_cells) inf->hierarchy_cells += v;
    for (auto v : G->host_mg_mx->level_nonzeros) inf->hierarchy_nonzeros += v;
  }
  inf->multigrid_setup_seconds = setup;
  if (code == CFDG_E031) return fail(code, "CFD-E031: incompatible flux in a closed fluid component");
  if (code == CFDG_E032) return fail(code, "CFD-E032: pressure CG lost positive definiteness");
  if (code == CFDG_E033) return fail(code, "CFD-E033: pressure iteration limit " + std::to_string(max_iter));
  if (code) return fail(code, "mixed-form projection failed");
  CU(cudaStreamSynchronize(G->stream));
  return 0;
}

int project_device(cfdg_grid* G, double* d_u, double* d_p, double dt, double tol, uint64_t max_iter,
                   const Poller& poll, cfdg_info* info) {
  if (G->precision == CFDG_PRECISION_MIXED && G->preconditioner == CFDG_PRECOND_MULTIGRID && G->structured)
    return project_mixed(G, d_u, d_p, dt, tol, max_iter, poll, info);
  const int N = (int)G->h.cells;
  cudaStream_t s = G->stream;
  k_projection_rhs<<<grid_blocks(N), BLOCK, 0, s>>>(G->g, G->d_fluid, d_u, dt, G->b, G->terms, N); tick(G);
  if (int e = solve_device(G, true, tol, max_iter, poll, info)) return e;
  k_correct_faces<<<grid_blocks(G->h.faces), BLOCK, 0, s>>>(G->d_kind, G->d_lo, G->d_hi, G->d_dist, G->x, dt, d_u,
                                                            G->h.faces, G->S); tick(G);
  k_add<<<grid_blocks(N), BLOCK, 0, s>>>(d_p, G->x, N, G->S); tick(G);
  launch_center(G, G->comp_groups, G->ncomp_groups, d_p, nullptr);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(s));
  return 0;
}

int check_grid(cfdg_grid* G) {
  if (!G) return fail(CFDG_ERR_INVALID, "null grid");
  return 0;
}

// ----------------------------------------------------------------- laminar time stepping
// One SSPRK2 step of the laminar flow with a projection per stage (solver.rs:879-960,
// flow_euler solver.rs:671-732): u1 = P(u + dt (R(u) - grad p)), u2 = P(u1 + dt (R(u1) -
// grad p1)), u <- (u + u2) / 2 with the fixed faces re-applied, p <- p2. R is the steady
// momentum right-hand side of laminar flow with the default donor-cell advection
// (flow.rs:426-525). Every face evaluates the reference's expression in its order
// (-fmad=false), so a step is bit-identical to the reference algorithm on the same grid.
struct FlowDev {
  int n[3];
  long long face_off[3];
  int fdim[3][3];
  double dx[3], size[3], vel[3], nu, acc[3];
  int bnd[3];
  const uint8_t* kind;
  const int *lo, *hi;
  const double* dist;
  const uint8_t* fluid;
};

__device__ __forceinline__ long long fface(const FlowDev& D, int a, int i, int j, int k) {
  return D.face_off[a] + ((long long)k * D.fdim[a][1] + j) * D.fdim[a][0] + i;
}

// grid.rs:631-645 cell_velocity, one array per axis.
__global__ void k_cell_velocity(FlowDev D, const double* __restrict__ u, double* __restrict__ cu, int N) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
    const int i = c % D.n[0], j = (c / D.n[0]) % D.n[1], k = c / (D.n[0] * D.n[1]);
    const int q[3] = {i, j, k};
    for (int a = 0; a < 3; ++a) {
      if (!D.fluid[c]) {
        cu[(long long)a * N + c] = 0.0;
        continue;
      }
      int p[3] = {q[0], q[1], q[2]};
      const double lo = u[fface(D, a, p[0], p[1], p[2])];
      p[a] += 1;
      const double hi = u[fface(D, a, p[0], p[1], p[2])];
      cu[(long long)a * N + c] = 0.5 * (lo + hi);
    }
  }
}

// flow.rs:66-154 ghost_values, laminar flow without moving walls.
__device__ __forceinline__ double ghost(const FlowDev& D, int a, const double center[3], int d, int side,
                                        double value) {
  const bool at_domain = side < 0 ? center[d] < D.dx[d] : center[d] > D.size[d] - D.dx[d];
  const int bc = D.bnd[d];
  if (at_domain && bc == 3) return value;  // slip
  if (at_domain && bc == 1) {              // open
    const double speed = D.vel[d] * (double)side;
    if (speed < -1e-12) return 2.0 * D.vel[a] - value;
    return value;
  }
  const double target = 0.0;
  return 2.0 * target - value;
}

// flow.rs:426-525 momentum_rhs (laminar, donor cell), then u + dt (rhs - grad p) and the
// fixed face values (solver.rs:695-719, grid.rs:683-691).
__global__ void k_momentum_update(FlowDev D, const double* __restrict__ u, const double* __restrict__ p,
                                  const double* __restrict__ cu, double dt, double* __restrict__ out, long long F,
                                  int N) {
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < F; f += (long long)gridDim.x * blockDim.x) {
    const int a = f >= D.face_off[2] ? 2 : (f >= D.face_off[1] ? 1 : 0);
    long long r = f - D.face_off[a];
    const int q[3] = {(int)(r % D.fdim[a][0]), (int)((r / D.fdim[a][0]) % D.fdim[a][1]),
                      (int)(r / ((long long)D.fdim[a][0] * D.fdim[a][1]))};
    const uint8_t kd = D.kind[f];
    if (kd == WALL || kd == SLIP || kd == BLOCKED) {
      out[f] = 0.0;
      continue;
    }
    if (kd == INLET) {
      out[f] = D.vel[a];
      continue;
    }
    const int lo = D.lo[f], hi = D.hi[f];
    double velocity[3];
    for (int d = 0; d < 3; ++d) {
      if (lo >= 0 && hi >= 0) velocity[d] = 0.5 * (cu[(long long)d * N + lo] + cu[(long long)d * N + hi]);
      else if (lo >= 0) velocity[d] = cu[(long long)d * N + lo];
      else if (hi >= 0) velocity[d] = cu[(long long)d * N + hi];
      else velocity[d] = 0.0;
    }
    double center[3];
    for (int d = 0; d < 3; ++d) center[d] = ((double)q[d] + (d == a ? 0.0 : 0.5)) * D.dx[d];
    const double uf = u[f];
    double rhs = 0.0;
    for (int d = 0; d < 3; ++d) {
      double vlo, vhi;
      for (int side = 0; side < 2; ++side) {
        int pq[3] = {q[0], q[1], q[2]};
        pq[d] += side ? 1 : -1;
        const bool exists = pq[d] >= 0 && pq[d] < D.fdim[a][d];
        double v;
        if (exists) {
          const long long nb = fface(D, a, pq[0], pq[1], pq[2]);
          const uint8_t nk = D.kind[nb];
          v = ((nk == WALL || nk == BLOCKED) && d != a) ? ghost(D, a, center, d, side ? 1 : -1, uf) : u[nb];
        } else {
          v = d == a ? uf : ghost(D, a, center, d, side ? 1 : -1, uf);
        }
        if (side) vhi = v;
        else vlo = v;
      }
      rhs = rhs - velocity[d] * (velocity[d] >= 0.0 ? (uf - vlo) / D.dx[d] : (vhi - uf) / D.dx[d]);
      const double mu = D.nu + 0.0;
      rhs = rhs + (mu * (vhi - uf) - mu * (uf - vlo)) / (D.dx[d] * D.dx[d]);
    }
    rhs = rhs + D.acc[a];
    rhs = rhs + (lo >= 0 && hi >= 0 ? 0.5 * (0.0 + 0.0) : 0.0);  // the RANS cross term, zero here
    double grad;
    if (kd == INTERIOR) grad = (p[hi] - p[lo]) / D.dist[f];
    else grad = lo >= 0 ? -p[lo] / D.dist[f] : p[hi] / D.dist[f];  // outlet
    out[f] = uf + dt * (rhs - grad);
  }
}

// SSPRK2 combination u <- (u + u2) / 2, then the fixed face values (solver.rs:937-946).
__global__ void k_ssprk_combine(FlowDev D, double* __restrict__ u, const double* __restrict__ u2, long long F) {
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < F; f += (long long)gridDim.x * blockDim.x) {
    const uint8_t kd = D.kind[f];
    const int a = f >= D.face_off[2] ? 2 : (f >= D.face_off[1] ? 1 : 0);
    if (kd == WALL || kd == SLIP || kd == BLOCKED) u[f] = 0.0;
    else if (kd == INLET) u[f] = D.vel[a];
    else u[f] = 0.5 * (u[f] + u2[f]);
  }
}

// ----------------------------------------------------------------- scalar transport
// transport.rs:651-699 rhs_into (linear upwind, zero inlet concentration) and
// solver.rs:808-855 advance_scalar. The reference loops over faces and applies each
// transporting face's flux / volume to its lo cell (subtracted) and hi cell (added); a
// cell therefore receives its faces in face order: x-lo, x-hi, y-lo, y-hi, z-lo, z-hi.
// Here each face's value is computed once by one thread of a 32x8 tile marching in z
// (x neighbours through warp shuffles, y neighbours through shared memory, z in
// registers) and each cell sums its six faces in that order: the same bits without
// atomics. The kernels are bound by the FP64 pipe (one FP64 add or multiply per SM and
// clock on this part), so FP64 operations that are exact in integer arithmetic are done
// there: a product with, or a quotient by, a power of two (0.5, and the face area,
// distance and cell volume of grids with power-of-two spacing) is an addition to the
// exponent field while the operand and result are normal numbers (the same real value,
// so the same bits; zeros, subnormals, infinities and NaNs take the FP64 instruction),
// and `x + 0.0` only turns -0.0 into +0.0.
// A factor 2^e (value v) when `ok`; otherwise the factor is not a power of two.
struct Pow2 {
  double v;
  int e;
  int ok;
};

struct ScalarDev {
  int n[3];
  long long face_off[3];
  int fdim[3][3];
  double volume;
  Pow2 inv_volume;  // 1/volume
  const uint8_t* kind;
  const uint8_t* fluid;
  const int *lo, *hi;
  const double *area, *dist;
  // Uniform grids: the area and distance of the transporting faces per axis and kind
  // (interior, inlet, outlet), equal bit for bit on every such face.
  double area_k[3][3], dist_k[3][3];
  Pow2 area_p[3][3], inv_dist_p[3][3];
};

constexpr int STX = 32, STY = 8;  // cells of one transport tile in x and y (its z extent is chosen per grid)

__device__ __forceinline__ int transport_slot(uint8_t k) { return k == INTERIOR ? 0 : (k == INLET ? 1 : 2); }

__device__ __forceinline__ double plus_zero(double x) {  // x + 0.0
  return __double_as_longlong(x) == (long long)0x8000000000000000ull ? 0.0 : x;
}

// The rare FP64 paths, out of line: an if-converted FP64 instruction whose lanes are all
// predicated off still takes its turn on the FP64 pipe.
__device__ __noinline__ double fp64_mul(double x, double y) { return x * y; }

// x * 2^e, the exponent field moved when x and the result are normal (bit-identical to the
// FP64 product, which is exact there), the FP64 product otherwise.
__device__ __forceinline__ double mul_pow2(double x, const Pow2& p) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  const int r = e + p.e;
  if (e != 0 && e != 0x7ff && r >= 1 && r <= 2046) return __longlong_as_double(b + ((long long)p.e << 52));
  if ((b & 0x7fffffffffffffffLL) == 0) return x;  // a signed zero stays itself
  return fp64_mul(x, p.v);
}

// x >= 0.0 on the bits: +0.0 and -0.0, and positive numbers up to +infinity; not NaN.
__device__ __forceinline__ bool nonneg(double x) {
  const long long b = __double_as_longlong(x);
  return (b & 0x7fffffffffffffffLL) == 0 || (b >= 0 && b <= 0x7ff0000000000000LL);
}
__device__ __forceinline__ double half(double x) { return mul_pow2(x, Pow2{0.5, -1, 1}); }

__device__ __forceinline__ double twice(double x) { return mul_pow2(x, Pow2{2.0, 1, 1}); }
__device__ __forceinline__ bool is_nan64(double x) {
  return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
__device__ __noinline__ bool fp64_prod_le0(double a, double b) { return a * b <= 0.0; }
// The exponent q of |x| = m 2^q, m in [1, 2), from its nonzero finite magnitude bits.
__device__ __forceinline__ int exp_of(long long mag) {
  const int e = (int)(mag >> 52);
  return e ? e - 1023 : -1074 + (63 - __clzll(mag));
}
// a * b <= 0.0 as the FP64 product and comparison decide it, on the bits where the signs and
// exponents settle it: a NaN operand or 0 * inf gives NaN (false); a zero operand a zero
// product (true); different signs a negative product or -0 (true); an infinite operand of
// the same sign +inf (false). Same-sign finite products are at least 2^-1074, the smallest
// subnormal, when qa + qb >= -1074 (false) and below 2^-1075, so rounded to zero, when
// qa + qb <= -1077 (true); the two exponent sums between go to the FP64 product.
__device__ __forceinline__ bool prod_le_zero(double a, double b) {
  const long long ua = __double_as_longlong(a), ub = __double_as_longlong(b);
  const long long ma = ua & 0x7fffffffffffffffLL, mb = ub & 0x7fffffffffffffffLL;
  const long long inf = 0x7ff0000000000000LL;
  if (ma > inf || mb > inf) return false;
  if (ma == 0 || mb == 0) return ma != inf && mb != inf;
  if ((ua ^ ub) < 0) return true;
  if (ma == inf || mb == inf) return false;
  const int q = exp_of(ma) + exp_of(mb);
  if (q >= -1074) return false;
  if (q <= -1077) return true;
  return fp64_prod_le0(a, b);
}
// minmod (transport.rs:510-516): 0 when a b <= 0 (the FP64 product, so an underflow to zero
// counts; decided by prod_le_zero), else signum(a) min(|a|, |b|). a is nonzero there, so signum(a) times the minimum
// is the minimum with a's sign; f64::min of two magnitudes is the smaller bit pattern (a
// NaN magnitude is above every number, and min returns the other operand); signum of a NaN
// is NaN, and so is the product.
__device__ __forceinline__ double minmod_bits(double a, double b) {
  if (prod_le_zero(a, b)) return 0.0;
  if (is_nan64(a)) return a;
  const long long ma = __double_as_longlong(a) & 0x7fffffffffffffffLL;
  const long long mb = __double_as_longlong(b) & 0x7fffffffffffffffLL;
  return __longlong_as_double((ma < mb ? ma : mb) | (__double_as_longlong(a) & (long long)0x8000000000000000ull));
}
// The monotonized-central slope (transport.rs:517-526) of a cell of value xc whose
// neighbours along the axis have values lo and hi (the cell's own value where the face
// between is not interior): minmod((hi - lo) / 2, minmod(2 (xc - lo), 2 (hi - xc))), the
// products by 0.5 and 2 through the exponent field.
__device__ __forceinline__ double mc_slope(double lo, double xc, double hi) {
  return minmod_bits(half(hi - lo), minmod_bits(twice(xc - lo), twice(hi - xc)));
}

// The flux / volume of face f on axis a between cells lo_cell and hi_cell (its structural
// neighbours, -1 outside the domain), evaluated on the field x; false if the face does not
// transport. UNI: the layout's lo/hi (interior iff both are fluid) and per-axis constants.
// P2 (with UNI): the volume and every transporting face's area and distance are powers of
// two, so the products and quotients by them go through the exponent field.
// MUSCL (transport.rs:670-694): the donor is the upwind cell's value plus (flow towards hi)
// or minus half its slope along a, whose neighbours are the cells across the upwind cell's
// two faces on a (faces f -+ one face stride; the grid is not periodic, so both exist).
template <bool UNI, bool P2, bool MUSCL = false>
__device__ __forceinline__ bool face_eval(const ScalarDev& D, int a, long long f, long long lo_cell,
                                          long long hi_cell, const double* __restrict__ x,
                                          const double* __restrict__ u, const double* __restrict__ d, double& pv) {
  const uint8_t k = D.kind[f];
  if (k != INTERIOR && k != INLET && k != OUTLET) return false;
  bool hl, hh;
  double area = 0.0, dist = 0.0;
  Pow2 area_p{0.0, 0, 0}, inv_dist_p{0.0, 0, 0};
  if (UNI) {
    if (k == INTERIOR) {
      hl = hh = true;
    } else {
      hl = lo_cell >= 0 && D.fluid[lo_cell];
      hh = hi_cell >= 0 && D.fluid[hi_cell];
    }
    const int t = transport_slot(k);
    if (P2) {
      area_p = D.area_p[a][t];
      inv_dist_p = D.inv_dist_p[a][t];
    } else {
      area = D.area_k[a][t];
      dist = D.dist_k[a][t];
    }
  } else {
    hl = D.lo[f] >= 0;
    hh = D.hi[f] >= 0;
    area = D.area[f];
    dist = D.dist[f];
  }
  const double cl = hl ? x[lo_cell] : 0.0, cr = hh ? x[hi_cell] : 0.0;
  const double uf = u[f];
  double donor;
  if (MUSCL) {
    const long long cs = a == 0 ? 1 : (a == 1 ? (long long)D.n[0] : (long long)D.n[0] * D.n[1]);
    const long long fs = a == 0 ? 1 : (a == 1 ? (long long)D.fdim[1][0] : (long long)D.fdim[2][0] * D.fdim[2][1]);
    // One slope per face, of the upwind cell, without a branch on the flow's sign: its
    // value vc, the neighbour across face f (vf) and the one across its other face on a
    // (vo, through face f -+ fs). donor = vc + h with h = +-slope / 2 equals the reference's
    // cl + slope / 2 or cr - slope / 2 bit for bit (a - b is a + (-b)); without an upwind
    // cell vc is the inlet value 0.0 and h = +-0.0, whose sum is 0.0 like the bare inlet value.
    const bool up = nonneg(uf);
    const double vc = up ? cl : cr;
    double h = 0.0;
    if (up ? hl : hh) {
      const long long fo = up ? f - fs : f + fs;
      const double vo = D.kind[fo] == INTERIOR ? x[up ? lo_cell - cs : hi_cell + cs] : vc;
      const double vf = k == INTERIOR ? (up ? cr : cl) : vc;
      h = half(mc_slope(up ? vo : vf, vc, up ? vf : vo));
    }
    donor = vc + (up ? h : -h);
  } else {
    // Donor: the upwind cell's value (+ 0.0 when it exists; the inlet value 0.0 otherwise,
    // whose + 0.0 is the same bits); `cr - 0.0` is cr for every cr.
    donor = nonneg(uf) ? plus_zero(cl) : cr;
  }
  double diffusivity;
  if (hl && hh) diffusivity = half(d[lo_cell] + d[hi_cell]);
  else if (hl) diffusivity = d[lo_cell];
  else if (hh) diffusivity = d[hi_cell];
  else diffusivity = 0.0;
  if (P2) {
    const double diff = k == OUTLET ? 0.0 : mul_pow2(diffusivity * (cl - cr), inv_dist_p);
    pv = mul_pow2(mul_pow2(uf * donor + diff, area_p), D.inv_volume);
  } else {
    const double diff = k == OUTLET ? 0.0 : diffusivity * (cl - cr) / dist;
    pv = (uf * donor + diff) * area / D.volume;
  }
  return true;
}

// MUSCL from a face's own lo and hi (the budget's boundary faces): the donor value of a
// face is the upwind cell's value plus (u >= 0: lo cell) or minus (hi cell) half its
// monotonized-central slope along the face's axis; neighbours count only through interior
// faces (transport.rs:502-526, 670-694).
// The face index of cell (i, j, k)'s face on axis a, side 0 (lo) or 1 (hi); on a periodic
// axis (n faces, not n + 1) the last cell's hi face is the wrap face 0.
__device__ __forceinline__ long long sc_face(const ScalarDev& D, int a, int i, int j, int k, int side) {
  int p[3] = {i, j, k};
  p[a] += side;
  if (p[a] >= D.fdim[a][a]) p[a] -= D.fdim[a][a];
  return D.face_off[a] + ((long long)p[2] * D.fdim[a][1] + p[1]) * D.fdim[a][0] + p[0];
}
__device__ __forceinline__ double sc_slope(const ScalarDev& D, const double* __restrict__ x, long long cell, int a) {
  const int i = (int)(cell % D.n[0]), j = (int)((cell / D.n[0]) % D.n[1]), k = (int)(cell / ((long long)D.n[0] * D.n[1]));
  const long long fl = sc_face(D, a, i, j, k, 0), fh = sc_face(D, a, i, j, k, 1);
  const double xc = x[cell];
  const double lo = D.kind[fl] == INTERIOR ? x[D.lo[fl]] : xc;
  const double hi = D.kind[fh] == INTERIOR ? x[D.hi[fh]] : xc;
  return mc_slope(lo, xc, hi);
}
// The flux (kg/s) of transporting face f on axis a evaluated on x, rhs_into's arithmetic
// from the face's own lo, hi, area and distance; false if the face does not transport.
__device__ __forceinline__ bool sc_flux(const ScalarDev& D, int a, long long f, const double* __restrict__ x,
                                        const double* __restrict__ u, const double* __restrict__ d, bool muscl,
                                        double& flux) {
  const uint8_t k = D.kind[f];
  if (k != INTERIOR && k != INLET && k != OUTLET) return false;
  const int lo = D.lo[f], hi = D.hi[f];
  const double cl = lo >= 0 ? x[lo] : 0.0, cr = hi >= 0 ? x[hi] : 0.0;
  const double uf = u[f];
  double donor;
  if (uf >= 0.0) donor = lo >= 0 ? cl + (muscl ? 0.5 * sc_slope(D, x, lo, a) : 0.0) : cl;
  else donor = hi >= 0 ? cr - (muscl ? 0.5 * sc_slope(D, x, hi, a) : 0.0) : cr;
  double diffusivity;
  if (lo >= 0 && hi >= 0) diffusivity = 0.5 * (d[lo] + d[hi]);
  else if (lo >= 0) diffusivity = d[lo];
  else if (hi >= 0) diffusivity = d[hi];
  else diffusivity = 0.0;
  const double diff = k == OUTLET ? 0.0 : diffusivity * (cl - cr) / D.dist[f];
  flux = (uf * donor + diff) * D.area[f];
  return true;
}

// The rates transport.rs rhs_into returns with the right-hand side (solver.rs:828-833):
// emitted = Σ source × volume, and over the faces on the domain boundary (lo or hi absent)
// the outward flux's positive part (outflow) and negative part (inflow), in kg/s, with the
// face flux (u donor + diffusion) area of the same transport faces. Per block, in part[3b ..
// 3b+2]; k_scalar_budget sums the blocks in order. The sums differ from the reference's
// sequential ones by rounding only (the budgets serve mass accounting, not bits).
constexpr int SR_BLOCKS = 128, SR_THREADS = 256;
__global__ void __launch_bounds__(SR_THREADS) k_scalar_rates(ScalarDev D, const double* __restrict__ x,
                                                            const double* __restrict__ u,
                                                            const double* __restrict__ d,
                                                            const double* __restrict__ source, long long N,
                                                            double* __restrict__ part, int muscl) {
  double em = 0.0, inflow = 0.0, outflow = 0.0;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x, nth = (long long)gridDim.x * blockDim.x;
  for (long long i = tid; i < N; i += nth) em += source[i];
  for (int a = 0; a < 3; ++a) {
    const int b = (a + 1) % 3, cc = (a + 2) % 3, nb = D.n[b], nc = D.n[cc];
    const long long plane = (long long)nb * nc;
    for (long long q = tid; q < 2 * plane; q += nth) {
      const int side = q >= plane ? 1 : 0;
      const long long r = q - side * plane;
      int pos[3];
      pos[a] = side ? D.n[a] : 0;
      pos[b] = (int)(r % nb);
      pos[cc] = (int)(r / nb);
      const long long f = D.face_off[a] + ((long long)pos[2] * D.fdim[a][1] + pos[1]) * D.fdim[a][0] + pos[0];
      const int lo = D.lo[f], hi = D.hi[f];
      if (lo >= 0 && hi >= 0) continue;  // not on the boundary (periodic wrap)
      double flux;
      if (!sc_flux(D, a, f, x, u, d, muscl != 0, flux)) continue;
      const double outward = lo >= 0 ? flux : -flux;
      outflow += fmax(outward, 0.0);
      inflow += fmax(-outward, 0.0);
    }
  }
  __shared__ double sh[3][SR_THREADS / 32];
  double v[3] = {em, inflow, outflow};
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < SR_THREADS / 32; ++w) t += sh[threadIdx.x][w];
    part[3 * blockIdx.x + threadIdx.x] = t;
  }
}

// The block sums of the two stages' rates in block order; the emission is the source sum
// times the volume. budget += dt (a + b) / 2 per quantity (solver.rs:851-853) when budget is
// set; rates (when set) receive the first stage's rates.
__global__ void k_scalar_budget(const double* __restrict__ pa, const double* __restrict__ pb, double volume, double dt,
                                double* __restrict__ budget, double* __restrict__ rates) {
  if (threadIdx.x >= 3) return;
  const int k = threadIdx.x;
  double a = 0.0, b = 0.0;
  for (int blk = 0; blk < SR_BLOCKS; ++blk) {
    a += pa[3 * blk + k];
    if (pb) b += pb[3 * blk + k];
  }
  if (k == 0) {
    a *= volume;
    b *= volume;
  }
  if (rates) rates[k] = a;
  if (budget) budget[k] += 0.5 * dt * (a + b);
}

// One pass of the SSPRK2 step over a tile of (32, 8, zs) cells. MODE 0 (solver.rs:845-847):
// stage = c + dt rhs(c). MODE 1 (solver.rs:848-850): c = (c + stage + dt rhs(stage)) / 2, in
// place (a thread reads c only at its own cell). Blocks are (32, 8); every thread reaches
// every barrier and shuffle.
template <bool UNI, bool P2, bool MUSCL, int MODE>
__global__ void __launch_bounds__(STX * STY) k_scalar_pass(ScalarDev D, double* __restrict__ c,
                                                          double* __restrict__ stage, const double* __restrict__ u,
                                                          const double* __restrict__ d,
                                                          const double* __restrict__ source, double dt, int zs) {
  __shared__ double s_pv[STY][STX];
  __shared__ uint8_t s_on[STY][STX];
  const double* __restrict__ x = MODE == 0 ? c : stage;  // the field the right-hand side reads
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nx = D.n[0], ny = D.n[1], nz = D.n[2];
  const int i = blockIdx.x * STX + tx, j = blockIdx.y * STY + ty;
  const int z0 = blockIdx.z * zs, z1 = min(z0 + zs, nz);
  const bool valid = i < nx && j < ny;
  const long long sx = nx, sxy = (long long)nx * ny;
  double zlo = 0.0;
  bool zlo_on = false;
  if (valid) {  // the z-lo face of the first slice
    const long long cell = z0 * sxy + j * sx + i;
    const long long f = D.face_off[2] + ((long long)z0 * D.fdim[2][1] + j) * D.fdim[2][0] + i;
    zlo_on = face_eval<UNI, P2, MUSCL>(D, 2, f, z0 > 0 ? cell - sxy : -1, cell, x, u, d, zlo);
  }
  for (int z = z0; z < z1; ++z) {
    const long long cell = z * sxy + j * sx + i;
    double xlo = 0.0, xhi = 0.0, ylo = 0.0, yhi = 0.0, zhi = 0.0;
    bool xlo_on = false, xhi_on = false, ylo_on = false, yhi_on = false, zhi_on = false;
    if (valid) {
      const long long fx = D.face_off[0] + ((long long)z * D.fdim[0][1] + j) * D.fdim[0][0] + i;
      xlo_on = face_eval<UNI, P2, MUSCL>(D, 0, fx, i > 0 ? cell - 1 : -1, cell, x, u, d, xlo);
      const long long fy = D.face_off[1] + ((long long)z * D.fdim[1][1] + j) * D.fdim[1][0] + i;
      ylo_on = face_eval<UNI, P2, MUSCL>(D, 1, fy, j > 0 ? cell - sx : -1, cell, x, u, d, ylo);
      const long long fz = D.face_off[2] + ((long long)(z + 1) * D.fdim[2][1] + j) * D.fdim[2][0] + i;
      zhi_on = face_eval<UNI, P2, MUSCL>(D, 2, fz, cell, z + 1 < nz ? cell + sxy : -1, x, u, d, zhi);
    }
    // x-hi: the next lane's x-lo, or computed here at the tile's or the domain's edge.
    const double nxt = __shfl_down_sync(0xffffffffu, xlo, 1);
    const int nxt_on = __shfl_down_sync(0xffffffffu, (int)xlo_on, 1);
    s_pv[ty][tx] = ylo;
    s_on[ty][tx] = ylo_on;
    __syncthreads();
    if (valid) {
      if (tx == STX - 1 || i == nx - 1) {
        const long long fx = D.face_off[0] + ((long long)z * D.fdim[0][1] + j) * D.fdim[0][0] + i + 1;
        xhi_on = face_eval<UNI, P2, MUSCL>(D, 0, fx, cell, i + 1 < nx ? cell + 1 : -1, x, u, d, xhi);
      } else {
        xhi = nxt;
        xhi_on = nxt_on != 0;
      }
      if (ty == STY - 1 || j == ny - 1) {
        const long long fy = D.face_off[1] + ((long long)z * D.fdim[1][1] + j + 1) * D.fdim[1][0] + i;
        yhi_on = face_eval<UNI, P2, MUSCL>(D, 1, fy, cell, j + 1 < ny ? cell + sx : -1, x, u, d, yhi);
      } else {
        yhi = s_pv[ty + 1][tx];
        yhi_on = s_on[ty + 1][tx] != 0;
      }
      double acc = source[cell];
      if (D.fluid[cell]) {  // a solid cell is on no face: its rate is its source
        if (xlo_on) acc = acc + xlo;
        if (xhi_on) acc = acc - xhi;
        if (ylo_on) acc = acc + ylo;
        if (yhi_on) acc = acc - yhi;
        if (zlo_on) acc = acc + zlo;
        if (zhi_on) acc = acc - zhi;
      }
      if (MODE == 0) stage[cell] = c[cell] + dt * acc;
      else c[cell] = half(c[cell] + stage[cell] + dt * acc);
    }
    zlo = zhi;
    zlo_on = zhi_on;
    __syncthreads();  // s_pv is rewritten by the next slice
  }
}

// Slices per block of the scalar passes: the z extent split so that the blocks' slices
// spread evenly over the SMs (the passes are FP64-pipe bound, so an SM's time follows the
// slices it is given: about ceil(blocks / SMs) zs), counting the z face each block
// evaluates once more than its slices need (a third of a slice's faces), among the splits
// that give every SM its four resident blocks (the smallest split where none does).
int scalar_zsplit(const int32_t n[3], int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  sms = std::max(sms, 1);
  const long long cols = (long long)((n[0] + STX - 1) / STX) * ((n[1] + STY - 1) / STY);
  int best = 2;
  double best_cost = 1e300;
  for (int zs = 2; zs <= 16; ++zs) {
    const long long blocks = cols * ((n[2] + zs - 1) / zs);
    if (zs > 2 && blocks < 4LL * sms) continue;
    const double cost = (double)((blocks + sms - 1) / sms) * std::min(zs, n[2]) * (1.0 + 1.0 / (3.0 * zs));
    if (cost < best_cost - 1e-9) {
      best_cost = cost;
      best = zs;
    }
  }
  return best;
}

FlowDev flow_dev(cfdg_grid* G) {
  FlowDev D{};
  for (int a = 0; a < 3; ++a) {
    D.n[a] = G->h.n[a];
    D.face_off[a] = G->g.face_off[a];
    for (int d = 0; d < 3; ++d) D.fdim[a][d] = G->g.fdim[a][d];
    D.dx[a] = G->h.dx[a];
    D.size[a] = G->flow_size[a];
    D.vel[a] = G->flow_vel[a];
    D.acc[a] = G->flow_acc[a];
    D.bnd[a] = G->flow_bnd[a];
  }
  D.nu = G->flow_nu;
  D.kind = G->d_kind;
  D.lo = G->d_lo;
  D.hi = G->d_hi;
  D.dist = G->d_dist;
  D.fluid = G->d_fluid;
  return D;
}

// One stage: out = u + dt (R(u) - grad p) with the fixed faces, then the projection of
// out with p1 (= p on entry) accumulating the pressure.
int flow_stage(cfdg_grid* G, const FlowDev& D, const double* u, double* out, double* p1, double dt, double tol,
               uint64_t max_iter, const Poller& P, cfdg_info* info) {
  const int N = (int)G->h.cells;
  const long long F = G->h.faces;
  cudaStream_t s = G->stream;
  k_cell_velocity<<<grid_blocks(N), BLOCK, 0, s>>>(D, u, G->st_cu, N); tick(G);
  k_momentum_update<<<grid_blocks((int)std::min<long long>(F, 1LL << 30)), BLOCK, 0, s>>>(D, u, p1, G->st_cu, dt, out, F, N);
  tick(G);
  return project_device(G, out, p1, dt, tol, max_iter, P, info);
}

}  // namespace

namespace cfdg {
int prepare_multigrid(cfdg_grid* G) {
  Poller P;
  return prepare_mg_impl(G, P, nullptr);
}

int mixed_host_hierarchy(cfdg_grid* G, std::shared_ptr<Hierarchy>& out) { return mixed_host_hierarchy_impl(G, out); }

int plain_compat_center(cfdg_grid* G, cudaStream_t s) {
  Scalars init{};
  CU(cudaMemcpyAsync(G->S, &init, sizeof(Scalars), cudaMemcpyHostToDevice, s));
  k_compat<<<G->ncomp_groups, BLOCK, 0, s>>>(G->comp_groups.off, G->comp_groups.col, G->b, G->terms, 1, G->S);
  count();
  CU(cudaMemcpyAsync(G->hS, G->S, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  if (G->hS->done == 2) return CFDG_E031;
  CU(cudaMemcpyAsync(G->bc, G->b, G->h.cells * 8, cudaMemcpyDeviceToDevice, s));
  plain_center(G, G->bc, s);
  return 0;
}

void plain_center(cfdg_grid* G, double* x, cudaStream_t s) {
  if (G->ncomp_groups == 0) return;
  k_center<<<G->ncomp_groups, BLOCK, 0, s>>>(G->comp_groups.off, G->comp_groups.col, x, nullptr);
  count();
}
}  // namespace cfdg

// ------------------------------------------------------------------ no-allocation residual
// Scratch of cfdg_residual_norm_noalloc: 2 * NOALLOC_MAX_BLOCKS partial sums and the
// last-block counter, 128 KiB + 256 B of static device memory that every GPU loading
// this library holds until the process exits. All calls share it.
static __device__ __align__(256) double g_noalloc_scratch[2 * NOALLOC_MAX_BLOCKS + 32];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {nullptr};  // device address of g_noalloc_scratch, per device

// Once per device, with that device current: the device address of the scratch array.
// In host code the symbol names a host-side stand-in, never a device address.
int noalloc_scratch(int device, double** out) {
  if (device < 0 || device >= 64) return fail(CFDG_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(CFDG_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[device] = (double*)ptr;
  }
  *out = g_noalloc_ptr[device];
  return 0;
}
}  // namespace

// ============================================================== C ABI

extern "C" {

const char* cfdg_last_error(void) { return t_error.c_str(); }

int cfdg_context_create(int device, uint64_t hbm_budget_bytes, cfdg_context** out) {
  if (!out) return fail(CFDG_ERR_INVALID, "null output pointer");
  *out = nullptr;
  int count = 0;
  CU(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(CFDG_ERR_CUDA, "no such CUDA device");
  CU(cudaSetDevice(device));
  size_t free_b = 0, total_b = 0;
  CU(cudaMemGetInfo(&free_b, &total_b));
  auto* c = new cfdg_context();
  c->device = device;
  c->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)(0.9 * (double)free_b);
  *out = c;
  return 0;
}

void cfdg_context_destroy(cfdg_context* ctx) {
  if (!ctx) return;
  bool free_now;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->destroyed = true;
    free_now = ctx->grids == 0;
  }
  if (free_now) delete ctx;
}

int cfdg_grid_open(cfdg_context* ctx, const cfdg_grid_desc* d, cfdg_grid** out) {
  if (!ctx || !d || !out) return fail(CFDG_ERR_INVALID, "null argument");
  *out = nullptr;
  CU(cudaSetDevice(ctx->device));
  auto G = std::make_unique<cfdg_grid>();
  G->ctx = ctx;
  HostGrid& h = G->h;
  for (int a = 0; a < 3; ++a) {
    h.n[a] = d->n[a];
    h.dx[a] = d->dx[a];
    h.periodic[a] = d->periodic[a] ? 1 : 0;
  }
  h.volume = d->volume;
  h.cells = (int64_t)d->n[0] * d->n[1] * d->n[2];
  h.faces = d->n_faces;
  if (h.cells <= 0 || h.faces <= 0 || !d->fluid || !d->face_kind || !d->face_lo || !d->face_hi || !d->face_area ||
      !d->face_distance || !d->component || (d->n_components && !d->anchored))
    return fail(CFDG_ERR_INVALID, "incomplete grid description");
  h.fluid.assign(d->fluid, d->fluid + h.cells);
  h.face_kind.assign(d->face_kind, d->face_kind + h.faces);
  h.face_lo.resize(h.faces);
  h.face_hi.resize(h.faces);
  for (int64_t f = 0; f < h.faces; ++f) {
    h.face_lo[f] = (int32_t)d->face_lo[f];
    h.face_hi[f] = (int32_t)d->face_hi[f];
  }
  h.face_area.assign(d->face_area, d->face_area + h.faces);
  h.face_distance.assign(d->face_distance, d->face_distance + h.faces);
  h.component.assign(d->component, d->component + h.cells);
  h.n_components = d->n_components;
  h.anchored.assign(d->anchored, d->anchored + d->n_components);
  std::string why = check_layout(h);
  if (!why.empty()) return fail(CFDG_ERR_INVALID, "grid description: " + why);
  G->preconditioner = d->preconditioner;
  G->precision = d->precision;
  if (G->preconditioner != CFDG_PRECOND_IC0 && G->preconditioner != CFDG_PRECOND_MULTIGRID)
    return fail(CFDG_ERR_INVALID, "unknown preconditioner");
  CU(cudaStreamCreateWithFlags(&G->own, cudaStreamNonBlocking));
  G->stream = G->own;
  CU(cudaEventCreate(&G->ev0));
  CU(cudaEventCreate(&G->ev1));
  Arena& A = G->arena;
  A.ctx = ctx;
  cudaStream_t s = G->stream;
  // Per-cell face flags.
  std::vector<uint16_t> flags(h.cells, 0);
  for (int a = 0; a < 3; ++a) {
    const int64_t* fd = h.face_dims[a];
    int64_t f = h.face_offset[a];
    for (int64_t k = 0; k < fd[2]; ++k)
      for (int64_t j = 0; j < fd[1]; ++j)
        for (int64_t i = 0; i < fd[0]; ++i, ++f) {
          uint8_t kind = h.face_kind[f];
          if (kind != INTERIOR && kind != OUTLET) continue;
          int lo = h.face_lo[f], hi = h.face_hi[f];
          unsigned base = kind == INTERIOR ? 0 : 6;
          if (lo >= 0) flags[lo] |= (uint16_t)(1u << (base + 2 * a + 1));  // upper face of lo
          if (hi >= 0 && !(kind == INTERIOR && lo == hi)) flags[hi] |= (uint16_t)(1u << (base + 2 * a));
          if (kind == INTERIOR && lo == hi) flags[lo] = (uint16_t)((flags[lo] & ~(1u << (2 * a + 1))) | (1u << (2 * a)));
        }
  }
  // Closed components (their cells, ascending).
  {
    std::vector<std::vector<int32_t>> members(h.n_components);
    for (int64_t c = 0; c < h.cells; ++c)
      if (h.component[c] >= 0 && !h.anchored[h.component[c]]) members[h.component[c]].push_back((int32_t)c);
    Csr groups;
    groups.off.push_back(0);
    for (auto& m : members)
      if (!m.empty()) {
        groups.col.insert(groups.col.end(), m.begin(), m.end());
        groups.off.push_back((int32_t)groups.col.size());
      }
    G->ncomp_groups = groups.rows();
    if (G->ncomp_groups)
      if (int e = upload_csr(A, groups, G->comp_groups, s)) return e;
  }
  std::vector<int32_t> lo32(h.face_lo.begin(), h.face_lo.end()), hi32(h.face_hi.begin(), h.face_hi.end());
  const int64_t N = h.cells, F = h.faces;
  int e = 0;
  if ((e = A.upload(&G->d_fluid, h.fluid, s)) || (e = A.upload(&G->d_flags, flags, s)) ||
      (e = A.upload(&G->d_kind, h.face_kind, s)) || (e = A.upload(&G->d_lo, lo32, s)) ||
      (e = A.upload(&G->d_hi, hi32, s)) || (e = A.alloc(&G->d_area, F)) || (e = A.alloc(&G->d_dist, F)) ||
      (e = A.alloc(&G->d_fw, F)) || (e = A.alloc(&G->x, N)) || (e = A.alloc(&G->r, N)) || (e = A.alloc(&G->z, N)) ||
      (e = A.alloc(&G->p, N)) || (e = A.alloc(&G->ap, N)) || (e = A.alloc(&G->bc, N)) || (e = A.alloc(&G->b, N)) ||
      (e = A.alloc(&G->terms, N)) || (e = A.alloc(&G->u, F)) || (e = A.alloc(&G->pp, N)) ||
      (e = A.alloc(&G->partials, MAX_BLOCKS)) || (e = A.alloc(&G->S, 1))) {
    A.release();
    return e;
  }
  CU(cudaMallocHost((void**)&G->hS, sizeof(Scalars)));
  CU(cudaMemsetAsync(G->S, 0, sizeof(Scalars), s));
  GridDev& g = G->g;
  for (int a = 0; a < 3; ++a) {
    g.n[a] = h.n[a];
    g.per[a] = h.periodic[a];
    g.face_off[a] = h.face_offset[a];
    for (int dd = 0; dd < 3; ++dd) g.fdim[a][dd] = (int)h.face_dims[a][dd];
    g.dx[a] = h.dx[a];
  }
  g.flags = G->d_flags;
  g.fw = G->d_fw;
  G->structured = !h.periodic[0] && !h.periodic[1] && !h.periodic[2] && h.n[0] >= 2 && h.n[1] >= 2 && h.n[2] >= 2;
  G->tiles_j = (h.n[1] + WTJ - 1) / WTJ;
  G->tiles_k = (h.n[2] + WTK - 1) / WTK;
  if ((e = A.alloc(&G->wave_sync, 2 + (size_t)G->tiles_j * G->tiles_k)) || (e = A.alloc(&G->wave_err, 1))) return e;
  CU(cudaMemsetAsync(G->wave_err, 0, sizeof(int), s));
  if ((e = refresh_weights(G.get()))) return e;
  CU(cudaStreamSynchronize(s));
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->grids += 1;
  }
  *out = G.release();
  return 0;
}

void cfdg_grid_close(cfdg_grid* G) {
  if (!G) return;
  cfdg_context* ctx = G->ctx;
  {
    std::lock_guard<std::mutex> lk(G->mu);
    cudaSetDevice(G->ctx->device);
    if (G->stream) cudaStreamSynchronize(G->stream);
    G->solo.reset();  // before the streams go: the batch may hold the grid's stream
    G->mixed.reset();
    reset_chunk(G);
    if (G->own) cudaStreamSynchronize(G->own);
    if (G->ic0) G->ic0->arena.release();
    if (G->mg) G->mg->arena.release();
    G->arena.release();
    if (G->hS) cudaFreeHost(G->hS);
    if (G->ev0) cudaEventDestroy(G->ev0);
    if (G->ev1) cudaEventDestroy(G->ev1);
    if (G->own) cudaStreamDestroy(G->own);
  }
  delete G;
  bool free_ctx;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->grids -= 1;
    free_ctx = ctx->destroyed && ctx->grids == 0;
  }
  if (free_ctx) delete ctx;
}

uint64_t cfdg_grid_device_bytes(const cfdg_grid* G) {
  if (!G) return 0;
  uint64_t b = G->arena.bytes;
  if (G->ic0) b += G->ic0->arena.bytes;
  if (G->mg) b += G->mg->arena.bytes;
  return b;
}

int cfdg_grid_update_faces(cfdg_grid* G, const double* area, const double* distance) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  if (area) G->h.face_area.assign(area, area + G->h.faces);
  if (distance) G->h.face_distance.assign(distance, distance + G->h.faces);
  if (int e = refresh_weights(G)) return e;
  reset_chunk(G);  // captured launches hold the weights by value
  G->faces_version += 1;
  G->mixed.reset();
  G->solo.reset();
  CU(cudaStreamSynchronize(G->stream));
  return 0;
}

int cfdg_grid_configure(cfdg_grid* G, int32_t preconditioner, int32_t precision) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  if (preconditioner != CFDG_PRECOND_IC0 && preconditioner != CFDG_PRECOND_MULTIGRID)
    return fail(CFDG_ERR_INVALID, "unknown preconditioner");
  if (preconditioner != G->preconditioner) reset_chunk(G);
  G->preconditioner = preconditioner;
  G->precision = precision;
  return 0;
}

int cfdg_grid_set_flow(cfdg_grid* G, const cfdg_flow_desc* flow) {
  if (int e = check_grid(G)) return e;
  if (!flow) return fail(CFDG_ERR_INVALID, "null flow");
  for (int a = 0; a < 3; ++a)
    if (flow->boundary[a] == 0 || flow->boundary[a] == 4)
      return fail(CFDG_ERR_UNSUPPORTED, "laminar stepping supports open, wall and slip boundaries");
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  if (!G->st_cu) {
    Arena& A = G->arena;
    if (int e = A.alloc(&G->st_cu, 3 * (size_t)G->h.cells)) return e;
    if (int e = A.alloc(&G->st_v, (size_t)G->h.faces)) return e;
    if (int e = A.alloc(&G->st_v2, (size_t)G->h.faces)) return e;
    if (int e = A.alloc(&G->st_p1, (size_t)G->h.cells)) return e;
  }
  for (int a = 0; a < 3; ++a) {
    G->flow_bnd[a] = flow->boundary[a];
    G->flow_size[a] = flow->size_m[a];
    G->flow_vel[a] = flow->velocity[a];
    G->flow_acc[a] = flow->acceleration[a];
  }
  G->flow_nu = flow->viscosity;
  G->has_flow = true;
  return 0;
}

int cfdg_step_device(cfdg_grid* G, double* d_u, double* d_p, double dt, double tol, uint64_t max_iter,
                     cfdg_poll_fn poll, void* poll_ctx, cfdg_info* info) {
  if (int e = check_grid(G)) return e;
  if (!d_u || !d_p) return fail(CFDG_ERR_INVALID, "null u or p");
  std::lock_guard<std::mutex> lk(G->mu);
  if (!G->has_flow) return fail(CFDG_ERR_INVALID, "cfdg_grid_set_flow has not been called for this grid");
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  Poller P;
  P.fn = poll;
  P.ctx = poll_ctx;
  const FlowDev D = flow_dev(G);
  const size_t N = G->h.cells;
  cfdg_info i1{}, i2{};
  // Stage outputs live in the grid's buffers until the step succeeds (the caller's u and
  // p stay unchanged on any error, as solver::step builds the next state beside it).
  CU(cudaMemcpyAsync(G->st_p1, d_p, N * 8, cudaMemcpyDeviceToDevice, s));
  if (int e = flow_stage(G, D, d_u, G->st_v, G->st_p1, dt, tol, max_iter, P, &i1)) return e;
  if (int e = flow_stage(G, D, G->st_v, G->st_v2, G->st_p1, dt, tol, max_iter, P, &i2)) return e;
  k_ssprk_combine<<<grid_blocks((int)std::min<long long>(G->h.faces, 1LL << 30)), BLOCK, 0, s>>>(D, d_u, G->st_v2,
                                                                                                 G->h.faces);
  tick(G);
  CU(cudaMemcpyAsync(d_p, G->st_p1, N * 8, cudaMemcpyDeviceToDevice, s));
  CU(cudaStreamSynchronize(s));
  if (info) {
    *info = i2;
    info->iterations = i1.iterations + i2.iterations;
    info->work_units = i1.work_units + i2.work_units;
    info->operator_applications = i1.operator_applications + i2.operator_applications;
    info->preconditioner_applications = i1.preconditioner_applications + i2.preconditioner_applications;
    info->true_residual_checks = i1.true_residual_checks + i2.true_residual_checks;
    info->device_seconds = i1.device_seconds + i2.device_seconds;
  }
  return 0;
}

// y (inverse: 1/y) as a power-of-two factor when y is a positive normal power of two whose
// reciprocal is normal too (a product with 1/y is then the quotient by y, rounding included).
static Pow2 pow2_of(double y, bool inverse) {
  Pow2 p{0.0, 0, 0};
  if (!(y > 0.0) || !std::isnormal(y)) return p;
  int e = 0;
  if (std::frexp(y, &e) != 0.5) return p;
  const int k = inverse ? 1 - e : e - 1;
  const double v = std::ldexp(1.0, k);
  if (!std::isnormal(v) || !std::isnormal(1.0 / v)) return p;
  return Pow2{v, k, 1};
}

// mode 0: one SSPRK2 step; 1: the step and its budget increments into d_budget (device,
// three doubles); 2: the current rates of d_c only, into the host array rates.
static int scalar_impl(cfdg_grid* G, const double* d_u, double* d_c, const double* d_diff, const double* d_source,
                       double dt, int mode, double* d_budget, double* rates) {
  if (int e = check_grid(G)) return e;
  if (!d_u || !d_c || !d_diff || !d_source) return fail(CFDG_ERR_INVALID, "null array");
  if ((mode == 1 && !d_budget) || (mode == 2 && !rates)) return fail(CFDG_ERR_INVALID, "null budget or rates");
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  for (int a = 0; a < 3; ++a)
    if (G->h.periodic[a]) return fail(CFDG_ERR_UNSUPPORTED, "scalar transport on the device: periodic axes");
  const int N = (int)G->h.cells;
  if (!G->st_sc) {
    if (int e = G->arena.alloc(&G->st_sc, (size_t)N)) return e;
  }
  ScalarDev D{};
  for (int a = 0; a < 3; ++a) {
    D.n[a] = G->h.n[a];
    D.face_off[a] = G->g.face_off[a];
    for (int d = 0; d < 3; ++d) D.fdim[a][d] = G->g.fdim[a][d];
  }
  D.volume = G->h.volume;
  D.inv_volume = pow2_of(G->h.volume, true);
  D.kind = G->d_kind;
  D.fluid = G->d_fluid;
  D.lo = G->d_lo;
  D.hi = G->d_hi;
  D.area = G->d_area;
  D.dist = G->d_dist;
  for (int a = 0; a < 3; ++a)
    for (int t = 0; t < 3; ++t) {
      D.area_k[a][t] = G->sc_area[a][t];
      D.dist_k[a][t] = G->sc_dist[a][t];
      D.area_p[a][t] = pow2_of(G->sc_area[a][t], false);
      D.inv_dist_p[a][t] = pow2_of(G->sc_dist[a][t], true);
    }
  double* stage = G->st_sc;
  cudaStream_t s = G->stream;
  if (mode != 0 && !G->sc_part) {
    if (int e = G->arena.alloc(&G->sc_part, (size_t)2 * 3 * SR_BLOCKS + 3)) return e;
  }
  if (mode == 2) {
    k_scalar_rates<<<SR_BLOCKS, SR_THREADS, 0, s>>>(D, d_c, d_u, d_diff, d_source, N, G->sc_part, G->sc_muscl);
    double* dr = G->sc_part + 6 * SR_BLOCKS;
    k_scalar_budget<<<1, 32, 0, s>>>(G->sc_part, nullptr, D.volume, 0.0, nullptr, dr);
    count(2);
    CU(cudaMemcpyAsync(rates, dr, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    return 0;
  }
  const int zs = scalar_zsplit(G->h.n, G->ctx->device);
  const dim3 blk(STX, STY), grd((G->h.n[0] + STX - 1) / STX, (G->h.n[1] + STY - 1) / STY, (G->h.n[2] + zs - 1) / zs);
  // The budget's rates: of c before the second pass overwrites it, and of the stage.
  auto rates_of_stages = [&]() {
    if (mode != 1) return;
    k_scalar_rates<<<SR_BLOCKS, SR_THREADS, 0, s>>>(D, d_c, d_u, d_diff, d_source, N, G->sc_part, G->sc_muscl);
    k_scalar_rates<<<SR_BLOCKS, SR_THREADS, 0, s>>>(D, stage, d_u, d_diff, d_source, N, G->sc_part + 3 * SR_BLOCKS,
                                                    G->sc_muscl);
    count(2);
  };
  bool p2 = G->sc_uniform && D.inv_volume.ok;
  for (int a = 0; a < 3; ++a)
    for (int t = 0; t < 3; ++t)
      if (G->sc_used[a][t]) p2 = p2 && D.area_p[a][t].ok && D.inv_dist_p[a][t].ok;
  auto passes = [&](auto uni, auto p2c, auto muscl) {
    constexpr bool U = decltype(uni)::value, P = decltype(p2c)::value, M = decltype(muscl)::value;
    k_scalar_pass<U, P, M, 0><<<grd, blk, 0, s>>>(D, d_c, stage, d_u, d_diff, d_source, dt, zs); tick(G);
    rates_of_stages();
    k_scalar_pass<U, P, M, 1><<<grd, blk, 0, s>>>(D, d_c, stage, d_u, d_diff, d_source, dt, zs); tick(G);
  };
  using T = std::true_type;
  using F = std::false_type;
  if (G->sc_muscl) {
    if (p2) passes(T{}, T{}, T{});
    else if (G->sc_uniform) passes(T{}, F{}, T{});
    else passes(F{}, F{}, T{});
  } else {
    if (p2) passes(T{}, T{}, F{});
    else if (G->sc_uniform) passes(T{}, F{}, F{});
    else passes(F{}, F{}, F{});
  }
  if (mode == 1) {
    k_scalar_budget<<<1, 32, 0, s>>>(G->sc_part, G->sc_part + 3 * SR_BLOCKS, D.volume, dt, d_budget, nullptr);
    count();
  }
  CU(cudaGetLastError());
  return 0;
}

int cfdg_scalar_step_device(cfdg_grid* G, const double* d_u, double* d_c, const double* d_diff, const double* d_source,
                            double dt) {
  return scalar_impl(G, d_u, d_c, d_diff, d_source, dt, 0, nullptr, nullptr);
}

int cfdg_grid_set_advection(cfdg_grid* G, int32_t muscl) {
  if (int e = check_grid(G)) return e;
  if (muscl != 0 && muscl != 1) return fail(CFDG_ERR_INVALID, "advection is 0 (linear upwind) or 1 (MUSCL)");
  std::lock_guard<std::mutex> lk(G->mu);
  G->sc_muscl = muscl;
  return 0;
}

int cfdg_scalar_step_budget(cfdg_grid* G, const double* d_u, double* d_c, const double* d_diff, const double* d_source,
                            double dt, double* d_budget) {
  return scalar_impl(G, d_u, d_c, d_diff, d_source, dt, 1, d_budget, nullptr);
}

int cfdg_scalar_rates(cfdg_grid* G, const double* d_u, const double* d_c, const double* d_diff, const double* d_source,
                      double* rates) {
  return scalar_impl(G, d_u, const_cast<double*>(d_c), d_diff, d_source, 0.0, 2, nullptr, rates);
}

// solver.rs:1035-1037: a receptor's value is Σ c[cell] w over its weights in order, an
// Iterator::sum (from -0.0); one thread per receptor keeps that order.
__global__ void k_receptors(const int64_t* __restrict__ off, const int32_t* __restrict__ cell,
                            const double* __restrict__ w, const double* __restrict__ c, double* __restrict__ out,
                            int n) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double acc = -0.0;
  for (long long k = off[r]; k < off[r + 1]; ++k) acc = acc + c[cell[k]] * w[k];
  out[r] = acc;
}

int cfdg_receptors_set(cfdg_grid* G, int32_t n, const int64_t* offsets, const int64_t* cells,
                       const double* weights) {
  if (int e = check_grid(G)) return e;
  if (n < 0 || (n > 0 && (!offsets || !cells || !weights))) return fail(CFDG_ERR_INVALID, "receptor arrays");
  if (n > 0 && offsets[0] != 0) return fail(CFDG_ERR_INVALID, "receptor offsets must start at 0");
  for (int32_t r = 0; r < n; ++r)
    if (offsets[r + 1] <= offsets[r]) return fail(CFDG_ERR_INVALID, "a receptor has no weight");
  const int64_t m = n > 0 ? offsets[n] : 0;
  for (int64_t k = 0; k < m; ++k)
    if (cells[k] < 0 || cells[k] >= G->h.cells) return fail(CFDG_ERR_INVALID, "a receptor cell is outside the grid");
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  // Grown arrays come from the grid's arena (released with the grid); smaller sets reuse them.
  if (n + 1 > G->rc_cap_n) {
    if (int e = G->arena.alloc(&G->rc_off, (size_t)n + 1)) return e;
    G->rc_cap_n = n + 1;
  }
  if (m > G->rc_cap_entries) {
    if (int e = G->arena.alloc(&G->rc_cell, (size_t)m)) return e;
    if (int e = G->arena.alloc(&G->rc_w, (size_t)m)) return e;
    G->rc_cap_entries = m;
  }
  std::vector<int32_t> c32(cells, cells + m);
  cudaStream_t s = G->stream;
  if (n > 0) {
    CU(cudaMemcpyAsync(G->rc_off, offsets, ((size_t)n + 1) * 8, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(G->rc_cell, c32.data(), (size_t)m * 4, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(G->rc_w, weights, (size_t)m * 8, cudaMemcpyHostToDevice, s));
  }
  CU(cudaStreamSynchronize(s));  // the host arrays may go away after the return
  G->rc_n = n;
  return 0;
}

int cfdg_receptors_sample(cfdg_grid* G, const double* d_c, double* d_out) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  if (G->rc_n == 0) return 0;
  if (!d_c || !d_out) return fail(CFDG_ERR_INVALID, "null array");
  CU(cudaSetDevice(G->ctx->device));
  const int n = G->rc_n;
  k_receptors<<<(n + 127) / 128, 128, 0, G->stream>>>(G->rc_off, G->rc_cell, G->rc_w, d_c, d_out, n); tick(G);
  CU(cudaGetLastError());
  return 0;
}

int cfdg_debug_momentum_update(cfdg_grid* G, const double* u, const double* p, double dt, double* out) {
  if (int e = check_grid(G)) return e;
  if (!u || !p || !out) return fail(CFDG_ERR_INVALID, "null array");
  std::lock_guard<std::mutex> lk(G->mu);
  if (!G->has_flow) return fail(CFDG_ERR_INVALID, "cfdg_grid_set_flow has not been called for this grid");
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  const size_t N = G->h.cells, F = G->h.faces;
  CU(cudaMemcpyAsync(G->st_v2, u, F * 8, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(G->st_p1, p, N * 8, cudaMemcpyHostToDevice, s));
  const FlowDev D = flow_dev(G);
  k_cell_velocity<<<grid_blocks((int)N), BLOCK, 0, s>>>(D, G->st_v2, G->st_cu, (int)N); tick(G);
  k_momentum_update<<<grid_blocks((int)std::min<size_t>(F, 1u << 30)), BLOCK, 0, s>>>(D, G->st_v2, G->st_p1, G->st_cu, dt,
                                                                                     G->st_v, (long long)F, (int)N);
  tick(G);
  CU(cudaMemcpyAsync(out, G->st_v, F * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

int cfdg_grid_set_cycle(cfdg_grid* G, int32_t nu_fine, int32_t nu_coarse) {
  if (int e = check_grid(G)) return e;
  if (nu_fine < 1 || nu_fine > 4 || nu_coarse < 1 || nu_coarse > 4)
    return fail(CFDG_ERR_INVALID, "sweep counts must be 1..4");
  std::lock_guard<std::mutex> lk(G->mu);
  if (G->mx_nu0 != nu_fine || G->mx_nuc != nu_coarse) G->solo.reset();
  G->mx_nu0 = nu_fine;
  G->mx_nuc = nu_coarse;
  return 0;
}

int cfdg_grid_set_sweep_tile(cfdg_grid* G, int32_t rows, int32_t stages) {
  if (int e = check_grid(G)) return e;
  const bool automatic = rows == 0 && stages == 0;
  if (!automatic && (!(rows == 8 || rows == 16 || rows == 32) || stages < 2 || stages > 8))
    return fail(CFDG_ERR_INVALID, "sweep tile: rows must be 8, 16 or 32 and stages 2..8 (or both 0)");
  std::lock_guard<std::mutex> lk(G->mu);
  if (G->mx_sweep_rows != rows || G->mx_sweep_stages != stages) G->solo.reset();
  G->mx_sweep_rows = rows;
  G->mx_sweep_stages = stages;
  return 0;
}

int cfdg_grid_set_coarse_scale(cfdg_grid* G, double alpha) {
  if (int e = check_grid(G)) return e;
  if (!(alpha > 0.0 && alpha < 2.0)) return fail(CFDG_ERR_INVALID, "the coarse-correction scale must lie in (0, 2)");
  std::lock_guard<std::mutex> lk(G->mu);
  if (G->mx_alpha != (float)alpha) {
    G->mixed.reset();  // the case state holds the scaled prolongation
    G->solo.reset();
  }
  G->mx_alpha = (float)alpha;
  return 0;
}

int cfdg_grid_set_coarse_layout(cfdg_grid* G, int32_t bins) {
  if (int e = check_grid(G)) return e;
  if (bins != 0 && bins != 1) return fail(CFDG_ERR_INVALID, "the coarse layout is 0 (aggregate order) or 1 (bin grid)");
  std::lock_guard<std::mutex> lk(G->mu);
  if (G->mx_bins != bins) {
    G->mixed.reset();  // the case state holds the first coarse level's numbering
    G->solo.reset();
  }
  G->mx_bins = bins;
  return 0;
}

int cfdg_project_device(cfdg_grid* G, double* d_u, double* d_p, double dt, double tol, uint64_t max_iter,
                        cfdg_poll_fn poll, void* poll_ctx, cfdg_info* info) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  Poller P;
  P.fn = poll;
  P.ctx = poll_ctx;
  return project_device(G, d_u, d_p, dt, tol, max_iter, P, info);
}

int cfdg_project(cfdg_grid* G, double* u, double* p, double dt, double tol, uint64_t max_iter, cfdg_poll_fn poll,
                 void* poll_ctx, cfdg_info* info) {
  if (int e = check_grid(G)) return e;
  if (!u || !p) return fail(CFDG_ERR_INVALID, "null u or p");
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  CU(cudaMemcpyAsync(G->u, u, G->h.faces * 8, cudaMemcpyHostToDevice, s));
  CU(cudaMemcpyAsync(G->pp, p, G->h.cells * 8, cudaMemcpyHostToDevice, s));
  Poller P;
  P.fn = poll;
  P.ctx = poll_ctx;
  if (int e = project_device(G, G->u, G->pp, dt, tol, max_iter, P, info)) return e;
  CU(cudaMemcpyAsync(u, G->u, G->h.faces * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(p, G->pp, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

int cfdg_solve_scaled(cfdg_grid* G, const double* b, const double* roundoff_scale, double tol, uint64_t max_iter,
                      cfdg_poll_fn poll, void* poll_ctx, double* x, cfdg_info* info) {
  if (int e = check_grid(G)) return e;
  if (!b || !x) return fail(CFDG_ERR_INVALID, "null b or x");
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  CU(cudaMemcpyAsync(G->b, b, G->h.cells * 8, cudaMemcpyHostToDevice, s));
  if (roundoff_scale) CU(cudaMemcpyAsync(G->terms, roundoff_scale, G->h.cells * 8, cudaMemcpyHostToDevice, s));
  Poller P;
  P.fn = poll;
  P.ctx = poll_ctx;
  if (int e = solve_device(G, roundoff_scale != nullptr, tol, max_iter, P, info)) return e;
  CU(cudaMemcpyAsync(x, G->x, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

int cfdg_apply(cfdg_grid* G, const double* x, double* y) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  CU(cudaMemcpyAsync(G->p, x, G->h.cells * 8, cudaMemcpyHostToDevice, s));
  launch_apply(G, G->p, G->ap);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(y, G->ap, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

int cfdg_center_nullspaces(cfdg_grid* G, double* x) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  CU(cudaMemcpyAsync(G->z, x, G->h.cells * 8, cudaMemcpyHostToDevice, s));
  launch_center(G, G->comp_groups, G->ncomp_groups, G->z, nullptr);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(x, G->z, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

int cfdg_multigrid_stats_json(cfdg_grid* G, char* buf, size_t cap) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->stats_mu);
  if (G->stats_json.empty()) return CFDG_PENDING;
  if (!buf || cap <= G->stats_json.size()) return fail(CFDG_ERR_INVALID, "buffer too small");
  std::memcpy(buf, G->stats_json.c_str(), G->stats_json.size() + 1);
  return 0;
}

int cfdg_debug_precondition(cfdg_grid* G, const double* r, double* z) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  Poller P;
  if (int e = prepare_preconditioner(G, P, nullptr)) return e;
  cudaStream_t s = G->stream;
  CU(cudaMemcpyAsync(G->r, r, G->h.cells * 8, cudaMemcpyHostToDevice, s));
  if (G->preconditioner == CFDG_PRECOND_MULTIGRID) launch_vcycle(G, G->r, G->z, nullptr);
  else launch_sweep_ic0(G, nullptr);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(z, G->z, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return check_wave(G);
}

int cfdg_debug_wave_stall(cfdg_grid* G, int32_t hold_tile, int64_t spin_limit) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  if (!G->structured) return fail(CFDG_ERR_UNSUPPORTED, "the grid has no wavefront sweeps (a periodic axis)");
  if (hold_tile < -1 || hold_tile >= G->tiles_j * G->tiles_k)
    return fail(CFDG_ERR_INVALID, "hold_tile must be -1 or a tile of the grid's wavefront");
  if (spin_limit < 1 || spin_limit > WAVE_SPIN_LIMIT)
    return fail(CFDG_ERR_INVALID, "spin_limit must lie in 1 .. " + std::to_string(WAVE_SPIN_LIMIT));
  G->wave_hold_tile = hold_tile;
  G->wave_spin_limit = spin_limit;
  reset_chunk(G);  // captured iteration chunks hold the sweeps' arguments
  return 0;
}

int cfdg_residual_norm_noalloc(cfdg_grid* G, const double* d_x, const double* d_b, double* d_out, void* stream) {
  if (int e = check_grid(G)) return e;
  if (!d_x || !d_b || !d_out) return fail(CFDG_ERR_INVALID, "null device pointer");
  const int64_t N = G->h.cells;
  if (N > (int64_t)NOALLOC_MAX_BLOCKS * NOALLOC_CHUNK)
    return fail(CFDG_ERR_INVALID, "cfdg_residual_norm_noalloc: the grid has " + std::to_string(N) +
                                      " cells; the no-allocation scratch covers at most " +
                                      std::to_string((int64_t)NOALLOC_MAX_BLOCKS * NOALLOC_CHUNK));
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  double* scratch = nullptr;
  if (int e = noalloc_scratch(G->ctx->device, &scratch)) return e;
  cudaStream_t s = stream ? (cudaStream_t)stream : G->stream;
  // The counter must start at zero; the partial sums are all rewritten by each call.
  CU(cudaMemsetAsync(scratch + 2 * NOALLOC_MAX_BLOCKS, 0, sizeof(unsigned), s));
  const int nb = (int)((N + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK);
  if (G->uniform) k_residual_norm_noalloc<true><<<nb, BLOCK, 0, s>>>(G->g, d_x, d_b, (int)N, scratch, d_out);
  else k_residual_norm_noalloc<false><<<nb, BLOCK, 0, s>>>(G->g, d_x, d_b, (int)N, scratch, d_out);
  count();
  CU(cudaGetLastError());
  return 0;
}

int cfdg_grid_set_stream(cfdg_grid* G, void* stream) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  CU(cudaStreamSynchronize(G->stream));
  G->stream = stream ? (cudaStream_t)stream : G->own;
  return 0;
}

uint64_t cfdg_launch_count(void) { return g_launches.load(); }

int cfdg_debug_time_kernel(cfdg_grid* G, int32_t which, int32_t reps, double* ms_per_launch,
                           double* algorithmic_bytes) {
  if (int e = check_grid(G)) return e;
  if (reps < 1) return fail(CFDG_ERR_INVALID, "reps must be positive");
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  Poller P;
  const double N = (double)G->h.cells;
  double nfluid = 0;
  for (auto v : G->h.fluid) nfluid += v;
  double bytes = 0;
  auto run = [&]() {
    switch (which) {
      case 0:
        launch_apply(G, G->p, G->ap);
        break;
      case 1:
        launch_gs(G, G->mg->levels[0], false, nullptr, G->mg->full0);
        break;
      case 2:
        launch_sweep_ic0(G, nullptr);
        break;
      default:
        launch_vcycle(G, G->r, G->z, nullptr);
        break;
    }
  };
  if (which == 0) {
    bytes = 18.0 * N;  // read x, read the u16 face flags, write y
  } else if (which == 1 || which == 3) {
    if (G->preconditioner != CFDG_PRECOND_MULTIGRID) return fail(CFDG_ERR_INVALID, "needs the multigrid preconditioner");
    if (int e = prepare_preconditioner(G, P, nullptr)) return e;
    bytes = which == 1 ? 25.0 * nfluid : 151.0 * nfluid;  // per-unit figures of the algorithm
  } else {
    if (G->preconditioner != CFDG_PRECOND_IC0) return fail(CFDG_ERR_INVALID, "needs the IC(0) preconditioner");
    if (int e = prepare_preconditioner(G, P, nullptr)) return e;
    bytes = 58.0 * N;  // forward 25 N + backward 33 N
  }
  k_fill<<<grid_blocks(G->h.cells), BLOCK, 0, G->stream>>>(G->p, 1.0, (int)G->h.cells, nullptr); tick(G);
  k_fill<<<grid_blocks(G->h.cells), BLOCK, 0, G->stream>>>(G->r, 1.0, (int)G->h.cells, nullptr); tick(G);
  run();
  run();
  CU(cudaEventRecord(G->ev0, G->stream));
  for (int i = 0; i < reps; ++i) run();
  CU(cudaEventRecord(G->ev1, G->stream));
  CU(cudaEventSynchronize(G->ev1));
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, G->ev0, G->ev1));
  if (ms_per_launch) *ms_per_launch = ms / reps;
  if (algorithmic_bytes) *algorithmic_bytes = bytes;
  return 0;
}

int cfdg_debug_projection_rhs(cfdg_grid* G, const double* u, double dt, double* b, double* terms) {
  if (int e = check_grid(G)) return e;
  std::lock_guard<std::mutex> lk(G->mu);
  CU(cudaSetDevice(G->ctx->device));
  cudaStream_t s = G->stream;
  CU(cudaMemcpyAsync(G->u, u, G->h.faces * 8, cudaMemcpyHostToDevice, s));
  k_projection_rhs<<<grid_blocks(G->h.cells), BLOCK, 0, s>>>(G->g, G->d_fluid, G->u, dt, G->b, G->terms,
                                                             (int)G->h.cells); tick(G);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(b, G->b, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaMemcpyAsync(terms, G->terms, G->h.cells * 8, cudaMemcpyDeviceToHost, s));
  CU(cudaStreamSynchronize(s));
  return 0;
}

}  // extern "C"
