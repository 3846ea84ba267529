// Pipelined wavefront sweeps over the structured fine level (one launch per sweep).
//
// A lexicographic sweep over the 7-point pattern in natural cell order (IC(0)
// forward/backward substitution, pressure.rs:225-240; Gauss-Seidel,
// multigrid.rs:272-281 / masked.rs:158-172) updates cell (i,j,k) after (i-1,j,k),
// (i,j-1,k) and (i,j,k-1). Each CTA owns a TJ x TK tile of x-pencils; thread (tj,tk)
// walks its pencil and handles cell i at local step s = i + tj + tk, so the cells of
// one step lie on a hyperplane of the tile. Values of the previous step come from
// shared memory (one barrier per step), the pencil's own predecessor from a register.
// Tiles depend on their (J-1,K) and (J,K-1) neighbours only through the boundary
// pencils: a tile publishes how many steps it has completed (release store, one step
// behind so that a single barrier per step orders it after the steps' stores) and a
// consumer at step s waits for s + TJ (resp. s + TK) of its producer (acquire load,
// bounded spin). Tiles are taken in a topological order from an atomic ticket, so a
// CTA only ever waits for tiles already held by running CTAs.
//
// Every cell is computed with the same operations in the same order as the
// reference's natural-order loop, so the result is bit-identical to it. Backward
// sweeps run the same machinery mirrored (i, j, k descending).
#pragma once
#include "plain_kernels.cuh"

namespace cfdg {

constexpr int WTJ = 8, WTK = 8;  // tile of pencils per CTA

enum WaveMode { IC0_FWD = 0, IC0_BWD = 1, GS_FWD = 2, GS_BWD = 3 };

struct WaveArgs {
  int n[3];
  int tiles_j, tiles_k;
  const uint16_t* flags;  // interior/outlet face bits per cell (GridDev::flags layout)
  const double* in;       // r (IC0_FWD) or rhs (GS_*)
  double* x;              // z (IC0_*; IC0_BWD in place) or x (GS_*, in place)
  const double* diag;     // IC(0) factor diagonal, or the level-0 matrix diagonal
  const double* lx;       // IC(0): lower coefficient of each row towards (i-1), (j-1), (k-1)
  const double* ly;
  const double* lz;
  // Gauss-Seidel weights: uniform per axis, or per face.
  int uniform;
  double w_in[3];
  const double* fw;
  long long face_off[3];
  int fdim[3][3];
  int* sync;        // [0] ticket, [1] abort, [2 ..] progress per tile
  int* error;       // persistent: set to 1 when a wait gave up
  const Scalars* S;
  long long spin_limit;  // polls before a wait gives up (WAVE_SPIN_LIMIT)
  int hold_tile;         // -1; a test of the bounded waits names a tile that never publishes
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int MODE>
__global__ void __launch_bounds__(WTJ* WTK) k_wave(WaveArgs A) {
  constexpr bool BWD = (MODE == IC0_BWD || MODE == GS_BWD);
  __shared__ double sh[2][WTK][WTJ];
  __shared__ int tile_s, bail_s;
  __shared__ int seen_j, seen_k;
  if (A.S && A.S->done) return;
  const int nx = A.n[0], ny = A.n[1], nz = A.n[2];
  const long long sx = 1, sy = nx, sz = (long long)nx * ny;
  const int tj = threadIdx.x % WTJ, tk = threadIdx.x / WTJ;
  if (threadIdx.x == 0) {
    tile_s = atomicAdd(&A.sync[0], 1);
    bail_s = 0;
    seen_j = 0;
    seen_k = 0;
  }
  __syncthreads();
  const int t = tile_s;
  int J = t % A.tiles_j, K = t / A.tiles_j;  // row-major tiles: producers have smaller tickets
  if (BWD) {
    J = A.tiles_j - 1 - J;
    K = A.tiles_k - 1 - K;
  }
  const int j = J * WTJ + tj, k = K * WTK + tk;
  const bool lane_ok = j < ny && k < nz;
  // Distance of this pencil from the tile's first pencil in sweep order.
  const int dj = BWD ? WTJ - 1 - tj : tj;
  const int dk = BWD ? WTK - 1 - tk : tk;
  const int nsteps = nx + WTJ + WTK - 2;
  // Producers: the tiles before this one in sweep order along j and along k.
  const int pj = BWD ? (J + 1 < A.tiles_j ? t - 1 : -1) : (J > 0 ? t - 1 : -1);
  const int pk = BWD ? (K + 1 < A.tiles_k ? t - A.tiles_j : -1) : (K > 0 ? t - A.tiles_j : -1);
  int* progress = A.sync + 2;
  double prev = 0.0;  // this pencil's value at the previous cell in sweep order
  for (int s = 0; s < nsteps; ++s) {
    if (threadIdx.x == 0) {
      // Every thread passed the barrier of step s - 1, so steps 0 .. s - 2 are stored.
      if (s > 1 && t != A.hold_tile) {
        __threadfence();
        st_release(&progress[t], s - 1);
      }
      // Boundary pencils at step s need step s + TJ - 1 (s + TK - 1) of the producers.
      const int need_j = min(s + WTJ, nsteps), need_k = min(s + WTK, nsteps);
      long long spins = 0;
      if (pj >= 0 && seen_j < need_j) {
        int v;
        while ((v = ld_acquire(&progress[pj])) < need_j) {
          if (++spins > A.spin_limit || ld_acquire(&A.sync[1])) {
            bail_s = 1;
            break;
          }
        }
        seen_j = v;
      }
      if (!bail_s && pk >= 0 && seen_k < need_k) {
        int v;
        while ((v = ld_acquire(&progress[pk])) < need_k) {
          if (++spins > A.spin_limit || ld_acquire(&A.sync[1])) {
            bail_s = 1;
            break;
          }
        }
        seen_k = v;
      }
      if (bail_s) {
        atomicExch(&A.sync[1], 1);
        atomicExch(A.error, 1);
      }
      __threadfence();
    }
    __syncthreads();
    if (bail_s) return;
    const int step_i = s - dj - dk;
    const double* cur_prev = &sh[(s + 1) & 1][0][0];
    double* cur = &sh[s & 1][0][0];
    if (lane_ok && step_i >= 0 && step_i < nx) {
      const int i = BWD ? nx - 1 - step_i : step_i;
      const long long c = ((long long)k * ny + j) * nx + i;
      const unsigned fl = A.flags[c];
      // Neighbour values already updated in this sweep ("new") along x, y, z.
      const bool has_ny = BWD ? j + 1 < ny : j > 0;
      const bool has_nz = BWD ? k + 1 < nz : k > 0;
      const bool in_tile_y = BWD ? tj + 1 < WTJ : tj > 0;
      const bool in_tile_z = BWD ? tk + 1 < WTK : tk > 0;
      const long long cy = BWD ? c + sy : c - sy, cz = BWD ? c + sz : c - sz;
      double newx = prev;
      double newy = 0.0, newz = 0.0;
      if (has_ny) newy = in_tile_y ? cur_prev[tk * WTJ + (BWD ? tj + 1 : tj - 1)] : __ldcg(&A.x[cy]);
      if (has_nz) newz = in_tile_z ? cur_prev[(BWD ? tk + 1 : tk - 1) * WTJ + tj] : __ldcg(&A.x[cz]);
      double v;
      if (MODE == IC0_FWD) {
        // Ascending columns: (k-1), (j-1), (i-1).
        v = A.in[c];
        if (fl & (1u << 4)) v = v - A.lz[c] * newz;
        if (fl & (1u << 2)) v = v - A.ly[c] * newy;
        if (fl & (1u << 0)) v = v - A.lx[c] * newx;
        v = v / A.diag[c];
      } else if (MODE == IC0_BWD) {
        // Rows (k+1), (j+1), (i+1) in descending order, each with its coefficient
        // towards this cell.
        v = __ldcg(&A.x[c]);
        if (fl & (1u << 5)) v = v - A.lz[c + sz] * newz;
        if (fl & (1u << 3)) v = v - A.ly[c + sy] * newy;
        if (fl & (1u << 1)) v = v - A.lx[c + sx] * newx;
        v = v / A.diag[c];
      } else {
        const double d = A.diag[c];
        if (d == 0.0) {
          v = 0.0;  // a cell with no faces in the operator: a sealed singleton, or a solid cell
        } else {
          // Row order x-lo, x-hi, y-lo, y-hi, z-lo, z-hi; entries are -w, and
          // v - (-w) x == v + w x exactly.
          double w[6];
          if (A.uniform) {
#pragma unroll
            for (int a = 0; a < 3; ++a) w[2 * a] = w[2 * a + 1] = A.w_in[a];
          } else {
            const int q[3] = {i, j, k};
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              int p[3] = {q[0], q[1], q[2]};
              w[2 * a] = A.fw[A.face_off[a] + ((long long)p[2] * A.fdim[a][1] + p[1]) * A.fdim[a][0] + p[0]];
              p[a] += 1;
              w[2 * a + 1] = A.fw[A.face_off[a] + ((long long)p[2] * A.fdim[a][1] + p[1]) * A.fdim[a][0] + p[0]];
            }
          }
          // Lower neighbours are "new" in a forward sweep, upper ones in a backward sweep.
          const double xlo = BWD ? (i > 0 ? __ldcg(&A.x[c - sx]) : 0.0) : newx;
          const double xhi = BWD ? newx : (i + 1 < nx ? __ldcg(&A.x[c + sx]) : 0.0);
          const double ylo = BWD ? (j > 0 ? __ldcg(&A.x[c - sy]) : 0.0) : newy;
          const double yhi = BWD ? newy : (j + 1 < ny ? __ldcg(&A.x[c + sy]) : 0.0);
          const double zlo = BWD ? (k > 0 ? __ldcg(&A.x[c - sz]) : 0.0) : newz;
          const double zhi = BWD ? newz : (k + 1 < nz ? __ldcg(&A.x[c + sz]) : 0.0);
          v = A.in[c];
          if (fl & (1u << 0)) v = v + w[0] * xlo;
          if (fl & (1u << 1)) v = v + w[1] * xhi;
          if (fl & (1u << 2)) v = v + w[2] * ylo;
          if (fl & (1u << 3)) v = v + w[3] * yhi;
          if (fl & (1u << 4)) v = v + w[4] * zlo;
          if (fl & (1u << 5)) v = v + w[5] * zhi;
          v = v / d;
        }
      }
      A.x[c] = v;
      cur[tk * WTJ + tj] = v;
      prev = v;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && t != A.hold_tile) {
    __threadfence();
    st_release(&progress[t], nsteps);
  }
}

}  // namespace cfdg
