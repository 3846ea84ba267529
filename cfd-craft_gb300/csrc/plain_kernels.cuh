// FP64 kernels of the plain (parity) form of the pressure projection.
//
// This translation unit is compiled with -fmad=false: like the reference (Rust
// never contracts a*b+c), every product and sum is rounded on its own, so the
// operator, the IC(0) substitutions, the Gauss-Seidel sweeps, the transfers and
// the face correction reproduce the reference bit for bit for the same inputs.
// Only the dot products and gauge means (tree reductions) differ from the
// reference's sequential sums, in the last bits.
#pragma once
#include <cstdint>

namespace cfdg {

constexpr int BLOCK = 256;
constexpr int MAX_BLOCKS = 152 * 8;  // fixed reduction width: deterministic sums
constexpr long long WAVE_SPIN_LIMIT = 1LL << 22;  // polls of a wavefront wait: about a second

// Per-cell face flags: bit (2a + side) interior face, bit (6 + 2a + side) outlet
// face, side 0 = lower face, 1 = upper face of axis a.
struct GridDev {
  int n[3];
  int per[3];
  long long face_off[3];
  int fdim[3][3];
  double dx[3];
  double w_in[3], w_out[3];  // uniform interior / outlet weight per axis
  const uint16_t* flags;     // [N]
  const double* fw;          // [F] per-face weight area/(distance*volume)
};

// Device-side PCG state; one per grid, read back by the host between chunks.
struct Scalars {
  double rz, norm, alpha, beta, rel, true_rel, tol;
  long long it, max_it, true_checks;
  int done;   // 0 running, 1 converged, 2 error, 3 iteration limit, 4 zero right-hand side
  int error;  // CFDG_E031 / CFDG_E032 when done == 2
  int check;  // the recurrent residual passed: run the true-residual gate
  unsigned counter;
};

}  // namespace cfdg
