// Device helpers shared by the per-molecule (tridiag.cu) and whole-GPU
// (tridiag_grid.cu) Householder eigensolvers.
#pragma once
#include <cuda_runtime.h>

namespace nddo {

__device__ __forceinline__ int tri_off(int i) { return (i * (i + 1)) >> 1; }

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Index range [lo, hi) of the eigenpairs a pass needs: the final pass all of
// them; an SCF iteration only the smaller of the occupied (0..nocc) and
// virtual (nocc..n) sets (the density is 2 X^T X or 2 I - 2 X^T X).
__host__ __device__ inline void hh_range(int n, int nocc, int final_pass, int* lo, int* hi) {
  if (final_pass) { *lo = 0; *hi = n; return; }
  if (n - nocc <= nocc) { *lo = nocc; *hi = n; }
  else { *lo = 0; *hi = nocc; }
}

}  // namespace nddo
