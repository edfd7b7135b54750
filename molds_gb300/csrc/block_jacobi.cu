// Kernel (d), large bases: batched two-sided block Jacobi, many CTAs per molecule.
//
// Replaces MolDS's Lapack::Dsyevd (src/wrappers/Lapack.cpp:102-160) for bases
// too large for the one-CTA shared-memory Jacobi (jacobi.cu).  The working
// matrix A (N' x N', N' = N rounded up to a multiple of 64) and the rotated
// basis V (rows = vectors, started from the previous iteration's eigenvectors)
// live in a per-molecule global workspace.  Indices are grouped into blocks of
// 32; a sweep runs the round-robin tournament over the N'/32 blocks, and in
// each round every disjoint block pair (I, J) is handled at once:
//   bj_sub:   the 64 x 64 matrix [A_II A_IJ; A_JI A_JJ] is diagonalised in
//             shared memory by cyclic Jacobi; its rotation Q (64 x 64) is kept;
//   bj_rows:  rows I u J of A and of V are replaced by Q^T (rows), tile by tile;
//   bj_cols:  columns I u J of A are replaced by (columns) Q.
// The updates are dense 64 x 64 x 64 tile products spread over many CTAs, so
// a single large molecule fills the GPU.  A molecule is done when a sweep
// finds every off-diagonal element below a relative threshold (2e-6 in FP32,
// 1e-13 in FP64, see BjTol); the host stops after the sweep in which every
// molecule of the launch is done.  The result is written as jacobi.cu
// writes it: eigenvalues ascending, eigenvectors as rows with component sum
// >= 0.
#include <cuda_runtime.h>
#include "nddo_batch.cuh"
#include "kernels.h"

namespace nddo {

constexpr int kBjB = 32;            // block size; a pair spans 64 indices
constexpr int kBjS = 2 * kBjB;      // sub-problem size
constexpr int kBjThreads = 256;

template <typename T> struct BjTol;
// The 64 x 64 x 64 tile updates leave round-off of about sqrt(64) ulp in the
// off-diagonal elements, so the stopping threshold sits above that level; the
// FP64 refinement of the mixed path squares the remaining FP32 error.
template <> struct BjTol<float> { static constexpr float rel = 2e-6f; };
template <> struct BjTol<double> { static constexpr double rel = 1e-13; };

__host__ __device__ inline int bj_np(int n) { return (n + kBjS - 1) / kBjS * kBjS; }

// blocks of pair k in round r of the tournament over nb blocks
__device__ __forceinline__ void bj_pair(int k, int r, int nb, int* I, int* J) {
  const int i1 = k, i2 = nb - 1 - k;
  const int p1 = (i1 == 0) ? 0 : ((i1 - 1 + r) % (nb - 1)) + 1;
  const int p2 = (i2 == 0) ? 0 : ((i2 - 1 + r) % (nb - 1)) + 1;
  *I = p1 < p2 ? p1 : p2;
  *J = p1 < p2 ? p2 : p1;
}

// per-molecule control record in the workspace
struct BjCtl {
  float scale;      // max |A_ii| at the start (stopping scale)
  int done;         // 1 once a sweep found nothing to rotate
  unsigned int offmax_bits;   // max |off-diagonal| seen in the current sweep (float bits)
  int sweeps;
  float prev_off;   // offmax of the previous sweep
  int pad[3];
};

// ---- setup: pad G into A, the basis into V, the stopping scale ----------------------
template <typename T, typename TCin>
__global__ void bj_init_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list,
                               const MolState* __restrict__ st, const T* __restrict__ G, const TCin* __restrict__ Cin,
                               T* __restrict__ Aws, T* __restrict__ Vws, long long stride, BjCtl* __restrict__ ctl) {
  const int slot = blockIdx.y;
  const int m = list[slot];
  if (st[m].status != kActive) return;
  const DevMol mol = mols[m];
  const int n = mol.nao, np = bj_np(n);
  T* A = Aws + slot * stride;
  T* V = Vws + slot * stride;
  const long long cnt = (long long)np * np;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / np), j = (int)(e % np);
    A[e] = (i < n && j < n) ? G[mol.mat0 + (long long)i * n + j] : (T)0;
    V[e] = (i < n && j < n) ? (T)Cin[mol.mat0 + (long long)i * n + j] : (T)(i == j ? 1 : 0);
  }
  if (blockIdx.x == 0) {
    __shared__ float red[kBjThreads / 32];
    float s = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fmaxf(s, fabsf((float)G[mol.mat0 + (long long)i * n + i]));
    for (int o = 16; o > 0; o >>= 1) s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      float mx = 0.f;
      for (int w = 0; w < kBjThreads / 32; ++w) mx = fmaxf(mx, red[w]);
      ctl[slot].scale = mx > 1e-30f ? mx : 1.f;
      ctl[slot].done = 0;
      ctl[slot].offmax_bits = 0u;
      ctl[slot].sweeps = 0;
      ctl[slot].prev_off = 3.0e38f;
    }
  }
}

// ---- sub-problem: diagonalise the 64 x 64 block of pair (I, J) ------------------------
template <typename T>
__global__ void __launch_bounds__(kBjThreads)
bj_sub_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
              int round, T* __restrict__ Aws, long long stride, T* __restrict__ Qws, long long qstride,
              int* __restrict__ qflag, BjCtl* __restrict__ ctl) {
  const int slot = blockIdx.y;
  const int m = list[slot];
  if (st[m].status != kActive || ctl[slot].done) return;
  const DevMol mol = mols[m];
  const int np = bj_np(mol.nao), nb = np / kBjB;
  const int k = blockIdx.x;
  if (k >= nb / 2) return;
  int I, J;
  bj_pair(k, round, nb, &I, &J);
  extern __shared__ __align__(16) unsigned char bj_smem[];
  T (*S)[kBjS + 1] = reinterpret_cast<T (*)[kBjS + 1]>(bj_smem);
  T (*Q)[kBjS + 1] = reinterpret_cast<T (*)[kBjS + 1]>(bj_smem + kBjS * (kBjS + 1) * sizeof(T));
  __shared__ T cs[kBjS];                 // c, s per pair of the inner tournament
  __shared__ int pq[kBjS];
  __shared__ int any_rot;
  __shared__ float offm[kBjThreads / 32];
  const T* A = Aws + slot * stride;
  const int tid = threadIdx.x;
  float off = 0.f;
  for (int e = tid; e < kBjS * kBjS; e += blockDim.x) {
    const int a = e / kBjS, b = e % kBjS;
    const int ga = (a < kBjB ? I * kBjB + a : J * kBjB + a - kBjB);
    const int gb = (b < kBjB ? I * kBjB + b : J * kBjB + b - kBjB);
    const T v = A[(long long)ga * np + gb];
    S[a][b] = v;
    Q[a][b] = (T)(a == b ? 1 : 0);
    if (a != b) off = fmaxf(off, fabsf((float)v));
  }
  for (int o = 16; o > 0; o >>= 1) off = fmaxf(off, __shfl_xor_sync(0xffffffffu, off, o));
  if ((tid & 31) == 0) offm[tid >> 5] = off;
  __syncthreads();
  const T thresh = BjTol<T>::rel * (T)ctl[slot].scale;
  if (tid == 0) {
    float mx = 0.f;
    for (int w = 0; w < kBjThreads / 32; ++w) mx = fmaxf(mx, offm[w]);
    atomicMax(&ctl[slot].offmax_bits, __float_as_uint(mx));
    any_rot = mx > (float)thresh;
  }
  __syncthreads();
  int* flag = qflag + (long long)slot * (nb / 2) + k;
  if (!any_rot) {
    if (tid == 0) *flag = 0;
    return;
  }
  // cyclic Jacobi on S, rotations accumulated in Q (S_final = Q^T S Q)
  for (int sweep = 0; sweep < 16; ++sweep) {
    int rotated = 0;
    for (int r = 0; r < kBjS - 1; ++r) {
      int rot_r = 0;
      if (tid < kBjS / 2) {
        int p, q;
        {
          const int i1 = tid, i2 = kBjS - 1 - tid;
          const int p1 = (i1 == 0) ? 0 : ((i1 - 1 + r) % (kBjS - 1)) + 1;
          const int p2 = (i2 == 0) ? 0 : ((i2 - 1 + r) % (kBjS - 1)) + 1;
          p = p1 < p2 ? p1 : p2;
          q = p1 < p2 ? p2 : p1;
        }
        const T apq = S[p][q];
        T c = 1, s = 0;
        if (fabs(apq) > thresh) {
          const T theta = (S[q][q] - S[p][p]) / (2 * apq);
          T t;
          if (fabs(theta) > (T)1e15) t = (T)0.5 / theta;
          else t = (theta >= 0 ? (T)1 : (T)-1) / (fabs(theta) + sqrt(theta * theta + (T)1));
          c = (T)1 / sqrt(t * t + (T)1);
          s = t * c;
          rot_r = 1;
        }
        cs[2 * tid] = c; cs[2 * tid + 1] = s;
        pq[2 * tid] = p; pq[2 * tid + 1] = q;
      }
      rotated |= rot_r;
      if (!__syncthreads_or(rot_r)) continue;
      // rows p, q of S
      for (int e = tid; e < (kBjS / 2) * kBjS; e += blockDim.x) {
        const int kk = e / kBjS, j = e % kBjS;
        const int p = pq[2 * kk], q = pq[2 * kk + 1];
        const T c = cs[2 * kk], s = cs[2 * kk + 1];
        const T a = S[p][j], b = S[q][j];
        S[p][j] = c * a - s * b;
        S[q][j] = s * a + c * b;
      }
      __syncthreads();
      // columns p, q of S and of Q
      for (int e = tid; e < (kBjS / 2) * kBjS; e += blockDim.x) {
        const int kk = e / kBjS, i = e % kBjS;
        const int p = pq[2 * kk], q = pq[2 * kk + 1];
        const T c = cs[2 * kk], s = cs[2 * kk + 1];
        const T a = S[i][p], b = S[i][q];
        S[i][p] = c * a - s * b;
        S[i][q] = s * a + c * b;
        const T qa = Q[i][p], qb = Q[i][q];
        Q[i][p] = c * qa - s * qb;
        Q[i][q] = s * qa + c * qb;
      }
      __syncthreads();
    }
    if (!__syncthreads_or(rotated)) break;
  }
  T* Qg = Qws + slot * qstride + (long long)k * kBjS * kBjS;
  for (int e = tid; e < kBjS * kBjS; e += blockDim.x) Qg[e] = Q[e / kBjS][e % kBjS];
  if (tid == 0) *flag = 1;
}

// ---- rows of A and V: X[R, tile] <- Q^T X[R, tile] -------------------------------
// grid.x = pairs x column tiles x {A, V}
template <typename T>
__global__ void __launch_bounds__(kBjThreads)
bj_rows_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
               int round, T* __restrict__ Aws, T* __restrict__ Vws, long long stride, const T* __restrict__ Qws,
               long long qstride, const int* __restrict__ qflag, const BjCtl* __restrict__ ctl, int max_pairs,
               int max_tiles) {
  const int slot = blockIdx.y;
  const int m = list[slot];
  if (st[m].status != kActive || ctl[slot].done) return;
  const DevMol mol = mols[m];
  const int np = bj_np(mol.nao), nb = np / kBjB, ntile = np / kBjS;
  const int which = blockIdx.x / (max_pairs * max_tiles);
  const int rem = blockIdx.x % (max_pairs * max_tiles);
  const int k = rem / max_tiles, tile = rem % max_tiles;
  if (k >= nb / 2 || tile >= ntile) return;
  if (!qflag[(long long)slot * (nb / 2) + k]) return;
  int I, J;
  bj_pair(k, round, nb, &I, &J);
  extern __shared__ __align__(16) unsigned char bj_smem[];
  T (*Qs)[kBjS + 1] = reinterpret_cast<T (*)[kBjS + 1]>(bj_smem);
  T (*Xs)[kBjS + 1] = reinterpret_cast<T (*)[kBjS + 1]>(bj_smem + kBjS * (kBjS + 1) * sizeof(T));
  const T* Qg = Qws + slot * qstride + (long long)k * kBjS * kBjS;
  T* X = (which == 0 ? Aws : Vws) + slot * stride;
  const int tid = threadIdx.x;
  for (int e = tid; e < kBjS * kBjS; e += blockDim.x) {
    const int a = e / kBjS, b = e % kBjS;
    Qs[a][b] = Qg[e];
    const int ga = (a < kBjB ? I * kBjB + a : J * kBjB + a - kBjB);
    Xs[a][b] = X[(long long)ga * np + tile * kBjS + b];
  }
  __syncthreads();
  // out[a][b] = sum_c Q[c][a] X[c][b]; thread: rows a0 + 16 i, column b
  const int b = tid & 63, a0 = tid >> 6;    // 4 row groups
  T acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0;
  for (int c = 0; c < kBjS; ++c) {
    const T x = Xs[c][b];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] += Qs[c][a0 + 4 * i] * x;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int a = a0 + 4 * i;
    const int ga = (a < kBjB ? I * kBjB + a : J * kBjB + a - kBjB);
    X[(long long)ga * np + tile * kBjS + b] = acc[i];
  }
}

// ---- columns of A: A[tile, R] <- A[tile, R] Q ------------------------------------
template <typename T>
__global__ void __launch_bounds__(kBjThreads)
bj_cols_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
               int round, T* __restrict__ Aws, long long stride, const T* __restrict__ Qws, long long qstride,
               const int* __restrict__ qflag, const BjCtl* __restrict__ ctl, int max_pairs, int max_tiles) {
  const int slot = blockIdx.y;
  const int m = list[slot];
  if (st[m].status != kActive || ctl[slot].done) return;
  const DevMol mol = mols[m];
  const int np = bj_np(mol.nao), nb = np / kBjB, ntile = np / kBjS;
  const int k = blockIdx.x / max_tiles, tile = blockIdx.x % max_tiles;
  if (k >= nb / 2 || tile >= ntile || k >= max_pairs) return;
  if (!qflag[(long long)slot * (nb / 2) + k]) return;
  int I, J;
  bj_pair(k, round, nb, &I, &J);
  extern __shared__ __align__(16) unsigned char bj_smem[];
  T (*Qs)[kBjS + 1] = reinterpret_cast<T (*)[kBjS + 1]>(bj_smem);
  T (*Xs)[kBjS + 1] = reinterpret_cast<T (*)[kBjS + 1]>(bj_smem + kBjS * (kBjS + 1) * sizeof(T));
  const T* Qg = Qws + slot * qstride + (long long)k * kBjS * kBjS;
  T* A = Aws + slot * stride;
  const int tid = threadIdx.x;
  for (int e = tid; e < kBjS * kBjS; e += blockDim.x) {
    const int a = e / kBjS, b = e % kBjS;
    Qs[a][b] = Qg[e];
    const int gb = (b < kBjB ? I * kBjB + b : J * kBjB + b - kBjB);
    Xs[a][b] = A[(long long)(tile * kBjS + a) * np + gb];
  }
  __syncthreads();
  // out[a][b] = sum_c X[a][c] Q[c][b]
  const int b = tid & 63, a0 = tid >> 6;
  T acc[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) acc[i] = 0;
  for (int c = 0; c < kBjS; ++c) {
    const T q = Qs[c][b];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] += Xs[a0 + 4 * i][c] * q;
  }
  const int gb = (b < kBjB ? I * kBjB + b : J * kBjB + b - kBjB);
#pragma unroll
  for (int i = 0; i < 16; ++i) A[(long long)(tile * kBjS + a0 + 4 * i) * np + gb] = acc[i];
}

// ---- end of sweep: a molecule is done when the sweep saw nothing above threshold -------
template <typename T>
__global__ void bj_sweep_end_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, int nlist,
                                    const MolState* __restrict__ st, BjCtl* __restrict__ ctl, int* __restrict__ pending) {
  int cnt = 0;
  for (int slot = threadIdx.x; slot < nlist; slot += blockDim.x) {
    const int m = list[slot];
    if (st[m].status != kActive || ctl[slot].done) continue;
    const float off = __uint_as_float(ctl[slot].offmax_bits);
    const float tol = (float)(BjTol<T>::rel * (T)ctl[slot].scale);
    ctl[slot].sweeps += 1;
    // done when nothing was above the threshold, or when the off-diagonal
    // stopped shrinking within a few thresholds of it (the tile updates'
    // round-off floor; Jacobi's quadratic convergence otherwise divides it by
    // far more than 2 per sweep)
    if (off <= tol || (off <= 16.f * tol && off > 0.5f * ctl[slot].prev_off)) ctl[slot].done = 1;
    else ++cnt;
    ctl[slot].prev_off = off;
    ctl[slot].offmax_bits = 0u;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  __shared__ int red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    *pending = t;
  }
}

// ---- sort ascending, sign fix, write eigenvector rows (FP64) and eigenvalues -----------
template <typename T>
__global__ void __launch_bounds__(kBjThreads)
bj_finish_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
                 const T* __restrict__ Aws, const T* __restrict__ Vws, long long stride, double* __restrict__ Cout,
                 double* __restrict__ eps_out, int* __restrict__ order_ws, int ord_stride,
                 const BjCtl* __restrict__ ctl, int* __restrict__ sweeps_out) {
  const int slot = blockIdx.x;
  const int m = list[slot];
  if (st[m].status != kActive) return;
  const DevMol mol = mols[m];
  const int n = mol.nao, np = bj_np(n);
  const T* A = Aws + slot * stride;
  const T* V = Vws + slot * stride;
  int* order = order_ws + (long long)slot * ord_stride;
  T* sgn = reinterpret_cast<T*>(order_ws + (long long)gridDim.x * ord_stride) + (long long)slot * ord_stride;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const T li = A[(long long)i * np + i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const T lj = A[(long long)j * np + j];
      rank += (lj < li) || (lj == li && j < i);
    }
    order[rank] = i;
    T sum = 0;
    for (int mu = 0; mu < n; ++mu) sum += V[(long long)i * np + mu];
    sgn[i] = sum < (T)0 ? (T)-1 : (T)1;
    eps_out[mol.vec0 + rank] = (double)li;
  }
  __syncthreads();
  double* Co = Cout + mol.mat0;
  for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
    const int r = (int)(e / n), mu = (int)(e % n);
    const int col = order[r];
    Co[e] = (double)(sgn[col] * V[(long long)col * np + mu]);
  }
  if (threadIdx.x == 0 && sweeps_out) sweeps_out[m] += ctl[slot].sweeps;
}

// ---------------------------------------------------------------------------------
size_t block_jacobi_workspace(int max_n, int nslots, int elem, long long* stride, long long* qstride) {
  const long long np = bj_np(max_n);
  *stride = np * np;
  *qstride = (np / kBjS) * (long long)kBjS * kBjS;
  const size_t mats = (size_t)nslots * (2 * *stride + *qstride) * elem;
  const size_t ctl = (size_t)nslots * (sizeof(BjCtl) + (np / kBjS) * sizeof(int)) + 64;
  const size_t ord = (size_t)nslots * np * (sizeof(int) + elem);
  return mats + ctl + ord + 1024;
}

template <typename T, typename TCin>
int launch_block_jacobi_impl(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                             const T* G, const TCin* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                             int* sweeps_out, int* h_pending, cudaStream_t s) {
  if (nlist <= 0) return 0;
  long long stride, qstride;
  block_jacobi_workspace(max_n, nlist, sizeof(T), &stride, &qstride);
  const int np = bj_np(max_n), nb = np / kBjB, pairs = nb / 2, tiles = np / kBjS;
  char* p = reinterpret_cast<char*>(ws);
  T* A = reinterpret_cast<T*>(p); p += (size_t)nlist * stride * sizeof(T);
  T* V = reinterpret_cast<T*>(p); p += (size_t)nlist * stride * sizeof(T);
  T* Q = reinterpret_cast<T*>(p); p += (size_t)nlist * qstride * sizeof(T);
  BjCtl* ctl = reinterpret_cast<BjCtl*>(p); p += ((size_t)nlist * sizeof(BjCtl) + 15) & ~(size_t)15;
  int* qflag = reinterpret_cast<int*>(p); p += ((size_t)nlist * pairs * sizeof(int) + 15) & ~(size_t)15;
  int* pending = reinterpret_cast<int*>(p); p += 16;
  int* order = reinterpret_cast<int*>(p);
  const size_t smem = 2 * kBjS * (kBjS + 1) * sizeof(T);
  cudaFuncSetAttribute(bj_sub_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(bj_rows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(bj_cols_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  bj_init_kernel<T, TCin><<<dim3(32, nlist), kBjThreads, 0, s>>>(mols, list, st, G, Cin, A, V, stride, ctl);
  int launches = 1, sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    for (int r = 0; r < nb - 1; ++r) {
      bj_sub_kernel<T><<<dim3(pairs, nlist), kBjThreads, smem, s>>>(mols, list, st, r, A, stride, Q, qstride, qflag,
                                                                     ctl);
      bj_rows_kernel<T><<<dim3(2 * pairs * tiles, nlist), kBjThreads, smem, s>>>(mols, list, st, r, A, V, stride, Q,
                                                                                  qstride, qflag, ctl, pairs, tiles);
      bj_cols_kernel<T><<<dim3(pairs * tiles, nlist), kBjThreads, smem, s>>>(mols, list, st, r, A, stride, Q, qstride,
                                                                             qflag, ctl, pairs, tiles);
      launches += 3;
    }
    bj_sweep_end_kernel<T><<<1, 256, 0, s>>>(mols, list, nlist, st, ctl, pending);
    cudaMemcpyAsync(h_pending, pending, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) break;
    launches += 1;
    if (*h_pending == 0) break;
  }
  bj_finish_kernel<T><<<nlist, kBjThreads, 0, s>>>(mols, list, st, A, V, stride, Cout, eps, order, np, ctl,
                                                   sweeps_out);
  return launches + 1;
}

int launch_block_jacobi_f32(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                            const float* G, const double* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                            int* sweeps_out, int* h_pending, cudaStream_t s) {
  return launch_block_jacobi_impl<float, double>(mols, list, nlist, max_n, st, G, Cin, Cout, eps, ws, max_sweeps, sweeps_out,
                                         h_pending, s);
}

int launch_block_jacobi_f32(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                            const float* G, const float* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                            int* sweeps_out, int* h_pending, cudaStream_t s) {
  return launch_block_jacobi_impl<float, float>(mols, list, nlist, max_n, st, G, Cin, Cout, eps, ws, max_sweeps,
                                                sweeps_out, h_pending, s);
}

int launch_block_jacobi_f64(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                            const double* G, const double* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                            int* sweeps_out, int* h_pending, cudaStream_t s) {
  return launch_block_jacobi_impl<double, double>(mols, list, nlist, max_n, st, G, Cin, Cout, eps, ws, max_sweeps, sweeps_out,
                                          h_pending, s);
}

}  // namespace nddo
