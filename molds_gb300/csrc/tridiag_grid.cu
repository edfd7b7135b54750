// Kernel (d), FP64 path for large molecules: the Householder eigensolver of
// tridiag.cu spread over many SMs per molecule.  One cooperative launch (one
// CTA per SM) serves up to one molecule per SM: each molecule gets a sub-grid
// of CTAs in proportion to N^3, with its own barrier words.
//
// Stands in for MolDS's Lapack::Dsyevd (src/wrappers/Lapack.cpp:102-160) on
// the bases that do not fit one SM: a one-CTA tridiagonalisation of N = 3072
// would run (2/3) N^3 FP64 FMAs on a single SM's two FMA pipes (seconds).
//
//   hh_tridiag_grid_kernel  A = Q T Q^T on the full square matrix (global
//       memory, 75 MB at N = 3072: L2-resident).  Trailing rows are owned
//       round-robin by the warps of the grid.  One grid barrier per column:
//       after barrier k every CTA holds p_k (written by the row owners) and
//       forms w_k, the next column (row k + 1 after update k, which its owner
//       never writes) and reflector k + 1 itself; each warp then updates its
//       rows with (v_k, w_k) and, in the same pass, forms their entries of
//       p_{k+1} = tau_{k+1} A v_{k+1}.  Updates use the lower-triangle formula
//       of tridiag.cu on both (i, j) and (j, i), so A stays exactly symmetric.
//   tri_orth_grid_kernel    re-orthogonalisation inside clusters of close
//       eigenvalues (gap below 1e-3 ||T||_1, dstein's criterion): blocks of
//       32 vectors, each projected twice against the earlier vectors of its
//       cluster (classical Gram-Schmidt with reorthogonalisation, as block
//       products spread over the grid), then orthonormalised within the block
//       by two Cholesky-QR passes restricted to cluster members.  The result
//       spans the same nested subspaces as vector-by-vector Gram-Schmidt.
//   hh_back_wide_kernel     X = Q Z like hh_back_kernel, with 16, 8 or 4
//       columns per CTA so that N x columns fits shared memory.
// The eigenvalues and inverse-iteration vectors come from tri_vectors_kernel
// (tridiag.cu) with its factors in global scratch.
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "nddo_batch.cuh"
#include "kernels.h"
#include "tridiag.cuh"

namespace nddo {

void cuda_check(cudaError_t e, const char* what);   // engine.cu: throws on error

constexpr int kGridThreads = 512;
constexpr int kGridWarps = kGridThreads / 32;
constexpr long long kGridWaitCycles = 4000000000LL;   // ~2 s: a CTA that has not arrived by then never will
constexpr int kOrthChunk = 256;                       // projection coefficients staged per chunk (64 KB)
constexpr int kWideWarps = 8;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Barrier over the CTAs of one molecule's sub-grid of a cooperative launch.
// bar[0] counts arrivals, bar[1] is the generation, bar[2] the error flag: a
// wait longer than kGridWaitCycles sets it, and every CTA of the sub-grid
// leaves at its next barrier.  The host zeroes the words before each launch.
struct GridBarrier {
  unsigned* bar;
  unsigned gen;
  unsigned nblocks;   // CTAs of this molecule's sub-grid
  __device__ bool sync(int* flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int ok = 1;
      if (ld_acquire_gpu(bar + 2) != 0) {
        ok = 0;
      } else {
        __threadfence();
        if (atomicAdd(bar, 1u) == nblocks - 1) {
          atomicExch(bar, 0u);
          __threadfence();
          atomicExch(bar + 1, gen + 1);
        } else {
          const long long t0 = clock64();
          while (ld_acquire_gpu(bar + 1) == gen) {
            if (ld_acquire_gpu(bar + 2) != 0) { ok = 0; break; }
            if (clock64() - t0 > kGridWaitCycles) { atomicExch(bar + 2, 1u); ok = 0; break; }
            __nanosleep(64);
          }
        }
        __threadfence();
      }
      *flag = ok;
    }
    ++gen;
    __syncthreads();
    return *flag != 0;
  }
};

// Householder reflector of the column held in v[j0..n): on return v[j0] = 1,
// v[j0+1..n) scaled (LAPACK dlarfg conventions, as hh_tridiag_kernel).
// Returns tau; *beta = the new subdiagonal entry.  CTA-wide.
__device__ double block_house(double* v, int j0, int n, double* red, double* hs, double* beta) {
  const int tid = threadIdx.x;
  double s = 0.0;
  for (int j = j0 + 1 + tid; j < n; j += kGridThreads) s = fma(v[j], v[j], s);
  s = warp_sum_d(s);
  if ((tid & 31) == 0) red[tid >> 5] = s;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int w = 0; w < kGridWarps; ++w) tot += red[w];
    const double alpha = v[j0];
    double tau = 0.0, bt = alpha, scal = 0.0;
    if (tot != 0.0) {
      const double nrm = sqrt(fma(alpha, alpha, tot));
      bt = alpha >= 0.0 ? -nrm : nrm;
      tau = (bt - alpha) / bt;
      scal = 1.0 / (alpha - bt);
    }
    hs[0] = tau;
    hs[1] = scal;
    hs[2] = bt;
    v[j0] = 1.0;
  }
  __syncthreads();
  const double scal = hs[1];
  for (int j = j0 + 1 + tid; j < n; j += kGridThreads) v[j] *= scal;
  __syncthreads();
  *beta = hs[2];
  return hs[0];
}

// first row >= imin owned by this warp: rows i = cta + G (warp + W t)
__device__ __forceinline__ int first_own_row(int imin, int cta, int G, int warp) {
  const int base = cta + G * warp, step = G * kGridWarps;
  if (base >= imin) return base;
  return base + ((imin - base + step - 1) / step) * step;
}

__device__ __forceinline__ void grid_fail(MolState* st, int mi) {
  if (threadIdx.x == 0) st[mi].status = kFailed;
}

__global__ void __launch_bounds__(kGridThreads, 1)
hh_tridiag_grid_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const int3* __restrict__ map,
                       MolState* __restrict__ st, int require_active, const double* __restrict__ F,
                       double* __restrict__ W, double* __restrict__ td, long long vstride, double* __restrict__ Aws,
                       double* __restrict__ scratch, unsigned* __restrict__ bars) {
  extern __shared__ __align__(16) double gsm[];
  __shared__ int flag;
  __shared__ double red[kGridWarps], wred[kGridWarps], hs[4];
  const int3 slot = map[blockIdx.x];   // (list entry, CTA within the molecule's sub-grid, sub-grid size)
  const int mi = list[slot.x];
  if (require_active && st[mi].status != kActive) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = slot.z, cta = slot.y, rstep = G * kGridWarps;
  const double* Fm = F + mol.mat0;
  double* A = Aws + mol.mat0;
  double* Wm = W + mol.mat0;
  double* dd = td + mol.vec0;
  double* ee = dd + vstride;
  double* tt = ee + vstride;
  double* pbuf = scratch + mol.mat0;         // p of two consecutive steps (2 x n)
  double* part = pbuf + 2 * (long long)n;    // per-CTA partial sums of p.v (2 x G)
  double* vk = gsm;                          // reflector of the step being applied
  double* wk = vk + n;                       // its w
  double* vn = wk + n;                       // the next reflector
  if (n < 3) {
    if (cta == 0 && tid == 0) {
      dd[0] = Fm[0];
      ee[0] = n == 2 ? Fm[1] : 0.0;
      tt[0] = 0.0;
      if (n == 2) { dd[1] = Fm[3]; ee[1] = 0.0; tt[1] = 0.0; }
    }
    return;
  }
  GridBarrier gb{bars + 4 * slot.x, 0u, (unsigned)G};

  // column 0 (= row 0) and reflector 0
  for (int j = 1 + tid; j < n; j += kGridThreads) vk[j] = Fm[j];
  __syncthreads();
  double beta;
  double tauk = block_house(vk, 1, n, red, hs, &beta);
  if (cta == 0) {
    if (tid == 0) { dd[0] = Fm[0]; ee[0] = beta; tt[0] = tauk; }
    for (int j = 1 + tid; j < n; j += kGridThreads) Wm[j] = vk[j];
  }
  // own rows i >= 1: copy into the workspace and form p_0
  {
    double wpart = 0.0;
    for (int i = first_own_row(1, cta, G, warp); i < n; i += rstep) {
      const double* fr = Fm + (long long)i * n;
      double* ar = A + (long long)i * n;
      double s = 0.0;
      for (int j = 1 + lane; j < n; j += 32) {
        const double a = fr[j];
        __stcg(ar + j, a);
        s = fma(a, vk[j], s);
      }
      s = warp_sum_d(s);
      const double pi = tauk * s;
      if (lane == 0) {
        __stcg(pbuf + i, pi);
        wpart = fma(pi, vk[i], wpart);
      }
    }
    if (lane == 0) wred[warp] = wpart;
    __syncthreads();
    if (tid == 0) {
      double c = 0.0;
      for (int w = 0; w < kGridWarps; ++w) c += wred[w];
      __stcg(part + cta, c);
    }
  }
  if (!gb.sync(&flag)) { grid_fail(st, mi); return; }

  for (int k = 0; k + 2 < n; ++k) {
    const int b = k & 1;
    // w_k = p_k - (tau_k / 2)(p_k . v_k) v_k
    if (warp == 0) {
      double s = 0.0;
      for (int c = lane; c < G; c += 32) s += __ldcg(part + b * G + c);
      s = warp_sum_d(s);
      if (lane == 0) hs[3] = s;
    }
    __syncthreads();
    const double ch = 0.5 * tauk * hs[3];
    const double* pk = pbuf + (long long)b * n;
    for (int j = k + 1 + tid; j < n; j += kGridThreads) wk[j] = fma(-ch, vk[j], __ldcg(pk + j));
    __syncthreads();
    const int r = k + 1;
    const double vr = vk[r], wr = wk[r];
    if (k + 3 < n) {
      // column r after update k (row r: its owner leaves it alone from now on)
      const double* arow = A + (long long)r * n;
      for (int j = r + 1 + tid; j < n; j += kGridThreads)
        vn[j] = fma(-vk[j], wr, fma(-wk[j], vr, __ldcg(arow + j)));
      double dnext = 0.0;
      if (tid == 0) dnext = fma(-vr, wr, fma(-wr, vr, __ldcg(arow + r)));
      __syncthreads();
      double betan;
      const double taun = block_house(vn, r + 1, n, red, hs, &betan);
      if (cta == 0) {
        if (tid == 0) { dd[r] = dnext; ee[r] = betan; tt[r] = taun; }
        for (int j = r + 1 + tid; j < n; j += kGridThreads) Wm[(long long)r * n + j] = vn[j];
      }
      // own rows i >= k + 2: A <- A - v w^T - w v^T, then p_{k+1} = tau A v_{k+1}
      double wpart = 0.0;
      double* pn = pbuf + (long long)(b ^ 1) * n;
      for (int i = first_own_row(k + 2, cta, G, warp); i < n; i += rstep) {
        const double vi = vk[i], wi = wk[i];
        double* ar = A + (long long)i * n;
        double s = 0.0;
        for (int j = k + 2 + lane; j < n; j += 32) {
          const double vj = vk[j], wj = wk[j];
          const bool low = i >= j;   // (big index, small index) of the lower-triangle formula
          const double vb = low ? vi : vj, wb = low ? wi : wj, vs = low ? vj : vi, ws = low ? wj : wi;
          const double a = fma(-vb, ws, fma(-wb, vs, __ldcg(ar + j)));
          __stcg(ar + j, a);
          s = fma(a, vn[j], s);
        }
        s = warp_sum_d(s);
        const double pi = taun * s;
        if (lane == 0) {
          __stcg(pn + i, pi);
          wpart = fma(pi, vn[i], wpart);
        }
      }
      if (lane == 0) wred[warp] = wpart;
      __syncthreads();
      if (tid == 0) {
        double c = 0.0;
        for (int w = 0; w < kGridWarps; ++w) c += wred[w];
        __stcg(part + (b ^ 1) * G + cta, c);
      }
      double* t = vk; vk = vn; vn = t;
      tauk = taun;
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
    } else if (cta == 0 && tid == 0) {
      // k = n - 3: the trailing 2 x 2 block after the last update
      const int q = n - 1;
      const double vq = vk[q], wq = wk[q];
      dd[r] = fma(-vr, wr, fma(-wr, vr, __ldcg(A + (long long)r * n + r)));
      ee[r] = fma(-vq, wr, fma(-wq, vr, __ldcg(A + (long long)r * n + q)));
      tt[r] = 0.0;
      dd[q] = fma(-vq, wq, fma(-wq, vq, __ldcg(A + (long long)q * n + q)));
      ee[q] = 0.0;
      tt[q] = 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Re-orthogonalisation inside clusters, over the grid.
// ---------------------------------------------------------------------------

// Partial products part[s][l - l_beg][j] = sum over the rows of split s of
// Z[i][l] Z[i][b0 + j], for l in [l_beg, l_end) and j < nb: the work items
// (32-wide tile of l, split of the rows) are spread over the CTAs; each CTA
// stages 32 rows of both column sets in shared memory per step and every
// thread accumulates two outputs (j = lane, l and l + 16).
__device__ void tile_products(const double* __restrict__ Zm, int n, int k, int l_beg, int l_end, int b0, int nb,
                              int S, double* __restrict__ part, double (*sa)[33], double (*sb)[33], int cta, int G) {
  const int L = l_end - l_beg, nlt = (L + 31) >> 5, items = nlt * S, R = (n + S - 1) / S;
  const int t = threadIdx.x, j = t & 31, l = t >> 5;
  for (int it = cta; it < items; it += G) {
    const int lt = it % nlt, sp = it / nlt;
    const int l0 = l_beg + 32 * lt, nl = min(32, l_end - l0);
    const int r0 = sp * R, r1 = min(n, r0 + R);
    double acc0 = 0.0, acc1 = 0.0;
    for (int rc = r0; rc < r1; rc += 32) {
      __syncthreads();
      for (int e = t; e < 2048; e += kGridThreads) {
        const int half = e >> 10, rr = (e >> 5) & 31, cc = e & 31, i = rc + rr;
        double v = 0.0;
        if (i < r1) {
          if (half == 0) { if (cc < nl) v = __ldcg(Zm + (long long)i * k + l0 + cc); }
          else if (cc < nb) v = __ldcg(Zm + (long long)i * k + b0 + cc);
        }
        if (half == 0) sa[rr][cc] = v; else sb[rr][cc] = v;
      }
      __syncthreads();
#pragma unroll 8
      for (int rr = 0; rr < 32; ++rr) {
        const double zb = sb[rr][j];
        acc0 = fma(sa[rr][l], zb, acc0);
        acc1 = fma(sa[rr][l + 16], zb, acc1);
      }
    }
    double* P = part + ((long long)sp * (nlt * 32) + 32 * lt) * 32;
    __stcg(P + l * 32 + j, acc0);
    __stcg(P + (l + 16) * 32 + j, acc1);
  }
}

__global__ void __launch_bounds__(kGridThreads, 1)
tri_orth_grid_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const int3* __restrict__ map,
                     MolState* __restrict__ st, int require_active, int final_pass, const double* __restrict__ td,
                     long long vstride, const double* __restrict__ eps, double* __restrict__ Z,
                     double* __restrict__ scratch, unsigned* __restrict__ bars) {
  extern __shared__ __align__(16) double osm[];
  __shared__ int flag;
  __shared__ double red[kGridWarps];
  __shared__ double sa[32][33], sb[32][33];
  __shared__ double rs[32];
  const int3 slot = map[blockIdx.x];
  const int mi = list[slot.x];
  if (require_active && st[mi].status != kActive) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  int lo, hi;
  hh_range(n, mol.nocc, final_pass, &lo, &hi);
  const int k = hi - lo;
  if (k < 2) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = slot.z, cta = slot.y;
  double* gs = osm;                                            // kOrthChunk x 32 coefficients
  int* cs = reinterpret_cast<int*>(gs + kOrthChunk * 32);      // cluster [cs, ce) of each column
  int* ce = cs + k;
  double* Zm = Z + mol.mat0;
  double* Gf = scratch + mol.mat0;                             // (k x 32) projection coefficients
  double* Mg = Gf + (long long)k * 32;                         // 32 x 32 Gram matrix
  double* part = Mg + 1024;                                    // partial products of the row splits
  // the molecule's scratch matrix holds N x N doubles: the splits are capped
  // so that the partial products fit behind the coefficients
  const long long part_cap = (long long)n * n - (long long)k * 32 - 1024;
  const double* tdd = td + mol.vec0;
  const double* tde = tdd + vstride;
  const double* ev = eps + mol.vec0 + lo;

  double nr = 0.0;
  for (int i = tid; i < n; i += kGridThreads) {
    const double r = fabs(tdd[i]) + (i + 1 < n ? fabs(tde[i]) : 0.0) + (i > 0 ? fabs(tde[i - 1]) : 0.0);
    nr = fmax(nr, r);
  }
  for (int o = 16; o > 0; o >>= 1) nr = fmax(nr, __shfl_xor_sync(0xffffffffu, nr, o));
  if (lane == 0) red[warp] = nr;
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int w = 0; w < kGridWarps; ++w) m = fmax(m, red[w]);
    const double ortol = 1e-3 * m;
    int c0 = 0;
    for (int c = 1; c <= k; ++c)
      if (c == k || ev[c] - ev[c - 1] >= ortol) {
        for (int q = c0; q < c; ++q) { cs[q] = c0; ce[q] = c; }
        c0 = c;
      }
  }
  __syncthreads();
  GridBarrier gb{bars + 4 * slot.x, 0u, (unsigned)G};
  const int rstep = G * kGridWarps;

  for (int b0 = 0; b0 < k; b0 += 32) {
    const int nb = min(32, k - b0);
    int cmin = b0;
    bool any = false;
    for (int q = 0; q < nb; ++q)
      if (ce[b0 + q] - cs[b0 + q] >= 2) { any = true; cmin = min(cmin, cs[b0 + q]); }
    if (!any) continue;
    const int L = b0 - cmin;
    const int jc = b0 + lane;

    // two projections against the earlier vectors of each column's cluster
    for (int pass = 0; pass < 2 && L > 0; ++pass) {
      const int nlt = (L + 31) >> 5;
      const int S = max(1, min(min(32, G / nlt), (int)(part_cap / (nlt * 1024))));
      tile_products(Zm, n, k, cmin, b0, b0, nb, S, part, sa, sb, cta, G);
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
      // coefficients: the sum over the splits, kept only within each column's cluster
      for (int e = cta * kGridThreads + tid; e < L * 32; e += G * kGridThreads) {
        const int l = cmin + (e >> 5), jj = e & 31;
        double v = 0.0;
        for (int sp = 0; sp < S; ++sp) v += __ldcg(part + (long long)sp * (nlt * 32) * 32 + e);
        const bool keep = jj < nb && ce[b0 + jj] - cs[b0 + jj] >= 2 && l >= cs[b0 + jj];
        __stcg(Gf + e, keep ? v : 0.0);
      }
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
      // z_j -= sum_l G[l][j] z_l on the warp's rows (four rows per round)
      const int rounds = (n + 4 * rstep - 1) / (4 * rstep);
      for (int t0 = 0; t0 < rounds; ++t0) {
        int rows[4];
        double acc[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = cta + G * (warp + kGridWarps * (4 * t0 + r));
          rows[r] = i < n ? i : -1;
          acc[r] = (i < n && lane < nb) ? __ldcg(Zm + (long long)i * k + jc) : 0.0;
        }
        for (int c0 = 0; c0 < L; c0 += kOrthChunk) {
          const int cn = min(kOrthChunk, L - c0);
          __syncthreads();
          for (int e = tid; e < cn * 32; e += kGridThreads) gs[e] = __ldcg(Gf + (long long)c0 * 32 + e);
          __syncthreads();
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            if (rows[r] < 0) continue;
            const double* zr = Zm + (long long)rows[r] * k + cmin + c0;
            for (int q0 = 0; q0 < cn; q0 += 32) {
              const double zl = q0 + lane < cn ? __ldcg(zr + q0 + lane) : 0.0;
              const int qn = min(32, cn - q0);
              for (int q = 0; q < qn; ++q)
                acc[r] = fma(-gs[(q0 + q) * 32 + lane], __shfl_sync(0xffffffffu, zl, q), acc[r]);
            }
          }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (rows[r] >= 0 && lane < nb) __stcg(Zm + (long long)rows[r] * k + jc, acc[r]);
      }
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
    }

    // two Cholesky-QR passes inside the block (cluster members only)
    for (int pass = 0; pass < 2; ++pass) {
      const int S = max(1, min(min(G, n >> 3), (int)(part_cap / 1024)));
      tile_products(Zm, n, k, b0, b0 + nb, b0, nb, S, part, sa, sb, cta, G);
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
      for (int e = cta * kGridThreads + tid; e < 1024; e += G * kGridThreads) {
        const int a = e >> 5, c = e & 31;
        double v = 0.0;
        for (int sp = 0; sp < S; ++sp) v += __ldcg(part + (long long)sp * 1024 + e);
        const bool in = a < nb && c < nb && ce[b0 + a] - cs[b0 + a] >= 2 && cs[b0 + a] == cs[b0 + c];
        __stcg(Mg + e, in ? v : (a == c ? 1.0 : 0.0));
      }
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
      // every CTA: M = L L^T (one warp, right-looking and unscaled: after the
      // loop L[a][q] = Ms[a][q] / sqrt(Ms[q][q])), then L^-1
      for (int e = tid; e < 1024; e += kGridThreads) sa[e >> 5][e & 31] = __ldcg(Mg + e);
      __syncthreads();
      if (warp == 0) {
        for (int c = 0; c < 32; ++c) {
          const double piv = fmax(sa[c][c], 1e-300);
          __syncwarp();
          if (lane > c) {
            const double f = sa[lane][c] / piv;
            for (int q = c + 1; q <= lane; ++q) sa[lane][q] = fma(-f, sa[q][c], sa[lane][q]);
          }
          __syncwarp();
        }
        rs[lane] = rsqrt(fmax(sa[lane][lane], 1e-300));
        __syncwarp();
        const int c = lane;   // column c of L^-1, by forward substitution
        for (int a = 0; a < c; ++a) sb[a][c] = 0.0;
        sb[c][c] = rs[c];
        for (int a = c + 1; a < 32; ++a) {
          double s = 0.0;
          for (int q = c; q < a; ++q) s = fma(sa[a][q] * rs[q], sb[q][c], s);
          sb[a][c] = -s * rs[a];
        }
      }
      __syncthreads();
      for (int i = cta + G * warp; i < n; i += rstep) {
        const double z = lane < nb ? __ldcg(Zm + (long long)i * k + jc) : 0.0;
        double y = 0.0;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const double zq = __shfl_sync(0xffffffffu, z, q);
          if (q <= lane) y = fma(sb[lane][q], zq, y);
        }
        if (lane < nb) __stcg(Zm + (long long)i * k + jc, y);
      }
      if (!gb.sync(&flag)) { grid_fail(st, mi); return; }
    }
  }
}

// ---------------------------------------------------------------------------
// X = Q Z with kCols columns per CTA (lanes: column lane % kCols, row slice
// lane / kCols; S = 8 * 32 / kCols row slices, row i in slice i mod S).
// Reflector j is staged in shared memory while every thread holds its share
// of reflector j - 1 in registers (loaded during the work on j), so the
// reflector rows cost one coalesced global read each.
// ---------------------------------------------------------------------------
constexpr int kBackPre = 24;   // reflector entries per thread held in registers: N <= 24 * 256

template <typename T, int kCols>
__global__ void __launch_bounds__(kWideWarps * 32)
hh_back_wide_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
                    int require_active, int require_phase, int final_pass, const double* __restrict__ W,
                    const double* __restrict__ td, long long vstride, const double* __restrict__ Z,
                    T* __restrict__ C) {
  extern __shared__ __align__(16) double bwm[];
  constexpr int kSpw = 32 / kCols, kS = kWideWarps * kSpw, kT = kWideWarps * 32;
  const int mi = list[blockIdx.x];
  if (require_active && st[mi].status != kActive) return;
  if (require_phase >= 0 && st[mi].phase != require_phase) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  int lo, hi;
  hh_range(n, mol.nocc, final_pass, &lo, &hi);
  const int k = hi - lo;
  const int cb = blockIdx.y * kCols;
  if (cb >= k) return;
  T* zs = reinterpret_cast<T*>(bwm);          // n x kCols
  T* red = zs + (long long)n * kCols;          // kWideWarps x kCols
  T* dotv = red + kWideWarps * kCols;          // kCols
  T* us = dotv + kCols;                        // the staged reflector (n)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c = lane % kCols, slice = warp * kSpw + lane / kCols;
  const double* Zm = Z + mol.mat0;
  const double* Wm = W + mol.mat0;
  const double* tt = td + mol.vec0 + 2 * vstride;
  const int col = cb + c;
  for (int i = slice; i < n; i += kS) zs[i * kCols + c] = col < k ? (T)Zm[(long long)i * k + col] : (T)0;
  if (n >= 3)
    for (int i = n - 2 + tid; i < n; i += kT) us[i] = (T)Wm[(long long)(n - 3) * n + i];
  __syncthreads();
  for (int j = n - 3; j >= 0; --j) {
    // reflector j - 1 (entries j .. n-1) into registers
    double pre[kBackPre];
    if (j > 0) {
      const double* ug = Wm + (long long)(j - 1) * n;
#pragma unroll
      for (int q = 0; q < kBackPre; ++q) {
        const int i = j + tid + q * kT;
        pre[q] = i < n ? ug[i] : 0.0;
      }
    }
    const T tau = (T)tt[j];
    if (tau != (T)0) {
      const int i0 = j + 1 + ((slice - (j + 1)) & (kS - 1));
      T part = 0;
      for (int i = i0; i < n; i += kS) part = fma(us[i], zs[i * kCols + c], part);
#pragma unroll
      for (int o = kCols; o < 32; o <<= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      if (lane < kCols) red[warp * kCols + lane] = part;
      __syncthreads();
      if (tid < kCols) {
        T sum = red[tid];
#pragma unroll
        for (int q = 1; q < kWideWarps; ++q) sum += red[q * kCols + tid];
        dotv[tid] = tau * sum;
      }
      __syncthreads();
      const T dt = dotv[c];
      for (int i = i0; i < n; i += kS) {
        T* z = zs + i * kCols + c;
        *z = fma(-dt, us[i], *z);
      }
    }
    __syncthreads();   // every thread is done with reflector j
    if (j > 0) {
#pragma unroll
      for (int q = 0; q < kBackPre; ++q) {
        const int i = j + tid + q * kT;
        if (i < n) us[i] = (T)pre[q];
      }
    }
    __syncthreads();
  }
  T* Cm = C + mol.mat0;
  for (int q = warp; q < kCols; q += kWideWarps) {
    const int cc = cb + q;
    if (cc >= k) break;
    T sgn = 1;
    if (final_pass) {
      // component sum in index order (src/wrappers/Lapack.cpp:139-150)
      T s = 0;
      if (lane == 0)
        for (int i = 0; i < n; ++i) s += zs[i * kCols + q];
      s = __shfl_sync(0xffffffffu, s, 0);
      sgn = s < (T)0 ? (T)-1 : (T)1;
    }
    T* row = Cm + (long long)(lo + cc) * n;
    for (int i = lane; i < n; i += 32) row[i] = sgn * zs[i * kCols + q];
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
namespace {

int optin_smem() {
  static int optin = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  });
  return optin;
}

int num_sms() {
  static int nsm = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  });
  return nsm;
}

constexpr int kStaticSmem = 20 * 1024;   // the kernels' static shared arrays, rounded up

size_t tridiag_grid_smem(int n) { return 3 * (size_t)n * sizeof(double); }
size_t orth_grid_smem(int k) { return (size_t)kOrthChunk * 32 * sizeof(double) + 2 * (size_t)k * sizeof(int); }
template <typename T>
size_t back_wide_smem(int n, int cols) {
  return ((size_t)n * cols + kWideWarps * cols + cols + (size_t)n) * sizeof(T);
}
template <typename T>
int back_wide_cols(int n) {
  for (int c : {16, 8, 4})
    if (back_wide_smem<T>(n, c) <= (size_t)optin_smem()) return c;
  return 0;
}

void set_attributes() {
  static std::once_flag once;
  std::call_once(once, [] {
    const int o = optin_smem();
    cudaFuncSetAttribute(hh_tridiag_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, o - kStaticSmem);
    cudaFuncSetAttribute(tri_orth_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, o - kStaticSmem);
    cudaFuncSetAttribute(hh_back_wide_kernel<double, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, o);
    cudaFuncSetAttribute(hh_back_wide_kernel<double, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, o);
    cudaFuncSetAttribute(hh_back_wide_kernel<double, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, o);
    cudaFuncSetAttribute(hh_back_wide_kernel<float, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, o);
    cudaFuncSetAttribute(hh_back_wide_kernel<float, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, o);
    cudaFuncSetAttribute(hh_back_wide_kernel<float, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, o);
  });
}

void cooperative(const void* fn, int nctas, int nlist, size_t smem, void** args, cudaStream_t s, unsigned* bars) {
  cuda_check(cudaMemsetAsync(bars, 0, 4 * sizeof(unsigned) * (size_t)nlist, s), "grid barrier reset");
  cuda_check(cudaLaunchCooperativeKernel(fn, dim3(nctas), dim3(kGridThreads), args, smem, s), "cooperative launch");
}

template <typename T>
void launch_back_wide(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                      int require_active, int require_phase, int final_pass, const double* W, const double* td,
                      long long vstride, const double* Z, T* C, cudaStream_t s) {
  const int cols = back_wide_cols<T>(max_n);
  const size_t sh = back_wide_smem<T>(max_n, cols);
  const dim3 g(nlist, (max_k + cols - 1) / cols);
  if (cols == 16)
    hh_back_wide_kernel<T, 16><<<g, kWideWarps * 32, sh, s>>>(mols, list, st, require_active, require_phase,
                                                               final_pass, W, td, vstride, Z, C);
  else if (cols == 8)
    hh_back_wide_kernel<T, 8><<<g, kWideWarps * 32, sh, s>>>(mols, list, st, require_active, require_phase,
                                                              final_pass, W, td, vstride, Z, C);
  else
    hh_back_wide_kernel<T, 4><<<g, kWideWarps * 32, sh, s>>>(mols, list, st, require_active, require_phase,
                                                              final_pass, W, td, vstride, Z, C);
}

}  // namespace

int hh_grid_max_n() {
  static int nmax = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    const size_t lim = (size_t)(optin_smem() - kStaticSmem);
    int n = 8;
    while (tridiag_grid_smem(n + 1) <= lim && orth_grid_smem(n + 1) <= lim && back_wide_cols<double>(n + 1) > 0 &&
           back_wide_cols<float>(n + 1) > 0 && n + 1 <= kBackPre * kWideWarps * 32)
      ++n;
    nmax = n;
  });
  return nmax;
}

int hh_grid_ctas() { return num_sms(); }

int hh_grid_assign(const int* n, int count, int G, int* map3) {
  if (count < 1 || count > G) return 0;
  // CTAs in proportion to N^3 (the tridiagonalisation's work), at least one each
  std::vector<double> c(count);
  std::vector<int> a(count);
  double tot = 0.0;
  for (int i = 0; i < count; ++i) { c[i] = (double)n[i] * n[i] * n[i]; tot += c[i]; }
  int used = 0;
  for (int i = 0; i < count; ++i) { a[i] = std::max(1, (int)(G * c[i] / tot)); used += a[i]; }
  while (used > G) {   // only possible through the minimum of one
    int best = -1;
    for (int i = 0; i < count; ++i)
      if (a[i] > 1 && (best < 0 || a[i] > a[best])) best = i;
    --a[best];
    --used;
  }
  while (used < G) {
    int best = 0;
    for (int i = 1; i < count; ++i)
      if (c[i] / a[i] > c[best] / a[best]) best = i;
    ++a[best];
    ++used;
  }
  int q = 0;
  for (int i = 0; i < count; ++i)
    for (int j = 0; j < a[i]; ++j, ++q) {
      map3[3 * q] = i;
      map3[3 * q + 1] = j;
      map3[3 * q + 2] = a[i];
    }
  return q;
}

void launch_hh_grid_tridiag(const DevMol* mols, const int* list, const int* map3, int nctas, int nlist, MolState* st,
                            int require_active, const double* F, double* W, double* td, long long vstride,
                            double* Aws, double* scratch, unsigned* bars, cudaStream_t s) {
  if (nlist <= 0) return;
  set_attributes();
  // the dynamic shared memory of the largest basis served (each CTA reads
  // its molecule's n on the device)
  const size_t sh = tridiag_grid_smem(hh_grid_max_n());
  const int3* map = reinterpret_cast<const int3*>(map3);
  void* args[] = {(void*)&mols, (void*)&list, (void*)&map, (void*)&st, (void*)&require_active, (void*)&F,
                  (void*)&W, (void*)&td, (void*)&vstride, (void*)&Aws, (void*)&scratch, (void*)&bars};
  cooperative((const void*)hh_tridiag_grid_kernel, nctas, nlist, sh, args, s, bars);
}

void launch_hh_grid_orth(const DevMol* mols, const int* list, const int* map3, int nctas, int nlist, int max_k,
                         MolState* st, int require_active, int final_pass, const double* td, long long vstride,
                         double* eps, double* Z, double* scratch, unsigned* bars, cudaStream_t s) {
  if (nlist <= 0 || max_k < 2) return;
  set_attributes();
  const size_t sh = orth_grid_smem(max_k);
  const int3* map = reinterpret_cast<const int3*>(map3);
  void* args[] = {(void*)&mols, (void*)&list, (void*)&map, (void*)&st, (void*)&require_active, (void*)&final_pass,
                  (void*)&td, (void*)&vstride, (void*)&eps, (void*)&Z, (void*)&scratch, (void*)&bars};
  cooperative((const void*)tri_orth_grid_kernel, nctas, nlist, sh, args, s, bars);
}

void launch_hh_grid_back(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                         int require_active, int final_pass, int mixed, const double* W, const double* td,
                         long long vstride, const double* Z, double* C, float* C32, cudaStream_t s) {
  if (nlist <= 0 || max_k <= 0) return;
  set_attributes();
  const int fp64_phase = (mixed && !final_pass) ? 1 : -1;
  launch_back_wide<double>(mols, list, nlist, max_n, max_k, st, require_active, fp64_phase, final_pass, W, td,
                           vstride, Z, C, s);
  if (fp64_phase == 1)
    launch_back_wide<float>(mols, list, nlist, max_n, max_k, st, require_active, 0, final_pass, W, td, vstride, Z,
                            C32, s);
}

}  // namespace nddo
