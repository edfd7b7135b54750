// Kernel (d), FP64 path: batched symmetric eigensolver by Householder
// tridiagonalisation, Sturm bisection, inverse iteration and
// back-transformation.
//
// Stands in for MolDS's Lapack::Dsyevd (src/wrappers/Lapack.cpp:102-160,
// called at src/cndo/Cndo2.cpp:652-655).  Output convention is the
// reference's: eigenvalues ascending, eigenvectors as ROWS of C with each
// row's component sum made >= 0 (Lapack.cpp:141-150).
//
// Why this algorithm on GB300: the chip issues FP64 at about two FMAs per
// clock per SM (1.2 TFLOP/s over 152 SMs), so an FP64 eigensolve is bound by
// its FP64 operation count, not by memory.  A warm-started cyclic Jacobi costs
// ~4 N^3 FMAs per sweep (3-4 sweeps per SCF iteration) plus the 2 N^3 of the
// warm-start transform.  Householder tridiagonalisation costs (2/3) N^3 FMAs,
// and during the SCF the density needs only the smaller of the occupied and
// virtual eigenvector sets (k vectors): the back-transformation costs N^2 k
// FMAs and P = 2 X^T X (or 2 I - 2 X^T X) N^2 k / 2.  All N eigenpairs are
// formed once, after the last iteration, for the MO energies and vectors.
//
// Kernels (each molecule's work depends only on its own data, so results are
// bitwise independent of the batch):
//   hh_tridiag_kernel   one CTA per molecule: A = Q T Q^T with the packed lower
//                       triangle in shared memory (or a global workspace for
//                       large N); reflector j goes to row j of W, d / e / tau
//                       to the tridiagonal arena
//   tri_vectors_kernel  one thread per wanted index: the eigenvalue of T by
//                       bisection on a division-free Sturm sequence, then two
//                       steps of inverse iteration with a partial-pivoting LU of
//                       T - lambda I (as LAPACK dstebz / dstein do)
//   tri_orth_kernel     one CTA per molecule: classical Gram-Schmidt, applied
//                       twice, within clusters of close eigenvalues (gap below
//                       1e-3 ||T||_1, dstein's criterion)
//   hh_back_kernel      X = Q Z, 32 columns per CTA, reflectors applied in
//                       reverse order; X written as rows of C (sign-fixed in the
//                       final pass)
#include <cuda_runtime.h>
#include <algorithm>
#include <mutex>
#include "nddo_batch.cuh"
#include "kernels.h"
#include "tuning.h"
#include "tridiag.cuh"

namespace nddo {

constexpr int kHhMaxThreads = 1024;   // the CTA size comes from the tuning table (256, 512 or 1024)
constexpr int kVecThreads = 32;   // one warp: 16 lane pairs, 16 eigenpairs per CTA
constexpr int kOrthThreads = 256;
constexpr size_t kOrthStaticSmem = (1024 + kOrthThreads / 32 + 1) * sizeof(double) + 1024;   // and some slack
constexpr int kBackCols = 32, kBackWarps = 8;

size_t hh_tridiag_smem_bytes(int n, bool a_in_smem) {
  size_t d = 3 * (size_t)n + 8;
  if (a_in_smem) d += (size_t)n * (n + 1) / 2;
  return d * sizeof(double);
}

static int g_hh_smem_max_n = -1;
static std::once_flag g_hh_once;

int hh_smem_max_n() {
  std::call_once(g_hh_once, [] {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    int n = 8;
    while (hh_tridiag_smem_bytes(n + 1, true) <= (size_t)optin) ++n;
    g_hh_smem_max_n = n;
  });
  return g_hh_smem_max_n;
}

// ---------------------------------------------------------------------------
// Tridiagonalisation (LAPACK dsytd2 'L' semantics, own parallel layout).
// Step k: x = A[k+1:, k]; H = I - tau u u^T with u = (1, x_1 s, ..., x_{m-1} s)
// zeroes x below its first entry; p = tau A22 u, w = p - (tau/2)(p.u) u,
// A22 <- A22 - u w^T - w u^T (lower triangle only).
// ---------------------------------------------------------------------------
template <bool kSmem>
__global__ void __launch_bounds__(kHhMaxThreads)
hh_tridiag_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
                  int require_active, const double* __restrict__ F, double* __restrict__ W, double* __restrict__ td,
                  long long vstride, double* __restrict__ Aws, int max_n_served) {
  extern __shared__ __align__(16) double hsm[];
  const int mi = list[blockIdx.x];
  if (require_active && st[mi].status != kActive) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  if (n > max_n_served) return;   // served by the whole-GPU kernel (tridiag_grid.cu)
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31, nwarps = nth >> 5;
  double* A = kSmem ? hsm : Aws + mol.mat0;
  double* v = kSmem ? hsm + (long long)n * (n + 1) / 2 : hsm;
  double* p = v + n;
  double* w = p + n;
  double* sc = w + n;   // [0] tau of the current step
  const double* Fm = F + mol.mat0;
  double* Wm = W + mol.mat0;
  double* dd = td + mol.vec0;
  double* ee = dd + vstride;
  double* tt = ee + vstride;

  for (int i = warp; i < n; i += nwarps)
    for (int j = lane; j <= i; j += 32) A[tri_off(i) + j] = Fm[(long long)i * n + j];
  __syncthreads();

  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - 1 - k;   // trailing size
    const int r0 = k + 1;      // first trailing row / column
    if (warp == 0) {
      double s = 0.0;
      for (int i = 1 + lane; i < m; i += 32) {
        const double x = A[tri_off(r0 + i) + k];
        s = fma(x, x, s);
      }
      s = warp_sum_d(s);
      const double alpha = A[tri_off(r0) + k];
      double tau = 0.0, beta = alpha, scal = 0.0;
      if (s != 0.0) {
        const double nrm = sqrt(fma(alpha, alpha, s));
        beta = alpha >= 0.0 ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      for (int i = lane; i < m; i += 32) {
        const double vi = i == 0 ? 1.0 : A[tri_off(r0 + i) + k] * scal;
        v[i] = vi;
        Wm[(long long)k * n + r0 + i] = vi;
      }
      if (lane == 0) {
        dd[k] = A[tri_off(k) + k];
        ee[k] = beta;
        tt[k] = tau;
        sc[k & 1] = tau;   // two slots: a warp may still read this step's value when warp 0 starts the next
      }
    }
    __syncthreads();
    const double tau = sc[k & 1];
    if (tau == 0.0) continue;   // uniform: H = I, nothing to update
    // p = tau A22 v: a group of g lanes per row (g a power of two, g * rows <= threads)
    int gsh = 0;
    while (gsh < 5 && (m << (gsh + 1)) <= nth) ++gsh;
    const int g = 1 << gsh, ngrp = nth >> gsh, grp = tid >> gsh, gl = tid & (g - 1);
    for (int i0 = 0; i0 < m; i0 += ngrp) {
      const int i = i0 + grp;
      double s = 0.0;
      if (i < m) {
        const int R = r0 + i;
        const int oR = tri_off(R) + r0;
        for (int j = gl; j < m; j += g) {
          const double a = j <= i ? A[oR + j] : A[tri_off(r0 + j) + R];
          s = fma(a, v[j], s);
        }
      }
      for (int o = g >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (i < m && gl == 0) p[i] = tau * s;
    }
    __syncthreads();
    if (warp == 0) {
      double s = 0.0;
      for (int i = lane; i < m; i += 32) s = fma(p[i], v[i], s);
      s = warp_sum_d(s);
      const double c = 0.5 * tau * s;
      for (int i = lane; i < m; i += 32) w[i] = fma(-c, v[i], p[i]);
    }
    __syncthreads();
    // A22 -= v w^T + w v^T on the lower triangle; rows i and m-1-i share a warp
    const int npair = (m + 1) >> 1;
    for (int q = warp; q < npair; q += nwarps) {
      const int i1 = q, i2 = m - 1 - q;
      const int len1 = i1 + 1, len = i2 == i1 ? len1 : len1 + i2 + 1;
      for (int t = lane; t < len; t += 32) {
        const bool first = t < len1;
        const int i = first ? i1 : i2;
        const int j = first ? t : t - len1;
        double* a = A + tri_off(r0 + i) + r0 + j;
        *a = fma(-v[i], w[j], fma(-w[i], v[j], *a));
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      dd[n - 2] = A[tri_off(n - 2) + n - 2];
      ee[n - 2] = A[tri_off(n - 1) + n - 2];
      tt[n - 2] = 0.0;
    }
    dd[n - 1] = A[tri_off(n - 1) + n - 1];
    ee[n - 1] = 0.0;
    tt[n - 1] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Tridiagonal eigenpairs.
// ---------------------------------------------------------------------------

// Sturm counts and the characteristic polynomial, by a lane pair.
//
// The count of eigenvalues of T below x is the number of sign changes of the
// leading principal minors P_0 = 1, P_1 = d_0 - x,
// P_{i+1} = (d_i - x) P_i - e_{i-1}^2 P_{i-1} (a zero minor takes the sign
// opposite to its predecessor); no divisions, and the pair (P_i, P_{i+1}) is
// rescaled by a power of two when it leaves [2^-256, 2^256].  A lane pair
// splits it as a twisted factorisation of T - x I at r = n/2 - 1: side 0 runs
// P_1 .. P_{r+1} and counts the changes of P_0 .. P_r; side 1 runs the
// trailing minors Q_i = det(T[i.., i..] - x I), Q_{n-1} .. Q_{r+1}, and counts
// the changes of Q_n = 1 .. Q_{r+1}; the pivot at the twist,
// gamma_r = det(T - x I) / (P_r Q_{r+1}) with
// det = Q_{r+1} P_{r+1} - e_r^2 P_r Q_{r+2}, adds one when negative (or zero).
// Both lanes do n/2 steps: half the latency of a count at the same FP64 work.
// With kDeriv the first and second x-derivatives run alongside (same
// recurrence: P'_{i+1} = (d_i - x) P'_i - P_i - e^2 P'_{i-1},
// P''_{i+1} = (d_i - x) P''_i - 2 P'_i - e^2 P''_{i-1}) and are rescaled with
// the minors, so det, det' and det'' share one scale factor.
template <bool kDeriv>
struct MinorPair {
  double p0, p1, q0, q1, r0, r1;   // value, first and second derivative of (P_{i-1}, P_i)
  __device__ __forceinline__ void step(double d, double e2, double x, int& s_prev, int& cnt, bool count) {
    const double t = d - x;
    const double p2 = fma(t, p1, -(e2 * p0));
    if (kDeriv) {
      const double q2 = fma(t, q1, -fma(e2, q0, p1));
      const double r2 = fma(t, r1, -fma(e2, r0, 2.0 * q1));
      q0 = q1; q1 = q2;
      r0 = r1; r1 = r2;
    }
    if (count) {
      const long long b = __double_as_longlong(p2);
      const int s = ((b << 1) == 0) ? (s_prev ^ 1) : (int)((unsigned long long)b >> 63);
      cnt += s != s_prev;
      s_prev = s;
    }
    p0 = p1;
    p1 = p2;
  }
  __device__ __forceinline__ void rescale() {
    const int e1 = (int)((__double_as_longlong(p0) >> 52) & 0x7ff);
    const int e0 = (int)((__double_as_longlong(p1) >> 52) & 0x7ff);
    const int em = e0 > e1 ? e0 : e1;
    if (em != 0 && (em > 1023 + 256 || em < 1023 - 256)) {
      const double scale = __longlong_as_double((long long)(2046 - em) << 52);
      p0 *= scale;
      p1 *= scale;
      if (kDeriv) { q0 *= scale; q1 *= scale; r0 *= scale; r1 *= scale; }
    }
  }
};

// One lane's half.  v[0..1] = (P_r, P_{r+1}) on side 0, (Q_{r+2}, Q_{r+1}) on
// side 1, their derivatives in v[2..3] and v[4..5]; sg = sign bit of P_r /
// Q_{r+1} as counted.
template <bool kDeriv>
__device__ __forceinline__ int sturm_half(const double* __restrict__ d, const double* __restrict__ e2, int n, int r,
                                          int side, double x, double* v, int* sg) {
  MinorPair<kDeriv> m;
  m.p0 = 1.0; m.q0 = 0.0; m.q1 = -1.0; m.r0 = 0.0; m.r1 = 0.0;
  int s_prev = 0, cnt = 0;
  if (side == 0) {
    m.p1 = d[0] - x;
    const long long b = __double_as_longlong(m.p1);
    const int s1 = ((b << 1) == 0) ? 1 : (int)((unsigned long long)b >> 63);
    if (r >= 1) { cnt = s1; s_prev = s1; }
    // P_2 .. P_r counted (four steps between range checks: a step changes |P|
    // by a factor far inside the 2^+-256 margin), then P_{r+1} uncounted
    int i = 1;
    for (; i + 4 <= r; i += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) m.step(d[i + u], e2[i + u - 1], x, s_prev, cnt, true);
      m.rescale();
    }
    for (; i < r; ++i) {
      m.step(d[i], e2[i - 1], x, s_prev, cnt, true);
      m.rescale();
    }
    if (r >= 1) {
      const int sr = s_prev;
      m.step(d[r], e2[r - 1], x, s_prev, cnt, false);   // (p0, p1) = (P_r, P_{r+1})
      *sg = sr;
    } else {
      *sg = 0;   // (P_0, P_1)
    }
  } else {
    m.p1 = d[n - 1] - x;   // Q_{n-1}
    const long long b = __double_as_longlong(m.p1);
    s_prev = ((b << 1) == 0) ? 1 : (int)((unsigned long long)b >> 63);
    cnt = s_prev;
    // Q_i = (d_i - x) Q_{i+1} - e_i^2 Q_{i+2}, i = n-2 down to r+1
    int i = n - 2;
    for (; i - 4 >= r; i -= 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) m.step(d[i - u], e2[i - u], x, s_prev, cnt, true);
      m.rescale();
    }
    for (; i > r; --i) {
      m.step(d[i], e2[i], x, s_prev, cnt, true);
      m.rescale();
    }
    *sg = s_prev;
  }
  v[0] = m.p0; v[1] = m.p1;
  if (kDeriv) { v[2] = m.q0; v[3] = m.q1; v[4] = m.r0; v[5] = m.r1; }
  return cnt;
}

// One evaluation at x by a lane pair (both lanes return the same values): the
// count of eigenvalues below x and, with kDeriv, det(T - x I) with its first
// two derivatives, scaled by one common power of two.
struct TriEval {
  int count;
  double f, f1, f2;
};

template <bool kDeriv>
__device__ __forceinline__ TriEval pair_eval(const double* __restrict__ d, const double* __restrict__ e2, int n,
                                             int r, int side, double e2r, double x) {
  double v[6], w[6];
  int sg;
  const int cp = sturm_half<kDeriv>(d, e2, n, r, side, x, v, &sg);
  const int co = __shfl_xor_sync(0xffffffffu, cp, 1);
  const int so = __shfl_xor_sync(0xffffffffu, sg, 1);
#pragma unroll
  for (int k = 0; k < (kDeriv ? 6 : 2); ++k) w[k] = __shfl_xor_sync(0xffffffffu, v[k], 1);
  const double* P = side ? w : v;   // (P_r, P_{r+1}) and derivatives
  const double* Q = side ? v : w;   // (Q_{r+2}, Q_{r+1}) and derivatives
  const int sP = side ? so : sg, sQ = side ? sg : so;
  TriEval out;
  out.f = fma(Q[1], P[1], -(e2r * P[0] * Q[0]));
  const long long bd = __double_as_longlong(out.f);
  const int gneg = ((bd << 1) == 0) ? 1 : ((int)((unsigned long long)bd >> 63) ^ sP ^ sQ);
  out.count = cp + co + gneg;
  out.f1 = out.f2 = 0.0;
  if (kDeriv) {
    out.f1 = fma(Q[3], P[1], Q[1] * P[3]) - e2r * fma(P[2], Q[0], P[0] * Q[2]);
    out.f2 = fma(Q[5], P[1], fma(2.0 * Q[3], P[3], Q[1] * P[5])) -
             e2r * fma(P[4], Q[0], fma(2.0 * P[2], Q[2], P[0] * Q[4]));
  }
  return out;
}

// The Sturm count of the FP32 copy of T (df, e2f) at x, split across the lane
// pair as pair_eval: the same recurrences on FP32's pipe, which has 64 times
// the FP64 one's throughput.  Such a count is exact for a perturbation of T
// of some ten eps_32 ||T||, so it only ever proposes starting points; every
// decision is taken on FP64 counts.
__device__ __forceinline__ int pair_count_f32(const float* __restrict__ df, const float* __restrict__ e2f, int n,
                                              int r, int side, float e2r, float x) {
  float p0 = 1.0f, p1;
  int s_prev = 0, cnt = 0, sg = 0;
  auto sgn = [](float v) { const unsigned b = __float_as_uint(v); return (b << 1) == 0 ? -1 : (int)(b >> 31); };
  auto step = [&](float dd, float ee, bool count) {
    const float p2 = fmaf(dd - x, p1, -(ee * p0));
    if (count) {
      const int sv = sgn(p2);
      const int sn = sv < 0 ? (s_prev ^ 1) : sv;   // a zero takes the sign opposite to its predecessor's
      cnt += sn != s_prev;
      s_prev = sn;
    }
    p0 = p1;
    p1 = p2;
    const int e0 = (int)((__float_as_uint(p0) >> 23) & 0xff), e1 = (int)((__float_as_uint(p1) >> 23) & 0xff);
    const int em = e0 > e1 ? e0 : e1;
    if (em != 0 && (em > 127 + 40 || em < 127 - 40)) {
      const float scale = __uint_as_float((unsigned)(254 - em) << 23);   // 2^(127 - em)
      p0 *= scale;
      p1 *= scale;
    }
  };
  if (side == 0) {
    p1 = df[0] - x;
    const int s1 = sgn(p1) < 0 ? 1 : sgn(p1);
    if (r >= 1) { cnt = s1; s_prev = s1; }
    for (int i = 1; i < r; ++i) step(df[i], e2f[i - 1], true);
    if (r >= 1) {
      sg = s_prev;
      step(df[r], e2f[r - 1], false);   // (p0, p1) = (P_r, P_{r+1})
    }
  } else {
    p1 = df[n - 1] - x;
    s_prev = sgn(p1) < 0 ? 1 : sgn(p1);
    cnt = s_prev;
    for (int i = n - 2; i > r; --i) step(df[i], e2f[i], true);
    sg = s_prev;
  }
  const int co = __shfl_xor_sync(0xffffffffu, cnt, 1);
  const int so = __shfl_xor_sync(0xffffffffu, sg, 1);
  const float w0 = __shfl_xor_sync(0xffffffffu, p0, 1);
  const float w1 = __shfl_xor_sync(0xffffffffu, p1, 1);
  const float P0 = side ? w0 : p0, P1 = side ? w1 : p1;
  const float Q0 = side ? p0 : w0, Q1 = side ? p1 : w1;
  const int sP = side ? so : sg, sQ = side ? sg : so;
  const float f = fmaf(Q1, P1, -(e2r * P0 * Q0));
  const int sf = sgn(f);
  return cnt + co + (sf < 0 ? 1 : (sf ^ sP ^ sQ));
}

// uniform pseudo-random value in [-0.5, 0.5): the start vector of inverse iteration
__device__ __forceinline__ double start_entry(unsigned int idx, unsigned int i) {
  unsigned long long z = ((unsigned long long)idx << 32) ^ (unsigned long long)(i * 0x9E3779B9u) ^ 0x2545F4914F6CDD1DULL;
  z ^= z >> 33; z *= 0xff51afd7ed558ccdULL;
  z ^= z >> 33; z *= 0xc4ceb9fe1a85ec53ULL;
  z ^= z >> 33;
  const double one_two = __longlong_as_double((long long)(0x3FF0000000000000ULL | (z >> 12)));
  return one_two - 1.5;
}

// One solve (T - lam I) y = b with the stored factors (forward elimination
// with the row interchanges, then back substitution), in place in x (element
// i at x[i * ld]).  b is the pseudo-random start vector (start) or scale * x;
// returns sum y_i^2, so the normalisation costs no extra pass.
// Both sweeps load the operands of kSolveBlock rows before storing their
// results: every row reads x only at rows no earlier store of the sweep has
// written (ld >= 1), so the order is the plain loop's, and the loads of a
// block overlap instead of each waiting for the previous row's store (the
// factors and the vector may live in L2, in the global scratch).
constexpr int kSolveBlock = 8;

template <typename PivT>
__device__ __forceinline__ double tri_solve(int n, int ld, double* __restrict__ x, const double* __restrict__ fl,
                                            const double* __restrict__ fu1i, const double* __restrict__ fu2,
                                            const PivT* __restrict__ piv, const double* __restrict__ e, bool start,
                                            double scale, unsigned idx) {
  double cb = start ? start_entry(idx, 0) : scale * x[0];
  int i = 0;
  for (; i + kSolveBlock < n; i += kSolveBlock) {   // rows i .. i + kSolveBlock - 1, all below n - 1
    double bn[kSolveBlock], l[kSolveBlock];
    bool pv[kSolveBlock];
#pragma unroll
    for (int u = 0; u < kSolveBlock; ++u) {
      const long long o = (long long)(i + u) * ld;
      bn[u] = start ? start_entry(idx, (unsigned)(i + u + 1)) : scale * x[o + ld];
      l[u] = fl[o];
      pv[u] = piv[o] != (PivT)0;
    }
#pragma unroll
    for (int u = 0; u < kSolveBlock; ++u) {
      const long long o = (long long)(i + u) * ld;
      if (pv[u]) { x[o] = bn[u]; cb = fma(-l[u], bn[u], cb); }
      else { x[o] = cb; cb = fma(-l[u], cb, bn[u]); }
    }
  }
  for (; i + 1 < n; ++i) {
    const long long o = (long long)i * ld;
    const double bn = start ? start_entry(idx, (unsigned)(i + 1)) : scale * x[o + ld];
    const double l = fl[o];
    if (piv[o]) { x[o] = bn; cb = fma(-l, bn, cb); }
    else { x[o] = cb; cb = fma(-l, cb, bn); }
  }
  const long long on = (long long)(n - 1) * ld;
  double x2 = 0.0, x1 = cb * fu1i[on];
  x[on] = x1;
  double ss = x1 * x1;
  i = n - 2;
  for (; i - kSolveBlock + 1 >= 0; i -= kSolveBlock) {   // rows i down to i - kSolveBlock + 1
    double u3[kSolveBlock], f2[kSolveBlock], xv[kSolveBlock], f1[kSolveBlock];
#pragma unroll
    for (int u = 0; u < kSolveBlock; ++u) {
      const long long o = (long long)(i - u) * ld;
      u3[u] = piv[o] ? e[i - u + 1] : 0.0;
      f2[u] = fu2[o];
      xv[u] = x[o];
      f1[u] = fu1i[o];
    }
#pragma unroll
    for (int u = 0; u < kSolveBlock; ++u) {
      const double xi = fma(-u3[u], x2, fma(-f2[u], x1, xv[u])) * f1[u];
      x[(long long)(i - u) * ld] = xi;
      ss = fma(xi, xi, ss);
      x2 = x1;
      x1 = xi;
    }
  }
  for (; i >= 0; --i) {
    const long long o = (long long)i * ld;
    const double u3 = piv[o] ? e[i + 1] : 0.0;
    const double xi = fma(-u3, x2, fma(-fu2[o], x1, x[o])) * fu1i[o];
    x[o] = xi;
    ss = fma(xi, xi, ss);
    x2 = x1;
    x1 = xi;
  }
  return ss;
}

// Inverse iteration for eigenvalue lam: T - lam I = P L U with partial
// pivoting (as LAPACK dlagtf), then two solves from a pseudo-random start;
// the normalised vector goes to out[i * out_ld].  The factors and the vector
// live at stride ld in shared memory or in the global scratch arenas.
template <typename PivT>
__device__ __forceinline__ void inverse_iteration(int n, int ld, const double* __restrict__ d,
                                                  const double* __restrict__ e, double lam, double tiny, unsigned idx,
                                                  double* __restrict__ fl, double* __restrict__ fu1i,
                                                  double* __restrict__ fu2, PivT* __restrict__ piv,
                                                  double* __restrict__ x, double* __restrict__ out, long long out_ld) {
  double cc = d[0] - lam, s1 = n > 1 ? e[0] : 0.0;
  for (int i = 0; i + 1 < n; ++i) {
    const long long o = (long long)i * ld;
    const double ei = e[i];
    const double a1 = d[i + 1] - lam;
    const double e1 = i + 2 < n ? e[i + 1] : 0.0;
    if (fabs(ei) > fabs(cc)) {
      const double r = 1.0 / ei;
      const double l = cc * r;
      fl[o] = l; fu1i[o] = r; fu2[o] = a1; piv[o] = (PivT)1;
      cc = fma(-l, a1, s1);
      s1 = -l * e1;
    } else {
      if (cc == 0.0) cc = tiny;
      const double r = 1.0 / cc;
      const double l = ei * r;
      fl[o] = l; fu1i[o] = r; fu2[o] = s1; piv[o] = (PivT)0;
      cc = fma(-l, s1, a1);
      s1 = e1;
    }
  }
  if (cc == 0.0) cc = tiny;
  fu1i[(long long)(n - 1) * ld] = 1.0 / cc;
  const double s1s = tri_solve(n, ld, x, fl, fu1i, fu2, piv, e, true, 1.0, idx);
  const double r1 = s1s > 0.0 ? rsqrt(s1s) : 0.0;
  const double s2s = tri_solve(n, ld, x, fl, fu1i, fu2, piv, e, false, r1, idx);
  const double r2 = s2s > 0.0 ? rsqrt(s2s) : 0.0;
  // out may be x itself (the global scratch path): each block's loads come
  // before its stores, and every element is read before it is written
  int i = 0;
  for (; i + kSolveBlock <= n; i += kSolveBlock) {
    double v[kSolveBlock];
#pragma unroll
    for (int u = 0; u < kSolveBlock; ++u) v[u] = x[(long long)(i + u) * ld];
#pragma unroll
    for (int u = 0; u < kSolveBlock; ++u) out[(long long)(i + u) * out_ld] = v[u] * r2;
  }
  for (; i < n; ++i) out[(long long)i * out_ld] = x[(long long)i * ld] * r2;
}

// grid: (list entry, chunk of `pairs` <= kVecPerCta indices); a lane pair per wanted
// index for its eigenvalue, the pair's first lane for its inverse iteration
constexpr int kVecPerCta = kVecThreads / 2;

__global__ void __launch_bounds__(kVecThreads)
tri_vectors_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
                   int require_active, int final_pass, const double* __restrict__ td, long long vstride,
                   double* __restrict__ eps, double* __restrict__ Z, double* __restrict__ S0, double* __restrict__ S1,
                   double* __restrict__ S2, double* __restrict__ S3, int vec_smem, int pairs) {
  extern __shared__ __align__(16) double vsm[];
  const int mi = list[blockIdx.x];
  if (require_active && st[mi].status != kActive) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  int lo, hi;
  hh_range(n, mol.nocc, final_pass, &lo, &hi);
  const int k = hi - lo;
  const int c0 = blockIdx.y * pairs;
  if (c0 >= k) return;
  double* d = vsm;
  double* e = d + n;
  double* e2 = e + n;
  double* red = e2 + n;   // 2 * (kVecThreads / 32)
  float* df = reinterpret_cast<float*>(red + 2 * (kVecThreads / 32));   // FP32 copy of d and e^2: n doubles' room
  float* e2f = df + n;
  const double* tdd = td + mol.vec0;
  const double* tde = tdd + vstride;
  const int tid = threadIdx.x;
  // Gershgorin interval and the 1-norm of T
  double gl = 1e300, gu = -1e300;
  for (int i = tid; i < n; i += kVecThreads) {
    const double di = tdd[i];
    const double ei = i + 1 < n ? tde[i] : 0.0;
    const double em = i > 0 ? tde[i - 1] : 0.0;
    d[i] = di;
    e[i] = ei;
    e2[i] = ei * ei;
    df[i] = (float)di;
    e2f[i] = (float)(ei * ei);
    const double r = fabs(ei) + fabs(em);
    gl = fmin(gl, di - r);
    gu = fmax(gu, di + r);
  }
  for (int o = 16; o > 0; o >>= 1) {
    gl = fmin(gl, __shfl_xor_sync(0xffffffffu, gl, o));
    gu = fmax(gu, __shfl_xor_sync(0xffffffffu, gu, o));
  }
  if ((tid & 31) == 0) { red[2 * (tid >> 5)] = gl; red[2 * (tid >> 5) + 1] = gu; }
  __syncthreads();
  gl = red[0];
  gu = red[1];
  for (int w = 1; w < kVecThreads / 32; ++w) { gl = fmin(gl, red[2 * w]); gu = fmax(gu, red[2 * w + 1]); }
  const double ulp = 2.220446049250313e-16;
  const double tnorm = fmax(fabs(gl), fabs(gu));
  const double pad = 2.0 * ulp * tnorm * n + 1e-300;
  gl -= pad;
  gu += pad;
  const double tiny = ulp * tnorm + 1e-300;   // replaces an exactly zero pivot

  const int side = tid & 1;
  const int c = c0 + (tid >> 1);
  const bool valid = (tid >> 1) < pairs && c < k;
  const int idx = lo + (valid ? c : 0);
  // Eigenvalue idx of T to round-off.  [a, b] always carries the true counts
  // of its ends (count(a) <= idx < count(b)).
  //  0. a starting point: bisection on FP32 counts (pair_count_f32) from the
  //     Gershgorin interval down to about 16 eps_32 ||T||; the eigenvalue of
  //     the same index from the previous pass of this SCF (eps; NaN after a
  //     cold start) replaces the interval's midpoint when it lies in the
  //     interval (it is then at least as close).  The FP64 count at the
  //     starting point narrows [a, b]; when it is idx or idx + 1 (no other
  //     eigenvalue between it and eigenvalue idx), step 2 starts from it;
  //  1. otherwise bisection on the count until [a, b] holds eigenvalue idx
  //     alone (count(a) = idx, count(b) = idx + 1), or is below the tolerance
  //     (a cluster: the midpoint is the eigenvalue);
  //  2. Laguerre's iteration on p(x) = det(T - x I), of degree n with real
  //     roots only: G = p'/p, H = G^2 - p''/p,
  //     x <- x - n / (G +- sqrt((n - 1)(n H - G^2))), the sign chosen to move
  //     towards eigenvalue idx (down when count(x) > idx).  For a real-rooted
  //     polynomial that step never passes the nearest root on its side and
  //     converges cubically, so it is taken only from a point whose count is
  //     idx or idx + 1 (the nearest root on the chosen side is then eigenvalue
  //     idx).  Each point's count narrows [a, b]; a point with another count,
  //     a step that would leave [a, b], and a step above round-off level that
  //     is not at most half the previous one bisect [a, b] instead.  (A cluster of m close
  //     eigenvalues beyond the wanted one, seen from a distance large against
  //     its width, acts like an m-fold root: Laguerre then converges only
  //     linearly, each step covering about m^-1/2 of the distance.)
  const double tol = 2.0 * ulp * tnorm;
  double a = gl, bnd = gu, lam = 0.0;
  if (n == 1) {
    lam = d[0];
  } else {
    const int r = n / 2 - 1;
    const double e2r = e2[r];
    int ca = 0, cb = n;
    bool adj = false;   // lam is a starting point with count idx or idx + 1
    {
      constexpr double kEps32 = 1.1920928955078125e-07;
      const float e2rf = e2f[r];
      double a32 = gl, b32 = gu;
      for (int it = 0; it < 48; ++it) {
        const bool go = valid && b32 - a32 > 16.0 * kEps32 * (fabs(a32) + fabs(b32) + tnorm);
        if (!__any_sync(0xffffffffu, go)) break;
        const double mid = 0.5 * (a32 + b32);
        const int c32 = pair_count_f32(df, e2f, n, r, side, e2rf, (float)mid);
        if (go) {
          if (c32 > idx) b32 = mid;
          else a32 = mid;
        }
      }
      const double xp = valid ? eps[mol.vec0 + idx] : 0.0;
      const double x0 = (xp >= a32 && xp <= b32) ? xp : 0.5 * (a32 + b32);   // the midpoint for NaN
      const TriEval ev = pair_eval<false>(d, e2, n, r, side, e2r, x0);
      if (valid && x0 > gl && x0 < gu) {
        if (ev.count > idx) { bnd = x0; cb = ev.count; }
        else { a = x0; ca = ev.count; }
        if (ev.count == idx || ev.count == idx + 1) { adj = true; lam = x0; }
      }
    }
    for (int it = 0; it < 80; ++it) {
      const bool done = !valid || adj || (ca == idx && cb == idx + 1) ||
                        bnd - a <= 2.0 * ulp * fmax(fabs(a), fabs(bnd)) + tol;
      if (__all_sync(0xffffffffu, done)) break;
      const double mid = 0.5 * (a + bnd);
      const TriEval ev = pair_eval<false>(d, e2, n, r, side, e2r, mid);
      if (!done) {
        if (ev.count > idx) { bnd = mid; cb = ev.count; }
        else { a = mid; ca = ev.count; }
      }
    }
    const bool isolated = ca == idx && cb == idx + 1;
    if (!adj) lam = 0.5 * (a + bnd);
    bool conv = !valid || !(adj || isolated);
    const double dn = (double)n;
    double prev_step = 1e300;
    for (int it = 0; it < 64; ++it) {
      if (__all_sync(0xffffffffu, conv)) break;
      const TriEval ev = pair_eval<true>(d, e2, n, r, side, e2r, lam);
      if (!conv) {
        double xn = lam;
        if (ev.f == 0.0) {
          conv = true;
        } else {
          const bool above = ev.count > idx;   // lam lies above eigenvalue idx
          if (above) { bnd = lam; cb = ev.count; }
          else { a = lam; ca = ev.count; }
          bool take = false, done = false;
          double step = 0.0, xl = 0.0;
          if (ev.count == idx || ev.count == idx + 1) {
            const double G = ev.f1 / ev.f;
            const double H = fma(G, G, -ev.f2 / ev.f);
            const double disc = sqrt(fmax((dn - 1.0) * fma(dn, H, -G * G), 0.0));
            const double den = above ? G + disc : G - disc;
            xl = lam - dn / den;
            const bool inside = xl >= a && xl <= bnd;
            step = fabs(xl - lam);
            done = inside && step <= 2.0 * ulp * fabs(lam) + 1e-300;
            // steps at round-off level never trigger the bisection
            take = inside && (done || step <= 0.5 * prev_step || step <= 64.0 * ulp * fabs(lam) + 1e-300);
          }
          if (take) { xn = xl; prev_step = step; }
          else { xn = 0.5 * (a + bnd); prev_step = 1e300; }
          if (done || bnd - a <= tol) conv = true;
        }
        lam = xn;
      }
    }
  }
  if (!valid || side) return;
  eps[mol.vec0 + idx] = lam;
  const int cl = tid >> 1;   // this pair's slot in the CTA
  if (vec_smem) {
    // factors and vector in shared memory, element i of slot cl at i * pairs + cl
    double* fl = red + 2 * (kVecThreads / 32) + n;
    double* fu1i = fl + (long long)n * pairs;
    double* fu2 = fu1i + (long long)n * pairs;
    double* xs = fu2 + (long long)n * pairs;
    unsigned char* piv = reinterpret_cast<unsigned char*>(xs + (long long)n * pairs);
    inverse_iteration(n, pairs, d, e, lam, tiny, (unsigned)idx, fl + cl, fu1i + cl, fu2 + cl, piv + cl, xs + cl,
                      Z + mol.mat0 + c, k);
  } else {
    double* x = Z + mol.mat0 + c;
    inverse_iteration(n, k, d, e, lam, tiny, (unsigned)idx, S0 + mol.mat0 + c, S1 + mol.mat0 + c, S2 + mol.mat0 + c,
                      S3 + mol.mat0 + c, x, x, k);
  }
}

// Re-orthogonalisation inside clusters of close eigenvalues: for each vector j
// of a cluster, z_j <- z_j - sum_{l<j} <z_l, z_j> z_l twice (classical
// Gram-Schmidt applied twice), then normalised.  One CTA per molecule.  When
// the launch's shared memory holds the molecule's vectors (stage != 0)
// and the molecule has a cluster, they are copied there first (row pitch
// k + 1: column accesses free of bank conflicts) and back at the end.
__global__ void __launch_bounds__(kOrthThreads)
tri_orth_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
                int require_active, int final_pass, const double* __restrict__ td, long long vstride,
                const double* __restrict__ eps, double* __restrict__ Z, int stage) {
  extern __shared__ __align__(16) double zsm[];
  __shared__ double dots[1024];
  __shared__ double red[kOrthThreads / 32];
  __shared__ double onenrm_s;
  const int mi = list[blockIdx.x];
  if (require_active && st[mi].status != kActive) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  int lo, hi;
  hh_range(n, mol.nocc, final_pass, &lo, &hi);
  const int k = hi - lo;
  if (k < 2) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarps = kOrthThreads / 32;
  const double* tdd = td + mol.vec0;
  const double* tde = tdd + vstride;
  double nr = 0.0;
  for (int i = tid; i < n; i += kOrthThreads) {
    const double r = fabs(tdd[i]) + (i + 1 < n ? fabs(tde[i]) : 0.0) + (i > 0 ? fabs(tde[i - 1]) : 0.0);
    nr = fmax(nr, r);
  }
  for (int o = 16; o > 0; o >>= 1) nr = fmax(nr, __shfl_xor_sync(0xffffffffu, nr, o));
  if (lane == 0) red[warp] = nr;
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int w = 0; w < nwarps; ++w) m = fmax(m, red[w]);
    onenrm_s = m;
  }
  __syncthreads();
  const double ortol = 1e-3 * onenrm_s;
  const double* ev = eps + mol.vec0 + lo;
  double* Zm = Z + mol.mat0;
  bool any = false;   // a pair of neighbours closer than ortol: some cluster to treat
  for (int c = 1 + tid; c < k; c += kOrthThreads) any = any || (ev[c] - ev[c - 1] < ortol);
  if (!__syncthreads_or(any)) return;
  double* Zw = Zm;
  long long ld = k;
  if (stage) {
    Zw = zsm;
    ld = k + 1;
    for (long long t = tid; t < (long long)n * k; t += kOrthThreads) zsm[(t / k) * ld + t % k] = Zm[t];
    __syncthreads();
  }
  int c0 = 0;
  while (c0 < k) {
    int c1 = c0 + 1;
    while (c1 < k && ev[c1] - ev[c1 - 1] < ortol) ++c1;
    if (c1 - c0 >= 2) {
      for (int j = c0 + 1; j < c1; ++j) {
        const int nprev = j - c0;
        for (int pass = 0; pass < 2; ++pass) {
          // dots with the earlier vectors of the cluster (warp per vector)
          for (int l0 = 0; l0 < nprev; l0 += 1024) {
            const int cnt = min(1024, nprev - l0);
            for (int q = warp; q < cnt; q += nwarps) {
              const int l = c0 + l0 + q;
              double s = 0.0;
              for (int i = lane; i < n; i += 32) s = fma(Zw[(long long)i * ld + l], Zw[(long long)i * ld + j], s);
              s = warp_sum_d(s);
              if (lane == 0) dots[q] = s;
            }
            __syncthreads();
            for (int i = tid; i < n; i += kOrthThreads) {
              double zj = Zw[(long long)i * ld + j];
              for (int q = 0; q < cnt; ++q) zj = fma(-dots[q], Zw[(long long)i * ld + c0 + l0 + q], zj);
              Zw[(long long)i * ld + j] = zj;
            }
            __syncthreads();
          }
        }
        double s = 0.0;
        for (int i = tid; i < n; i += kOrthThreads) { const double z = Zw[(long long)i * ld + j]; s = fma(z, z, s); }
        s = warp_sum_d(s);
        if (lane == 0) red[warp] = s;
        __syncthreads();
        double tot = 0.0;
        for (int w = 0; w < nwarps; ++w) tot += red[w];
        const double r = tot > 0.0 ? rsqrt(tot) : 0.0;
        for (int i = tid; i < n; i += kOrthThreads) Zw[(long long)i * ld + j] *= r;
        __syncthreads();
      }
    }
    c0 = c1;
  }
  if (stage)
    for (long long t = tid; t < (long long)n * k; t += kOrthThreads) Zm[t] = zsm[(t / k) * ld + t % k];
}

// X = Q Z with Q = H_0 H_1 ... H_{n-3}: H_{n-3} is applied first.  CTA = 32
// columns (lanes) x 8 row slices (warps, row i belongs to warp i mod 8); the
// columns sit in shared memory (pitch 33).  Output: row lo + c of C; in the
// final pass each row's component sum is made >= 0.  T = double: the FP64
// path; T = float: the FP32 phase of the mixed-precision path (reflectors and
// vectors rounded to FP32 as they are staged, FP32 arithmetic, rows of the
// FP32 shadow C32).  require_phase >= 0 serves only molecules in that phase.
template <typename T>
__global__ void __launch_bounds__(kBackCols * kBackWarps)
hh_back_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, const MolState* __restrict__ st,
               int require_active, int require_phase, int final_pass, const double* __restrict__ W,
               const double* __restrict__ td, long long vstride, const double* __restrict__ Z, T* __restrict__ C) {
  extern __shared__ __align__(16) double bsm[];
  const int mi = list[blockIdx.x];
  if (require_active && st[mi].status != kActive) return;
  if (require_phase >= 0 && st[mi].phase != require_phase) return;
  const DevMol mol = mols[mi];
  const int n = mol.nao;
  int lo, hi;
  hh_range(n, mol.nocc, final_pass, &lo, &hi);
  const int k = hi - lo;
  const int cb = blockIdx.y * kBackCols;
  if (cb >= k) return;
  constexpr int kP = kBackCols + 1;
  T* zs = reinterpret_cast<T*>(bsm);                                   // n x kP
  T* red = zs + (long long)n * kP;                                     // 2 x kBackWarps x kBackCols
  T* dotv = red + 2 * kBackWarps * kBackCols;                          // 2 x kBackCols
  T* taus = dotv + 2 * kBackCols;                                      // n
  T* urow = taus + n;                                                  // 2 n (FP32: staged reflectors;
                                                                       // FP64: the pairs' u_{j-1}.u_j)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const double* Zm = Z + mol.mat0;
  const double* Wm = W + mol.mat0;
  const double* tt = td + mol.vec0 + 2 * vstride;
  const int c = cb + lane;
  for (int i = warp; i < n; i += kBackWarps) zs[i * kP + lane] = c < k ? (T)Zm[(long long)i * k + c] : (T)0;
  for (int i = tid; i < n; i += kBackCols * kBackWarps) taus[i] = (T)tt[i];
  int jstart = n - 3;
  if (sizeof(T) == 8) {
    // FP64: reflectors in pairs (j, j - 1), one reduction round per pair.
    // With d = u^T z over the unmodified z and c = u_{j-1}^T u_j,
    //   H_{j-1} H_j z = z - a u_j - b u_{j-1},  a = tau_j d_j,
    //   b = tau_{j-1} (d_{j-1} - c a),
    // the same two FMAs per element and reflector as one at a time, with
    // half the barriers and single-warp sums.  c of every pair first.
    T* cs = urow;
    for (int q = warp; n - 3 - 2 * q >= 1; q += kBackWarps) {
      const int j = n - 3 - 2 * q;
      const double* uj = Wm + (long long)j * n;          // valid from row j + 1
      const double* um = Wm + (long long)(j - 1) * n;    // valid from row j
      double sc = 0.0;
      for (int i = j + 1 + lane; i < n; i += 32) sc = fma(um[i], uj[i], sc);
      sc = warp_sum_d(sc);
      if (lane == 0) cs[q] = (T)sc;
    }
    __syncthreads();
    int j = n - 3;
    for (; j >= 1; j -= 2) {
      const T tj = taus[j], tm = taus[j - 1];
      if (tj == (T)0 && tm == (T)0) continue;   // uniform: both H = I
      const double* uj = Wm + (long long)j * n;
      const double* um = Wm + (long long)(j - 1) * n;
      const int i0 = j + ((warp - j) & (kBackWarps - 1));   // this warp's first row >= j
      T pj = 0, pm = 0;
      for (int i = i0; i < n; i += kBackWarps) {
        const T z = zs[i * kP + lane];
        const T vj = i > j ? (T)uj[i] : (T)0;
        pj = fma(vj, z, pj);
        pm = fma((T)um[i], z, pm);
      }
      red[warp * kBackCols + lane] = pj;
      red[(kBackWarps + warp) * kBackCols + lane] = pm;
      __syncthreads();
      if (warp == 0) {
        T sj = red[lane], sm = red[kBackWarps * kBackCols + lane];
#pragma unroll
        for (int q = 1; q < kBackWarps; ++q) {
          sj += red[q * kBackCols + lane];
          sm += red[(kBackWarps + q) * kBackCols + lane];
        }
        const T a = tj * sj;
        dotv[lane] = a;
        dotv[kBackCols + lane] = tm * (sm - cs[(n - 3 - j) >> 1] * a);
      }
      __syncthreads();
      const T a = dotv[lane], b = dotv[kBackCols + lane];
      for (int i = i0; i < n; i += kBackWarps) {
        T* zp = zs + i * kP + lane;
        const T vj = i > j ? (T)uj[i] : (T)0;
        *zp = fma(-b, (T)um[i], fma(-a, vj, *zp));
      }
    }
    jstart = j;   // 0 when one reflector is left, else -1
  }
  __syncthreads();
  int par = 0;   // parity of the reflectors applied so far (tau == 0 ones are skipped)
  for (int j = jstart; j >= 0; --j) {
    const T tau = taus[j];
    if (tau == (T)0) continue;
    const double* ug = Wm + (long long)j * n;
    const T* u;
    if (sizeof(T) == 4) {
      // two staging rows: a warp still updating with the previous applied
      // reflector reads the other one
      T* ur = urow + par * n;
      par ^= 1;
      for (int i = j + 1 + tid; i < n; i += kBackCols * kBackWarps) ur[i] = (T)ug[i];
      __syncthreads();
      u = ur;
    } else {
      u = reinterpret_cast<const T*>(ug);
    }
    // row slices are fixed (row i belongs to warp i mod 8), so a warp only
    // reads rows it updated itself at the previous reflector
    const int i0 = j + 1 + ((warp - (j + 1)) & (kBackWarps - 1));
    T part = 0;
    for (int i = i0; i < n; i += kBackWarps) part = fma(u[i], zs[i * kP + lane], part);
    red[warp * kBackCols + lane] = part;
    __syncthreads();
    if (warp == 0) {
      T sum = red[lane];
#pragma unroll
      for (int q = 1; q < kBackWarps; ++q) sum += red[q * kBackCols + lane];
      dotv[lane] = tau * sum;
    }
    __syncthreads();
    const T dt = dotv[lane];
    for (int i = i0; i < n; i += kBackWarps) {
      T* z = zs + i * kP + lane;
      *z = fma(-dt, u[i], *z);
    }
  }
  __syncthreads();
  // rows of C: warp per row, lanes over the components
  T* Cm = C + mol.mat0;
  for (int q = warp; q < kBackCols; q += kBackWarps) {
    const int cc = cb + q;
    if (cc >= k) break;
    T sgn = 1;
    if (final_pass) {
      // component sum in index order, as Lapack::Dsyevd's phase fix does
      // (src/wrappers/Lapack.cpp:139-150): a row whose sum is zero up to
      // round-off gets the sign that order of summation gives
      T s = 0;
      if (lane == 0)
        for (int i = 0; i < n; ++i) s += zs[i * kP + q];
      s = __shfl_sync(0xffffffffu, s, 0);
      sgn = s < (T)0 ? (T)-1 : (T)1;
    }
    T* row = Cm + (long long)(lo + cc) * n;
    for (int i = lane; i < n; i += 32) row[i] = sgn * zs[i * kP + q];
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static std::once_flag g_hh_attr_once;

static void hh_set_attributes() {
  std::call_once(g_hh_attr_once, [] {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncSetAttribute(hh_tridiag_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(hh_tridiag_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(hh_back_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(hh_back_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(tri_vectors_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(tri_orth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         optin - (int)kOrthStaticSmem);
  });
}

// tri_vectors_kernel: d, e, e^2 and the reduction slots; with vec_smem also
// the factors, vector and pivot flags of its `pairs` inverse iterations
size_t tri_vectors_smem_bytes(int n, bool vec_smem, int pairs) {
  size_t b = (4 * (size_t)n + 2 * (kVecThreads / 32)) * sizeof(double);   // d, e, e^2, FP32 d and e^2, slots
  if (vec_smem) b += (size_t)n * pairs * (4 * sizeof(double) + 1);
  return b;
}

static int hh_optin_smem() {
  static int optin = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  });
  return optin;
}

size_t hh_back_smem_bytes(int n) {
  return ((size_t)n * (kBackCols + 1) + 2 * kBackWarps * kBackCols + 2 * kBackCols + 3 * n) * sizeof(double);
}

int hh_back_max_n() {
  static int nmax = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int n = 8;
    while (hh_back_smem_bytes(n + 1) <= (size_t)hh_optin_smem()) ++n;
    nmax = n;
  });
  return nmax;
}

void hh_prepare() {
  hh_set_attributes();
  hh_smem_max_n();
  hh_back_max_n();
}

void launch_hh_tridiag(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                       int require_active, const double* F, double* W, double* td, long long vstride, double* Aws,
                       int max_n_served, cudaStream_t s) {
  if (nlist <= 0 || max_n <= 0) return;
  hh_set_attributes();
  const bool smem = max_n <= hh_smem_max_n();
  const size_t sh = hh_tridiag_smem_bytes(max_n, smem);
  const int threads = tuned_tridiag_threads(max_n);
  if (smem)
    hh_tridiag_kernel<true><<<nlist, threads, sh, s>>>(mols, list, st, require_active, F, W, td, vstride, Aws,
                                                       max_n_served);
  else
    hh_tridiag_kernel<false><<<nlist, threads, sh, s>>>(mols, list, st, require_active, F, W, td, vstride, Aws,
                                                        max_n_served);
}

void launch_tri_vectors(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                        int require_active, int final_pass, const double* td, long long vstride, double* eps,
                        double* Z, double* const* S4, cudaStream_t s) {
  if (nlist <= 0 || max_k <= 0) return;
  hh_set_attributes();
  const int pairs = std::max(1, std::min(kVecPerCta, tuned_vec_pairs(max_n)));
  const bool vec_smem = tuned_vec_smem(max_n) && tri_vectors_smem_bytes(max_n, true, pairs) <= (size_t)hh_optin_smem();
  const size_t vsh = tri_vectors_smem_bytes(max_n, vec_smem, pairs);
  dim3 gv(nlist, (max_k + pairs - 1) / pairs);
  tri_vectors_kernel<<<gv, kVecThreads, vsh, s>>>(mols, list, st, require_active, final_pass, td, vstride, eps, Z,
                                                  S4[0], S4[1], S4[2], S4[3], vec_smem ? 1 : 0, pairs);
}

void launch_hh_vectors(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                       int require_active, int final_pass, int mixed, const double* W, const double* td,
                       long long vstride, double* eps, double* Z, double* const* S4, double* C, float* C32,
                       cudaStream_t s) {
  if (nlist <= 0 || max_k <= 0) return;
  launch_tri_vectors(mols, list, nlist, max_n, max_k, st, require_active, final_pass, td, vstride, eps, Z, S4, s);
  // the vectors of the launch's largest molecule in shared memory when they fit
  const size_t osh = (size_t)max_n * (max_k + 1) * sizeof(double);
  const int stage = osh + kOrthStaticSmem <= (size_t)hh_optin_smem() ? 1 : 0;
  tri_orth_kernel<<<nlist, kOrthThreads, stage ? osh : 0, s>>>(mols, list, st, require_active, final_pass, td,
                                                                vstride, eps, Z, stage);
  dim3 gb(nlist, (max_k + kBackCols - 1) / kBackCols);
  // mixed precision: FP32 back-transformation for molecules still in the FP32 phase
  const int fp64_phase = (mixed && !final_pass) ? 1 : -1;
  hh_back_kernel<double><<<gb, kBackCols * kBackWarps, hh_back_smem_bytes(max_n), s>>>(
      mols, list, st, require_active, fp64_phase, final_pass, W, td, vstride, Z, C);
  if (fp64_phase == 1)
    hh_back_kernel<float><<<gb, kBackCols * kBackWarps, hh_back_smem_bytes(max_n), s>>>(
        mols, list, st, require_active, 0, final_pass, W, td, vstride, Z, C32);
}

}  // namespace nddo
