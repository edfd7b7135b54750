// Kernel (d): batched two-sided cyclic Jacobi eigensolver, one CTA per molecule.
//
// Replaces MolDS's Lapack::Dsyevd on the SCF path (src/wrappers/Lapack.cpp:102-160,
// called at src/cndo/Cndo2.cpp:652-655).  Output convention is the reference's:
// eigenvalues ascending, eigenvectors as ROWS of C, each row's component sum
// made >= 0.
//
// Layout: the symmetric working matrix is stored as its packed upper triangle
// and the accumulated rotations V as a full N'xN' matrix, both in shared memory
// when they fit (N' <= 194 in FP32, <= 138 in FP64); otherwise the kernel runs
// on a per-molecule workspace in global memory (L2-resident for these sizes).
// N' = N rounded up to even; an odd N gets a decoupled dummy index.
//
// Parallel ordering: round-robin tournament.  In round r the N'/2 disjoint
// pairs (p, q) are rotated at once; every 2x2 block of the matrix is then
// updated exactly once per round as J_I^T B J_K, and V as V J.
//
// Warm start: V starts from the previous iteration's eigenvectors and the
// matrix from C_prev F C_prev^T (computed by the transform GEMMs), so late SCF
// iterations converge in one or two sweeps.
#include <cooperative_groups.h>
#include <mutex>
#include <cuda_runtime.h>
#include "nddo_batch.cuh"
#include "kernels.h"

namespace nddo {

constexpr int kJacobiThreads = 1024;

__host__ __device__ inline long long jac_pk(int i, int j, int n) {   // packed upper, i <= j
  return (long long)i * (2 * n - i + 1) / 2 + (j - i);
}

// vector access of V rows: float4 in FP32, double2 in FP64
template <typename T> struct Vec4;
template <> struct Vec4<float> {
  typedef float4 type;
  static constexpr int width = 4;
  __device__ static float4 rot1(float4 a, float4 b, float c, float s) {
    return make_float4(c * a.x - s * b.x, c * a.y - s * b.y, c * a.z - s * b.z, c * a.w - s * b.w);
  }
  __device__ static float4 rot2(float4 a, float4 b, float c, float s) {
    return make_float4(s * a.x + c * b.x, s * a.y + c * b.y, s * a.z + c * b.z, s * a.w + c * b.w);
  }
};
template <> struct Vec4<double> {
  typedef double2 type;
  static constexpr int width = 2;
  __device__ static double2 rot1(double2 a, double2 b, double c, double s) {
    return make_double2(c * a.x - s * b.x, c * a.y - s * b.y);
  }
  __device__ static double2 rot2(double2 a, double2 b, double c, double s) {
    return make_double2(s * a.x + c * b.x, s * a.y + c * b.y);
  }
};

// Rotation that annihilates a_pq: t = tan(phi) is the root of
// a_pq t^2 + (a_qq - a_pp) t - a_pq = 0 with |t| <= 1, c = 1 / sqrt(1 + t^2).
__device__ __forceinline__ void jac_rotation(float app, float aqq, float apq, float* t_out, float* c, float* s) {
  const float theta = (aqq - app) / (2.f * apq);
  float t;
  if (fabsf(theta) > 1e15f) t = 0.5f / theta;
  else t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
  *c = 1.f / sqrtf(t * t + 1.f);
  *s = t * *c;
  *t_out = t;
}
// FP64: GB300 runs FP64 at 1/64 of the FP32 rate and FP64 divides and square
// roots are long dependent sequences, so t starts from the FP32 formula (with
// a_qq - a_pp formed in FP64) and takes one Newton step on the quadratic
// (error (1e-7)^2), and c = rsqrt(1 + t^2) takes two Newton steps from the FP32
// reciprocal square root: one FP64 divide instead of three divides and two
// square roots.
__device__ __forceinline__ void jac_rotation(double app, double aqq, double apq, double* t_out, double* c,
                                             double* s) {
  const double d = aqq - app;
  const float thetaf = (float)d / (2.f * (float)apq);
  float tf;
  if (fabsf(thetaf) > 1e15f) tf = 0.5f / thetaf;
  else tf = (thetaf >= 0.f ? 1.f : -1.f) / (fabsf(thetaf) + sqrtf(thetaf * thetaf + 1.f));
  double t = (double)tf;
  const double g = fma(apq * t, t, fma(d, t, -apq));
  const double gp = fma(2.0 * apq, t, d);
  t -= g / gp;
  const double x = fma(t, t, 1.0);
  double cc = (double)rsqrtf((float)x);
  cc = cc * fma(-0.5 * x, cc * cc, 1.5);
  cc = cc * fma(-0.5 * x, cc * cc, 1.5);
  *c = cc;
  *s = t * cc;
  *t_out = t;
}

template <typename T> struct JacTol;
template <> struct JacTol<float> { static constexpr float rel = 3e-7f; };
template <> struct JacTol<double> { static constexpr double rel = 2e-14; };

// working size: n rounded up to a multiple of 4 (even for the round-robin
// pairing, and 16-byte rows of V for vector loads); padding indices are
// decoupled (zero off-diagonal) and never rotated
__host__ __device__ inline int jac_np(int n) { return (n + 3) & ~3; }

size_t jacobi_smem_bytes(int n, int elem, bool v_in_smem, bool a_in_smem) {
  const long long np = jac_np(n);
  long long b = 0;
  if (a_in_smem) b += np * (np + 1) / 2 * elem;
  if (v_in_smem) b += np * np * elem;
  b += (np / 2) * 2 * elem;        // c, s
  b += (np / 2) * 2 * 4;           // p, q
  b += np * 4 + np * elem;         // column order + sign
  b += np * 4 + 16;                // packed row offsets (+ alignment of the packed matrix)
  b += (np / 2) * 4;               // rotation flags
  b += 64 * 8 + 16;                // reduction scratch (+ alignment slack)
  return (size_t)((b + 15) & ~15LL);
}

template <typename T, typename TCin>
__global__ void __launch_bounds__(kJacobiThreads)
jacobi_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list, const MolState* __restrict__ st,
              int require_active, const T* __restrict__ G, const TCin* __restrict__ Cin, int use_basis,
              double* __restrict__ Cout, double* __restrict__ eps_out, T* __restrict__ Aws, T* __restrict__ Vws,
              long long ws_stride, int a_in_smem, int v_in_smem, int max_sweeps, int* __restrict__ sweeps_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = mol_list[blockIdx.x];
  if (require_active && st[m].status != kActive) return;
  const DevMol mol = mols[m];
  const int n = mol.nao;
  const int np = jac_np(n);
  const int half = np / 2;
  const long long npk = (long long)np * (np + 1) / 2;

  unsigned char* ptr = smem_raw;
  T* A;
  T* V;
  // V first: its rows must stay 16-byte aligned for vector access
  if (v_in_smem) { V = reinterpret_cast<T*>(ptr); ptr += (long long)np * np * sizeof(T); }
  else V = Vws + (long long)blockIdx.x * ws_stride;
  if (a_in_smem) { A = reinterpret_cast<T*>(ptr); ptr += ((npk * sizeof(T) + 15) & ~15LL); }
  else A = Aws + (long long)blockIdx.x * ws_stride;
  T* cs = reinterpret_cast<T*>(ptr); ptr += 2 * half * sizeof(T);
  int* pq = reinterpret_cast<int*>(ptr); ptr += 2 * half * sizeof(int);
  int* order = reinterpret_cast<int*>(ptr); ptr += np * sizeof(int);
  T* sgn = reinterpret_cast<T*>(ptr); ptr += np * sizeof(T);
  int* rowoff = reinterpret_cast<int*>(ptr); ptr += np * sizeof(int);
  int* rot = reinterpret_cast<int*>(ptr); ptr += half * sizeof(int);
  T* red = reinterpret_cast<T*>(((uintptr_t)ptr + 7) & ~(uintptr_t)7);

  const int tid = threadIdx.x, nth = blockDim.x;
  const T* Gm = G + mol.mat0;
  const TCin* Cm = Cin + mol.mat0;

  // ---- load ------------------------------------------------------------------
  for (long long e = tid; e < npk; e += nth) {
    // decode packed index -> (i, j): row i holds np - i entries
    int i = 0;
    long long rem = e;
    // rows are long; a short scan per element is acceptable for a one-time load
    {
      // solve i from e using the closed form, then fix rounding
      double b = 2.0 * np + 1.0;
      double disc = b * b - 8.0 * (double)e;
      i = (int)((b - sqrt(disc)) * 0.5);
      if (i < 0) i = 0;
      while (i > 0 && jac_pk(i, i, np) > e) --i;
      while (i + 1 < np && jac_pk(i + 1, i + 1, np) <= e) ++i;
      rem = e - jac_pk(i, i, np);
    }
    const int j = i + (int)rem;
    T v = 0;
    if (i < n && j < n) v = Gm[(long long)i * n + j];
    A[e] = v;
  }
  // V is kept transposed: row i of V holds eigenvector i (V[i][mu] = C_prev[i][mu])
  for (long long e = tid; e < (long long)np * np; e += nth) {
    const int i = (int)(e / np), mu = (int)(e % np);
    T v;
    if (mu < n && i < n) v = use_basis ? (T)Cm[(long long)i * n + mu] : (T)(mu == i ? 1 : 0);
    else v = (T)(mu == i ? 1 : 0);
    V[e] = v;
  }
  for (int i = tid; i < np; i += nth) rowoff[i] = (int)jac_pk(i, i, np);
  __syncthreads();

  // matrix scale for the stopping test
  T scale = 0;
  for (int i = tid; i < n; i += nth) { T d = fabs(A[rowoff[i]]); scale = d > scale ? d : scale; }
  for (int o = 16; o > 0; o >>= 1) { T t = __shfl_xor_sync(0xffffffffu, scale, o); scale = t > scale ? t : scale; }
  if ((tid & 31) == 0) red[tid >> 5] = scale;
  __syncthreads();
  if (tid == 0) {
    T s = 0;
    for (int w = 0; w < (nth >> 5); ++w) s = red[w] > s ? red[w] : s;
    red[32] = s > (T)1e-30 ? s : (T)1;
  }
  __syncthreads();
  const T thresh = JacTol<T>::rel * red[32];
  __syncthreads();

  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    // A sweep that would rotate nothing is replaced by one parallel scan of
    // every off-diagonal element: when all are at the threshold or below, the
    // matrix is already diagonal to the accuracy the sweep would certify.
    if (sweep > 0) {
      T m = 0;
      for (int i = tid; i < n; i += nth) {
        const int oi = rowoff[i];
        for (int j = i + 1; j < n; ++j) { const T a = fabs(A[oi + (j - i)]); m = a > m ? a : m; }
      }
      if (!__syncthreads_or(m > thresh)) break;
    }
    T offmax = 0;
    for (int r = 0; r < np - 1; ++r) {
      // pairs and rotations of this round; rotations below the stopping
      // threshold are skipped (they could not change the result it certifies)
      int any = 0;
      for (int k = tid; k < half; k += nth) {
        const int i1 = k, i2 = np - 1 - k;
        const int p1 = (i1 == 0) ? 0 : ((i1 - 1 + r) % (np - 1)) + 1;
        const int p2 = (i2 == 0) ? 0 : ((i2 - 1 + r) % (np - 1)) + 1;
        const int p = p1 < p2 ? p1 : p2, q = p1 < p2 ? p2 : p1;
        const T apq = A[rowoff[p] + (q - p)];
        T c = 1, s = 0;
        const T aa = fabs(apq);
        offmax = aa > offmax ? aa : offmax;
        const int doit = aa > thresh;
        if (doit) {
          const T app = A[rowoff[p]], aqq = A[rowoff[q]];
          T t;
          jac_rotation(app, aqq, apq, &t, &c, &s);
          // diagonal block: exact update, off-diagonal element annihilated
          A[rowoff[p]] = app - t * apq;
          A[rowoff[q]] = aqq + t * apq;
          A[rowoff[p] + (q - p)] = 0;
        }
        cs[2 * k] = c; cs[2 * k + 1] = s;
        pq[2 * k] = p; pq[2 * k + 1] = q;
        rot[k] = doit;
        any |= doit;
      }
      if (!__syncthreads_or(any)) continue;
      // A <- J^T A J for the off-diagonal 2x2 blocks (I < K) touching a rotated
      // pair.  A warp owns the row pairs rp and half-1-rp (balanced lengths);
      // its lanes walk K.
      const int warp = tid >> 5, lane = tid & 31, nwarps = nth >> 5;
      for (int rp = warp; rp < (half + 1) / 2; rp += nwarps) {
        for (int side = 0; side < 2; ++side) {
          const int I = side == 0 ? rp : half - 1 - rp;
          if (side == 1 && I == rp) break;
          const int rI = rot[I];
          const int p = pq[2 * I], q = pq[2 * I + 1];
          const int op = rowoff[p], oq = rowoff[q];
          const T c = cs[2 * I], s = cs[2 * I + 1];
          for (int K = I + 1 + lane; K < half; K += 32) {
            if (!(rI | rot[K])) continue;
            const int r2 = pq[2 * K], s2 = pq[2 * K + 1];
            const int i_pr = p < r2 ? op + (r2 - p) : rowoff[r2] + (p - r2);
            const int i_ps = p < s2 ? op + (s2 - p) : rowoff[s2] + (p - s2);
            const int i_qr = q < r2 ? oq + (r2 - q) : rowoff[r2] + (q - r2);
            const int i_qs = q < s2 ? oq + (s2 - q) : rowoff[s2] + (q - s2);
            const T b00 = A[i_pr], b01 = A[i_ps], b10 = A[i_qr], b11 = A[i_qs];
            const T c2 = cs[2 * K], s2n = cs[2 * K + 1];
            // Y = J_I^T B
            const T y00 = c * b00 - s * b10, y01 = c * b01 - s * b11;
            const T y10 = s * b00 + c * b10, y11 = s * b01 + c * b11;
            // X = Y J_K
            A[i_pr] = y00 * c2 - y01 * s2n;
            A[i_ps] = y00 * s2n + y01 * c2;
            A[i_qr] = y10 * c2 - y11 * s2n;
            A[i_qs] = y10 * s2n + y11 * c2;
          }
        }
      }
      // V <- V J: rows p and q of V (eigenvectors p, q), one warp per pair,
      // four (two in FP64) consecutive components per lane
      typedef typename Vec4<T>::type V4;
      const int nv = np / Vec4<T>::width;
      for (int k = warp; k < half; k += nwarps) {
        if (!rot[k]) continue;
        const int p = pq[2 * k], q = pq[2 * k + 1];
        const T c = cs[2 * k], s = cs[2 * k + 1];
        V4* vp = reinterpret_cast<V4*>(V + (long long)p * np);
        V4* vq = reinterpret_cast<V4*>(V + (long long)q * np);
        for (int m = lane; m < nv; m += 32) {
          const V4 a = vp[m], b = vq[m];
          vp[m] = Vec4<T>::rot1(a, b, c, s);
          vq[m] = Vec4<T>::rot2(a, b, c, s);
        }
      }
      __syncthreads();
    }
    // sweep converged when every rotation it applied was at round-off level
    for (int o = 16; o > 0; o >>= 1) { T t = __shfl_xor_sync(0xffffffffu, offmax, o); offmax = t > offmax ? t : offmax; }
    if ((tid & 31) == 0) red[tid >> 5] = offmax;
    __syncthreads();
    if (tid == 0) {
      T mx = 0;
      for (int w = 0; w < (nth >> 5); ++w) mx = red[w] > mx ? red[w] : mx;
      red[33] = mx;
    }
    __syncthreads();
    const bool done = red[33] <= thresh;
    __syncthreads();
    if (done) { ++sweep; break; }
  }

  // ---- sort ascending, sign fix, write rows ------------------------------------
  for (int i = tid; i < np; i += nth) {
    if (i >= n) continue;
    const T li = A[rowoff[i]];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const T lj = A[rowoff[j]];
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
  for (long long e = tid; e < (long long)n * n; e += nth) {
    const int r = (int)(e / n), mu = (int)(e % n);
    const int col = order[r];
    Co[e] = (double)(sgn[col] * V[(long long)col * np + mu]);
  }
  if (tid == 0 && sweeps_out) sweeps_out[m] += sweep;   // cumulative over the SCF
}

template <typename T, typename TCin>
void launch_jacobi_impl(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                        int require_active, const T* G, const TCin* Cin, int use_basis, double* Cout,
                        double* eps, T* Aws, T* Vws, long long ws_stride, int max_sweeps, int* sweeps_out,
                        cudaStream_t s) {
  if (nlist <= 0) return;
  const int elem = sizeof(T);
  const size_t limit = 232448;
  bool a_sm = true, v_sm = true;
  if (jacobi_smem_bytes(max_n, elem, true, true) > limit) {
    v_sm = false;
    if (jacobi_smem_bytes(max_n, elem, false, true) > limit) a_sm = false;
  }
  const size_t bytes = jacobi_smem_bytes(max_n, elem, v_sm, a_sm);
  // the opt-in bound is set to the device limit (the same value on every call),
  // so launches from several host threads never race on it
  cudaFuncSetAttribute(jacobi_kernel<T, TCin>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
  // block size from the bucket's basis: the per-round barriers cost more with
  // more warps, and a small matrix has too little work per round for 32 warps
  const int threads = max_n <= 64 ? 256 : (max_n <= 128 ? 512 : kJacobiThreads);
  jacobi_kernel<T, TCin><<<nlist, threads, bytes, s>>>(mols, mol_list, st, require_active, G, Cin, use_basis,
                                                        Cout, eps, Aws, Vws, ws_stride, a_sm ? 1 : 0,
                                                        v_sm ? 1 : 0, max_sweeps, sweeps_out);
}

void launch_jacobi_f32(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                       int require_active, const float* G, const double* Cin, int use_basis, double* Cout,
                       double* eps, float* Aws, float* Vws, long long ws_stride, int max_sweeps,
                       int* sweeps_out, cudaStream_t s) {
  launch_jacobi_impl<float, double>(mols, mol_list, nlist, max_n, st, require_active, G, Cin, use_basis, Cout, eps, Aws,
                            Vws, ws_stride, max_sweeps, sweeps_out, s);
}

void launch_jacobi_f32(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                       int require_active, const float* G, const float* Cin, int use_basis, double* Cout,
                       double* eps, float* Aws, float* Vws, long long ws_stride, int max_sweeps,
                       int* sweeps_out, cudaStream_t s) {
  launch_jacobi_impl<float, float>(mols, mol_list, nlist, max_n, st, require_active, G, Cin, use_basis, Cout, eps,
                                   Aws, Vws, ws_stride, max_sweeps, sweeps_out, s);
}

void launch_jacobi_f64(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                       int require_active, const double* G, const double* Cin, int use_basis, double* Cout,
                       double* eps, double* Aws, double* Vws, long long ws_stride, int max_sweeps,
                       int* sweeps_out, cudaStream_t s) {
  launch_jacobi_impl<double, double>(mols, mol_list, nlist, max_n, st, require_active, G, Cin, use_basis, Cout, eps, Aws,
                             Vws, ws_stride, max_sweeps, sweeps_out, s);
}

bool jacobi_needs_workspace(int max_n, int elem, bool* a_global, bool* v_global) {
  const size_t limit = 232448;
  *a_global = false; *v_global = false;
  if (jacobi_smem_bytes(max_n, elem, true, true) > limit) {
    *v_global = true;
    if (jacobi_smem_bytes(max_n, elem, false, true) > limit) *a_global = true;
  }
  return *a_global || *v_global;
}

// ---------------------------------------------------------------------------
// One molecule on a cluster of kJcCluster CTAs (FP64, the plain one-molecule
// path): the same round-robin two-sided Jacobi as jacobi_kernel, with the
// matrix and the eigenvector rows spread over the cluster's shared memory, so
// a single diagonalisation runs on kJcCluster SMs instead of one.
//
// Layout: row i of the upper triangle of A (entries j >= i) and row i of V
// live in CTA i % kJcCluster at local row i / kJcCluster; every element is
// reached through the cluster's distributed shared memory.  Each round:
//   1. every CTA computes all rotations of the round from the same elements
//      (identical tables in every CTA, no exchange), then cluster barrier;
//   2. the 2x2 diagonal blocks (by the owner of row p), the off-diagonal 2x2
//      blocks and the column slices of the V rows are updated, the work spread
//      over all CTAs, then cluster barrier.
// Every branch around a barrier depends only on values all CTAs computed
// identically, so all CTAs of a cluster pass the same barriers.
// ---------------------------------------------------------------------------
constexpr int kJcCluster = 8;

struct JcView {
  double* A[kJcCluster];
  double* V[kJcCluster];
  int np;
  __device__ __forceinline__ double* a(int x, int y) const {   // upper-triangle element (x, y)
    const int i = x < y ? x : y, j = x < y ? y : x;
    return A[i % kJcCluster] + (long long)(i / kJcCluster) * np + j;
  }
  __device__ __forceinline__ double* v(int i, int mu) const {
    return V[i % kJcCluster] + (long long)(i / kJcCluster) * np + mu;
  }
};

size_t jacobi_cluster_smem_bytes(int n) {
  const long long np = jac_np(n), half = np / 2;
  const long long rows = (np + kJcCluster - 1) / kJcCluster;
  long long b = 2 * rows * np * 8;     // A and V rows
  b += half * (2 * 8 + 2 * 4 + 4 + 4 * 8);   // c, s; p, q; flag; t, app, aqq, apq
  b += sizeof(JcView) + kJcCluster * 4 + 64;   // DSMEM pointers, cluster flags, alignment
  b += 64 * 8;                         // reduction scratch
  return (size_t)((b + 15) & ~15LL);
}

__global__ void __cluster_dims__(kJcCluster, 1, 1) __launch_bounds__(512)
jacobi_cluster_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                      const MolState* __restrict__ st, int require_active, const double* __restrict__ G,
                      const double* __restrict__ F, const double* __restrict__ Cin, int use_basis,
                      double* __restrict__ Cout, double* __restrict__ eps_out, int max_sweeps,
                      int* __restrict__ sweeps_out) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int m = mol_list[blockIdx.x / kJcCluster];
  if (require_active && st[m].status != kActive) return;   // the whole cluster returns
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DevMol mol = mols[m];
  const int n = mol.nao, np = jac_np(n), half = np / 2;
  const int rows = (np + kJcCluster - 1) / kJcCluster;
  unsigned char* ptr = smem_raw;
  double* Aloc = reinterpret_cast<double*>(ptr); ptr += (size_t)rows * np * 8;
  double* Vloc = reinterpret_cast<double*>(ptr); ptr += (size_t)rows * np * 8;
  double* cs = reinterpret_cast<double*>(ptr); ptr += (size_t)half * 16;
  double* dg = reinterpret_cast<double*>(ptr); ptr += (size_t)half * 32;   // t, app, aqq, apq
  int* pq = reinterpret_cast<int*>(ptr); ptr += (size_t)half * 8;
  int* rot = reinterpret_cast<int*>(ptr); ptr += (size_t)half * 4;
  JcView* view = reinterpret_cast<JcView*>(((uintptr_t)ptr + 15) & ~(uintptr_t)15);
  ptr = reinterpret_cast<unsigned char*>(view + 1);
  int* cflag = reinterpret_cast<int*>(ptr); ptr += kJcCluster * 4;
  double* red = reinterpret_cast<double*>(((uintptr_t)ptr + 7) & ~(uintptr_t)7);
  const int tid = threadIdx.x, nth = blockDim.x;
  if (tid == 0) {
    for (int r = 0; r < kJcCluster; ++r) {
      view->A[r] = cluster.map_shared_rank(Aloc, r);
      view->V[r] = cluster.map_shared_rank(Vloc, r);
    }
    view->np = np;
  }
  // ---- load this CTA's rows ------------------------------------------------
  const double* Cm = Cin + mol.mat0;
  if (F) {
    // warm-start transform G = C F C^T fused in (G == nullptr): rows of
    // T = C F into A, then the upper part of G's rows, G_ij = T_i . C_j, into V
    const double* Fm = F + mol.mat0;
    for (long long e = tid; e < (long long)rows * np; e += nth) {
      const int lr = (int)(e / np), b = (int)(e % np);
      const int i = lr * kJcCluster + rank;
      double t = 0.0;
      if (i < n && b < n)
        for (int a = 0; a < n; ++a) t = fma(Cm[(long long)i * n + a], Fm[(long long)a * n + b], t);
      Aloc[e] = t;
    }
    __syncthreads();
    for (long long e = tid; e < (long long)rows * np; e += nth) {
      const int lr = (int)(e / np), j = (int)(e % np);
      const int i = lr * kJcCluster + rank;
      double g = 0.0;
      if (i < n && j < n && j >= i)
        for (int b = 0; b < n; ++b) g = fma(Aloc[(long long)lr * np + b], Cm[(long long)j * n + b], g);
      Vloc[e] = g;
    }
    __syncthreads();
    for (long long e = tid; e < (long long)rows * np; e += nth) Aloc[e] = Vloc[e];
    for (long long e = tid; e < (long long)rows * np; e += nth) {
      const int lr = (int)(e / np), j = (int)(e % np);
      const int i = lr * kJcCluster + rank;
      Vloc[e] = (i < n && j < n) ? Cm[(long long)i * n + j] : ((i == j) ? 1.0 : 0.0);
    }
  } else {
    const double* Gm = G + mol.mat0;
    for (long long e = tid; e < (long long)rows * np; e += nth) {
      const int lr = (int)(e / np), j = (int)(e % np);
      const int i = lr * kJcCluster + rank;
      double a = 0.0, v = (i == j) ? 1.0 : 0.0;
      if (i < np) {
        if (i < n && j < n && j >= i) a = Gm[(long long)i * n + j];
        if (i < n && j < n && use_basis) v = Cm[(long long)i * n + j];
      }
      Aloc[e] = a;
      Vloc[e] = v;
    }
  }
  cluster.sync();
  const JcView& W = *view;
  // scale for the stopping test: every CTA reads every diagonal element
  double scale = 0.0;
  for (int i = tid; i < n; i += nth) { const double d = fabs(*W.a(i, i)); scale = d > scale ? d : scale; }
  for (int o = 16; o > 0; o >>= 1) { const double t = __shfl_xor_sync(0xffffffffu, scale, o); scale = t > scale ? t : scale; }
  if ((tid & 31) == 0) red[tid >> 5] = scale;
  __syncthreads();
  if (tid == 0) {
    double sc = 0.0;
    for (int w = 0; w < (nth >> 5); ++w) sc = red[w] > sc ? red[w] : sc;
    red[32] = sc > 1e-30 ? sc : 1.0;
  }
  __syncthreads();
  const double thresh = JacTol<double>::rel * red[32];
  const int groups = half / 2;                 // row-pair groups (I, half-1-I): half - 1 blocks each
  const long long nblk = (long long)groups * (half - 1);
  const int cw = (np + kJcCluster - 1) / kJcCluster;   // V columns per CTA
  const int c0 = rank * cw, c1 = min(np, c0 + cw);

  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (sweep > 0) {
      // any off-diagonal element above the threshold in this CTA's rows?
      int big = 0;
      for (int lr = tid; lr < rows; lr += nth) {
        const int i = lr * kJcCluster + rank;
        if (i >= n) continue;
        for (int j = i + 1; j < n; ++j) big |= fabs(Aloc[(long long)lr * np + j]) > thresh;
      }
      big = __syncthreads_or(big);
      if (tid < kJcCluster) cluster.map_shared_rank(cflag, tid)[rank] = big;
      cluster.sync();
      int any = 0;
      for (int r = 0; r < kJcCluster; ++r) any |= cflag[r];
      cluster.sync();                          // flags read before the next write
      if (!any) break;
    }
    double offmax = 0.0;
    for (int r = 0; r < np - 1; ++r) {
      int any = 0;
      for (int k = tid; k < half; k += nth) {
        const int i1 = k, i2 = np - 1 - k;
        const int p1 = (i1 == 0) ? 0 : ((i1 - 1 + r) % (np - 1)) + 1;
        const int p2 = (i2 == 0) ? 0 : ((i2 - 1 + r) % (np - 1)) + 1;
        const int p = p1 < p2 ? p1 : p2, q = p1 < p2 ? p2 : p1;
        // the three loads are issued together: one distributed-shared-memory
        // round trip per round instead of two
        const double apq = *W.a(p, q), app_in = *W.a(p, p), aqq_in = *W.a(q, q);
        double c = 1.0, sn = 0.0, t = 0.0, app = 0.0, aqq = 0.0;
        const double aa = fabs(apq);
        offmax = aa > offmax ? aa : offmax;
        const int doit = aa > thresh;
        if (doit) {
          app = app_in;
          aqq = aqq_in;
          jac_rotation(app, aqq, apq, &t, &c, &sn);
        }
        cs[2 * k] = c; cs[2 * k + 1] = sn;
        dg[4 * k] = t; dg[4 * k + 1] = app; dg[4 * k + 2] = aqq; dg[4 * k + 3] = apq;
        pq[2 * k] = p; pq[2 * k + 1] = q;
        rot[k] = doit;
        any |= doit;
      }
      // identical in every CTA: the whole cluster skips or rotates together
      if (!__syncthreads_or(any)) continue;
      // all reads of the round's inputs done before any CTA writes: the values
      // are already consumed (the tables above hold their results), so the
      // arrive needs no release fence
      asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
      // diagonal 2x2 blocks: the owner of row p writes them
      for (int k = tid; k < half; k += nth) {
        if (!rot[k] || (pq[2 * k] % kJcCluster) != rank) continue;
        const int p = pq[2 * k], q = pq[2 * k + 1];
        const double t = dg[4 * k], app = dg[4 * k + 1], aqq = dg[4 * k + 2], apq = dg[4 * k + 3];
        *W.a(p, p) = app - t * apq;
        *W.a(q, q) = aqq + t * apq;
        *W.a(p, q) = 0.0;
      }
      // off-diagonal 2x2 blocks (I < K) over the whole cluster
      for (long long b = (long long)rank * nth + tid; b < nblk; b += (long long)kJcCluster * nth) {
        const int g = (int)(b / (half - 1)), e = (int)(b % (half - 1));
        const int I1 = g, I2 = half - 1 - g;
        int I, K;
        if (e < half - 1 - I1) { I = I1; K = I1 + 1 + e; } else { I = I2; K = I2 + 1 + (e - (half - 1 - I1)); }
        if (!(rot[I] | rot[K])) continue;
        const int p = pq[2 * I], q = pq[2 * I + 1], r2 = pq[2 * K], s2 = pq[2 * K + 1];
        const double c = cs[2 * I], sn = cs[2 * I + 1], c2 = cs[2 * K], s2n = cs[2 * K + 1];
        double* e_pr = W.a(p, r2);
        double* e_ps = W.a(p, s2);
        double* e_qr = W.a(q, r2);
        double* e_qs = W.a(q, s2);
        const double b00 = *e_pr, b01 = *e_ps, b10 = *e_qr, b11 = *e_qs;
        const double y00 = c * b00 - sn * b10, y01 = c * b01 - sn * b11;
        const double y10 = sn * b00 + c * b10, y11 = sn * b01 + c * b11;
        *e_pr = y00 * c2 - y01 * s2n;
        *e_ps = y00 * s2n + y01 * c2;
        *e_qr = y10 * c2 - y11 * s2n;
        *e_qs = y10 * s2n + y11 * c2;
      }
      // V rows p, q: this CTA's column slice of every rotated pair
      if (c1 > c0) {
        const int w = c1 - c0;
        for (int e = tid; e < half * w; e += nth) {
          const int k = e / w, mu = c0 + (e - k * w);
          if (!rot[k]) continue;
          const int p = pq[2 * k], q = pq[2 * k + 1];
          const double c = cs[2 * k], sn = cs[2 * k + 1];
          double* vp = W.v(p, mu);
          double* vq = W.v(q, mu);
          const double a = *vp, bq = *vq;
          *vp = c * a - sn * bq;
          *vq = sn * a + c * bq;
        }
      }
      cluster.sync();                          // the round's writes visible everywhere
    }
    // converged when every rotation the sweep applied was at round-off level
    // (offmax is identical in every CTA: all of them saw every pivot)
    for (int o = 16; o > 0; o >>= 1) { const double t = __shfl_xor_sync(0xffffffffu, offmax, o); offmax = t > offmax ? t : offmax; }
    if ((tid & 31) == 0) red[tid >> 5] = offmax;
    __syncthreads();
    if (tid == 0) {
      double mx = 0.0;
      for (int w = 0; w < (nth >> 5); ++w) mx = red[w] > mx ? red[w] : mx;
      red[33] = mx;
    }
    __syncthreads();
    const bool done = red[33] <= thresh;
    __syncthreads();
    if (done) { ++sweep; break; }
  }

  // ---- rank by eigenvalue, sign fix, write this CTA's rows ------------------
  for (int lr = tid; lr < rows; lr += nth) {
    const int i = lr * kJcCluster + rank;
    if (i >= n) continue;
    const double li = Aloc[(long long)lr * np + i];
    int rk = 0;
    for (int j = 0; j < n; ++j) {
      const double lj = *W.a(j, j);
      rk += (lj < li) || (lj == li && j < i);
    }
    double sum = 0.0;
    for (int mu = 0; mu < n; ++mu) sum += Vloc[(long long)lr * np + mu];
    const double sg = sum < 0.0 ? -1.0 : 1.0;
    eps_out[mol.vec0 + rk] = li;
    double* Co = Cout + mol.mat0 + (long long)rk * n;
    for (int mu = 0; mu < n; ++mu) Co[mu] = sg * Vloc[(long long)lr * np + mu];
  }
  if (rank == 0 && tid == 0 && sweeps_out) sweeps_out[m] += sweep;
  cluster.sync();                              // no CTA leaves while others read its diagonal
}

// Clusters that fit at once on this device for the cluster kernel at basis n
// (0: not launchable, use the one-CTA kernel).  Queried once, for the largest
// basis the kernel serves (the largest shared-memory footprint), under
// std::call_once: lanes of the server call this from several host threads.
int jacobi_cluster_capacity(int n) {
  static std::once_flag once;
  static int capacity = 0;
  std::call_once(once, []() {
    const size_t bytes = jacobi_cluster_smem_bytes(kSmallJacobiMaxN);
    int val = 0;
    if (bytes <= 232448 &&
        cudaFuncSetAttribute(jacobi_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448) ==
            cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kJcCluster, 1, 1);
      cfg.blockDim = dim3(512, 1, 1);
      cfg.dynamicSmemBytes = bytes;
      cudaLaunchAttribute attr;
      attr.id = cudaLaunchAttributeClusterDimension;
      attr.val.clusterDim.x = kJcCluster;
      attr.val.clusterDim.y = 1;
      attr.val.clusterDim.z = 1;
      cfg.attrs = &attr;
      cfg.numAttrs = 1;
      if (cudaOccupancyMaxActiveClusters(&val, jacobi_cluster_kernel, &cfg) != cudaSuccess) val = 0;
    }
    cudaGetLastError();
    capacity = val;
  });
  return n <= kSmallJacobiMaxN ? capacity : 0;
}

void launch_jacobi_cluster_f64(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                               int require_active, const double* G, const double* F, const double* Cin, int use_basis,
                               double* Cout, double* eps, int max_sweeps, int* sweeps_out, cudaStream_t s) {
  if (nlist <= 0) return;
  const size_t bytes = jacobi_cluster_smem_bytes(max_n);
  const int threads = jac_np(max_n) <= 64 ? 256 : 512;
  jacobi_cluster_kernel<<<nlist * kJcCluster, threads, bytes, s>>>(mols, mol_list, st, require_active, G, F, Cin,
                                                                   use_basis, Cout, eps, max_sweeps, sweeps_out);
}

}  // namespace nddo
