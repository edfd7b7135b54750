// Kernels (c) and (e): batched dense contractions and the density-DIIS step.
//
// (c) gemm_kernel -- one launch multiplies a list of per-molecule matrices of
//     different shapes ("jobs"); each CTA computes one 64x64 tile of one job.
//     Used for the warm-start transform G = C_prev F C_prev^T, the density
//     P = 2 C_occ^T C_occ (MolDS Cndo2::CalcOrbitalElectronPopulation,
//     src/cndo/Cndo2.cpp:1702-1719 via Blas::Dsyrk) and the FP64 subspace
//     refinement of the mixed-precision path.  The arithmetic type is a template
//     parameter: FP32 in the early iterations, FP64 after the switch and on the
//     plain FP64 path.
//
// (e) DIIS -- partial / solve / apply kernels: RMS density change and convergence
//     test (Cndo2::SatisfyConvergenceCriterion, src/cndo/Cndo2.cpp:1472-1517),
//     density DIIS with MolDS's exact window/acceptance rules (Cndo2::DoDIIS,
//     :920-1028) and damping (Cndo2::DoDamp, :1030-1061).  The DIIS history is
//     a ring buffer instead of MolDS's memmove shift; the linear system is
//     assembled in chronological order so it is the same system.  All
//     reductions use fixed-order trees.
#include <cuda_runtime.h>
#include "nddo_batch.cuh"
#include "kernels.h"

namespace nddo {

constexpr int kTile = 64, kTileK = 16, kGemmThreads = 256;

template <typename TA, typename TB, typename TC, typename TAcc, bool TA_, bool TB_>
__global__ void __launch_bounds__(kGemmThreads)
gemm_kernel(const GemmJob* __restrict__ jobs, int njobs, const TA* __restrict__ A, const TB* __restrict__ B,
            TC* __restrict__ C, const MolState* __restrict__ st, int require_active, int require_phase) {
  __shared__ TAcc As[kTileK][kTile + 1];
  __shared__ TAcc Bs[kTileK][kTile + 1];
  // job of this tile (jobs sorted by tile0)
  int lo = 0, hi = njobs - 1;
  const int t = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].tile0 <= t) lo = mid; else hi = mid - 1;
  }
  const GemmJob job = jobs[lo];
  if (require_active && st[job.mol].status != kActive) return;
  if (require_phase >= 0 && st[job.mol].phase != require_phase) return;
  const int local = t - job.tile0;
  int tm, tn;
  if (job.sym) {
    // upper-triangle tile order: row tm holds tiles tm..T-1
    const int T = job.tiles_n;
    tm = 0;
    int rem = local;
    while (rem >= T - tm) { rem -= T - tm; ++tm; }
    tn = tm + rem;
  } else {
    tm = local / job.tiles_n;
    tn = local % job.tiles_n;
  }
  const int row0 = tm * kTile, col0 = tn * kTile;
  const TA* Aj = A + job.a_off;
  const TB* Bj = B + job.b_off;
  TC* Cj = C + job.c_off;
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  TAcc acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0;

  for (int k0 = 0; k0 < job.K; k0 += kTileK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * kGemmThreads;
      int ii, kk;
      if (TA_) { kk = e >> 6; ii = e & 63; } else { ii = e >> 4; kk = e & 15; }
      const int gi = row0 + ii, gk = k0 + kk;
      TAcc v = 0;
      if (gi < job.M && gk < job.K) v = (TAcc)(TA_ ? Aj[(long long)gk * job.lda + gi] : Aj[(long long)gi * job.lda + gk]);
      As[kk][ii] = v;
      int jj, kb;
      if (TB_) { jj = e >> 4; kb = e & 15; } else { kb = e >> 6; jj = e & 63; }
      const int gj = col0 + jj, gkb = k0 + kb;
      TAcc w = 0;
      if (gj < job.N && gkb < job.K) w = (TAcc)(TB_ ? Bj[(long long)gj * job.ldb + gkb] : Bj[(long long)gkb * job.ldb + gj]);
      Bs[kb][jj] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTileK; ++kk) {
      TAcc a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gi = row0 + ty * 4 + i;
    if (gi >= job.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gj = col0 + tx * 4 + j;
      if (gj >= job.N) continue;
      TC* c = Cj + (long long)gi * job.ldc + gj;
      double v = job.alpha * (double)acc[i][j];
      if (gi == gj) v += job.diag;
      *c = (TC)(job.beta != 0.0 ? v + job.beta * (double)(*c) : v);
      if (job.sym && tm != tn) {   // mirror (beta is zero for symmetric jobs)
        TC* cm = Cj + (long long)gj * job.ldc + gi;
        *cm = (TC)v;
      }
    }
  }
}

int gemm_tiles(int M, int N) { return ((M + kTile - 1) / kTile) * ((N + kTile - 1) / kTile); }
int gemm_tiles_n(int N) { return (N + kTile - 1) / kTile; }
int gemm_tiles_sym(int N) { const int T = (N + kTile - 1) / kTile; return T * (T + 1) / 2; }

#define GEMM_LAUNCH(TA, TB, TC, TACC)                                                                        \
  void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const TA* A, const TB* B, TC* C, bool ta,      \
                   bool tb, TACC /*acc tag*/, const MolState* st, int require_active, int require_phase,        \
                   cudaStream_t s) {                                                                         \
    if (ntiles <= 0 || njobs <= 0) return;                                                                   \
    if (!ta && !tb) gemm_kernel<TA, TB, TC, TACC, false, false><<<ntiles, kGemmThreads, 0, s>>>(jobs, njobs, A, B, C, st, require_active, require_phase); \
    else if (ta && !tb) gemm_kernel<TA, TB, TC, TACC, true, false><<<ntiles, kGemmThreads, 0, s>>>(jobs, njobs, A, B, C, st, require_active, require_phase); \
    else if (!ta && tb) gemm_kernel<TA, TB, TC, TACC, false, true><<<ntiles, kGemmThreads, 0, s>>>(jobs, njobs, A, B, C, st, require_active, require_phase); \
    else gemm_kernel<TA, TB, TC, TACC, true, true><<<ntiles, kGemmThreads, 0, s>>>(jobs, njobs, A, B, C, st, require_active, require_phase); \
  }
GEMM_LAUNCH(double, double, double, double)
GEMM_LAUNCH(double, double, double, float)
GEMM_LAUNCH(double, double, float, float)
GEMM_LAUNCH(float, double, float, float)
GEMM_LAUNCH(double, float, float, float)
GEMM_LAUNCH(float, double, double, float)
#undef GEMM_LAUNCH

// ---------------------------------------------------------------------------
// deterministic block reduction helpers (blockDim = 256)
// ---------------------------------------------------------------------------
constexpr int kDiisThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += scratch[i];
    scratch[32] = r;
  }
  __syncthreads();
  r = scratch[32];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) { double t = __shfl_xor_sync(0xffffffffu, v, o); v = t > v ? t : v; }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = scratch[i] > r ? scratch[i] : r;
    scratch[32] = r;
  }
  __syncthreads();
  const double r = scratch[32];
  __syncthreads();
  return r;
}

// One SCF bookkeeping step per molecule, after the new density P is formed,
// in three launches so that each molecule's N^2 streams are spread over many
// CTAs: (1) partial sums over fixed chunks of the molecule's matrix (sum e^2,
// max |e|, the new B row) while the new history entry is written; (2) one
// thread per molecule reduces the chunks in order and runs the convergence
// test, the DIIS solve, damping and the phase switch; (3) the extrapolation
// and damping over the same chunks.  The chunking depends only on N, and the
// chunk partials are reduced in a fixed order, so a molecule's result does not
// depend on the rest of the batch.
constexpr int kDiisChunksMax = 64;
constexpr int kDiisPart = 2 + kMaxDiis;     // sum e^2, max |e|, dots

__device__ __forceinline__ int diis_chunks(long long n2) {
  const long long c = (n2 + 4095) / 4096;
  return (int)(c < kDiisChunksMax ? (c < 1 ? 1 : c) : kDiisChunksMax);
}

struct DiisStep {          // decisions of kernel (2) read by kernel (3)
  double coef[kMaxDiis];
  int apply, damp, active, pad;
};

__global__ void __launch_bounds__(kDiisThreads)
diis_partial_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list, const MolState* __restrict__ st,
                    ScfParamsDev prm, const double* __restrict__ P, const double* __restrict__ Pold,
                    double* __restrict__ hist_dens, double* __restrict__ hist_err, long long hist_stride,
                    double* __restrict__ part) {
  __shared__ double scratch[40];
  const int li = blockIdx.y;
  const int m = mol_list[li];
  const MolState s = st[m];
  if (s.status != kActive) return;
  const DevMol mol = mols[m];
  const long long n2 = (long long)mol.nao * mol.nao;
  const int chunks = diis_chunks(n2);
  if ((int)blockIdx.x >= chunks) return;
  const long long len = (n2 + chunks - 1) / chunks;
  const long long lo = blockIdx.x * len, hi = (lo + len < n2) ? lo + len : n2;
  const bool is_guess = (s.iter == 0 && s.requires_guess);
  const int M = prm.diis_m;
  const bool do_diis = !is_guess && M > 0;
  const int slot = do_diis ? (s.diis_count % M) : 0;
  const int count = do_diis ? min(s.diis_count + 1, M) : 0;
  const double* Pm = P + mol.mat0;
  const double* Po = Pold + mol.mat0;
  double* dslot = hist_dens + slot * hist_stride + mol.mat0;
  double* eslot = hist_err + slot * hist_stride + mol.mat0;
  double sq = 0.0, mx = 0.0;
  double dots[kMaxDiis];
#pragma unroll
  for (int k = 0; k < kMaxDiis; ++k) dots[k] = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double p = Pm[i];
    const double e = p - Po[i];
    sq += e * e;
    const double ae = fabs(e);
    mx = ae > mx ? ae : mx;
    if (do_diis) {
      dslot[i] = p;
      eslot[i] = e;
#pragma unroll
      for (int k = 0; k < kMaxDiis; ++k)
        if (k < count) dots[k] += (k == slot ? e : hist_err[k * hist_stride + mol.mat0 + i]) * e;
    }
  }
  const double sumsq = block_sum(sq, scratch);
  const double maxe = block_max(mx, scratch);
  double dsum[kMaxDiis];
#pragma unroll
  for (int k = 0; k < kMaxDiis; ++k) dsum[k] = (k < count) ? block_sum(dots[k], scratch) : 0.0;
  if (threadIdx.x == 0) {
    double* o = part + ((long long)li * kDiisChunksMax + blockIdx.x) * kDiisPart;
    o[0] = sumsq;
    o[1] = maxe;
    for (int k = 0; k < kMaxDiis; ++k) o[2 + k] = dsum[k];
  }
}

__global__ void diis_solve_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list, int nlist,
                                  MolState* __restrict__ st, ScfParamsDev prm, const double* __restrict__ part,
                                  DiisStep* __restrict__ steps, TraceEntry* __restrict__ trace, int trace_len) {
  const int li = blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= nlist) return;
  DiisStep out;
  for (int k = 0; k < kMaxDiis; ++k) out.coef[k] = 0.0;
  out.apply = 0; out.damp = 0; out.active = 0; out.pad = 0;
  const int m = mol_list[li];
  MolState* s = st + m;
  if (s->status != kActive) { steps[li] = out; return; }
  out.active = 1;
  const DevMol mol = mols[m];
  const long long n2 = (long long)mol.nao * mol.nao;
  const int chunks = diis_chunks(n2);
  const int iter = s->iter;
  const bool is_guess = (iter == 0 && s->requires_guess);
  const int M = prm.diis_m;
  const bool do_diis = !is_guess && M > 0;
  const int slot = do_diis ? (s->diis_count % M) : 0;
  const int count = do_diis ? min(s->diis_count + 1, M) : 0;
  double sumsq = 0.0, maxe = 0.0, dsum[kMaxDiis];
  for (int k = 0; k < kMaxDiis; ++k) dsum[k] = 0.0;
  for (int c = 0; c < chunks; ++c) {      // fixed order
    const double* p = part + ((long long)li * kDiisChunksMax + c) * kDiisPart;
    sumsq += p[0];
    maxe = p[1] > maxe ? p[1] : maxe;
    for (int k = 0; k < kMaxDiis; ++k) dsum[k] += p[2 + k];
  }
  const double rms = sqrt(sumsq / (double)n2);
  if (trace && iter < trace_len) {
    TraceEntry te;
    te.rms = rms; te.diis_err = s->diis_err; te.diis_on = s->diis_on; te.damp_on = s->damp_on;
    trace[(long long)m * trace_len + iter] = te;
  }
  s->rms = rms;
  if (rms < prm.rms_density) {
    s->status = kConverged;
    out.active = 0;
    steps[li] = out;
    return;
  }
  if (!is_guess) {
    if (do_diis) {
      for (int k = 0; k < count; ++k) { s->B[k * kMaxDiis + slot] = dsum[k]; s->B[slot * kMaxDiis + k] = dsum[k]; }
      s->diis_count += 1;
      s->diis_head = slot;
      s->diis_err = maxe;
      const bool apply = (M <= iter) && (prm.diis_end < maxe) && (maxe < prm.diis_start) && (count == M);
      if (apply) {
        // chronological order: oldest ... newest
        int chron[kMaxDiis];
        for (int k = 0; k < M; ++k) chron[k] = (slot + 1 + k) % M;
        double a[(kMaxDiis + 1) * (kMaxDiis + 1)], b[kMaxDiis + 1];
        const int n = M + 1;
        for (int i = 0; i < M; ++i)
          for (int j = 0; j < M; ++j) a[i * n + j] = s->B[chron[i] * kMaxDiis + chron[j]];
        for (int i = 0; i < M; ++i) { a[i * n + M] = -1.0; a[M * n + i] = -1.0; b[i] = 0.0; }
        a[M * n + M] = 0.0;
        b[M] = -1.0;
        // Gaussian elimination with partial pivoting; an exactly zero pivot
        // means a singular system, which MolDS answers by skipping the step
        bool singular = false;
        for (int c = 0; c < n && !singular; ++c) {
          int piv = c;
          for (int r = c + 1; r < n; ++r) if (fabs(a[r * n + c]) > fabs(a[piv * n + c])) piv = r;
          if (a[piv * n + c] == 0.0) { singular = true; break; }
          if (piv != c) {
            for (int j = 0; j < n; ++j) { double t = a[c * n + j]; a[c * n + j] = a[piv * n + j]; a[piv * n + j] = t; }
            double t = b[c]; b[c] = b[piv]; b[piv] = t;
          }
          for (int r = c + 1; r < n; ++r) {
            const double f = a[r * n + c] / a[c * n + c];
            for (int j = c; j < n; ++j) a[r * n + j] -= f * a[c * n + j];
            b[r] -= f * b[c];
          }
        }
        if (!singular) {
          for (int c = n - 1; c >= 0; --c) {
            double v = b[c];
            for (int j = c + 1; j < n; ++j) v -= a[c * n + j] * b[j];
            b[c] = v / a[c * n + c];
          }
          for (int k = 0; k < M; ++k) out.coef[k] = b[k];
          out.apply = 1;
        }
      }
      s->diis_on = out.apply;
    }
    out.damp = (prm.damping_weight > 0.0 && prm.damping_thresh < rms) ? 1 : 0;
    s->damp_on = out.damp;
    if (prm.precision == 1 && s->phase == 0 && do_diis && maxe < prm.switch_error) s->phase = 1;
  }
  s->iter = iter + 1;
  if (s->iter >= prm.max_iter) s->status = kNotConverged;
  steps[li] = out;
}

__global__ void __launch_bounds__(kDiisThreads)
diis_apply_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list, const MolState* __restrict__ st,
                  ScfParamsDev prm, double* __restrict__ P, const double* __restrict__ Pold,
                  const double* __restrict__ hist_dens, long long hist_stride, const DiisStep* __restrict__ steps) {
  const int li = blockIdx.y;
  const DiisStep d = steps[li];
  if (!d.active || (!d.apply && !d.damp)) return;
  const int m = mol_list[li];
  const DevMol mol = mols[m];
  const long long n2 = (long long)mol.nao * mol.nao;
  const int chunks = diis_chunks(n2);
  if ((int)blockIdx.x >= chunks) return;
  const long long len = (n2 + chunks - 1) / chunks;
  const long long lo = blockIdx.x * len, hi = (lo + len < n2) ? lo + len : n2;
  const int M = prm.diis_m;
  double* Pm = P + mol.mat0;
  const double* Po = Pold + mol.mat0;
  // the newest entry is the one this iteration pushed (diis_head)
  const int newest = st[m].diis_head;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    double v = Pm[i];
    if (d.apply) {
      // P = sum_k c_k P_k in chronological order (MolDS sums the stored
      // densities in slot order through Dgemv)
      v = 0.0;
      for (int k = 0; k < M; ++k) {
        const int rs = (newest + 1 + k) % M;
        v += d.coef[k] * hist_dens[rs * hist_stride + mol.mat0 + i];
      }
    }
    if (d.damp) v = v * (1.0 - prm.damping_weight) + prm.damping_weight * Po[i];
    Pm[i] = v;
  }
}

void launch_diis(const DevMol* mols, const int* mol_list, int nlist, MolState* st, const ScfParamsDev& prm,
                 double* P, const double* Pold, double* hist_dens, double* hist_err, long long hist_stride,
                 TraceEntry* trace, int trace_len, void* scratch, cudaStream_t s) {
  if (nlist <= 0) return;
  double* part = static_cast<double*>(scratch);
  DiisStep* steps = reinterpret_cast<DiisStep*>(part + (size_t)nlist * kDiisChunksMax * kDiisPart);
  diis_partial_kernel<<<dim3(kDiisChunksMax, nlist), kDiisThreads, 0, s>>>(mols, mol_list, st, prm, P, Pold, hist_dens,
                                                                          hist_err, hist_stride, part);
  diis_solve_kernel<<<(nlist + 63) / 64, 64, 0, s>>>(mols, mol_list, nlist, st, prm, part, steps, trace, trace_len);
  diis_apply_kernel<<<dim3(kDiisChunksMax, nlist), kDiisThreads, 0, s>>>(mols, mol_list, st, prm, P, Pold, hist_dens,
                                                                        hist_stride, steps);
}

size_t diis_scratch_bytes(int slots) {
  return (size_t)slots * kDiisChunksMax * kDiisPart * sizeof(double) + (size_t)slots * sizeof(DiisStep) + 256;
}

// ---------------------------------------------------------------------------
// small elementwise helpers
// ---------------------------------------------------------------------------
// FP64 refinement (one Newton step of Ogita & Aishima's eigenvector refinement,
// restricted to the occupied columns): with approximate eigenvectors x and
// eigenvalues lam, K_ai = -(x_a^T F x_i - lam_i x_a^T x_i) / (lam_a - lam_i),
// a virtual, i occupied.  The overlap term removes the first-order error left
// by the non-orthogonality of FP32 eigenvectors.
__global__ void newton_scale_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                                    const MolState* __restrict__ st, int require_phase, double* __restrict__ K,
                                    const double* __restrict__ O, const double* __restrict__ eps) {
  const int m = mol_list[blockIdx.y];
  if (st[m].status != kActive || (require_phase >= 0 && st[m].phase != require_phase)) return;
  const DevMol mol = mols[m];
  const int n = mol.nao, o = mol.nocc, v = n - o;
  const long long cnt = (long long)v * o;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e / o), i = (int)(e % o);
    const double li = eps[mol.vec0 + i];
    const double gap = eps[mol.vec0 + o + a] - li;
    K[mol.mat0 + e] = -(K[mol.mat0 + e] - li * O[mol.mat0 + e]) / gap;
  }
}

void launch_newton_scale(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, int require_phase,
                         double* K, const double* O, const double* eps, cudaStream_t s) {
  if (nlist <= 0) return;
  newton_scale_kernel<<<dim3(8, nlist), 256, 0, s>>>(mols, mol_list, st, require_phase, K, O, eps);
}

// D = M - I in place (o x o): the first-order (Y^T Y)^-1 = I - D is applied by
// the caller as Z = Y - D Y.
__global__ void neumann_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                               const MolState* __restrict__ st, int require_phase, double* __restrict__ Mm) {
  const int m = mol_list[blockIdx.y];
  if (st[m].status != kActive || (require_phase >= 0 && st[m].phase != require_phase)) return;
  const DevMol mol = mols[m];
  const int o = mol.nocc;
  const long long cnt = (long long)o * o;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / o), j = (int)(e % o);
    if (i == j) Mm[mol.mat0 + e] -= 1.0;
  }
}

void launch_neumann(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, int require_phase,
                    double* M, cudaStream_t s) {
  if (nlist <= 0) return;
  neumann_kernel<<<dim3(8, nlist), 256, 0, s>>>(mols, mol_list, st, require_phase, M);
}

// copy the first `rows` rows of C (n x n, row-major) into dst (rows x n)
__global__ void copy_rows_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                                 const MolState* __restrict__ st, int require_phase, const double* __restrict__ src,
                                 double* __restrict__ dst) {
  const int m = mol_list[blockIdx.y];
  if (st[m].status != kActive || (require_phase >= 0 && st[m].phase != require_phase)) return;
  const DevMol mol = mols[m];
  const long long cnt = (long long)mol.nocc * mol.nao;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x)
    dst[mol.mat0 + e] = src[mol.mat0 + e];
}

void launch_copy_occ_rows(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, int require_phase,
                          const double* src, double* dst, cudaStream_t s) {
  if (nlist <= 0) return;
  copy_rows_kernel<<<dim3(8, nlist), 256, 0, s>>>(mols, mol_list, st, require_phase, src, dst);
}

// FP32 shadows of the basis C (twice: operand and Newton-Schulz output) and of
// F for the tensor-core chain of the FP32 phase: one conversion per element
// and iteration instead of one per tile that loads it
__global__ void tc_shadows_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                                  const MolState* __restrict__ st, const double* __restrict__ C,
                                  const double* __restrict__ F, float* __restrict__ Cf, float* __restrict__ Cf2,
                                  float* __restrict__ Ff) {
  const int m = mol_list[blockIdx.y];
  if (st[m].status != kActive) return;
  const DevMol mol = mols[m];
  const long long cnt = (long long)mol.nao * mol.nao;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
    const float c = (float)C[mol.mat0 + e];
    Cf[mol.mat0 + e] = c;
    Cf2[mol.mat0 + e] = c;
    Ff[mol.mat0 + e] = (float)F[mol.mat0 + e];
  }
}

void launch_tc_shadows(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, const double* C,
                       const double* F, float* Cf, float* Cf2, float* Ff, cudaStream_t s) {
  if (nlist <= 0) return;
  tc_shadows_kernel<<<dim3(16, nlist), 256, 0, s>>>(mols, mol_list, st, C, F, Cf, Cf2, Ff);
}

// copy each listed active molecule's N x N block (src -> dst, same offsets)
__global__ void copy_matrices_kernel(const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                                     const MolState* __restrict__ st, const double* __restrict__ src,
                                     double* __restrict__ dst) {
  const int m = mol_list[blockIdx.y];
  if (st[m].status != kActive) return;
  const DevMol mol = mols[m];
  const long long cnt = (long long)mol.nao * mol.nao;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x)
    dst[mol.mat0 + e] = src[mol.mat0 + e];
}

void launch_copy_matrices(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, const double* src,
                          double* dst, cudaStream_t s) {
  if (nlist <= 0) return;
  copy_matrices_kernel<<<dim3(16, nlist), 256, 0, s>>>(mols, mol_list, st, src, dst);
}

}  // namespace nddo
