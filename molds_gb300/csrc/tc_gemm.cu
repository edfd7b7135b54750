// Kernel (c) on the tensor cores: batched 3xTF32 GEMM with tcgen05.
//
// The FP32-phase contractions of the mixed-precision path -- the warm-start
// transform G = C F C^T, the Newton-Schulz step C <- 1.5 C - 0.5 (C C^T) C and
// the phase-0 density P = 2 C_occ^T C_occ -- run here instead of on the CUDA
// cores.  One CTA computes one 128 x 128 tile of one job of the same job list
// the CUDA-core gemm_kernel takes (per-molecule matrices of different sizes).
//
//   * operands: loaded from global (FP64 or FP32, either orientation),
//     rounded to FP32, split x = hi + lo with hi = tf32(x) (round to nearest)
//     and stored to shared memory in the K-major, no-swizzle canonical layout
//     (core matrix 8 rows x 16 bytes; K-adjacent core matrices 128 B apart,
//     8-row groups 1 KB apart for a 32-wide K chunk);
//   * MMA: one thread issues tcgen05.mma.cta_group::1.kind::tf32 (M = N = 128,
//     K = 8) for hi*hi + hi*lo + lo*hi into one FP32 accumulator in tensor
//     memory (128 columns allocated per CTA), then tcgen05.commit to an
//     mbarrier that the CTA waits on (bounded: a wait that runs out sets the
//     error word and the tile is skipped);
//   * epilogue: each warp reads its 32 accumulator lanes (rows) with
//     tcgen05.ld and writes alpha * acc + beta * C.
// The three products give about 2e-6 relative accuracy (measured against
// FP64), an order above FP32 SIMT accumulation: the FP32 phase only has to
// bring the SCF to the FP64 switch (DIIS error 1e-4), and the FP64 Newton step
// of phase 1 squares the remaining eigenvector error.
#include <cuda_runtime.h>
#include <stdint.h>
#include "nddo_batch.cuh"
#include "kernels.h"

namespace nddo {

constexpr int kTcT = 128;          // tile edge (M = N of one MMA)
constexpr int kTcK = 32;           // K chunk staged per round
constexpr int kTcThreads = 256;
constexpr int kTcTileBytes = kTcT * kTcK * 4;
constexpr int kTcOutLd = kTcT + 1;          // padded row of the output staging tile
constexpr int kTcSmem = (4 * kTcTileBytes > kTcT * kTcOutLd * 4) ? 4 * kTcTileBytes : kTcT * kTcOutLd * 4;

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in the K-major no-swizzle layout of a 128 x 32 tile
__device__ __forceinline__ int tc_off(int r, int k) {
  return ((r >> 3) * (kTcK / 4) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);                    // start address
  d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;              // K-adjacent core matrices
  d |= (uint64_t)(((kTcK / 4) * 128u >> 4) & 0x3FFF) << 32; // 8-row groups
  d |= (uint64_t)1 << 46;                                   // descriptor version
  return d;                                                 // layout: no swizzle
}

__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
               :: "r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

template <typename TA, typename TB, typename TC, bool TA_, bool TB_>
__global__ void __launch_bounds__(kTcThreads, 2)
tc_gemm_kernel(const GemmJob* __restrict__ jobs, int njobs, const TA* __restrict__ A, const TB* __restrict__ B,
               TC* __restrict__ C, const MolState* __restrict__ st, int require_active, int require_phase,
               int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  // job of this tile (jobs sorted by tc_tile0)
  int lo = 0, hi = njobs - 1;
  const int t = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].tc_tile0 <= t) lo = mid; else hi = mid - 1;
  }
  const GemmJob job = jobs[lo];
  if (require_active && st[job.mol].status != kActive) return;
  if (require_phase >= 0 && st[job.mol].phase != require_phase) return;
  const int local = t - job.tc_tile0;
  int tm, tn;
  if (job.sym) {
    const int T = job.tc_tiles_n;
    tm = 0;
    int rem = local;
    while (rem >= T - tm) { rem -= T - tm; ++tm; }
    tn = tm + rem;
  } else {
    tm = local / job.tc_tiles_n;
    tn = local % job.tc_tiles_n;
  }
  const int row0 = tm * kTcT, col0 = tn * kTcT;
  const TA* Aj = A + job.a_off;
  const TB* Bj = B + job.b_off;
  TC* Cj = C + job.c_off;
  unsigned char* a_hi = tc_sm;
  unsigned char* a_lo = tc_sm + kTcTileBytes;
  unsigned char* b_hi = tc_sm + 2 * kTcTileBytes;
  unsigned char* b_lo = tc_sm + 3 * kTcTileBytes;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(tc_smem_u32(&tmem_base)), "r"(kTcT));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(tc_smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  // kind::tf32: D = F32, A = B = TF32, both K-major, N = M = 128
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcT >> 3) << 17) |
                         ((uint32_t)(kTcT >> 4) << 24);
  uint32_t phase = 0;
  bool ok = true;
  int issued = 0;
  for (int k0 = 0; k0 < job.K; k0 += kTcK) {
    // stage A rows row0.. (r, k) and B columns col0.. (n, k), both K-major.
    // A warp fills whole core matrices (8 rows x 4 k = 128 contiguous bytes,
    // lane l -> row l / 4, k l % 4), so the shared-memory stores never
    // conflict; all global loads of a chunk are issued before any store.
    constexpr int kPer = kTcT * kTcK / 32 / (kTcThreads / 32);   // core matrices per warp and operand
    constexpr int kBatch = 8;                                     // loads in flight per operand
#pragma unroll
    for (int i0 = 0; i0 < kPer; i0 += kBatch) {
      float va[kBatch], vb[kBatch];
#pragma unroll
      for (int i = 0; i < kBatch; ++i) {
        const int cm = warp + (i0 + i) * (kTcThreads / 32);
        const int r = (cm >> 3) * 8 + (lane >> 2), k = (cm & 7) * 4 + (lane & 3);
        const int gi = row0 + r, gj = col0 + r, gk = k0 + k;
        va[i] = (gi < job.M && gk < job.K)
                    ? (float)(TA_ ? Aj[(long long)gk * job.lda + gi] : Aj[(long long)gi * job.lda + gk]) : 0.f;
        vb[i] = (gj < job.N && gk < job.K)
                    ? (float)(TB_ ? Bj[(long long)gj * job.ldb + gk] : Bj[(long long)gk * job.ldb + gj]) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < kBatch; ++i) {
        const int cm = warp + (i0 + i) * (kTcThreads / 32);
        const float ha = tc_tf32(va[i]), hb = tc_tf32(vb[i]);
        reinterpret_cast<float*>(a_hi)[cm * 32 + lane] = ha;
        reinterpret_cast<float*>(a_lo)[cm * 32 + lane] = va[i] - ha;
        reinterpret_cast<float*>(b_hi)[cm * 32 + lane] = hb;
        reinterpret_cast<float*>(b_lo)[cm * 32 + lane] = vb[i] - hb;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ah = tc_smem_u32(a_hi), al = tc_smem_u32(a_lo), bh = tc_smem_u32(b_hi), bl = tc_smem_u32(b_lo);
      for (int s = 0; s < kTcK / 8; ++s) {
        const uint32_t off = s * 256;   // two K-adjacent core matrices per K = 8 step
        tc_mma(tmem, tc_desc(ah + off), tc_desc(bh + off), idesc, issued ? 1u : 0u);
        tc_mma(tmem, tc_desc(ah + off), tc_desc(bl + off), idesc, 1u);
        tc_mma(tmem, tc_desc(al + off), tc_desc(bh + off), idesc, 1u);
        issued = 1;
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                   :: "r"(tc_smem_u32(&mbar)));
    }
    // every thread waits for the MMAs before the staging buffers are reused
    uint32_t done = 0;
    for (int it = 0; it < (1 << 24) && !done; ++it) {
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                   " selp.u32 %0, 1, 0, p;\n}"
                   : "=r"(done) : "r"(tc_smem_u32(&mbar)), "r"(phase));
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!__syncthreads_and(done != 0)) { ok = false; break; }
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
  } else {
    // warp w reads TMEM lanes 32 (w % 4) .. + 31 (a warp may only access its
    // quarter of the lanes; warps w and w + 4 take alternate column groups)
    // into a padded shared tile, which is then written out row-coalesced
    float* S = reinterpret_cast<float*>(tc_sm);   // the operand tiles are no longer needed
    const int q = warp & 3, half = warp >> 2;
    const int r = q * 32 + lane;
    for (int c0 = half * 8; c0 < kTcT; c0 += 16) {
      uint32_t v[8];
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                   : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int j = 0; j < 8; ++j) S[r * kTcOutLd + c0 + j] = __uint_as_float(v[j]);
    }
    __syncthreads();
    for (int e = tid; e < kTcT * kTcT; e += kTcThreads) {
      const int i = e / kTcT, j = e % kTcT;
      const int gi = row0 + i, gj = col0 + j;
      if (gi < job.M && gj < job.N) {
        TC* c = Cj + (long long)gi * job.ldc + gj;
        if (sizeof(TC) == 4) {            // FP32 output: FP32 arithmetic (GB300's FP64 pipe is 1/64 rate)
          const float a = (float)job.alpha * S[i * kTcOutLd + j];
          *c = (TC)(job.beta != 0.0 ? a + (float)job.beta * (float)(*c) : a);
        } else {
          double a = job.alpha * (double)S[i * kTcOutLd + j];
          if (gi == gj) a += job.diag;
          *c = (TC)(job.beta != 0.0 ? a + job.beta * (double)(*c) : a);
        }
      }
      if (job.sym && tm != tn) {
        // mirror tile (beta is zero for symmetric jobs): C[col0 + i][row0 + j] = acc[j][i]
        const int mi = col0 + i, mj = row0 + j;
        if (mi < job.N && mj < job.M) Cj[(long long)mi * job.ldc + mj] = (TC)((float)job.alpha * S[j * kTcOutLd + i]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTcT));
}

int tc_gemm_tiles(int M, int N) { return ((M + kTcT - 1) / kTcT) * ((N + kTcT - 1) / kTcT); }
int tc_gemm_tiles_n(int N) { return (N + kTcT - 1) / kTcT; }
int tc_gemm_tiles_sym(int N) { const int T = (N + kTcT - 1) / kTcT; return T * (T + 1) / 2; }

template <typename TA, typename TB, typename TC, bool TA_, bool TB_>
static void tc_launch(const GemmJob* jobs, int njobs, int ntiles, const TA* A, const TB* B, TC* C,
                      const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s) {
  cudaFuncSetAttribute(tc_gemm_kernel<TA, TB, TC, TA_, TB_>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  // several 64 KB CTAs per SM: ask for the largest shared-memory carveout
  cudaFuncSetAttribute(tc_gemm_kernel<TA, TB, TC, TA_, TB_>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  tc_gemm_kernel<TA, TB, TC, TA_, TB_><<<ntiles, kTcThreads, kTcSmem, s>>>(jobs, njobs, A, B, C, st, require_active,
                                                                            require_phase, err);
}

#define TC_LAUNCH(TA, TB, TC)                                                                                      \
  void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const TA* A, const TB* B, TC* C, bool ta,       \
                      bool tb, const MolState* st, int require_active, int require_phase, int* err,              \
                      cudaStream_t s) {                                                                           \
    if (ntiles <= 0 || njobs <= 0) return;                                                                        \
    if (!ta && !tb) tc_launch<TA, TB, TC, false, false>(jobs, njobs, ntiles, A, B, C, st, require_active, require_phase, err, s); \
    else if (ta && !tb) tc_launch<TA, TB, TC, true, false>(jobs, njobs, ntiles, A, B, C, st, require_active, require_phase, err, s); \
    else if (!ta && tb) tc_launch<TA, TB, TC, false, true>(jobs, njobs, ntiles, A, B, C, st, require_active, require_phase, err, s); \
    else tc_launch<TA, TB, TC, true, true>(jobs, njobs, ntiles, A, B, C, st, require_active, require_phase, err, s); \
  }
TC_LAUNCH(float, float, float)
TC_LAUNCH(double, double, float)
TC_LAUNCH(float, double, double)
TC_LAUNCH(double, float, float)
TC_LAUNCH(double, double, double)
TC_LAUNCH(float, float, double)
#undef TC_LAUNCH

}  // namespace nddo
