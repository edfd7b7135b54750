// Host-visible launchers of the NDDO kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include "nddo_batch.cuh"

namespace nddo {

// one matrix product of a batched GEMM launch: C = alpha op(A) op(B) + beta C
struct GemmJob {
  long long a_off, b_off, c_off;
  int M, N, K;
  int lda, ldb, ldc;
  int mol;
  int tiles_n;
  int tile0;
  double alpha, beta;
  int sym;          // 1: C is symmetric; only tiles on/above the diagonal are computed and mirrored
  int tc_tiles_n;   // the same job in 128 x 128 tiles (tensor-core kernel)
  int tc_tile0;
  int pad;
  double diag;      // added to the diagonal of C (CUDA-core kernel): C = alpha op(A) op(B) + beta C + diag I
};

int gemm_tiles(int M, int N);
int gemm_tiles_sym(int N);
// tensor-core (tcgen05, 3xTF32) batched GEMM, tc_gemm.cu
int tc_gemm_tiles(int M, int N);
int tc_gemm_tiles_n(int N);
int tc_gemm_tiles_sym(int N);
void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const double* B, float* C, bool ta,
                    bool tb, const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s);
void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const float* A, const double* B, double* C, bool ta,
                    bool tb, const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s);
void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const float* B, float* C, bool ta,
                    bool tb, const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s);
void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const float* A, const float* B, float* C, bool ta,
                    bool tb, const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s);
void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const double* B, double* C, bool ta,
                    bool tb, const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s);
void launch_tc_gemm(const GemmJob* jobs, int njobs, int ntiles, const float* A, const float* B, double* C, bool ta,
                    bool tb, const MolState* st, int require_active, int require_phase, int* err, cudaStream_t s);
// block Jacobi (block_jacobi.cu) for bases above the one-CTA Jacobi's limit
constexpr int kSmallJacobiMaxN = 194;
// FP64 lists of at most this many molecules with a basis of at least
// kClusterJacobiMinN use the cluster Jacobi (one 8-CTA cluster per molecule)
constexpr int kClusterJacobiMaxMols = 8;
constexpr int kClusterJacobiMinN = 32;
constexpr int kJacobiBuckets = 9;   // size buckets of a molecule list (edges in Batch::upload_list)
size_t block_jacobi_workspace(int max_n, int nslots, int elem, long long* stride, long long* qstride);
int launch_block_jacobi_f32(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                            const float* G, const double* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                            int* sweeps_out, int* h_pending, cudaStream_t s);
int launch_block_jacobi_f32(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                            const float* G, const float* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                            int* sweeps_out, int* h_pending, cudaStream_t s);
int launch_block_jacobi_f64(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                            const double* G, const double* Cin, double* Cout, double* eps, void* ws, int max_sweeps,
                            int* sweeps_out, int* h_pending, cudaStream_t s);
// FP32 shadows for the tensor-core chain: Cf = Cf2 = float(C), Ff = float(F)
void launch_tc_shadows(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, const double* C,
                       const double* F, float* Cf, float* Cf2, float* Ff, cudaStream_t s);
void launch_copy_matrices(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, const double* src,
                          double* dst, cudaStream_t s);
int gemm_tiles_n(int N);

// pair_fock.cu
void upload_params(const nddo_atom_params* p, cudaStream_t s);
void launch_pair_kernel(const DevAtom* atoms, const DevPair* pairs, long long npairs, const DevMol* mols,
                        const EriTable* eri, const OverlapTable* ovt, double* blocks, double* H,
                        double* ecore_pair, cudaStream_t s);
// pair integrals with the pair list split by type: sp-sp pairs one warp each,
// pairs with a hydrogen one thread each
void launch_pair_kernels_split(const DevAtom* atoms, const DevPair* pairs, const int* heavy_list, long long n_heavy,
                               const int* light_list, long long n_light, const DevMol* mols, const EriTable* eri,
                               const OverlapTable* ovt, double* blocks, double* H, double* ecore_pair,
                               cudaStream_t s);
void launch_hcore_kernel(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list,
                         int nlist, const double* blocks, const double* ecore_pair, const EriTable* eri,
                         const double* epc, double* H, MolState* st, cudaStream_t s);
void launch_fock_kernel(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list,
                        int nlist, int max_atoms, const double* blocks, const double* H, const double* P, double* F,
                        double* Pold, const MolState* st, int mode_override, int copy_old, int require_active,
                        cudaStream_t s);
// empirical dispersion energy requested for the list (AM1-D / PM3-D always add it)
struct VdwParams {
  int on;
  double s6, d;
};
// analytic forces (Hartree/bohr) of molecule m from its converged density P:
// pair gradients into grad (3 per pair), then forces (3 per atom)
void launch_forces(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, int m, long long pair0,
                   long long npairs, int natoms, const EriTable* eri, const OverlapTable* ovt, const double* P,
                   VdwParams vdw, double* grad, double* forces, cudaStream_t s);
void launch_energy_kernel(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list,
                          int nlist, const double* P, const double* F, const double* H, MolState* st,
                          double* charges, VdwParams vdw, cudaStream_t s);
// dipole moment of the listed molecules into MolState::dipole; partial holds
// nlist * kDipChunks * 4 doubles
constexpr int kDipChunks = 64;
void launch_dipole(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list, int nlist,
                   int max_atoms, const double* P, const double* H, double* partial, MolState* st, cudaStream_t s);
// STO-6G Cartesian matrix of molecule m: X = 3 x N x N doubles
void launch_cartesian_matrix(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, int m, int natoms,
                             double* X, cudaStream_t s);

// jacobi.cu
bool jacobi_needs_workspace(int max_n, int elem, bool* a_global, bool* v_global);
void launch_jacobi_f32(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                       int require_active, const float* G, const double* Cin, int use_basis, double* Cout,
                       double* eps, float* Aws, float* Vws, long long ws_stride, int max_sweeps,
                       int* sweeps_out, cudaStream_t s);
void launch_jacobi_f32(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                       int require_active, const float* G, const float* Cin, int use_basis, double* Cout,
                       double* eps, float* Aws, float* Vws, long long ws_stride, int max_sweeps,
                       int* sweeps_out, cudaStream_t s);
// one molecule per cluster of 8 CTAs (FP64); jacobi_cluster_capacity(n) > 0
// when the cluster kernel can run at basis n on this device.  With F given
// (and G null) the kernel forms G = Cin F Cin^T itself.
int jacobi_cluster_capacity(int n);
void launch_jacobi_cluster_f64(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                               int require_active, const double* G, const double* F, const double* Cin, int use_basis,
                               double* Cout, double* eps, int max_sweeps, int* sweeps_out, cudaStream_t s);
void launch_jacobi_f64(const DevMol* mols, const int* mol_list, int nlist, int max_n, const MolState* st,
                       int require_active, const double* G, const double* Cin, int use_basis, double* Cout,
                       double* eps, double* Aws, double* Vws, long long ws_stride, int max_sweeps,
                       int* sweeps_out, cudaStream_t s);

// tridiag.cu: FP64 Householder tridiagonalisation + bisection + inverse
// iteration + back-transformation.  td holds d, e, tau of every molecule at
// vec0, vec0 + vstride, vec0 + 2 vstride; W (N x N arena) the reflectors.
int hh_smem_max_n();     // largest basis whose packed matrix fits one CTA's shared memory
int hh_back_max_n();     // largest basis the back-transformation kernel serves
void hh_prepare();       // one-time kernel attributes and device limits (before any stream capture)
// molecules above max_n_served are skipped (the whole-GPU path serves them)
void launch_hh_tridiag(const DevMol* mols, const int* list, int nlist, int max_n, const MolState* st,
                       int require_active, const double* F, double* W, double* td, long long vstride, double* Aws,
                       int max_n_served, cudaStream_t s);
// eigenvalues (bisection + Laguerre) and inverse-iteration vectors of T into
// eps and the columns of Z (N x k per molecule)
void launch_tri_vectors(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                        int require_active, int final_pass, const double* td, long long vstride, double* eps,
                        double* Z, double* const* S4, cudaStream_t s);
// eigenpairs of the SCF pass (final_pass = 0: the smaller of the occupied and
// virtual sets) or of every index (final_pass = 1) into eps and rows of C;
// Z and S4[0..3] are N x N scratch arenas
// mixed = 1: molecules in the FP32 phase get FP32 vectors in the rows of C32
// (the FP64 phase and the final pass write C)
void launch_hh_vectors(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                       int require_active, int final_pass, int mixed, const double* W, const double* td,
                       long long vstride, double* eps, double* Z, double* const* S4, double* C, float* C32,
                       cudaStream_t s);

// tridiag_grid.cu: the same eigensolver for large molecules on many SMs each.
// A cooperative launch of nctas CTAs (one per SM) serves nlist <= nctas
// molecules of list; map3 holds per CTA (entry of list, CTA index within the
// molecule's sub-grid, sub-grid size), from hh_grid_assign; bars = 4 words of
// barrier state per entry.  scratch = another N x N scratch arena.  A
// sub-grid barrier that waits longer than about two seconds marks the
// molecule failed.
int hh_grid_max_n();     // largest basis the whole-GPU path serves
// Bases from this size on share the whole-GPU kernels when few of them are in
// a list (Batch::build_jobs).  Above the serving middle lane's largest basis
// (400), so that only one serving lane issues cooperative launches.
constexpr int kGridShareMinN = 401;
int hh_grid_ctas();      // CTAs of one cooperative launch (the SM count)
// CTA split of G CTAs over count molecules of bases n[] (N^3 shares, at least
// one each): writes 3 ints per CTA into map3, returns the CTAs used (0 if
// count > G)
int hh_grid_assign(const int* n, int count, int G, int* map3);
void launch_hh_grid_tridiag(const DevMol* mols, const int* list, const int* map3, int nctas, int nlist, MolState* st,
                            int require_active, const double* F, double* W, double* td, long long vstride,
                            double* Aws, double* scratch, unsigned* bars, cudaStream_t s);
void launch_hh_grid_orth(const DevMol* mols, const int* list, const int* map3, int nctas, int nlist, int max_k,
                         MolState* st, int require_active, int final_pass, const double* td, long long vstride,
                         double* eps, double* Z, double* scratch, unsigned* bars, cudaStream_t s);
// X = Q Z for every molecule of list (grid: molecules x column groups)
void launch_hh_grid_back(const DevMol* mols, const int* list, int nlist, int max_n, int max_k, const MolState* st,
                         int require_active, int final_pass, int mixed, const double* W, const double* td,
                         long long vstride, const double* Z, double* C, float* C32, cudaStream_t s);

// scf_kernels.cu
void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const double* B, double* C,
                 bool ta, bool tb, double acc_tag, const MolState* st, int require_active, int require_phase,
                 cudaStream_t s);
void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const double* B, double* C,
                 bool ta, bool tb, float acc_tag, const MolState* st, int require_active, int require_phase,
                 cudaStream_t s);
void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const double* B, float* C,
                 bool ta, bool tb, float acc_tag, const MolState* st, int require_active, int require_phase,
                 cudaStream_t s);
void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const float* A, const double* B, float* C,
                 bool ta, bool tb, float acc_tag, const MolState* st, int require_active, int require_phase,
                 cudaStream_t s);
void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const double* A, const float* B, float* C,
                 bool ta, bool tb, float acc_tag, const MolState* st, int require_active, int require_phase,
                 cudaStream_t s);
void launch_gemm(const GemmJob* jobs, int njobs, int ntiles, const float* A, const double* B, double* C,
                 bool ta, bool tb, float acc_tag, const MolState* st, int require_active, int require_phase,
                 cudaStream_t s);
// DIIS in three launches (partial sums, per-molecule solve, apply); scratch
// holds diis_scratch_bytes(nlist) bytes
size_t diis_scratch_bytes(int slots);
void launch_diis(const DevMol* mols, const int* mol_list, int nlist, MolState* st, const ScfParamsDev& prm,
                 double* P, const double* Pold, double* hist_dens, double* hist_err, long long hist_stride,
                 TraceEntry* trace, int trace_len, void* scratch, cudaStream_t s);

void launch_newton_scale(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, int require_phase,
                         double* K, const double* O, const double* eps, cudaStream_t s);
void launch_neumann(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, int require_phase,
                    double* M, cudaStream_t s);
void launch_copy_occ_rows(const DevMol* mols, const int* mol_list, int nlist, const MolState* st, int require_phase,
                          const double* src, double* dst, cudaStream_t s);

}  // namespace nddo
