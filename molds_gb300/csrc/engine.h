// Host engine: owns one device, one stream and any number of device-resident
// molecule batches, and drives the batched SCF state machine.
#pragma once
#include <cuda_runtime.h>
#include <map>
#include <memory>
#include <string>
#include <vector>
#include "kernels.h"

namespace nddo {

struct MoleculeInput {
  int theory = NDDO_PM3;
  std::vector<int> Z;
  std::vector<double> xyz;   // bohr, 3 per atom
  // environmental point charges (MolDS EPC block): x, y, z in bohr and the
  // charge, 4 per point charge
  std::vector<double> epc;
};

struct ScfSettings {
  int max_iter = 100;
  double rms_density = 1e-8;
  double damping_thresh = 1.0;
  double damping_weight = 0.8;
  int diis_num_error_vect = 5;
  double diis_start_error = 1e-2;
  double diis_end_error = 1e-8;
  int precision = 0;            // 0 FP64 throughout, 1 mixed (FP32 eigen phase + FP64 refinement)
  double switch_error = 1e-4;   // mixed: FP64 phase once the DIIS error is below this
  int max_sweeps = 30;
  int keep_trace = 1;
  int tensor_cores = 1;         // mixed: FP32-phase GEMMs on tcgen05 (3xTF32) instead of CUDA cores
  int dipole = 1;               // dipole moment after convergence (MolDS DoSCF always computes it)
  int vdw = 0;                  // empirical dispersion energy (SCF block "vdW yes"; always on for AM1-D / PM3-D)
  double vdw_s6 = 1.40, vdw_d = 23.0;
  int eigensolver = 0;          // FP64 eigensolves: 0 auto (Householder), 1 Jacobi, 2 Householder
  int graphs = 1;               // replay each SCF iteration from a captured CUDA graph (Householder path,
                                // profiling off)
};

// settings that change the launches of an SCF iteration (a captured graph is
// replayed only while they are unchanged)
bool same_launches(const ScfSettings& a, const ScfSettings& b);

// kernel classes timed by the optional per-launch CUDA-event profiler
enum KernelClass {
  kKPair = 0, kKHcore, kKFock, kKOrtho, kKTransform, kKJacobi, kKDensity, kKRefine, kKDiis, kKEnergy, kKDipole,
  kKTridiag, kKEigvec, kKNumClasses
};
const char* kernel_class_name(int k);

struct MolResult {
  int status = 0;               // MolStatus
  int iterations = 0;
  double energy = 0, core_repulsion = 0, heat_of_formation = 0, final_rms = 0, final_diis_error = 0;
  double dipole[9] = {};        // total, electronic, core (x, y, z) [a.u.] when ScfSettings::dipole
  double vdw_energy = 0;        // empirical dispersion energy, included in energy
  double core_epc = 0;          // Coulomb energy of the cores and the point charges, included in energy
};

class Engine;

// Arena sizes of a molecule pool (elements of each arena).
struct BatchCapacity {
  int slots = 0;               // molecules resident at once
  long long atoms = 0, pairs = 0, blocks = 0, mat = 0, vec = 0;
  long long epcs = 0;          // environmental point charges
  int max_n = 0;               // largest basis admitted
  int ws_slots = 0;            // molecules per Jacobi launch that need a global-memory workspace
};

// First-fit allocator of element ranges inside one arena (coalescing frees).
class ArenaAlloc {
 public:
  void reset(long long capacity);
  long long alloc(long long n);          // offset, or -1 when no free range is large enough
  void release(long long off, long long n);
  long long free_total() const;
 private:
  std::map<long long, long long> free_;  // offset -> length
};

// A set of molecules resident on the device with every buffer the SCF needs.
// Two modes: a fixed batch (every molecule given at construction), or a pool
// with fixed arena capacities into which molecules are admitted and released
// one at a time (the serving loop).
class Batch {
 public:
  Batch(Engine* eng, const std::vector<MoleculeInput>& mols, int diis_m, cudaStream_t stream = nullptr);
  Batch(Engine* eng, const BatchCapacity& cap, int diis_m, cudaStream_t stream);
  ~Batch();
  Batch(const Batch&) = delete;
  Batch& operator=(const Batch&) = delete;

  int size() const { return (int)h_mols.size(); }
  int max_n() const { return cap_.max_n; }
  long long epc_capacity() const { return cap_.epcs; }
  cudaStream_t stream() const { return stream_; }

  // pool mode: place a molecule (slot index, or -1 when an arena or the slot
  // table is full) and give its space back
  int admit(const MoleculeInput& in);
  void release(int slot);
  // device bytes one element of the per-molecule N x N arena costs (all buffers)
  static size_t bytes_per_mat_element(int diis_m);
  // pair integrals, H and core-core energy of the listed molecules
  void integrals(const std::vector<int>& which);
  // count_active without a host wait: the count and per-slot active flags land
  // in pinned host memory, and `done` is recorded after the copies
  void count_active_async(const std::vector<int>& which, int* h_count, char* h_active, cudaEvent_t done);
  // asynchronous copies into pinned host memory (complete at the next stream sync)
  void copy_states_async(MolState* host);
  void copy_charges_async(int m, double* host);
  int nao(int m) const { return h_mols[m].nao; }
  int natoms(int m) const { return h_mols[m].natoms; }
  int nocc(int m) const { return h_mols[m].nocc; }
  size_t device_bytes() const { return bytes_; }

  // One-time work: pair integrals, H, core-core energy.
  void integrals();
  // Full SCF for every molecule; requires_guess as in MolDS DoSCF(requiresGuess).
  void scf(const ScfSettings& s, bool requires_guess);
  // Initialise the SCF state of the listed molecules (serving: admission).
  void begin(const ScfSettings& s, const std::vector<int>& which, bool requires_guess);
  // One SCF iteration over the listed (active) molecules.
  void iterate(const ScfSettings& s, const std::vector<int>& which);
  // Energies / charges of the listed molecules after convergence.
  void finish(const ScfSettings& s, const std::vector<int>& which);
  // Number of still-active molecules among `which` (synchronises).
  int count_active(const std::vector<int>& which);
  // One SCF iteration, replayed from a captured CUDA graph when the settings
  // allow it (iterate() otherwise)
  void iterate_graph(const ScfSettings& s, const std::vector<int>& which);
  long long graph_launches() const { return graph_launches_; }

  // results (synchronise and copy out)
  void results(std::vector<MolResult>* out);
  void copy_matrix(int which_matrix, int m, double* host) const;   // 0 H, 1 F, 2 P, 3 C
  void copy_eps(int m, double* host) const;
  void copy_charges(int m, double* host) const;
  // analytic forces (Hartree/bohr, natoms x 3) of molecule m's converged SCF
  void forces(const ScfSettings& s, int m, double* host);
  void copy_blocks(int m, double* host, size_t* count) const;
  void copy_trace(int m, std::vector<TraceEntry>* out) const;
  // STO-6G Cartesian matrix <mu| r_k |nu> of molecule m, 3 x N x N doubles (synchronises)
  void cartesian_matrix(int m, double* host) const;
  void set_density(int m, const double* host);

  const std::vector<DevMol>& mol_table() const { return h_mols; }
  void set_coordinates(const double* xyz);          // bohr, 3 per atom, batch order
  // new coordinates of one molecule (pool mode: the slot's atoms only); the
  // density, eigenvectors and DIIS arrays are kept, so a following
  // scf(..., requires_guess = false) starts from the previous density
  void set_molecule_coordinates(int m, const double* xyz);
  // per-kernel-class timing with CUDA events on the launching stream
  // Enabling creates the event pool up front (kProfEvents), so the timed
  // region that follows does not pay for cudaEventCreate.
  void set_profiling(bool on);
  void profile_collect(double* ms, long long* launches, double* work);  // accumulates since last reset
  void profile_reset();
  long long launches() const { return launches_; }
  long long jacobi_sweeps() const;   // Jacobi sweeps summed over molecules since the last begin()
  double* dev_H() const { return d_H; }
  double* dev_P() const { return d_P; }

 private:
  void allocate(const BatchCapacity& cap);
  int list_max_atoms() const;   // largest molecule (atoms) of the current list
  void build_jobs(const std::vector<int>& which);
  void upload_list(const std::vector<int>& which);
  void eigen_step(const ScfSettings& s);
  void density_step(const ScfSettings& s);
  // FP64 Householder path (tridiag.cu): used for this list and these settings
  bool householder(const ScfSettings& s) const;
  // eigenpairs of the current list from each molecule's last
  // tridiagonalisation: final_pass = 0 the density's set, 1 every index (MO
  // energies and vectors)
  void hh_vectors(const ScfSettings& s, int final_pass, int require_active);

  Engine* eng_;
  cudaStream_t stream_;
  int diis_m_;
  bool pool_ = false;
  BatchCapacity cap_;
  ArenaAlloc a_atoms_, a_pairs_, a_blocks_, a_mat_, a_vec_, a_epc_;
  std::vector<int> free_slots_;
  std::vector<long long> slot_blocks_;   // block-arena length of each occupied slot
  size_t bytes_ = 0;
  long long mat_total_ = 0, vec_total_ = 0;
  int max_n_ = 0, max_iter_alloc_ = 0;

  std::vector<DevAtom> h_atoms;
  std::vector<double> h_epc;      // point charges, 4 doubles each
  std::vector<DevPair> h_pairs;
  std::vector<DevMol> h_mols;
  long long blk_total_ = 0;

  DevAtom* d_atoms = nullptr;
  double* d_epc = nullptr;
  DevPair* d_pairs = nullptr;
  DevMol* d_mols = nullptr;
  int* d_list = nullptr;
  double* d_blocks = nullptr;
  double* d_ecore_pair = nullptr;
  int* d_heavy_pairs = nullptr;   // indices of sp-sp pairs
  int* d_light_pairs = nullptr;   // indices of pairs with a hydrogen (X-H first, then H-H)
  long long n_heavy_ = 0, n_light_ = 0;
  double *d_H = nullptr, *d_F = nullptr, *d_P = nullptr, *d_Pold = nullptr, *d_C = nullptr, *d_eps = nullptr;
  double *d_hist_dens = nullptr, *d_hist_err = nullptr;
  float *d_G32 = nullptr, *d_T32 = nullptr;
  float *d_Cf = nullptr, *d_Cnf = nullptr, *d_Ff = nullptr;   // FP32 shadows of the tensor-core chain
  double *d_G64 = nullptr, *d_T64 = nullptr;
  double* d_S[6] = {};
  double* d_td = nullptr;                // tridiagonal d, e, tau (3 x vec arena)
  int list_max_n_ = 0, hh_max_k_ = 0;    // largest basis and density-set size of the current list
  // Householder path: molecules up to hh_back_max_n() on the per-molecule
  // kernels (hh_small_, with their largest basis and density-set size), the
  // larger ones one at a time on the whole-GPU kernels (hh_large_)
  std::vector<int> hh_small_, hh_large_;
  int* d_hh_small_ = nullptr;
  int* d_hh_large_ = nullptr;
  int hh_small_max_n_ = 0, hh_small_max_k_ = 0;
  int hh_large_max_n_ = 0, hh_large_max_k_ = 0;
  std::vector<int> bucket_hh_max_n_;     // per size bucket: largest basis on the per-molecule kernels
  int hh_served_max_n_ = 0;              // the per-molecule kernels serve bases up to this; larger: whole-GPU kernels
  // whole-GPU path: the large molecules in chunks of at most one per SM, each
  // chunk one cooperative launch whose CTAs are split over its molecules
  struct GridChunk { int first, count, nctas, map_off, max_k; };
  std::vector<GridChunk> grid_chunks_;
  int grid_ctas_ = 0;                    // CTAs of a cooperative launch (the SM count)
  int* d_gridmap_ = nullptr;             // per CTA: list entry, CTA in the sub-grid, sub-grid size
  int* h_gridmap_ = nullptr;             // pinned staging of d_gridmap_
  unsigned* d_gridbar_ = nullptr;        // barrier words, 4 per molecule of a chunk
  double* d_pgrad_ = nullptr;            // pair gradients of forces() (grown on demand)
  double* d_forces_ = nullptr;
  long long pgrad_cap_ = 0, forces_cap_ = 0;
  float *d_jA32 = nullptr, *d_jV32 = nullptr;
  void* d_bj_ws = nullptr;               // block-Jacobi workspace (bases above kSmallJacobiMaxN)
  int* h_bj_pending = nullptr;           // pinned: molecules still rotating after a block-Jacobi sweep
  double *d_jA64 = nullptr, *d_jV64 = nullptr;
  long long jws_stride_ = 0;
  MolState* d_state = nullptr;
  TraceEntry* d_trace = nullptr;
  double* d_charges = nullptr;
  int* d_sweeps = nullptr;
  int* d_count = nullptr;
  int* d_tc_err = nullptr;               // set by a tensor-core GEMM whose MMA wait ran out
  void* d_diis_ws = nullptr;             // DIIS partial sums and decisions (diis_scratch_bytes)
  double* d_dip_ws = nullptr;            // dipole partial sums (slots x kDipChunks x 4)
  char* d_active = nullptr;

  // current molecule list and its GEMM job tables
  std::vector<int> cur_list_;
  std::vector<std::vector<int>> buckets_;      // jacobi size buckets (indices into cur_list_)
  std::vector<int*> d_bucket_lists_;     // persistent, one per size bucket, `slots` entries each
  std::vector<int*> bucket_dev_;         // device list of each non-empty bucket of the current list
  void run_jacobi(bool fp32, const ScfSettings& s, const double* Cin, const float* Cin32 = nullptr,
                  const double* F = nullptr);
  bool cluster_jacobi(int bucket) const;   // FP64 bucket served by the cluster Jacobi
  std::vector<int> bucket_max_n_;
  struct JobSet { GemmJob* d = nullptr; int n = 0; int tiles = 0; int tc_tiles = 0; int cap = 0; };
  GemmJob* h_jobs_ = nullptr;             // pinned staging of the job tables
  int* h_lists_ = nullptr;                // pinned staging of the molecule / bucket lists
  int job_cap_ = 0;
  JobSet j_trans1_, j_trans2_, j_dens_, j_w_, j_kt_, j_yt_, j_m_, j_d2_, j_z_, j_p_, j_ns1_, j_ns2_, j_ov_, j_hh_;
  void free_jobs();
  void make_jobset(JobSet* js, const std::vector<GemmJob>& jobs);

  // captured SCF iteration
  cudaGraphExec_t graph_exec_ = nullptr;
  ScfSettings graph_settings_;
  long long graph_layout_ = -1;           // layout_version_ the graph was captured for
  long long layout_version_ = 0;          // bumped whenever the job tables and size buckets are rebuilt
  long long graph_kernels_ = 0;           // kernels in one replay
  long long graph_launches_ = 0;          // replays so far
  // pipelined convergence checks: pinned counts and their events (two blocks in flight)
  int* h_block_count_ = nullptr;
  char* h_block_active_ = nullptr;
  cudaEvent_t block_ev_[2] = {nullptr, nullptr};

  // profiler
  long long launches_ = 0;   // kernels launched by this batch so far
  bool prof_on_ = false;
  struct Rec { cudaEvent_t a, b; int cls; double work; };
  std::vector<cudaEvent_t> ev_pool_;
  size_t ev_used_ = 0;
  std::vector<Rec> recs_;
  double prof_ms_[kKNumClasses] = {};
  long long prof_launches_[kKNumClasses] = {};
  double prof_work_[kKNumClasses] = {};
  cudaEvent_t next_event();
  int prof_begin(int cls, double work);
  void prof_end(int handle);
  // algorithmic work of the molecules still active (flop counts, see engine.cu)
  double active_work_estimate(int cls) const;
  std::vector<char> active_host_;
};

// A fixed batch split into groups of molecules, each a Batch with its own
// stream, run concurrently by one host thread per group: the latency-bound
// one-CTA Jacobi of one group overlaps the FP64-bound refinement and the
// memory-bound Fock build of the others, and the tail wave of a group's
// launches no longer leaves SMs idle.  Molecule results do not depend on the
// grouping (every kernel works per molecule).
class GroupedBatch {
 public:
  GroupedBatch(Engine* eng, const std::vector<MoleculeInput>& mols, int diis_m, int groups);
  ~GroupedBatch();
  static int default_groups(int n_mol);
  int size() const { return n_; }
  int groups() const { return (int)g_.size(); }
  // integrals + SCF + energies of every molecule; requires_guess = false
  // starts every molecule from its previous density (DoSCF(false))
  void run(const ScfSettings& s, bool requires_guess = true);
  void results(std::vector<MolResult>* out);
  void copy_charges(int m, double* host) const;
  void copy_matrix(int which_matrix, int m, double* host) const;
  void cartesian_matrix(int m, double* host) const;
  void forces(const ScfSettings& s, int m, double* host);   // analytic forces of molecule m (natoms x 3)
  void set_coordinates(const double* xyz);
  size_t device_bytes() const;
  long long launches() const;
  long long graph_launches() const;
  long long jacobi_sweeps() const;
  void set_profiling(bool on);
  void profile_reset();
  void profile_collect(double* ms, long long* launches, double* work);   // summed over the groups' streams
  void timer(int op, double* ms);                 // 0 start, 1 stop, 2 elapsed wall time over all streams

 private:
  const Batch& locate(int m, int* local) const;
  int n_ = 0;
  std::vector<std::unique_ptr<Batch>> g_;
  std::vector<cudaStream_t> streams_;
  std::vector<int> first_mol_, first_atom_;
  std::vector<cudaEvent_t> t0_, t1_;
  int device_ = 0;
};

class Engine {
 public:
  explicit Engine(int device);
  ~Engine();
  cudaStream_t stream() const { return stream_; }
  int device() const { return device_; }
  const EriTable* eri() const { return d_eri_; }
  const OverlapTable* ovt() const { return d_ovt_; }

 private:
  int device_;
  cudaStream_t stream_ = nullptr;
  EriTable* d_eri_ = nullptr;
  OverlapTable* d_ovt_ = nullptr;
};

// throws std::runtime_error with the CUDA error text
void cuda_check(cudaError_t e, const char* what);

// basis functions of a molecule (unknown elements count zero; layout rejects them)
int molecule_nao(const MoleculeInput& in);

}  // namespace nddo
