/*
 * C ABI of the GB300 NDDO (MNDO / AM1 / PM3) closed-shell SCF.
 *
 * Plain C types only: a MolDS build (or any FFI) binds these entry points in
 * place of its CPU Fock build and LAPACK eigensolver on the SCF path.  Each
 * declaration names the MolDS interface it stands in for (paths relative to
 * the MolDS source tree).
 *
 * Conventions
 *   - Coordinates are in bohr (MolDS converts Angstrom input at parse time,
 *     src/base/InputParser.cpp:545-547).
 *   - Orbital order per atom is s, py, pz, px (src/base/Enums.h:98-108).
 *   - Return codes: 0 = OK, 1 = SCF not converged, negative = error; the text
 *     of the last error is returned by nddo_last_error().
 *   - Buffers are caller-owned; inputs are copied in, results copied out.
 *   - One context per host thread.
 */
#ifndef MOLDS_GB300_NDDO_GPU_H
#define MOLDS_GB300_NDDO_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nddo_ctx nddo_ctx;

/* AM1-D / PM3-D: MolDS's dispersion-corrected sets (THEORY am1-d / pm3-d;
 * src/am1/Am1D.cpp, src/pm3/Pm3D.cpp) and PDDG/PM3 (THEORY pm3/pddg;
 * src/pm3/Pm3Pddg.cpp).  AM1-D and PDDG/PM3: H, C, N, O and S; PM3-D: H, C,
 * N, O, F, S, Cl. */
enum {
  NDDO_THEORY_MNDO = 0, NDDO_THEORY_AM1 = 1, NDDO_THEORY_PM3 = 2, NDDO_THEORY_AM1D = 3, NDDO_THEORY_PM3D = 4,
  NDDO_THEORY_PM3PDDG = 5
};
enum { NDDO_PRECISION_FP64 = 0, NDDO_PRECISION_MIXED = 1 };
/* FP64 eigensolver of the SCF (Lapack::Dsyevd's stand-in): AUTO and
 * HOUSEHOLDER = Householder tridiagonalisation + bisection + inverse
 * iteration; JACOBI = the warm-started cyclic Jacobi. */
enum { NDDO_EIGEN_AUTO = 0, NDDO_EIGEN_JACOBI = 1, NDDO_EIGEN_HOUSEHOLDER = 2 };
enum {
  NDDO_OK = 0,
  NDDO_NOT_CONVERGED = 1,
  NDDO_ERR_ARGUMENT = -1,
  NDDO_ERR_CUDA = -2,
  NDDO_ERR_BUDGET = -3,
  NDDO_ERR_STATE = -4
};
enum { NDDO_STATUS_ACTIVE = 0, NDDO_STATUS_CONVERGED = 1, NDDO_STATUS_NOT_CONVERGED = 2, NDDO_STATUS_FAILED = 3 };

/* SCF block of the MolDS input (src/base/InputParser.cpp:646-734) plus the
 * precision choice of this implementation. */
typedef struct {
  int max_iter;                /* max_iter                                  */
  double rms_density;          /* rms_density                               */
  double damping_thresh;       /* damping_thresh                            */
  double damping_weight;       /* damping_weight                            */
  int diis_num_error_vect;     /* diis_num_error_vect (0..8)                */
  double diis_start_error;     /* diis_start_error                          */
  double diis_end_error;       /* diis_end_error                            */
  int precision;               /* NDDO_PRECISION_FP64 or NDDO_PRECISION_MIXED */
  double fp64_switch_error;    /* mixed: FP64 phase once the DIIS error is below this */
  int tensor_cores;            /* mixed: FP32-phase GEMMs on the tensor cores (1, default) or CUDA cores (0) */
  int dipole;                  /* dipole moment after convergence (1, default, as DoSCF) or skipped (0) */
  int vdw;                     /* vdW yes/no: empirical dispersion energy (always on for AM1-D / PM3-D) */
  double vdw_s6;               /* vdW_s6 (default 1.40; AM1-D / PM3-D use 1.40)  */
  double vdw_d;                /* vdW_d  (default 23;  AM1-D / PM3-D use 23)    */
  int eigensolver;             /* NDDO_EIGEN_* for FP64 eigensolves (default AUTO) */
} nddo_scf_params;

typedef struct {
  int status;                  /* NDDO_STATUS_*                              */
  int iterations;              /* SCF iterations run (MolDS prints 0..iterations-1) */
  double energy;               /* electronic energy incl. core repulsion [Eh] */
  double core_repulsion;       /* [Eh]                                       */
  double heat_of_formation;    /* [Eh]; meaningful for MNDO only             */
  double final_rms;            /* last RMS density change                    */
  double final_diis_error;     /* last DIIS error (max |P_new - P_old|)      */
  double dipole[9];            /* total, electronic, core dipole (x, y, z) [a.u.]; 0 with dipole = 0
                                  (Cndo2::OutputSCFDipole, src/cndo/Cndo2.cpp:1126-1185) */
  double vdw_energy;           /* empirical dispersion energy [Eh], included in energy (0 when off) */
  double core_epc_coulomb;     /* sum over cores and environmental point charges of Z_A q / R [Eh],
                                  included in energy (0 without point charges; Cndo2.cpp:418-426) */
} nddo_scf_result;

/* Defaults of src/base/Parameters.cpp:133-139 (precision = FP64). */
void nddo_default_params(nddo_scf_params* p);

/* Engine on one GPU.  hbm_budget_bytes = 0 means no limit; MolDS's analogue is
 * the MEMORY limit_heap check (src/base/MallocerFreer.cpp:62-72). */
int nddo_create(int device, size_t hbm_budget_bytes, nddo_ctx** out);
void nddo_destroy(nddo_ctx* ctx);
const char* nddo_last_error(const nddo_ctx* ctx);

/* ElectronicStructure::SetMolecule (src/base/ElectronicStructure.h:27,
 * Mndo::SetMolecule src/mndo/Mndo.cpp:110-138).  Validates the elements and
 * the electron count (odd -> error, src/cndo/Cndo2.cpp:351-357) and computes
 * the one-time pair integrals, overlap and core-core terms. */
int nddo_set_molecule(nddo_ctx* ctx, int theory, int n_atoms, const int* atomic_numbers, const double* xyz_bohr);
/* nddo_set_molecule with environmental point charges: MolDS's EPC block
 * (InputParser::ParseEpcsConfiguration, src/base/InputParser.cpp:626-644,
 * Molecule::AddEpc) as n_epc rows of x, y, z [bohr] and charge.  Each charge
 * q adds -q (mu nu|s s) to the one-centre blocks of every non-guess Fock
 * matrix (Mndo::GetFockDiagElement / GetFockOffDiagElement,
 * src/mndo/Mndo.cpp:474-484, 546-556; the atom-EPC integrals with rho = 0,
 * :6602-6613) and sum Z_A q / R to the energy (Mndo.cpp:329-331).
 * n_epc = 0 is nddo_set_molecule.  nddo_set_coordinates moves the atoms and
 * keeps the point charges in place. */
int nddo_set_molecule_epc(nddo_ctx* ctx, int theory, int n_atoms, const int* atomic_numbers, const double* xyz_bohr,
                          int n_epc, const double* epc_xyzq);
/* New coordinates for the molecule already set (same atoms, bohr), as the MD /
 * MC / optimiser drivers move MolDS's Molecule in place before calling
 * DoSCF(false) (src/md/MD.cpp:108): the one-time integrals are recomputed and
 * the density of the last SCF is kept, so nddo_scf(..., requires_guess = 0)
 * starts from it. */
int nddo_set_coordinates(nddo_ctx* ctx, const double* xyz_bohr);
int nddo_num_aos(const nddo_ctx* ctx);
int nddo_num_atoms(const nddo_ctx* ctx);

/* ElectronicStructure::DoSCF(bool requiresGuess) (src/base/ElectronicStructure.h:28,
 * Cndo2::DoSCF src/cndo/Cndo2.cpp:585-729).  Returns NDDO_NOT_CONVERGED when
 * max_iter is reached (MolDS throws "SCF did not met convergence criterion"). */
int nddo_scf(nddo_ctx* ctx, const nddo_scf_params* params, int requires_guess, nddo_scf_result* result);

/* Getters after nddo_scf (src/base/ElectronicStructure.h:30-39). */
int nddo_get_energies_mo(nddo_ctx* ctx, double* out_n);          /* GetEnergiesMO: N ascending      */
int nddo_get_fock_matrix(nddo_ctx* ctx, double* out_nn);         /* GetFockMatrix: eigenvector rows */
int nddo_get_density(nddo_ctx* ctx, double* out_nn);             /* orbital electron population P   */
int nddo_get_mulliken(nddo_ctx* ctx, double* out_natoms);        /* Mulliken charges (Cndo2.cpp:1187-1199) */
int nddo_get_core_hamiltonian(nddo_ctx* ctx, double* out_nn);    /* H = F(P = 0) (Cndo2.cpp:1359-1367) */
/* Total, electronic and core dipole moments (x, y, z each) [a.u.] of the last
 * SCF: origin at the centre of core mass, electronic part -sum P X + c sum P S
 * (Cndo2::CalcElectronicDipoleMomentGroundState / CalcCoreDipoleMoment,
 * src/cndo/Cndo2.cpp:1871-1944). */
int nddo_get_dipole(nddo_ctx* ctx, double* out9);
/* STO-6G Cartesian matrix <mu| r_k |nu> [bohr], 3 x N x N doubles (k = x, y, z):
 * MolDS's cartesianMatrix (Cndo2::CalcCartesianMatrixByGTOExpansion,
 * src/cndo/Cndo2.cpp:1946-2130).  Needs only a molecule. */
int nddo_get_cartesian_matrix(nddo_ctx* ctx, double* out_3nn);
/* The SCF section of MolDS's output for the last nddo_scf, as Cndo2::DoSCF
 * prints it between its banners (src/cndo/Cndo2.cpp:585-729): the iteration
 * log (:1505-1510), then OutputSCFResults (:1299-1303: MO energies, energies,
 * dipoles, Mulliken charges; MNDO adds the heat of formation,
 * src/mndo/Mndo.cpp:412-420) and the elapsed time; a non-converged SCF ends
 * after the iteration log, where MolDS throws.  Writes at most cap - 1 chars
 * and a terminating NUL into out (may be NULL); *needed = full length + 1. */
int nddo_scf_output_text(nddo_ctx* ctx, char* out, size_t cap, size_t* needed);
/* The same text from explicit values (no GPU needed): per iteration rms,
 * diis_error, diis_on, damp_on (iterations entries); epc != 0 adds the
 * point-charge lines with core_epc (Cndo2.cpp:1090-1115); dipole = 9 doubles
 * (total, electronic, core; x y z) or NULL for no dipole block;
 * sum_pairs = n_sum_pairs (first, last) atom index pairs. */
int nddo_format_scf_text(int theory, int n_atoms, const int* Z, int n_ao, int n_occ, int iterations,
                         const double* rms, const double* diis_error, const int* diis_on, const int* damp_on,
                         int converged, const double* eps, double energy, double core_repulsion, int vdw,
                         double vdw_energy, int epc, double core_epc, const double* dipole, const double* charges,
                         double heat_of_formation, int n_sum_pairs, const int* sum_pairs, double seconds, char* out,
                         size_t cap, size_t* needed);
/* Forces on the atoms (-dE/dR, Hartree/bohr, n_atoms x 3 row-major) of the
 * last converged SCF, ground state: Mndo::CalcForce
 * (src/mndo/Mndo.cpp:2711-2986) as read by ElectronicStructure::GetForce.
 * Analytic: the pair terms of the energy (two-centre integrals, electron-core
 * attractions, resonance, core-core, dispersion) differentiated exactly with
 * the converged density held fixed.  As in the reference, environmental
 * point charges enter only through that density: Mndo::CalcForce has no
 * atom-EPC term. */
int nddo_get_forces(nddo_ctx* ctx, double* out_natoms_x3);
/* The SCF option sum_charges (InputParser.cpp:694-700,
 * Parameters::AddSumChargesIndexPairsSCF): n_pairs (first, last) atom index
 * pairs whose Mulliken charges the output text sums (Cndo2.cpp:1203-1220). */
int nddo_set_sum_charges(nddo_ctx* ctx, int n_pairs, const int* pairs);
/* Per-iteration log of Cndo2::SatisfyConvergenceCriterion (Cndo2.cpp:1505-1510).
 * Returns the number of entries written (>= 0; compare it with max_entries,
 * not with the status codes) or a negative NDDO_ERR_* code. */
int nddo_get_trace(nddo_ctx* ctx, int max_entries, double* rms, double* diis_error, int* diis_on, int* damp_on);
/* Packed space-frame (mu nu|la si) blocks of all atom pairs a < b, row-major
 * pair order; 10x10 (sp-sp), 10x1, 1x10 or 1x1 doubles per pair.  With
 * out == NULL only *count is set.  Replaces the A x A x 4^4 twoElecsTwoAtomCores
 * store of Mndo::CalcTwoElecsTwoAtomCores (src/mndo/Mndo.cpp:3703-3820). */
int nddo_get_pair_blocks(nddo_ctx* ctx, double* out, size_t* count);

/* Many independent molecules in one batched, device-resident SCF: the
 * repeated-DoSCF callers (RPMD beads, src/rpmd/RPMD.cpp:78-84; MD/MC/optimiser
 * steps) and throughput runs.  Molecule i has n_atoms[i] atoms; Z and xyz are
 * concatenated over molecules.  results has n_mol entries, charges has
 * sum(n_atoms) entries (may be NULL).  The context keeps the device arrays of
 * the last call: a call with the same molecules (theory, DIIS window, atom
 * counts, elements) uploads only the new coordinates. */
int nddo_batch_scf(nddo_ctx* ctx, int theory, int n_mol, const int* n_atoms, const int* atomic_numbers,
                   const double* xyz_bohr, const nddo_scf_params* params, nddo_scf_result* results,
                   double* charges);

/* A device-resident batch: the molecules' geometry, integrals, densities and
 * DIIS history stay on the GPU between calls, so repeated SCFs of the same
 * molecules (MD / MC / optimiser steps that call DoSCF again, src/md/MD.cpp:108,
 * src/mc/MC.cpp:124) pay no allocation and no re-upload. */
typedef struct nddo_batch nddo_batch;
int nddo_batch_create(nddo_ctx* ctx, int theory, int n_mol, const int* n_atoms, const int* atomic_numbers,
                      const double* xyz_bohr, int diis_num_error_vect, nddo_batch** out);
/* nddo_batch_create with environmental point charges per molecule (as
 * nddo_set_molecule_epc): n_epc[i] charges for molecule i (n_epc may be
 * NULL: none), their rows of x, y, z [bohr] and charge concatenated in
 * molecule order in epc_xyzq.  nddo_batch_set_coordinates moves the atoms
 * only; nddo_scf_result.core_epc_coulomb carries each molecule's core-EPC
 * energy. */
int nddo_batch_create_epc(nddo_ctx* ctx, int theory, int n_mol, const int* n_atoms, const int* atomic_numbers,
                          const double* xyz_bohr, const int* n_epc, const double* epc_xyzq, int diis_num_error_vect,
                          nddo_batch** out);
/* Integrals + SCF + energies of every molecule, on the device only. */
int nddo_batch_run(nddo_batch* b, const nddo_scf_params* params);
/* As nddo_batch_run with DoSCF's requiresGuess: 0 starts every molecule from
 * its density of the previous run (after nddo_batch_set_coordinates: the
 * warm start of MD steps and RPMD beads, src/rpmd/RPMD.cpp:78-84); the first
 * run of a batch always starts from the guess. */
int nddo_batch_run_ex(nddo_batch* b, const nddo_scf_params* params, int requires_guess);
/* New coordinates for all atoms (same atoms, batch order), bohr. */
int nddo_batch_set_coordinates(nddo_batch* b, const double* xyz_bohr);
int nddo_batch_results(nddo_batch* b, nddo_scf_result* results, double* charges);
/* Density P (which 0) or eigenvector rows C (which 1) of molecule m of the
 * batch after nddo_batch_run: n_ao(m) x n_ao(m) doubles, row-major. */
int nddo_batch_get_matrix(nddo_batch* b, int which, int m, double* out);
/* Forces (Hartree/bohr, n_atoms x 3) of molecule m of a resident batch after
 * nddo_batch_run / nddo_batch_run_ex (as nddo_get_forces): the force callers
 * of MolDS's MD / RPMD drivers for the batch's molecules (src/md/MD.cpp:108-113,
 * src/rpmd/RPMD.cpp). */
int nddo_batch_get_forces(nddo_batch* h, int m, double* out_natoms_x3);
size_t nddo_batch_device_bytes(const nddo_batch* b);
void nddo_batch_destroy(nddo_batch* b);
/* Per-kernel-class CUDA-event timing on the launching stream: after enabling,
 * nddo_batch_kernel_times returns, per class, the accumulated milliseconds,
 * the number of timed launches and the algorithmic work of those launches
 * (FLOPs for contractions and the eigensolver, bytes for memory-bound steps).
 * Returns the number of classes. */
int nddo_batch_profile(nddo_batch* b, int enable);
int nddo_batch_kernel_times(nddo_batch* b, int max_classes, double* ms, long long* launches, double* work);
const char* nddo_kernel_class_name(int k);
/* CUDA events on the batch's stream: op 0 records the start, op 1 the stop,
 * op 2 synchronises and writes the elapsed milliseconds to *ms. */
int nddo_batch_timer(nddo_batch* b, int op, double* ms);
/* Number of CUDA kernels this batch has launched so far (kernels replayed
 * from a captured graph included). */
long long nddo_batch_launch_count(const nddo_batch* b);
/* Number of CUDA-graph launches so far: each SCF iteration of a molecule group
 * is captured once and replayed (MolDS has no counterpart; its SCF loop,
 * Cndo2::DoSCF src/cndo/Cndo2.cpp:585-729, calls its routines directly). */
long long nddo_batch_graph_launch_count(const nddo_batch* b);
/* Jacobi sweeps summed over the molecules of the last run (eigensolver work). */
long long nddo_batch_jacobi_sweeps(nddo_batch* b);

/* Serving: a request loop over single-point SCFs with continuous batching.
 * Stands in for the reference's one-molecule-per-process use of DoSCF
 * (src/base/MolDS.cpp:165-178) when many independent requests arrive over
 * time.  Requests are queued by nddo_server_submit (host only, returns at
 * once) and routed by basis size to lanes; each lane admits queued requests
 * in arrival order as its HBM arenas free up (the budget is split between the
 * lanes), keeps every admitted molecule's integrals, density and DIIS history
 * on the device, and runs SCF iterations over all of its molecules at once;
 * a molecule leaves at the iteration boundary after it converges.
 * nddo_server_poll drives the lanes without blocking on the GPU (at most
 * max_wait_us of host time) and returns finished requests: out[k] for
 * k < *n_out, their Mulliken charges concatenated in charges (up to
 * charges_capacity doubles; a result that does not fit stays queued for the
 * next poll).  Times are seconds on the server's clock (nddo_server_clock).
 * A molecule's result does not depend on which other requests share its
 * lane: every kernel works per molecule with fixed-order reductions. */
typedef struct nddo_server nddo_server;
typedef struct {
  long long ticket;            /* returned by nddo_server_submit            */
  int status;                  /* NDDO_STATUS_CONVERGED / NOT_CONVERGED / FAILED */
  int iterations;
  int n_atoms;
  int lane;
  double energy, core_repulsion, heat_of_formation, final_rms;
  double t_submit, t_admit, t_done;
  double core_epc_coulomb;     /* core-EPC Coulomb energy [Eh], included in energy (0 without charges) */
} nddo_serve_result;
int nddo_server_create(nddo_ctx* ctx, const nddo_scf_params* params, size_t hbm_budget_bytes, int max_basis,
                       nddo_server** out);
int nddo_server_submit(nddo_server* s, int theory, int n_atoms, const int* atomic_numbers, const double* xyz_bohr,
                       long long* ticket);
/* nddo_server_submit with environmental point charges (as
 * nddo_set_molecule_epc): n_epc rows of x, y, z [bohr] and charge.  Each
 * lane's pool holds as many point charges as atoms; a request with more
 * than its lane can ever hold is refused with NDDO_ERR_ARGUMENT. */
int nddo_server_submit_epc(nddo_server* s, int theory, int n_atoms, const int* atomic_numbers, const double* xyz_bohr,
                           int n_epc, const double* epc_xyzq, long long* ticket);
int nddo_server_poll(nddo_server* s, int max_wait_us, int max_results, nddo_serve_result* out, double* charges,
                     size_t charges_capacity, int* n_out);
/* Requests queued (not yet admitted) and molecules in the SCF. */
int nddo_server_pending(const nddo_server* s, int* queued, int* in_flight);
double nddo_server_clock(const nddo_server* s);
size_t nddo_server_device_bytes(const nddo_server* s);
void nddo_server_destroy(nddo_server* s);

/* Measured arithmetic peak of this GPU's CUDA cores (not the tensor cores):
 * a dependent-FMA loop over every SM, FP32 (precision 0) or FP64 (1), in
 * TFLOP/s.  The denominator of the eigensolver's roofline. */
int nddo_measure_fma_peak(nddo_ctx* ctx, int precision, double* tflops);

/* Allocation-free pair integrals.  No counterpart in the reference: MolDS
 * allocates its integral store itself.  For callers that cannot call
 * cudaMalloc (a host program that owns all device memory through its own
 * arena, code where a device allocation is forbidden or may not fail), this
 * computes what nddo_set_molecule computes -- the packed pair blocks (layout of
 * nddo_get_pair_blocks), the core Hamiltonian H (n_ao x n_ao, row-major) and
 * the core-core energy -- into the caller's device buffers d_pair_blocks and
 * d_core_hamiltonian, and allocates nothing: its scratch is one fixed static
 * device array of about 4.3 MB that every GPU loading the library keeps until
 * exit.  Inputs (atomic numbers, coordinates in bohr) are host arrays;
 * core_repulsion is a host output (may be NULL); stream is a cudaStream_t (NULL
 * = default stream); err/err_len receive the message of a failure.
 * Limit: n_atoms <= 512; larger molecules are rejected with NDDO_ERR_BUDGET.
 * The first call on a device sets that device up (resolves the array's address
 * and uploads constant tables).  No call may be made on a stream that is being
 * captured (each call copies from host memory and synchronises); such a call
 * returns NDDO_ERR_ARGUMENT.  Calls share the one array, so calls that overlap
 * on the GPU race; serialise them. */
int nddo_pair_integrals_noalloc(int device, int theory, int n_atoms, const int* atomic_numbers,
                                const double* xyz_bohr, double* d_pair_blocks, size_t pair_block_capacity,
                                double* d_core_hamiltonian, double* core_repulsion, void* stream,
                                char* err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* MOLDS_GB300_NDDO_GPU_H */
