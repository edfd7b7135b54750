// Device-side layout of a batch of molecules.
//
// A batch holds any number of molecules of any size.  Per molecule, every
// N x N matrix lives in its own arena (H, F, P, P_old, C, workspaces) at the
// same element offset `mat0`; pair integral blocks live in one double arena at
// per-pair offsets.  All kernels take the batch tables plus a list of the
// molecules they should touch, so converged molecules simply drop out of the
// list and new ones (serving) join without any other molecule noticing.
#pragma once
#include <cstdint>
#include "nddo_math.cuh"

namespace nddo {

constexpr int kNumParamSlots = NDDO_NUM_THEORY_SLOTS * NDDO_NUM_ELEMENTS;
constexpr int kMaxDiis = 8;

struct DevAtom {
  double x, y, z;   // bohr
  int pidx;         // theory * NDDO_NUM_ELEMENTS + element index
  int ao0;          // first AO (molecule-local)
  int nao;          // 1 or 4
  int mol;
};

struct DevPair {
  int a, b;         // batch-global atom indices, a < b, same molecule
  int mol;
  int pad;
  long long blk;    // offset (doubles) of the packed (mu nu|la si) block
};

struct DevMol {
  int natoms, nao, nocc, theory;
  int atom0, pair0, npairs;
  int nepc;         // environmental point charges acting on this molecule
  long long mat0;   // element offset of this molecule's N x N matrices
  long long vec0;   // element offset of this molecule's length-N vectors
  long long epc0;   // first point charge (x, y, z in bohr, charge: 4 doubles each)
};

// SCF state machine of one molecule (MolDS Cndo2::DoSCF, src/cndo/Cndo2.cpp:585-729)
enum MolStatus { kActive = 0, kConverged = 1, kNotConverged = 2, kFailed = 3 };

struct MolState {
  int iter;           // iteration about to run / running
  int status;
  int phase;          // 0: FP32 eigen phase, 1: FP64 refinement phase (mixed precision)
  int requires_guess;
  int diis_on, damp_on;
  int diis_count;     // entries pushed so far
  int diis_head;      // ring slot of the newest entry
  int sweeps;         // Jacobi sweeps of the last diagonalization
  int flags;
  double rms, diis_err, ecore, energy, heat_of_formation, energy_electronic;
  double B[kMaxDiis * kMaxDiis];   // <e_i, e_j> over ring slots
  double dipole[9];   // total, electronic, core dipole (x, y, z each) [a.u.] after convergence
  double vdw_energy;  // empirical dispersion energy (0 when off)
  double ecore_epc;   // Coulomb energy of the cores in the point charges' field
};

struct TraceEntry {
  double rms, diis_err;
  int diis_on, damp_on;
};

struct ScfParamsDev {
  int max_iter;
  int diis_m;
  double rms_density, damping_thresh, damping_weight, diis_start, diis_end;
  double switch_error;      // mixed precision: FP64 phase once the DIIS error is below this
  int precision;            // 0 = FP64 throughout, 1 = mixed
  int pad;
};

__host__ __device__ inline long long pair_index(int a, int b, int natoms) {
  // a < b, molecule-local atom indices; row-major over a < b
  return (long long)a * natoms - ((long long)a * (a + 1)) / 2 + (b - a - 1);
}

}  // namespace nddo
