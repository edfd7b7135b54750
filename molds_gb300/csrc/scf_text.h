// The SCF section of MolDS's output text (scf_text.cpp).
#pragma once
#include <string>

namespace nddo {

struct ScfText {
  int theory = 0;                   // NDDO_THEORY_*
  int n_atoms = 0;
  const int* Z = nullptr;           // atomic numbers
  int n_ao = 0, nocc = 0;
  int iterations = 0;               // entries of the iteration log
  const double* rms = nullptr;      // per iteration: RMS density change
  const double* diis_error = nullptr;
  const int* diis_on = nullptr;
  const int* damp_on = nullptr;
  int converged = 0;                // the results follow only a converged SCF
  const double* eps = nullptr;      // MO energies [a.u.]
  double energy = 0.0;              // total energy (includes core repulsion and vdW)
  double core_repulsion = 0.0;
  int vdw = 0;                      // the vdW lines (AM1-D, PM3-D, or the vdW option)
  double vdw_energy = 0.0;
  int epc = 0;                      // the point-charge lines (the molecule has environmental point charges)
  double core_epc = 0.0;            // Coulomb energy of the cores and the point charges
  const double* dipole = nullptr;   // 9: total, electronic, core (x, y, z); null: no dipole block
  const double* charges = nullptr;  // Mulliken charges
  int n_sum = 0;                    // SCF option sum_charges: pairs (first, last) of atom indices
  const int* sum_pairs = nullptr;
  double heat_of_formation = 0.0;   // MNDO
  double seconds = 0.0;             // the elapsed-time line
};

std::string format_scf_text(const ScfText& t);

}  // namespace nddo
