/*
 * C++ host layer over the C ABI of nddo_gpu.h, with the call surface of
 * MolDS's ElectronicStructure (src/base/ElectronicStructure.h:23-53):
 * GetTheoryType, SetMolecule, DoSCF(requiresGuess), GetFockMatrix (eigenvector
 * rows), GetEnergiesMO, GetElectronicEnergy(0), GetCoreRepulsionEnergy,
 * GetVdWCorrectionEnergy, OutputSCFResults.  Errors are thrown as MolDSException, a
 * std::domain_error like MolDS's (src/base/MolDSException.h:26-41), carrying
 * the C ABI's status code.  Header-only; link with -lnddo_gb300.
 *
 * Out of this path (no counterpart here): DoCIS, GetForce, DoFrequencis and
 * the overlap-with-another-configuration calls.
 */
#ifndef MOLDS_GB300_NDDO_ELECTRONIC_STRUCTURE_HPP
#define MOLDS_GB300_NDDO_ELECTRONIC_STRUCTURE_HPP

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "nddo_gpu.h"

namespace molds_gb300 {

enum TheoryType {
  MNDO = NDDO_THEORY_MNDO,
  AM1 = NDDO_THEORY_AM1,
  PM3 = NDDO_THEORY_PM3,
  AM1D = NDDO_THEORY_AM1D,
  PM3D = NDDO_THEORY_PM3D,
  PM3PDDG = NDDO_THEORY_PM3PDDG
};

class MolDSException : public std::domain_error {
 public:
  MolDSException(const std::string& cause, int code) : std::domain_error(cause), code_(code) {}
  int Code() const { return code_; }   // NDDO_* status of the failing call

 private:
  int code_;
};

// Atoms of one molecule: atomic numbers and Cartesian coordinates in bohr.
struct Molecule {
  std::vector<int> atomicNumbers;
  std::vector<double> xyz;   // 3 per atom
  // environmental point charges (MolDS's EPC block, Molecule::AddEpc):
  // x, y, z in bohr and the charge, 4 per point charge
  std::vector<double> epcs;
};

// SCF block with MolDS's defaults (src/base/Parameters.cpp:133-142).
struct ScfParameters : nddo_scf_params {
  ScfParameters() { nddo_default_params(this); }
};

class ElectronicStructure {
 public:
  explicit ElectronicStructure(TheoryType theory, const ScfParameters& params = ScfParameters(), int device = 0,
                               std::size_t hbmBudgetBytes = 0)
      : theory_(theory), params_(params) {
    const int rc = nddo_create(device, hbmBudgetBytes, &ctx_);
    if (rc != NDDO_OK) {
      const std::string msg = ctx_ ? nddo_last_error(ctx_) : "nddo_create failed";
      nddo_destroy(ctx_);
      ctx_ = nullptr;
      throw MolDSException(msg, rc);
    }
  }
  ~ElectronicStructure() { nddo_destroy(ctx_); }
  ElectronicStructure(const ElectronicStructure&) = delete;
  ElectronicStructure& operator=(const ElectronicStructure&) = delete;

  TheoryType GetTheoryType() const { return theory_; }

  // Non-owning, as MolDS's SetMolecule (src/base/MolDS.cpp:166-171); the
  // one-time integrals are computed here.
  void SetMolecule(const Molecule* molecule) {
    if (!molecule) throw MolDSException("null molecule", NDDO_ERR_ARGUMENT);
    const int n = static_cast<int>(molecule->atomicNumbers.size());
    if (molecule->xyz.size() != 3 * molecule->atomicNumbers.size())
      throw MolDSException("coordinate count does not match atom count", NDDO_ERR_ARGUMENT);
    if (molecule->epcs.size() % 4) throw MolDSException("point charges need x, y, z and a charge each", NDDO_ERR_ARGUMENT);
    const int nEpc = static_cast<int>(molecule->epcs.size() / 4);
    Check(nddo_set_molecule_epc(ctx_, theory_, n, molecule->atomicNumbers.data(), molecule->xyz.data(), nEpc,
                                nEpc ? molecule->epcs.data() : nullptr));
    molecule_ = molecule;
    n_ = nddo_num_aos(ctx_);
    hasScf_ = false;
  }

  // The molecule moved (same atoms): new integrals, last density kept for DoSCF(false).
  void SetCoordinates(const double* xyzBohr) { Check(nddo_set_coordinates(ctx_, xyzBohr)); }

  void DoSCF(bool requiresGuess = true) {
    nddo_scf_result r;
    const int rc = nddo_scf(ctx_, &params_, requiresGuess ? 1 : 0, &r);
    result_ = r;
    Check(rc);
    hasScf_ = true;
    eps_.assign(n_, 0.0);
    Check(nddo_get_energies_mo(ctx_, eps_.data()));
    fock_.assign(static_cast<std::size_t>(n_) * n_, 0.0);
    Check(nddo_get_fock_matrix(ctx_, fock_.data()));
    rows_.resize(n_);
    for (int i = 0; i < n_; ++i) rows_[i] = fock_.data() + static_cast<std::size_t>(i) * n_;
    charges_.assign(molecule_->atomicNumbers.size(), 0.0);
    Check(nddo_get_mulliken(ctx_, charges_.data()));
  }

  // After DoSCF: eigenvectors as rows, sign-normalised (src/wrappers/Lapack.cpp:141-150).
  double const* const* GetFockMatrix() const { Need(); return rows_.data(); }
  double const* GetEnergiesMO() const { Need(); return eps_.data(); }
  double GetElectronicEnergy(int elecState) const {
    Need();
    if (elecState != 0) throw MolDSException("only the ground state is computed on this path", NDDO_ERR_ARGUMENT);
    return result_.energy;   // includes the core repulsion and the vdW term, as MolDS's
  }
  double GetCoreRepulsionEnergy() const { Need(); return result_.core_repulsion; }
  double GetVdWCorrectionEnergy() const { Need(); return result_.vdw_energy; }
  // sum over cores and environmental point charges of Z_A q / R, included in the energy
  double GetCoreEpcCoulombEnergy() const { Need(); return result_.core_epc_coulomb; }
  double GetHeatsFormation() const { Need(); return result_.heat_of_formation; }
  int GetIterations() const { Need(); return result_.iterations; }
  double const* GetMullikenCharges() const { Need(); return charges_.data(); }
  // total, electronic, core dipole (x, y, z each) [a.u.]
  double const* GetDipoleMoments() const { Need(); return result_.dipole; }
  int GetTotalNumberAOs() const { return n_; }
  // Forces -dE/dR on the atoms [Hartree/bohr], n_atoms x 3 row-major, of the
  // last converged SCF (MolDS GetForce after CalcForce, src/mndo/Mndo.cpp:2711-2986).
  std::vector<double> GetForce() const {
    Need();
    std::vector<double> f(3 * molecule_->atomicNumbers.size());
    Check(nddo_get_forces(ctx_, f.data()));
    return f;
  }
  // The SCF section of MolDS's output for the last DoSCF (the text
  // Cndo2::DoSCF prints between its banners, src/cndo/Cndo2.cpp:585-729,
  // with OutputSCFResults :1299-1303).
  std::string OutputSCFResults() const {
    Need();
    std::size_t need = 0;
    Check(nddo_scf_output_text(ctx_, nullptr, 0, &need));
    std::string text(need, '\0');
    Check(nddo_scf_output_text(ctx_, &text[0], need, &need));
    text.resize(need > 0 ? need - 1 : 0);
    return text;
  }

 private:
  void Check(int rc) const {
    if (rc != NDDO_OK) throw MolDSException(nddo_last_error(ctx_), rc);
  }
  void Need() const {
    if (!hasScf_) throw MolDSException("no SCF result", NDDO_ERR_STATE);
  }

  nddo_ctx* ctx_ = nullptr;
  TheoryType theory_;
  ScfParameters params_;
  const Molecule* molecule_ = nullptr;
  int n_ = 0;
  bool hasScf_ = false;
  nddo_scf_result result_{};
  std::vector<double> eps_, fock_, charges_;
  std::vector<double*> rows_;
};

}  // namespace molds_gb300

#endif  // MOLDS_GB300_NDDO_ELECTRONIC_STRUCTURE_HPP
