// Drives the C++ host layer (include/nddo_electronic_structure.hpp) the way
// MolDS's main drives an ElectronicStructure (src/base/MolDS.cpp:165-178):
// SetMolecule, DoSCF, then the getters.  Input file: the theory number, then
// one atom per line "Z x y z" in bohr, and environmental point charges as
// lines "epc x y z q" (bohr, charge).  Optional arguments: max_iter
// rms_density damping_thresh damping_weight diis_num_error_vect
// diis_start_error diis_end_error.  Exit code 3 when the engine throws.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "nddo_electronic_structure.hpp"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s molecule.txt [max_iter rms damp_thresh damp_weight diis_n diis_start diis_end]\n",
                 argv[0]);
    return 2;
  }
  std::ifstream in(argv[1]);
  int theory = 0;
  in >> theory;
  molds_gb300::Molecule mol;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string head;
    if (!(ls >> head)) continue;
    double x, y, w, q;
    if (head == "epc") {
      if (ls >> x >> y >> w >> q) mol.epcs.insert(mol.epcs.end(), {x, y, w, q});
      continue;
    }
    if (!(ls >> x >> y >> w)) continue;
    mol.atomicNumbers.push_back(std::atoi(head.c_str()));
    mol.xyz.push_back(x);
    mol.xyz.push_back(y);
    mol.xyz.push_back(w);
  }
  molds_gb300::ScfParameters p;
  if (argc >= 9) {
    p.max_iter = std::atoi(argv[2]);
    p.rms_density = std::atof(argv[3]);
    p.damping_thresh = std::atof(argv[4]);
    p.damping_weight = std::atof(argv[5]);
    p.diis_num_error_vect = std::atoi(argv[6]);
    p.diis_start_error = std::atof(argv[7]);
    p.diis_end_error = std::atof(argv[8]);
  }
  try {
    molds_gb300::ElectronicStructure es(static_cast<molds_gb300::TheoryType>(theory), p);
    es.SetMolecule(&mol);
    es.DoSCF(true);
    std::printf("energy %.15e\n", es.GetElectronicEnergy(0));
    std::printf("core_repulsion %.15e\n", es.GetCoreRepulsionEnergy());
    std::printf("vdw %.15e\n", es.GetVdWCorrectionEnergy());
    std::printf("core_epc %.15e\n", es.GetCoreEpcCoulombEnergy());
    std::printf("iterations %d\n", es.GetIterations());
    const int n = es.GetTotalNumberAOs();
    std::printf("homo %.15e\n", es.GetEnergiesMO()[0]);
    std::printf("eps_last %.15e\n", es.GetEnergiesMO()[n - 1]);
    double sum = 0.0;
    for (int mu = 0; mu < n; ++mu) sum += es.GetFockMatrix()[0][mu];
    std::printf("row0_sum %.15e\n", sum);
    for (std::size_t a = 0; a < mol.atomicNumbers.size(); ++a) std::printf("charge %.15e\n", es.GetMullikenCharges()[a]);
    for (int k = 0; k < 3; ++k) std::printf("dipole %.15e\n", es.GetDipoleMoments()[k]);
    try {
      es.GetElectronicEnergy(1);
    } catch (const molds_gb300::MolDSException& e) {
      std::printf("excited_state_error %d\n", e.Code());
    }
    // MolDS's SCF section, last: everything after the marker line is the text
    std::printf("scf_text\n%s", es.OutputSCFResults().c_str());
    return 0;
  } catch (const molds_gb300::MolDSException& e) {
    std::printf("error %d %s\n", e.Code(), e.what());
    return 3;
  }
}
