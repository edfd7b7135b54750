// The SCF section of MolDS's output text, from the results of one SCF.
//
// Reproduces what Cndo2::DoSCF prints between its start and done banners
// (src/cndo/Cndo2.cpp:585-729): the iteration log of
// SatisfyConvergenceCriterion (:1505-1510), the convergence message, then
// OutputSCFResults (:1299-1303): OutputMOEnergies (:1063-1078),
// OutputSCFEnergies (:1080-1124, with the point-charge lines :1090-1115),
// OutputSCFDipole (:1126-1185),
// OutputSCFMulliken (:1187-1221, with the sum_charges option), for MNDO the heat of formation
// (src/mndo/Mndo.cpp:412-420), and the elapsed-time line and done banner.
// The labels and number formats are the reference's, so that its output
// files can be compared line by line.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "nddo_units.h"
#include "scf_text.h"

namespace nddo {
namespace {

const char* theory_label(int theory) {
  static const char* names[] = {"MNDO", "AM1", "PM3", "AM1-D", "PM3-D", "PM3/PDDG"};
  return (theory >= 0 && theory < 6) ? names[theory] : "?";
}

void add(std::string* out, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void add(std::string* out, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  const int n = vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (n > 0) out->append(buf, (size_t)std::min(n, (int)sizeof(buf) - 1));
}

void dipole_line(std::string* out, const char* label, const char* sep, double x, double y, double z) {
  const double m = std::sqrt(std::pow(x, 2.0) + std::pow(y, 2.0) + std::pow(z, 2.0));
  add(out, "%s%s%e\t%e\t%e\t%e\t\t%e\t%e\t%e\t%e\n\n", label, sep, x, y, z, m, x / NDDO_DEBYE2AU, y / NDDO_DEBYE2AU,
      z / NDDO_DEBYE2AU, m / NDDO_DEBYE2AU);
}

}  // namespace

std::string format_scf_text(const ScfText& t) {
  std::string o;
  const char* th = theory_label(t.theory);
  add(&o, "**********  START: %s-SCF  **********\n", th);
  o += "\t\t\t|  RMS density  | DIIS error | DIIS on/off | damping on/off |\n";
  for (int i = 0; i < t.iterations; ++i)
    add(&o, "\tSCF iter %d\t%e\t%e\t%s\t\t%s\n", i, t.rms[i], t.diis_error[i], t.diis_on[i] ? "on" : "",
        t.damp_on[i] ? "on" : "");
  if (!t.converged) return o;   // MolDS throws here: no results, no done banner
  add(&o, "\n\n\n\t\t%s-SCF met convergence criterion(^^b\n\n\n", th);
  // MO energies
  o += "\t\t\t| i-th | occ/unocc |  e[a.u.]  |  e[eV]  | \n";
  for (int mo = 0; mo < t.n_ao; ++mo)
    add(&o, "\tEnergy of MO:\t%d\t%s\t%e\t%e\n", mo, mo < t.nocc ? "occ" : "unocc", t.eps[mo], t.eps[mo] / NDDO_EV2AU);
  o += "\n";
  // energies
  const bool vdw = t.vdw != 0;
  o += "\t\t\t\t|   [a.u.]   |   [eV]   |\n";
  add(&o, "\tElectronic energy(SCF):\t%e\t%e\n", t.energy, t.energy / NDDO_EV2AU);
  if (t.epc)
    o += vdw ? "\tNote that this electronic energy includes core-repulsions, core-EPC coulomb, and vdW correction.\n\n"
             : "\tNote that this electronic energy includes core-repulsions and core-EPC coulomb.\n\n";
  else
    o += vdw ? "\tNote that this electronic energy includes core-repulsions and vdW correction.\n\n"
             : "\tNote that this electronic energy includes core-repulsions.\n\n";
  o += "\t\t\t\t|   [a.u.]   |   [eV]   |\n";
  add(&o, "\tCore repulsion energy:\t%e\t%e\n\n", t.core_repulsion, t.core_repulsion / NDDO_EV2AU);
  if (t.epc) {
    o += "\t\t\t\t\t\t\t\t|   [a.u.]   |   [eV]   |\n";
    add(&o, "\tCoulomb interaction between cores and EPCs energy:\t%e\t%e\n\n", t.core_epc, t.core_epc / NDDO_EV2AU);
  }
  if (vdw) {
    o += "\t\t\t\t\t\t|   [a.u.]   |   [eV]   |\n";
    add(&o, "\tEmpirical van der Waals correction:\t%e\t%e\n\n", t.vdw_energy, t.vdw_energy / NDDO_EV2AU);
  }
  // dipole moments: total = electronic + core, as the reference forms it
  if (t.dipole) {
    const double* e = t.dipole + 3;
    const double* c = t.dipole + 6;
    o += "\t\t\t\t\t|   x[a.u.]   |   y[a.u.]   |   z[a.u.]   |  magnitude[a.u.]  |\t\t|  x[debye]  |  y[debye]  |  "
         "z[debye]  |  magnitude[debye]  |\n";
    dipole_line(&o, "\tTotal Dipole moment(SCF):", "\t", e[0] + c[0], e[1] + c[1], e[2] + c[2]);
    o += "\t\t\t\t\t|  x[a.u.]  |  y[a.u.]  |  z[a.u.]  |  magnitude[a.u.]  |\t\t|  x[debye]  |  y[debye]  |  "
         "z[debye]  |  magnitude[debye]  |\n";
    dipole_line(&o, "\tElectronic Dipole moment(SCF):", "\t", e[0], e[1], e[2]);
    o += "\t\t\t\t\t|  x[a.u.]  |  y[a.u.]  |  z[a.u.]  |  magnitude[a.u.]  |\t\t|  x[debye]  |  y[debye]  |  "
         "z[debye]  |  magnitude[debye]  |\n";
    dipole_line(&o, "\tCore Dipole moment:", "\t\t", c[0], c[1], c[2]);
  }
  // Mulliken charges
  o += "\t\t\t\t| k-th eigenstate | i-th atom | atom type | core charge[a.u.] | Mulliken charge[a.u.]| \n";
  for (int a = 0; a < t.n_atoms; ++a) {
    const int e = nddo_element_index(t.Z[a]);
    const char* sym = e >= 0 ? nddo_elements[e].symbol : "?";
    const double core = e >= 0 ? (double)nddo_elements[e].core_charge : 0.0;
    add(&o, "\tMulliken charge(SCF):\t%d\t%d\t%s\t%e\t%e\n", 0, a, sym, core, t.charges[a]);
  }
  o += "\n";
  if (t.n_sum > 0) {   // OutputSCFMulliken's sums over atom ranges (Cndo2.cpp:1203-1220)
    o += "\t\t\t\t| k-th eigenstate | first atom | last atom | sum[a.u.] | \n";
    for (int i = 0; i < t.n_sum; ++i) {
      const int f = t.sum_pairs[2 * i], l = t.sum_pairs[2 * i + 1];
      double sum = 0.0;
      for (int a = std::max(f, 0); a <= l && a < t.n_atoms; ++a) sum += t.charges[a];
      add(&o, "\tSummation of Mulliken(SCF):\t%d\t%d\t%d\t%e\n", 0, f, l, sum);
    }
    o += "\n";
  }
  if (t.theory == 0) {   // Mndo::OutputSCFResults; AM1, PM3 and their variants print no heat of formation
    o += "\t\t\t\t|  [a.u.]  |  [Kcal/mol]  | \n";
    add(&o, "\tHeats of formation:\t%e\t%e\n\n", t.heat_of_formation, t.heat_of_formation / NDDO_KCAL2AU);
  }
  add(&o, "\tElapsed time(omp) for the SCF = %lf[s].\n**********  DONE: %s-SCF  **********\n\n\n", t.seconds, th);
  return o;
}

}  // namespace nddo
