/*
 * Unit constants and the per-atom parameter record in atomic units.
 *
 * The constants are MolDS's own (src/base/Parameters.cpp:45-48), not CODATA:
 * energies at the 1e-8 Eh level only agree with MolDS when the same eV, Angstrom
 * and kcal/mol conversions are used.  Plain C; usable from C, C++ and CUDA.
 */
#ifndef MOLDS_GB300_NDDO_UNITS_H
#define MOLDS_GB300_NDDO_UNITS_H

#include <math.h>
#include "nddo_elements.h"
#include "nddo_dipole.h"
#include "nddo_dispersion.h"

#define NDDO_EV2AU   0.03674903
#define NDDO_ANG2AU  (1.0 / 0.5291772)
#define NDDO_KCAL2AU 0.00159360175
#define NDDO_DEBYE2AU 0.393430191

/* Everything a pair or Fock kernel needs about one atom, in atomic units. */
typedef struct {
  double core_charge;
  double u[2];          /* U_ss, U_pp                                  */
  double zeta[2];       /* Slater exponents of s and p                 */
  double beta[2];       /* resonance parameters of s and p             */
  double alpha;         /* core-core exponent [1/bohr]                 */
  double gss, gsp, gpp, gp2, hsp, hpp;
  double d[3];          /* charge separations of monopole/dipole/quadrupole (d[0] = 0) */
  double rho[3];        /* additive terms of monopole/dipole/quadrupole */
  double gk[4], gl[4], gm[4];   /* Gaussian core-core terms (a.u.)     */
  double e_atom, dhf_atom;      /* MNDO heat-of-formation bookkeeping  */
  double sto_norm[2];   /* Slater normalisation (2 zeta)^(n+1/2) / sqrt((2n)!) of s and p */
  double core_mass;     /* atomic mass [a.u.] - valence electrons: weight of the dipole origin */
  double vdw_c6;        /* dispersion C6 coefficient [a.u.] (0: none)  */
  double vdw_r0;        /* van der Waals radius [bohr]                 */
  double pddg_pa[2];    /* PDDG/PM3 core-core pre-factors [a.u.] (0 elsewhere) */
  double pddg_da[2];    /* PDDG/PM3 core-core distances [bohr]         */
  int n_ao;             /* 1 or 4                                      */
  int principal_n;      /* 1, 2 or 3                                   */
  int atomic_number;
  int pad;
} nddo_atom_params;

/* Converts the published parameters of one element to atomic units with the
 * same operations MolDS applies when it fills its Atom objects
 * (e.g. alpha = a / angstrom2AU, L = l / angstrom2AU^2, M = m * angstrom2AU). */
static inline int nddo_fill_atom_params(int theory, int atomic_number, nddo_atom_params* out) {
  int e = nddo_element_index(atomic_number);
  if (e < 0 || theory < 0 || theory >= NDDO_NUM_THEORY_SLOTS) return -1;
  const nddo_dispersion_element* dsp = nddo_dispersion_lookup(atomic_number);
  /* AM1-D / PM3-D: the AM1 / PM3 set with the overrides of nddo_dispersion.h */
  const nddo_pddg_element* pg = nddo_pddg_lookup(atomic_number);
  const int base = theory == NDDO_AM1D ? NDDO_AM1 : ((theory == NDDO_PM3D || theory == NDDO_PM3PDDG) ? NDDO_PM3 : theory);
  if ((theory == NDDO_AM1D || theory == NDDO_PM3D) && !dsp) return -1;
  if (theory == NDDO_AM1D && !dsp->has_am1d) return -1;
  if (theory == NDDO_PM3PDDG && !pg) return -1;
  const nddo_element* el = &nddo_elements[e];
  const nddo_theory_params* t = &el->t[base];
  int i;
  out->core_charge = (double)el->core_charge;
  out->u[0] = t->u_s * NDDO_EV2AU;
  out->u[1] = t->u_p * NDDO_EV2AU;
  out->zeta[0] = t->zeta_s;
  out->zeta[1] = t->zeta_p;
  out->beta[0] = t->beta_s * NDDO_EV2AU;
  out->beta[1] = t->beta_p * NDDO_EV2AU;
  out->alpha = t->alpha / NDDO_ANG2AU;
  out->gss = t->gss * NDDO_EV2AU;
  out->gsp = t->gsp * NDDO_EV2AU;
  out->gpp = t->gpp * NDDO_EV2AU;
  out->gp2 = t->gp2 * NDDO_EV2AU;
  out->hsp = t->hsp * NDDO_EV2AU;
  out->hpp = 0.5 * (out->gpp - out->gp2);
  out->d[0] = 0.0;
  out->d[1] = t->d1;
  out->d[2] = t->d2;
  for (i = 0; i < 3; ++i) out->rho[i] = (t->rho_div[i] != 0.0) ? 0.5 / t->rho_div[i] : 0.0;
  for (i = 0; i < 4; ++i) {
    out->gk[i] = t->gk[i] * NDDO_EV2AU;
    out->gl[i] = t->gl[i] / pow(NDDO_ANG2AU, 2.0);
    out->gm[i] = t->gm[i] * NDDO_ANG2AU;
  }
  out->e_atom = t->e_atom * NDDO_EV2AU;
  out->dhf_atom = t->dhf_atom * NDDO_KCAL2AU;
  out->core_mass = nddo_atomic_mass_gmol(atomic_number) * NDDO_GMOLIN2AU - (double)el->core_charge;
  out->vdw_c6 = dsp ? dsp->c6 * NDDO_J2AU * pow(10.0 * NDDO_ANG2AU, 6.0) / NDDO_AVOGADRO : 0.0;
  out->vdw_r0 = dsp ? dsp->r0 * NDDO_ANG2AU : 0.0;
  out->pddg_pa[0] = out->pddg_pa[1] = out->pddg_da[0] = out->pddg_da[1] = 0.0;
  if (theory == NDDO_PM3PDDG) {
    out->u[0] = pg->u_s * NDDO_EV2AU;
    out->u[1] = pg->u_p * NDDO_EV2AU;
    out->zeta[0] = pg->zeta_s;
    out->zeta[1] = pg->zeta_p;
    out->beta[0] = pg->beta_s * NDDO_EV2AU;
    out->beta[1] = pg->beta_p * NDDO_EV2AU;
    out->alpha = pg->alpha / NDDO_ANG2AU;
    out->d[1] = pg->d1;
    out->d[2] = pg->d2;
    for (i = 0; i < 3; ++i) out->rho[i] = pg->rho[i];
    for (i = 0; i < 4; ++i) {
      out->gk[i] = i < 2 ? pg->gk[i] * NDDO_EV2AU : 0.0;
      out->gl[i] = i < 2 ? pg->gl[i] / pow(NDDO_ANG2AU, 2.0) : 0.0;
      out->gm[i] = i < 2 ? pg->gm[i] * NDDO_ANG2AU : 0.0;
    }
    for (i = 0; i < 2; ++i) {
      out->pddg_pa[i] = pg->pa[i] * NDDO_EV2AU;
      out->pddg_da[i] = pg->da[i] * NDDO_ANG2AU;
    }
  } else if (base != theory) {
    const double* o = theory == NDDO_AM1D ? dsp->am1d : dsp->pm3d;
    out->u[0] = o[0] * NDDO_EV2AU;
    out->u[1] = o[1] * NDDO_EV2AU;
    out->beta[0] = o[2] * NDDO_EV2AU;
    out->beta[1] = o[3] * NDDO_EV2AU;
    out->alpha = o[4] / NDDO_ANG2AU;
  }
  {
    double f = 1.0;
    int k;
    for (k = 2; k <= 2 * el->principal_n; ++k) f *= k;
    out->sto_norm[0] = pow(2.0 * out->zeta[0], el->principal_n + 0.5) / sqrt(f);
    out->sto_norm[1] = (out->zeta[1] > 0.0) ? pow(2.0 * out->zeta[1], el->principal_n + 0.5) / sqrt(f) : 0.0;
  }
  out->n_ao = el->n_ao;
  out->principal_n = el->principal_n;
  out->atomic_number = atomic_number;
  out->pad = 0;
  return 0;
}

#endif /* MOLDS_GB300_NDDO_UNITS_H */
