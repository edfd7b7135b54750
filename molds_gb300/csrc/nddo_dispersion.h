/*
 * AM1-D and PM3-D, MolDS's dispersion-corrected variants, and the empirical
 * van der Waals energy.  Plain C; included by C, C++ and CUDA alike.
 *
 * AM1-D / PM3-D are the AM1 / PM3 parameter sets with U_s, U_p, beta_s,
 * beta_p and the core-core exponent alpha replaced by the values of
 * src/base/atoms/<El>atom.cpp (e.g. Catom.cpp:155-159 and 219-223), and the
 * dispersion energy always on with s6 = 1.40, d = 23
 * (src/base/InputParser.cpp:1657-1664, src/base/Parameters.cpp:60-61).  MolDS
 * defines them for H, C, N, O and S only.
 *
 * Dispersion energy (Grimme's damped C6 / R^6 form, src/cndo/Cndo2.cpp:464-513):
 *   E = -s6 sum_{A<B} C6_AB f(R_AB) / R_AB^6,  C6_AB = 2 C6_A C6_B / (C6_A + C6_B),
 *   f(R) = 1 / (1 + exp(-d (R / (r0_A + r0_B) - 1))),
 * with the C6 coefficients [J nm^6 / mol] and radii [Angstrom] of the element
 * files (e.g. Catom.cpp:60-63), converted with MolDS's constants
 * (src/base/Parameters.cpp:46-56).
 */
#ifndef MOLDS_GB300_NDDO_DISPERSION_H
#define MOLDS_GB300_NDDO_DISPERSION_H

/* parameter slots beyond the three published sets of nddo_elements.h */
enum { NDDO_AM1D = 3, NDDO_PM3D = 4, NDDO_NUM_THEORY_SLOTS = 5 };

#define NDDO_J2AU      (1.0e18 / 4.35974394)   /* src/base/Parameters.cpp:46 */
#define NDDO_AVOGADRO  6.0221415e23            /* src/base/Parameters.cpp:56 */
#define NDDO_VDW_S6_D  1.40                    /* s6 of AM1-D / PM3-D */
#define NDDO_VDW_DAMP_D 23.0                   /* d of AM1-D / PM3-D */

typedef struct {
  int atomic_number;
  double c6;        /* [J nm^6 / mol] */
  double r0;        /* [Angstrom] */
  double am1d[5];   /* U_s, U_p, beta_s, beta_p [eV], alpha [1/Angstrom] */
  double pm3d[5];
} nddo_dispersion_element;

enum { NDDO_NUM_DISPERSION_ELEMENTS = 5 };

static const nddo_dispersion_element nddo_dispersion_elements[NDDO_NUM_DISPERSION_ELEMENTS] = {
  { 1, 0.16, 1.110,
    { -11.223791, 0.0, -6.376265, 0.0, 3.577756 },
    { -13.054076, 0.0, -5.628901, 0.0, 3.417532 } },
  { 6, 1.65, 1.610,
    { -52.183798, -39.368413, -15.682341, -7.804762, 2.625506 },
    { -47.275431, -36.268916, -11.941466, -9.819760, 2.721152 } },
  { 7, 1.11, 1.550,
    { -71.997845, -57.401718, -20.092408, -18.470679, 2.968737 },
    { -49.348460, -47.543768, -14.068411, -20.039292, 3.060404 } },
  { 8, 0.70, 1.490,
    { -97.610588, -78.589700, -29.502481, -29.495380, 4.633699 },
    { -86.960302, -71.926845, -45.234302, -24.788037, 3.387806 } },
  { 16, 10.3, 1.870,
    { -57.235044, -48.307513, -3.311308, -7.256468, 2.309315 },
    { -50.249536, -43.968965, -8.397415, -7.594232, 2.234331 } },
};

static inline const nddo_dispersion_element* nddo_dispersion_lookup(int atomic_number) {
  int i;
  for (i = 0; i < NDDO_NUM_DISPERSION_ELEMENTS; ++i)
    if (nddo_dispersion_elements[i].atomic_number == atomic_number) return &nddo_dispersion_elements[i];
  return 0;
}

#endif /* MOLDS_GB300_NDDO_DISPERSION_H */
