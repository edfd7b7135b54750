/*
 * The NDDO variants beyond MNDO / AM1 / PM3: AM1-D and PM3-D (MolDS's
 * dispersion-corrected sets) with the empirical van der Waals energy, and
 * PDDG/PM3.  Plain C; included by C, C++ and CUDA alike.
 *
 * AM1-D / PM3-D are the AM1 / PM3 parameter sets with U_s, U_p, beta_s,
 * beta_p and the core-core exponent alpha replaced by the values of
 * src/base/atoms/<El>atom.cpp (e.g. Catom.cpp:155-159 and 219-223), and the
 * dispersion energy always on with s6 = 1.40, d = 23
 * (src/base/InputParser.cpp:1657-1664, src/base/Parameters.cpp:60-61).  MolDS
 * gives H, C, N, O and S their own AM1-D / PM3-D values; its F and Cl PM3-D
 * sets are PM3's (Fatom.cpp:213-217, Clatom.cpp:231-235), and their AM1-D
 * alpha is never assigned (Fatom.cpp:153, Clatom.cpp:171), so AM1-D is served
 * for H, C, N, O, S and PM3-D for all seven elements.  Every element carries
 * the C6 coefficient and radius of the vdW option.
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
enum { NDDO_AM1D = 3, NDDO_PM3D = 4, NDDO_PM3PDDG = 5, NDDO_NUM_THEORY_SLOTS = 6 };

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
  int has_am1d;     /* 0: no AM1-D set (F, Cl: the reference never assigns their AM1-D alpha) */
} nddo_dispersion_element;

enum { NDDO_NUM_DISPERSION_ELEMENTS = 7 };

static const nddo_dispersion_element nddo_dispersion_elements[NDDO_NUM_DISPERSION_ELEMENTS] = {
  { 1, 0.16, 1.110,
    { -11.223791, 0.0, -6.376265, 0.0, 3.577756 },
    { -13.054076, 0.0, -5.628901, 0.0, 3.417532 }, 1 },
  { 6, 1.65, 1.610,
    { -52.183798, -39.368413, -15.682341, -7.804762, 2.625506 },
    { -47.275431, -36.268916, -11.941466, -9.819760, 2.721152 }, 1 },
  { 7, 1.11, 1.550,
    { -71.997845, -57.401718, -20.092408, -18.470679, 2.968737 },
    { -49.348460, -47.543768, -14.068411, -20.039292, 3.060404 }, 1 },
  { 8, 0.70, 1.490,
    { -97.610588, -78.589700, -29.502481, -29.495380, 4.633699 },
    { -86.960302, -71.926845, -45.234302, -24.788037, 3.387806 }, 1 },
  { 16, 10.3, 1.870,
    { -57.235044, -48.307513, -3.311308, -7.256468, 2.309315 },
    { -50.249536, -43.968965, -8.397415, -7.594232, 2.234331 }, 1 },
  /* F and Cl: C6 and radius for the vdW option; their PM3-D set is PM3's
   * (Fatom.cpp:213-217, Clatom.cpp:231-235) */
  { 9, 0.57, 1.430,
    { 0, 0, 0, 0, 0 },
    { -110.435303, -105.685047, -48.405939, -27.744660, 3.358921 }, 0 },
  { 17, 8.00, 1.820,
    { 0, 0, 0, 0, 0 },
    { -100.626747, -53.614396, -27.528560, -11.593922, 2.517296 }, 0 },
};

static inline const nddo_dispersion_element* nddo_dispersion_lookup(int atomic_number) {
  int i;
  for (i = 0; i < NDDO_NUM_DISPERSION_ELEMENTS; ++i)
    if (nddo_dispersion_elements[i].atomic_number == atomic_number) return &nddo_dispersion_elements[i];
  return 0;
}

/*
 * PDDG/PM3 (Repasky, Chandrasekhar, Jorgensen, J. Comput. Chem. 23, 1601
 * (2002); src/pm3/Pm3Pddg.cpp): its own U, zeta, beta, alpha, multipole
 * distances D1, D2, additive terms rho0..rho2 and two core-core Gaussians
 * (the one-centre integrals stay PM3's, src/base/atoms/Atom.cpp:950-1061),
 * plus the pairwise PDDG term of Pm3Pddg::GetDiatomCoreRepulsionEnergy
 * (Pm3Pddg.cpp:143-165, 239-245):
 *   (1 / (n_A + n_B)) sum_{i,j} (n_A Pa_i + n_B Pb_j) exp(-10 A^-2 (R - Da_i - Db_j)^2),
 * n = valence electrons.  Values of src/base/atoms/<El>atom.cpp (e.g.
 * Catom.cpp:190-218); H, C, N, O, S only (Pm3Pddg.cpp:134-141).
 */
typedef struct {
  int atomic_number;
  double u_s, u_p, zeta_s, zeta_p, beta_s, beta_p;   /* [eV], [1/bohr], [eV] */
  double alpha;                                      /* [1/Angstrom] */
  double d1, d2;                                     /* [bohr] */
  double rho[3];                                     /* [bohr] */
  double gk[2], gl[2], gm[2];                        /* [eV], [1/Angstrom^2], [Angstrom] */
  double pa[2], da[2];                               /* [eV], [Angstrom] */
} nddo_pddg_element;

enum { NDDO_NUM_PDDG_ELEMENTS = 5 };

static const nddo_pddg_element nddo_pddg_elements[NDDO_NUM_PDDG_ELEMENTS] = {
  { 1, -12.893272, 0.0, 0.972786, 0.0, -6.152654, 0.0, 3.381686, 0.0, 0.0, { 0.919616, 0.0, 0.0 },
    { 1.122244, -1.069737 }, { 4.707790, 5.857995 }, { 1.547099, 1.567893 },
    { 0.057193, -0.034823 }, { 0.663395, 1.081901 } },
  { 6, -48.241241, -36.461256, 1.567864, 1.846659, -11.952818, -9.922411, 2.725772, 0.831413, 0.663222,
    { 1.214657, 0.848467, 0.652785 },
    { 0.048906, 0.047697 }, { 5.765340, 5.973721 }, { 1.682232, 0.894406 },
    { -0.000743, 0.000985 }, { 0.836915, 1.585236 } },
  { 7, -49.454546, -47.757406, 2.035807, 2.324327, -14.117230, -19.938509, 2.849124, 0.654855, 0.526924,
    { 1.142818, 0.991235, 0.676704 },
    { 1.513320, -1.511892 }, { 5.904394, 6.030014 }, { 1.728376, 1.734108 },
    { -0.003160, 0.012501 }, { 1.004172, 1.516336 } },
  { 8, -87.412505, -72.183070, 3.814565, 2.318011, -44.874553, -24.601939, 3.225309, 0.403741, 0.528360,
    { 0.863494, 0.936266, 0.624291 },
    { -1.138455, 1.146007 }, { 6.000043, 5.963494 }, { 1.622362, 1.614788 },
    { -0.001000, -0.001522 }, { 1.360685, 1.366407 } },
  { 16, -43.906366, -43.461348, 1.012002, 1.876999, -2.953912, -8.507779, 2.539751, 1.006989, 0.891487,
    { 1.517625, 0.711672, 0.754336 },
    { -0.330692, 0.024171 }, { 6.000000, 6.000000 }, { 0.823837, 2.017756 },
    { 0.120434, -0.002663 }, { 0.672870, 2.032340 } },
};

static inline const nddo_pddg_element* nddo_pddg_lookup(int atomic_number) {
  int i;
  for (i = 0; i < NDDO_NUM_PDDG_ELEMENTS; ++i)
    if (nddo_pddg_elements[i].atomic_number == atomic_number) return &nddo_pddg_elements[i];
  return 0;
}

#endif /* MOLDS_GB300_NDDO_DISPERSION_H */
