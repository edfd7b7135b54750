/*
 * Data of the dipole-moment property of the NDDO SCF: the STO-6G expansion of
 * the valence Slater orbitals and the atomic masses that place the dipole
 * origin.  Plain C; included by C, C++ and CUDA translation units alike.
 *
 * STO-6G: R. F. Stewart, J. Chem. Phys. 52, 431 (1970), Tables I and II --
 * the least-squares expansion of a Slater orbital of exponent 1 in six
 * normalised Gaussians, phi = sum_i d_i g(alpha_i zeta^2).  The values are the
 * ones MolDS uses (src/base/GTOExpansionSTO.cpp:314-347), per valence shell:
 * K (1s), L (2s, 2p), M (3s, 3p).
 *
 * Masses [g/mol]: the standard atomic weights of src/base/atoms/<El>atom.cpp
 * (e.g. Catom.cpp:49), converted with MolDS's g/mol -> a.u. factor
 * (src/base/Parameters.cpp:53).  MolDS's dipole origin is the "centre of core
 * mass" with core mass = atomic mass [a.u.] - number of valence electrons
 * (src/base/atoms/Atom.h:34, src/base/Molecule.cpp:396-419).
 */
#ifndef MOLDS_GB300_NDDO_DIPOLE_H
#define MOLDS_GB300_NDDO_DIPOLE_H

#define NDDO_GMOLIN2AU (1.0e5 / (6.0221415 * 9.1095))   /* src/base/Parameters.cpp:53 */
#define NDDO_DEBYE2AU  0.393430191                       /* src/base/Parameters.cpp:57 */

/* [shell K, L, M][s, p][primitive] */
static const double nddo_sto6g_exp[3][2][6] = {
  { { 2.310303149e01, 4.235915534e00, 1.185056519e00, 4.070988982e-1, 1.580884151e-1, 6.510953954e-2 },
    { 0, 0, 0, 0, 0, 0 } },
  { { 2.768496241e01, 5.077140627e00, 1.426786050e00, 2.040335729e-1, 9.260298399e-2, 4.416183978e-2 },
    { 5.868285913e00, 1.530329631e00, 5.475665231e-1, 2.288932733e-1, 1.046655969e-1, 4.948220127e-2 } },
  { { 3.273031938e00, 9.200611311e-1, 3.593349765e-1, 8.636686991e-2, 4.797373812e-2, 2.724741144e-2 },
    { 5.077973607e00, 1.340786940e00, 2.248434849e-1, 1.131741848e-1, 6.076408893e-2, 3.315424265e-2 } },
};
static const double nddo_sto6g_coef[3][2][6] = {
  { { 9.163596280e-3, 4.936149294e-2, 1.685383049e-1, 3.705627997e-1, 4.164915298e-1, 1.303340841e-1 },
    { 0, 0, 0, 0, 0, 0 } },
  { { -4.151277819e-3, -2.067024148e-2, -5.150303337e-2, 3.346271174e-1, 5.621061301e-1, 1.712994697e-1 },
    { 7.924233646e-3, 5.144104825e-2, 1.898400060e-1, 4.049863191e-1, 4.012362861e-1, 1.051855189e-1 } },
  { { -6.775596947e-3, -5.639325779e-2, -1.587656086e-1, 5.534527651e-1, 5.015351020e-1, 7.223633674e-2 },
    { -3.329929840e-3, -1.419488340e-2, 1.639395770e-1, 4.485358256e-1, 3.908813050e-1, 7.411456232e-2 } },
};

/* Standard atomic weight [g/mol] of the elements with NDDO parameters (0 otherwise). */
static inline double nddo_atomic_mass_gmol(int atomic_number) {
  switch (atomic_number) {
    case 1: return 1.00794;
    case 6: return 12.0107;
    case 7: return 14.00674;
    case 8: return 15.9994;
    case 9: return 18.9984032;
    case 16: return 32.066;
    case 17: return 35.453;
    default: return 0.0;
  }
}

#endif /* MOLDS_GB300_NDDO_DIPOLE_H */
