/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C restatement of the MolDS NDDO (MNDO / AM1 / PM3) one-time
 * integrals, Fock build and core-core energy.  Only tests/, the smoke check in
 * __graft_entry__.py and bench.py's CPU-baseline leg load this file (as
 * oracle/_build/liboracle.so through ctypes), and only as the checker or as the
 * timed CPU reference: the CUDA product path never links or calls it.
 *
 * What it follows in the reference (paths relative to the MolDS tree):
 *   orbital order s, py, pz, px ............ src/base/Enums.h:98-108
 *   overlap (diatomic frame, rotated) ...... src/cndo/Cndo2.cpp:4030-4146, 5801-5869, 6091-6221
 *   rotation matrix (gamma = 0) ............ src/cndo/Cndo2.cpp:5498-5527, src/base/EularAngle.cpp:38-64
 *   local two-centre integrals ............. src/mndo/Mndo.cpp:4886-5238 (Dewar-Thiel 1977 Eqs. 29-49)
 *   multipole-multipole terms .............. src/mndo/Mndo.cpp:6592-6834 (Eqs. 52-65)
 *   4-index rotation ....................... src/mndo/Mndo.cpp:4223-4293
 *   Fock elements .......................... src/mndo/Mndo.cpp:422-650, src/cndo/Cndo2.cpp:1526-1636
 *   core-core (MNDO + H-N/H-O rule) ........ src/mndo/Mndo.cpp:223-240, 319-327
 *   AM1/PM3 Gaussian core-core terms ....... src/am1/Am1.cpp:145-170, src/am1/Am1.h:45-47
 *   PDDG/PM3 core-core term ................ src/pm3/Pm3Pddg.cpp:143-165, 239-245
 *   Cartesian (dipole) matrix, STO-6G ...... src/cndo/Cndo2.cpp:1946-2057, 2068-2130, 2149-2400
 *   Gaussian overlaps (s, p) ............... src/cndo/Cndo2.cpp:4563-4575, 4601-5153
 *
 * The STO overlap is evaluated here by my own expansion in prolate-spheroidal
 * coordinates (the integrand is a polynomial in xi, eta times exp(-p xi - q eta),
 * integrated with the standard A_k / B_k auxiliary integrals); MolDS uses the
 * tabulated reduced-overlap coefficients of Pople's book instead.  Both compute
 * the same Slater-orbital overlap; B_k here uses a power series for small |q|,
 * which avoids the cancellation of the closed form.
 */
#include <math.h>
#include <string.h>
#include <stdlib.h>

/* Per-atom parameters in atomic units.  The oracle does not include the
 * product's parameter tables: oracle/parameters.py builds each record from
 * tests/golden/reference_parameters.json (the values MolDS's
 * SetAtomicParameters assigns, read from the reference sources as text) and
 * installs it with oracle_set_atom; the unit constant and the STO-6G tables
 * come from the same file. */
typedef struct {
  double core_charge;
  double u[2], zeta[2], beta[2], alpha;
  double gss, gsp, gpp, gp2, hsp, hpp;
  double d[3], rho[3];
  double gk[4], gl[4], gm[4];
  double e_atom, dhf_atom, core_mass, vdw_c6, vdw_r0;
  double pddg_pa[2], pddg_da[2];
  int n_ao, principal_n, atomic_number;
} oracle_atom;

enum { ORACLE_MNDO = 0, ORACLE_PM3PDDG = 5, ORACLE_SLOTS = 6, ORACLE_MAXZ = 18, ORACLE_REC = 44 };
static oracle_atom g_tab[ORACLE_SLOTS][ORACLE_MAXZ];
static int g_have[ORACLE_SLOTS][ORACLE_MAXZ];
static double g_ang2au = 0.0;                       /* Parameters::angstrom2AU */
static double g_sto_exp[3][2][6], g_sto_coef[3][2][6];

/* rec: the ORACLE_REC doubles of oracle/parameters.py RECORD */
int oracle_set_atom(int theory, int Z, const double* rec) {
  if (theory < 0 || theory >= ORACLE_SLOTS || Z < 1 || Z >= ORACLE_MAXZ) return -1;
  oracle_atom* a = &g_tab[theory][Z];
  int k = 0;
  a->core_charge = rec[k++];
  a->u[0] = rec[k++]; a->u[1] = rec[k++];
  a->zeta[0] = rec[k++]; a->zeta[1] = rec[k++];
  a->beta[0] = rec[k++]; a->beta[1] = rec[k++];
  a->alpha = rec[k++];
  a->gss = rec[k++]; a->gsp = rec[k++]; a->gpp = rec[k++]; a->gp2 = rec[k++]; a->hsp = rec[k++]; a->hpp = rec[k++];
  for (int i = 0; i < 3; ++i) a->d[i] = rec[k++];
  for (int i = 0; i < 3; ++i) a->rho[i] = rec[k++];
  for (int i = 0; i < 4; ++i) a->gk[i] = rec[k++];
  for (int i = 0; i < 4; ++i) a->gl[i] = rec[k++];
  for (int i = 0; i < 4; ++i) a->gm[i] = rec[k++];
  a->e_atom = rec[k++]; a->dhf_atom = rec[k++]; a->core_mass = rec[k++];
  a->vdw_c6 = rec[k++]; a->vdw_r0 = rec[k++];
  a->pddg_pa[0] = rec[k++]; a->pddg_pa[1] = rec[k++]; a->pddg_da[0] = rec[k++]; a->pddg_da[1] = rec[k++];
  a->n_ao = (int)rec[k++]; a->principal_n = (int)rec[k++]; a->atomic_number = (int)rec[k++];
  g_have[theory][Z] = 1;
  return k == ORACLE_REC ? 0 : -1;
}

/* ex, co: [shell K, L, M][s, p][6] */
void oracle_set_constants(double angstrom2au, const double* ex, const double* co) {
  g_ang2au = angstrom2au;
  memcpy(g_sto_exp, ex, sizeof(g_sto_exp));
  memcpy(g_sto_coef, co, sizeof(g_sto_coef));
}

static int oracle_fill(int theory, int Z, oracle_atom* out) {
  if (theory < 0 || theory >= ORACLE_SLOTS || Z < 1 || Z >= ORACLE_MAXZ || !g_have[theory][Z]) return -1;
  *out = g_tab[theory][Z];
  return 0;
}

enum { ORB_S = 0, ORB_PY = 1, ORB_PZ = 2, ORB_PX = 3 };

/* ------------------------------------------------------------------------ */
/* Overlap                                                                  */
/* ------------------------------------------------------------------------ */

#define PDEG 12
typedef struct { double c[PDEG][PDEG]; } poly2;   /* c[i][j] * xi^i * eta^j */

static void poly_one(poly2* p) { memset(p, 0, sizeof(*p)); p->c[0][0] = 1.0; }

static void poly_mul(poly2* out, const poly2* a, const poly2* b) {
  poly2 r; memset(&r, 0, sizeof(r));
  for (int i = 0; i < PDEG; ++i)
    for (int j = 0; j < PDEG; ++j) {
      double x = a->c[i][j];
      if (x == 0.0) continue;
      for (int k = 0; k + i < PDEG; ++k)
        for (int l = 0; l + j < PDEG; ++l) r.c[i + k][j + l] += x * b->c[k][l];
    }
  *out = r;
}

/* multiply by (c0 + cx*xi + ce*eta + cxe*xi*eta + cxx*xi^2 + cee*eta^2) */
static void poly_mul_lin(poly2* p, double c0, double cx, double ce, double cxe, double cxx, double cee) {
  poly2 f; memset(&f, 0, sizeof(f));
  f.c[0][0] = c0; f.c[1][0] = cx; f.c[0][1] = ce; f.c[1][1] = cxe; f.c[2][0] = cxx; f.c[0][2] = cee;
  poly_mul(p, p, &f);
}

/* A_k(p) = int_1^inf xi^k exp(-p xi) dxi, upward recurrence (stable, p > 0) */
static void aux_a(double p, int kmax, double* a) {
  double e = exp(-p);
  a[0] = e / p;
  for (int k = 1; k <= kmax; ++k) a[k] = (e + k * a[k - 1]) / p;
}

/* B_k(q) = int_-1^1 eta^k exp(-q eta) deta */
static void aux_b(double q, int kmax, double* b) {
  if (fabs(q) < 3.0) {
    for (int k = 0; k <= kmax; ++k) {
      double term = 1.0, sum = 0.0;   /* term = (-q)^m / m! */
      for (int m = 0; m < 80; ++m) {
        if (((k + m) & 1) == 0) sum += term * 2.0 / (double)(k + m + 1);
        term *= -q / (double)(m + 1);
        if (m > 8 && fabs(term) < 1e-300) break;
      }
      b[k] = sum;
    }
  } else {
    double ep = exp(q), em = exp(-q);
    b[0] = (ep - em) / q;
    for (int k = 1; k <= kmax; ++k) b[k] = (k * b[k - 1] + ((k & 1) ? -ep : ep) - em) / q;
  }
}

static double factorial(int n) { double f = 1.0; for (int i = 2; i <= n; ++i) f *= i; return f; }

/* kind: 0 = s, 1 = p sigma, 2 = p pi.  Overlap of two normalized Slater
 * orbitals, A at the origin and B at +R on the common z axis. */
double oracle_sto_overlap_local(int na, int kinda, double za, int nb, int kindb, double zb, double R) {
  poly2 pa, pb, prod;
  poly_one(&pa); poly_one(&pb);
  int ea = (kinda == 0) ? na - 1 : na - 2;
  int eb = (kindb == 0) ? nb - 1 : nb - 2;
  for (int i = 0; i < ea; ++i) poly_mul_lin(&pa, 0, 1, 1, 0, 0, 0);      /* (xi + eta)  */
  for (int i = 0; i < eb; ++i) poly_mul_lin(&pb, 0, 1, -1, 0, 0, 0);     /* (xi - eta)  */
  if (kinda == 1) poly_mul_lin(&pa, 1, 0, 0, 1, 0, 0);                    /* (1 + xi eta) */
  if (kindb == 1) poly_mul_lin(&pb, -1, 0, 0, 1, 0, 0);                   /* (xi eta - 1) */
  poly_mul(&prod, &pa, &pb);
  double ang;
  if (kinda == 2 && kindb == 2) {
    poly_mul_lin(&prod, -1, 0, 0, 0, 1, 0);   /* (xi^2 - 1) */
    poly_mul_lin(&prod, 1, 0, 0, 0, 0, -1);   /* (1 - eta^2) */
    ang = 0.75;
  } else if (kinda == 2 || kindb == 2) {
    return 0.0;
  } else {
    ang = 0.5 * ((kinda == 1) ? sqrt(3.0) : 1.0) * ((kindb == 1) ? sqrt(3.0) : 1.0);
  }
  poly_mul_lin(&prod, 0, 0, 0, 0, 1, -1);     /* volume element (xi^2 - eta^2) */
  double p = 0.5 * R * (za + zb), q = 0.5 * R * (za - zb);
  double A[PDEG], B[PDEG];
  aux_a(p, PDEG - 1, A);
  aux_b(q, PDEG - 1, B);
  double s = 0.0;
  for (int i = 0; i < PDEG; ++i)
    for (int j = 0; j < PDEG; ++j)
      if (prod.c[i][j] != 0.0) s += prod.c[i][j] * A[i] * B[j];
  double norm = pow(2.0 * za, na + 0.5) * pow(2.0 * zb, nb + 0.5) / sqrt(factorial(2 * na) * factorial(2 * nb));
  return norm * ang * pow(0.5 * R, na + nb + 1) * s;
}

/* ------------------------------------------------------------------------ */
/* Rotation: rows = space-frame orbital, columns = diatomic-frame orbital,   */
/* local z along A->B, gamma = 0.                                           */
/* ------------------------------------------------------------------------ */
static void rotation_matrix(const double* ra, const double* rb, double T[4][4]) {
  double x = rb[0] - ra[0], y = rb[1] - ra[1], z = rb[2] - ra[2];
  double r = sqrt(x * x + y * y + z * z);
  double rxy = sqrt(x * x + y * y);
  double cb = z / r, sb = rxy / r;
  double ca = 1.0, sa = 0.0;
  if (!(x == 0.0 && y == 0.0)) { ca = x / rxy; sa = y / rxy; }
  memset(T, 0, sizeof(double) * 16);
  T[ORB_S][ORB_S] = 1.0;
  T[ORB_PY][ORB_PY] = ca;  T[ORB_PY][ORB_PZ] = sa * sb; T[ORB_PY][ORB_PX] = sa * cb;
  T[ORB_PZ][ORB_PY] = 0.0; T[ORB_PZ][ORB_PZ] = cb;      T[ORB_PZ][ORB_PX] = -sb;
  T[ORB_PX][ORB_PY] = -sa; T[ORB_PX][ORB_PZ] = ca * sb; T[ORB_PX][ORB_PX] = ca * cb;
}

/* ------------------------------------------------------------------------ */
/* Multipole-multipole interactions (Dewar & Thiel 1977, Eqs. 52-65)         */
/* ------------------------------------------------------------------------ */
enum { MQ = 0, MUX, MUY, MUZ, QXX, QYY, QZZ, QXZ, QYZ, QXY, MP_NONE };
static int mp_l(int m) { return m == MQ ? 0 : (m <= MUZ ? 1 : 2); }

static double iv(double x) { return 1.0 / sqrt(x); }

/* [ma on A | mb on B], R along +z from A to B; da, db charge separations of the
 * two multipoles, a2 = (rho_A + rho_B)^2. */
static double mp_int(int ma, int mb, double R, double da, double db, double a2) {
  double R2 = R * R;
  switch (ma) {
    case MQ:
      switch (mb) {
        case MQ: return iv(R2 + a2);
        case MUZ: return 0.5 * iv((R + db) * (R + db) + a2) - 0.5 * iv((R - db) * (R - db) + a2);
        case QXX: case QYY: return 0.5 * iv(R2 + 4 * db * db + a2) - 0.5 * iv(R2 + a2);
        case QZZ:
          return 0.25 * iv((R + 2 * db) * (R + 2 * db) + a2) - 0.5 * iv(R2 + a2)
               + 0.25 * iv((R - 2 * db) * (R - 2 * db) + a2);
        default: return 0.0;
      }
    case MUX: case MUY:
      if (mb == ma) return 0.5 * iv(R2 + (da - db) * (da - db) + a2) - 0.5 * iv(R2 + (da + db) * (da + db) + a2);
      if ((ma == MUX && mb == QXZ) || (ma == MUY && mb == QYZ)) {
        double rm = (R - db) * (R - db), rp = (R + db) * (R + db);
        double dm = (da - db) * (da - db), dp = (da + db) * (da + db);
        return -0.25 * iv(rm + dm + a2) + 0.25 * iv(rm + dp + a2) + 0.25 * iv(rp + dm + a2) - 0.25 * iv(rp + dp + a2);
      }
      return 0.0;
    case MUZ:
      switch (mb) {
        case MQ: return -mp_int(MQ, MUZ, R, db, da, a2);
        case MUZ:
          return 0.25 * iv((R + da - db) * (R + da - db) + a2) - 0.25 * iv((R + da + db) * (R + da + db) + a2)
               - 0.25 * iv((R - da - db) * (R - da - db) + a2) + 0.25 * iv((R - da + db) * (R - da + db) + a2);
        case QXX: case QYY:
          return -0.25 * iv((R + da) * (R + da) + 4 * db * db + a2) + 0.25 * iv((R - da) * (R - da) + 4 * db * db + a2)
               + 0.25 * iv((R + da) * (R + da) + a2) - 0.25 * iv((R - da) * (R - da) + a2);
        case QZZ:
          return -0.125 * iv((R + da - 2 * db) * (R + da - 2 * db) + a2) + 0.125 * iv((R - da - 2 * db) * (R - da - 2 * db) + a2)
               - 0.125 * iv((R + da + 2 * db) * (R + da + 2 * db) + a2) + 0.125 * iv((R - da + 2 * db) * (R - da + 2 * db) + a2)
               + 0.25 * iv((R + da) * (R + da) + a2) - 0.25 * iv((R - da) * (R - da) + a2);
        default: return 0.0;
      }
    case QXX: case QYY:
      switch (mb) {
        case MQ: return mp_int(MQ, QXX, R, db, da, a2);
        case MUZ: return -mp_int(MUZ, QXX, R, db, da, a2);
        case QXX: case QYY:
          if (mb == ma)
            return 0.125 * iv(R2 + 4 * (da - db) * (da - db) + a2) + 0.125 * iv(R2 + 4 * (da + db) * (da + db) + a2)
                 - 0.25 * iv(R2 + 4 * da * da + a2) - 0.25 * iv(R2 + 4 * db * db + a2) + 0.25 * iv(R2 + a2);
          return 0.25 * iv(R2 + 4 * da * da + 4 * db * db + a2) - 0.25 * iv(R2 + 4 * da * da + a2)
               - 0.25 * iv(R2 + 4 * db * db + a2) + 0.25 * iv(R2 + a2);
        case QZZ:
          return 0.125 * iv((R - 2 * db) * (R - 2 * db) + 4 * da * da + a2) + 0.125 * iv((R + 2 * db) * (R + 2 * db) + 4 * da * da + a2)
               - 0.125 * iv((R - 2 * db) * (R - 2 * db) + a2) - 0.125 * iv((R + 2 * db) * (R + 2 * db) + a2)
               - 0.25 * iv(R2 + 4 * da * da + a2) + 0.25 * iv(R2 + a2);
        default: return 0.0;
      }
    case QZZ:
      switch (mb) {
        case MQ: return mp_int(MQ, QZZ, R, db, da, a2);
        case MUZ: return -mp_int(MUZ, QZZ, R, db, da, a2);
        case QXX: case QYY: return mp_int(QXX, QZZ, R, db, da, a2);
        case QZZ:
          return 0.0625 * (iv((R + 2 * da - 2 * db) * (R + 2 * da - 2 * db) + a2) + iv((R + 2 * da + 2 * db) * (R + 2 * da + 2 * db) + a2)
                         + iv((R - 2 * da - 2 * db) * (R - 2 * da - 2 * db) + a2) + iv((R - 2 * da + 2 * db) * (R - 2 * da + 2 * db) + a2))
               - 0.125 * (iv((R + 2 * da) * (R + 2 * da) + a2) + iv((R - 2 * da) * (R - 2 * da) + a2)
                        + iv((R + 2 * db) * (R + 2 * db) + a2) + iv((R - 2 * db) * (R - 2 * db) + a2))
               + 0.25 * iv(R2 + a2);
        default: return 0.0;
      }
    case QXZ: case QYZ:
      if ((ma == QXZ && mb == MUX) || (ma == QYZ && mb == MUY)) return -mp_int(mb, ma, R, db, da, a2);
      if (mb == ma) {
        double p1 = (R + da - db) * (R + da - db), p2 = (R + da + db) * (R + da + db);
        double p3 = (R - da - db) * (R - da - db), p4 = (R - da + db) * (R - da + db);
        double dm = (da - db) * (da - db), dp = (da + db) * (da + db);
        return 0.125 * (iv(p1 + dm + a2) - iv(p1 + dp + a2) - iv(p2 + dm + a2) + iv(p2 + dp + a2)
                      - iv(p3 + dm + a2) + iv(p3 + dp + a2) + iv(p4 + dm + a2) - iv(p4 + dp + a2));
      }
      return 0.0;
    default:
      return 0.0;
  }
}

/* multipoles of the charge distribution mu*nu on one atom (local frame) */
static int decompose(int mu, int nu, int* out) {
  if (mu > nu) { int t = mu; mu = nu; nu = t; }
  if (mu == ORB_S && nu == ORB_S) { out[0] = MQ; return 1; }
  if (mu == ORB_S) { out[0] = (nu == ORB_PX) ? MUX : (nu == ORB_PY) ? MUY : MUZ; return 1; }
  if (mu == nu) { out[0] = MQ; out[1] = (mu == ORB_PX) ? QXX : (mu == ORB_PY) ? QYY : QZZ; return 2; }
  /* two different p orbitals: py(1) < pz(2) < px(3) */
  if (mu == ORB_PY && nu == ORB_PZ) { out[0] = QYZ; return 1; }
  if (mu == ORB_PZ && nu == ORB_PX) { out[0] = QXZ; return 1; }
  out[0] = QXY; return 1;   /* py, px */
}

static double local_eri(int mu, int nu, int la, int si, double R,
                        const oracle_atom* A, const oracle_atom* B) {
  int ma[2], mb[2];
  int na = decompose(mu, nu, ma), nb = decompose(la, si, mb);
  if (na == 1 && nb == 1 && ma[0] == QXY && mb[0] == QXY) {
    /* (px py|px py) = 1/2 [(px px|px px) - (px px|py py)]  (DT 1977 Eq. 49) */
    return 0.5 * (local_eri(ORB_PX, ORB_PX, ORB_PX, ORB_PX, R, A, B) - local_eri(ORB_PX, ORB_PX, ORB_PY, ORB_PY, R, A, B));
  }
  double v = 0.0;
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) {
      if (ma[i] == QXY || mb[j] == QXY) continue;
      int la_ = mp_l(ma[i]), lb_ = mp_l(mb[j]);
      double rr = A->rho[la_] + B->rho[lb_];
      v += mp_int(ma[i], mb[j], R, A->d[la_], B->d[lb_], rr * rr);
    }
  return v;
}

/* ------------------------------------------------------------------------ */
/* Pair quantities                                                          */
/* ------------------------------------------------------------------------ */
static const int kind_of_local[4] = {0, 2, 1, 2};  /* s, py (pi), pz (sigma), px (pi) */

/* space-frame overlap block S[mu][nu] (mu on A, nu on B) */
static void pair_overlap(const oracle_atom* A, const double* ra,
                         const oracle_atom* B, const double* rb, double S[4][4]) {
  double T[4][4], L[4][4];
  double x = rb[0] - ra[0], y = rb[1] - ra[1], z = rb[2] - ra[2];
  double R = sqrt(x * x + y * y + z * z);
  rotation_matrix(ra, rb, T);
  memset(L, 0, sizeof(L));
  for (int i = 0; i < A->n_ao; ++i)
    for (int j = 0; j < B->n_ao; ++j) {
      if (kind_of_local[i] == 2 || kind_of_local[j] == 2) {
        if (i != j) continue;
      }
      L[i][j] = oracle_sto_overlap_local(A->principal_n, kind_of_local[i], A->zeta[i == 0 ? 0 : 1],
                                         B->principal_n, kind_of_local[j], B->zeta[j == 0 ? 0 : 1], R);
    }
  for (int m = 0; m < 4; ++m)
    for (int n = 0; n < 4; ++n) {
      double s = 0.0;
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) s += T[m][i] * L[i][j] * T[n][j];
      S[m][n] = (m < A->n_ao && n < B->n_ao) ? s : 0.0;
    }
}

/* space-frame (mu nu|la si) block, mu,nu on A and la,si on B; 256 doubles */
static void pair_eri(const oracle_atom* A, const double* ra,
                     const oracle_atom* B, const double* rb, double W[4][4][4][4]) {
  double T[4][4], L[4][4][4][4], tmp[4][4][4][4];
  double x = rb[0] - ra[0], y = rb[1] - ra[1], z = rb[2] - ra[2];
  double R = sqrt(x * x + y * y + z * z);
  int nA = A->n_ao, nB = B->n_ao;
  memset(L, 0, sizeof(L));
  for (int i = 0; i < nA; ++i)
    for (int j = 0; j < nA; ++j)
      for (int k = 0; k < nB; ++k)
        for (int l = 0; l < nB; ++l) L[i][j][k][l] = local_eri(i, j, k, l, R, A, B);
  rotation_matrix(ra, rb, T);
  /* four one-index transforms */
  for (int a = 0; a < 4; ++a) for (int j = 0; j < 4; ++j) for (int k = 0; k < 4; ++k) for (int l = 0; l < 4; ++l) {
    double s = 0; for (int i = 0; i < 4; ++i) s += T[a][i] * L[i][j][k][l]; tmp[a][j][k][l] = s; }
  for (int a = 0; a < 4; ++a) for (int b = 0; b < 4; ++b) for (int k = 0; k < 4; ++k) for (int l = 0; l < 4; ++l) {
    double s = 0; for (int j = 0; j < 4; ++j) s += T[b][j] * tmp[a][j][k][l]; L[a][b][k][l] = s; }
  for (int a = 0; a < 4; ++a) for (int b = 0; b < 4; ++b) for (int c = 0; c < 4; ++c) for (int l = 0; l < 4; ++l) {
    double s = 0; for (int k = 0; k < 4; ++k) s += T[c][k] * L[a][b][k][l]; tmp[a][b][c][l] = s; }
  for (int a = 0; a < 4; ++a) for (int b = 0; b < 4; ++b) for (int c = 0; c < 4; ++c) for (int d = 0; d < 4; ++d) {
    double s = 0; for (int l = 0; l < 4; ++l) s += T[d][l] * tmp[a][b][c][l];
    W[a][b][c][d] = (a < nA && b < nA && c < nB && d < nB) ? s : 0.0; }
}

static int is_n_or_o(const oracle_atom* p) { return p->atomic_number == 7 || p->atomic_number == 8; }

/* E_AB; sssS = (s_A s_A | s_B s_B) */
static double pair_core_core(int theory, const oracle_atom* A, const oracle_atom* B, double R, double ssss) {
  double f;
  if (A->atomic_number == 1 && is_n_or_o(B))
    f = 1.0 + (R / g_ang2au) * exp(-B->alpha * R) + exp(-A->alpha * R);
  else if (B->atomic_number == 1 && is_n_or_o(A))
    f = 1.0 + (R / g_ang2au) * exp(-A->alpha * R) + exp(-B->alpha * R);
  else
    f = 1.0 + exp(-A->alpha * R) + exp(-B->alpha * R);
  double e = A->core_charge * B->core_charge * ssss * f;
  if (theory != ORACLE_MNDO) {
    double t = 0.0;
    for (int i = 0; i < 4; ++i) {
      t += A->gk[i] * exp(-A->gl[i] * pow(R - A->gm[i], 2.0));
      t += B->gk[i] * exp(-B->gl[i] * pow(R - B->gm[i], 2.0));
    }
    e += A->core_charge * B->core_charge * t * g_ang2au / R;
  }
  if (theory == ORACLE_PM3PDDG) {
    /* Pm3Pddg::GetDiatomCoreRepulsionEnergy, src/pm3/Pm3Pddg.cpp:143-165, 239-245 */
    int na = (int)A->core_charge, nb = (int)B->core_charge;
    double temp = 0.0;
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        temp += ((double)na * A->pddg_pa[i] + (double)nb * B->pddg_pa[j]) *
                exp(-10.0 / (g_ang2au * g_ang2au) * pow(R - A->pddg_da[i] - B->pddg_da[j], 2.0));
    e += temp / (na + nb);
  }
  return e;
}

/* ------------------------------------------------------------------------ */
/* Exported API (ctypes)                                                    */
/* ------------------------------------------------------------------------ */

static int fill_params(int theory, int natoms, const int* Z, oracle_atom* P, int* first) {
  int n = 0;
  for (int a = 0; a < natoms; ++a) {
    if (oracle_fill(theory, Z[a], &P[a]) != 0) return -1;
    first[a] = n;
    n += P[a].n_ao;
  }
  return n;
}

int oracle_num_aos(int theory, int natoms, const int* Z) {
  int n = 0;
  for (int a = 0; a < natoms; ++a) {
    oracle_atom p;
    if (oracle_fill(theory, Z[a], &p) != 0) return -1;
    n += p.n_ao;
  }
  return n;
}

/* Builds the overlap matrix S (N x N), the space-frame pair integrals
 * eri[pair][4][4][4][4] for pairs a < b in row-major pair order, and the
 * core-core energy.  Returns N or a negative error. */
int oracle_integrals(int theory, int natoms, const int* Z, const double* xyz,
                     double* S, double* eri, double* ecore) {
  oracle_atom* P = (oracle_atom*)malloc(sizeof(oracle_atom) * (natoms > 0 ? natoms : 1));
  int* first = (int*)malloc(sizeof(int) * (natoms > 0 ? natoms : 1));
  int N = fill_params(theory, natoms, Z, P, first);
  if (N < 0) { free(P); free(first); return -1; }
  memset(S, 0, sizeof(double) * (size_t)N * N);
  for (int m = 0; m < N; ++m) S[(size_t)m * N + m] = 1.0;
  double ec = 0.0;
  size_t pair = 0;
  for (int a = 0; a < natoms; ++a)
    for (int b = a + 1; b < natoms; ++b, ++pair) {
      const double* ra = xyz + 3 * a; const double* rb = xyz + 3 * b;
      double Sab[4][4];
      pair_overlap(&P[a], ra, &P[b], rb, Sab);
      for (int m = 0; m < P[a].n_ao; ++m)
        for (int n = 0; n < P[b].n_ao; ++n) {
          S[(size_t)(first[a] + m) * N + first[b] + n] = Sab[m][n];
          S[(size_t)(first[b] + n) * N + first[a] + m] = Sab[m][n];
        }
      double (*W)[4][4][4] = (double (*)[4][4][4])(eri + pair * 256);
      pair_eri(&P[a], ra, &P[b], rb, W);
      double dx = rb[0] - ra[0], dy = rb[1] - ra[1], dz = rb[2] - ra[2];
      double R = sqrt(dx * dx + dy * dy + dz * dz);
      ec += pair_core_core(theory, &P[a], &P[b], R, W[0][0][0][0]);
    }
  *ecore = ec;
  free(P); free(first);
  return N;
}

/* Environmental point charges (MolDS EPC).  For every atom A and point
 * charge (x, y, z, q): V[mu][nu] += -q (mu nu|s s)_{A,EPC} on A's one-centre
 * block, the integral taken as for an atom pair with the EPC an s-only centre
 * (src/base/atoms/mm/EnvironmentalPointCharge.cpp:29-35) and both rho set to
 * zero (src/mndo/Mndo.cpp:3822-3935, 6602-6613); the Fock matrix gets V in
 * every non-guess build (Mndo.cpp:474-484, 546-556).  *ecore_epc = sum
 * Z_A q / R (Mndo.cpp:329-331, src/cndo/Cndo2.cpp:418-426).  V is N x N and
 * is added to.  Returns N or a negative error. */
int oracle_epc(int theory, int natoms, const int* Z, const double* xyz, int nepc, const double* epc,
               double* V, double* ecore_epc) {
  oracle_atom* P = (oracle_atom*)malloc(sizeof(oracle_atom) * (natoms > 0 ? natoms : 1));
  int* first = (int*)malloc(sizeof(int) * (natoms > 0 ? natoms : 1));
  int N = fill_params(theory, natoms, Z, P, first);
  if (N < 0) { free(P); free(first); return -1; }
  oracle_atom pc;
  memset(&pc, 0, sizeof(pc));
  pc.n_ao = 1;
  double e = 0.0;
  for (int a = 0; a < natoms; ++a) {
    oracle_atom A = P[a];
    A.rho[0] = A.rho[1] = A.rho[2] = 0.0;
    const double* ra = xyz + 3 * a;
    for (int i = 0; i < nepc; ++i) {
      const double* rp = epc + 4 * i;
      const double q = rp[3];
      double W[4][4][4][4];
      pair_eri(&A, ra, &pc, rp, W);
      for (int m = 0; m < A.n_ao; ++m)
        for (int n = 0; n < A.n_ao; ++n)
          V[(size_t)(first[a] + m) * N + first[a] + n] += -1.0 * q * W[m][n][0][0];
      double dx = rp[0] - ra[0], dy = rp[1] - ra[1], dz = rp[2] - ra[2];
      e += A.core_charge * q / sqrt(dx * dx + dy * dy + dz * dz);
    }
  }
  *ecore_epc = e;
  free(P); free(first);
  return N;
}

static double coulomb1(const oracle_atom* p, int m, int n) {
  if (m == 0 && n == 0) return p->gss;
  if (m == 0 || n == 0) return p->gsp;
  return (m == n) ? p->gpp : p->gp2;
}
static double exchange1(const oracle_atom* p, int m, int n) {
  if (m == n) return coulomb1(p, m, n);
  if (m == 0 || n == 0) return p->hsp;
  return p->hpp;
}

/* F (N x N, full symmetric) from density P.  guess != 0 gives the MolDS guess
 * Fock (U on the diagonal, 1/2(beta_mu + beta_nu) S_mu,nu between atoms). */
int oracle_fock(int theory, int natoms, const int* Z, const double* S, const double* eri,
                const double* Pd, int guess, double* F) {
  oracle_atom* P = (oracle_atom*)malloc(sizeof(oracle_atom) * (natoms > 0 ? natoms : 1));
  int* first = (int*)malloc(sizeof(int) * (natoms > 0 ? natoms : 1));
  int N = fill_params(theory, natoms, Z, P, first);
  if (N < 0) { free(P); free(first); return -1; }
  memset(F, 0, sizeof(double) * (size_t)N * N);
#define PD(i, j) Pd[(size_t)(i) * N + (j)]
#define FF(i, j) F[(size_t)(i) * N + (j)]
  /* one-centre terms */
  for (int a = 0; a < natoms; ++a) {
    int fa = first[a], na = P[a].n_ao;
    for (int m = 0; m < na; ++m) {
      FF(fa + m, fa + m) = P[a].u[m == 0 ? 0 : 1];
      if (guess) continue;
      double t = 0.0;
      for (int n = 0; n < na; ++n) t += PD(fa + n, fa + n) * (coulomb1(&P[a], m, n) - 0.5 * exchange1(&P[a], m, n));
      FF(fa + m, fa + m) += t;
      for (int n = 0; n < na; ++n)
        if (n != m) FF(fa + m, fa + n) += (1.5 * exchange1(&P[a], m, n) - 0.5 * coulomb1(&P[a], m, n)) * PD(fa + m, fa + n);
    }
  }
  /* two-centre terms */
  size_t pair = 0;
  for (int a = 0; a < natoms; ++a)
    for (int b = a + 1; b < natoms; ++b, ++pair) {
      const double (*W)[4][4][4] = (const double (*)[4][4][4])(eri + pair * 256);
      int fa = first[a], fb = first[b], na = P[a].n_ao, nb = P[b].n_ao;
      for (int m = 0; m < na; ++m)
        for (int n = 0; n < nb; ++n) {
          double v = 0.5 * (P[a].beta[m == 0 ? 0 : 1] + P[b].beta[n == 0 ? 0 : 1]) * S[(size_t)(fa + m) * N + fb + n];
          if (!guess) {
            for (int s = 0; s < na; ++s)
              for (int l = 0; l < nb; ++l) v -= 0.5 * PD(fa + s, fb + l) * W[m][s][n][l];
          }
          FF(fa + m, fb + n) += v;
          FF(fb + n, fa + m) += v;
        }
      if (guess) continue;
      /* Coulomb + electron-core on A from B */
      for (int m = 0; m < na; ++m)
        for (int n = 0; n < na; ++n) {
          double t = 0.0;
          for (int l = 0; l < nb; ++l)
            for (int s = 0; s < nb; ++s) t += PD(fb + l, fb + s) * W[m][n][l][s];
          t -= P[b].core_charge * W[m][n][0][0];
          FF(fa + m, fa + n) += t;
        }
      /* Coulomb + electron-core on B from A */
      for (int l = 0; l < nb; ++l)
        for (int s = 0; s < nb; ++s) {
          double t = 0.0;
          for (int m = 0; m < na; ++m)
            for (int n = 0; n < na; ++n) t += PD(fa + m, fa + n) * W[m][n][l][s];
          t -= P[a].core_charge * W[0][0][l][s];
          FF(fb + l, fb + s) += t;
        }
    }
#undef PD
#undef FF
  free(P); free(first);
  return N;
}

/* per-atom parameters needed by the Python driver: core charge, n_ao,
 * E_atom and dHf_atom (MNDO).  out has 4 doubles per atom. */
int oracle_atom_info(int theory, int natoms, const int* Z, double* out) {
  for (int a = 0; a < natoms; ++a) {
    oracle_atom p;
    if (oracle_fill(theory, Z[a], &p) != 0) return -1;
    out[4 * a + 0] = p.core_charge;
    out[4 * a + 1] = p.n_ao;
    out[4 * a + 2] = p.e_atom;
    out[4 * a + 3] = p.dhf_atom;
  }
  return 0;
}

/* Charge separations D_0..D_2 and additive terms rho_0..rho_2 of one
 * element's multipoles (out[0..5]), as the pair integrals use them. */
int oracle_multipole_params(int theory, int Z, double* out) {
  oracle_atom p;
  if (oracle_fill(theory, Z, &p) != 0) return -1;
  for (int l = 0; l < 3; ++l) { out[l] = p.d[l]; out[3 + l] = p.rho[l]; }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Cartesian (dipole) matrix <mu| r_k |nu> by the STO-6G expansion           */
/* ------------------------------------------------------------------------ */

/* axis of each orbital in MolDS's order (s, py, pz, px); -1 for s */
static const int axis_of_orb[4] = {-1, 1, 2, 0};

/* (s_A|s_B) of two normalised s Gaussians (Cndo2.cpp:4563-4575) */
static double gto_sasb(double a, double b, double R) {
  double t1 = 2.0 * sqrt(a * b) / (a + b);
  double t2 = -1.0 * (a * b) / (a + b);
  return t1 * sqrt(t1) * exp(t2 * R * R);
}

/* Overlap of normalised s / p Gaussians, p given by its axis (-1 = s);
 * d = A - B (Cndo2.cpp:4601-5153, the s and p cases). */
static double gto_overlap(int ia, double a, int ib, double b, const double* d, double sasb) {
  double p = a + b, ab = a * b, v;
  if (ia < 0 && ib < 0) v = 1.0;
  else if (ia < 0) v = 2.0 * a * sqrt(b) * d[ib] / p;
  else if (ib < 0) v = -2.0 * sqrt(a) * b * d[ia] / p;
  else if (ia == ib) v = 4.0 * sqrt(ab) / p * (-1.0 * (d[ia] * d[ia]) * ab / p + 0.5);
  else v = -4.0 * ab * sqrt(ab) / (p * p) * d[ia] * d[ib];
  return v * sasb;
}

/* <g_A| r_k |g_B> of normalised s / p Gaussians in absolute coordinates
 * (Cndo2.cpp:2149-2400, the s and p cases). */
static double gto_cartesian(int ia, double a, const double* ra, int ib, double b, const double* rb,
                            int k, double sasb) {
  const double p = a + b, ab = a * b;
  const double d[3] = {ra[0] - rb[0], ra[1] - rb[1], ra[2] - rb[2]};
  if (ia < 0 && ib < 0) return (a * ra[k] + b * rb[k]) / p * sasb;
  if (ia < 0)   /* r_k g_s(A) = g_pk(A) / (2 sqrt a) + A_k g_s(A) */
    return gto_overlap(k, a, ib, b, d, sasb) / (2.0 * sqrt(a)) + ra[k] * gto_overlap(-1, a, ib, b, d, sasb);
  if (ib < 0)
    return gto_overlap(ia, a, k, b, d, sasb) / (2.0 * sqrt(b)) + rb[k] * gto_overlap(ia, a, -1, b, d, sasb);
  const double f = 4.0 * sqrt(ab) / (p * p);
  if (ia == ib && k == ia) {
    double t1 = a * ra[k] + b * rb[k], t2 = a * ra[k] - a * rb[k], t3 = b * ra[k] - b * rb[k];
    return (0.5 * (t1 + t2 - t3) - t1 * t2 * t3 / p) * f * sasb;
  }
  if (ia == ib) {
    double t1 = a * ra[ia] - a * rb[ia], t2 = b * ra[ia] - b * rb[ia];
    return (0.5 - t1 * t2 / p) * (a * ra[k] + b * rb[k]) * f * sasb;
  }
  if (k == ib) {
    double t1 = a * ra[k] + b * rb[k], t2 = a * ra[k] - a * rb[k];
    return (0.5 + t1 * t2 / p) * (b * ra[ia] - b * rb[ia]) * (-f) * sasb;
  }
  if (k == ia) {
    double t1 = a * ra[k] + b * rb[k], t2 = b * ra[k] - b * rb[k];
    return (0.5 - t1 * t2 / p) * (a * ra[ib] - a * rb[ib]) * f * sasb;
  }
  {
    double t1 = b * ra[ia] - b * rb[ia], t2 = a * ra[k] + b * rb[k], t3 = a * ra[ib] - a * rb[ib];
    return -f / p * (t1 * t2 * t3) * sasb;
  }
}

/* X[3][N][N]: every AO pair, same atom included, each element summed over the
 * 6 x 6 primitive pairs (Cndo2.cpp:1946-2057, 2068-2130).  Returns N. */
int oracle_cartesian(int theory, int natoms, const int* Z, const double* xyz, double* X) {
  oracle_atom* P = (oracle_atom*)malloc(sizeof(oracle_atom) * (natoms > 0 ? natoms : 1));
  int* first = (int*)malloc(sizeof(int) * (natoms > 0 ? natoms : 1));
  int N = fill_params(theory, natoms, Z, P, first);
  if (N < 0) { free(P); free(first); return -1; }
  const size_t NN = (size_t)N * N;
  for (int A = 0; A < natoms; ++A)
    for (int B = 0; B < natoms; ++B) {
      const double* ra = xyz + 3 * A; const double* rb = xyz + 3 * B;
      const double dx = ra[0] - rb[0], dy = ra[1] - rb[1], dz = ra[2] - rb[2];
      const double R = sqrt(dx * dx + dy * dy + dz * dz);
      const int shA = P[A].principal_n - 1, shB = P[B].principal_n - 1;
      for (int mu = 0; mu < P[A].n_ao; ++mu)
        for (int nu = 0; nu < P[B].n_ao; ++nu) {
          const int la = mu == 0 ? 0 : 1, lb = nu == 0 ? 0 : 1;
          const double zA = P[A].zeta[la], zB = P[B].zeta[lb];
          double acc[3] = {0.0, 0.0, 0.0};
          for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
              const double c = g_sto_coef[shA][la][i] * g_sto_coef[shB][lb][j];
              const double a = (zA * zA) * g_sto_exp[shA][la][i];
              const double b = (zB * zB) * g_sto_exp[shB][lb][j];
              const double sasb = gto_sasb(a, b, R);
              for (int k = 0; k < 3; ++k)
                acc[k] += c * gto_cartesian(axis_of_orb[mu], a, ra, axis_of_orb[nu], b, rb, k, sasb);
            }
          const size_t e = (size_t)(first[A] + mu) * N + first[B] + nu;
          for (int k = 0; k < 3; ++k) X[k * NN + e] = acc[k];
        }
    }
  free(P); free(first);
  return N;
}

/* Core mass of every atom: atomic mass [a.u.] - valence electrons
 * (src/base/atoms/Atom.h:34). */
int oracle_core_masses(int theory, int natoms, const int* Z, double* out) {
  for (int a = 0; a < natoms; ++a) {
    oracle_atom p;
    if (oracle_fill(theory, Z[a], &p) != 0) return -1;
    out[a] = p.core_mass;
  }
  return 0;
}

/* Dispersion data of every atom: C6 [a.u.] and van der Waals radius [bohr]
 * (src/base/atoms/<El>atom.cpp, e.g. Catom.cpp:60-63); 2 doubles per atom. */
int oracle_vdw_params(int theory, int natoms, const int* Z, double* out) {
  for (int a = 0; a < natoms; ++a) {
    oracle_atom p;
    if (oracle_fill(theory, Z[a], &p) != 0) return -1;
    out[2 * a] = p.vdw_c6;
    out[2 * a + 1] = p.vdw_r0;
  }
  return 0;
}

