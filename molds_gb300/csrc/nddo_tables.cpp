// Host construction of the constant tables used by the pair kernel.
//
// (1) EriTable: each distinct local two-centre integral of Dewar & Thiel (1977)
//     as a flat list of point-charge terms.  The multipole-multipole
//     interactions are Eqs. 52-65 of that paper as MolDS writes them in
//     src/mndo/Mndo.cpp:6592-6834; the charge-distribution decomposition of
//     each integral is Eqs. 29-48 (Mndo.cpp:4911-5223).  An interaction with
//     the two atoms swapped (e.g. [mu_z, q] = -[q, mu_z] with A and B
//     exchanged, Mndo.cpp:6631-6634) is emitted by swapping the D/rho roles of
//     the terms and, where MolDS negates, the coefficients.
// (2) OverlapTable: polynomial coefficients of the Slater-orbital overlap in
//     prolate-spheroidal coordinates (my own expansion; MolDS uses Pople's
//     tabulated reduced-overlap coefficients, src/cndo/Cndo2.cpp:6185-6221).
#include "nddo_tables.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace nddo {

namespace {

enum Mp { MQ, MUX, MUY, MUZ, QXX, QYY, QZZ, QXZ, QYZ };
int mp_l(int m) { return m == MQ ? 0 : (m <= MUZ ? 1 : 2); }

struct T6 { double coef; int c1, c2, c3, c4, c5, c6; };

// [ma on A | mb on B] in the orientation where A is the first atom
std::vector<T6> interaction(int ma, int mb);

std::vector<T6> swapped(const std::vector<T6>& v, double sign) {
  std::vector<T6> out;
  for (const T6& t : v) out.push_back({sign * t.coef, t.c2, t.c1, t.c4, t.c3, t.c6, t.c5});
  return out;
}

std::vector<T6> interaction(int ma, int mb) {
  // Eq. 52
  if (ma == MQ && mb == MQ) return {{1.0, 0, 0, 0, 0, 0, 0}};
  // Eq. 53
  if (ma == MQ && mb == MUZ) return {{0.5, 0, 1, 0, 0, 0, 0}, {-0.5, 0, -1, 0, 0, 0, 0}};
  if (ma == MUZ && mb == MQ) return swapped(interaction(MQ, MUZ), -1.0);
  // Eq. 54
  if (ma == MQ && (mb == QXX || mb == QYY)) return {{0.5, 0, 0, 0, 2, 0, 0}, {-0.5, 0, 0, 0, 0, 0, 0}};
  if ((ma == QXX || ma == QYY) && mb == MQ) return swapped(interaction(MQ, QXX), 1.0);
  // Eq. 55
  if (ma == MQ && mb == QZZ)
    return {{0.25, 0, 2, 0, 0, 0, 0}, {-0.5, 0, 0, 0, 0, 0, 0}, {0.25, 0, -2, 0, 0, 0, 0}};
  if (ma == QZZ && mb == MQ) return swapped(interaction(MQ, QZZ), 1.0);
  // Eq. 56
  if ((ma == MUX && mb == MUX) || (ma == MUY && mb == MUY))
    return {{0.5, 0, 0, 1, -1, 0, 0}, {-0.5, 0, 0, 1, 1, 0, 0}};
  // Eq. 57
  if (ma == MUZ && mb == MUZ)
    return {{0.25, 1, -1, 0, 0, 0, 0}, {-0.25, 1, 1, 0, 0, 0, 0},
            {-0.25, -1, -1, 0, 0, 0, 0}, {0.25, -1, 1, 0, 0, 0, 0}};
  // Eq. 58
  if ((ma == MUX && mb == QXZ) || (ma == MUY && mb == QYZ))
    return {{-0.25, 0, -1, 1, -1, 0, 0}, {0.25, 0, -1, 1, 1, 0, 0},
            {0.25, 0, 1, 1, -1, 0, 0}, {-0.25, 0, 1, 1, 1, 0, 0}};
  if ((ma == QXZ && mb == MUX) || (ma == QYZ && mb == MUY)) return swapped(interaction(MUX, QXZ), -1.0);
  // Eq. 59
  if (ma == MUZ && (mb == QXX || mb == QYY))
    return {{-0.25, 1, 0, 0, 2, 0, 0}, {0.25, -1, 0, 0, 2, 0, 0},
            {0.25, 1, 0, 0, 0, 0, 0}, {-0.25, -1, 0, 0, 0, 0, 0}};
  if ((ma == QXX || ma == QYY) && mb == MUZ) return swapped(interaction(MUZ, QXX), -1.0);
  // Eq. 60
  if (ma == MUZ && mb == QZZ)
    return {{-0.125, 1, -2, 0, 0, 0, 0}, {0.125, -1, -2, 0, 0, 0, 0},
            {-0.125, 1, 2, 0, 0, 0, 0}, {0.125, -1, 2, 0, 0, 0, 0},
            {0.25, 1, 0, 0, 0, 0, 0}, {-0.25, -1, 0, 0, 0, 0, 0}};
  if (ma == QZZ && mb == MUZ) return swapped(interaction(MUZ, QZZ), -1.0);
  // Eq. 61
  if ((ma == QXX && mb == QXX) || (ma == QYY && mb == QYY))
    return {{0.125, 0, 0, 2, -2, 0, 0}, {0.125, 0, 0, 2, 2, 0, 0},
            {-0.25, 0, 0, 2, 0, 0, 0}, {-0.25, 0, 0, 0, 2, 0, 0}, {0.25, 0, 0, 0, 0, 0, 0}};
  // Eq. 62
  if ((ma == QXX && mb == QYY) || (ma == QYY && mb == QXX))
    return {{0.25, 0, 0, 2, 0, 0, 2}, {-0.25, 0, 0, 2, 0, 0, 0},
            {-0.25, 0, 0, 0, 2, 0, 0}, {0.25, 0, 0, 0, 0, 0, 0}};
  // Eq. 63
  if ((ma == QXX || ma == QYY) && mb == QZZ)
    return {{0.125, 0, -2, 2, 0, 0, 0}, {0.125, 0, 2, 2, 0, 0, 0},
            {-0.125, 0, -2, 0, 0, 0, 0}, {-0.125, 0, 2, 0, 0, 0, 0},
            {-0.25, 0, 0, 2, 0, 0, 0}, {0.25, 0, 0, 0, 0, 0, 0}};
  if (ma == QZZ && (mb == QXX || mb == QYY)) return swapped(interaction(QXX, QZZ), 1.0);
  // Eq. 64
  if (ma == QZZ && mb == QZZ)
    return {{0.0625, 2, -2, 0, 0, 0, 0}, {0.0625, 2, 2, 0, 0, 0, 0},
            {0.0625, -2, -2, 0, 0, 0, 0}, {0.0625, -2, 2, 0, 0, 0, 0},
            {-0.125, 2, 0, 0, 0, 0, 0}, {-0.125, -2, 0, 0, 0, 0, 0},
            {-0.125, 0, 2, 0, 0, 0, 0}, {-0.125, 0, -2, 0, 0, 0, 0},
            {0.25, 0, 0, 0, 0, 0, 0}};
  // Eq. 65
  if ((ma == QXZ && mb == QXZ) || (ma == QYZ && mb == QYZ))
    return {{0.125, 1, -1, 1, -1, 0, 0}, {-0.125, 1, -1, 1, 1, 0, 0},
            {-0.125, 1, 1, 1, -1, 0, 0}, {0.125, 1, 1, 1, 1, 0, 0},
            {-0.125, -1, -1, 1, -1, 0, 0}, {0.125, -1, -1, 1, 1, 0, 0},
            {0.125, -1, 1, 1, -1, 0, 0}, {-0.125, -1, 1, 1, 1, 0, 0}};
  return {};
}

void add_interaction(EriTable& t, int slot, int ma, int mb) {
  for (const T6& x : interaction(ma, mb)) {
    int n = t.nterms[slot]++;
    EriTerm& e = t.terms[slot][n];
    e.coef = x.coef;
    e.la = (signed char)mp_l(ma);
    e.lb = (signed char)mp_l(mb);
    e.c1 = (signed char)x.c1; e.c2 = (signed char)x.c2; e.c3 = (signed char)x.c3;
    e.c4 = (signed char)x.c4; e.c5 = (signed char)x.c5; e.c6 = (signed char)x.c6;
  }
}

// polynomial in (xi, eta)
struct Poly { double c[kOvDeg][kOvDeg]; };
Poly poly_one() { Poly p; std::memset(&p, 0, sizeof(p)); p.c[0][0] = 1; return p; }
Poly poly_mul(const Poly& a, const Poly& b) {
  Poly r; std::memset(&r, 0, sizeof(r));
  for (int i = 0; i < kOvDeg; ++i)
    for (int j = 0; j < kOvDeg; ++j) {
      if (a.c[i][j] == 0) continue;
      for (int k = 0; i + k < kOvDeg; ++k)
        for (int l = 0; j + l < kOvDeg; ++l) r.c[i + k][j + l] += a.c[i][j] * b.c[k][l];
    }
  return r;
}
Poly lin(double c0, double cx, double ce, double cxe, double cxx, double cee) {
  Poly p; std::memset(&p, 0, sizeof(p));
  p.c[0][0] = c0; p.c[1][0] = cx; p.c[0][1] = ce; p.c[1][1] = cxe; p.c[2][0] = cxx; p.c[0][2] = cee;
  return p;
}

// kind: 0 s, 1 p-sigma, 2 p-pi
Poly overlap_poly(int na, int kinda, int nb, int kindb) {
  Poly pa = poly_one(), pb = poly_one();
  int ea = kinda == 0 ? na - 1 : na - 2;
  int eb = kindb == 0 ? nb - 1 : nb - 2;
  for (int i = 0; i < ea; ++i) pa = poly_mul(pa, lin(0, 1, 1, 0, 0, 0));    // xi + eta
  for (int i = 0; i < eb; ++i) pb = poly_mul(pb, lin(0, 1, -1, 0, 0, 0));   // xi - eta
  if (kinda == 1) pa = poly_mul(pa, lin(1, 0, 0, 1, 0, 0));                 // 1 + xi eta
  if (kindb == 1) pb = poly_mul(pb, lin(-1, 0, 0, 1, 0, 0));                // xi eta - 1
  Poly p = poly_mul(pa, pb);
  if (kinda == 2 && kindb == 2) {
    p = poly_mul(p, lin(-1, 0, 0, 0, 1, 0));   // xi^2 - 1
    p = poly_mul(p, lin(1, 0, 0, 0, 0, -1));   // 1 - eta^2
  }
  return poly_mul(p, lin(0, 0, 0, 0, 1, -1));  // volume element xi^2 - eta^2
}

}  // namespace

void build_eri_table(EriTable* t) {
  std::memset(t, 0, sizeof(*t));
  // charge distributions: xx = q + Qxx, zz = q + Qzz, sz = mu_z, sx = mu_x, xz = Qxz
  add_interaction(*t, 0, MQ, MQ);
  add_interaction(*t, 1, MQ, MQ); add_interaction(*t, 1, MQ, QXX);
  add_interaction(*t, 2, MQ, MQ); add_interaction(*t, 2, MQ, QZZ);
  add_interaction(*t, 3, MQ, MQ); add_interaction(*t, 3, QXX, MQ);
  add_interaction(*t, 4, MQ, MQ); add_interaction(*t, 4, QZZ, MQ);
  add_interaction(*t, 5, MQ, MQ); add_interaction(*t, 5, MQ, QXX); add_interaction(*t, 5, QXX, MQ); add_interaction(*t, 5, QXX, QXX);
  add_interaction(*t, 6, MQ, MQ); add_interaction(*t, 6, MQ, QYY); add_interaction(*t, 6, QXX, MQ); add_interaction(*t, 6, QXX, QYY);
  add_interaction(*t, 7, MQ, MQ); add_interaction(*t, 7, MQ, QZZ); add_interaction(*t, 7, QXX, MQ); add_interaction(*t, 7, QXX, QZZ);
  add_interaction(*t, 8, MQ, MQ); add_interaction(*t, 8, MQ, QXX); add_interaction(*t, 8, QZZ, MQ); add_interaction(*t, 8, QZZ, QXX);
  add_interaction(*t, 9, MQ, MQ); add_interaction(*t, 9, MQ, QZZ); add_interaction(*t, 9, QZZ, MQ); add_interaction(*t, 9, QZZ, QZZ);
  add_interaction(*t, 10, MUZ, MQ);
  add_interaction(*t, 11, MUZ, MQ); add_interaction(*t, 11, MUZ, QXX);
  add_interaction(*t, 12, MUZ, MQ); add_interaction(*t, 12, MUZ, QZZ);
  add_interaction(*t, 13, MQ, MUZ);
  add_interaction(*t, 14, MQ, MUZ); add_interaction(*t, 14, QXX, MUZ);
  add_interaction(*t, 15, MQ, MUZ); add_interaction(*t, 15, QZZ, MUZ);
  add_interaction(*t, 16, MUX, MUX);
  add_interaction(*t, 17, MUZ, MUZ);
  add_interaction(*t, 18, MUX, QXZ);
  add_interaction(*t, 19, QXZ, MUX);
  add_interaction(*t, 20, QXZ, QXZ);
  // slot 21 = 1/2 [slot 5 - slot 6], evaluated after the term loops

  // local packed indices: 0 ss, 1 s-py, 2 s-pz, 3 s-px, 4 py-py, 5 py-pz, 6 py-px,
  // 7 pz-pz, 8 pz-px, 9 px-px (local x = px, y = py, z = pz)
  std::memset(t->slot_of, -1, sizeof(t->slot_of));
  auto set = [&](int P, int Q, int s) { t->slot_of[P][Q] = (signed char)s; };
  set(0, 0, 0);
  set(0, 9, 1); set(0, 4, 1);
  set(0, 7, 2);
  set(9, 0, 3); set(4, 0, 3);
  set(7, 0, 4);
  set(9, 9, 5); set(4, 4, 5);
  set(9, 4, 6); set(4, 9, 6);
  set(9, 7, 7); set(4, 7, 7);
  set(7, 9, 8); set(7, 4, 8);
  set(7, 7, 9);
  set(2, 0, 10);
  set(2, 9, 11); set(2, 4, 11);
  set(2, 7, 12);
  set(0, 2, 13);
  set(9, 2, 14); set(4, 2, 14);
  set(7, 2, 15);
  set(3, 3, 16); set(1, 1, 16);
  set(2, 2, 17);
  set(3, 8, 18); set(1, 5, 18);
  set(8, 3, 19); set(5, 1, 19);
  set(8, 8, 20); set(5, 5, 20);
  set(6, 6, 21);
}

void build_overlap_table(OverlapTable* t) {
  std::memset(t, 0, sizeof(*t));
  const int kinds[kNumOvCombos][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}, {2, 2}};
  const double s3 = std::sqrt(3.0);
  t->ang[0] = 0.5; t->ang[1] = 0.5 * s3; t->ang[2] = 0.5 * s3; t->ang[3] = 1.5; t->ang[4] = 0.75;
  for (int na = 1; na <= 3; ++na)
    for (int nb = 1; nb <= 3; ++nb)
      for (int c = 0; c < kNumOvCombos; ++c) {
        int ka = kinds[c][0], kb = kinds[c][1];
        if ((ka != 0 && na < 2) || (kb != 0 && nb < 2)) continue;
        Poly p = overlap_poly(na, ka, nb, kb);
        std::memcpy(t->coef[na - 1][nb - 1][c], p.c, sizeof(p.c));
        int n = 0, km = 0;
        for (int i = 0; i < kOvDeg; ++i)
          for (int j = 0; j < kOvDeg; ++j)
            if (p.c[i][j] != 0.0 && n < kOvMaxTerms) {
              t->ti[na - 1][nb - 1][c][n] = (unsigned char)i;
              t->tj[na - 1][nb - 1][c][n] = (unsigned char)j;
              t->tc[na - 1][nb - 1][c][n] = p.c[i][j];
              if (i > km) km = i;
              if (j > km) km = j;
              ++n;
            }
        t->nterms[na - 1][nb - 1][c] = n;
        t->kmax[na - 1][nb - 1][c] = km;
      }
}

}  // namespace nddo
