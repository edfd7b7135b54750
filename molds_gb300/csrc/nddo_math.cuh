// Per-pair NDDO mathematics shared by the pair kernel and its host-side tests.
//
// Everything here is __host__ __device__ so that the same code that runs in
// the pair kernel can be checked against the oracle on a CPU.
//
// Local (diatomic-frame) two-centre integrals follow Dewar & Thiel,
// Theor. Chim. Acta 46, 89 (1977), Eqs. 29-49 and 52-65, as MolDS evaluates
// them (src/mndo/Mndo.cpp:4886-5238, 6592-6834).  Instead of the reference's
// recursive case tree, every multipole-multipole interaction is expanded into
// a flat list of point-charge terms
//        coef / sqrt((R + c1 DA + c2 DB)^2 + (c3 DA + c4 DB)^2 + (c5 DA + c6 DB)^2 + (rhoA + rhoB)^2)
// built once on the host (nddo_tables.cpp); a lane of the pair kernel then
// evaluates one local integral as a uniform loop over its terms.
#pragma once
#include <cmath>
#include "nddo_units.h"

namespace nddo {

constexpr int kMaxTermsPerSlot = 24;
constexpr int kNumSlots = 22;     // distinct local integrals of an sp-sp pair

// one point-charge term of a local integral
struct EriTerm {
  double coef;
  signed char la, lb;             // multipole order (0,1,2) on A and B: selects D and rho
  signed char c1, c2, c3, c4, c5, c6;
};

// Local integral slot -> list of terms.  Slot numbering (x, y, z local p's):
//  0 (ss|ss)  1 (ss|xx)  2 (ss|zz)  3 (xx|ss)  4 (zz|ss)  5 (xx|xx)  6 (xx|yy)
//  7 (xx|zz)  8 (zz|xx)  9 (zz|zz) 10 (sz|ss) 11 (sz|xx) 12 (sz|zz) 13 (ss|sz)
// 14 (xx|sz) 15 (zz|sz) 16 (sx|sx) 17 (sz|sz) 18 (sx|xz) 19 (xz|sx) 20 (xz|xz)
// 21 (xy|xy) = 1/2 [(xx|xx) - (xx|yy)]
struct EriTable {
  int nterms[kNumSlots];
  EriTerm terms[kNumSlots][kMaxTermsPerSlot];
  // local packed 10x10 entry (mu<=nu on A, la<=si on B) -> slot (or -1 = zero)
  signed char slot_of[10][10];
};

// Overlap polynomial tables: S_local = norm * ang * (R/2)^(na+nb+1) *
//   sum_ij coef[i][j] A_i(p) B_j(q), p = R(za+zb)/2, q = R(za-zb)/2.
constexpr int kOvDeg = 12;
constexpr int kNumOvCombos = 5;   // ss, s-sigma, sigma-s, sigma-sigma, pi-pi
constexpr int kOvMaxTerms = 64;
struct OverlapTable {
  double coef[3][3][kNumOvCombos][kOvDeg][kOvDeg];   // [na-1][nb-1][combo][i][j]
  double ang[kNumOvCombos];
  // the same polynomials as compact lists of nonzero terms, and the highest
  // A / B index each needs (thread-per-pair evaluation)
  int nterms[3][3][kNumOvCombos];
  int kmax[3][3][kNumOvCombos];
  unsigned char ti[3][3][kNumOvCombos][kOvMaxTerms];
  unsigned char tj[3][3][kNumOvCombos][kOvMaxTerms];
  double tc[3][3][kNumOvCombos][kOvMaxTerms];
};

// packed (mu<=nu) index for the orbital order s, py, pz, px
__host__ __device__ inline int pack_index(int m, int n) {
  if (m > n) { int t = m; m = n; n = t; }
  return m * 4 - (m * (m - 1)) / 2 + (n - m);   // (0,0)=0 .. (3,3)=9
}
__host__ __device__ inline void unpack_index(int k, int* m, int* n) {
  const int mm[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
  const int nn[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
  *m = mm[k]; *n = nn[k];
}

template <typename T>
__host__ __device__ inline T eval_term(const EriTerm& t, T R, const T* dA, const T* dB,
                                       const T* rA, const T* rB) {
  T da = dA[t.la], db = dB[t.lb];
  T l = R + (T)t.c1 * da + (T)t.c2 * db;
  T u = (T)t.c3 * da + (T)t.c4 * db;
  T v = (T)t.c5 * da + (T)t.c6 * db;
  T a = rA[t.la] + rB[t.lb];
  T arg = l * l + u * u + v * v + a * a;
  return t.coef * ((T)1 / sqrt(arg));
}

// rotation: rows = space-frame orbital (s, py, pz, px), columns = local
// orbital, local z along A->B and gamma = 0 (MolDS Cndo2.cpp:5498-5527 with
// EularAngle.cpp:38-64, written without trigonometric round trips).
template <typename T>
__host__ __device__ inline void rotation_matrix(T x, T y, T z, T Rm[4][4]) {
  T r = sqrt(x * x + y * y + z * z);
  T rxy = sqrt(x * x + y * y);
  T cb = z / r, sb = rxy / r;
  T ca = 1, sa = 0;
  if (!(x == (T)0 && y == (T)0)) { ca = x / rxy; sa = y / rxy; }
  for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) Rm[i][j] = 0;
  Rm[0][0] = 1;
  Rm[1][1] = ca;  Rm[1][2] = sa * sb; Rm[1][3] = sa * cb;
  Rm[2][1] = 0;   Rm[2][2] = cb;      Rm[2][3] = -sb;
  Rm[3][1] = -sa; Rm[3][2] = ca * sb; Rm[3][3] = ca * cb;
}

// T2[(mu nu)][(i j)] for packed pairs: the rotation of a product of two
// orbitals, symmetrised over the local pair so that a symmetric local block
// L[(ij)][(kl)] (stored once per unordered pair) rotates as T2 L T2^T.
template <typename T>
__host__ __device__ inline T pair_rotation(const T Rm[4][4], int P, int Q) {
  int m, n, i, j;
  unpack_index(P, &m, &n);
  unpack_index(Q, &i, &j);
  if (i == j) return Rm[m][i] * Rm[n][i];
  return Rm[m][i] * Rm[n][j] + Rm[m][j] * Rm[n][i];
}

// A_k(p) = int_1^inf xi^k e^{-p xi}: closed sum, every k independent
template <typename T>
__host__ __device__ inline T aux_a(int k, T p) {
  // e^{-p} * sum_{m=0}^{k} k!/m! / p^{k-m+1}
  T s = 0, term = (T)1 / p;        // m = k term: 1/p
  for (int m = k; m >= 0; --m) {
    s += term;
    term *= (T)m / p;              // next: k!/(m-1)! / p^{k-m+2}
  }
  return exp(-p) * s;
}

// B_k(q) = int_-1^1 eta^k e^{-q eta}: series for |q| < 3, closed sums otherwise
template <typename T>
__host__ __device__ inline T aux_b(int k, T q) {
  if (fabs(q) < (T)3) {
    T term = 1, sum = 0;
    for (int m = 0; m < 80; ++m) {
      if (((k + m) & 1) == 0) sum += term * (T)2 / (T)(k + m + 1);
      term *= -q / (T)(m + 1);
    }
    return sum;
  }
  // B_k = [-e^{-q} sum_m k!/(k-m)! q^{-(m+1)}] + [(-1)^k e^{q} sum_m (-1)^m k!/(k-m)! q^{-(m+1)}]
  T s1 = 0, s2 = 0, f = (T)1 / q;
  for (int m = 0; m <= k; ++m) {
    s1 += f;
    s2 += (m & 1) ? -f : f;
    f *= (T)(k - m) / q;
  }
  T sgn = (k & 1) ? (T)-1 : (T)1;
  return -exp(-q) * s1 + sgn * exp(q) * s2;
}

// All A_k(p), k = 0..kmax, by the upward recurrence A_k = (e^-p + k A_{k-1}) / p
// (stable for p > 0: every term is positive).
template <typename T>
__host__ __device__ inline void aux_a_all(T p, int kmax, T* a) {
  const T e = exp(-p), ip = (T)1 / p;
  T v = e * ip;
  a[0] = v;
  for (int k = 1; k <= kmax; ++k) { v = (e + (T)k * v) * ip; a[k] = v; }
}

// All B_k(q), k = 0..kmax.  For |q| <= 4: B_kmax from its power series, then
// the downward recurrence B_{k-1} = (q B_k - (-1)^k e^q + e^-q) / k, which
// damps errors by |q|/k per step.  For |q| > 4: the upward recurrence
// B_k = (k B_{k-1} + (-1)^k e^q - e^-q) / q from B_0 = (e^q - e^-q) / q, whose
// error growth k/|q| per step stays below 11!/4^11 overall.  inv[j] = 1/j.
template <typename T, typename IT>
__host__ __device__ inline void aux_b_all(T q, int kmax, T* b, const IT* inv) {
  const T ep = exp(q), em = exp(-q);
  if (fabs(q) <= (T)4) {
    T term = 1, sum = 0;
    for (int m = 0; m < 80; ++m) {
      if (((kmax + m) & 1) == 0) sum += (T)2 * term * inv[kmax + m + 1];
      term *= -q * inv[m + 1];
      if (fabs(term) < (T)1e-19) break;
    }
    b[kmax] = sum;
    for (int k = kmax; k > 0; --k) b[k - 1] = (q * b[k] - ((k & 1) ? -ep : ep) + em) * inv[k];
  } else {
    const T iq = (T)1 / q;
    T v = (ep - em) * iq;
    b[0] = v;
    for (int k = 1; k <= kmax; ++k) { v = ((T)k * v + ((k & 1) ? -ep : ep) - em) * iq; b[k] = v; }
  }
}

}  // namespace nddo
