// Kernels (a) and (b): one-time pair integrals and the NDDO Fock build.
//
// (a) pair_kernel -- one warp per atom pair of every molecule in the batch.
//     Evaluates the distinct diatomic-frame two-centre integrals from the term
//     table (lane = local integral), rotates the packed 10x10 block to the
//     molecular frame as T2 L T2^T (T2 = symmetrised product rotation), and
//     stores it with coalesced lane-strided stores.  The same warp computes the
//     Slater overlap of the pair (diatomic frame, then rotated), the resonance
//     block 1/2 (beta_mu + beta_nu) S_mu,nu of the core Hamiltonian, and the
//     core-core repulsion E_AB.
//     MolDS: Mndo::CalcTwoElecsTwoAtomCores (src/mndo/Mndo.cpp:3703-3820),
//     CalcDiatomicTwoElecsTwoCores (:3948-4025), RotateDiatomicTwoElecsTwoCores
//     ToSpaceFrame (:4223-4293), Cndo2::CalcOverlapAOs (src/cndo/Cndo2.cpp:
//     4030-4146), Mndo::GetDiatomCoreRepulsionEnergy (:319-327, :223-240) and
//     Am1::GetDiatomCoreRepulsionEnergy (src/am1/Am1.cpp:145-170).
//
// (b) hcore_kernel / fock_kernel -- one CTA per molecule, one warp per atom.
//     Coulomb terms of the diagonal block of atom A are gathered from all
//     partner blocks by the lanes and reduced with a fixed shuffle tree, so the
//     result does not depend on scheduling (bitwise reproducible, alone or in a
//     batch).  Exchange blocks are written by the lane that owns the pair.
//     MolDS: Cndo2::CalcFockMatrix (src/cndo/Cndo2.cpp:1526-1636) with
//     Mndo::GetFockDiagElement (src/mndo/Mndo.cpp:422-488), GetFockOffDiagElement
//     (:490-580), GetCoulombInt/GetExchangeInt (:583-639), GetElectronCoreAttraction
//     (:643-650).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include "nddo_batch.cuh"
#include "kernels.h"
#include "nddo_dual.cuh"

namespace nddo {

__constant__ nddo_atom_params c_params[kNumParamSlots];
__constant__ double c_inv[128];   // c_inv[j] = 1 / j

void upload_primitives(const nddo_atom_params* p, cudaStream_t s);

void upload_params(const nddo_atom_params* p, cudaStream_t s) {
  static double inv[128];
  inv[0] = 0.0;
  for (int j = 1; j < 128; ++j) inv[j] = 1.0 / (double)j;
  cudaMemcpyToSymbolAsync(c_params, p, sizeof(nddo_atom_params) * kNumParamSlots, 0,
                          cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_inv, inv, sizeof(inv), 0, cudaMemcpyHostToDevice, s);
  upload_primitives(p, s);
}

__device__ __forceinline__ double sel3(int i, double a, double b, double c) {
  return i == 0 ? a : (i == 1 ? b : c);
}

constexpr int kPairWarps = 4;

// E_AB of MNDO (Mndo.cpp:223-240, 319-327) plus the AM1/PM3 Gaussians
// (Am1.cpp:145-170); ssss = (s_A s_A | s_B s_B).
template <typename T>
__device__ __forceinline__ T core_core(const nddo_atom_params& pa, const nddo_atom_params& pb, T R, T ssss,
                                       int theory) {
  T f;
  const bool a_no = (pa.atomic_number == 7 || pa.atomic_number == 8);
  const bool b_no = (pb.atomic_number == 7 || pb.atomic_number == 8);
  if (pa.atomic_number == 1 && b_no)
    f = 1.0 + (R / NDDO_ANG2AU) * exp(-pb.alpha * R) + exp(-pa.alpha * R);
  else if (pb.atomic_number == 1 && a_no)
    f = 1.0 + (R / NDDO_ANG2AU) * exp(-pa.alpha * R) + exp(-pb.alpha * R);
  else
    f = 1.0 + exp(-pa.alpha * R) + exp(-pb.alpha * R);
  T e = (double)(pa.core_charge * pb.core_charge) * ssss * f;
  if (theory != NDDO_MNDO) {
    T t = 0.0;
    for (int i = 0; i < 4; ++i) {
      if (pa.gk[i] != 0.0) { const T d = R - pa.gm[i]; t += pa.gk[i] * exp(-pa.gl[i] * (d * d)); }
      if (pb.gk[i] != 0.0) { const T d = R - pb.gm[i]; t += pb.gk[i] * exp(-pb.gl[i] * (d * d)); }
    }
    e += (double)(pa.core_charge * pb.core_charge) * t * NDDO_ANG2AU / R;
  }
  if (theory == NDDO_PM3PDDG) {
    // PDDG term (Pm3Pddg.cpp:143-165, 239-245); n = valence electrons = core charge
    const double na = pa.core_charge, nb = pb.core_charge;
    T t = 0.0;
    for (int i = 0; i < 2; ++i)
      for (int k = 0; k < 2; ++k) {
        const T x = R - pa.pddg_da[i] - pb.pddg_da[k];
        t += (na * pa.pddg_pa[i] + nb * pb.pddg_pa[k]) * exp(-10.0 / (NDDO_ANG2AU * NDDO_ANG2AU) * (x * x));
      }
    e += t / (na + nb);
  }
  return e;
}

// One overlap combination of the pair in the diatomic frame (thread-level):
// norm * ang * (R/2)^(na+nb+1) * sum_t c_t A_i(p) B_j(q).
template <typename T>
__device__ __forceinline__ T overlap_combo(const OverlapTable* __restrict__ ovt, int na, int nb, int c, double za,
                                           double zb, double norm, T R) {
  const int km = ovt->kmax[na - 1][nb - 1][c];
  T a[12], b[12];
  aux_a_all(0.5 * R * (za + zb), km, a);
  aux_b_all(0.5 * R * (za - zb), km, b, c_inv);
  T s = 0.0;
  const int nt = ovt->nterms[na - 1][nb - 1][c];
  for (int t = 0; t < nt; ++t)
    s += ovt->tc[na - 1][nb - 1][c][t] * a[ovt->ti[na - 1][nb - 1][c][t]] * b[ovt->tj[na - 1][nb - 1][c][t]];
  T rp = 1.0;
  for (int i = 0; i < na + nb + 1; ++i) rp *= 0.5 * R;
  return (norm * ovt->ang[c]) * rp * s;
}

__device__ __forceinline__ double slot_value(const EriTable* __restrict__ eri, int slot, double R,
                                             const nddo_atom_params& pa, const nddo_atom_params& pb) {
  double v = 0.0;
  const int nt = eri->nterms[slot];
  for (int t = 0; t < nt; ++t) {
    const EriTerm e = eri->terms[slot][t];
    const double da = e.la == 0 ? pa.d[0] : (e.la == 1 ? pa.d[1] : pa.d[2]);
    const double db = e.lb == 0 ? pb.d[0] : (e.lb == 1 ? pb.d[1] : pb.d[2]);
    const double ra = e.la == 0 ? pa.rho[0] : (e.la == 1 ? pa.rho[1] : pa.rho[2]);
    const double rb = e.lb == 0 ? pb.rho[0] : (e.lb == 1 ? pb.rho[1] : pb.rho[2]);
    const double l = R + (double)e.c1 * da + (double)e.c2 * db;
    const double u = (double)e.c3 * da + (double)e.c4 * db;
    const double w = (double)e.c5 * da + (double)e.c6 * db;
    const double a = ra + rb;
    v += e.coef * rsqrt(l * l + u * u + w * w + a * a);
  }
  return v;
}

// Pairs with at least one hydrogen, one thread per pair.  With X the atom
// carrying p orbitals (if any) and u the unit vector from X to H, the rotated
// block (X mu nu | H s s) of the local values s0 = (ss|ss), s3 = (xx|ss),
// s4 = (zz|ss), s10 = (sz|ss) is
//   (s s | s s) = s0,   (s p_mu | s s) = s10 u_mu,
//   (p_mu p_nu | s s) = s3 delta_mu,nu + (s4 - s3) u_mu u_nu,
// which is T2 L T2^T written out for this sparsity (the local z axis is u).
// Block layout is the same for both atom orders: 10 or 1 doubles.
__global__ void __launch_bounds__(128)
pair_light_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs,
                  const int* __restrict__ list, long long n, const DevMol* __restrict__ mols,
                  const EriTable* __restrict__ eri, const OverlapTable* __restrict__ ovt,
                  double* __restrict__ blocks, double* __restrict__ H, double* __restrict__ ecore_pair) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int p = list[t];
  const DevPair pr = pairs[p];
  const DevAtom A = atoms[pr.a], B = atoms[pr.b];
  const bool swap = (A.nao == 1 && B.nao == 4);
  const DevAtom X = swap ? B : A, Y = swap ? A : B;       // Y is a hydrogen
  const nddo_atom_params& px = c_params[X.pidx];
  const nddo_atom_params& py = c_params[Y.pidx];
  const DevMol mol = mols[pr.mol];
  const double dx = Y.x - X.x, dy = Y.y - X.y, dz = Y.z - X.z;
  const double R = sqrt(dx * dx + dy * dy + dz * dz);
  const double iR = 1.0 / R;
  const double u[4] = {0.0, dy * iR, dz * iR, dx * iR};   // orbital order s, py, pz, px
  const double s0 = slot_value(eri, 0, R, px, py);
  double* out = blocks + pr.blk;
  const long long ld = mol.nao;
  double Sss, Sps = 0.0;
  Sss = overlap_combo(ovt, px.principal_n, py.principal_n, 0, px.zeta[0], py.zeta[0],
                      px.sto_norm[0] * py.sto_norm[0], R);
  if (X.nao == 4) {
    const double s3 = slot_value(eri, 3, R, px, py);
    const double s4 = slot_value(eri, 4, R, px, py);
    const double s10 = slot_value(eri, 10, R, px, py);
    for (int P = 0; P < 10; ++P) {
      int m, k;
      unpack_index(P, &m, &k);
      double v;
      if (m == 0 && k == 0) v = s0;
      else if (m == 0) v = s10 * u[k];
      else v = (m == k ? s3 : 0.0) + (s4 - s3) * u[m] * u[k];
      out[P] = v;
    }
    Sps = overlap_combo(ovt, px.principal_n, py.principal_n, 2, px.zeta[1], py.zeta[0],
                        px.sto_norm[1] * py.sto_norm[0], R);
  } else {
    out[0] = s0;
  }
  // resonance entries 1/2 (beta_mu + beta_H) S_mu,H  (S_p,H = u_mu S_sigma-s)
  for (int mu = 0; mu < X.nao; ++mu) {
    const double sv = (mu == 0) ? Sss : u[mu] * Sps;
    const double h = 0.5 * (px.beta[mu == 0 ? 0 : 1] + py.beta[0]) * sv;
    const long long r = X.ao0 + mu, c = Y.ao0;
    H[mol.mat0 + r * ld + c] = h;
    H[mol.mat0 + c * ld + r] = h;
  }
  ecore_pair[p] = core_core(px, py, R, s0, mol.theory);
}

__global__ void __launch_bounds__(kPairWarps * 32)
pair_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs, const int* __restrict__ list,
            long long npairs, const DevMol* __restrict__ mols, const EriTable* __restrict__ eri,
            const OverlapTable* __restrict__ ovt, double* __restrict__ blocks,
            double* __restrict__ H, double* __restrict__ ecore_pair) {
  __shared__ double s_val[kPairWarps][24];
  __shared__ double s_T2[kPairWarps][100];
  __shared__ double s_L[kPairWarps][100];
  __shared__ double s_M[kPairWarps][100];
  __shared__ double s_ab[kPairWarps][4][24];
  __shared__ double s_ov[kPairWarps][8];
  __shared__ double s_R[kPairWarps][16];
  const unsigned full = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long pi = (long long)blockIdx.x * kPairWarps + warp;
  if (pi >= npairs) return;
  const long long p = list ? list[pi] : pi;

  const DevPair pr = pairs[p];
  const DevAtom A = atoms[pr.a], B = atoms[pr.b];
  const DevMol mol = mols[pr.mol];
  const nddo_atom_params& pa = c_params[A.pidx];
  const nddo_atom_params& pb = c_params[B.pidx];
  const double dx = B.x - A.x, dy = B.y - A.y, dz = B.z - A.z;
  const double R = sqrt(dx * dx + dy * dy + dz * dz);
  const int nA = A.nao, nB = B.nao;
  const int dA = nA == 4 ? 10 : 1, dB = nB == 4 ? 10 : 1;

  // ---- rotation matrix (lane 0) ------------------------------------------
  if (lane == 0) {
    double Rm[4][4];
    rotation_matrix(dx, dy, dz, Rm);
    for (int i = 0; i < 16; ++i) s_R[warp][i] = Rm[i >> 2][i & 3];
  }

  // ---- local two-centre integrals: lane = slot ----------------------------
  double val = 0.0;
  if (lane < 21) {
    bool need;
    if (nA == 4 && nB == 4) need = true;
    else if (nA == 4) need = (lane == 0 || lane == 3 || lane == 4 || lane == 10);
    else if (nB == 4) need = (lane == 0 || lane == 1 || lane == 2 || lane == 13);
    else need = (lane == 0);
    if (need) {
      const int nt = eri->nterms[lane];
      for (int t = 0; t < nt; ++t) {
        const EriTerm e = eri->terms[lane][t];
        const double da = sel3(e.la, pa.d[0], pa.d[1], pa.d[2]);
        const double db = sel3(e.lb, pb.d[0], pb.d[1], pb.d[2]);
        const double ra = sel3(e.la, pa.rho[0], pa.rho[1], pa.rho[2]);
        const double rb = sel3(e.lb, pb.rho[0], pb.rho[1], pb.rho[2]);
        const double l = R + (double)e.c1 * da + (double)e.c2 * db;
        const double u = (double)e.c3 * da + (double)e.c4 * db;
        const double v = (double)e.c5 * da + (double)e.c6 * db;
        const double a = ra + rb;
        const double arg = l * l + u * u + v * v + a * a;
        val += e.coef * rsqrt(arg);
      }
    }
  }
  const double s5 = __shfl_sync(full, val, 5), s6 = __shfl_sync(full, val, 6);
  if (lane == 21) val = (nA == 4 && nB == 4) ? 0.5 * (s5 - s6) : 0.0;
  if (lane < 22) s_val[warp][lane] = val;

  // ---- overlap auxiliary integrals: lane zc computes A_0..11 of zeta combination
  //      zc, lane 4 + zc its B_0..11 (zc: ss, s-p, p-s, p-p exponents) --------
  const int na = pa.principal_n, nb = pb.principal_n;
  if (lane < 8) {
    const int zc = lane & 3;
    const bool need = (zc == 0) || (zc == 1 && nB == 4) || (zc == 2 && nA == 4) || (zc == 3 && nA == 4 && nB == 4);
    double v[12];
    if (need) {
      const double za = (zc >= 2) ? pa.zeta[1] : pa.zeta[0];
      const double zb = (zc & 1) ? pb.zeta[1] : pb.zeta[0];
      if (lane < 4) aux_a_all(0.5 * R * (za + zb), 6, v);
      else aux_b_all(0.5 * R * (za - zb), 6, v, c_inv);
    } else {
#pragma unroll
      for (int k = 0; k < 12; ++k) v[k] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < 12; ++k) s_ab[warp][zc][(lane < 4 ? 0 : 12) + k] = v[k];
  }
  __syncwarp();

  // ---- T2 (pair rotation) and local block L ---------------------------------
  for (int e = lane; e < 100; e += 32) {
    const int P = e / 10, Q = e % 10;
    int m, n, i, j;
    unpack_index(P, &m, &n);
    unpack_index(Q, &i, &j);
    const double* Rm = s_R[warp];
    s_T2[warp][e] = (i == j) ? Rm[m * 4 + i] * Rm[n * 4 + i]
                             : Rm[m * 4 + i] * Rm[n * 4 + j] + Rm[m * 4 + j] * Rm[n * 4 + i];
    double l = 0.0;
    if (P < dA && Q < dB) {
      const int sl = eri->slot_of[P][Q];
      if (sl >= 0) l = s_val[warp][sl];
    }
    s_L[warp][e] = l;
  }
  // overlap sums, lane = combination (ss, s-sigma, sigma-s, sigma-sigma, pi-pi)
  if (lane < 5) {
    const int c = lane;
    const bool need = (c == 0) || (c == 1 && nB == 4) || (c == 2 && nA == 4) || (c >= 3 && nA == 4 && nB == 4);
    double s = 0.0;
    if (need) {
      const int zc = (c == 4) ? 3 : c;
      const int nt = ovt->nterms[na - 1][nb - 1][c];
      for (int t = 0; t < nt; ++t)
        s += ovt->tc[na - 1][nb - 1][c][t] * s_ab[warp][zc][ovt->ti[na - 1][nb - 1][c][t]] *
             s_ab[warp][zc][12 + ovt->tj[na - 1][nb - 1][c][t]];
      const double norm = pa.sto_norm[c >= 2 ? 1 : 0] * pb.sto_norm[(c == 1 || c >= 3) ? 1 : 0];
      double rp = 1.0;
      for (int i = 0; i < na + nb + 1; ++i) rp *= 0.5 * R;
      s *= norm * ovt->ang[c] * rp;
    }
    s_ov[warp][c] = s;
  }
  __syncwarp();

  // ---- M = L T2^T,  W = T2 M ----------------------------------------------
  for (int e = lane; e < dA * 10; e += 32) {
    const int P = e / 10, Qp = e % 10;
    double s = 0.0;
    if (Qp < dB)
      for (int Q = 0; Q < dB; ++Q) s += s_L[warp][P * 10 + Q] * s_T2[warp][Qp * 10 + Q];
    s_M[warp][e] = s;
  }
  __syncwarp();
  double* out = blocks + pr.blk;
  for (int e = lane; e < dA * dB; e += 32) {
    const int Pp = e / dB, Qp = e % dB;
    double s = 0.0;
    for (int P = 0; P < dA; ++P) s += s_T2[warp][Pp * 10 + P] * s_M[warp][P * 10 + Qp];
    out[e] = s;
  }

  // ---- resonance block of H:  1/2 (beta_mu + beta_nu) S_mu,nu --------------
  if (lane < 16) {
    const int mu = lane >> 2, nu = lane & 3;
    if (mu < nA && nu < nB) {
      double Ls[4][4] = {};
      Ls[0][0] = s_ov[warp][0];
      Ls[0][2] = s_ov[warp][1];
      Ls[2][0] = s_ov[warp][2];
      Ls[2][2] = s_ov[warp][3];
      Ls[1][1] = s_ov[warp][4];
      Ls[3][3] = s_ov[warp][4];
      const double* Rm = s_R[warp];
      double s = 0.0;
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) s += Rm[mu * 4 + i] * Ls[i][j] * Rm[nu * 4 + j];
      const double h = 0.5 * (pa.beta[mu == 0 ? 0 : 1] + pb.beta[nu == 0 ? 0 : 1]) * s;
      const long long ld = mol.nao;
      const long long r0 = A.ao0 + mu, c0 = B.ao0 + nu;
      H[mol.mat0 + r0 * ld + c0] = h;
      H[mol.mat0 + c0 * ld + r0] = h;
    }
  }

  // ---- core-core repulsion --------------------------------------------------
  if (lane == 0) ecore_pair[p] = core_core(pa, pb, R, s_val[warp][0], mol.theory);
}

// warp-wide sum with a fixed tree (bitwise reproducible)
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block (a,b) of the molecule, with a flag telling whether atom `self` owns the rows
__device__ __forceinline__ const double* partner_block(const DevPair* __restrict__ pairs, const double* blocks,
                                                       const DevMol& mol, int self, int other, bool* self_rows) {
  const int a = self < other ? self : other, b = self < other ? other : self;
  *self_rows = self < other;
  return blocks + pairs[mol.pair0 + pair_index(a, b, mol.natoms)].blk;
}

constexpr int kFockThreads = 256;

// Local integral (A's multipoles | a bare point charge): the slot's terms with
// both rho set to zero (MolDS Mndo::GetSemiEmpiricalMultipoleInteraction,
// src/mndo/Mndo.cpp:6602-6613, for an atom-EPC pair) and no charge separation
// on the point charge, whose only multipole is its monopole.
__device__ __forceinline__ double epc_slot_value(const EriTable* __restrict__ eri, int slot, double R,
                                                 const nddo_atom_params& pa) {
  double v = 0.0;
  const int nt = eri->nterms[slot];
  for (int t = 0; t < nt; ++t) {
    const EriTerm e = eri->terms[slot][t];
    const double da = e.la == 0 ? pa.d[0] : (e.la == 1 ? pa.d[1] : pa.d[2]);
    const double l = R + (double)e.c1 * da;
    const double u = (double)e.c3 * da;
    const double w = (double)e.c5 * da;
    v += e.coef * rsqrt(l * l + u * u + w * w);
  }
  return v;
}

// One-centre block of H (U on the diagonal plus the attraction of every other
// core, -Z_B (mu nu|s_B s_B)) and the molecule's core-core energy.  With
// environmental point charges each adds -q (mu nu|s s) to the block (MolDS
// Mndo::GetFockDiagElement / GetFockOffDiagElement, src/mndo/Mndo.cpp:474-484,
// 546-556, present in every non-guess Fock matrix and so in H = F(P = 0) of
// the energy, src/cndo/Cndo2.cpp:1324-1416), the block rotated from the local
// values exactly as a pair with a hydrogen (pair_light_kernel), and the
// cores' energy in their field, sum Z_A q / R (Mndo.cpp:329-331,
// Cndo2.cpp:418-426), goes to ecore_epc.
__global__ void __launch_bounds__(kFockThreads)
hcore_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs, const DevMol* __restrict__ mols,
             const int* __restrict__ mol_list, const double* __restrict__ blocks,
             const double* __restrict__ ecore_pair, const EriTable* __restrict__ eri,
             const double* __restrict__ epc, double* __restrict__ H, MolState* __restrict__ st) {
  __shared__ double s_epc[kFockThreads / 32];
  const int m = mol_list[blockIdx.x];
  const DevMol mol = mols[m];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const long long ld = mol.nao;
  double e_epc = 0.0;   // this lane's share of sum Z_A q / R
  for (int ia = warp; ia < mol.natoms; ia += nwarps) {
    const DevAtom A = atoms[mol.atom0 + ia];
    const int dA = A.nao == 4 ? 10 : 1;
    double acc[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.0;
    for (int ib = lane; ib < mol.natoms; ib += 32) {
      if (ib == ia) continue;
      const DevAtom Bt = atoms[mol.atom0 + ib];
      const double zb = c_params[Bt.pidx].core_charge;
      bool rows;
      const double* blk = partner_block(pairs, blocks, mol, ia, ib, &rows);
      const int dB = Bt.nao == 4 ? 10 : 1;
#pragma unroll
      for (int k = 0; k < 10; ++k)
        if (k < dA) acc[k] -= zb * (rows ? blk[k * dB] : blk[k]);
    }
    if (mol.nepc > 0) {
      const nddo_atom_params& pa = c_params[A.pidx];
      for (int i = lane; i < mol.nepc; i += 32) {
        const double* pc = epc + 4 * (mol.epc0 + i);
        const double dx = pc[0] - A.x, dy = pc[1] - A.y, dz = pc[2] - A.z, q = pc[3];
        const double R = sqrt(dx * dx + dy * dy + dz * dz);
        const double iR = 1.0 / R;
        e_epc += pa.core_charge * q / R;
        acc[0] -= q * epc_slot_value(eri, 0, R, pa);
        if (dA == 10) {
          const double s3 = epc_slot_value(eri, 3, R, pa);
          const double s4 = epc_slot_value(eri, 4, R, pa);
          const double s10 = epc_slot_value(eri, 10, R, pa);
          const double u[4] = {0.0, dy * iR, dz * iR, dx * iR};   // orbital order s, py, pz, px
#pragma unroll
          for (int k = 1; k < 10; ++k) {
            int mu, nu;
            unpack_index(k, &mu, &nu);
            const double v = mu == 0 ? s10 * u[nu] : (mu == nu ? s3 : 0.0) + (s4 - s3) * u[mu] * u[nu];
            acc[k] -= q * v;
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = warp_sum(acc[k]);
    if (lane < dA) {
      int mu, nu;
      unpack_index(lane, &mu, &nu);
      double v = 0.0;
#pragma unroll
      for (int k = 0; k < 10; ++k) if (k == lane) v = acc[k];
      if (mu == nu) v += c_params[A.pidx].u[mu == 0 ? 0 : 1];
      const long long r = A.ao0 + mu, c = A.ao0 + nu;
      H[mol.mat0 + r * ld + c] = v;
      H[mol.mat0 + c * ld + r] = v;
    }
  }
  e_epc = warp_sum(e_epc);
  if (lane == 0) s_epc[warp] = e_epc;
  __syncthreads();
  if (warp == 0) {
    double s = 0.0;
    for (int k = lane; k < mol.npairs; k += 32) s += ecore_pair[mol.pair0 + k];
    s = warp_sum(s);
    if (lane == 0) {
      st[m].ecore = s;
      double e = 0.0;
      for (int w = 0; w < nwarps; ++w) e += s_epc[w];
      st[m].ecore_epc = e;
    }
  }
}

__device__ __forceinline__ double g_one(const nddo_atom_params& p, int m, int n) {   // coulomb
  if (m == 0 && n == 0) return p.gss;
  if (m == 0 || n == 0) return p.gsp;
  return m == n ? p.gpp : p.gp2;
}
__device__ __forceinline__ double h_one(const nddo_atom_params& p, int m, int n) {   // exchange
  if (m == n) return g_one(p, m, n);
  if (m == 0 || n == 0) return p.hsp;
  return p.hpp;
}

// F = H + G(P) (mode 0), the MolDS guess Fock (mode 1: U on the diagonal,
// zero one-centre off-diagonal, resonance blocks between atoms), or H itself
// (mode 2).  P_old <- P is copied on the way when copy_old is set.
__global__ void __launch_bounds__(kFockThreads)
fock_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs, const DevMol* __restrict__ mols,
            const int* __restrict__ mol_list, const double* __restrict__ blocks, const double* __restrict__ H,
            const double* __restrict__ P, double* __restrict__ F, double* __restrict__ Pold,
            const MolState* __restrict__ st, int mode_override, int copy_old, int require_active) {
  // grid: x = groups of atom rows (a warp per atom row), y = molecule
  const int m = mol_list[blockIdx.y];
  const DevMol mol = mols[m];
  const MolState s = st[m];
  if (require_active && s.status != kActive) return;
  int mode = mode_override;
  if (mode < 0) mode = (s.iter == 0 && s.requires_guess) ? 1 : 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const long long ld = mol.nao;
  const double* Pm = P + mol.mat0;
  const double* Hm = H + mol.mat0;
  double* Fm = F + mol.mat0;
  const long long n2 = ld * ld;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, tstep = (long long)gridDim.x * blockDim.x;
  if (copy_old) {
    double* Po = Pold + mol.mat0;
    for (long long i = t0; i < n2; i += tstep) Po[i] = Pm[i];
  }
  if (mode == 2) {
    for (long long i = t0; i < n2; i += tstep) Fm[i] = Hm[i];
    return;
  }
  for (int ia = blockIdx.x * nwarps + warp; ia < mol.natoms; ia += gridDim.x * nwarps) {
    const DevAtom A = atoms[mol.atom0 + ia];
    const nddo_atom_params& pa = c_params[A.pidx];
    const int nA = A.nao, dA = nA == 4 ? 10 : 1;
    const int fa = A.ao0;
    double acc[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) acc[k] = 0.0;
    if (mode == 0) {
      // Coulomb: sum_B sum_{la si in B} P_la,si (mu nu|la si)
      for (int ib = lane; ib < mol.natoms; ib += 32) {
        if (ib == ia) continue;
        const DevAtom Bt = atoms[mol.atom0 + ib];
        const int nB = Bt.nao, dB = nB == 4 ? 10 : 1, fb = Bt.ao0;
        double pB[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) {
          pB[q] = 0.0;
          if (q < dB) {
            int l, sg;
            unpack_index(q, &l, &sg);
            pB[q] = Pm[(fb + l) * ld + fb + sg] * (l == sg ? 1.0 : 2.0);
          }
        }
        bool rows;
        const double* blk = partner_block(pairs, blocks, mol, ia, ib, &rows);
        if (rows) {
#pragma unroll
          for (int k = 0; k < 10; ++k) {
            if (k >= dA) break;
            double t = 0.0;
#pragma unroll
            for (int q = 0; q < 10; ++q) if (q < dB) t += blk[k * dB + q] * pB[q];
            acc[k] += t;
          }
        } else {
#pragma unroll
          for (int k = 0; k < 10; ++k) {
            if (k >= dA) break;
            double t = 0.0;
#pragma unroll
            for (int q = 0; q < 10; ++q) if (q < dB) t += blk[q * dA + k] * pB[q];
            acc[k] += t;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < 10; ++k) acc[k] = warp_sum(acc[k]);
    }
    // one-centre block
    if (lane < dA) {
      int mu, nu;
      unpack_index(lane, &mu, &nu);
      double v;
      if (mode == 1) {
        v = (mu == nu) ? pa.u[mu == 0 ? 0 : 1] : 0.0;
      } else {
        double j = 0.0;
#pragma unroll
        for (int k = 0; k < 10; ++k) if (k == lane) j = acc[k];
        v = Hm[(fa + mu) * ld + fa + nu];
        if (mu == nu) {
          double t = 0.0;
          for (int n = 0; n < nA; ++n) t += Pm[(fa + n) * ld + fa + n] * (g_one(pa, mu, n) - 0.5 * h_one(pa, mu, n));
          v += t;
        } else {
          v += (1.5 * h_one(pa, mu, nu) - 0.5 * g_one(pa, mu, nu)) * Pm[(fa + mu) * ld + fa + nu];
        }
        v += j;
      }
      Fm[(fa + mu) * ld + fa + nu] = v;
      Fm[(fa + nu) * ld + fa + mu] = v;
    }
    // two-centre blocks (A, B > A): resonance + exchange -1/2 sum P_nu,si (mu nu|la si)
    for (int ib = ia + 1 + lane; ib < mol.natoms; ib += 32) {
      const DevAtom Bt = atoms[mol.atom0 + ib];
      const int nB = Bt.nao, dB = nB == 4 ? 10 : 1, fb = Bt.ao0;
      const double* blk = blocks + pairs[mol.pair0 + pair_index(ia, ib, mol.natoms)].blk;
      double pab[4][4];
      if (mode == 0) {
        for (int n = 0; n < nA; ++n)
          for (int sg = 0; sg < nB; ++sg) pab[n][sg] = Pm[(fa + n) * ld + fb + sg];
      }
      for (int mu = 0; mu < nA; ++mu)
        for (int la = 0; la < nB; ++la) {
          double v = Hm[(fa + mu) * ld + fb + la];
          if (mode == 0) {
            double k = 0.0;
            for (int n = 0; n < nA; ++n)
              for (int sg = 0; sg < nB; ++sg) k += pab[n][sg] * blk[pack_index(mu, n) * dB + pack_index(la, sg)];
            v -= 0.5 * k;
          }
          Fm[(fa + mu) * ld + fb + la] = v;
          Fm[(fb + la) * ld + fa + mu] = v;
        }
    }
  }
}

void launch_pair_kernel(const DevAtom* atoms, const DevPair* pairs, long long npairs, const DevMol* mols,
                        const EriTable* eri, const OverlapTable* ovt, double* blocks, double* H,
                        double* ecore_pair, cudaStream_t s) {
  if (npairs <= 0) return;
  const long long grid = (npairs + kPairWarps - 1) / kPairWarps;
  pair_kernel<<<(unsigned)grid, kPairWarps * 32, 0, s>>>(atoms, pairs, nullptr, npairs, mols, eri, ovt, blocks, H,
                                                         ecore_pair);
}

void launch_pair_kernels_split(const DevAtom* atoms, const DevPair* pairs, const int* heavy_list, long long n_heavy,
                               const int* light_list, long long n_light, const DevMol* mols, const EriTable* eri,
                               const OverlapTable* ovt, double* blocks, double* H, double* ecore_pair,
                               cudaStream_t s) {
  if (n_heavy > 0) {
    const long long grid = (n_heavy + kPairWarps - 1) / kPairWarps;
    pair_kernel<<<(unsigned)grid, kPairWarps * 32, 0, s>>>(atoms, pairs, heavy_list, n_heavy, mols, eri, ovt, blocks,
                                                           H, ecore_pair);
  }
  if (n_light > 0) {
    const long long grid = (n_light + 127) / 128;
    pair_light_kernel<<<(unsigned)grid, 128, 0, s>>>(atoms, pairs, light_list, n_light, mols, eri, ovt, blocks, H,
                                                     ecore_pair);
  }
}

void launch_hcore_kernel(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list,
                         int nlist, const double* blocks, const double* ecore_pair, const EriTable* eri,
                         const double* epc, double* H, MolState* st, cudaStream_t s) {
  if (nlist <= 0) return;
  hcore_kernel<<<nlist, kFockThreads, 0, s>>>(atoms, pairs, mols, mol_list, blocks, ecore_pair, eri, epc, H, st);
}

void launch_fock_kernel(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list,
                        int nlist, int max_atoms, const double* blocks, const double* H, const double* P, double* F,
                        double* Pold, const MolState* st, int mode_override, int copy_old, int require_active,
                        cudaStream_t s) {
  if (nlist <= 0) return;
  const int rows = kFockThreads / 32;
  dim3 grid((max_atoms + rows - 1) / rows, nlist);
  fock_kernel<<<grid, kFockThreads, 0, s>>>(atoms, pairs, mols, mol_list, blocks, H, P, F, Pold, st, mode_override,
                                            copy_old, require_active);
}

// E = 1/2 sum P (F + H) + E_core + E_vdW (Cndo2::CalcElecSCFEnergy, src/cndo/Cndo2.cpp:1324-1416),
// Mulliken charges q_A = Z_A - sum_{mu in A} P_mu,mu (Cndo2.cpp:1187-1199, 1733-1747)
// and, for MNDO, the heat of formation (Mndo::CalcHeatsFormation, src/mndo/Mndo.cpp:395-404).
// E_vdW: the empirical dispersion energy of Cndo2::CalcVdWCorrectionEnergy
// (Cndo2.cpp:464-513), on when requested or for AM1-D / PM3-D (which fix
// s6 = 1.40, d = 23).
__global__ void __launch_bounds__(kFockThreads)
energy_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs, const DevMol* __restrict__ mols,
              const int* __restrict__ mol_list, const double* __restrict__ P, const double* __restrict__ F,
              const double* __restrict__ H, MolState* __restrict__ st, double* __restrict__ charges, VdwParams vdw) {
  __shared__ double red[32], red_v[32];
  const int m = mol_list[blockIdx.x];
  const DevMol mol = mols[m];
  const long long n2 = (long long)mol.nao * mol.nao;
  double acc = 0.0;
  for (long long i = threadIdx.x; i < n2; i += blockDim.x)
    acc += P[mol.mat0 + i] * (F[mol.mat0 + i] + H[mol.mat0 + i]);
  acc = warp_sum(acc);
  const bool dtheory = mol.theory == NDDO_AM1D || mol.theory == NDDO_PM3D;
  const bool vdw_on = vdw.on || dtheory;
  const double s6 = dtheory ? NDDO_VDW_S6_D : vdw.s6, dd = dtheory ? NDDO_VDW_DAMP_D : vdw.d;
  double ev = 0.0;
  if (vdw_on)
    for (int t = threadIdx.x; t < mol.npairs; t += blockDim.x) {
      const DevPair pr = pairs[mol.pair0 + t];
      const DevAtom A = atoms[pr.a], B = atoms[pr.b];
      const nddo_atom_params& pa = c_params[A.pidx];
      const nddo_atom_params& pb = c_params[B.pidx];
      const double csum = pa.vdw_c6 + pb.vdw_c6;
      if (csum <= 0.0) continue;
      const double dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
      const double R = sqrt(dx * dx + dy * dy + dz * dz);
      const double c6 = 2.0 * pa.vdw_c6 * pb.vdw_c6 / csum;
      const double damp = 1.0 / (1.0 + exp(-1.0 * dd * (R / (pa.vdw_r0 + pb.vdw_r0) - 1.0)));
      ev += -1.0 * s6 * c6 * damp / (R * R * R * R * R * R);
    }
  ev = warp_sum(ev);
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = acc; red_v[threadIdx.x >> 5] = ev; }
  __syncthreads();
  for (int a = threadIdx.x; a < mol.natoms; a += blockDim.x) {
    const DevAtom A = atoms[mol.atom0 + a];
    double pop = 0.0;
    for (int k = 0; k < A.nao; ++k) pop += P[mol.mat0 + (long long)(A.ao0 + k) * mol.nao + A.ao0 + k];
    charges[mol.atom0 + a] = c_params[A.pidx].core_charge - pop;
  }
  if (threadIdx.x == 0) {
    double e = 0.0, v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { e += red[w]; v += red_v[w]; }
    e *= 0.5;
    MolState* s = st + m;
    s->energy_electronic = e;
    s->vdw_energy = v;
    s->energy = e + s->ecore + s->ecore_epc + v;
    double hof = s->energy;
    for (int a = 0; a < mol.natoms; ++a) {
      const nddo_atom_params& pa = c_params[atoms[mol.atom0 + a].pidx];
      hof -= pa.e_atom;
      hof += pa.dhf_atom;
    }
    s->heat_of_formation = hof;
  }
}

void launch_energy_kernel(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list,
                          int nlist, const double* P, const double* F, const double* H, MolState* st,
                          double* charges, VdwParams vdw, cudaStream_t s) {
  if (nlist <= 0) return;
  energy_kernel<<<nlist, kFockThreads, 0, s>>>(atoms, pairs, mols, mol_list, P, F, H, st, charges, vdw);
}

// ---------------------------------------------------------------------------
// (c) Dipole moment after convergence.
//
// MolDS builds the Cartesian matrix X_k,mu,nu = <mu| r_k |nu> of every AO pair
// (same atom included) from the STO-6G expansion of each Slater orbital
// (Cndo2::CalcCartesianMatrixByGTOExpansion, src/cndo/Cndo2.cpp:1946-2130) and
// then forms mu_elec = -sum P X + c sum P S with c the centre of core mass,
// and mu_core = sum_A Z_A (R_A - c) (Cndo2.cpp:1871-1944).  Here the matrix is
// never stored: one warp takes one atom pair (or one atom), its lanes take the
// 6 x 6 primitive pairs of each shell pair, and every primitive block is
// contracted with P at once.
//
// Primitive integrals: normalised Cartesian Gaussians, s = N e^{-a|r-A|^2},
// p_i = 2 sqrt(a) (r_i - A_i) s.  With p = a + b, the product centre Pc,
// PA = Pc - A, PB = Pc - B and h = 1/(2p), the one-dimensional moments of
// (x-A)^i (x-B)^j follow from the Obara-Saika recurrence:
//   s10 = PA, s01 = PB, s11 = PA PB + h, s02 = PB^2 + h, s12 = PA PB^2 + (PA + 2 PB) h,
// and x = (x - B) + B turns them into moments of the position operator:
//   m00 = Pc, m10 = s11 + B PA, m01 = s02 + B PB, m11 = s12 + B s11.
// The three-dimensional integral is (s|s) times the product over directions,
// (s|s) = (2 sqrt(ab) / p)^{3/2} e^{-mu R^2}, mu = ab / p.
//
// Screen: a primitive pair with mu R^2 > 46 (e^{-46} = 1e-20) is skipped.
// Its elements are below 1e-17 (coefficients, normalisation and moments are
// O(1..100)), far below the FP64 rounding of the sums they would join.
// ---------------------------------------------------------------------------
constexpr int kDipThreads = 256;
constexpr double kDipScreen = 46.0;

// Per parameter slot and shell (s, p): the six primitive exponents a_i =
// zeta^2 alpha_i and factors f_i = d_i (2 sqrt(a_i) for p) a_i^{3/4}, so that a
// primitive pair's weight is 2^{3/2} f_i f_j p^{-3/2} e^{-mu R^2}.
__device__ double g_prim[kNumParamSlots][2][2][6];

void upload_primitives(const nddo_atom_params* p, cudaStream_t s) {
  static double prim[kNumParamSlots][2][2][6];
  for (int slot = 0; slot < kNumParamSlots; ++slot)
    for (int l = 0; l < 2; ++l)
      for (int i = 0; i < 6; ++i) {
        const int sh = p[slot].principal_n - 1;
        const double z = p[slot].zeta[l];
        const bool ok = sh >= 0 && sh < 3 && (l == 0 || p[slot].n_ao > 1) && z > 0.0;
        const double a = ok ? z * z * nddo_sto6g_exp[sh][l][i] : 0.0;
        double f = ok ? nddo_sto6g_coef[sh][l][i] * std::pow(a, 0.75) : 0.0;
        if (ok && l == 1) f *= 2.0 * std::sqrt(a);
        prim[slot][l][0][i] = a;
        prim[slot][l][1][i] = f;
      }
  cudaMemcpyToSymbolAsync(g_prim, prim, sizeof(prim), 0, cudaMemcpyHostToDevice, s);
}

// One primitive pair's X block (weighted), out[k][i][j]: k the axis of r, i / j
// the p axis (0 for an s shell).  Returns false when the pair is screened.
template <int LA, int LB>
__device__ __forceinline__ bool prim_block(const double* ra, const double* rb, const double* d, double R2, double a,
                                           double fa, double b, double fb,
                                           double (&out)[3][LA ? 3 : 1][LB ? 3 : 1]) {
  constexpr int NA = LA ? 3 : 1, NB = LB ? 3 : 1;
  const double r = rsqrt(a + b);          // p^{-1/2}
  const double ip = r * r;
  const double x = a * b * ip * R2;
  if (x > kDipScreen) return false;
  const double w = 2.8284271247461903 * fa * fb * (r * ip) * exp(-x);
  const double h = 0.5 * ip;
  double Pc[3], PA[3], PB[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    Pc[q] = (a * ra[q] + b * rb[q]) * ip;
    PA[q] = -b * ip * d[q];
    PB[q] = a * ip * d[q];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int i = 0; i < NA; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        double v;
        if (!LA && !LB) {
          v = Pc[k];
        } else if (!LA) {
          v = (k == j) ? PB[j] * PB[j] + h + rb[j] * PB[j] : PB[j] * Pc[k];
        } else if (!LB) {
          v = (k == i) ? PA[i] * PB[i] + h + rb[i] * PA[i] : PA[i] * Pc[k];
        } else if (i == j) {
          const double s11 = PA[i] * PB[i] + h;
          v = (k == i) ? PA[i] * PB[i] * PB[i] + (PA[i] + 2.0 * PB[i]) * h + rb[i] * s11 : s11 * Pc[k];
        } else {
          v = (k == i)   ? (PA[i] * PB[i] + h + rb[i] * PA[i]) * PB[j]
              : (k == j) ? PA[i] * (PB[j] * PB[j] + h + rb[j] * PB[j])
                         : PA[i] * PB[j] * Pc[k];
        }
        out[k][i][j] = w * v;
      }
  return true;
}

// AO index within an atom of p axis i (MolDS order s, py, pz, px)
__device__ __forceinline__ int ao_of_axis(int i) { return i == 0 ? 3 : i; }

// acc[k] += sum_{i, j} Wa_ij X_k,ij of one primitive pair, Wa in axis order
// (Wa[0][*] for an s shell on A, Wa[*][0] for an s shell on B).  The sums over
// i, j are folded into row / column sums: with U_k = sum_j Wa_kj PB_j,
// V_k = sum_i Wa_ik PA_i, Q = sum_k PA_k U_k, D = sum_i Wa_ii PA_i PB_i and
// T = sum_i Wa_ii s11_i, the p-p contraction for axis k is
//   Wa_kk m11_k + (T - Wa_kk s11_k) Pc_k + U'_k m10_k + V'_k m01_k
//   + (Q - D - PA_k U'_k - PB_k V'_k) Pc_k,  U'_k = U_k - Wa_kk PB_k, V'_k = V_k - Wa_kk PA_k,
// the terms of the block with k = i = j, i = j != k, k = i != j, k = j != i and
// i, j, k all different.
template <int LA, int LB>
__device__ __forceinline__ void prim_contract(const double* ra, const double* rb, const double* d, double R2,
                                              double a, double fa, double b, double fb, const double (&Wa)[3][3],
                                              double* acc) {
  const double r = rsqrt(a + b);          // p^{-1/2}
  const double ip = r * r;
  const double x = a * b * ip * R2;
  const double w = 2.8284271247461903 * fa * fb * (r * ip) * exp(-x);
  const double h = 0.5 * ip;
  double Pc[3], PA[3], PB[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    Pc[q] = (a * ra[q] + b * rb[q]) * ip;
    PA[q] = -b * ip * d[q];
    PB[q] = a * ip * d[q];
  }
  if (!LA && !LB) {
    const double ws = w * Wa[0][0];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k] += ws * Pc[k];
  } else if (!LA) {
    const double sPB = Wa[0][0] * PB[0] + Wa[0][1] * PB[1] + Wa[0][2] * PB[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double m01 = PB[k] * PB[k] + h + rb[k] * PB[k];
      acc[k] += w * (Wa[0][k] * m01 + Pc[k] * (sPB - Wa[0][k] * PB[k]));
    }
  } else if (!LB) {
    const double sPA = Wa[0][0] * PA[0] + Wa[1][0] * PA[1] + Wa[2][0] * PA[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double m10 = PA[k] * PB[k] + h + rb[k] * PA[k];
      acc[k] += w * (Wa[k][0] * m10 + Pc[k] * (sPA - Wa[k][0] * PA[k]));
    }
  } else {
    double s11[3], U[3], V[3];
    double T = 0.0, D = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      s11[i] = PA[i] * PB[i] + h;
      T += Wa[i][i] * s11[i];
      D += Wa[i][i] * PA[i] * PB[i];
      U[i] = Wa[i][0] * PB[0] + Wa[i][1] * PB[1] + Wa[i][2] * PB[2];
      V[i] = Wa[0][i] * PA[0] + Wa[1][i] * PA[1] + Wa[2][i] * PA[2];
    }
    const double Q = PA[0] * U[0] + PA[1] * U[1] + PA[2] * U[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double m10 = s11[k] + rb[k] * PA[k];
      const double m01 = PB[k] * PB[k] + h + rb[k] * PB[k];
      const double m11 = PA[k] * PB[k] * PB[k] + (PA[k] + 2.0 * PB[k]) * h + rb[k] * s11[k];
      const double Ur = U[k] - Wa[k][k] * PB[k];
      const double Vr = V[k] - Wa[k][k] * PA[k];
      acc[k] += w * (Wa[k][k] * m11 + (T - Wa[k][k] * s11[k]) * Pc[k] + Ur * m10 + Vr * m01 +
                     (Q - D - PA[k] * Ur - PB[k] * Vr) * Pc[k]);
    }
  }
}

// acc[k] += sum_{mu, nu} W_mu,nu X_k,mu,nu of the shell pair (LA, LB).  The
// warp screens the 36 primitive pairs (mu R^2 > 46, tested without a divide
// as a b R^2 > 46 (a + b)) and hands the survivors out lane by lane, so a
// distant atom pair with few survivors takes one pass.  Called by all lanes.
template <int LA, int LB>
__device__ __forceinline__ void shell_contract_warp(const double* ra, const double* rb, const double* d, double R2,
                                                    const double* pa_a, const double* pa_f, const double* pb_a,
                                                    const double* pb_f, const double (&W)[4][4], int lane,
                                                    double* acc) {
  double Wa[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Wa[i][j] = W[LA ? ao_of_axis(i) : 0][LB ? ao_of_axis(j) : 0];
  const double a0 = pa_a[lane / 6], b0 = pb_a[lane % 6];
  const bool keep0 = !(a0 * b0 * R2 > kDipScreen * (a0 + b0));
  bool keep1 = false;
  if (lane < 4) {
    const double a1 = pa_a[(lane + 32) / 6], b1 = pb_a[(lane + 32) % 6];
    keep1 = !(a1 * b1 * R2 > kDipScreen * (a1 + b1));
  }
  const unsigned m0 = __ballot_sync(0xffffffffu, keep0);
  const unsigned m1 = __ballot_sync(0xffffffffu, keep1);
  const int n0 = __popc(m0), n = n0 + __popc(m1);
  for (int slot = lane; slot < n; slot += 32) {
    // position of the (slot)-th set bit (0-based) of m0, then of m1
    unsigned m = slot < n0 ? m0 : m1;
    for (int q = slot < n0 ? slot : slot - n0; q > 0; --q) m &= m - 1;
    const int e = (slot < n0 ? 0 : 32) + __ffs(m) - 1;
    const int i6 = e / 6, j6 = e - 6 * (e / 6);
    prim_contract<LA, LB>(ra, rb, d, R2, pa_a[i6], pa_f[i6], pb_a[j6], pb_f[j6], Wa, acc);
  }
}

// CTAs of one molecule's dipole sums: a function of the molecule alone, so a
// molecule's result does not depend on the batch it runs in.
__host__ __device__ __forceinline__ int dipole_chunks(int natoms) {
  const long long items = (long long)natoms + (long long)natoms * (natoms - 1) / 2;
  const long long c = (items + 4LL * (kDipThreads / 32) - 1) / (4LL * (kDipThreads / 32));
  return (int)(c < 1 ? 1 : (c > kDipChunks ? kDipChunks : c));
}

// One work item: atom t of the molecule (t < natoms, the same-atom block) or
// atom pair t - natoms (a < b).  Returns the batch-global atom indices.
__device__ __forceinline__ void dipole_item(const DevMol& mol, const DevPair* __restrict__ pairs, long long t,
                                            int* ia, int* ib) {
  if (t < mol.natoms) {
    *ia = *ib = mol.atom0 + (int)t;
  } else {
    const DevPair pr = pairs[mol.pair0 + (t - mol.natoms)];
    *ia = pr.a;
    *ib = pr.b;
  }
}

// Partial sums per CTA: sum W X (x, y, z) and sum P S.  W = P_mu,nu + P_nu,mu
// for two different atoms (both triangles of MolDS's full-matrix dot product),
// P_mu,nu within one atom.  The inter-atom block of H is exactly
// 1/2 (beta_mu + beta_nu) S_mu,nu, so S is read back from H; within an atom S
// is the identity (Cndo2.cpp:4135-4140).  One warp per item.
__global__ void __launch_bounds__(kDipThreads, 2)
dipole_partial_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs,
                      const DevMol* __restrict__ mols, const int* __restrict__ mol_list,
                      const double* __restrict__ P, const double* __restrict__ H, double* __restrict__ partial) {
  __shared__ double s_prim[kNumParamSlots][2][2][6];
  __shared__ double red[kDipThreads / 32][4];
  const DevMol mol = mols[mol_list[blockIdx.y]];
  const int chunks = dipole_chunks(mol.natoms);
  if ((int)blockIdx.x >= chunks) return;
  for (int i = threadIdx.x; i < kNumParamSlots * 24; i += blockDim.x) (&s_prim[0][0][0][0])[i] = (&g_prim[0][0][0][0])[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int kWarps = kDipThreads / 32;
  const long long items = (long long)mol.natoms + mol.npairs;
  const long long ld = mol.nao;
  const double* Pm = P + mol.mat0;
  const double* Hm = H + mol.mat0;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long t = (long long)blockIdx.x * kWarps + warp; t < items; t += (long long)chunks * kWarps) {
    int ia, ib;
    dipole_item(mol, pairs, t, &ia, &ib);
    const DevAtom A = atoms[ia], B = atoms[ib];
    const bool same = ia == ib;
    double W[4][4];
#pragma unroll
    for (int mu = 0; mu < 4; ++mu)
#pragma unroll
      for (int nu = 0; nu < 4; ++nu) {
        double w = 0.0;
        if (mu < A.nao && nu < B.nao) {
          const long long r = A.ao0 + mu, c = B.ao0 + nu;
          w = Pm[r * ld + c];
          if (!same) w += Pm[c * ld + r];
        }
        W[mu][nu] = w;
      }
    // sum P S: lane e takes element (e / 4, e % 4) of the block
    if (lane < 16) {
      const int mu = lane >> 2, nu = lane & 3;
      if (mu < A.nao && nu < B.nao) {
        const long long r = A.ao0 + mu, c = B.ao0 + nu;
        if (!same) {
          const double bs = c_params[A.pidx].beta[mu == 0 ? 0 : 1] + c_params[B.pidx].beta[nu == 0 ? 0 : 1];
          acc[3] += (Pm[r * ld + c] + Pm[c * ld + r]) * (2.0 * Hm[r * ld + c] / bs);
        } else if (mu == nu) {
          acc[3] += Pm[r * ld + c];
        }
      }
    }
    const double ra[3] = {A.x, A.y, A.z}, rb[3] = {B.x, B.y, B.z};
    const double d[3] = {ra[0] - rb[0], ra[1] - rb[1], ra[2] - rb[2]};
    const double R2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double* As = s_prim[A.pidx][0][0];
    const double* Af = s_prim[A.pidx][0][1];
    const double* Bs = s_prim[B.pidx][0][0];
    const double* Bf = s_prim[B.pidx][0][1];
    const double* Ap = s_prim[A.pidx][1][0];
    const double* Apf = s_prim[A.pidx][1][1];
    const double* Bp = s_prim[B.pidx][1][0];
    const double* Bpf = s_prim[B.pidx][1][1];
    shell_contract_warp<0, 0>(ra, rb, d, R2, As, Af, Bs, Bf, W, lane, acc);
    if (B.nao > 1) shell_contract_warp<0, 1>(ra, rb, d, R2, As, Af, Bp, Bpf, W, lane, acc);
    if (A.nao > 1) shell_contract_warp<1, 0>(ra, rb, d, R2, Ap, Apf, Bs, Bf, W, lane, acc);
    if (A.nao > 1 && B.nao > 1) shell_contract_warp<1, 1>(ra, rb, d, R2, Ap, Apf, Bp, Bpf, W, lane, acc);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double v = warp_sum(acc[q]);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0.0;
    for (int w = 0; w < kWarps; ++w) v += red[w][threadIdx.x];
    partial[((long long)blockIdx.y * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = v;
  }
}

// One thread per molecule: chunk sums in a fixed order, the centre of core
// mass (src/base/Molecule.cpp:396-419), the core dipole and the electronic
// dipole; MolState::dipole = total, electronic, core (x, y, z each).
__global__ void dipole_finish_kernel(const DevAtom* __restrict__ atoms, const DevMol* __restrict__ mols,
                                     const int* __restrict__ mol_list, int nlist, int grid_chunks,
                                     const double* __restrict__ partial, MolState* __restrict__ st) {
  const int li = blockIdx.x * blockDim.x + threadIdx.x;
  if (li >= nlist) return;
  const int m = mol_list[li];
  const DevMol mol = mols[m];
  const int chunks = dipole_chunks(mol.natoms);
  double sum[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = 0; c < chunks; ++c)
    for (int q = 0; q < 4; ++q) sum[q] += partial[((long long)li * grid_chunks + c) * 4 + q];
  double center[3] = {0.0, 0.0, 0.0}, mass = 0.0;
  for (int a = 0; a < mol.natoms; ++a) {
    const DevAtom A = atoms[mol.atom0 + a];
    const double cm = c_params[A.pidx].core_mass;
    mass += cm;
    center[0] += A.x * cm;
    center[1] += A.y * cm;
    center[2] += A.z * cm;
  }
  for (int k = 0; k < 3; ++k) center[k] /= mass;
  double core[3] = {0.0, 0.0, 0.0};
  for (int a = 0; a < mol.natoms; ++a) {
    const DevAtom A = atoms[mol.atom0 + a];
    const double z = c_params[A.pidx].core_charge;
    core[0] += z * (A.x - center[0]);
    core[1] += z * (A.y - center[1]);
    core[2] += z * (A.z - center[2]);
  }
  MolState* s = st + m;
  for (int k = 0; k < 3; ++k) {
    const double elec = -sum[k] + center[k] * sum[3];
    s->dipole[k] = elec + core[k];
    s->dipole[3 + k] = elec;
    s->dipole[6 + k] = core[k];
  }
}

void launch_dipole(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, const int* mol_list, int nlist,
                   int max_atoms, const double* P, const double* H, double* partial, MolState* st, cudaStream_t s) {
  if (nlist <= 0) return;
  const int chunks = dipole_chunks(max_atoms);   // the largest molecule's count sets the grid
  dipole_partial_kernel<<<dim3(chunks, nlist), kDipThreads, 0, s>>>(atoms, pairs, mols, mol_list, P, H, partial);
  dipole_finish_kernel<<<(nlist + 127) / 128, 128, 0, s>>>(atoms, mols, mol_list, nlist, chunks, partial, st);
}

// X[k][mu][nu] of molecule m (3 x N x N doubles, row-major), both triangles:
// the matrix MolDS keeps as cartesianMatrix (Cndo2.cpp:1946-2057).  One thread
// per atom pair (or atom) and shell pair; not on the SCF path.
template <int LA, int LB>
__device__ __forceinline__ void shell_store(const double* ra, const double* rb, const double* d, double R2,
                                            const double* pa_a, const double* pa_f, const double* pb_a,
                                            const double* pb_f, int ao0A, int ao0B, long long N,
                                            double* __restrict__ X) {
  constexpr int NA = LA ? 3 : 1, NB = LB ? 3 : 1;
  double sum[3][NA][NB] = {};
  for (int i6 = 0; i6 < 6; ++i6)
    for (int j6 = 0; j6 < 6; ++j6) {
      double blk[3][NA][NB];
      if (!prim_block<LA, LB>(ra, rb, d, R2, pa_a[i6], pa_f[i6], pb_a[j6], pb_f[j6], blk)) continue;
      for (int k = 0; k < 3; ++k)
        for (int i = 0; i < NA; ++i)
          for (int j = 0; j < NB; ++j) sum[k][i][j] += blk[k][i][j];
    }
  const long long NN = N * N;
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < NA; ++i)
      for (int j = 0; j < NB; ++j) {
        const long long r = ao0A + (LA ? ao_of_axis(i) : 0), c = ao0B + (LB ? ao_of_axis(j) : 0);
        X[k * NN + r * N + c] = sum[k][i][j];
        X[k * NN + c * N + r] = sum[k][i][j];
      }
}

__global__ void __launch_bounds__(kDipThreads)
cartesian_matrix_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs,
                        const DevMol* __restrict__ mols, int m, double* __restrict__ X) {
  const DevMol mol = mols[m];
  const long long items = (long long)mol.natoms + mol.npairs;
  const long long N = mol.nao;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < items;
       t += (long long)gridDim.x * blockDim.x) {
    int ia, ib;
    dipole_item(mol, pairs, t, &ia, &ib);
    const DevAtom A = atoms[ia], B = atoms[ib];
    const double ra[3] = {A.x, A.y, A.z}, rb[3] = {B.x, B.y, B.z};
    const double d[3] = {ra[0] - rb[0], ra[1] - rb[1], ra[2] - rb[2]};
    const double R2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double* As = g_prim[A.pidx][0][0];
    const double* Af = g_prim[A.pidx][0][1];
    const double* Bs = g_prim[B.pidx][0][0];
    const double* Bf = g_prim[B.pidx][0][1];
    const double* Ap = g_prim[A.pidx][1][0];
    const double* Apf = g_prim[A.pidx][1][1];
    const double* Bp = g_prim[B.pidx][1][0];
    const double* Bpf = g_prim[B.pidx][1][1];
    shell_store<0, 0>(ra, rb, d, R2, As, Af, Bs, Bf, A.ao0, B.ao0, N, X);
    if (B.nao > 1) shell_store<0, 1>(ra, rb, d, R2, As, Af, Bp, Bpf, A.ao0, B.ao0, N, X);
    if (A.nao > 1) shell_store<1, 0>(ra, rb, d, R2, Ap, Apf, Bs, Bf, A.ao0, B.ao0, N, X);
    if (A.nao > 1 && B.nao > 1) shell_store<1, 1>(ra, rb, d, R2, Ap, Apf, Bp, Bpf, A.ao0, B.ao0, N, X);
  }
}

void launch_cartesian_matrix(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, int m, int natoms,
                             double* X, cudaStream_t s) {
  const long long items = (long long)natoms + (long long)natoms * (natoms - 1) / 2;
  const int blocks = (int)std::max(1LL, std::min<long long>(4096, (items + kDipThreads - 1) / kDipThreads));
  cartesian_matrix_kernel<<<blocks, kDipThreads, 0, s>>>(atoms, pairs, mols, m, X);
}

// ---------------------------------------------------------------------------
// Analytic energy gradient (forces) of a converged SCF, for the molecules of
// a list (Mndo::CalcForce, src/mndo/Mndo.cpp:2711-2986, ground state).
//
// With the density P fixed at convergence (the SCF energy is stationary in
// the orbitals and NDDO has no basis-overlap terms) the energy depends on the
// geometry only through the pair terms, each a function of the pair's
// relative position d = R_B - R_A:
//   E_AB = sum_PQ C_PQ W_PQ(d) + sum_{mu in A, la in B} P_mu,la (beta_mu + beta_la) S_mu,la(d)
//          + E_core(d) [+ E_vdW(d)]
// with W = T2 L T2^T the rotated (mu nu|la si) block, C_PQ = m_P m_Q P_P P_Q
// - 1/2 X_PQ (Coulomb and exchange, m = 2 for mu != nu, X summed over both
// orbital orders) plus the electron-core attractions -Z_B (mu nu|s_B s_B) on
// the (mu nu, ss) column and -Z_A on the (ss, la si) row.  One thread per
// pair evaluates E_AB in dual numbers seeded with d (the exact derivatives of
// the same local integrals, rotation and overlaps the pair kernels use), and
// writes dE_AB/dd; the gradient of atom i is then
//   g_i = sum_{a < i} dE_ai/dd - sum_{b > i} dE_ib/dd   (fixed order).
// The local frame here is z along d and x from the coordinate axis least
// aligned with it (smooth in d near every axis); the rotated integrals do not
// depend on the azimuth of the frame (the local integrals are cylindrically
// symmetric), so they equal the pair kernels' values.
// ---------------------------------------------------------------------------
namespace {

__device__ void smooth_frame(const Dual3& x, const Dual3& y, const Dual3& z, Dual3 Rm[4][4]) {
  const Dual3 r = sqrt(x * x + y * y + z * z);
  const Dual3 ez[3] = {x / r, y / r, z / r};
  int k = 0;
  for (int i = 1; i < 3; ++i)
    if (::fabs(ez[i].v) < ::fabs(ez[k].v)) k = i;
  Dual3 ex[3] = {-ez[k] * ez[0], -ez[k] * ez[1], -ez[k] * ez[2]};
  ex[k] += 1.0;
  const Dual3 nx = sqrt(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]);
  for (int i = 0; i < 3; ++i) ex[i] /= nx;
  const Dual3 ey[3] = {ez[1] * ex[2] - ez[2] * ex[1], ez[2] * ex[0] - ez[0] * ex[2], ez[0] * ex[1] - ez[1] * ex[0]};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) Rm[i][j] = 0.0;
  Rm[0][0] = 1.0;
  // rows: space-frame orbitals s, py, pz, px; columns: local s, y, z, x
  const int comp[4] = {-1, 1, 2, 0};
  for (int row = 1; row < 4; ++row) {
    Rm[row][1] = ey[comp[row]];
    Rm[row][2] = ez[comp[row]];
    Rm[row][3] = ex[comp[row]];
  }
}

}  // namespace

__global__ void __launch_bounds__(64)
pair_grad_kernel(const DevAtom* __restrict__ atoms, const DevPair* __restrict__ pairs, long long pair0,
                 long long npairs, const DevMol* __restrict__ mols, const EriTable* __restrict__ eri,
                 const OverlapTable* __restrict__ ovt, const double* __restrict__ P, VdwParams vdw,
                 double* __restrict__ grad) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npairs) return;
  const long long p = pair0 + t;
  const DevPair pr = pairs[p];
  const DevAtom A = atoms[pr.a], B = atoms[pr.b];
  const DevMol mol = mols[pr.mol];
  const nddo_atom_params& pa = c_params[A.pidx];
  const nddo_atom_params& pb = c_params[B.pidx];
  const int nA = A.nao, nB = B.nao, dA = nA == 4 ? 10 : 1, dB = nB == 4 ? 10 : 1;
  const Dual3 dx(B.x - A.x, 1.0, 0.0, 0.0), dy(B.y - A.y, 0.0, 1.0, 0.0), dz(B.z - A.z, 0.0, 0.0, 1.0);
  const Dual3 R = sqrt(dx * dx + dy * dy + dz * dz);
  const double* Pm = P + mol.mat0;
  const long long ld = mol.nao;

  // local integrals (the slots this pair's orbitals need)
  Dual3 val[kNumSlots];
  {
    const Dual3 dAv[3] = {pa.d[0], pa.d[1], pa.d[2]}, dBv[3] = {pb.d[0], pb.d[1], pb.d[2]};
    const Dual3 rAv[3] = {pa.rho[0], pa.rho[1], pa.rho[2]}, rBv[3] = {pb.rho[0], pb.rho[1], pb.rho[2]};
    for (int sl = 0; sl < 21; ++sl) {
      bool need;
      if (nA == 4 && nB == 4) need = true;
      else if (nA == 4) need = (sl == 0 || sl == 3 || sl == 4 || sl == 10);
      else if (nB == 4) need = (sl == 0 || sl == 1 || sl == 2 || sl == 13);
      else need = (sl == 0);
      Dual3 v = 0.0;
      if (need)
        for (int k = 0; k < eri->nterms[sl]; ++k) v += eval_term(eri->terms[sl][k], R, dAv, dBv, rAv, rBv);
      val[sl] = v;
    }
    val[21] = (nA == 4 && nB == 4) ? 0.5 * (val[5] - val[6]) : Dual3(0.0);
  }
  Dual3 Rm[4][4];
  smooth_frame(dx, dy, dz, Rm);

  // C: the density factors of each (mu nu, la si) integral
  double C[10][10];
  {
    double pA[10], pB[10], mA[10], mB[10];
    for (int q = 0; q < dA; ++q) {
      int m, n;
      unpack_index(q, &m, &n);
      pA[q] = Pm[(A.ao0 + m) * ld + A.ao0 + n];
      mA[q] = m == n ? 1.0 : 2.0;
    }
    for (int q = 0; q < dB; ++q) {
      int m, n;
      unpack_index(q, &m, &n);
      pB[q] = Pm[(B.ao0 + m) * ld + B.ao0 + n];
      mB[q] = m == n ? 1.0 : 2.0;
    }
    for (int q = 0; q < dA; ++q) {
      int a, b;
      unpack_index(q, &a, &b);
      for (int r = 0; r < dB; ++r) {
        int c, e;
        unpack_index(r, &c, &e);
        // exchange: both orders of (a b) and of (c e)
        double x = 0.0;
        for (int o1 = 0; o1 < (a == b ? 1 : 2); ++o1) {
          const int u = o1 ? b : a, w = o1 ? a : b;
          for (int o2 = 0; o2 < (c == e ? 1 : 2); ++o2) {
            const int y = o2 ? e : c, z = o2 ? c : e;
            x += Pm[(A.ao0 + u) * ld + B.ao0 + y] * Pm[(A.ao0 + w) * ld + B.ao0 + z];
          }
        }
        C[q][r] = mA[q] * mB[r] * pA[q] * pB[r] - 0.5 * x;
      }
    }
    for (int q = 0; q < dA; ++q) C[q][0] += -(double)pb.core_charge * mA[q] * pA[q];
    for (int r = 0; r < dB; ++r) C[0][r] += -(double)pa.core_charge * mB[r] * pB[r];
  }

  // two-electron and electron-core part: sum_PQ C_PQ (T2 L T2^T)_PQ
  Dual3 e_pair = 0.0;
  {
    Dual3 T2[10][10];
    for (int q = 0; q < 10; ++q)
      for (int r = 0; r < 10; ++r) T2[q][r] = (q < dA || q < dB) ? pair_rotation(Rm, q, r) : Dual3(0.0);
    // M[P][Q'] = sum_Q L[P][Q] T2[Q'][Q]
    for (int Pl = 0; Pl < dA; ++Pl) {
      Dual3 Mrow[10];
      for (int Qp = 0; Qp < dB; ++Qp) {
        Dual3 acc = 0.0;
        for (int Q = 0; Q < dB; ++Q) {
          const int sl = eri->slot_of[Pl][Q];
          if (sl >= 0) acc += val[sl] * T2[Qp][Q];
        }
        Mrow[Qp] = acc;
      }
      // W[P'][Q'] = sum_P T2[P'][P] M[P][Q']: accumulate C[P'][Q'] T2[P'][P] M[P][Q']
      for (int Pp = 0; Pp < dA; ++Pp) {
        Dual3 cm = 0.0;
        for (int Qp = 0; Qp < dB; ++Qp) cm += C[Pp][Qp] * Mrow[Qp];
        e_pair += T2[Pp][Pl] * cm;
      }
    }
  }

  // resonance: sum P_mu,la (beta_mu + beta_la) S_mu,la
  {
    const int na = pa.principal_n, nb = pb.principal_n;
    Dual3 ov[5];
    for (int c = 0; c < 5; ++c) {
      const bool need = (c == 0) || (c == 1 && nB == 4) || (c == 2 && nA == 4) || (c >= 3 && nA == 4 && nB == 4);
      if (!need) { ov[c] = 0.0; continue; }
      const double za = c >= 2 ? pa.zeta[1] : pa.zeta[0];
      const double zb = (c == 1 || c >= 3) ? pb.zeta[1] : pb.zeta[0];
      const double norm = pa.sto_norm[c >= 2 ? 1 : 0] * pb.sto_norm[(c == 1 || c >= 3) ? 1 : 0];
      ov[c] = overlap_combo(ovt, na, nb, c, za, zb, norm, R);
    }
    Dual3 Ls[4][4];
    Ls[0][0] = ov[0]; Ls[0][2] = ov[1]; Ls[2][0] = ov[2]; Ls[2][2] = ov[3]; Ls[1][1] = ov[4]; Ls[3][3] = ov[4];
    for (int mu = 0; mu < nA; ++mu)
      for (int la = 0; la < nB; ++la) {
        Dual3 sv = 0.0;
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j)
            if (i == j || (i == 0 && j == 2) || (i == 2 && j == 0)) sv += Rm[mu][i] * Ls[i][j] * Rm[la][j];
        const double w = Pm[(A.ao0 + mu) * ld + B.ao0 + la] * (pa.beta[mu == 0 ? 0 : 1] + pb.beta[la == 0 ? 0 : 1]);
        e_pair += w * sv;
      }
  }

  // core-core repulsion (with the AM1 / PM3 Gaussians and the PDDG term)
  e_pair += core_core(pa, pb, R, val[0], mol.theory);

  // empirical dispersion (energy_kernel's pair term)
  const bool dtheory = mol.theory == NDDO_AM1D || mol.theory == NDDO_PM3D;
  if (vdw.on || dtheory) {
    const double s6 = dtheory ? NDDO_VDW_S6_D : vdw.s6, dd = dtheory ? NDDO_VDW_DAMP_D : vdw.d;
    const double csum = pa.vdw_c6 + pb.vdw_c6;
    if (csum > 0.0) {
      const double c6 = 2.0 * pa.vdw_c6 * pb.vdw_c6 / csum;
      const Dual3 damp = 1.0 / (1.0 + exp(-1.0 * dd * (R / (pa.vdw_r0 + pb.vdw_r0) - 1.0)));
      const Dual3 R2 = R * R;
      e_pair += (-1.0 * s6 * c6) * damp / (R2 * R2 * R2);
    }
  }
  grad[3 * t] = e_pair.d[0];
  grad[3 * t + 1] = e_pair.d[1];
  grad[3 * t + 2] = e_pair.d[2];
}

// forces F_i = -g_i of one molecule's atoms from its pair gradients
__global__ void force_reduce_kernel(const DevMol* __restrict__ mols, int m, const double* __restrict__ grad,
                                    double* __restrict__ forces) {
  const DevMol mol = mols[m];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mol.natoms) return;
  double g[3] = {0.0, 0.0, 0.0};
  for (int a = 0; a < i; ++a) {
    const long long q = pair_index(a, i, mol.natoms);
    for (int k = 0; k < 3; ++k) g[k] += grad[3 * q + k];
  }
  for (int b = i + 1; b < mol.natoms; ++b) {
    const long long q = pair_index(i, b, mol.natoms);
    for (int k = 0; k < 3; ++k) g[k] -= grad[3 * q + k];
  }
  for (int k = 0; k < 3; ++k) forces[3 * i + k] = -g[k];
}

void launch_forces(const DevAtom* atoms, const DevPair* pairs, const DevMol* mols, int m, long long pair0,
                   long long npairs, int natoms, const EriTable* eri, const OverlapTable* ovt, const double* P,
                   VdwParams vdw, double* grad, double* forces, cudaStream_t s) {
  if (npairs > 0)
    pair_grad_kernel<<<(unsigned)((npairs + 63) / 64), 64, 0, s>>>(atoms, pairs, pair0, npairs, mols, eri, ovt, P,
                                                                      vdw, grad);
  force_reduce_kernel<<<(natoms + 127) / 128, 128, 0, s>>>(mols, m, grad, forces);
}

}  // namespace nddo
