// Host engine of the batched NDDO SCF.
//
// The SCF of every molecule in a batch follows MolDS Cndo2::DoSCF
// (src/cndo/Cndo2.cpp:585-729) step for step:
//   iteration:  P_old <- P;  F <- guess Fock (iteration 0) or H + G(P);
//               diagonalise F;  P <- 2 C_occ^T C_occ;  RMS test;  DIIS;  damping
//   after convergence:  F(P), H  ->  E = 1/2 sum P (F + H) + E_core, Mulliken charges.
// Each step is one launch over all active molecules of the batch; a converged
// molecule drops out of every later launch by its own state flag.
#include "engine.h"
#include "tuning.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "nddo_tables.h"

namespace nddo {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
static T* dalloc(size_t count, size_t* total) {
  T* p = nullptr;
  if (count == 0) count = 1;
  cuda_check(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
  *total += count * sizeof(T);
  return p;
}

// ---------------------------------------------------------------------------
__global__ void init_state_kernel(const DevMol* __restrict__ mols, const int* __restrict__ list, int n,
                                  MolState* __restrict__ st, double* __restrict__ C, double* __restrict__ P,
                                  double* __restrict__ eps, int requires_guess, int reset_density,
                                  double* __restrict__ hist_dens, double* __restrict__ hist_err, int diis_m,
                                  long long mat_total, int* __restrict__ sweeps) {
  const int m = list[blockIdx.x];
  const DevMol mol = mols[m];
  const long long n2 = (long long)mol.nao * mol.nao;
  if (threadIdx.x == 0) {
    MolState s;
    memset(&s, 0, sizeof(s));
    s.status = kActive;
    s.requires_guess = requires_guess;
    s.ecore = st[m].ecore;   // computed by the integral pass
    s.ecore_epc = st[m].ecore_epc;
    st[m] = s;
    if (sweeps) sweeps[m] = 0;
  }
  // a run from the previous density (requires_guess = 0) also keeps the
  // previous eigenvectors as the eigensolver's warm-start basis
  // a cold start also forgets the eigenvalues of the last solve, which the
  // FP64 eigensolver would otherwise take as starting points
  if (reset_density)
    for (int i = threadIdx.x; i < mol.nao; i += blockDim.x) eps[mol.vec0 + i] = __longlong_as_double(0x7ff8000000000000LL);
  if (reset_density)
    for (long long i = threadIdx.x; i < n2; i += blockDim.x) {
      const long long r = i / mol.nao, c = i % mol.nao;
      C[mol.mat0 + i] = (r == c) ? 1.0 : 0.0;
      P[mol.mat0 + i] = 0.0;
    }
  // the DIIS window starts zero-filled (as the reference's zero-initialised history)
  for (int k = 0; k < diis_m; ++k)
    for (long long i = threadIdx.x; i < n2; i += blockDim.x) {
      hist_dens[k * mat_total + mol.mat0 + i] = 0.0;
      hist_err[k * mat_total + mol.mat0 + i] = 0.0;
    }
}

__global__ void count_active_kernel(const int* __restrict__ list, int n, const MolState* __restrict__ st,
                                    int* __restrict__ out, char* __restrict__ active) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int c = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int a = (st[list[i]].status == kActive);
    active[list[i]] = (char)a;
    c += a;
  }
  atomicAdd(&cnt, c);
  __syncthreads();
  if (threadIdx.x == 0) *out = cnt;
}

// ---------------------------------------------------------------------------
Engine::Engine(int device) : device_(device) {
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  static EriTable eri;
  static OverlapTable ovt;
  static bool built = false;
  if (!built) { build_eri_table(&eri); build_overlap_table(&ovt); built = true; }
  cuda_check(cudaMalloc(&d_eri_, sizeof(EriTable)), "cudaMalloc eri");
  cuda_check(cudaMalloc(&d_ovt_, sizeof(OverlapTable)), "cudaMalloc ovt");
  cuda_check(cudaMemcpyAsync(d_eri_, &eri, sizeof(EriTable), cudaMemcpyHostToDevice, stream_), "copy eri");
  cuda_check(cudaMemcpyAsync(d_ovt_, &ovt, sizeof(OverlapTable), cudaMemcpyHostToDevice, stream_), "copy ovt");
  nddo_atom_params params[kNumParamSlots];
  std::memset(params, 0, sizeof(params));
  static const int zs[NDDO_NUM_ELEMENTS] = {1, 6, 7, 8, 9, 16, 17};
  for (int t = 0; t < NDDO_NUM_THEORY_SLOTS; ++t)
    for (int e = 0; e < NDDO_NUM_ELEMENTS; ++e) nddo_fill_atom_params(t, zs[e], &params[t * NDDO_NUM_ELEMENTS + e]);
  upload_params(params, stream_);
  cuda_check(cudaStreamSynchronize(stream_), "engine init");
}

Engine::~Engine() {
  cudaFree(d_eri_);
  cudaFree(d_ovt_);
  if (stream_) cudaStreamDestroy(stream_);
}

// ---------------------------------------------------------------------------
void ArenaAlloc::reset(long long capacity) {
  free_.clear();
  if (capacity > 0) free_[0] = capacity;
}

long long ArenaAlloc::alloc(long long n) {
  if (n <= 0) return 0;
  for (auto it = free_.begin(); it != free_.end(); ++it) {
    if (it->second < n) continue;
    const long long off = it->first, len = it->second;
    free_.erase(it);
    if (len > n) free_[off + n] = len - n;
    return off;
  }
  return -1;
}

void ArenaAlloc::release(long long off, long long n) {
  if (n <= 0) return;
  auto it = free_.emplace(off, n).first;
  auto nx = std::next(it);
  if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
  if (it != free_.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
  }
}

long long ArenaAlloc::free_total() const {
  long long t = 0;
  for (const auto& kv : free_) t += kv.second;
  return t;
}

namespace {
// Checks one molecule and lays out its atoms and pairs (indices relative to
// the molecule); mirrors the checks MolDS makes when it reads a molecule.
struct MolLayout {
  std::vector<DevAtom> atoms;
  std::vector<DevPair> pairs;   // a, b relative; blk relative
  int nao = 0, nocc = 0;
  long long blocks = 0;
};

MolLayout layout_molecule(const MoleculeInput& in) {
  MolLayout L;
  const int na = (int)in.Z.size();
  if (na < 1) throw std::invalid_argument("molecule without atoms");
  if ((int)in.xyz.size() != 3 * na) throw std::invalid_argument("coordinate count does not match atom count");
  if (in.theory < 0 || in.theory >= NDDO_NUM_THEORY_SLOTS) throw std::invalid_argument("unknown theory");
  int ao = 0, nelec = 0;
  for (int a = 0; a < na; ++a) {
    const int e = nddo_element_index(in.Z[a]);
    nddo_atom_params probe;
    if (e < 0 || nddo_fill_atom_params(in.theory, in.Z[a], &probe) != 0)
      throw std::invalid_argument("element " + std::to_string(in.Z[a]) + " has no parameters for this theory");
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(in.xyz[3 * a + k])) throw std::invalid_argument("non-finite coordinate");
    DevAtom at;
    at.x = in.xyz[3 * a]; at.y = in.xyz[3 * a + 1]; at.z = in.xyz[3 * a + 2];
    at.pidx = in.theory * NDDO_NUM_ELEMENTS + e;
    at.ao0 = ao;
    at.nao = nddo_elements[e].n_ao;
    at.mol = 0;
    ao += at.nao;
    nelec += nddo_elements[e].core_charge;
    L.atoms.push_back(at);
  }
  if (nelec % 2) throw std::invalid_argument("Total number of valence electrons is odd. totalNumberValenceElectrons=" + std::to_string(nelec));
  L.nao = ao;
  L.nocc = nelec / 2;
  // point charges (src/base/InputParser.cpp:626-644): a charge on an atom's
  // position would make its Coulomb terms infinite
  if (in.epc.size() % 4) throw std::invalid_argument("point charges need x, y, z and a charge each");
  for (size_t i = 0; i < in.epc.size(); i += 4) {
    for (int k = 0; k < 4; ++k)
      if (!std::isfinite(in.epc[i + k])) throw std::invalid_argument("non-finite point charge");
    for (const DevAtom& A : L.atoms)
      if (A.x == in.epc[i] && A.y == in.epc[i + 1] && A.z == in.epc[i + 2])
        throw std::invalid_argument("a point charge at an atom's position");
  }
  for (int a = 0; a < na; ++a)
    for (int b = a + 1; b < na; ++b) {
      const DevAtom& A = L.atoms[a];
      const DevAtom& B = L.atoms[b];
      const double dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
      if (dx == 0.0 && dy == 0.0 && dz == 0.0) throw std::invalid_argument("two atoms at the same position");
      DevPair p;
      p.a = a; p.b = b; p.mol = 0; p.pad = 0;
      p.blk = L.blocks;
      L.blocks += (long long)(A.nao == 4 ? 10 : 1) * (B.nao == 4 ? 10 : 1);
      L.pairs.push_back(p);
    }
  return L;
}

inline long long round32(long long x) { return (x + 31) / 32 * 32; }
}  // namespace

int molecule_nao(const MoleculeInput& in) {
  int ao = 0;
  for (int z : in.Z) {
    const int e = nddo_element_index(z);
    if (e >= 0) ao += nddo_elements[e].n_ao;
  }
  return ao;
}


size_t Batch::bytes_per_mat_element(int diis_m) {
  // H F P P_old C G64 T64 + six refinement buffers (FP64), G32 T32 + three tensor-core
  // shadows (FP32), DIIS history
  return 13 * sizeof(double) + 5 * sizeof(float) + 2 * (size_t)std::max(diis_m, 1) * sizeof(double);
}

Batch::Batch(Engine* eng, const std::vector<MoleculeInput>& mols, int diis_m, cudaStream_t stream)
    : eng_(eng), stream_(stream ? stream : eng->stream()), diis_m_(diis_m) {
  if (diis_m_ < 0 || diis_m_ > kMaxDiis) throw std::invalid_argument("diis_num_error_vect out of range (0..8)");
  if (mols.empty()) throw std::invalid_argument("empty batch");
  long long mat = 0, vec = 0;
  for (size_t m = 0; m < mols.size(); ++m) {
    MolLayout L = layout_molecule(mols[m]);
    DevMol dm;
    std::memset(&dm, 0, sizeof(dm));
    dm.natoms = (int)L.atoms.size();
    dm.theory = mols[m].theory;
    dm.atom0 = (int)h_atoms.size();
    dm.pair0 = (int)h_pairs.size();
    dm.nao = L.nao;
    dm.nocc = L.nocc;
    for (DevAtom a : L.atoms) { a.mol = (int)m; h_atoms.push_back(a); }
    for (DevPair p : L.pairs) {
      p.a += dm.atom0; p.b += dm.atom0; p.mol = (int)m; p.blk += blk_total_;
      h_pairs.push_back(p);
    }
    blk_total_ += L.blocks;
    dm.npairs = (int)L.pairs.size();
    dm.nepc = (int)(mols[m].epc.size() / 4);
    dm.epc0 = (long long)(h_epc.size() / 4);
    h_epc.insert(h_epc.end(), mols[m].epc.begin(), mols[m].epc.end());
    dm.mat0 = mat;
    dm.vec0 = vec;
    mat += round32((long long)L.nao * L.nao);
    vec += round32(L.nao);
    max_n_ = std::max(max_n_, L.nao);
    h_mols.push_back(dm);
  }
  BatchCapacity cap;
  cap.slots = (int)h_mols.size();
  cap.atoms = (long long)h_atoms.size();
  cap.pairs = (long long)h_pairs.size();
  cap.blocks = blk_total_;
  cap.mat = mat;
  cap.vec = vec;
  cap.epcs = (long long)(h_epc.size() / 4);
  cap.max_n = max_n_;
  cap.ws_slots = cap.slots;
  allocate(cap);
  const int nm = (int)h_mols.size();
  cuda_check(cudaMemcpyAsync(d_atoms, h_atoms.data(), h_atoms.size() * sizeof(DevAtom), cudaMemcpyHostToDevice, stream_), "upload atoms");
  if (!h_epc.empty())
    cuda_check(cudaMemcpyAsync(d_epc, h_epc.data(), h_epc.size() * sizeof(double), cudaMemcpyHostToDevice, stream_), "upload point charges");
  if (!h_pairs.empty())
    cuda_check(cudaMemcpyAsync(d_pairs, h_pairs.data(), h_pairs.size() * sizeof(DevPair), cudaMemcpyHostToDevice, stream_), "upload pairs");
  cuda_check(cudaMemcpyAsync(d_mols, h_mols.data(), nm * sizeof(DevMol), cudaMemcpyHostToDevice, stream_), "upload mols");
  cuda_check(cudaStreamSynchronize(stream_), "upload batch");
}

Batch::Batch(Engine* eng, const BatchCapacity& cap, int diis_m, cudaStream_t stream)
    : eng_(eng), stream_(stream ? stream : eng->stream()), diis_m_(diis_m) {
  if (diis_m_ < 0 || diis_m_ > kMaxDiis) throw std::invalid_argument("diis_num_error_vect out of range (0..8)");
  if (cap.slots < 1 || cap.mat < 1 || cap.max_n < 1) throw std::invalid_argument("empty pool capacity");
  pool_ = true;
  max_n_ = cap.max_n;
  allocate(cap);
  h_atoms.assign(cap.atoms, DevAtom{});
  h_pairs.assign(cap.pairs, DevPair{});
  h_epc.assign(4 * (size_t)cap.epcs, 0.0);
  DevMol empty;
  std::memset(&empty, 0, sizeof(empty));
  h_mols.assign(cap.slots, empty);
  slot_blocks_.assign(cap.slots, 0);
  a_atoms_.reset(cap.atoms);
  a_pairs_.reset(cap.pairs);
  a_blocks_.reset(cap.blocks);
  a_mat_.reset(cap.mat);
  a_vec_.reset(cap.vec);
  a_epc_.reset(cap.epcs);
  for (int k = cap.slots - 1; k >= 0; --k) free_slots_.push_back(k);
  cuda_check(cudaMemcpyAsync(d_mols, h_mols.data(), cap.slots * sizeof(DevMol), cudaMemcpyHostToDevice, stream_), "upload mols");
  cuda_check(cudaStreamSynchronize(stream_), "pool init");
}

void Batch::allocate(const BatchCapacity& cap) {
  cap_ = cap;
  const int nm = cap.slots;
  const long long mat = cap.mat, vec = cap.vec;
  mat_total_ = mat;
  vec_total_ = vec;
  d_atoms = dalloc<DevAtom>(cap.atoms, &bytes_);
  d_epc = dalloc<double>(4 * (size_t)cap.epcs, &bytes_);
  d_pairs = dalloc<DevPair>(cap.pairs, &bytes_);
  d_mols = dalloc<DevMol>(nm, &bytes_);
  d_list = dalloc<int>(nm, &bytes_);
  d_blocks = dalloc<double>(cap.blocks, &bytes_);
  d_ecore_pair = dalloc<double>(cap.pairs, &bytes_);
  d_heavy_pairs = dalloc<int>(cap.pairs, &bytes_);
  d_light_pairs = dalloc<int>(cap.pairs, &bytes_);
  d_H = dalloc<double>(mat, &bytes_);
  d_F = dalloc<double>(mat, &bytes_);
  d_P = dalloc<double>(mat, &bytes_);
  d_Pold = dalloc<double>(mat, &bytes_);
  d_C = dalloc<double>(mat, &bytes_);
  d_eps = dalloc<double>(vec, &bytes_);
  d_hist_dens = dalloc<double>((size_t)std::max(diis_m_, 1) * mat, &bytes_);
  d_hist_err = dalloc<double>((size_t)std::max(diis_m_, 1) * mat, &bytes_);
  d_G32 = dalloc<float>(mat, &bytes_);
  d_T32 = dalloc<float>(mat, &bytes_);
  d_Cf = dalloc<float>(mat, &bytes_);
  d_Cnf = dalloc<float>(mat, &bytes_);
  d_Ff = dalloc<float>(mat, &bytes_);
  d_G64 = dalloc<double>(mat, &bytes_);
  d_T64 = dalloc<double>(mat, &bytes_);
  for (int i = 0; i < 6; ++i) d_S[i] = dalloc<double>(mat, &bytes_);
  d_td = dalloc<double>(3 * (size_t)vec, &bytes_);
  d_hh_small_ = dalloc<int>(nm, &bytes_);
  d_hh_large_ = dalloc<int>(nm, &bytes_);
  grid_ctas_ = hh_grid_ctas();
  d_gridmap_ = dalloc<int>(3 * ((size_t)nm + grid_ctas_), &bytes_);
  cuda_check(cudaHostAlloc(&h_gridmap_, sizeof(int) * 3 * ((size_t)nm + grid_ctas_), cudaHostAllocDefault),
             "cudaHostAlloc");
  d_gridbar_ = dalloc<unsigned>(4 * (size_t)grid_ctas_, &bytes_);
  d_state = dalloc<MolState>(nm, &bytes_);
  d_charges = dalloc<double>(cap.atoms, &bytes_);
  d_sweeps = dalloc<int>(nm, &bytes_);
  d_count = dalloc<int>(1, &bytes_);
  d_tc_err = dalloc<int>(1, &bytes_);
  {
    const size_t b = diis_scratch_bytes(nm);
    cuda_check(cudaMalloc(&d_diis_ws, b), "cudaMalloc DIIS scratch");
    bytes_ += b;
  }
  d_dip_ws = dalloc<double>((size_t)nm * kDipChunks * 4, &bytes_);
  d_active = dalloc<char>(nm, &bytes_);
  cuda_check(cudaMemsetAsync(d_state, 0, nm * sizeof(MolState), stream_), "memset state");
  cuda_check(cudaMemsetAsync(d_sweeps, 0, nm * sizeof(int), stream_), "memset sweeps");
  cuda_check(cudaMemsetAsync(d_tc_err, 0, sizeof(int), stream_), "memset tc err");
  cuda_check(cudaMemsetAsync(d_H, 0, mat * sizeof(double), stream_), "memset H");
  cuda_check(cudaMemsetAsync(d_P, 0, mat * sizeof(double), stream_), "memset P");
  cuda_check(cudaMemsetAsync(d_hist_dens, 0, std::max(diis_m_, 1) * mat * sizeof(double), stream_), "memset hist");
  cuda_check(cudaMemsetAsync(d_hist_err, 0, std::max(diis_m_, 1) * mat * sizeof(double), stream_), "memset hist");
  // Jacobi workspaces: the one-CTA kernel spills V (and A) of FP64 bases above
  // 138 to global memory; bases above kSmallJacobiMaxN use the block Jacobi
  bool ag, vg;
  const int small_n = std::min(cap.max_n, kSmallJacobiMaxN);
  const long long np = (small_n + 3) & ~3;   // the Jacobi working size (see jacobi.cu)
  jws_stride_ = np * np;
  const int ws = std::max(1, std::min(cap.ws_slots, nm));
  if (jacobi_needs_workspace(small_n, 4, &ag, &vg)) {
    d_jA32 = dalloc<float>(ag ? (size_t)ws * jws_stride_ : 1, &bytes_);
    d_jV32 = dalloc<float>((size_t)ws * jws_stride_, &bytes_);
  }
  if (jacobi_needs_workspace(small_n, 8, &ag, &vg)) {
    d_jA64 = dalloc<double>(ag ? (size_t)ws * jws_stride_ : 1, &bytes_);
    d_jV64 = dalloc<double>((size_t)ws * jws_stride_, &bytes_);
  }
  if (cap.max_n > kSmallJacobiMaxN) {
    long long st, qst;
    const size_t b = block_jacobi_workspace(cap.max_n, ws, (int)sizeof(double), &st, &qst);
    cuda_check(cudaMalloc(&d_bj_ws, b), "cudaMalloc block-Jacobi workspace");
    bytes_ += b;
  }
  cuda_check(cudaHostAlloc(&h_bj_pending, sizeof(int), cudaHostAllocDefault), "cudaHostAlloc");
  cuda_check(cudaHostAlloc(&h_block_count_, 2 * sizeof(int), cudaHostAllocDefault), "cudaHostAlloc");
  cuda_check(cudaHostAlloc(&h_block_active_, 2 * (size_t)nm, cudaHostAllocDefault), "cudaHostAlloc");
  for (int k = 0; k < 2; ++k)
    cuda_check(cudaEventCreateWithFlags(&block_ev_[k], cudaEventDisableTiming), "cudaEventCreate");
  cap_.ws_slots = ws;
  // persistent job tables and lists: one job per molecule per GEMM kind
  job_cap_ = nm;
  JobSet* all[] = {&j_trans1_, &j_trans2_, &j_dens_, &j_w_, &j_kt_, &j_yt_, &j_m_, &j_d2_, &j_z_, &j_p_, &j_ns1_, &j_ns2_, &j_ov_, &j_hh_};
  for (JobSet* j : all) { j->d = dalloc<GemmJob>(job_cap_, &bytes_); j->cap = job_cap_; }
  cuda_check(cudaHostAlloc(&h_jobs_, sizeof(GemmJob) * (size_t)job_cap_ * 14, cudaHostAllocDefault), "cudaHostAlloc jobs");
  cuda_check(cudaHostAlloc(&h_lists_, sizeof(int) * (size_t)nm * (kJacobiBuckets + 3), cudaHostAllocDefault),
             "cudaHostAlloc lists");
  for (int b = 0; b < kJacobiBuckets; ++b) d_bucket_lists_.push_back(dalloc<int>(nm, &bytes_));
  cuda_check(cudaStreamSynchronize(stream_), "allocate");
}

int Batch::admit(const MoleculeInput& in) {
  if (!pool_) throw std::logic_error("admit on a fixed batch");
  MolLayout L = layout_molecule(in);
  if (L.nao > cap_.max_n) throw std::invalid_argument("molecule larger than the pool's largest basis");
  if ((long long)(in.epc.size() / 4) > cap_.epcs) throw std::invalid_argument("more point charges than the pool holds");
  if (free_slots_.empty()) return -1;
  const long long na = (long long)L.atoms.size(), npr = (long long)L.pairs.size();
  const long long nmat = round32((long long)L.nao * L.nao), nvec = round32(L.nao);
  const long long oa = a_atoms_.alloc(na);
  if (oa < 0) return -1;
  const long long op = a_pairs_.alloc(npr);
  if (op < 0) { a_atoms_.release(oa, na); return -1; }
  const long long ob = a_blocks_.alloc(L.blocks);
  if (ob < 0) { a_atoms_.release(oa, na); a_pairs_.release(op, npr); return -1; }
  const long long om = a_mat_.alloc(nmat);
  if (om < 0) { a_atoms_.release(oa, na); a_pairs_.release(op, npr); a_blocks_.release(ob, L.blocks); return -1; }
  const long long ov = a_vec_.alloc(nvec);
  if (ov < 0) {
    a_atoms_.release(oa, na); a_pairs_.release(op, npr); a_blocks_.release(ob, L.blocks); a_mat_.release(om, nmat);
    return -1;
  }
  const long long ne = (long long)(in.epc.size() / 4);
  const long long oe = ne > 0 ? a_epc_.alloc(ne) : 0;
  if (oe < 0) {
    a_atoms_.release(oa, na); a_pairs_.release(op, npr); a_blocks_.release(ob, L.blocks); a_mat_.release(om, nmat);
    a_vec_.release(ov, nvec);
    return -1;
  }
  const int slot = free_slots_.back();
  free_slots_.pop_back();
  DevMol dm;
  std::memset(&dm, 0, sizeof(dm));
  dm.natoms = (int)na;
  dm.nao = L.nao;
  dm.nocc = L.nocc;
  dm.theory = in.theory;
  dm.atom0 = (int)oa;
  dm.pair0 = (int)op;
  dm.npairs = (int)npr;
  dm.mat0 = om;
  dm.vec0 = ov;
  dm.nepc = (int)ne;
  dm.epc0 = oe;
  for (long long a = 0; a < na; ++a) { DevAtom x = L.atoms[a]; x.mol = slot; h_atoms[oa + a] = x; }
  std::copy(in.epc.begin(), in.epc.end(), h_epc.begin() + 4 * oe);
  for (long long k = 0; k < npr; ++k) {
    DevPair p = L.pairs[k];
    p.a += (int)oa; p.b += (int)oa; p.mol = slot; p.blk += ob;
    h_pairs[op + k] = p;
  }
  h_mols[slot] = dm;
  slot_blocks_[slot] = L.blocks;
  // a slot number can now stand for a different molecule: the job tables and
  // size buckets of any cached list are stale
  cur_list_.clear();
  buckets_.clear();
  cuda_check(cudaMemcpyAsync(d_atoms + oa, &h_atoms[oa], na * sizeof(DevAtom), cudaMemcpyHostToDevice, stream_), "upload atoms");
  if (npr) cuda_check(cudaMemcpyAsync(d_pairs + op, &h_pairs[op], npr * sizeof(DevPair), cudaMemcpyHostToDevice, stream_), "upload pairs");
  if (ne)
    cuda_check(cudaMemcpyAsync(d_epc + 4 * oe, &h_epc[4 * oe], 4 * ne * sizeof(double), cudaMemcpyHostToDevice, stream_),
               "upload point charges");
  cuda_check(cudaMemcpyAsync(d_mols + slot, &h_mols[slot], sizeof(DevMol), cudaMemcpyHostToDevice, stream_), "upload mol");
  return slot;
}

void Batch::release(int slot) {
  if (!pool_ || slot < 0 || slot >= (int)h_mols.size() || h_mols[slot].natoms == 0) return;
  DevMol& d = h_mols[slot];
  const long long n = d.nao;
  a_atoms_.release(d.atom0, d.natoms);
  a_pairs_.release(d.pair0, d.npairs);
  if (d.npairs > 0) a_blocks_.release(h_pairs[d.pair0].blk, slot_blocks_[slot]);
  a_mat_.release(d.mat0, round32(n * n));
  a_vec_.release(d.vec0, round32(n));
  if (d.nepc > 0) a_epc_.release(d.epc0, d.nepc);
  std::memset(&d, 0, sizeof(d));
  slot_blocks_[slot] = 0;
  free_slots_.push_back(slot);
  cur_list_.clear();
  buckets_.clear();
}

Batch::~Batch() {
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  for (cudaEvent_t e : block_ev_) if (e) cudaEventDestroy(e);
  if (h_block_count_) cudaFreeHost(h_block_count_);
  if (h_block_active_) cudaFreeHost(h_block_active_);
  free_jobs();
  for (cudaEvent_t e : ev_pool_) cudaEventDestroy(e);
  for (int* p : d_bucket_lists_) cudaFree(p);
  if (h_jobs_) cudaFreeHost(h_jobs_);
  if (h_lists_) cudaFreeHost(h_lists_);
  if (h_bj_pending) cudaFreeHost(h_bj_pending);
  if (d_bj_ws) cudaFree(d_bj_ws);
  if (d_diis_ws) cudaFree(d_diis_ws);
  void* ptrs[] = {d_atoms, d_epc, d_pairs, d_mols, d_list, d_blocks, d_ecore_pair, d_H, d_F, d_P, d_Pold, d_C, d_eps,
                  d_hist_dens, d_hist_err, d_G32, d_T32, d_Cf, d_Cnf, d_Ff, d_G64, d_T64, d_jA32, d_jV32, d_jA64, d_jV64,
                  d_state, d_trace, d_charges, d_sweeps, d_count, d_active, d_heavy_pairs, d_light_pairs, d_tc_err, d_dip_ws};
  for (void* p : ptrs) if (p) cudaFree(p);
  for (int i = 0; i < 6; ++i) if (d_S[i]) cudaFree(d_S[i]);
  if (d_td) cudaFree(d_td);
  void* hh[] = {d_hh_small_, d_hh_large_, d_gridmap_, d_gridbar_, d_pgrad_, d_forces_};
  for (void* p : hh) if (p) cudaFree(p);
  if (h_gridmap_) cudaFreeHost(h_gridmap_);
}

void Batch::free_jobs() {
  JobSet* all[] = {&j_trans1_, &j_trans2_, &j_dens_, &j_w_, &j_kt_, &j_yt_, &j_m_, &j_d2_, &j_z_, &j_p_, &j_ns1_, &j_ns2_, &j_ov_, &j_hh_};
  for (JobSet* j : all) { if (j->d) cudaFree(j->d); j->d = nullptr; j->n = 0; j->tiles = 0; j->cap = 0; }
}

void Batch::make_jobset(JobSet* js, const std::vector<GemmJob>& jobs_in) {
  // staging slot of this job set inside the pinned table
  JobSet* all[] = {&j_trans1_, &j_trans2_, &j_dens_, &j_w_, &j_kt_, &j_yt_, &j_m_, &j_d2_, &j_z_, &j_p_, &j_ns1_, &j_ns2_, &j_ov_, &j_hh_};
  int idx = 0;
  while (all[idx] != js) ++idx;
  GemmJob* stage = h_jobs_ + (size_t)idx * job_cap_;
  if ((int)jobs_in.size() > js->cap) throw std::logic_error("GEMM job table overflow");
  int tiles = 0, tc_tiles = 0;
  for (size_t k = 0; k < jobs_in.size(); ++k) {
    GemmJob j = jobs_in[k];
    j.tile0 = tiles;
    j.tiles_n = gemm_tiles_n(j.N);
    j.tc_tile0 = tc_tiles;
    j.tc_tiles_n = tc_gemm_tiles_n(j.N);
    if (j.M > 0 && j.N > 0) {
      tiles += j.sym ? gemm_tiles_sym(j.N) : gemm_tiles(j.M, j.N);
      tc_tiles += j.sym ? tc_gemm_tiles_sym(j.N) : tc_gemm_tiles(j.M, j.N);
    }
    stage[k] = j;
  }
  js->n = (int)jobs_in.size();
  js->tiles = tiles;
  js->tc_tiles = tc_tiles;
  if (jobs_in.empty()) return;
  cuda_check(cudaMemcpyAsync(js->d, stage, jobs_in.size() * sizeof(GemmJob), cudaMemcpyHostToDevice, stream_), "upload jobs");
}

static GemmJob job(long long a, long long b, long long c, int M, int N, int K, int lda, int ldb, int ldc, int mol,
                   double alpha = 1.0, double beta = 0.0, int sym = 0) {
  GemmJob j;
  std::memset(&j, 0, sizeof(j));
  j.a_off = a; j.b_off = b; j.c_off = c; j.M = M; j.N = N; j.K = K; j.lda = lda; j.ldb = ldb; j.ldc = ldc;
  j.mol = mol; j.alpha = alpha; j.beta = beta; j.sym = sym;
  return j;
}

void Batch::build_jobs(const std::vector<int>& which) {
  std::vector<GemmJob> t1, t2, dn, w, kt, yt, mm, d2, z, pp, ns1, ns2, ov, hh;
  for (int m : which) {
    const DevMol& d = h_mols[m];
    const int n = d.nao, o = d.nocc, v = n - o;
    const long long b = d.mat0;
    ns1.push_back(job(b, b, b, n, n, n, n, n, n, m, 1.0, 0.0, 1)); // M = C C^T        (B transposed, symmetric)
    ns2.push_back(job(b, b, b, n, n, n, n, n, n, m, -0.5, 1.5)); // C' = 1.5 C - 0.5 M C
    t1.push_back(job(b, b, b, n, n, n, n, n, n, m));            // T = F C^T          (B transposed)
    t2.push_back(job(b, b, b, n, n, n, n, n, n, m));            // G = C T
    dn.push_back(job(b, b, b, n, n, o, n, n, n, m, 2.0, 0.0, 1)); // P = 2 C_o^T C_o  (A transposed, symmetric)
    // Householder path: the density from the smaller eigenvector set, rows
    // [lo, hi) of C: P = 2 C_o^T C_o, or P = 2 I - 2 C_v^T C_v
    if (v <= o) {
      GemmJob j = job(b + (long long)o * n, b + (long long)o * n, b, n, n, v, n, n, n, m, -2.0, 0.0, 1);
      j.diag = 2.0;
      hh.push_back(j);
    } else {
      hh.push_back(job(b, b, b, n, n, o, n, n, n, m, 2.0, 0.0, 1));
    }
    if (o > 0 && v > 0) {
      w.push_back(job(b + (long long)o * n, b, b, v, n, n, n, n, n, m));   // U = C_v F  (v x n)
      kt.push_back(job(b, b, b, v, o, n, n, n, o, m));                      // Kt = U C_o^T  (B transposed)
      ov.push_back(job(b + (long long)o * n, b, b, v, o, n, n, n, o, m));   // O = C_v C_o^T (B transposed)
      yt.push_back(job(b, b + (long long)o * n, b, o, n, v, o, n, n, m, 1.0, 1.0));  // Yt = C_o + K^T C_v (A transposed)
      mm.push_back(job(b, b, b, o, o, n, n, n, o, m, 1.0, 0.0, 1));         // M = Yt Yt^T   (B transposed, symmetric)
      z.push_back(job(b, b, b, o, n, o, o, n, n, m, -1.0, 1.0));            // Z = Yt - D Yt
      pp.push_back(job(b, b, b, n, n, o, n, n, n, m, 2.0, 0.0, 1));         // P = 2 Yt^T Z  (A transposed, symmetric)
    }
  }
  make_jobset(&j_trans1_, t1); make_jobset(&j_trans2_, t2); make_jobset(&j_dens_, dn);
  make_jobset(&j_w_, w); make_jobset(&j_kt_, kt); make_jobset(&j_yt_, yt); make_jobset(&j_m_, mm);
  make_jobset(&j_d2_, d2); make_jobset(&j_z_, z); make_jobset(&j_p_, pp);
  make_jobset(&j_ns1_, ns1); make_jobset(&j_ns2_, ns2); make_jobset(&j_ov_, ov);
  make_jobset(&j_hh_, hh);
  list_max_n_ = 0;
  hh_max_k_ = 0;
  hh_small_.clear();
  hh_large_.clear();
  hh_small_max_n_ = hh_small_max_k_ = hh_large_max_n_ = hh_large_max_k_ = 0;
  // Householder path: bases above the per-molecule kernels' limit always go to
  // the whole-GPU kernels; so do bases of at least kGridShareMinN while at
  // most a quarter as many of them as SMs are in the list (each then gets
  // four or more SMs instead of one)
  const int per_molecule = hh_back_max_n();
  int n_big = 0;
  for (int m : which) n_big += h_mols[m].nao >= kGridShareMinN;
  const bool share = 4 * n_big <= grid_ctas_;
  // largest basis the per-molecule kernels serve; every larger molecule of the
  // list is tridiagonalised by the whole-GPU kernels alone
  hh_served_max_n_ = share ? std::min(per_molecule, kGridShareMinN - 1) : per_molecule;
  for (int m : which) {
    const DevMol& d = h_mols[m];
    const int kd = std::min(d.nocc, d.nao - d.nocc);
    list_max_n_ = std::max(list_max_n_, d.nao);
    hh_max_k_ = std::max(hh_max_k_, kd);
    if (d.nao <= hh_served_max_n_) {
      hh_small_.push_back(m);
      hh_small_max_n_ = std::max(hh_small_max_n_, d.nao);
      hh_small_max_k_ = std::max(hh_small_max_k_, kd);
    } else {
      hh_large_.push_back(m);
      hh_large_max_n_ = std::max(hh_large_max_n_, d.nao);
      hh_large_max_k_ = std::max(hh_large_max_k_, kd);
    }
  }
  // chunks of at most grid_ctas_ molecules and their CTA maps
  grid_chunks_.clear();
  int off = 0;
  for (int f = 0; f < (int)hh_large_.size(); f += grid_ctas_) {
    GridChunk c;
    c.first = f;
    c.count = std::min(grid_ctas_, (int)hh_large_.size() - f);
    std::vector<int> ns(c.count);
    c.max_k = 0;
    for (int i = 0; i < c.count; ++i) {
      const DevMol& d = h_mols[hh_large_[f + i]];
      ns[i] = d.nao;
      c.max_k = std::max(c.max_k, std::min(d.nocc, d.nao - d.nocc));
    }
    c.map_off = off;
    c.nctas = hh_grid_assign(ns.data(), c.count, grid_ctas_, h_gridmap_ + off);
    off += 3 * c.nctas;
    grid_chunks_.push_back(c);
  }
}

void Batch::upload_list(const std::vector<int>& which) {
  if (which == cur_list_ && !buckets_.empty()) return;
  if ((int)which.size() > cap_.slots) throw std::logic_error("molecule list longer than the slot table");
  // the pinned staging buffers may still feed copies of the previous list
  cuda_check(cudaStreamSynchronize(stream_), "list staging");
  cur_list_ = which;
  // every launch shape of an iteration (grids, shared memory, job tables)
  // follows from this rebuild: a captured graph is only valid for this layout
  ++layout_version_;
  const int nm = cap_.slots;
  std::copy(which.begin(), which.end(), h_lists_);
  if (!which.empty())
    cuda_check(cudaMemcpyAsync(d_list, h_lists_, which.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), "upload list");
  build_jobs(which);
  {
    // the Householder path's two lists (staged behind the bucket lists)
    int* stage = h_lists_ + (size_t)(kJacobiBuckets + 1) * nm;
    std::copy(hh_small_.begin(), hh_small_.end(), stage);
    std::copy(hh_large_.begin(), hh_large_.end(), stage + nm);
    if (!hh_small_.empty())
      cuda_check(cudaMemcpyAsync(d_hh_small_, stage, hh_small_.size() * sizeof(int), cudaMemcpyHostToDevice, stream_),
                 "upload list");
    if (!hh_large_.empty()) {
      cuda_check(cudaMemcpyAsync(d_hh_large_, stage + nm, hh_large_.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 stream_),
                 "upload list");
      const GridChunk& last = grid_chunks_.back();
      cuda_check(cudaMemcpyAsync(d_gridmap_, h_gridmap_, sizeof(int) * (last.map_off + 3 * last.nctas),
                                 cudaMemcpyHostToDevice, stream_),
                 "upload grid map");
    }
  }
  // Jacobi size buckets: smaller molecules get a smaller shared-memory
  // footprint; the first edge keeps bases below the cluster Jacobi's minimum
  // apart from the ones it serves, so a molecule's kernel follows its own size
  buckets_.clear();
  bucket_max_n_.clear();
  bucket_hh_max_n_.clear();
  bucket_dev_.clear();
  const int edges[kJacobiBuckets] = {kClusterJacobiMinN - 1, 64, 96, 128, 160, 194, 256, 338, 1 << 30};
  int lo = 0, bi = 0;
  for (int hi : edges) {
    std::vector<int> b;
    int mx = 0, mx_hh = 0;
    for (int m : which) {
      const int n = h_mols[m].nao;
      if (n > lo && n <= hi) {
        b.push_back(m);
        mx = std::max(mx, n);
        if (n <= hh_served_max_n_) mx_hh = std::max(mx_hh, n);
      }
    }
    lo = hi;
    const int slot = bi++;
    if (b.empty()) continue;
    int* stage = h_lists_ + (size_t)(slot + 1) * nm;
    std::copy(b.begin(), b.end(), stage);
    cuda_check(cudaMemcpyAsync(d_bucket_lists_[slot], stage, b.size() * sizeof(int), cudaMemcpyHostToDevice, stream_),
               "upload bucket");
    buckets_.push_back(b);
    bucket_max_n_.push_back(mx);
    bucket_hh_max_n_.push_back(mx_hh);
    bucket_dev_.push_back(d_bucket_lists_[slot]);
  }
}

int Batch::list_max_atoms() const {
  int mx = 1;
  for (int m : cur_list_) mx = std::max(mx, h_mols[m].natoms);
  return mx;
}

const char* kernel_class_name(int k) {
  static const char* names[kKNumClasses] = {"pair_integrals", "core_hamiltonian", "fock_build", "basis_orthonormalise",
                                            "warm_start_transform", "jacobi_eigensolver", "density", "fp64_refinement",
                                            "diis", "energy", "dipole", "tridiagonalisation",
                                            "tridiagonal_eigenvectors"};
  return (k >= 0 && k < kKNumClasses) ? names[k] : "?";
}

void Batch::set_profiling(bool on) {
  constexpr size_t kProfEvents = 8192;   // about 14 SCF runs of 14 iterations
  if (on)
    while (ev_pool_.size() < kProfEvents) {
      cudaEvent_t e;
      cuda_check(cudaEventCreate(&e), "cudaEventCreate");
      ev_pool_.push_back(e);
    }
  prof_on_ = on;
}

cudaEvent_t Batch::next_event() {
  if (ev_used_ == ev_pool_.size()) {
    cudaEvent_t e;
    cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    ev_pool_.push_back(e);
  }
  return ev_pool_[ev_used_++];
}

int Batch::prof_begin(int cls, double work) {
  if (!prof_on_) return -1;
  Rec r;
  r.a = next_event();
  r.b = next_event();
  r.cls = cls;
  r.work = work;
  cuda_check(cudaEventRecord(r.a, stream_), "cudaEventRecord");
  recs_.push_back(r);
  return (int)recs_.size() - 1;
}

void Batch::prof_end(int h) {
  if (h < 0) return;
  cuda_check(cudaEventRecord(recs_[h].b, stream_), "cudaEventRecord");
}

void Batch::profile_collect(double* ms, long long* launches, double* work) {
  cuda_check(cudaStreamSynchronize(stream_), "profile sync");
  for (const Rec& r : recs_) {
    float t = 0.f;
    cuda_check(cudaEventElapsedTime(&t, r.a, r.b), "cudaEventElapsedTime");
    prof_ms_[r.cls] += t;
    prof_launches_[r.cls] += 1;
    prof_work_[r.cls] += r.work;
  }
  recs_.clear();
  ev_used_ = 0;
  for (int k = 0; k < kKNumClasses; ++k) {
    if (ms) ms[k] = prof_ms_[k];
    if (launches) launches[k] = prof_launches_[k];
    if (work) work[k] = prof_work_[k];
  }
}

void Batch::profile_reset() {
  cuda_check(cudaStreamSynchronize(stream_), "profile sync");
  recs_.clear();
  ev_used_ = 0;
  for (int k = 0; k < kKNumClasses; ++k) { prof_ms_[k] = 0; prof_launches_[k] = 0; prof_work_[k] = 0; }
}

// Algorithmic work of one launch over the molecules that are still active:
// FLOPs for the contractions and the eigensolver (eigensolve counted as
// 10/3 N^3 whatever the method), bytes for the memory-bound steps.
double Batch::active_work_estimate(int cls) const {
  double w = 0.0;
  for (int m : cur_list_) {
    if (!active_host_.empty() && !active_host_[m]) continue;
    const DevMol& d = h_mols[m];
    const double n = d.nao, o = d.nocc, v = n - o;
    switch (cls) {
      case kKJacobi: w += 10.0 / 3.0 * n * n * n; break;
      // the tridiagonalisation share of the (10/3) N^3 eigensolver convention
      case kKTridiag: w += 4.0 / 3.0 * n * n * n; break;
      // back-transformation of the k = min(o, v) density vectors (2 N^2 k flops)
      case kKEigvec: w += 2.0 * n * n * std::min(o, v); break;
      case kKTransform: w += 4.0 * n * n * n; break;
      case kKOrtho: w += 4.0 * n * n * n; break;
      case kKDensity: w += 2.0 * n * n * o; break;
      case kKRefine: w += 2 * v * n * n + 4 * n * v * o + 2 * n * o * o + 2 * n * n * o; break;   // FP64 products
      case kKDiis: w += 8.0 * n * n * (2.0 * diis_m_ + 3.0); break;
      case kKFock: {
        double blk = 0.0;
        for (int k = 0; k < d.npairs; ++k) {
          const DevPair& p = h_pairs[d.pair0 + k];
          blk += (h_atoms[p.a].nao == 4 ? 10 : 1) * (h_atoms[p.b].nao == 4 ? 10 : 1);
        }
        w += 8.0 * blk + 16.0 * n * n;
        break;
      }
      default: break;
    }
  }
  return w;
}

long long Batch::jacobi_sweeps() const {
  std::vector<int> h(h_mols.size());
  cuda_check(cudaMemcpyAsync(h.data(), d_sweeps, h.size() * sizeof(int), cudaMemcpyDeviceToHost, stream_), "sweeps");
  cuda_check(cudaStreamSynchronize(stream_), "sweeps");
  long long t = 0;
  for (int v : h) t += v;
  return t;
}

void Batch::set_coordinates(const double* xyz) {
  for (size_t a = 0; a < h_atoms.size(); ++a) {
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(xyz[3 * a + k])) throw std::invalid_argument("non-finite coordinate");
    h_atoms[a].x = xyz[3 * a]; h_atoms[a].y = xyz[3 * a + 1]; h_atoms[a].z = xyz[3 * a + 2];
  }
  for (const DevPair& p : h_pairs) {
    const DevAtom& A = h_atoms[p.a];
    const DevAtom& B = h_atoms[p.b];
    if (A.x == B.x && A.y == B.y && A.z == B.z) throw std::invalid_argument("two atoms at the same position");
  }
  cuda_check(cudaMemcpyAsync(d_atoms, h_atoms.data(), h_atoms.size() * sizeof(DevAtom), cudaMemcpyHostToDevice, stream_),
             "upload atoms");
}

void Batch::set_molecule_coordinates(int m, const double* xyz) {
  if (m < 0 || m >= (int)h_mols.size()) throw std::invalid_argument("molecule index out of range");
  const DevMol& d = h_mols[m];
  for (int a = 0; a < 3 * d.natoms; ++a)
    if (!std::isfinite(xyz[a])) throw std::invalid_argument("non-finite coordinate");
  for (int k = 0; k < d.npairs; ++k) {
    const DevPair& p = h_pairs[d.pair0 + k];
    const double* A = xyz + 3 * (p.a - d.atom0);
    const double* B = xyz + 3 * (p.b - d.atom0);
    if (A[0] == B[0] && A[1] == B[1] && A[2] == B[2]) throw std::invalid_argument("two atoms at the same position");
  }
  for (int a = 0; a < d.natoms; ++a) {
    DevAtom& at = h_atoms[d.atom0 + a];
    at.x = xyz[3 * a]; at.y = xyz[3 * a + 1]; at.z = xyz[3 * a + 2];
  }
  cuda_check(cudaMemcpyAsync(d_atoms + d.atom0, h_atoms.data() + d.atom0, d.natoms * sizeof(DevAtom),
                             cudaMemcpyHostToDevice, stream_), "upload atoms");
}

void Batch::integrals() {
  std::vector<int> all(h_mols.size());
  for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
  integrals(all);
}

void Batch::integrals(const std::vector<int>& which) {
  if (which.empty()) return;
  upload_list(which);
  // pair index lists of the listed molecules: sp-sp pairs for the warp kernel,
  // X-H then H-H pairs for the thread-per-pair kernel
  std::vector<int> heavy, xh, hh;
  double blk = 0.0;
  for (int m : which) {
    const DevMol& d = h_mols[m];
    for (int k = 0; k < d.npairs; ++k) {
      const int pi = d.pair0 + k;
      const int na = h_atoms[h_pairs[pi].a].nao, nb = h_atoms[h_pairs[pi].b].nao;
      blk += (double)((na == 4 ? 10 : 1) * (nb == 4 ? 10 : 1));
      if (na == 4 && nb == 4) heavy.push_back(pi);
      else if (na == 4 || nb == 4) xh.push_back(pi);
      else hh.push_back(pi);
    }
  }
  xh.insert(xh.end(), hh.begin(), hh.end());
  n_heavy_ = (long long)heavy.size();
  n_light_ = (long long)xh.size();
  if (!heavy.empty())
    cuda_check(cudaMemcpyAsync(d_heavy_pairs, heavy.data(), heavy.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), "upload heavy pairs");
  if (!xh.empty())
    cuda_check(cudaMemcpyAsync(d_light_pairs, xh.data(), xh.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), "upload light pairs");
  int h = prof_begin(kKPair, 8.0 * blk);
  launches_ += 2;
  launch_pair_kernels_split(d_atoms, d_pairs, d_heavy_pairs, n_heavy_, d_light_pairs, n_light_, d_mols, eng_->eri(),
                            eng_->ovt(), d_blocks, d_H, d_ecore_pair, stream_);
  prof_end(h);
  cuda_check(cudaGetLastError(), "pair_kernel");
  h = prof_begin(kKHcore, 0.0);
  launches_ += 1;
  launch_hcore_kernel(d_atoms, d_pairs, d_mols, d_list, (int)which.size(), d_blocks, d_ecore_pair, eng_->eri(), d_epc,
                      d_H, d_state, stream_);
  prof_end(h);
  cuda_check(cudaGetLastError(), "hcore_kernel");
  // the pageable index vectors above must outlive their copies
  cuda_check(cudaStreamSynchronize(stream_), "integrals");
}

static ScfParamsDev to_dev(const ScfSettings& s) {
  ScfParamsDev p;
  std::memset(&p, 0, sizeof(p));
  p.max_iter = s.max_iter;
  p.diis_m = s.diis_num_error_vect;
  p.rms_density = s.rms_density;
  p.damping_thresh = s.damping_thresh;
  p.damping_weight = s.damping_weight;
  p.diis_start = s.diis_start_error;
  p.diis_end = s.diis_end_error;
  p.switch_error = s.switch_error;
  p.precision = s.precision;
  return p;
}

void Batch::begin(const ScfSettings& s, const std::vector<int>& which, bool requires_guess) {
  if (s.diis_num_error_vect != diis_m_) throw std::invalid_argument("DIIS window differs from the batch allocation");
  if (s.keep_trace && s.max_iter > max_iter_alloc_) {
    if (d_trace) cudaFree(d_trace);
    cuda_check(cudaMalloc(&d_trace, (size_t)h_mols.size() * s.max_iter * sizeof(TraceEntry)), "cudaMalloc trace");
    max_iter_alloc_ = s.max_iter;
  }
  if (which.empty()) return;
  upload_list(which);
  active_host_.resize(h_mols.size(), 0);
  for (int m : which) active_host_[m] = 1;
  launches_ += 1;
  init_state_kernel<<<(unsigned)which.size(), 256, 0, stream_>>>(d_mols, d_list, (int)which.size(), d_state, d_C,
                                                                 d_P, d_eps, requires_guess ? 1 : 0, requires_guess ? 1 : 0,
                                                                 d_hist_dens, d_hist_err, diis_m_, mat_total_, d_sweeps);
  cuda_check(cudaGetLastError(), "init_state");
}

// One Jacobi launch per size bucket; buckets whose molecules need a
// global-memory workspace are split into launches of at most ws_slots CTAs.
bool Batch::cluster_jacobi(int b) const {
  return bucket_max_n_[b] >= kClusterJacobiMinN && bucket_max_n_[b] <= kSmallJacobiMaxN &&
         (int)buckets_[b].size() <= kClusterJacobiMaxMols && jacobi_cluster_capacity(bucket_max_n_[b]) > 0;
}

void Batch::run_jacobi(bool fp32, const ScfSettings& s, const double* Cin, const float* Cin32, const double* F) {
  for (size_t b = 0; b < buckets_.size(); ++b) {
    bool ag, vg;
    const int nb = (int)buckets_[b].size();
    if (bucket_max_n_[b] > kSmallJacobiMaxN) {
      // block Jacobi, many CTAs per molecule, at most ws_slots molecules per call
      for (int k0 = 0; k0 < nb; k0 += cap_.ws_slots) {
        const int cnt = std::min(cap_.ws_slots, nb - k0);
        if (fp32 && Cin32)
          launches_ += launch_block_jacobi_f32(d_mols, bucket_dev_[b] + k0, cnt, bucket_max_n_[b], d_state, d_G32,
                                               Cin32, d_C, d_eps, d_bj_ws, s.max_sweeps, d_sweeps, h_bj_pending,
                                               stream_);
        else if (fp32)
          launches_ += launch_block_jacobi_f32(d_mols, bucket_dev_[b] + k0, cnt, bucket_max_n_[b], d_state, d_G32, Cin,
                                               d_C, d_eps, d_bj_ws, s.max_sweeps, d_sweeps, h_bj_pending, stream_);
        else
          launches_ += launch_block_jacobi_f64(d_mols, bucket_dev_[b] + k0, cnt, bucket_max_n_[b], d_state, d_G64, Cin,
                                               d_C, d_eps, d_bj_ws, s.max_sweeps, d_sweeps, h_bj_pending, stream_);
      }
      continue;
    }
    // FP64, few molecules (the plain one-molecule path): one cluster of CTAs
    // per molecule puts several SMs' FP64 units on each diagonalisation
    if (!fp32 && cluster_jacobi((int)b)) {
      launches_ += 1;
      launch_jacobi_cluster_f64(d_mols, bucket_dev_[b], nb, bucket_max_n_[b], d_state, 1, F ? nullptr : d_G64, F, Cin,
                                1, d_C, d_eps, s.max_sweeps, d_sweeps, stream_);
      continue;
    }
    const int chunk = jacobi_needs_workspace(bucket_max_n_[b], fp32 ? 4 : 8, &ag, &vg) ? cap_.ws_slots : nb;
    for (int k0 = 0; k0 < nb; k0 += chunk) {
      const int cnt = std::min(chunk, nb - k0);
      launches_ += 1;
      if (fp32 && Cin32)
        launch_jacobi_f32(d_mols, bucket_dev_[b] + k0, cnt, bucket_max_n_[b], d_state, 1, d_G32, Cin32, 1, d_C, d_eps,
                          d_jA32, d_jV32, jws_stride_, s.max_sweeps, d_sweeps, stream_);
      else if (fp32)
        launch_jacobi_f32(d_mols, bucket_dev_[b] + k0, cnt, bucket_max_n_[b], d_state, 1, d_G32, Cin, 1, d_C, d_eps,
                          d_jA32, d_jV32, jws_stride_, s.max_sweeps, d_sweeps, stream_);
      else
        launch_jacobi_f64(d_mols, bucket_dev_[b] + k0, cnt, bucket_max_n_[b], d_state, 1, d_G64, Cin, 1, d_C, d_eps,
                          d_jA64, d_jV64, jws_stride_, s.max_sweeps, d_sweeps, stream_);
    }
  }
}

bool Batch::householder(const ScfSettings& s) const {
  return s.eigensolver != 1 && list_max_n_ <= hh_grid_max_n();
}

void Batch::hh_vectors(const ScfSettings& s, int final_pass, int require_active) {
  const int mixed = s.precision == 1 ? 1 : 0;
  if (!hh_small_.empty()) {
    const int max_k = final_pass ? hh_small_max_n_ : hh_small_max_k_;
    launches_ += (mixed && !final_pass) ? 4 : 3;
    launch_hh_vectors(d_mols, d_hh_small_, (int)hh_small_.size(), hh_small_max_n_, max_k, d_state, require_active,
                      final_pass, mixed, d_G64, d_td, vec_total_, d_eps, d_T64, d_S, d_C, d_Cf, stream_);
  }
  if (!hh_large_.empty()) {
    const int nl = (int)hh_large_.size();
    const int max_k = final_pass ? hh_large_max_n_ : hh_large_max_k_;
    launches_ += 1;
    launch_tri_vectors(d_mols, d_hh_large_, nl, hh_large_max_n_, max_k, d_state, require_active, final_pass, d_td,
                       vec_total_, d_eps, d_T64, d_S, stream_);
    for (const GridChunk& c : grid_chunks_) {
      launches_ += 1;
      launch_hh_grid_orth(d_mols, d_hh_large_ + c.first, d_gridmap_ + c.map_off, c.nctas, c.count,
                          final_pass ? hh_large_max_n_ : c.max_k, d_state, require_active, final_pass, d_td,
                          vec_total_, d_eps, d_T64, d_S[5], d_gridbar_, stream_);
    }
    launches_ += (mixed && !final_pass) ? 2 : 1;
    launch_hh_grid_back(d_mols, d_hh_large_, nl, hh_large_max_n_, max_k, d_state, require_active, final_pass, mixed,
                        d_G64, d_td, vec_total_, d_T64, d_C, d_Cf, stream_);
  }
}

void Batch::eigen_step(const ScfSettings& s) {
  if (householder(s)) {
    // FP64 Householder tridiagonalisation (one launch per size bucket, each
    // with its own shared-memory footprint), then the density's eigenpairs
    int h = prof_begin(kKTridiag, active_work_estimate(kKTridiag));
    for (size_t b = 0; b < buckets_.size(); ++b) {
      if (bucket_hh_max_n_[b] == 0) continue;
      launches_ += 1;
      launch_hh_tridiag(d_mols, bucket_dev_[b], (int)buckets_[b].size(), bucket_hh_max_n_[b], d_state, 1, d_F, d_G64,
                        d_td, vec_total_, d_S[4], hh_served_max_n_, stream_);
    }
    // the whole-GPU path: each chunk's molecules share one cooperative launch
    for (const GridChunk& c : grid_chunks_) {
      launches_ += 1;
      launch_hh_grid_tridiag(d_mols, d_hh_large_ + c.first, d_gridmap_ + c.map_off, c.nctas, c.count, d_state, 1,
                             d_F, d_G64, d_td, vec_total_, d_S[4], d_S[5], d_gridbar_, stream_);
    }
    prof_end(h);
    h = prof_begin(kKEigvec, active_work_estimate(kKEigvec));
    hh_vectors(s, 0, 1);
    prof_end(h);
  } else if (s.precision == 0) {
    // size buckets on the cluster Jacobi (a few molecules) form G = C F C^T
    // inside it on the cluster's SMs; the transform GEMMs run only when some
    // bucket uses the one-CTA Jacobi (a molecule's path depends on its bucket
    // alone, not on whether other buckets need the GEMMs)
    bool gemms = false;
    for (size_t b = 0; b < buckets_.size(); ++b) gemms = gemms || !cluster_jacobi((int)b);
    if (gemms) {
      int h = prof_begin(kKTransform, active_work_estimate(kKTransform));
      launches_ += 2;
      launch_gemm(j_trans1_.d, j_trans1_.n, j_trans1_.tiles, d_F, d_C, d_T64, false, true, 0.0, d_state, 1, -1, stream_);
      launch_gemm(j_trans2_.d, j_trans2_.n, j_trans2_.tiles, d_C, d_T64, d_G64, false, false, 0.0, d_state, 1, -1,
                  stream_);
      prof_end(h);
    }
    int h = prof_begin(kKJacobi, active_work_estimate(kKJacobi));
    run_jacobi(false, s, d_C, nullptr, d_F);
    prof_end(h);
  } else {
    // The FP32 rotations of each iteration erode the orthonormality of the
    // warm-start basis; one Newton-Schulz step C <- 1.5 C - 0.5 (C C^T) C
    // (FP32 accumulation) restores it to FP32 round-off before it is reused.
    if (s.tensor_cores) {
      // tensor-core chain on FP32 shadows: Cf = Cnf = float(C), Ff = float(F);
      // M = Cf Cf^T, Cnf = 1.5 Cnf - 0.5 M Cf, T = Ff Cnf^T, G = Cnf T
      launches_ += 6;
      int h = prof_begin(kKOrtho, active_work_estimate(kKOrtho));
      launch_tc_shadows(d_mols, d_list, (int)cur_list_.size(), d_state, d_C, d_F, d_Cf, d_Cnf, d_Ff, stream_);
      launch_tc_gemm(j_ns1_.d, j_ns1_.n, j_ns1_.tc_tiles, d_Cf, d_Cf, d_T32, false, true, d_state, 1, -1, d_tc_err,
                     stream_);
      launch_tc_gemm(j_ns2_.d, j_ns2_.n, j_ns2_.tc_tiles, d_T32, d_Cf, d_Cnf, false, false, d_state, 1, -1, d_tc_err,
                     stream_);
      prof_end(h);
      h = prof_begin(kKTransform, active_work_estimate(kKTransform));
      launch_tc_gemm(j_trans1_.d, j_trans1_.n, j_trans1_.tc_tiles, d_Ff, d_Cnf, d_T32, false, true, d_state, 1, -1,
                     d_tc_err, stream_);
      launch_tc_gemm(j_trans2_.d, j_trans2_.n, j_trans2_.tc_tiles, d_Cnf, d_T32, d_G32, false, false, d_state, 1, -1,
                     d_tc_err, stream_);
      prof_end(h);
      h = prof_begin(kKJacobi, active_work_estimate(kKJacobi));
      run_jacobi(true, s, nullptr, d_Cnf);
      prof_end(h);
    } else {
      double* Cn = d_T64;
      launches_ += 5;
      int h = prof_begin(kKOrtho, active_work_estimate(kKOrtho));
      launch_copy_matrices(d_mols, d_list, (int)cur_list_.size(), d_state, d_C, Cn, stream_);
      launch_gemm(j_ns1_.d, j_ns1_.n, j_ns1_.tiles, d_C, d_C, d_T32, false, true, 0.0f, d_state, 1, -1, stream_);
      launch_gemm(j_ns2_.d, j_ns2_.n, j_ns2_.tiles, d_T32, d_C, Cn, false, false, 0.0f, d_state, 1, -1, stream_);
      prof_end(h);
      h = prof_begin(kKTransform, active_work_estimate(kKTransform));
      launch_gemm(j_trans1_.d, j_trans1_.n, j_trans1_.tiles, d_F, Cn, d_T32, false, true, 0.0f, d_state, 1, -1, stream_);
      launch_gemm(j_trans2_.d, j_trans2_.n, j_trans2_.tiles, Cn, d_T32, d_G32, false, false, 0.0f, d_state, 1, -1,
                  stream_);
      prof_end(h);
      h = prof_begin(kKJacobi, active_work_estimate(kKJacobi));
      run_jacobi(true, s, Cn);
      prof_end(h);
    }
  }
  cuda_check(cudaGetLastError(), "eigen step");
}

void Batch::density_step(const ScfSettings& s) {
  if (householder(s)) {
    // P = 2 X^T X or 2 I - 2 X^T X from the density's eigenvector rows: FP64
    // on the CUDA cores; in the FP32 phase of the mixed path from the FP32
    // rows on the tensor cores (3xTF32, FP32 accumulation)
    const bool mixed = s.precision == 1;
    int h = prof_begin(kKDensity, active_work_estimate(kKDensity));
    launches_ += 1;
    launch_gemm(j_hh_.d, j_hh_.n, j_hh_.tiles, d_C, d_C, d_P, true, false, 0.0, d_state, 1, mixed ? 1 : -1, stream_);
    if (mixed) {
      launches_ += 1;
      launch_tc_gemm(j_hh_.d, j_hh_.n, j_hh_.tc_tiles, d_Cf, d_Cf, d_P, true, false, d_state, 1, 0, d_tc_err, stream_);
    }
    prof_end(h);
  } else if (s.precision == 0) {
    launches_ += 1;
    int h = prof_begin(kKDensity, active_work_estimate(kKDensity));
    launch_gemm(j_dens_.d, j_dens_.n, j_dens_.tiles, d_C, d_C, d_P, true, false, 0.0, d_state, 1, -1, stream_);
    prof_end(h);
  } else {
    // FP32 phase: density from the FP32 eigenvectors
    launches_ += 12;
    int h = prof_begin(kKDensity, active_work_estimate(kKDensity));
    if (s.tensor_cores)
      launch_tc_gemm(j_dens_.d, j_dens_.n, j_dens_.tc_tiles, d_C, d_C, d_P, true, false, d_state, 1, 0, d_tc_err, stream_);
    else
      launch_gemm(j_dens_.d, j_dens_.n, j_dens_.tiles, d_C, d_C, d_P, true, false, 0.0f, d_state, 1, 0, stream_);
    prof_end(h);
    h = prof_begin(kKRefine, active_work_estimate(kKRefine));
    // FP64 phase: one Newton step on the occupied subspace, then P = 2 Y (Y^T Y)^-1 Y^T
    const int nl = (int)cur_list_.size();
    double *W = d_S[0], *K = d_S[1], *Yt = d_S[2], *Mm = d_S[3], *O = d_S[4], *Z = d_S[5];
    // Kt = C_v F C_o^T as (C_v F) C_o^T: 2 v n^2 + 2 v n o flops instead of 2 n^2 o + 2 v n o
    launch_gemm(j_w_.d, j_w_.n, j_w_.tiles, d_C, d_F, W, false, false, 0.0, d_state, 1, 1, stream_);
    launch_gemm(j_kt_.d, j_kt_.n, j_kt_.tiles, W, d_C, K, false, true, 0.0, d_state, 1, 1, stream_);
    launch_gemm(j_ov_.d, j_ov_.n, j_ov_.tiles, d_C, d_C, O, false, true, 0.0, d_state, 1, 1, stream_);
    launch_newton_scale(d_mols, d_list, nl, d_state, 1, K, O, d_eps, stream_);
    // Yt = C_o + K^T C_v: K is ~1e-7, so its product needs only FP32
    // accumulation (error ~1e-14 absolute); the sum is formed in FP64
    launch_copy_occ_rows(d_mols, d_list, nl, d_state, 1, d_C, Yt, stream_);
    launch_gemm(j_yt_.d, j_yt_.n, j_yt_.tiles, K, d_C, Yt, true, false, 0.0f, d_state, 1, 1, stream_);
    launch_gemm(j_m_.d, j_m_.n, j_m_.tiles, Yt, Yt, Mm, false, true, 0.0, d_state, 1, 1, stream_);
    // (Y^T Y)^-1 = I - D + O(D^2) with D = Y^T Y - I: D is at the FP32 round-off
    // of the orthonormalised basis (~1e-7), so the second-order term is ~1e-14;
    // Z = (I - D) Yt = Yt - D Yt, where D Yt (~1e-7) again needs only FP32
    // accumulation
    launch_neumann(d_mols, d_list, nl, d_state, 1, Mm, stream_);
    launch_copy_occ_rows(d_mols, d_list, nl, d_state, 1, Yt, Z, stream_);
    launch_gemm(j_z_.d, j_z_.n, j_z_.tiles, Mm, Yt, Z, false, false, 0.0f, d_state, 1, 1, stream_);
    launch_gemm(j_p_.d, j_p_.n, j_p_.tiles, Yt, Z, d_P, true, false, 0.0, d_state, 1, 1, stream_);
    prof_end(h);
  }
  cuda_check(cudaGetLastError(), "density step");
}

void Batch::iterate(const ScfSettings& s, const std::vector<int>& which) {
  upload_list(which);
  const int nl = (int)which.size();
  launches_ += 4;   // fock + three DIIS kernels
  int h = prof_begin(kKFock, active_work_estimate(kKFock));
  launch_fock_kernel(d_atoms, d_pairs, d_mols, d_list, nl, list_max_atoms(), d_blocks, d_H, d_P, d_F, d_Pold, d_state, -1,
                     1, 1, stream_);
  prof_end(h);
  cuda_check(cudaGetLastError(), "fock_kernel");
  eigen_step(s);
  density_step(s);
  h = prof_begin(kKDiis, active_work_estimate(kKDiis));
  launch_diis(d_mols, d_list, nl, d_state, to_dev(s), d_P, d_Pold, d_hist_dens, d_hist_err, mat_total_,
              s.keep_trace ? d_trace : nullptr, max_iter_alloc_, d_diis_ws, stream_);
  prof_end(h);
  cuda_check(cudaGetLastError(), "diis_kernel");
}

bool same_launches(const ScfSettings& a, const ScfSettings& b) {
  return a.max_iter == b.max_iter && a.rms_density == b.rms_density && a.damping_thresh == b.damping_thresh &&
         a.damping_weight == b.damping_weight && a.diis_num_error_vect == b.diis_num_error_vect &&
         a.diis_start_error == b.diis_start_error && a.diis_end_error == b.diis_end_error &&
         a.precision == b.precision && a.switch_error == b.switch_error && a.max_sweeps == b.max_sweeps &&
         a.keep_trace == b.keep_trace && a.tensor_cores == b.tensor_cores && a.eigensolver == b.eigensolver;
}

// The launches of one SCF iteration depend only on the molecule list and the
// settings, and every kernel reads the per-molecule state from device memory,
// so an iteration captured once can be replayed: one graph launch instead of
// a dozen kernel launches.  Not while profiling (per-launch events), nor on the
// block Jacobi, which reads a host flag between its sweeps, nor for lists with
// a molecule on the whole-GPU eigensolver (its cooperative launches run long
// enough that a launch costs nothing, and are not captured).
void Batch::iterate_graph(const ScfSettings& s, const std::vector<int>& which) {
  upload_list(which);   // outside any capture: may synchronise when the list changes
  if (!s.graphs || prof_on_ || !householder(s) || !hh_large_.empty()) {
    iterate(s, which);
    return;
  }
  if (!graph_exec_ || !same_launches(graph_settings_, s) || graph_layout_ != layout_version_) {
    if (graph_exec_) { cudaGraphExecDestroy(graph_exec_); graph_exec_ = nullptr; }
    hh_prepare();
    const long long before = launches_;
    cudaGraph_t g = nullptr;
    cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
      iterate(s, which);
    } catch (...) {
      cudaStreamEndCapture(stream_, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    cuda_check(cudaStreamEndCapture(stream_, &g), "end capture");
    const cudaError_t e = cudaGraphInstantiate(&graph_exec_, g, 0);
    cudaGraphDestroy(g);
    cuda_check(e, "graph instantiate");
    graph_kernels_ = launches_ - before;
    launches_ = before;
    graph_settings_ = s;
    graph_layout_ = layout_version_;
  }
  cuda_check(cudaGraphLaunch(graph_exec_, stream_), "graph launch");
  launches_ += graph_kernels_;
  ++graph_launches_;
}

int Batch::count_active(const std::vector<int>& which) {
  upload_list(which);
  launches_ += 1;
  count_active_kernel<<<1, 256, 0, stream_>>>(d_list, (int)which.size(), d_state, d_count, d_active);
  int h = 0;
  cuda_check(cudaMemcpyAsync(&h, d_count, sizeof(int), cudaMemcpyDeviceToHost, stream_), "count copy");
  if (prof_on_) {
    active_host_.resize(h_mols.size());
    cuda_check(cudaMemcpyAsync(active_host_.data(), d_active, h_mols.size(), cudaMemcpyDeviceToHost, stream_),
               "active copy");
  }
  cuda_check(cudaStreamSynchronize(stream_), "count sync");
  return h;
}

void Batch::count_active_async(const std::vector<int>& which, int* h_count, char* h_active, cudaEvent_t done) {
  upload_list(which);
  launches_ += 1;
  count_active_kernel<<<1, 256, 0, stream_>>>(d_list, (int)which.size(), d_state, d_count, d_active);
  cuda_check(cudaMemcpyAsync(h_count, d_count, sizeof(int), cudaMemcpyDeviceToHost, stream_), "count copy");
  cuda_check(cudaMemcpyAsync(h_active, d_active, h_mols.size(), cudaMemcpyDeviceToHost, stream_), "active copy");
  cuda_check(cudaEventRecord(done, stream_), "count event");
}

void Batch::copy_states_async(MolState* host) {
  cuda_check(cudaMemcpyAsync(host, d_state, h_mols.size() * sizeof(MolState), cudaMemcpyDeviceToHost, stream_), "state copy");
}

void Batch::copy_charges_async(int m, double* host) {
  const DevMol& d = h_mols[m];
  cuda_check(cudaMemcpyAsync(host, d_charges + d.atom0, d.natoms * sizeof(double), cudaMemcpyDeviceToHost, stream_), "copy charges");
}

void Batch::finish(const ScfSettings& s, const std::vector<int>& which) {
  upload_list(which);
  const int nl = (int)which.size();
  const int max_atoms = list_max_atoms();
  // every eigenpair of the last diagonalised Fock matrix: MO energies and
  // eigenvector rows, as Dsyevd leaves them after the last iteration
  if (householder(s)) hh_vectors(s, 1, 0);
  launches_ += 2;
  int h = prof_begin(kKEnergy, 0.0);
  launch_fock_kernel(d_atoms, d_pairs, d_mols, d_list, nl, max_atoms, d_blocks, d_H, d_P, d_F, d_Pold, d_state, 0,
                     0, 0, stream_);
  VdwParams vdw;
  vdw.on = s.vdw;
  vdw.s6 = s.vdw_s6;
  vdw.d = s.vdw_d;
  launch_energy_kernel(d_atoms, d_pairs, d_mols, d_list, nl, d_P, d_F, d_H, d_state, d_charges, vdw, stream_);
  prof_end(h);
  if (s.dipole) {
    launches_ += 2;
    h = prof_begin(kKDipole, 0.0);
    launch_dipole(d_atoms, d_pairs, d_mols, d_list, nl, max_atoms, d_P, d_H, d_dip_ws, d_state, stream_);
    prof_end(h);
  }
  cuda_check(cudaGetLastError(), "finish");
}

void Batch::scf(const ScfSettings& s, bool requires_guess) {
  std::vector<int> all(h_mols.size());
  for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
  begin(s, all, requires_guess);
  // Iterations are enqueued in blocks (three for one molecule, whose
  // iterations are short, two otherwise).  After each block the count of
  // still-active molecules is copied to pinned memory behind an event, and
  // the host reads a block's count only after it has enqueued the next block,
  // so the device never waits for the host.  Every kernel of an iteration
  // skips molecules that are no longer active, so the iterations enqueued past
  // convergence change nothing (and cost only their empty launches).
  const int block = all.size() == 1 ? 3 : tuned_check_block();
  int it = 0, nblock = 0;
  while (it < s.max_iter) {
    for (int b = 0; b < block && it < s.max_iter; ++b, ++it) iterate_graph(s, all);
    const int slot = nblock & 1;
    count_active_async(all, h_block_count_ + slot, h_block_active_ + (size_t)slot * cap_.slots, block_ev_[slot]);
    ++nblock;
    if (nblock >= 2) {
      const int prev = (nblock - 2) & 1;
      cuda_check(cudaEventSynchronize(block_ev_[prev]), "block count");
      if (prof_on_) std::copy(h_block_active_ + (size_t)prev * cap_.slots,
                              h_block_active_ + (size_t)prev * cap_.slots + h_mols.size(), active_host_.begin());
      if (h_block_count_[prev] == 0) break;
    }
  }
  finish(s, all);
  int tc_err = 0;
  cuda_check(cudaMemcpyAsync(&tc_err, d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, stream_), "tc err");
  cuda_check(cudaStreamSynchronize(stream_), "scf");
  if (tc_err) throw std::runtime_error("tensor-core GEMM: an MMA completion wait ran out");
}

void Batch::results(std::vector<MolResult>* out) {
  std::vector<MolState> st(h_mols.size());
  cuda_check(cudaMemcpyAsync(st.data(), d_state, st.size() * sizeof(MolState), cudaMemcpyDeviceToHost, stream_), "state copy");
  cuda_check(cudaStreamSynchronize(stream_), "results");
  out->resize(st.size());
  for (size_t m = 0; m < st.size(); ++m) {
    MolResult& r = (*out)[m];
    r.status = st[m].status;
    r.iterations = st[m].status == kConverged ? st[m].iter + 1 : st[m].iter;
    r.energy = st[m].energy;
    r.core_repulsion = st[m].ecore;
    r.heat_of_formation = st[m].heat_of_formation;
    r.final_rms = st[m].rms;
    r.final_diis_error = st[m].diis_err;
    for (int k = 0; k < 9; ++k) r.dipole[k] = st[m].dipole[k];
    r.vdw_energy = st[m].vdw_energy;
    r.core_epc = st[m].ecore_epc;
  }
}

void Batch::cartesian_matrix(int m, double* host) const {
  const DevMol& d = h_mols[m];
  const size_t bytes = 3 * (size_t)d.nao * d.nao * sizeof(double);
  double* X = nullptr;
  cuda_check(cudaMalloc(&X, bytes), "cudaMalloc cartesian matrix");
  launch_cartesian_matrix(d_atoms, d_pairs, d_mols, m, d.natoms, X, stream_);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, X, bytes, cudaMemcpyDeviceToHost, stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  cudaFree(X);
  cuda_check(e, "cartesian matrix");
}

void Batch::copy_matrix(int which, int m, double* host) const {
  const double* src = which == 0 ? d_H : which == 1 ? d_F : which == 2 ? d_P : d_C;
  const DevMol& d = h_mols[m];
  cuda_check(cudaMemcpyAsync(host, src + d.mat0, (size_t)d.nao * d.nao * sizeof(double), cudaMemcpyDeviceToHost, stream_), "copy matrix");
  cuda_check(cudaStreamSynchronize(stream_), "copy matrix");
}

void Batch::copy_eps(int m, double* host) const {
  const DevMol& d = h_mols[m];
  cuda_check(cudaMemcpyAsync(host, d_eps + d.vec0, d.nao * sizeof(double), cudaMemcpyDeviceToHost, stream_), "copy eps");
  cuda_check(cudaStreamSynchronize(stream_), "copy eps");
}

void Batch::copy_charges(int m, double* host) const {
  const DevMol& d = h_mols[m];
  cuda_check(cudaMemcpyAsync(host, d_charges + d.atom0, d.natoms * sizeof(double), cudaMemcpyDeviceToHost, stream_), "copy charges");
  cuda_check(cudaStreamSynchronize(stream_), "copy charges");
}

void Batch::forces(const ScfSettings& s, int m, double* host) {
  const DevMol& d = h_mols[m];
  if (3LL * d.npairs > pgrad_cap_) {
    if (d_pgrad_) cudaFree(d_pgrad_);
    d_pgrad_ = nullptr;
    pgrad_cap_ = std::max(3LL * d.npairs, 3LL);
    cuda_check(cudaMalloc(&d_pgrad_, pgrad_cap_ * sizeof(double)), "cudaMalloc pair gradients");
  }
  if (3LL * d.natoms > forces_cap_) {
    if (d_forces_) cudaFree(d_forces_);
    d_forces_ = nullptr;
    forces_cap_ = 3LL * d.natoms;
    cuda_check(cudaMalloc(&d_forces_, forces_cap_ * sizeof(double)), "cudaMalloc forces");
  }
  VdwParams vdw;
  vdw.on = s.vdw;
  vdw.s6 = s.vdw_s6;
  vdw.d = s.vdw_d;
  launch_forces(d_atoms, d_pairs, d_mols, m, d.pair0, d.npairs, d.natoms, eng_->eri(), eng_->ovt(), d_P, vdw,
                d_pgrad_, d_forces_, stream_);
  cuda_check(cudaGetLastError(), "forces");
  cuda_check(cudaMemcpyAsync(host, d_forces_, 3 * (size_t)d.natoms * sizeof(double), cudaMemcpyDeviceToHost, stream_),
             "copy forces");
  cuda_check(cudaStreamSynchronize(stream_), "forces");
}

void Batch::copy_blocks(int m, double* host, size_t* count) const {
  const DevMol& d = h_mols[m];
  long long first = d.npairs ? h_pairs[d.pair0].blk : 0;
  long long last = first;
  if (d.npairs) {
    const DevPair& p = h_pairs[d.pair0 + d.npairs - 1];
    last = p.blk + (long long)(h_atoms[p.a].nao == 4 ? 10 : 1) * (h_atoms[p.b].nao == 4 ? 10 : 1);
  }
  *count = (size_t)(last - first);
  if (host && *count)
    cuda_check(cudaMemcpyAsync(host, d_blocks + first, *count * sizeof(double), cudaMemcpyDeviceToHost, stream_), "copy blocks");
  cuda_check(cudaStreamSynchronize(stream_), "copy blocks");
}

void Batch::copy_trace(int m, std::vector<TraceEntry>* out) const {
  out->assign(max_iter_alloc_, TraceEntry{});
  if (!d_trace || max_iter_alloc_ == 0) return;
  cuda_check(cudaMemcpyAsync(out->data(), d_trace + (size_t)m * max_iter_alloc_, max_iter_alloc_ * sizeof(TraceEntry),
                             cudaMemcpyDeviceToHost, stream_), "copy trace");
  cuda_check(cudaStreamSynchronize(stream_), "copy trace");
}

void Batch::set_density(int m, const double* host) {
  const DevMol& d = h_mols[m];
  cuda_check(cudaMemcpyAsync(d_P + d.mat0, host, (size_t)d.nao * d.nao * sizeof(double), cudaMemcpyHostToDevice, stream_), "set density");
  cuda_check(cudaStreamSynchronize(stream_), "set density");
}

}  // namespace nddo
