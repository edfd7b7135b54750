// Allocation-free variant of the one-time pair-integral pass.
//
// Some callers cannot call cudaMalloc: a host program that owns every byte of
// device memory through its own arena (an MD or QM/MM engine that hands us
// slices of its buffers), code running where device allocation is forbidden
// or would serialise against other work (a latency-critical loop, a process
// whose allocator must not be bypassed), or a caller that needs the call to
// succeed without any chance of an out-of-memory failure at that point.  For
// them, nddo_pair_integrals_noalloc computes the same pair blocks, core
// Hamiltonian and core-core energy as nddo_set_molecule, writing into device
// buffers the caller passes, and takes all of its scratch (atom and pair
// tables, per-pair core-core energies, constant tables) from one file-scope
// static device array of fixed size.  Every GPU that loads this library holds
// that array (about 4.3 MB) until the process exits.
//
// The first call on a device sets it up: it resolves the array's device
// address with cudaGetSymbolAddress (with that device current) and uploads
// the constant tables.  No call may be made on a stream that is being
// captured: every call copies its inputs from host memory and ends with a
// stream synchronisation, so a call on a capturing stream is rejected with
// NDDO_ERR_ARGUMENT.
// Every call shares the one array and leaves the last call's contents in it:
// calls that overlap on the GPU (different streams, or different host threads)
// race and must be serialised by the caller.
#include "../../include/nddo_gpu.h"

#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "engine.h"
#include "nddo_tables.h"

namespace nddo {
namespace {

constexpr int kNoAllocMaxAtoms = 512;
constexpr long long kNoAllocMaxPairs = (long long)kNoAllocMaxAtoms * (kNoAllocMaxAtoms - 1) / 2;

// layout of the scratch array (byte offsets, each 256-byte aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffAtoms = 0;
constexpr size_t kOffPairs = align256(kOffAtoms + sizeof(DevAtom) * kNoAllocMaxAtoms);
constexpr size_t kOffMol = align256(kOffPairs + sizeof(DevPair) * kNoAllocMaxPairs);
constexpr size_t kOffList = align256(kOffMol + sizeof(DevMol));
constexpr size_t kOffState = align256(kOffList + sizeof(int));
constexpr size_t kOffEcore = align256(kOffState + sizeof(MolState));
constexpr size_t kOffRowOff = align256(kOffEcore + sizeof(double) * kNoAllocMaxPairs);
constexpr size_t kOffEri = align256(kOffRowOff + sizeof(long long) * kNoAllocMaxAtoms);
constexpr size_t kOffOvt = align256(kOffEri + sizeof(EriTable));
constexpr size_t kScratchBytes = align256(kOffOvt + sizeof(OverlapTable));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// pair table of one molecule: pair p = (a, b), a < b, row-major; block offsets
// from the per-row offsets computed on the host
__global__ void noalloc_pairs_kernel(const DevAtom* __restrict__ atoms, int natoms,
                                     const long long* __restrict__ row_off, DevPair* __restrict__ pairs) {
  const long long npairs = (long long)natoms * (natoms - 1) / 2;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npairs;
       p += (long long)gridDim.x * blockDim.x) {
    // row a holds natoms - 1 - a pairs; find a with pair_index(a, a+1) <= p
    int a = 0;
    {
      const double nn = (double)natoms;
      const double disc = (2.0 * nn - 1.0) * (2.0 * nn - 1.0) - 8.0 * (double)p;
      a = (int)((2.0 * nn - 1.0 - sqrt(disc > 0.0 ? disc : 0.0)) * 0.5);
      if (a < 0) a = 0;
      if (a > natoms - 2) a = natoms - 2;
      while (a > 0 && pair_index(a, a + 1, natoms) > p) --a;
      while (a + 1 <= natoms - 2 && pair_index(a + 1, a + 2, natoms) <= p) ++a;
    }
    const int b = a + 1 + (int)(p - pair_index(a, a + 1, natoms));
    const int da = atoms[a].nao == 4 ? 10 : 1;
    long long blk = row_off[a];
    for (int c = a + 1; c < b; ++c) blk += (long long)da * (atoms[c].nao == 4 ? 10 : 1);
    DevPair pr;
    pr.a = a;
    pr.b = b;
    pr.mol = 0;
    pr.pad = 0;
    pr.blk = blk;
    pairs[p] = pr;
  }
}

int set_error(char* err, size_t len, int code, const char* msg) {
  if (err && len) {
    std::strncpy(err, msg, len - 1);
    err[len - 1] = '\0';
  }
  return code;
}

// one-time set-up of `device` (that device must be current)
int setup_device(int device, cudaStream_t s, unsigned char** out, char* err, size_t len) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[device]) {
    *out = g_scratch_ptr[device];
    return 0;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr)
    return set_error(err, len, NDDO_ERR_CUDA, cudaGetErrorString(e));
  unsigned char* base = static_cast<unsigned char*>(p);
  static EriTable eri;
  static OverlapTable ovt;
  static bool built = false;
  if (!built) { build_eri_table(&eri); build_overlap_table(&ovt); built = true; }
  e = cudaMemcpyAsync(base + kOffEri, &eri, sizeof(EriTable), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + kOffOvt, &ovt, sizeof(OverlapTable), cudaMemcpyHostToDevice, s);
  nddo_atom_params params[kNumParamSlots];
  std::memset(params, 0, sizeof(params));
  static const int zs[NDDO_NUM_ELEMENTS] = {1, 6, 7, 8, 9, 16, 17};
  for (int t = 0; t < NDDO_NUM_THEORY_SLOTS; ++t)
    for (int k = 0; k < NDDO_NUM_ELEMENTS; ++k) nddo_fill_atom_params(t, zs[k], &params[t * NDDO_NUM_ELEMENTS + k]);
  // The element parameters live in the library's __constant__ table, which
  // the engine (nddo_create / nddo_set_molecule) fills with the same default
  // parameter sets; both paths assume those defaults, so this upload writes
  // the values an engine on this device already holds.
  if (e == cudaSuccess) {
    upload_params(params, s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // host tables above live on this stack frame
  if (e != cudaSuccess) return set_error(err, len, NDDO_ERR_CUDA, cudaGetErrorString(e));
  g_scratch_ptr[device] = base;
  *out = base;
  return 0;
}

}  // namespace
}  // namespace nddo

extern "C" int nddo_pair_integrals_noalloc(int device, int theory, int n_atoms, const int* atomic_numbers,
                                           const double* xyz_bohr, double* d_pair_blocks, size_t pair_block_capacity,
                                           double* d_core_hamiltonian, double* core_repulsion, void* stream,
                                           char* err, size_t err_len) {
  using namespace nddo;
  if (device < 0 || device >= kMaxDevices) return set_error(err, err_len, NDDO_ERR_ARGUMENT, "device index out of range");
  if (theory < 0 || theory >= NDDO_NUM_THEORY_SLOTS) return set_error(err, err_len, NDDO_ERR_ARGUMENT, "unknown theory");
  if (n_atoms < 1 || !atomic_numbers || !xyz_bohr || !d_pair_blocks || !d_core_hamiltonian)
    return set_error(err, err_len, NDDO_ERR_ARGUMENT, "null argument or no atoms");
  if (n_atoms > kNoAllocMaxAtoms) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "n_atoms=%d exceeds the allocation-free limit of %d atoms", n_atoms,
                  kNoAllocMaxAtoms);
    return set_error(err, err_len, NDDO_ERR_BUDGET, msg);
  }
  // host-side tables on the stack (no heap, no device allocation)
  DevAtom atoms[kNoAllocMaxAtoms];
  long long row_off[kNoAllocMaxAtoms];
  int ao = 0;
  for (int a = 0; a < n_atoms; ++a) {
    const int e = nddo_element_index(atomic_numbers[a]);
    nddo_atom_params probe;
    if (e < 0 || nddo_fill_atom_params(theory, atomic_numbers[a], &probe) != 0)
      return set_error(err, err_len, NDDO_ERR_ARGUMENT, "element has no parameters for this theory");
    for (int k = 0; k < 3; ++k)
      if (!(xyz_bohr[3 * a + k] == xyz_bohr[3 * a + k]) || xyz_bohr[3 * a + k] - xyz_bohr[3 * a + k] != 0.0)
        return set_error(err, err_len, NDDO_ERR_ARGUMENT, "non-finite coordinate");
    atoms[a].x = xyz_bohr[3 * a];
    atoms[a].y = xyz_bohr[3 * a + 1];
    atoms[a].z = xyz_bohr[3 * a + 2];
    atoms[a].pidx = theory * NDDO_NUM_ELEMENTS + e;
    atoms[a].ao0 = ao;
    atoms[a].nao = nddo_elements[e].n_ao;
    atoms[a].mol = 0;
    ao += atoms[a].nao;
  }
  long long need = 0;
  for (int a = 0; a < n_atoms; ++a) {
    row_off[a] = need;
    const int da = atoms[a].nao == 4 ? 10 : 1;
    for (int b = a + 1; b < n_atoms; ++b) {
      if (atoms[a].x == atoms[b].x && atoms[a].y == atoms[b].y && atoms[a].z == atoms[b].z)
        return set_error(err, err_len, NDDO_ERR_ARGUMENT, "two atoms at the same position");
      need += (long long)da * (atoms[b].nao == 4 ? 10 : 1);
    }
  }
  if ((size_t)need > pair_block_capacity) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "pair_block_capacity=%zu doubles is smaller than the %lld this molecule needs",
                  pair_block_capacity, need);
    return set_error(err, err_len, NDDO_ERR_ARGUMENT, msg);
  }
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return set_error(err, err_len, NDDO_ERR_CUDA, "cudaGetDevice failed");
  cudaError_t ce = cudaSetDevice(device);
  if (ce != cudaSuccess) return set_error(err, err_len, NDDO_ERR_CUDA, cudaGetErrorString(ce));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    ce = cudaStreamIsCapturing(s, &cap);
    if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
      cudaSetDevice(prev);
      return set_error(err, err_len, ce != cudaSuccess ? NDDO_ERR_CUDA : NDDO_ERR_ARGUMENT,
                       ce != cudaSuccess ? cudaGetErrorString(ce)
                                         : "the stream is being captured: this call copies from host memory and "
                                           "synchronises, so it cannot be recorded into a graph");
    }
  }
  unsigned char* base = nullptr;
  int rc = setup_device(device, s, &base, err, err_len);
  if (rc == 0) {
    DevAtom* d_atoms = reinterpret_cast<DevAtom*>(base + kOffAtoms);
    DevPair* d_pairs = reinterpret_cast<DevPair*>(base + kOffPairs);
    DevMol* d_mol = reinterpret_cast<DevMol*>(base + kOffMol);
    int* d_list = reinterpret_cast<int*>(base + kOffList);
    MolState* d_state = reinterpret_cast<MolState*>(base + kOffState);
    double* d_ecore = reinterpret_cast<double*>(base + kOffEcore);
    long long* d_rowoff = reinterpret_cast<long long*>(base + kOffRowOff);
    const EriTable* d_eri = reinterpret_cast<const EriTable*>(base + kOffEri);
    const OverlapTable* d_ovt = reinterpret_cast<const OverlapTable*>(base + kOffOvt);
    DevMol mol;
    std::memset(&mol, 0, sizeof(mol));
    mol.natoms = n_atoms;
    mol.nao = ao;
    mol.theory = theory;
    mol.npairs = (int)((long long)n_atoms * (n_atoms - 1) / 2);
    const int zero = 0;
    ce = cudaMemcpyAsync(d_atoms, atoms, sizeof(DevAtom) * n_atoms, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_rowoff, row_off, sizeof(long long) * n_atoms, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_mol, &mol, sizeof(DevMol), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_list, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
    // the state's core-core accumulator must start from zero
    if (ce == cudaSuccess) ce = cudaMemsetAsync(d_state, 0, sizeof(MolState), s);
    if (ce == cudaSuccess && mol.npairs > 0) {
      const long long np = mol.npairs;
      const int grid = (int)((np + 255) / 256 < 1024 ? (np + 255) / 256 : 1024);
      noalloc_pairs_kernel<<<grid, 256, 0, s>>>(d_atoms, n_atoms, d_rowoff, d_pairs);
      ce = cudaGetLastError();
      if (ce == cudaSuccess) {
        launch_pair_kernel(d_atoms, d_pairs, np, d_mol, d_eri, d_ovt, d_pair_blocks, d_core_hamiltonian, d_ecore, s);
        ce = cudaGetLastError();
      }
    }
    if (ce == cudaSuccess) {
      launch_hcore_kernel(d_atoms, d_pairs, d_mol, d_list, 1, d_pair_blocks, d_ecore, d_eri, nullptr,
                          d_core_hamiltonian, d_state, s);
      ce = cudaGetLastError();
    }
    double ecore = 0.0;
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(&ecore, reinterpret_cast<unsigned char*>(d_state) + offsetof(MolState, ecore), sizeof(double),
                           cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);   // stack tables and ecore must outlive the copies
    if (ce != cudaSuccess) rc = set_error(err, err_len, NDDO_ERR_CUDA, cudaGetErrorString(ce));
    else if (core_repulsion) *core_repulsion = ecore;
  }
  cudaSetDevice(prev);
  return rc;
}
