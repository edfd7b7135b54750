// extern "C" boundary (include/nddo_gpu.h) over the batched engine.
#include "../../include/nddo_gpu.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"
#include "scf_text.h"
#include "server.h"

struct nddo_batch {
  nddo_ctx* ctx;
  std::unique_ptr<nddo::GroupedBatch> b;
  std::vector<int> n_atoms;
  bool dipole = false;          // the last nddo_batch_run computed dipole moments
  bool ran = false;             // a run completed: every molecule has a density to start from
  nddo::ScfSettings last;       // settings of the last run (the forces' dispersion term)
};

namespace {
// Calibration kernel: eight independent FMA chains per thread.
template <typename T>
__global__ void fma_peak_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double fma_peak(cudaStream_t s, int iters) {
  int dev = 0, sms = 0;
  nddo::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  nddo::cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
  const int blocks = sms * 4, threads = 256;
  T* out = nullptr;
  nddo::cuda_check(cudaMalloc(&out, sizeof(T) * blocks * threads), "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_peak_kernel<T><<<blocks, threads, 0, s>>>(out, 16, (T)0.999, (T)0.001);
  double best = 0.0;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    fma_peak_kernel<T><<<blocks, threads, 0, s>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double tf = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    best = tf > best ? tf : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  nddo::cuda_check(cudaGetLastError(), "fma_peak_kernel");
  return best;
}
}  // namespace

struct nddo_server {
  nddo_ctx* ctx;
  std::unique_ptr<nddo::Server> s;
  nddo::ServeResult held;      // a result that did not fit the caller's charge buffer
  bool has_held = false;
};

struct nddo_ctx {
  std::unique_ptr<nddo::Engine> engine;
  // nddo_batch_scf keeps its last batch: a call with the same molecules
  // (theory, DIIS window, atom counts and elements) reuses the device arrays
  // and uploads only the new coordinates
  std::unique_ptr<nddo::GroupedBatch> batch_cache;
  std::vector<int> cache_natoms, cache_Z;
  int cache_theory = -1, cache_diis = -1;
  std::unique_ptr<nddo::Batch> mol;      // current molecule (SetMolecule / DoSCF API)
  nddo::ScfSettings last_settings;
  bool has_scf = false;
  std::vector<int> Z;                    // elements of the current molecule (the output text)
  int n_epc = 0;                         // its environmental point charges
  int theory = 0;
  double scf_seconds = 0.0;              // host wall time of the last nddo_scf
  std::vector<int> sum_pairs;            // SCF option sum_charges (first, last atom index pairs)
  size_t budget = 0;
  std::string err;
};

namespace {

nddo::ScfSettings to_settings(const nddo_scf_params* p) {
  nddo::ScfSettings s;
  if (p) {
    s.max_iter = p->max_iter;
    s.rms_density = p->rms_density;
    s.damping_thresh = p->damping_thresh;
    s.damping_weight = p->damping_weight;
    s.diis_num_error_vect = p->diis_num_error_vect;
    s.diis_start_error = p->diis_start_error;
    s.diis_end_error = p->diis_end_error;
    s.precision = p->precision;
    s.switch_error = p->fp64_switch_error;
    s.tensor_cores = p->tensor_cores;
    s.dipole = p->dipole;
    s.vdw = p->vdw;
    s.vdw_s6 = p->vdw_s6;
    s.vdw_d = p->vdw_d;
    s.eigensolver = p->eigensolver;
  }
  return s;
}

int fail(nddo_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

template <typename F>
int guarded(nddo_ctx* ctx, F&& f) {
  if (!ctx) return NDDO_ERR_ARGUMENT;
  try {
    return f();
  } catch (const std::invalid_argument& e) {
    return fail(ctx, NDDO_ERR_ARGUMENT, e.what());
  } catch (const std::exception& e) {
    return fail(ctx, NDDO_ERR_CUDA, e.what());
  }
}

bool valid_params(const nddo_scf_params* p, std::string* why) {
  if (!p) { *why = "null SCF parameters"; return false; }
  if (p->max_iter < 1) { *why = "max_iter must be >= 1"; return false; }
  if (p->diis_num_error_vect < 0 || p->diis_num_error_vect > nddo::kMaxDiis) { *why = "diis_num_error_vect must be in 0..8"; return false; }
  if (p->precision != NDDO_PRECISION_FP64 && p->precision != NDDO_PRECISION_MIXED) { *why = "unknown precision"; return false; }
  if (!(p->rms_density > 0.0)) { *why = "rms_density must be > 0"; return false; }
  if (p->vdw && !(p->vdw_s6 >= 0.0 && p->vdw_d > 0.0)) { *why = "vdw_s6 must be >= 0 and vdw_d > 0"; return false; }
  if (p->eigensolver < NDDO_EIGEN_AUTO || p->eigensolver > NDDO_EIGEN_HOUSEHOLDER) { *why = "unknown eigensolver"; return false; }
  return true;
}

}  // namespace

extern "C" {

void nddo_default_params(nddo_scf_params* p) {
  if (!p) return;
  p->max_iter = 100;
  p->rms_density = 1e-8;
  p->damping_thresh = 1.0;
  p->damping_weight = 0.8;
  p->diis_num_error_vect = 5;
  p->diis_start_error = 1e-2;
  p->diis_end_error = 1e-8;
  p->precision = NDDO_PRECISION_FP64;
  p->fp64_switch_error = 1e-4;
  p->tensor_cores = 1;
  p->dipole = 1;
  p->vdw = 0;
  p->vdw_s6 = 1.40;
  p->vdw_d = 23.0;
  p->eigensolver = NDDO_EIGEN_AUTO;
}

int nddo_create(int device, size_t hbm_budget_bytes, nddo_ctx** out) {
  if (!out) return NDDO_ERR_ARGUMENT;
  *out = nullptr;
  nddo_ctx* ctx = new nddo_ctx();
  ctx->budget = hbm_budget_bytes;
  try {
    ctx->engine.reset(new nddo::Engine(device));
  } catch (const std::exception& e) {
    // keep the context so the caller can read the message, but report failure
    ctx->err = e.what();
    *out = ctx;
    return NDDO_ERR_CUDA;
  }
  *out = ctx;
  return NDDO_OK;
}

void nddo_destroy(nddo_ctx* ctx) {
  if (!ctx) return;
  ctx->batch_cache.reset();
  ctx->mol.reset();
  ctx->engine.reset();
  delete ctx;
}

const char* nddo_last_error(const nddo_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int nddo_set_molecule(nddo_ctx* ctx, int theory, int n_atoms, const int* Z, const double* xyz) {
  return nddo_set_molecule_epc(ctx, theory, n_atoms, Z, xyz, 0, nullptr);
}

int nddo_set_molecule_epc(nddo_ctx* ctx, int theory, int n_atoms, const int* Z, const double* xyz, int n_epc,
                          const double* epc) {
  return guarded(ctx, [&]() {
    if (!ctx->engine) return fail(ctx, NDDO_ERR_STATE, "engine not initialised");
    if (n_atoms < 1 || !Z || !xyz) return fail(ctx, NDDO_ERR_ARGUMENT, "need at least one atom");
    if (n_epc < 0 || (n_epc > 0 && !epc)) return fail(ctx, NDDO_ERR_ARGUMENT, "invalid point charges");
    nddo::MoleculeInput in;
    in.theory = theory;
    in.Z.assign(Z, Z + n_atoms);
    in.xyz.assign(xyz, xyz + 3 * (size_t)n_atoms);
    if (n_epc > 0) in.epc.assign(epc, epc + 4 * (size_t)n_epc);
    ctx->has_scf = false;
    // The molecule lives in a one-slot pool that is kept between calls: a new
    // molecule that fits the pool's arenas reuses them (no device allocation
    // on the repeated SetMolecule/DoSCF path); a larger one grows the pool.
    int nao = 0;
    for (int a = 0; a < n_atoms; ++a) {
      const int e = nddo_element_index(Z[a]);
      nao += e < 0 ? 1 : nddo_elements[e].n_ao;
    }
    int slot = -1;
    if (ctx->mol) {
      ctx->mol->release(0);
      if (nao <= ctx->mol->max_n() && n_epc <= ctx->mol->epc_capacity()) {
        try {
          slot = ctx->mol->admit(in);
        } catch (...) {
          ctx->mol.reset();   // an invalid molecule leaves no molecule set
          throw;
        }
      }
    }
    if (slot < 0) {
      ctx->mol.reset();
      nddo::BatchCapacity c;
      const long long na = n_atoms, np = na * (na - 1) / 2;
      c.slots = 1;
      c.atoms = na;
      c.pairs = np;
      c.blocks = 100 * np;
      c.mat = ((long long)nao * nao + 31) / 32 * 32;
      c.vec = (nao + 31) / 32 * 32;
      c.max_n = nao;
      c.ws_slots = 1;
      c.epcs = n_epc;
      std::unique_ptr<nddo::Batch> b(new nddo::Batch(ctx->engine.get(), c, 5, nullptr));
      if (ctx->budget && b->device_bytes() > ctx->budget)
        return fail(ctx, NDDO_ERR_BUDGET, "molecule needs " + std::to_string(b->device_bytes()) + " bytes of HBM, budget is " + std::to_string(ctx->budget));
      slot = b->admit(in);      // throws for an invalid molecule (nothing is kept then)
      if (slot != 0) return fail(ctx, NDDO_ERR_STATE, "molecule does not fit its own pool");
      ctx->mol = std::move(b);
    }
    ctx->mol->integrals(std::vector<int>{0});
    ctx->Z.assign(Z, Z + n_atoms);
    ctx->n_epc = n_epc;
    ctx->theory = theory;
    return (int)NDDO_OK;
  });
}

int nddo_num_aos(const nddo_ctx* ctx) { return (ctx && ctx->mol) ? ctx->mol->nao(0) : -1; }
int nddo_num_atoms(const nddo_ctx* ctx) { return (ctx && ctx->mol) ? ctx->mol->natoms(0) : -1; }

int nddo_scf(nddo_ctx* ctx, const nddo_scf_params* params, int requires_guess, nddo_scf_result* result) {
  return guarded(ctx, [&]() {
    if (!ctx->mol) return fail(ctx, NDDO_ERR_STATE, "A molecule is not set.");
    std::string why;
    if (!valid_params(params, &why)) return fail(ctx, NDDO_ERR_ARGUMENT, why);
    nddo::ScfSettings s = to_settings(params);
    if (s.diis_num_error_vect != 5) {
      // the DIIS history is sized at SetMolecule; rebuild for another window
      // (rare: the MolDS default and every reference input use 5)
      return fail(ctx, NDDO_ERR_ARGUMENT, "diis_num_error_vect other than 5 requires nddo_batch_scf");
    }
    if (!requires_guess && !ctx->has_scf) requires_guess = 1;
    const auto t0 = std::chrono::steady_clock::now();
    ctx->mol->scf(s, requires_guess != 0);
    std::vector<nddo::MolResult> r;
    ctx->mol->results(&r);
    ctx->scf_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    ctx->last_settings = s;
    ctx->has_scf = true;
    if (result) {
      result->status = r[0].status;
      result->iterations = r[0].iterations;
      result->energy = r[0].energy;
      result->core_repulsion = r[0].core_repulsion;
      result->heat_of_formation = r[0].heat_of_formation;
      result->final_rms = r[0].final_rms;
      result->final_diis_error = r[0].final_diis_error;
      for (int k = 0; k < 9; ++k) result->dipole[k] = s.dipole ? r[0].dipole[k] : 0.0;
      result->vdw_energy = r[0].vdw_energy;
      result->core_epc_coulomb = r[0].core_epc;
    }
    if (r[0].status != nddo::kConverged)
      return fail(ctx, NDDO_NOT_CONVERGED,
                  "SCF did not met convergence criterion. maxIterationsSCF=" + std::to_string(s.max_iter));
    return (int)NDDO_OK;
  });
}

static int getter(nddo_ctx* ctx, double* out, int what) {
  return guarded(ctx, [&]() {
    if (!ctx->mol || !ctx->has_scf) return fail(ctx, NDDO_ERR_STATE, "no SCF result");
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output buffer");
    if (what == 10) ctx->mol->copy_eps(0, out);
    else if (what == 11) ctx->mol->copy_charges(0, out);
    else ctx->mol->copy_matrix(what, 0, out);
    return (int)NDDO_OK;
  });
}

int nddo_get_energies_mo(nddo_ctx* ctx, double* out) { return getter(ctx, out, 10); }
int nddo_get_fock_matrix(nddo_ctx* ctx, double* out) { return getter(ctx, out, 3); }
int nddo_get_density(nddo_ctx* ctx, double* out) { return getter(ctx, out, 2); }
int nddo_get_mulliken(nddo_ctx* ctx, double* out) { return getter(ctx, out, 11); }

int nddo_set_coordinates(nddo_ctx* ctx, const double* xyz) {
  return guarded(ctx, [&]() {
    if (!ctx->mol) return fail(ctx, NDDO_ERR_STATE, "A molecule is not set.");
    if (!xyz) return fail(ctx, NDDO_ERR_ARGUMENT, "null coordinates");
    ctx->mol->set_molecule_coordinates(0, xyz);   // validates before it changes anything
    ctx->mol->integrals(std::vector<int>{0});
    return (int)NDDO_OK;
  });
}

int nddo_get_dipole(nddo_ctx* ctx, double* out) {
  return guarded(ctx, [&]() {
    if (!ctx->mol || !ctx->has_scf) return fail(ctx, NDDO_ERR_STATE, "no SCF result");
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output buffer");
    if (!ctx->last_settings.dipole) return fail(ctx, NDDO_ERR_STATE, "the last SCF ran with dipole = 0");
    std::vector<nddo::MolResult> r;
    ctx->mol->results(&r);
    for (int k = 0; k < 9; ++k) out[k] = r[0].dipole[k];
    return (int)NDDO_OK;
  });
}

int nddo_get_cartesian_matrix(nddo_ctx* ctx, double* out) {
  return guarded(ctx, [&]() {
    if (!ctx->mol) return fail(ctx, NDDO_ERR_STATE, "A molecule is not set.");
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output buffer");
    ctx->mol->cartesian_matrix(0, out);
    return (int)NDDO_OK;
  });
}

int nddo_get_core_hamiltonian(nddo_ctx* ctx, double* out) {
  return guarded(ctx, [&]() {
    if (!ctx->mol) return fail(ctx, NDDO_ERR_STATE, "A molecule is not set.");
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output buffer");
    ctx->mol->copy_matrix(0, 0, out);
    return (int)NDDO_OK;
  });
}

namespace {
int copy_text(const std::string& text, char* out, size_t cap, size_t* needed) {
  if (needed) *needed = text.size() + 1;
  if (out && cap > 0) {
    const size_t n = std::min(cap - 1, text.size());
    std::memcpy(out, text.data(), n);
    out[n] = '\0';
  }
  return (int)NDDO_OK;
}
}  // namespace

int nddo_scf_output_text(nddo_ctx* ctx, char* out, size_t cap, size_t* needed) {
  return guarded(ctx, [&]() {
    if (!ctx->mol || !ctx->has_scf) return fail(ctx, NDDO_ERR_STATE, "no SCF result");
    std::vector<nddo::TraceEntry> tr;
    ctx->mol->copy_trace(0, &tr);
    std::vector<nddo::MolResult> r;
    ctx->mol->results(&r);
    const int its = std::min<int>((int)tr.size(), r[0].iterations);
    std::vector<double> rms(its), derr(its);
    std::vector<int> on(its), damp(its);
    for (int i = 0; i < its; ++i) {
      rms[i] = tr[i].rms;
      derr[i] = tr[i].diis_err;
      on[i] = tr[i].diis_on;
      damp[i] = tr[i].damp_on;
    }
    const int n = ctx->mol->nao(0);
    std::vector<double> eps(n), q(ctx->Z.size());
    ctx->mol->copy_eps(0, eps.data());
    ctx->mol->copy_charges(0, q.data());
    int nelec = 0;
    for (int z : ctx->Z) {
      const int e = nddo_element_index(z);
      nelec += e < 0 ? 0 : nddo_elements[e].core_charge;
    }
    nddo::ScfText t;
    t.theory = ctx->theory;
    t.n_atoms = (int)ctx->Z.size();
    t.Z = ctx->Z.data();
    t.n_ao = n;
    t.nocc = nelec / 2;
    t.iterations = its;
    t.rms = rms.data();
    t.diis_error = derr.data();
    t.diis_on = on.data();
    t.damp_on = damp.data();
    t.converged = r[0].status == nddo::kConverged;
    t.eps = eps.data();
    t.energy = r[0].energy;
    t.core_repulsion = r[0].core_repulsion;
    t.vdw = ctx->last_settings.vdw || ctx->theory == NDDO_THEORY_AM1D || ctx->theory == NDDO_THEORY_PM3D;
    t.vdw_energy = r[0].vdw_energy;
    t.epc = ctx->n_epc > 0;
    t.core_epc = r[0].core_epc;
    t.dipole = ctx->last_settings.dipole ? r[0].dipole : nullptr;
    t.charges = q.data();
    t.heat_of_formation = r[0].heat_of_formation;
    t.seconds = ctx->scf_seconds;
    t.n_sum = (int)ctx->sum_pairs.size() / 2;
    t.sum_pairs = ctx->sum_pairs.data();
    return copy_text(nddo::format_scf_text(t), out, cap, needed);
  });
}

int nddo_get_forces(nddo_ctx* ctx, double* out) {
  return guarded(ctx, [&]() {
    if (!ctx->mol || !ctx->has_scf) return fail(ctx, NDDO_ERR_STATE, "no SCF result");
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output buffer");
    std::vector<nddo::MolResult> r;
    ctx->mol->results(&r);
    if (r[0].status != nddo::kConverged) return fail(ctx, NDDO_ERR_STATE, "forces need a converged SCF");
    ctx->mol->forces(ctx->last_settings, 0, out);
    return (int)NDDO_OK;
  });
}

int nddo_set_sum_charges(nddo_ctx* ctx, int n_pairs, const int* pairs) {
  return guarded(ctx, [&]() {
    if (n_pairs < 0 || (n_pairs > 0 && !pairs)) return fail(ctx, NDDO_ERR_ARGUMENT, "invalid sum_charges pairs");
    for (int i = 0; i < n_pairs; ++i)
      if (pairs[2 * i] < 0 || pairs[2 * i + 1] < pairs[2 * i])
        return fail(ctx, NDDO_ERR_ARGUMENT, "sum_charges needs 0 <= first <= last");
    ctx->sum_pairs.assign(pairs, pairs + 2 * (size_t)n_pairs);
    return (int)NDDO_OK;
  });
}

int nddo_format_scf_text(int theory, int n_atoms, const int* Z, int n_ao, int n_occ, int iterations,
                         const double* rms, const double* diis_error, const int* diis_on, const int* damp_on,
                         int converged, const double* eps, double energy, double core_repulsion, int vdw,
                         double vdw_energy, int epc, double core_epc, const double* dipole, const double* charges,
                         double heat_of_formation, int n_sum_pairs, const int* sum_pairs, double seconds, char* out,
                         size_t cap, size_t* needed) {
  try {
    if (n_sum_pairs < 0 || (n_sum_pairs > 0 && !sum_pairs)) return NDDO_ERR_ARGUMENT;
    if (n_atoms < 1 || !Z || n_ao < 1 || iterations < 0 || (iterations > 0 && (!rms || !diis_error || !diis_on || !damp_on)) ||
        (converged && (!eps || !charges)))
      return NDDO_ERR_ARGUMENT;
    nddo::ScfText t;
    t.theory = theory;
    t.n_atoms = n_atoms;
    t.Z = Z;
    t.n_ao = n_ao;
    t.nocc = n_occ;
    t.iterations = iterations;
    t.rms = rms;
    t.diis_error = diis_error;
    t.diis_on = diis_on;
    t.damp_on = damp_on;
    t.converged = converged;
    t.eps = eps;
    t.energy = energy;
    t.core_repulsion = core_repulsion;
    t.vdw = vdw;
    t.vdw_energy = vdw_energy;
    t.epc = epc;
    t.core_epc = core_epc;
    t.dipole = dipole;
    t.charges = charges;
    t.heat_of_formation = heat_of_formation;
    t.seconds = seconds;
    t.n_sum = n_sum_pairs;
    t.sum_pairs = sum_pairs;
    return copy_text(nddo::format_scf_text(t), out, cap, needed);
  } catch (...) {
    return NDDO_ERR_ARGUMENT;
  }
}

int nddo_get_trace(nddo_ctx* ctx, int max_entries, double* rms, double* derr, int* on, int* damp) {
  return guarded(ctx, [&]() {
    if (!ctx->mol || !ctx->has_scf) return fail(ctx, NDDO_ERR_STATE, "no SCF result");
    std::vector<nddo::TraceEntry> t;
    ctx->mol->copy_trace(0, &t);
    std::vector<nddo::MolResult> r;
    ctx->mol->results(&r);
    const int n = std::min<int>(max_entries, std::min<int>((int)t.size(), r[0].iterations));
    for (int i = 0; i < n; ++i) {
      if (rms) rms[i] = t[i].rms;
      if (derr) derr[i] = t[i].diis_err;
      if (on) on[i] = t[i].diis_on;
      if (damp) damp[i] = t[i].damp_on;
    }
    return n;
  });
}

int nddo_get_pair_blocks(nddo_ctx* ctx, double* out, size_t* count) {
  return guarded(ctx, [&]() {
    if (!ctx->mol) return fail(ctx, NDDO_ERR_STATE, "A molecule is not set.");
    if (!count) return fail(ctx, NDDO_ERR_ARGUMENT, "null count");
    ctx->mol->copy_blocks(0, out, count);
    return (int)NDDO_OK;
  });
}

int nddo_batch_scf(nddo_ctx* ctx, int theory, int n_mol, const int* n_atoms, const int* Z, const double* xyz,
                   const nddo_scf_params* params, nddo_scf_result* results, double* charges) {
  return guarded(ctx, [&]() {
    if (!ctx->engine) return fail(ctx, NDDO_ERR_STATE, "engine not initialised");
    if (n_mol < 1 || !n_atoms || !Z || !xyz || !results) return fail(ctx, NDDO_ERR_ARGUMENT, "bad batch arguments");
    std::string why;
    if (!valid_params(params, &why)) return fail(ctx, NDDO_ERR_ARGUMENT, why);
    nddo::ScfSettings s = to_settings(params);
    s.keep_trace = 0;
    std::vector<nddo::MoleculeInput> mols(n_mol);
    size_t off = 0;
    for (int i = 0; i < n_mol; ++i) {
      if (n_atoms[i] < 1) return fail(ctx, NDDO_ERR_ARGUMENT, "molecule without atoms");
      mols[i].theory = theory;
      mols[i].Z.assign(Z + off, Z + off + n_atoms[i]);
      mols[i].xyz.assign(xyz + 3 * off, xyz + 3 * (off + n_atoms[i]));
      off += n_atoms[i];
    }
    const bool hit = ctx->batch_cache && ctx->cache_theory == theory && ctx->cache_diis == s.diis_num_error_vect &&
                     ctx->cache_natoms.size() == (size_t)n_mol &&
                     std::equal(n_atoms, n_atoms + n_mol, ctx->cache_natoms.begin()) &&
                     ctx->cache_Z.size() == off && std::equal(Z, Z + off, ctx->cache_Z.begin());
    if (hit) {
      try {
        ctx->batch_cache->set_coordinates(xyz);
      } catch (...) {
        ctx->batch_cache.reset();   // a rejected geometry leaves no half-updated batch behind
        throw;
      }
    } else {
      ctx->batch_cache.reset();
      std::unique_ptr<nddo::GroupedBatch> nb(new nddo::GroupedBatch(ctx->engine.get(), mols, s.diis_num_error_vect,
                                                                    nddo::GroupedBatch::default_groups(n_mol)));
      if (ctx->budget && nb->device_bytes() > ctx->budget)
        return fail(ctx, NDDO_ERR_BUDGET, "batch needs " + std::to_string(nb->device_bytes()) + " bytes of HBM, budget is " + std::to_string(ctx->budget));
      ctx->batch_cache = std::move(nb);
      ctx->cache_theory = theory;
      ctx->cache_diis = s.diis_num_error_vect;
      ctx->cache_natoms.assign(n_atoms, n_atoms + n_mol);
      ctx->cache_Z.assign(Z, Z + off);
    }
    nddo::GroupedBatch& b = *ctx->batch_cache;
    b.run(s);
    std::vector<nddo::MolResult> r;
    b.results(&r);
    int rc = NDDO_OK;
    off = 0;
    for (int i = 0; i < n_mol; ++i) {
      results[i].status = r[i].status;
      results[i].iterations = r[i].iterations;
      results[i].energy = r[i].energy;
      results[i].core_repulsion = r[i].core_repulsion;
      results[i].heat_of_formation = r[i].heat_of_formation;
      results[i].final_rms = r[i].final_rms;
      results[i].final_diis_error = r[i].final_diis_error;
      for (int k = 0; k < 9; ++k) results[i].dipole[k] = s.dipole ? r[i].dipole[k] : 0.0;
      results[i].vdw_energy = r[i].vdw_energy;
      results[i].core_epc_coulomb = r[i].core_epc;
      if (r[i].status != nddo::kConverged) rc = NDDO_NOT_CONVERGED;
      if (charges) b.copy_charges(i, charges + off);
      off += n_atoms[i];
    }
    if (rc != NDDO_OK) ctx->err = "SCF did not met convergence criterion for at least one molecule";
    return rc;
  });
}

int nddo_batch_create(nddo_ctx* ctx, int theory, int n_mol, const int* n_atoms, const int* Z, const double* xyz,
                      int diis_m, nddo_batch** out) {
  return nddo_batch_create_epc(ctx, theory, n_mol, n_atoms, Z, xyz, nullptr, nullptr, diis_m, out);
}

int nddo_batch_create_epc(nddo_ctx* ctx, int theory, int n_mol, const int* n_atoms, const int* Z, const double* xyz,
                          const int* n_epc, const double* epc, int diis_m, nddo_batch** out) {
  return guarded(ctx, [&]() {
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    if (!ctx->engine) return fail(ctx, NDDO_ERR_STATE, "engine not initialised");
    if (n_mol < 1 || !n_atoms || !Z || !xyz) return fail(ctx, NDDO_ERR_ARGUMENT, "bad batch arguments");
    if (diis_m < 0 || diis_m > nddo::kMaxDiis) return fail(ctx, NDDO_ERR_ARGUMENT, "diis_num_error_vect must be in 0..8");
    std::vector<nddo::MoleculeInput> mols(n_mol);
    size_t off = 0, eoff = 0;
    for (int i = 0; i < n_mol; ++i) {
      if (n_atoms[i] < 1) return fail(ctx, NDDO_ERR_ARGUMENT, "molecule without atoms");
      mols[i].theory = theory;
      mols[i].Z.assign(Z + off, Z + off + n_atoms[i]);
      mols[i].xyz.assign(xyz + 3 * off, xyz + 3 * (off + n_atoms[i]));
      off += n_atoms[i];
      const int ne = n_epc ? n_epc[i] : 0;
      if (ne < 0 || (ne > 0 && !epc)) return fail(ctx, NDDO_ERR_ARGUMENT, "invalid point charges");
      if (ne > 0) mols[i].epc.assign(epc + 4 * eoff, epc + 4 * (eoff + ne));
      eoff += ne;
    }
    std::unique_ptr<nddo::GroupedBatch> b(
        new nddo::GroupedBatch(ctx->engine.get(), mols, diis_m, nddo::GroupedBatch::default_groups(n_mol)));
    if (ctx->budget && b->device_bytes() > ctx->budget)
      return fail(ctx, NDDO_ERR_BUDGET, "batch needs " + std::to_string(b->device_bytes()) + " bytes of HBM, budget is " + std::to_string(ctx->budget));
    nddo_batch* h = new nddo_batch();
    h->ctx = ctx;
    h->b = std::move(b);
    h->n_atoms.assign(n_atoms, n_atoms + n_mol);
    *out = h;
    return (int)NDDO_OK;
  });
}

int nddo_batch_run_ex(nddo_batch* h, const nddo_scf_params* params, int requires_guess) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() {
    std::string why;
    if (!valid_params(params, &why)) return fail(h->ctx, NDDO_ERR_ARGUMENT, why);
    nddo::ScfSettings s = to_settings(params);
    s.keep_trace = 0;
    h->dipole = false;
    // no previous density before the first run: the guess, as DoSCF's first call
    const bool guess = requires_guess != 0 || !h->ran;
    h->ran = false;
    h->b->run(s, guess);
    h->ran = true;
    h->dipole = s.dipole != 0;
    h->last = s;
    return (int)NDDO_OK;
  });
}

int nddo_batch_run(nddo_batch* h, const nddo_scf_params* params) { return nddo_batch_run_ex(h, params, 1); }

int nddo_batch_set_coordinates(nddo_batch* h, const double* xyz) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() {
    if (!xyz) return fail(h->ctx, NDDO_ERR_ARGUMENT, "null coordinates");
    h->b->set_coordinates(xyz);
    return (int)NDDO_OK;
  });
}

int nddo_batch_results(nddo_batch* h, nddo_scf_result* results, double* charges) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() {
    if (!results) return fail(h->ctx, NDDO_ERR_ARGUMENT, "null results");
    std::vector<nddo::MolResult> r;
    h->b->results(&r);
    int rc = NDDO_OK;
    size_t off = 0;
    for (size_t i = 0; i < r.size(); ++i) {
      results[i].status = r[i].status;
      results[i].iterations = r[i].iterations;
      results[i].energy = r[i].energy;
      results[i].core_repulsion = r[i].core_repulsion;
      results[i].heat_of_formation = r[i].heat_of_formation;
      results[i].final_rms = r[i].final_rms;
      results[i].final_diis_error = r[i].final_diis_error;
      for (int k = 0; k < 9; ++k) results[i].dipole[k] = h->dipole ? r[i].dipole[k] : 0.0;
      results[i].vdw_energy = r[i].vdw_energy;
      results[i].core_epc_coulomb = r[i].core_epc;
      if (r[i].status != nddo::kConverged) rc = NDDO_NOT_CONVERGED;
      if (charges) h->b->copy_charges((int)i, charges + off);
      off += h->n_atoms[i];
    }
    if (rc != NDDO_OK) h->ctx->err = "SCF did not met convergence criterion for at least one molecule";
    return rc;
  });
}

int nddo_batch_get_matrix(nddo_batch* h, int which, int m, double* out) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() -> int {
    if (!out || m < 0 || m >= h->b->size() || (which != 0 && which != 1))
      return fail(h->ctx, NDDO_ERR_ARGUMENT, "bad matrix request");
    h->b->copy_matrix(which == 0 ? 2 : 3, m, out);
    return (int)NDDO_OK;
  });
}

int nddo_batch_get_forces(nddo_batch* h, int m, double* out) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() -> int {
    if (!out || m < 0 || m >= h->b->size()) return fail(h->ctx, NDDO_ERR_ARGUMENT, "bad forces request");
    if (!h->ran) return fail(h->ctx, NDDO_ERR_STATE, "no SCF result");
    std::vector<nddo::MolResult> r;
    h->b->results(&r);
    if (r[m].status != nddo::kConverged) return fail(h->ctx, NDDO_ERR_STATE, "forces need a converged SCF");
    h->b->forces(h->last, m, out);
    return (int)NDDO_OK;
  });
}

size_t nddo_batch_device_bytes(const nddo_batch* h) { return h ? h->b->device_bytes() : 0; }

long long nddo_batch_launch_count(const nddo_batch* h) { return h ? h->b->launches() : -1; }
long long nddo_batch_graph_launch_count(const nddo_batch* h) { return h ? h->b->graph_launches() : -1; }

long long nddo_batch_jacobi_sweeps(nddo_batch* h) {
  if (!h) return -1;
  try {
    return h->b->jacobi_sweeps();
  } catch (const std::exception& e) {
    h->ctx->err = e.what();
    return -1;
  }
}

void nddo_batch_destroy(nddo_batch* h) { delete h; }

int nddo_batch_profile(nddo_batch* h, int enable) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() {
    h->b->profile_reset();
    h->b->set_profiling(enable != 0);
    return (int)NDDO_OK;
  });
}

int nddo_batch_kernel_times(nddo_batch* h, int max_classes, double* ms, long long* launches, double* work) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() {
    double a[nddo::kKNumClasses], w[nddo::kKNumClasses];
    long long l[nddo::kKNumClasses];
    h->b->profile_collect(a, l, w);
    const int n = std::min<int>(max_classes, nddo::kKNumClasses);
    for (int k = 0; k < n; ++k) {
      if (ms) ms[k] = a[k];
      if (launches) launches[k] = l[k];
      if (work) work[k] = w[k];
    }
    return (int)nddo::kKNumClasses;
  });
}

const char* nddo_kernel_class_name(int k) { return nddo::kernel_class_name(k); }

int nddo_batch_timer(nddo_batch* h, int op, double* ms) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() {
    h->b->timer(op, ms);
    return (int)NDDO_OK;
  });
}

int nddo_measure_fma_peak(nddo_ctx* ctx, int precision, double* tflops) {
  return guarded(ctx, [&]() {
    if (!ctx->engine || !tflops) return fail(ctx, NDDO_ERR_ARGUMENT, "bad arguments");
    cudaStream_t s = ctx->engine->stream();
    *tflops = precision == 0 ? fma_peak<float>(s, 200000) : fma_peak<double>(s, 20000);
    return (int)NDDO_OK;
  });
}


int nddo_server_create(nddo_ctx* ctx, const nddo_scf_params* params, size_t hbm_budget_bytes, int max_basis,
                       nddo_server** out) {
  return guarded(ctx, [&]() -> int {
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    std::string why;
    if (!valid_params(params, &why)) return fail(ctx, NDDO_ERR_ARGUMENT, why);
    if (hbm_budget_bytes == 0) hbm_budget_bytes = ctx->budget ? ctx->budget : (size_t)64 << 30;
    if (ctx->budget && hbm_budget_bytes > ctx->budget)
      return fail(ctx, NDDO_ERR_BUDGET, "server budget exceeds the context budget");
    std::unique_ptr<nddo_server> h(new nddo_server());
    h->ctx = ctx;
    h->s.reset(new nddo::Server(ctx->engine.get(), to_settings(params), hbm_budget_bytes, max_basis));
    *out = h.release();
    return (int)NDDO_OK;
  });
}

int nddo_server_submit(nddo_server* h, int theory, int n_atoms, const int* Z, const double* xyz, long long* ticket) {
  return nddo_server_submit_epc(h, theory, n_atoms, Z, xyz, 0, nullptr, ticket);
}

int nddo_server_submit_epc(nddo_server* h, int theory, int n_atoms, const int* Z, const double* xyz, int n_epc,
                           const double* epc, long long* ticket) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() -> int {
    if (n_atoms < 1 || !Z || !xyz || !ticket) return fail(h->ctx, NDDO_ERR_ARGUMENT, "bad request arguments");
    if (n_epc < 0 || (n_epc > 0 && !epc)) return fail(h->ctx, NDDO_ERR_ARGUMENT, "invalid point charges");
    nddo::MoleculeInput in;
    in.theory = theory;
    in.Z.assign(Z, Z + n_atoms);
    in.xyz.assign(xyz, xyz + 3 * (size_t)n_atoms);
    if (n_epc > 0) in.epc.assign(epc, epc + 4 * (size_t)n_epc);
    *ticket = h->s->submit(in);
    return (int)NDDO_OK;
  });
}

int nddo_server_poll(nddo_server* h, int max_wait_us, int max_results, nddo_serve_result* out, double* charges,
                     size_t charges_capacity, int* n_out) {
  if (!h) return NDDO_ERR_ARGUMENT;
  return guarded(h->ctx, [&]() -> int {
    if (!n_out || (max_results > 0 && !out)) return fail(h->ctx, NDDO_ERR_ARGUMENT, "bad poll arguments");
    *n_out = 0;
    if (!h->has_held) h->s->poll(max_wait_us < 0 ? 0 : max_wait_us);
    size_t used = 0;
    while (*n_out < max_results) {
      if (!h->has_held) {
        if (!h->s->take(&h->held)) break;
        h->has_held = true;
      }
      const nddo::ServeResult& r = h->held;
      if (charges && used + r.charges.size() > charges_capacity) {
        if (*n_out == 0 && r.charges.size() > charges_capacity)
          return fail(h->ctx, NDDO_ERR_ARGUMENT, "charge buffer smaller than one result");
        break;
      }
      nddo_serve_result& o = out[*n_out];
      o.ticket = r.ticket; o.status = r.status; o.iterations = r.iterations; o.n_atoms = r.natoms; o.lane = r.lane;
      o.energy = r.energy; o.core_repulsion = r.core_repulsion; o.heat_of_formation = r.heat_of_formation;
      o.final_rms = r.final_rms; o.t_submit = r.t_submit; o.t_admit = r.t_admit; o.t_done = r.t_done;
      o.core_epc_coulomb = r.core_epc;
      if (charges) {
        std::copy(r.charges.begin(), r.charges.end(), charges + used);
        used += r.charges.size();
      }
      h->has_held = false;
      ++*n_out;
    }
    return (int)NDDO_OK;
  });
}

int nddo_server_pending(const nddo_server* h, int* queued, int* in_flight) {
  if (!h) return NDDO_ERR_ARGUMENT;
  if (queued) *queued = h->s->queued();
  if (in_flight) *in_flight = h->s->in_flight();
  return NDDO_OK;
}

double nddo_server_clock(const nddo_server* h) { return h ? h->s->now() : 0.0; }

size_t nddo_server_device_bytes(const nddo_server* h) { return h ? h->s->device_bytes() : 0; }

void nddo_server_destroy(nddo_server* h) { delete h; }

}  // extern "C"
