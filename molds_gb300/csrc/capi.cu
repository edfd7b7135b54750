// extern "C" boundary (include/nddo_gpu.h) over the batched engine.
#include "../../include/nddo_gpu.h"

#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"

struct nddo_ctx {
  std::unique_ptr<nddo::Engine> engine;
  std::unique_ptr<nddo::Batch> mol;      // current molecule (SetMolecule / DoSCF API)
  nddo::ScfSettings last_settings;
  bool has_scf = false;
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
  ctx->mol.reset();
  ctx->engine.reset();
  delete ctx;
}

const char* nddo_last_error(const nddo_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int nddo_set_molecule(nddo_ctx* ctx, int theory, int n_atoms, const int* Z, const double* xyz) {
  return guarded(ctx, [&]() {
    if (!ctx->engine) return fail(ctx, NDDO_ERR_STATE, "engine not initialised");
    if (n_atoms < 1 || !Z || !xyz) return fail(ctx, NDDO_ERR_ARGUMENT, "need at least one atom");
    nddo::MoleculeInput in;
    in.theory = theory;
    in.Z.assign(Z, Z + n_atoms);
    in.xyz.assign(xyz, xyz + 3 * (size_t)n_atoms);
    ctx->mol.reset();
    ctx->has_scf = false;
    std::unique_ptr<nddo::Batch> b(new nddo::Batch(ctx->engine.get(), {in}, 5));
    if (ctx->budget && b->device_bytes() > ctx->budget)
      return fail(ctx, NDDO_ERR_BUDGET, "molecule needs " + std::to_string(b->device_bytes()) + " bytes of HBM, budget is " + std::to_string(ctx->budget));
    b->integrals();
    ctx->mol = std::move(b);
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
    ctx->mol->scf(s, requires_guess != 0);
    std::vector<nddo::MolResult> r;
    ctx->mol->results(&r);
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

int nddo_get_core_hamiltonian(nddo_ctx* ctx, double* out) {
  return guarded(ctx, [&]() {
    if (!ctx->mol) return fail(ctx, NDDO_ERR_STATE, "A molecule is not set.");
    if (!out) return fail(ctx, NDDO_ERR_ARGUMENT, "null output buffer");
    ctx->mol->copy_matrix(0, 0, out);
    return (int)NDDO_OK;
  });
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
    nddo::Batch b(ctx->engine.get(), mols, s.diis_num_error_vect);
    if (ctx->budget && b.device_bytes() > ctx->budget)
      return fail(ctx, NDDO_ERR_BUDGET, "batch needs " + std::to_string(b.device_bytes()) + " bytes of HBM, budget is " + std::to_string(ctx->budget));
    b.integrals();
    b.scf(s, true);
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
      if (r[i].status != nddo::kConverged) rc = NDDO_NOT_CONVERGED;
      if (charges) b.copy_charges(i, charges + off);
      off += n_atoms[i];
    }
    if (rc != NDDO_OK) ctx->err = "SCF did not met convergence criterion for at least one molecule";
    return rc;
  });
}

}  // extern "C"
