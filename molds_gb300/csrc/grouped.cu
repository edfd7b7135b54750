// Grouped batch: concurrent molecule groups on their own streams (engine.h).
#include <algorithm>
#include <cstdlib>
#include <exception>
#include <stdexcept>
#include <thread>

#include "engine.h"
#include "kernels.h"
#include "tuning.h"

namespace nddo {

int GroupedBatch::default_groups(int n_mol) {
  // concurrent molecule groups by batch size, from the autotuner's table;
  // MOLDS_GB300_GROUPS overrides the count (sweeps)
  if (const char* e = std::getenv("MOLDS_GB300_GROUPS")) {
    const int g = std::atoi(e);
    if (g >= 1) return std::min(g, std::max(1, n_mol));
  }
  return tuned_groups(n_mol);
}

GroupedBatch::GroupedBatch(Engine* eng, const std::vector<MoleculeInput>& mols, int diis_m, int groups) {
  if (mols.empty()) throw std::invalid_argument("empty batch");
  n_ = (int)mols.size();
  device_ = eng->device();
  groups = std::max(1, std::min(groups, n_));
  // molecules that may run on the whole-GPU eigensolver take every SM in its
  // cooperative launches: two groups with such molecules must not wait for
  // each other's SMs, so such batches run as one group
  for (const MoleculeInput& m : mols)
    if (molecule_nao(m) >= kGridShareMinN) { groups = 1; break; }
  // contiguous groups of near-equal molecule count, in input order
  int atom = 0, mol = 0;
  for (int g = 0; g < groups; ++g) {
    const int cnt = n_ / groups + (g < n_ % groups ? 1 : 0);
    std::vector<MoleculeInput> part(mols.begin() + mol, mols.begin() + mol + cnt);
    cudaStream_t st = nullptr;
    if (g == 0 && groups == 1) {
      st = eng->stream();
    } else {
      cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "group stream");
      streams_.push_back(st);
    }
    first_mol_.push_back(mol);
    first_atom_.push_back(atom);
    g_.emplace_back(new Batch(eng, part, diis_m, st));
    for (const MoleculeInput& m : part) atom += (int)m.Z.size();
    mol += cnt;
  }
  first_mol_.push_back(mol);
  first_atom_.push_back(atom);
}

GroupedBatch::~GroupedBatch() {
  for (cudaEvent_t e : t0_) cudaEventDestroy(e);
  for (cudaEvent_t e : t1_) cudaEventDestroy(e);
  g_.clear();
  for (cudaStream_t s : streams_) cudaStreamDestroy(s);
}

void GroupedBatch::run(const ScfSettings& s, bool requires_guess) {
  if (g_.size() == 1) {
    g_[0]->integrals();
    g_[0]->scf(s, requires_guess);
    return;
  }
  std::vector<std::exception_ptr> err(g_.size());
  std::vector<std::thread> th;
  for (size_t g = 0; g < g_.size(); ++g)
    th.emplace_back([&, g]() {
      try {
        cuda_check(cudaSetDevice(device_), "cudaSetDevice");
        g_[g]->integrals();
        g_[g]->scf(s, requires_guess);
      } catch (...) {
        err[g] = std::current_exception();
      }
    });
  for (std::thread& t : th) t.join();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
}

const Batch& GroupedBatch::locate(int m, int* local) const {
  if (m < 0 || m >= n_) throw std::invalid_argument("molecule index out of range");
  const int g = (int)(std::upper_bound(first_mol_.begin(), first_mol_.end(), m) - first_mol_.begin()) - 1;
  *local = m - first_mol_[g];
  return *g_[g];
}

void GroupedBatch::results(std::vector<MolResult>* out) {
  out->clear();
  for (auto& b : g_) {
    std::vector<MolResult> r;
    b->results(&r);
    out->insert(out->end(), r.begin(), r.end());
  }
}

void GroupedBatch::copy_charges(int m, double* host) const {
  int l = 0;
  const Batch& b = locate(m, &l);
  b.copy_charges(l, host);
}

void GroupedBatch::forces(const ScfSettings& s, int m, double* host) {
  int l = 0;
  const Batch& b = locate(m, &l);
  for (auto& g : g_)
    if (g.get() == &b) { g->forces(s, l, host); return; }
}

void GroupedBatch::copy_matrix(int which, int m, double* host) const {
  int l = 0;
  const Batch& b = locate(m, &l);
  b.copy_matrix(which, l, host);
}

void GroupedBatch::cartesian_matrix(int m, double* host) const {
  int l = 0;
  const Batch& b = locate(m, &l);
  b.cartesian_matrix(l, host);
}

void GroupedBatch::set_coordinates(const double* xyz) {
  for (size_t g = 0; g < g_.size(); ++g) g_[g]->set_coordinates(xyz + 3 * (size_t)first_atom_[g]);
}

size_t GroupedBatch::device_bytes() const {
  size_t t = 0;
  for (const auto& b : g_) t += b->device_bytes();
  return t;
}

long long GroupedBatch::launches() const {
  long long t = 0;
  for (const auto& b : g_) t += b->launches();
  return t;
}

long long GroupedBatch::graph_launches() const {
  long long t = 0;
  for (const auto& b : g_) t += b->graph_launches();
  return t;
}

long long GroupedBatch::jacobi_sweeps() const {
  long long t = 0;
  for (const auto& b : g_) t += b->jacobi_sweeps();
  return t;
}

void GroupedBatch::set_profiling(bool on) {
  for (auto& b : g_) b->set_profiling(on);
}

void GroupedBatch::profile_reset() {
  for (auto& b : g_) b->profile_reset();
}

void GroupedBatch::profile_collect(double* ms, long long* launches, double* work) {
  for (int k = 0; k < kKNumClasses; ++k) { ms[k] = 0; launches[k] = 0; work[k] = 0; }
  for (auto& b : g_) {
    double a[kKNumClasses], w[kKNumClasses];
    long long l[kKNumClasses];
    b->profile_collect(a, l, w);
    for (int k = 0; k < kKNumClasses; ++k) { ms[k] += a[k]; launches[k] += l[k]; work[k] += w[k]; }
  }
}

// Start and stop events on every group's stream (recorded while the streams
// are idle); the elapsed time is from the first start to the last stop.
void GroupedBatch::timer(int op, double* ms) {
  const size_t G = g_.size();
  if (t0_.empty()) {
    t0_.resize(G);
    t1_.resize(G);
    for (size_t g = 0; g < G; ++g) {
      cuda_check(cudaEventCreate(&t0_[g]), "cudaEventCreate");
      cuda_check(cudaEventCreate(&t1_[g]), "cudaEventCreate");
    }
  }
  if (op == 0) {
    for (size_t g = 0; g < G; ++g) cuda_check(cudaEventRecord(t0_[g], g_[g]->stream()), "cudaEventRecord");
  } else if (op == 1) {
    for (size_t g = 0; g < G; ++g) cuda_check(cudaEventRecord(t1_[g], g_[g]->stream()), "cudaEventRecord");
  } else {
    float best = 0.f;
    for (size_t g = 0; g < G; ++g) {
      cuda_check(cudaEventSynchronize(t1_[g]), "cudaEventSynchronize");
      for (size_t h = 0; h < G; ++h) {
        float t = 0.f;
        cuda_check(cudaEventElapsedTime(&t, t0_[h], t1_[g]), "cudaEventElapsedTime");
        best = std::max(best, t);
      }
    }
    if (ms) *ms = best;
  }
}

}  // namespace nddo
