// Serving loop (see server.h).
#include "server.h"

#include <algorithm>
#include <stdexcept>
#include <thread>

namespace nddo {

namespace {
// Arena bytes that accompany one element of the N x N arena: pair blocks
// (at most 3.2 N^2 doubles, an all-heavy molecule), pair records, energies and
// index lists (at most N^2 / 2 pairs), atoms and charges (at most N^2 / 16).
constexpr double kBlocksPerMat = 3.2, kPairsPerMat = 0.5, kAtomsPerMat = 1.0 / 16.0;
constexpr double kEpcsPerAtom = 1.0;   // point-charge arena: as many charges as atoms
constexpr int kSmallLaneMaxN = 194;   // tridiagonalisation in shared memory
constexpr int kMidLaneMaxN = 400;

BatchCapacity lane_capacity(size_t bytes, int max_n, int min_n, int diis_m, int ws_slots) {
  const double per_mat = (double)Batch::bytes_per_mat_element(diis_m) + kBlocksPerMat * 8.0 +
                         kPairsPerMat * (sizeof(DevPair) + 8.0 + 8.0) +
                         kAtomsPerMat * (sizeof(DevAtom) + 8.0 + kEpcsPerAtom * 4 * sizeof(double));
  // the Jacobi workspaces come off the top
  const long long np = (max_n + 63) / 64 * 64;
  const double ws_bytes = max_n > 138 ? (double)ws_slots * np * np * (2 * 4 + 3 * 8) : 0.0;
  if ((double)bytes <= ws_bytes * 1.25) throw std::invalid_argument("HBM budget too small for the serving lanes");
  BatchCapacity c;
  c.mat = (long long)(((double)bytes - ws_bytes) / per_mat);
  c.blocks = (long long)(kBlocksPerMat * c.mat) + 128;
  c.pairs = (long long)(kPairsPerMat * c.mat) + 64;
  c.atoms = (long long)(kAtomsPerMat * c.mat) + 64;
  c.epcs = (long long)(kEpcsPerAtom * (double)c.atoms);
  const long long min_mat = std::max<long long>(32, ((long long)min_n * min_n + 31) / 32 * 32);
  c.vec = c.mat / 4 + 1024;
  c.slots = (int)std::max<long long>(1, std::min<long long>(4096, c.mat / min_mat));
  c.max_n = max_n;
  c.ws_slots = ws_slots;
  if (c.mat < (long long)max_n * max_n) throw std::invalid_argument("HBM budget too small for the largest basis");
  return c;
}
}  // namespace

Server::Server(Engine* eng, const ScfSettings& s, size_t hbm_budget, int max_basis) : eng_(eng), s_(s) {
  if (max_basis < 2) throw std::invalid_argument("max_basis must be >= 2");
  s_.keep_trace = 0;
  t0_ = std::chrono::steady_clock::now();
  const int m = s_.diis_num_error_vect;
  // lanes by basis size: the per-molecule eigensolver with its matrix in shared
  // memory (<= 194), in a global workspace up to 400, and the larger ones
  // (whole-GPU eigensolver kernels when few are resident; the only lane that
  // issues cooperative launches)
  struct Spec { int lo, hi; double share; int min_n, ws; };
  std::vector<Spec> specs;
  if (max_basis <= kSmallLaneMaxN) specs.push_back({0, max_basis, 1.0, 2, 1});
  else if (max_basis <= kMidLaneMaxN) {
    specs.push_back({0, kSmallLaneMaxN, 0.4, 2, 1});
    specs.push_back({kSmallLaneMaxN, max_basis, 0.6, kSmallLaneMaxN + 1, 32});
  } else {
    specs.push_back({0, kSmallLaneMaxN, 0.3, 2, 1});
    specs.push_back({kSmallLaneMaxN, kMidLaneMaxN, 0.3, kSmallLaneMaxN + 1, 32});
    specs.push_back({kMidLaneMaxN, max_basis, 0.4, kMidLaneMaxN + 1, 16});
  }
  int prio_lo = 0, prio_hi = 0;   // numerically lower = higher priority
  cuda_check(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi), "stream priorities");
  for (size_t k = 0; k < specs.size(); ++k) {
    const Spec& sp = specs[k];
    std::unique_ptr<Lane> L(new Lane());
    L->index = (int)k;
    L->lo = sp.lo;
    L->hi = sp.hi;
    const int prio = k == 0 ? prio_hi : prio_lo;
    cuda_check(cudaStreamCreateWithPriority(&L->stream, cudaStreamNonBlocking, prio), "lane stream");
    cuda_check(cudaEventCreateWithFlags(&L->ev, cudaEventDisableTiming), "lane event");
    BatchCapacity c = lane_capacity((size_t)(sp.share * (double)hbm_budget), sp.hi, sp.min_n, m, sp.ws);
    L->b.reset(new Batch(eng_, c, m, L->stream));
    const int slots = c.slots;
    L->slot_ticket.assign(slots, -1);
    L->slot_tsubmit.assign(slots, 0.0);
    L->slot_tadmit.assign(slots, 0.0);
    cuda_check(cudaHostAlloc(&L->h_count, sizeof(int), cudaHostAllocDefault), "pinned");
    cuda_check(cudaHostAlloc(&L->h_active, slots, cudaHostAllocDefault), "pinned");
    cuda_check(cudaHostAlloc(&L->h_states, slots * sizeof(MolState), cudaHostAllocDefault), "pinned");
    cuda_check(cudaHostAlloc(&L->h_charges, c.atoms * sizeof(double), cudaHostAllocDefault), "pinned");
    lanes_.push_back(std::move(L));
  }
  for (auto& L : lanes_) L->th = std::thread(&Server::lane_loop, this, L.get());
}

Server::~Server() {
  stop_ = true;
  for (auto& L : lanes_) {
    { std::lock_guard<std::mutex> g(L->mu); }
    L->cv.notify_all();
  }
  for (auto& L : lanes_) if (L->th.joinable()) L->th.join();
  for (auto& L : lanes_) {
    if (L->stream) cudaStreamSynchronize(L->stream);
    L->b.reset();
    if (L->h_count) cudaFreeHost(L->h_count);
    if (L->h_active) cudaFreeHost(L->h_active);
    if (L->h_states) cudaFreeHost(L->h_states);
    if (L->h_charges) cudaFreeHost(L->h_charges);
    if (L->ev) cudaEventDestroy(L->ev);
    if (L->stream) cudaStreamDestroy(L->stream);
  }
}

double Server::now() const {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

size_t Server::device_bytes() const {
  size_t t = 0;
  for (const auto& L : lanes_) t += L->b->device_bytes();
  return t;
}

std::string Server::error() const {
  std::lock_guard<std::mutex> g(done_mu_);
  return error_;
}

long long Server::submit(const MoleculeInput& in) {
  {
    std::lock_guard<std::mutex> g(done_mu_);
    if (!error_.empty()) throw std::runtime_error("server stopped: " + error_);
  }
  if (in.theory < 0 || in.theory >= NDDO_NUM_THEORY_SLOTS) throw std::invalid_argument("unknown theory");
  int nao = 0, nelec = 0;
  for (int z : in.Z) {
    const int e = nddo_element_index(z);
    nddo_atom_params probe;
    if (e < 0 || nddo_fill_atom_params(in.theory, z, &probe) != 0)
      throw std::invalid_argument("element " + std::to_string(z) + " has no parameters for this theory");
    nao += nddo_elements[e].n_ao;
    nelec += nddo_elements[e].core_charge;
  }
  if (in.Z.empty()) throw std::invalid_argument("molecule without atoms");
  if ((int)in.xyz.size() != 3 * (int)in.Z.size()) throw std::invalid_argument("coordinate count does not match atom count");
  if (in.theory < 0 || in.theory >= NDDO_NUM_THEORY_SLOTS) throw std::invalid_argument("unknown theory");
  if (nelec % 2) throw std::invalid_argument("Total number of valence electrons is odd. totalNumberValenceElectrons=" + std::to_string(nelec));
  if (in.epc.size() % 4) throw std::invalid_argument("point charges need x, y, z and a charge each");
  for (auto& L : lanes_) {
    if (nao > L->lo && nao <= L->hi) {
      if ((long long)(in.epc.size() / 4) > L->b->epc_capacity())
        throw std::invalid_argument("more point charges than the lane's pool holds");
      const long long t = next_ticket_++;
      ++outstanding_;
      {
        std::lock_guard<std::mutex> g(L->mu);
        L->queue.emplace_back(t, in);
        L->queue_t.push_back(now());
        L->n_queued = (int)L->queue.size();
      }
      L->cv.notify_one();
      return t;
    }
  }
  throw std::invalid_argument("molecule with " + std::to_string(nao) + " basis functions exceeds the server's largest basis");
}

int Server::queued() const {
  int q = 0;
  for (const auto& L : lanes_) q += L->n_queued;
  return q;
}

int Server::in_flight() const {
  // submitted, not queued and not yet published (admitted, in the SCF, or
  // between the two inside a lane step)
  const long long f = outstanding_ - queued();
  return (int)(f > 0 ? f : 0);
}

void Server::publish(ServeResult&& r) {
  {
    std::lock_guard<std::mutex> g(done_mu_);
    done_.push_back(std::move(r));
    --outstanding_;
  }
  done_cv_.notify_all();
}

bool Server::take(ServeResult* out) {
  std::lock_guard<std::mutex> g(done_mu_);
  if (done_.empty()) return false;
  *out = std::move(done_.front());
  done_.pop_front();
  return true;
}

int Server::poll(int max_wait_us) {
  std::unique_lock<std::mutex> g(done_mu_);
  if (done_.empty() && error_.empty() && max_wait_us > 0)
    done_cv_.wait_for(g, std::chrono::microseconds(max_wait_us),
                      [&] { return !done_.empty() || !error_.empty(); });
  if (!error_.empty() && done_.empty()) throw std::runtime_error("server stopped: " + error_);
  return (int)done_.size();
}

void Server::lane_loop(Lane* L) {
  try {
    cuda_check(cudaSetDevice(eng_->device()), "cudaSetDevice");
    while (!stop_) {
      if (!lane_step(*L)) {
        // idle: wait for a request
        std::unique_lock<std::mutex> g(L->mu);
        L->cv.wait_for(g, std::chrono::milliseconds(50), [&] { return stop_ || !L->queue.empty(); });
      }
    }
  } catch (const std::exception& e) {
    {
      std::lock_guard<std::mutex> g(done_mu_);
      if (error_.empty()) error_ = "lane " + std::to_string(L->index) + ": " + e.what();
    }
    done_cv_.notify_all();
  }
}

// One step of a lane: admit queued requests that fit, run one SCF iteration
// over every molecule in flight, retire the molecules it finished.  Returns
// false when the lane had nothing to do.
bool Server::lane_step(Lane& L) {
  Batch& b = *L.b;
  // admission in arrival order while the head request fits the lane's arenas
  std::vector<int> fresh;
  for (;;) {
    std::pair<long long, MoleculeInput> req;
    double tq = 0.0;
    {
      std::lock_guard<std::mutex> g(L.mu);
      if (L.queue.empty()) break;
      req = L.queue.front();
      tq = L.queue_t.front();
    }
    int slot = -1;
    bool invalid = false;
    try {
      slot = b.admit(req.second);
    } catch (const std::invalid_argument&) {
      invalid = true;   // a molecule its layout rejects (coincident atoms, a charge on an atom, ...)
    }
    if (invalid || (slot < 0 && L.active.empty() && fresh.empty())) {
      // rejected, or cannot fit even into an empty lane: fail the request rather than wait forever
      ServeResult r;
      r.ticket = req.first;
      r.status = kFailed;
      r.natoms = (int)req.second.Z.size();
      r.t_submit = tq;
      r.t_admit = r.t_done = now();
      r.lane = L.index;
      {
        std::lock_guard<std::mutex> g(L.mu);
        L.queue.pop_front();
        L.queue_t.pop_front();
        L.n_queued = (int)L.queue.size();
      }
      publish(std::move(r));
      continue;
    }
    if (slot < 0) break;
    {
      std::lock_guard<std::mutex> g(L.mu);
      L.queue.pop_front();
      L.queue_t.pop_front();
      L.n_queued = (int)L.queue.size();
    }
    L.slot_ticket[slot] = req.first;
    L.slot_tsubmit[slot] = tq;
    L.slot_tadmit[slot] = now();
    fresh.push_back(slot);
  }
  if (!fresh.empty()) {
    b.integrals(fresh);
    b.begin(s_, fresh, true);
    L.active.insert(L.active.end(), fresh.begin(), fresh.end());
  }
  L.n_active = (int)L.active.size();
  if (L.active.empty()) return false;
  b.iterate(s_, L.active);
  b.count_active_async(L.active, L.h_count, L.h_active, L.ev);
  cuda_check(cudaEventSynchronize(L.ev), "lane iteration");
  std::vector<int> fin, still;
  for (int m : L.active) (L.h_active[m] ? still : fin).push_back(m);
  if (!fin.empty()) {
    b.finish(s_, fin);
    b.copy_states_async(L.h_states);
    for (int m : fin) b.copy_charges_async(m, L.h_charges + b.mol_table()[m].atom0);
    cuda_check(cudaStreamSynchronize(L.stream), "lane results");
    const double t = now();
    for (int m : fin) {
      const MolState& st = L.h_states[m];
      const DevMol& d = b.mol_table()[m];
      ServeResult r;
      r.ticket = L.slot_ticket[m];
      r.status = st.status;
      r.iterations = st.status == kConverged ? st.iter + 1 : st.iter;
      r.energy = st.energy;
      r.core_repulsion = st.ecore;
      r.heat_of_formation = st.heat_of_formation;
      r.final_rms = st.rms;
      r.core_epc = st.ecore_epc;
      r.natoms = d.natoms;
      r.lane = L.index;
      r.t_submit = L.slot_tsubmit[m];
      r.t_admit = L.slot_tadmit[m];
      r.t_done = t;
      r.charges.assign(L.h_charges + d.atom0, L.h_charges + d.atom0 + d.natoms);
      L.slot_ticket[m] = -1;
      b.release(m);
      publish(std::move(r));
    }
  }
  L.active.swap(still);
  L.n_active = (int)L.active.size();
  return true;
}

}  // namespace nddo
