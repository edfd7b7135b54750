// Serving loop: continuous batching of single-point SCF requests.
//
// Requests are routed by basis size to lanes (a lane = one molecule pool with
// its own stream and its own host thread).  Each lane keeps every admitted
// molecule's integrals, density, eigenvectors and DIIS history resident on
// the device and runs one SCF iteration at a time over all of its molecules
// in flight; at every iteration boundary the molecules that converged leave
// (energy, charges, slot released) and queued requests that fit the lane's
// HBM arenas join.  Lanes advance independently, so a lane of large molecules
// never holds back the iterations of a lane of small ones; the small-molecule
// lane's stream has the highest priority.  A molecule's arithmetic does not
// depend on its neighbours (every kernel works per molecule with fixed-order
// reductions), so its result is the same alone and in any mix.
#pragma once
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace nddo {

struct ServeResult {
  long long ticket = -1;
  int status = 0, iterations = 0, natoms = 0, lane = 0;
  double energy = 0, core_repulsion = 0, heat_of_formation = 0, final_rms = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;   // seconds on the server clock
  double core_epc = 0;                            // core-point-charge Coulomb energy (included in energy)
  std::vector<double> charges;
};

class Server {
 public:
  // hbm_budget: device bytes for all lanes together; max_basis: largest N accepted
  Server(Engine* eng, const ScfSettings& s, size_t hbm_budget, int max_basis);
  ~Server();
  Server(const Server&) = delete;
  Server& operator=(const Server&) = delete;

  long long submit(const MoleculeInput& in);      // throws std::invalid_argument for a bad molecule
  // Waits up to max_wait_us for a finished request; returns how many are ready.
  int poll(int max_wait_us);
  bool take(ServeResult* out);
  int queued() const;
  int in_flight() const;
  double now() const;
  size_t device_bytes() const;
  // a lane thread's CUDA error, if any (the lane stops; the text is kept here)
  std::string error() const;

 private:
  struct Lane {
    int index = 0;
    int lo = 0, hi = 0;                       // basis sizes routed here: lo < N <= hi
    cudaStream_t stream = nullptr;
    std::unique_ptr<Batch> b;
    std::mutex mu;                            // guards queue / queue_t
    std::condition_variable cv;
    std::deque<std::pair<long long, MoleculeInput>> queue;
    std::deque<double> queue_t;               // submit time of each queued request (parallel to queue)
    std::atomic<int> n_queued{0}, n_active{0};
    // owned by the lane thread
    std::vector<int> active;
    std::vector<long long> slot_ticket;
    std::vector<double> slot_tsubmit, slot_tadmit;
    int* h_count = nullptr;
    char* h_active = nullptr;
    MolState* h_states = nullptr;
    double* h_charges = nullptr;
    cudaEvent_t ev = nullptr;
    std::thread th;
  };
  void lane_loop(Lane* L);
  bool lane_step(Lane& L);
  void publish(ServeResult&& r);

  Engine* eng_;
  ScfSettings s_;
  std::vector<std::unique_ptr<Lane>> lanes_;
  mutable std::mutex done_mu_;
  std::condition_variable done_cv_;
  std::deque<ServeResult> done_;
  std::string error_;
  std::atomic<bool> stop_{false};
  std::atomic<long long> next_ticket_{0};
  std::atomic<long long> outstanding_{0};   // submitted and not yet published
  std::chrono::steady_clock::time_point t0_;
};

}  // namespace nddo
