// Many WHIR proofs on one GPU: a pool of workers, each a host thread with its
// own stream (Context) and a reusable Prover, so that the kernels of
// different proofs overlap on the device while each proof waits on its own
// transcript round trips.  Jobs are released in arrival order; a job is
// admitted when it has arrived, a worker is free and the device bytes held
// by all workers stay within a budget.
//
// A job is the reference harness (crates/whir/src/test.rs:218-235) on one
// polynomial: commit, then per claim draw an expanded point and write the
// evaluation, then open; or the commitment alone.  The proof bytes of a job
// do not depend on which worker ran it or what ran beside it.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <chrono>
#include <functional>
#include <string>
#include <vector>

#include "prover.h"

namespace whir {

struct Job {
  Params params;
  const uint32_t *poly = nullptr;  // 2^k words, host or device memory
  bool on_device = false;
  int n_claims = 0;
  bool commit_only = false;
  double arrival = 0;  // seconds after the start of the run
  // results
  std::vector<uint8_t> proof;  // transcript bytes (the root is the first 32)
  uint32_t checkpoint = 0;     // one base element drawn after the proof
  int status = 0;
  std::string error;
  double start = 0, done = 0;  // seconds after the start of the run
  int worker = -1;
};

// Lock-step groups: a worker that takes the job at the head of the queue
// also takes later jobs that have arrived and are compatible with it (the
// same shape), up to max_group(head), to prove them together.  grow(worker,
// group) is the device bytes that worker would add to run the group; it is
// called on the worker's own thread with the admission lock held.
struct Grouping {
  std::function<bool(size_t head, size_t job)> compatible;
  std::function<int(size_t head)> max_group;
  std::function<size_t(int worker, const std::vector<int> &group)> grow;
};

// Release order and memory gate, independent of how a job is executed.
class Admission {
 public:
  using Clock = std::chrono::steady_clock;
  // need[j]: device bytes a worker holds while running job j alone; held[w]:
  // bytes worker w already holds
  Admission(const std::vector<double> &arrival, const std::vector<size_t> &need, size_t budget,
            const std::vector<size_t> &held, bool honor_arrival, Clock::time_point t0,
            const Grouping *grouping = nullptr);
  ~Admission();
  Admission(const Admission &) = delete;
  Admission &operator=(const Admission &) = delete;
  // Blocks until the next job (in arrival order) may start on `worker`;
  // returns it with the jobs grouped with it (the head first), or an empty
  // list when every job has been handed out.  A job whose need alone exceeds
  // the budget is returned alone with *too_big set, and so is a job that no
  // idle worker can hold next to what the others keep while nothing runs
  // (buffers only grow, so waiting would never end).  A group that does not
  // fit the budget is halved until it does (down to the head alone).
  std::vector<int> take(int worker, bool *too_big);
  // the worker finished its job and now holds `held` device bytes
  void release(int worker, size_t held);
  // the worker (taking no job) now holds `held` device bytes
  void set_held(int worker, size_t held);
  size_t peak_bytes() const { return peak_; }
  const std::vector<size_t> &held() const { return held_; }

 private:
  size_t grow_of(int worker, const std::vector<int> &group) const;
  void update_held(int worker, size_t held);  // with the lock held
  std::vector<size_t> order_;  // job indices by arrival
  std::vector<char> taken_;    // handed out (possibly ahead of the head, in a group)
  const Grouping *grouping_;
  std::vector<double> arrival_;
  std::vector<size_t> need_;
  size_t budget_;
  bool honor_;
  Clock::time_point t0_;
  size_t head_ = 0;
  std::vector<size_t> held_;  // bytes held per worker
  size_t total_ = 0, peak_ = 0;
  size_t running_ = 0;           // groups handed out and not yet released
  std::vector<char> blocked_;    // workers that found the head job does not fit
  size_t blocked_head_ = (size_t)-1;
  struct Sync;
  Sync *sync_;
};

struct RunStats {
  double seconds = 0;
  size_t peak_bytes = 0;
};

// Runs `jobs` on one host thread per entry of `states` (a worker's persistent
// state, created on first use by make_worker on its own thread).
// exec(state, group) does the work of a group of jobs (one job unless
// grouping is given) and returns the device bytes the worker holds
// afterwards.  held[w] (in/out) is what worker w holds across runs.
// prepare (optional) runs once on each worker thread before it takes jobs
// and returns the device bytes the worker then holds.  When exec throws, the
// group's jobs fail with the error and the worker goes on with later jobs;
// held_of (optional) then gives what the worker holds (a proof that failed
// may have grown its buffers first), else its holding before the group.
RunStats run_jobs(std::vector<Job> &jobs, std::vector<void *> &states, std::vector<size_t> &held,
                  size_t budget, bool honor_arrival,
                  const std::function<size_t(const Params &)> &need,
                  const std::function<void *(int worker)> &make_worker,
                  const std::function<size_t(void *state, std::vector<Job *> &group)> &exec,
                  const std::function<size_t(void *state)> &prepare = nullptr,
                  const Grouping *grouping = nullptr,
                  const std::function<size_t(void *state)> &held_of = nullptr);

// A pool of GPU workers on one device, kept between runs: each worker's
// stream, pinned staging and prover buffers stay allocated, so a run starts
// warm.  One run at a time.
class Server {
 public:
  Server(int device, int workers, size_t budget);
  ~Server();
  Server(const Server &) = delete;
  Server &operator=(const Server &) = delete;
  RunStats run(std::vector<Job> &jobs, bool honor_arrival);
  int workers() const { return (int)states_.size(); }
  // Lock-step groups of same-shape jobs (BatchProver): at most max_group
  // jobs per group; 1 proves every job alone; 0 restores the default.
  void set_lockstep(int max_group) { lockstep_ = max_group > 0 ? max_group : kLockstepDefault; }
  static constexpr int kLockstepDefault = 64;
  // a group holds at most 2^kGroupLog evaluations in all
  static constexpr int kGroupLog = 26;
  // jobs of at least 2^kPriorityK evaluations run on high-priority streams
  static constexpr int kPriorityK = 22;

 private:
  int device_;
  size_t budget_;
  int lockstep_ = kLockstepDefault;
  std::vector<void *> states_;
  std::vector<size_t> held_;
  struct Lock;
  Lock *lock_;
};

}  // namespace whir
