// Job runner for batched and served proving (see batch.h).
#include "batch.h"

#include "batch_prover.h"

#include <algorithm>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>

namespace whir {

struct Admission::Sync {
  std::mutex mu;
  std::condition_variable cv;
};

Admission::Admission(const std::vector<double> &arrival, const std::vector<size_t> &need,
                     size_t budget, const std::vector<size_t> &held, bool honor_arrival,
                     Clock::time_point t0, const Grouping *grouping)
    : taken_(arrival.size(), 0), grouping_(grouping), arrival_(arrival), need_(need),
      budget_(budget), honor_(honor_arrival), t0_(t0), held_(held), blocked_(held.size(), 0),
      sync_(new Sync) {
  order_.resize(arrival.size());
  for (size_t i = 0; i < order_.size(); i++) order_[i] = i;
  // ties keep submission order
  std::stable_sort(order_.begin(), order_.end(),
                   [&](size_t a, size_t b) { return arrival_[a] < arrival_[b]; });
  for (size_t h : held_) total_ += h;
  peak_ = total_;
}

Admission::~Admission() { delete sync_; }

size_t Admission::grow_of(int worker, const std::vector<int> &group) const {
  if (grouping_ && grouping_->grow) return grouping_->grow(worker, group);
  // buffers only grow: the worker ends up holding max(held, need)
  const size_t nd = need_[group[0]];
  return nd > held_[worker] ? nd - held_[worker] : 0;
}

std::vector<int> Admission::take(int worker, bool *too_big) {
  std::unique_lock<std::mutex> lock(sync_->mu);
  *too_big = false;
  for (;;) {
    while (head_ < order_.size() && taken_[order_[head_]]) head_++;
    if (head_ >= order_.size()) return {};
    size_t j = order_[head_];
    if (honor_) {
      auto due = t0_ + std::chrono::duration_cast<Clock::duration>(
                           std::chrono::duration<double>(arrival_[j]));
      if (Clock::now() < due) {
        sync_->cv.wait_until(lock, due);
        continue;
      }
    }
    if (need_[j] > budget_) {  // can never run: hand it out to be failed
      taken_[j] = 1;
      head_++;
      *too_big = true;
      running_++;
      sync_->cv.notify_all();
      return {(int)j};
    }
    std::vector<int> group{(int)j};
    if (grouping_) {
      const int mx = grouping_->max_group(j);
      const auto now = Clock::now();
      for (size_t q = head_ + 1; q < order_.size() && (int)group.size() < mx; q++) {
        const size_t c = order_[q];
        if (taken_[c] || need_[c] > budget_) continue;
        if (honor_ && now < t0_ + std::chrono::duration_cast<Clock::duration>(
                                      std::chrono::duration<double>(arrival_[c])))
          break;  // arrival order: no later job has arrived either
        if (grouping_->compatible(j, c)) group.push_back((int)c);
      }
    }
    for (;;) {
      const size_t grow = grow_of(worker, group);
      if (total_ + grow <= budget_) {
        for (int g : group) taken_[g] = 1;
        held_[worker] += grow;
        total_ += grow;
        peak_ = std::max(peak_, total_);
        running_++;
        sync_->cv.notify_all();
        return group;
      }
      if (group.size() == 1) break;
      group.resize(group.size() / 2);
    }
    // The head does not fit beside what the other workers hold.  A release
    // may free enough; but when nothing runs and every worker has found it
    // does not fit, no release will come: fail it instead of waiting.
    if (blocked_head_ != j) {
      std::fill(blocked_.begin(), blocked_.end(), 0);
      blocked_head_ = j;
    }
    blocked_[worker] = 1;
    if (running_ == 0 && std::all_of(blocked_.begin(), blocked_.end(), [](char b) { return b; })) {
      taken_[j] = 1;
      head_++;
      *too_big = true;
      running_++;
      sync_->cv.notify_all();
      return {(int)j};
    }
    sync_->cv.wait(lock);
  }
}

void Admission::release(int worker, size_t held) {
  std::lock_guard<std::mutex> lock(sync_->mu);
  running_--;
  update_held(worker, held);
}

void Admission::set_held(int worker, size_t held) {
  std::lock_guard<std::mutex> lock(sync_->mu);
  update_held(worker, held);
}

void Admission::update_held(int worker, size_t held) {
  blocked_head_ = (size_t)-1;  // the holdings changed: every worker looks again
  total_ = total_ - held_[worker] + held;
  held_[worker] = held;
  peak_ = std::max(peak_, total_);
  sync_->cv.notify_all();
}

RunStats run_jobs(std::vector<Job> &jobs, std::vector<void *> &states, std::vector<size_t> &held,
                  size_t budget, bool honor_arrival,
                  const std::function<size_t(const Params &)> &need,
                  const std::function<void *(int worker)> &make_worker,
                  const std::function<size_t(void *state, std::vector<Job *> &group)> &exec,
                  const std::function<size_t(void *state)> &prepare,
                  const Grouping *grouping,
                  const std::function<size_t(void *state)> &held_of) {
  const int workers = (int)states.size();
  if (workers < 1 || held.size() != states.size()) throw WhirError(-1, "at least one worker");
  std::vector<double> arr(jobs.size());
  std::vector<size_t> nd(jobs.size());
  for (size_t i = 0; i < jobs.size(); i++) {
    if (!(jobs[i].arrival >= 0)) throw WhirError(-1, "negative arrival time");
    arr[i] = jobs[i].arrival;
    nd[i] = need(jobs[i].params);
  }
  auto t0 = Admission::Clock::now();
  auto secs = [&] {
    return std::chrono::duration<double>(Admission::Clock::now() - t0).count();
  };
  Admission adm(arr, nd, budget, held, honor_arrival, t0, grouping);
  std::vector<std::thread> th;
  std::vector<std::string> start_err(workers);
  for (int w = 0; w < workers; w++) {
    th.emplace_back([&, w] {
      if (!states[w]) {
        try {
          states[w] = make_worker(w);
        } catch (const std::exception &e) {
          start_err[w] = e.what();
        }
      }
      void *state = states[w];
      if (state && prepare) {
        try {
          adm.set_held(w, prepare(state));
        } catch (const std::exception &e) {
          start_err[w] = e.what();
          state = nullptr;  // its jobs fail with the reason
        }
      }
      for (;;) {
        bool too_big = false;
        std::vector<int> taken = adm.take(w, &too_big);
        if (taken.empty()) break;
        std::vector<Job *> group;
        const double start = secs();
        for (int j : taken) {
          group.push_back(&jobs[j]);
          jobs[j].worker = w;
          jobs[j].start = start;
        }
        size_t now_held = adm.held()[w];
        int status = 0;
        std::string error;
        if (!state) {
          status = -5;
          error = "worker could not start: " + start_err[w];
          now_held = 0;
        } else if (too_big) {
          status = -4;
          error = "job does not fit the device budget (alone, or beside the buffers the idle "
                  "workers keep)";
        } else {
          bool failed = false;
          try {
            now_held = exec(state, group);
          } catch (const WhirError &e) {
            status = e.code;
            error = e.what();
            failed = true;
          } catch (const std::exception &e) {
            status = -5;
            error = e.what();
            failed = true;
          }
          if (failed && held_of) now_held = std::max(now_held, held_of(state));
        }
        const double done = secs();
        for (Job *job : group) {
          job->status = status;
          job->error = error;
          job->done = done;
        }
        adm.release(w, now_held);
      }
    });
  }
  for (auto &t : th) t.join();
  held = adm.held();
  RunStats st;
  st.seconds = secs();
  st.peak_bytes = adm.peak_bytes();
  return st;
}

namespace {
struct GpuWorker {
  std::unique_ptr<Context> ctx;
  std::unique_ptr<Prover> prover;
  std::unique_ptr<BatchProver> group_prover;  // lock-step groups, made on first use
  size_t bytes() const {
    return (prover ? prover->device_bytes() : 0) + (group_prover ? group_prover->device_bytes() : 0);
  }
};
bool same_shape(const Job &a, const Job &b) {
  const Params &p = a.params, &q = b.params;
  return p.k == q.k && p.folding == q.folding && p.rate == q.rate &&
         p.initial_reduction == q.initial_reduction && p.soundness == q.soundness &&
         p.security_level == q.security_level && a.n_claims == b.n_claims &&
         a.commit_only == b.commit_only && a.on_device == b.on_device;
}
}  // namespace

struct Server::Lock {
  std::mutex mu;
};

Server::Server(int device, int workers, size_t budget)
    : device_(device), budget_(budget), states_(workers, nullptr), held_(workers, 0),
      lock_(new Lock) {
  if (workers < 1 || workers > 256) {
    delete lock_;
    throw WhirError(-1, "workers out of range");
  }
}

Server::~Server() {
  for (void *s : states_) {
    auto *w = static_cast<GpuWorker *>(s);
    if (!w) continue;
    cudaSetDevice(device_);
    if (w->ctx) cudaStreamSynchronize(w->ctx->stream());
    delete w;
  }
  delete lock_;
}

RunStats Server::run(std::vector<Job> &jobs, bool honor_arrival) {
  std::lock_guard<std::mutex> guard(lock_->mu);
  for (auto &j : jobs) {
    if (!j.poly) throw WhirError(-1, "job without a polynomial");
    if (j.n_claims < 0 || j.n_claims > 64) throw WhirError(-1, "claims per job out of range");
    Prover::workspace_bytes(j.params);  // validates the parameters
  }
  const int device = device_;
  // more than one worker: poll-and-yield waits, so that workers waiting on
  // the GPU leave the host cores to the workers that have host work
  const bool yield = states_.size() > 1;
  auto need = [](const Params &p) { return Prover::workspace_bytes(p); };
  auto make = [device, yield](int) -> void * {
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    std::unique_ptr<GpuWorker> w(new GpuWorker);
    w->ctx.reset(new Context(device));
    w->ctx->set_yield_wait(yield);
    return w.release();
  };
  // Grow every worker's buffers to all shapes of this run first, in a pass
  // of its own before the run's clock starts: a buffer that grows during
  // the run frees its old allocation, and cudaFree synchronises every stream
  // of the device, stalling all workers (the served stream's p99 latency
  // rose from 20 to 150+ ms when that happened).  Only when every worker
  // can hold the union of the shapes within the budget.
  std::vector<Params> shapes;
  for (auto &j : jobs) {
    bool seen = false;
    for (auto &q : shapes)
      seen = seen || (q.k == j.params.k && q.folding == j.params.folding &&
                      q.rate == j.params.rate && q.initial_reduction == j.params.initial_reduction &&
                      q.soundness == j.params.soundness &&
                      q.security_level == j.params.security_level);
    if (!seen) shapes.push_back(j.params);
  }
  if (!shapes.empty() && workspace_union_bytes(shapes) * states_.size() <= budget_) {
    auto prepare = [device, &shapes](void *state) -> size_t {
      cuda_check(cudaSetDevice(device), "cudaSetDevice");
      auto *w = static_cast<GpuWorker *>(state);
      if (!w->prover) w->prover.reset(new Prover(w->ctx.get(), shapes[0]));
      for (auto &p : shapes) {
        w->prover->set_params(p);
        w->prover->reserve();
      }
      cuda_check(cudaStreamSynchronize(w->ctx->stream()), "sync");
      return w->bytes();
    };
    std::vector<Job> none;
    run_jobs(none, states_, held_, budget_, false, need, make, nullptr, prepare);
  }
  const int host_threads = (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
  auto exec = [device, host_threads](void *state, std::vector<Job *> &group) -> size_t {
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    auto *w = static_cast<GpuWorker *>(state);
    const Job &head = *group[0];
    // large jobs set the tail latency: their blocks go first on the device
    w->ctx->set_high_priority(head.params.k >= Server::kPriorityK);
    if (group.size() > 1) {  // lock step: every pass of the group in one launch
      if (!w->group_prover)
        w->group_prover.reset(new BatchProver(w->ctx.get(), head.params, host_threads));
      else
        w->group_prover->set_params(head.params);
      std::vector<Transcript> ts(group.size());
      std::vector<Transcript *> tp;
      std::vector<const uint32_t *> polys;
      for (size_t i = 0; i < group.size(); i++) {
        tp.push_back(&ts[i]);
        polys.push_back(group[i]->poly);
      }
      w->group_prover->prove(tp, polys, head.on_device, head.commit_only ? 0 : head.n_claims,
                             head.commit_only, [&](int i) {
                               group[i]->checkpoint = ts[i].draw_fe();
                               group[i]->proof = ts[i].bytes();
                             });
      return w->bytes();
    }
    Job &job = *group[0];
    if (!w->prover) w->prover.reset(new Prover(w->ctx.get(), job.params));
    else w->prover->set_params(job.params);
    Transcript ts;
    std::vector<int> ks{job.params.k};
    if (job.commit_only) {
      w->prover->commit(ts, job.poly, job.on_device, ks);
    } else {
      std::vector<std::vector<int>> groups(job.n_claims, std::vector<int>{0});
      w->prover->prove(ts, job.poly, job.on_device, ks, groups);
    }
    job.checkpoint = ts.draw_fe();
    job.proof = ts.bytes();
    return w->bytes();
  };
  // lock-step groups: jobs of one shape, at most lockstep_ of them, at most
  // 2^kGroupLog evaluations in all, and no more than the batched kernels take
  Grouping grouping;
  std::vector<int> group_cap(jobs.size(), 1);
  for (size_t j = 0; j < jobs.size(); j++) {
    const int by_size = jobs[j].params.k >= kGroupLog ? 1 : 1 << (kGroupLog - jobs[j].params.k);
    group_cap[j] = std::max(1, std::min({lockstep_, by_size, BatchProver::max_batch(jobs[j].params)}));
  }
  grouping.compatible = [&jobs](size_t h, size_t j) { return same_shape(jobs[h], jobs[j]); };
  grouping.max_group = [&group_cap](size_t h) { return group_cap[h]; };
  std::vector<void *> &states = states_;
  grouping.grow = [&jobs, &states](int worker, const std::vector<int> &group) -> size_t {
    const auto *w = static_cast<const GpuWorker *>(states[worker]);
    const Params &p = jobs[group[0]].params;
    if (group.size() == 1) {
      const size_t need = Prover::workspace_bytes(p), have = w && w->prover ? w->prover->device_bytes() : 0;
      return need > have ? need - have : 0;
    }
    const size_t need = BatchProver::workspace_bytes(p, (int)group.size());
    const size_t have = w && w->group_prover ? w->group_prover->device_bytes() : 0;
    return need > have ? need - have : 0;
  };
  // after a failed proof: what the worker's buffers hold now
  auto held_of = [](void *state) -> size_t { return static_cast<GpuWorker *>(state)->bytes(); };
  return run_jobs(jobs, states_, held_, budget_, honor_arrival, need, make, exec, nullptr,
                  lockstep_ > 1 ? &grouping : nullptr, held_of);
}

}  // namespace whir
