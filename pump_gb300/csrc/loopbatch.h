// Grouped search loops of a planning batch: the batch workers' queries reach
// their search loops at different times; a worker whose query is ready joins
// the group being formed, and one of them launches the loop graph
// (search_loop_graph) once for the whole group.  The graph's kernels then
// serve every query of the group in each iteration (HSMC's blocks take the
// chunks of all the queries' wavefronts), and its while node repeats the
// iteration until every query's loop has ended, so a group costs the launches
// and host waits of one query.
#pragma once

#include <chrono>
#include <condition_variable>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "search.h"

namespace pump {

// Shape class of a loop graph: its kernels' template parameters and shared
// memory follow these (a group takes its queries' largest; obs_cap is the
// box count rounded up to 32).
struct LoopShape {
  int lazy, mode, obs_cap, num_disc, max_hs, particles;
};

class LoopBatcher {
 public:
  // members: the worker threads that may call run(); max_group: queries per
  // launch (at most kLoopGroupMax); window_us: how long the first waiting
  // query waits for others before its group is launched; slots: groups that
  // may run at once.
  LoopBatcher(int device, int members, int max_group, int window_us, int slots);
  ~LoopBatcher();
  LoopBatcher(const LoopBatcher &) = delete;
  LoopBatcher &operator=(const LoopBatcher &) = delete;
  // PUMP_OK, or the error of setting up the slots (run() then returns it)
  pump_status_t status() const { return init_; }

  // Runs the loop of the query whose argument block is at d_args (device),
  // written on the caller's stream before `ready` was recorded there.
  // Returns once the group's graph has finished (the query's loop state is
  // then in d_args->L); an error of the launch is the whole group's.
  pump_status_t run(LoopArgs *d_args, const LoopShape &shape, cudaEvent_t ready);
  // The calling member has no more queries: groups no longer wait for it.
  void leave();

  struct Slot;  // a group in flight: device table, staging, stream, graphs

 private:
  struct Member {
    LoopArgs *args;
    LoopShape shape;
    cudaEvent_t ready;
    std::chrono::steady_clock::time_point arrived;
    bool taken = false, done = false;
    pump_status_t status = PUMP_OK;
  };
  pump_status_t launch(Slot *slot, const std::vector<Member *> &group);

  int device_, max_group_, alive_, running_ = 0;
  pump_status_t init_ = PUMP_OK;
  std::chrono::microseconds window_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::vector<Member *> pending_;  // in arrival order
  std::vector<Slot *> slots_, free_;
};

}  // namespace pump
