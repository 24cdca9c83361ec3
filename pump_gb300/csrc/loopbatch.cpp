// Grouped search loops of a planning batch (loopbatch.h).
#include "loopbatch.h"

#include <algorithm>
#include <cstring>

#include "common.cuh"

namespace pump {

struct LoopBatcher::Slot {
  int device = 0;
  LoopGroup *d_group = nullptr;  // the table the slot's graphs read
  LoopGroup *h_group = nullptr;  // pinned staging of the table
  cudaStream_t stream = nullptr, capture = nullptr;
  struct Graph {
    LoopShape shape;
    int gcap;
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;  // instantiated per (shape class, group capacity)
  bool healthy = true;
};

namespace {

using clk = std::chrono::steady_clock;

// Slots (and their instantiated graphs) are kept across batches, as the
// batch workers' contexts are.
std::mutex g_slot_mu;
std::vector<LoopBatcher::Slot *> g_idle_slots;

void slot_destroy(LoopBatcher::Slot *s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (const auto &g : s->graphs) cudaGraphExecDestroy(g.exec);
  if (s->d_group) cudaFree(s->d_group);
  if (s->h_group) cudaFreeHost(s->h_group);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->capture) cudaStreamDestroy(s->capture);
  cudaGetLastError();
  delete s;
}

pump_status_t slot_take(int device, LoopBatcher::Slot **out) {
  *out = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_slot_mu);
    for (size_t i = 0; i < g_idle_slots.size(); ++i)
      if (g_idle_slots[i]->device == device) {
        *out = g_idle_slots[i];
        g_idle_slots.erase(g_idle_slots.begin() + (long)i);
        return PUMP_OK;
      }
  }
  auto *s = new LoopBatcher::Slot();
  s->device = device;
  pump_status_t st = cuda_status(cudaMalloc(&s->d_group, sizeof(LoopGroup)), "cudaMalloc");
  if (st == PUMP_OK)
    st = cuda_status(cudaMallocHost(&s->h_group, sizeof(LoopGroup)), "cudaMallocHost");
  if (st == PUMP_OK)
    st = cuda_status(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking),
                     "cudaStreamCreateWithFlags");
  if (st == PUMP_OK)
    st = cuda_status(cudaStreamCreateWithFlags(&s->capture, cudaStreamNonBlocking),
                     "cudaStreamCreateWithFlags");
  if (st != PUMP_OK) {
    slot_destroy(s);
    return st;
  }
  *out = s;
  return PUMP_OK;
}

void slot_give(LoopBatcher::Slot *s) {
  if (!s->healthy || cudaStreamQuery(s->stream) != cudaSuccess) {
    slot_destroy(s);
    return;
  }
  std::lock_guard<std::mutex> lk(g_slot_mu);
  g_idle_slots.push_back(s);
}

bool same_shape(const LoopShape &a, const LoopShape &b) {
  return a.lazy == b.lazy && a.mode == b.mode && a.obs_cap == b.obs_cap &&
         a.num_disc == b.num_disc && a.max_hs == b.max_hs && a.particles == b.particles;
}

}  // namespace

LoopBatcher::LoopBatcher(int device, int members, int max_group, int window_us, int slots)
    : device_(device),
      max_group_(std::max(1, std::min(max_group, kLoopGroupMax))),
      alive_(members),
      window_(std::max(0, window_us)) {
  for (int k = 0; k < std::max(1, slots) && init_ == PUMP_OK; ++k) {
    Slot *s = nullptr;
    init_ = slot_take(device, &s);
    if (s) {
      slots_.push_back(s);
      free_.push_back(s);
    }
  }
}

LoopBatcher::~LoopBatcher() {
  for (Slot *s : slots_) slot_give(s);
}

void LoopBatcher::leave() {
  std::lock_guard<std::mutex> lk(mu_);
  --alive_;
  cv_.notify_all();
}

pump_status_t LoopBatcher::run(LoopArgs *d_args, const LoopShape &shape, cudaEvent_t ready) {
  if (init_ != PUMP_OK) return init_;
  Member me{d_args, shape, ready, clk::now()};
  std::unique_lock<std::mutex> lk(mu_);
  pending_.push_back(&me);
  cv_.notify_all();
  while (!me.done) {
    if (me.taken) {  // the group's leader reports its end
      cv_.wait(lk);
      continue;
    }
    // launch now when the group is full, when every member still planning
    // is waiting here or running a group (no other query can come), or when
    // the longest-waiting query has waited its window
    const auto due = pending_.front()->arrived + window_;
    const bool full = (int)pending_.size() >= max_group_;
    const bool all_here = (int)pending_.size() + running_ >= alive_;
    if (!free_.empty() && (full || all_here || clk::now() >= due)) {
      std::vector<Member *> group{&me};
      for (Member *m : pending_)
        if (m != &me && (int)group.size() < max_group_ && m->shape.lazy == shape.lazy &&
            m->shape.mode == shape.mode)
          group.push_back(m);
      for (Member *m : group) m->taken = true;
      pending_.erase(std::remove_if(pending_.begin(), pending_.end(),
                                    [](const Member *m) { return m->taken; }),
                     pending_.end());
      Slot *slot = free_.back();
      free_.pop_back();
      running_ += (int)group.size();
      lk.unlock();
      const pump_status_t st = launch(slot, group);
      lk.lock();
      if (st != PUMP_OK) slot->healthy = false;
      running_ -= (int)group.size();
      free_.push_back(slot);
      for (Member *m : group) {
        m->status = st;
        m->done = true;
      }
      cv_.notify_all();
      continue;
    }
    if (free_.empty()) cv_.wait(lk);
    else cv_.wait_until(lk, due);
  }
  return me.status;
}

pump_status_t LoopBatcher::launch(Slot *sl, const std::vector<Member *> &group) {
  LoopShape sh = group[0]->shape;
  for (const Member *m : group) {
    sh.obs_cap = std::max(sh.obs_cap, m->shape.obs_cap);
    sh.num_disc = std::max(sh.num_disc, m->shape.num_disc);
    sh.max_hs = std::max(sh.max_hs, m->shape.max_hs);
    sh.particles = std::max(sh.particles, m->shape.particles);
  }
  int gcap = 1;
  while (gcap < (int)group.size()) gcap <<= 1;
  cudaGraphExec_t exec = nullptr;
  for (const Slot::Graph &g : sl->graphs)
    if (g.gcap == gcap && same_shape(g.shape, sh)) exec = g.exec;
  if (!exec) {
    PUMP_TRY(search_loop_graph(sl->d_group, gcap, sh.lazy != 0, sh.mode, sh.obs_cap, sh.num_disc,
                               sh.max_hs, sh.particles, sl->capture, &exec));
    sl->graphs.push_back({sh, gcap, exec});
  }
  LoopGroup *hg = sl->h_group;
  std::memset(hg, 0, sizeof *hg);
  hg->nq = (int)group.size();
  for (size_t i = 0; i < group.size(); ++i) hg->args[i] = group[i]->args;
  PUMP_CUDA_TRY(cudaMemcpyAsync(sl->d_group, hg, sizeof(LoopGroup), cudaMemcpyHostToDevice,
                                sl->stream));
  for (const Member *m : group) PUMP_CUDA_TRY(cudaStreamWaitEvent(sl->stream, m->ready, 0));
  PUMP_CUDA_TRY(cudaGraphLaunch(exec, sl->stream));
  return cuda_status(cudaStreamSynchronize(sl->stream), "grouped search loop");
}

}  // namespace pump
