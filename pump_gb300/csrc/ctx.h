// Library context: the device it runs on and grow-only scratch buffers that
// are reused across calls (allocation happens only when a call needs more
// than any earlier call on the same context did).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "pump.h"

namespace pump {

class Ctx {
 public:
  enum Slot {
    kSelect = 0,   // radix-select state + histogram
    kCompact,      // compaction tile status words
    kPlanA,        // planner buffers (see plan.cpp)
    kNumSlots
  };
  explicit Ctx(int device) : device_(device) {
    for (int i = 0; i < kNumSlots; ++i) { buf_[i] = nullptr; cap_[i] = 0; }
  }
  ~Ctx();
  static Ctx *from(pump_ctx *c) { return reinterpret_cast<Ctx *>(c); }
  pump_ctx *handle() { return reinterpret_cast<pump_ctx *>(this); }
  int device() const { return device_; }
  pump_status_t activate();
  // Device buffer of at least `bytes` for `slot` (contents undefined).
  pump_status_t scratch(int slot, size_t bytes, void **out);

 private:
  int device_;
  void *buf_[kNumSlots];
  size_t cap_[kNumSlots];
};

// Internal device-side entry points shared between translation units.
pump_status_t select_kth_device(Ctx *ctx, const float *d_v, long long n, long long k,
                                const float **d_result, cudaStream_t stream);
pump_status_t build_edges_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N,
                                 float rn, long long max_edges, int *d_src, int *d_dst,
                                 float *d_copt, float *d_topt, int *d_go_start,
                                 long long *h_num_edges, cudaStream_t stream);
pump_status_t frontier_compact_device(Ctx *ctx, const uint8_t *d_flags, int N, int *d_active,
                                      int *d_count, int **d_error_out, cudaStream_t stream);
pump_status_t bvp_path_states(const float *d_xs, const int *d_seg, const float *d_tsample,
                              const float *d_tau, int total, float *d_out, cudaStream_t stream);

}  // namespace pump
