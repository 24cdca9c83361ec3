// Launch-shape autotuner.  A kernel with several launch shapes that compute
// the same results (block sizes, grid sizes) asks for its shape per
// (kernel, shape class) on the current device.  The first call of a shape
// class runs every candidate on the call's own inputs, on the call's stream,
// times each (the second of two runs, CUDA events), and records the fastest;
// later calls reuse the record.  The records are process-wide, guarded by a
// mutex; tuning can be switched off (pump_tune_enable, or PUMP_TUNE=0 in the
// environment), and then each kernel uses its default shape.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "pump.h"

namespace pump {

enum TuneKernel {
  kTuneBvpPairs = 0,   // bvp_pairs_precision_kernel block size
  kTuneDiscretize,     // discretize_kernel block size
  kTuneFreeEdges,      // free_edges_staged_kernel block size
  kTuneCompactRn,      // three-kernel compaction grid: rn superset pass
  kTuneCompactEdges,   // three-kernel compaction grid: edge lists
  kNumTune
};

// Shape class of a size: its power-of-two bucket.
inline uint64_t tune_bucket(long long n) {
  uint64_t b = 0;
  while (n > 1) {
    n >>= 1;
    ++b;
  }
  return b;
}

// Candidate index for `kernel` and shape class `key` (n candidates, index
// `fallback` when tuning is off).  Without a record, run(c) launches
// candidate c on `stream` (a complete launch of the computation, so running
// it again rewrites the same results); every candidate runs twice and the
// faster second run wins.  run(*choice) is NOT called again for the caller:
// after tuning, the results of the last candidate run are in place, and
// *ran is set so the caller does not launch once more.
pump_status_t tune_choice(int kernel, uint64_t key, int n, int fallback, cudaStream_t stream,
                          const std::function<pump_status_t(int)> &run, int *choice, bool *ran);

}  // namespace pump
