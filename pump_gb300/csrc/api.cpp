// Context, status reporting and the reference input-file reader.
#include <cuda_runtime.h>

#include <cstdarg>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"
#include "ctx.h"

namespace pump {

namespace {
thread_local char g_last_error[512] = "";
}

pump_status_t set_error(pump_status_t s, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
  va_end(ap);
  return s;
}

pump_status_t cuda_status(cudaError_t e, const char *where) {
  if (e == cudaSuccess) return PUMP_OK;
  if (e == cudaErrorMemoryAllocation)
    return set_error(PUMP_ERR_NO_MEMORY, "%s: %s", where, cudaGetErrorString(e));
  return set_error(PUMP_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

pump_status_t launch_status(const char *kernel) { return cuda_status(cudaGetLastError(), kernel); }

Ctx::~Ctx() {
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(device_);
  if (refine_graph.exec) cudaGraphExecDestroy(refine_graph.exec);
  for (const LoopGraph &g : loop_graphs) cudaGraphExecDestroy(g.exec);
  if (capture_stream) cudaStreamDestroy(capture_stream);
  if (loop_ready) cudaEventDestroy(loop_ready);
  for (int i = 0; i < kNumSlots; ++i)
    if (buf_[i]) cudaFree(buf_[i]);
  for (void *p : retired_) cudaFree(p);
  for (int i = 0; i < kNumPin; ++i)
    if (pin_[i]) cudaFreeHost(pin_[i]);
  for (void *p : retired_pinned_) cudaFreeHost(p);
  for (const ArenaChunk &c : arena_) cudaFree(c.p);
  if (arena_done_) cudaEventDestroy(arena_done_);
  if (prev >= 0) cudaSetDevice(prev);
}

pump_status_t Ctx::arena_begin(cudaStream_t s) {
  if (arena_pending_ && arena_stream_ != s) PUMP_CUDA_TRY(cudaStreamWaitEvent(s, arena_done_, 0));
  if (arena_.size() > 1) {
    // the last call needed several chunks: one chunk with room for all of
    // them replaces them (freed in order on s, after the last call's work)
    const size_t want = arena_total_ + arena_total_ / 4;
    for (const ArenaChunk &c : arena_) PUMP_CUDA_TRY(cudaFreeAsync(c.p, s));
    arena_.clear();
    char *p = nullptr;
    PUMP_CUDA_TRY(pool_malloc_async((void **)&p, want, s));
    arena_.push_back({p, want});
  }
  arena_used_ = 0;
  arena_total_ = 0;
  arena_stream_ = s;
  return PUMP_OK;
}

pump_status_t Ctx::arena_take(size_t bytes, void **out) {
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes == 0) bytes = 256;
  if (arena_.empty() || arena_used_ + bytes > arena_.back().cap) {
    size_t cap = arena_.empty() ? (size_t)64 << 20 : arena_.back().cap * 2;
    if (cap < bytes) cap = bytes;
    char *p = nullptr;
    PUMP_CUDA_TRY(pool_malloc_async((void **)&p, cap, arena_stream_));
    arena_.push_back({p, cap});
    arena_used_ = 0;
  }
  *out = arena_.back().p + arena_used_;
  arena_used_ += bytes;
  arena_total_ += bytes;
  return PUMP_OK;
}

void Ctx::arena_end(cudaStream_t s) {
  if (!arena_done_ && cudaEventCreateWithFlags(&arena_done_, cudaEventDisableTiming) != cudaSuccess) {
    arena_done_ = nullptr;
    cudaStreamSynchronize(s);  // no event: the call's work is complete instead
    arena_pending_ = false;
    return;
  }
  arena_pending_ = cudaEventRecord(arena_done_, s) == cudaSuccess;
  if (!arena_pending_) cudaStreamSynchronize(s);
}

pump_status_t Ctx::pinned(int slot, size_t bytes, void **out) {
  if (slot < 0 || slot >= kNumPin) return set_error(PUMP_ERR_BAD_INPUT, "pinned slot %d", slot);
  if (bytes == 0) bytes = 1;
  if (pin_cap_[slot] < bytes) {
    if (pin_[slot]) {
      retired_pinned_.push_back(pin_[slot]);
      pin_[slot] = nullptr;
      pin_cap_[slot] = 0;
    }
    const size_t cap = bytes + bytes / 2 + 4096;
    PUMP_CUDA_TRY(cudaMallocHost(&pin_[slot], cap));
    pin_cap_[slot] = cap;
  }
  *out = pin_[slot];
  return PUMP_OK;
}

namespace {
// Particle tables shared by every context of the process, per device and
// (seed, P, T): generated once on the first requester's stream; an event
// lets requesters on other streams wait for the generation.  Kept until the
// process exits (9.8 MB for the default 2048 particles x 400 steps).
struct TableEntry {
  int device;
  uint64_t seed;
  int P, T;
  float *ptr;
  cudaEvent_t ready;
};
std::mutex g_table_mutex;
std::vector<TableEntry> g_tables;
}  // namespace

pump_status_t Ctx::particle_table(uint64_t seed, int P, int T, const float **out,
                                  cudaStream_t stream) {
  std::lock_guard<std::mutex> lock(g_table_mutex);
  for (const TableEntry &e : g_tables)
    if (e.device == device_ && e.seed == seed && e.P == P && e.T == T) {
      PUMP_CUDA_TRY(cudaStreamWaitEvent(stream, e.ready, 0));
      *out = e.ptr;
      return PUMP_OK;
    }
  TableEntry e{device_, seed, P, T, nullptr, nullptr};
  PUMP_CUDA_TRY(cudaMalloc(&e.ptr, sizeof(float) * 3 * ((size_t)P * T + T)));
  PUMP_TRY(particle_tables_async(seed, P, T, e.ptr, nullptr, stream));
  PUMP_TRY(particle_rowmax_async(e.ptr, P, T, e.ptr + 3 * (size_t)P * T, stream));
  PUMP_CUDA_TRY(cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming));
  PUMP_CUDA_TRY(cudaEventRecord(e.ready, stream));
  g_tables.push_back(e);
  *out = e.ptr;
  return PUMP_OK;
}

cudaError_t pool_malloc_async(void **p, size_t bytes, cudaStream_t stream) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, stream);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      e = cudaMemPoolCreate(&pools[dev], &props);
      if (e != cudaSuccess) {
        pools[dev] = nullptr;
        return e;
      }
      unsigned long long keep = ~0ull;
      e = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
      if (e != cudaSuccess) return e;
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}

pump_status_t smem_attr(const void *fn, size_t bytes) {
  // the default limit (48 KB) covers a kernel's static and dynamic shared
  // memory together, so the kernel's static size is read once per function
  struct Entry {
    int dev;
    const void *fn;
    size_t static_bytes, dyn_max;  // dyn_max: dynamic size allowed so far
  };
  static std::mutex mu;
  static std::vector<Entry> set;
  constexpr size_t kDefault = 48 * 1024;
  int dev = 0;
  PUMP_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  Entry *e = nullptr;
  for (auto &x : set)
    if (x.dev == dev && x.fn == fn) e = &x;
  if (!e) {
    cudaFuncAttributes fa{};
    PUMP_CUDA_TRY(cudaFuncGetAttributes(&fa, fn));
    const size_t st = fa.sharedSizeBytes;
    set.push_back({dev, fn, st, st < kDefault ? kDefault - st : 0});
    e = &set.back();
  }
  if (bytes <= e->dyn_max) return PUMP_OK;
  PUMP_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  e->dyn_max = bytes;
  return PUMP_OK;
}

pump_status_t Ctx::activate() { return cuda_status(cudaSetDevice(device_), "cudaSetDevice"); }

pump_status_t Ctx::scratch(int slot, size_t bytes, void **out) {
  if (slot < 0 || slot >= kNumSlots) return set_error(PUMP_ERR_BAD_INPUT, "scratch slot %d", slot);
  if (bytes == 0) bytes = 1;
  if (cap_[slot] < bytes) {
    if (buf_[slot]) {
      // queued work may still use it: freed with the context
      retired_.push_back(buf_[slot]);
      buf_[slot] = nullptr;
      cap_[slot] = 0;
    }
    size_t cap = bytes + bytes / 2;
    PUMP_CUDA_TRY(cudaMalloc(&buf_[slot], cap));
    cap_[slot] = cap;
  }
  *out = buf_[slot];
  return PUMP_OK;
}

}  // namespace pump

using namespace pump;

extern "C" const char *pump_status_string(pump_status_t s) {
  switch (s) {
    case PUMP_OK: return "ok";
    case PUMP_ERR_BAD_INPUT: return "bad input";
    case PUMP_ERR_CAPACITY: return "capacity exceeded";
    case PUMP_ERR_TIMEOUT: return "bounded wait gave up";
    case PUMP_ERR_CUDA: return "CUDA error";
    case PUMP_ERR_NO_SOLUTION: return "no solution";
    case PUMP_ERR_NO_MEMORY: return "out of device memory";
  }
  return "unknown status";
}

extern "C" const char *pump_last_error(void) { return g_last_error; }

extern "C" const char *pump_version(void) { return "pump_gb300 0.1 (sm_103a)"; }

extern "C" pump_status_t pump_ctx_create(int device, pump_ctx **out) {
  if (!out) return set_error(PUMP_ERR_BAD_INPUT, "pump_ctx_create: null out");
  int n = 0;
  PUMP_CUDA_TRY(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_ctx_create: device %d of %d", device, n);
  Ctx *c = new (std::nothrow) Ctx(device);
  if (!c) return set_error(PUMP_ERR_NO_MEMORY, "pump_ctx_create: host allocation");
  *out = c->handle();
  return c->activate();
}

extern "C" pump_status_t pump_ctx_destroy(pump_ctx *ctx) {
  delete Ctx::from(ctx);
  return PUMP_OK;
}

// Defaults of mainPUMP.cu:51-72 and obstacles.cu:3-10.
extern "C" void pump_problem_defaults(pump_problem *pb) {
  static const float kObs[36] = {
      0.05f, 0.20f, -3.1f, -3.1f, -3.1f, -3.1f, 0.45f, 0.35f, 3.1f, 3.1f, 3.1f, 3.1f,
      0.70f, 0.30f, -3.1f, -3.1f, -3.1f, -3.1f, 0.90f, 0.50f, 3.1f, 3.1f, 3.1f, 3.1f,
      0.30f, 0.60f, -3.1f, -3.1f, -3.1f, -3.1f, 0.80f, 0.75f, 3.1f, 3.1f, 3.1f, 3.1f};
  static const float kLo[6] = {0, 0, 0.01f, -1, -1, -0.5f};
  static const float kHi[6] = {1, 1, 0.3f, 1, 1, 0.5f};
  std::memset(pb, 0, sizeof *pb);
  pb->N = 1000;
  pb->num_disc = 8;
  pb->num_hsmc = 128;
  pb->num_mc = 2048;
  pb->table_rows = 400;
  pb->num_obstacles = 3;
  pb->obstacles = kObs;
  for (int d = 0; d < 6; ++d) {
    pb->init[d] = d < 3 ? 0.1f : 0.0f;
    pb->goal[d] = d < 3 ? 0.9f : 0.0f;
    pb->lo[d] = kLo[d];
    pb->hi[d] = kHi[d];
  }
  pb->offset_mult = 0.5f;
  pb->cp_target = 0.01f;
  pb->cp_factor = 2.0f;
  pb->seed = 0x9E3779B97F4A7C15ull;
  pb->bvp_mode = PUMP_BVP_PARITY;
  pb->refine_iters = 0;
  pb->refine_lambda = 10.0f;
  pb->samples = nullptr;
  pb->max_paths = 0;
  pb->disc_len = 0.0f;
  pb->disc_min = 3;
}

namespace {
thread_local std::vector<float> g_input_obstacles;
}

// Same field order and conversions as mainPUMP.cu:152-230: comma-separated
// fields read with getline(',') and converted with stringstream >>.
extern "C" pump_status_t pump_read_input(const char *path, pump_problem *pb) {
  if (!path || !pb) return set_error(PUMP_ERR_BAD_INPUT, "pump_read_input: null argument");
  std::ifstream file(path);
  if (!file.good()) return set_error(PUMP_ERR_BAD_INPUT, "pump_read_input: cannot read %s", path);
  std::string v;
  auto rd = [&](float &out) {
    std::getline(file, v, ',');
    std::stringstream ss(v);
    ss >> out;
  };
  for (int d = 0; d < 6; ++d) rd(pb->init[d]);
  for (int d = 0; d < 6; ++d) rd(pb->goal[d]);
  for (int d = 0; d < 6; ++d) rd(pb->lo[d]);
  for (int d = 0; d < 6; ++d) rd(pb->hi[d]);
  rd(pb->offset_mult);
  {
    std::getline(file, v, ',');
    std::stringstream ss(v);
    int n = 0;
    ss >> n;
    if (n < 0 || n > 1000000) return set_error(PUMP_ERR_BAD_INPUT, "pump_read_input: %d obstacles", n);
    pb->num_obstacles = n;
  }
  g_input_obstacles.assign((size_t)pb->num_obstacles * 12, 0.0f);
  for (size_t i = 0; i < g_input_obstacles.size(); ++i) rd(g_input_obstacles[i]);
  pb->obstacles = g_input_obstacles.data();
  return PUMP_OK;
}
