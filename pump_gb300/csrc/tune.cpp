// Launch-shape autotuner (tune.h) and its C ABI.
#include "tune.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "common.cuh"

namespace pump {
namespace {

const char *const kTuneNames[kNumTune] = {"bvp_pairs_precision", "discretize", "free_edges",
                                           "compact_rn", "compact_edges"};

struct Record {
  int choice;
  float ms[8];
  int n;
};

std::mutex g_tune_mutex;
std::map<std::tuple<int, int, uint64_t>, Record> g_records;  // (device, kernel, key)

std::atomic<int> &tune_flag() {
  static std::atomic<int> flag([] {
    const char *e = std::getenv("PUMP_TUNE");
    return (e && e[0] == '0') ? 0 : 1;
  }());
  return flag;
}

}  // namespace

pump_status_t tune_choice(int kernel, uint64_t key, int n, int fallback, cudaStream_t stream,
                          const std::function<pump_status_t(int)> &run, int *choice, bool *ran) {
  *ran = false;
  *choice = fallback;
  if (n <= 1 || !tune_flag().load()) return PUMP_OK;
  int dev = 0;
  PUMP_CUDA_TRY(cudaGetDevice(&dev));
  const auto k = std::make_tuple(dev, kernel, key);
  {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_records.find(k);
    if (it != g_records.end()) {
      *choice = it->second.choice;
      return PUMP_OK;
    }
  }
  if (n > 8) n = 8;
  cudaEvent_t ev[2 * 8 + 1];
  for (int i = 0; i < 2 * n + 1; ++i) PUMP_CUDA_TRY(cudaEventCreate(&ev[i]));
  pump_status_t st = PUMP_OK;
  // candidate c: a warm-up run, then the timed run between ev[2c+1] and ev[2c+2]
  PUMP_CUDA_TRY(cudaEventRecord(ev[0], stream));
  for (int c = 0; c < n && st == PUMP_OK; ++c) {
    st = run(c);
    if (st == PUMP_OK) st = cuda_status(cudaEventRecord(ev[2 * c + 1], stream), "cudaEventRecord");
    if (st == PUMP_OK) st = run(c);
    if (st == PUMP_OK) st = cuda_status(cudaEventRecord(ev[2 * c + 2], stream), "cudaEventRecord");
  }
  Record rec{};
  rec.n = n;
  if (st == PUMP_OK) st = cuda_status(cudaEventSynchronize(ev[2 * n]), "cudaEventSynchronize");
  if (st == PUMP_OK) {
    float best = 0;
    for (int c = 0; c < n; ++c) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[2 * c + 1], ev[2 * c + 2]);
      rec.ms[c] = ms;
      if (c == 0 || ms < best) {
        best = ms;
        rec.choice = c;
      }
    }
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_records.emplace(k, rec);  // a concurrent tuner of the same class keeps its own
    *choice = rec.choice;
    *ran = true;
  }
  for (int i = 0; i < 2 * n + 1; ++i) cudaEventDestroy(ev[i]);
  // the results in place are the last candidate's (all candidates compute the same)
  return st;
}

}  // namespace pump

using namespace pump;

extern "C" void pump_tune_enable(int on) { tune_flag().store(on ? 1 : 0); }

extern "C" void pump_tune_reset(void) {
  std::lock_guard<std::mutex> lk(g_tune_mutex);
  g_records.clear();
}

extern "C" int pump_tune_report(char *buf, size_t len) {
  std::string out;
  {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    for (const auto &kv : g_records) {
      char line[256];
      int w = std::snprintf(line, sizeof line, "device %d %s class %llu: candidate %d of %d (ms",
                            std::get<0>(kv.first), kTuneNames[std::get<1>(kv.first)],
                            (unsigned long long)std::get<2>(kv.first), kv.second.choice,
                            kv.second.n);
      for (int c = 0; c < kv.second.n && w > 0 && w < (int)sizeof line; ++c)
        w += std::snprintf(line + w, sizeof line - w, " %.4f", kv.second.ms[c]);
      out += line;
      out += ")\n";
    }
  }
  if (buf && len > 0) {
    const size_t m = out.size() < len - 1 ? out.size() : len - 1;
    std::memcpy(buf, out.data(), m);
    buf[m] = '\0';
  }
  return (int)out.size();
}
