/*
 * CPU launcher for the reference's kernels compiled as host C++ (shim.h).
 *
 * Test infrastructure only.  Built into oracle/_ref/libpumpref_cpu_N<NUM>.so
 * together with the reference's own kernel sources; fake_cudart.cpp forwards
 * every `<<<grid, block>>>` launch of the reference's host code here by the
 * kernel's (demangled) name.  Blocks run in parallel on OpenMP threads, the
 * threads of one block run one after another, which is exact for these
 * kernels: none of them communicates between threads except the obstacle
 * copy into dynamic shared memory of cacheHalfspaces (hsmc.cu:17-23), which
 * the launcher performs before the block runs, with the same bound the
 * kernel uses (threadIdx.x < 12 * numObstacles).
 */
#include <cxxabi.h>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>

#include "2pBVP.cuh"
#include "collisionCheck.cuh"
#include "sampler.cuh"
#include "hsmc.cuh"
#include "PUMP.cuh"
#include "collisionProbability.cuh"

thread_local refcpu_idx3 threadIdx;
thread_local refcpu_idx3 blockIdx;
thread_local refcpu_idx3 blockDim;
thread_local refcpu_idx3 gridDim;
// dynamic shared memory of cacheHalfspaces / cacheHalfspacesEdge (hsmc.cu:17,110)
thread_local float s_obstacles[65536];

namespace {

template <class... A, size_t... I>
void call_impl(void (*f)(A...), void **args, std::index_sequence<I...>) {
  f(*reinterpret_cast<A *>(args[I])...);
}
template <class... A>
void call(void (*f)(A...), void **args) {
  call_impl(f, args, std::index_sequence_for<A...>{});
}

typedef void (*adapter_t)(void **);

struct Entry {
  const char *name;
  adapter_t fn;
  int obs_arg;   // index of the obstacle pointer for smem kernels, else -1
  int nobs_arg;  // index of the obstacle count
};

const Entry kTable[] = {
    {"fillCoptsTopts", [](void **a) { call(&fillCoptsTopts, a); }, -1, -1},
    {"sampleFree", [](void **a) { call(&sampleFree, a); }, -1, -1},
    {"freeEdges", [](void **a) { call(&freeEdges, a); }, -1, -1},
    {"setupAsBs", [](void **a) { call(&setupAsBs, a); }, -1, -1},
    {"cacheHalfspaces", [](void **a) { call(&cacheHalfspaces, a); }, 5, 3},
    {"cacheHalfspacesEdge", [](void **a) { call(&cacheHalfspacesEdge, a); }, 6, 4},
    {"setupValidParticles", [](void **a) { call(&setupValidParticles, a); }, -1, -1},
    {"propagateValidParticles", [](void **a) { call(&propagateValidParticles, a); }, -1, -1},
    {"propagateValidParticlesMany", [](void **a) { call(&propagateValidParticlesMany, a); }, -1, -1},
    {"calculateCP_HSMC", [](void **a) { call(&calculateCP_HSMC, a); }, -1, -1},
    {"MCCP", [](void **a) { call(&MCCP, a); }, -1, -1},
};

const Entry *lookup(const char *mangled) {
  std::string base;
  int status = 0;
  char *dem = abi::__cxa_demangle(mangled, nullptr, nullptr, &status);
  if (status == 0 && dem) {
    base = dem;
    std::free(dem);
    size_t p = base.find('(');
    if (p != std::string::npos) base.resize(p);
  } else {
    base = mangled;
  }
  for (const Entry &e : kTable)
    if (base == e.name) return &e;
  return nullptr;
}

}  // namespace

extern "C" int refcpu_launch(const char *mangled, unsigned gx, unsigned gy, unsigned gz,
                             unsigned bx, unsigned by, unsigned bz, void **args) {
  const Entry *e = lookup(mangled);
  if (!e) {
    std::fprintf(stderr, "refcpu_launch: no CPU entry for kernel %s\n", mangled);
    return 1;
  }
  const long long nblocks = (long long)gx * gy * gz;
#pragma omp parallel for schedule(dynamic, 16)
  for (long long b = 0; b < nblocks; ++b) {
    gridDim = {gx, gy, gz};
    blockDim = {bx, by, bz};
    blockIdx = {(unsigned)(b % gx), (unsigned)((b / gx) % gy), (unsigned)(b / ((long long)gx * gy))};
    if (e->obs_arg >= 0) {
      const float *obs = *reinterpret_cast<float **>(args[e->obs_arg]);
      const int nobs = *reinterpret_cast<int *>(args[e->nobs_arg]);
      const unsigned n = (unsigned)(12 * nobs) < bx ? (unsigned)(12 * nobs) : bx;
      for (unsigned i = 0; i < n; ++i) s_obstacles[i] = obs[i];
    }
    for (unsigned tz = 0; tz < bz; ++tz)
      for (unsigned ty = 0; ty < by; ++ty)
        for (unsigned tx = 0; tx < bx; ++tx) {
          threadIdx = {tx, ty, tz};
          e->fn(args);
        }
  }
  return 0;
}
