/*
 * A CPU stand-in for the CUDA runtime, linked under the reference's own host
 * code (mainPUMP.cu, PUMP.cu, collisionProbability.cu ... compiled by nvcc's
 * host pass) so the unmodified reference program runs on a machine without a
 * GPU and serves as the parity oracle.
 *
 *  - device memory is host memory (cudaMalloc = malloc, cudaMemcpy = memcpy);
 *  - every kernel launch is forwarded by name to refcpu_launch() in the CPU
 *    kernel library (launcher.cpp), which runs the reference's own kernel
 *    bodies compiled as host C++;
 *  - with PUMPREF_DUMP=<dir>, the outputs of each launch are appended to
 *    binary files in <dir> (the golden-vector dump);
 *  - with PUMPREF_BVP_FROM=<dir>, the fillCoptsTopts launch reads its outputs
 *    from <dir>/copts.f32 and <dir>/topts.f32 instead of computing them: the
 *    pair times and costs of the reference's own kernel run on a GPU, so the
 *    rest of the program runs on what the reference's GPU computed there.
 *
 * Particle table extension: the reference reads the time-major particle
 * table at row time/dt without a bound (PUMP.cu:637-647), i.e. past its
 * 100-row allocation for paths longer than 5 s.  That read is undefined in
 * the reference; this oracle (and the library) define it as the next rows of
 * the same particle stream: the allocation that receives xcombTime gets
 * PUMPREF_TABLE_ROWS rows (default 400) of the extended stream.
 *
 * Test infrastructure only.
 */
#include <cuda_runtime_api.h>
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "../pump_oracle.h"

extern float xcomb[];
extern float xcombTime[];
extern "C" const float *refsupport_table_tmajor(int *rows, int *particles);

namespace {

// function-local statics: the reference's registration constructors run
// before this file's namespace-scope objects would be initialised
std::map<const void *, std::string> &names() {
  static std::map<const void *, std::string> m;
  return m;
}
struct Config { dim3 g, b; size_t shmem; void *stream; };
Config g_cfg;
typedef int (*launch_fn)(const char *, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, void **);
launch_fn g_launch = nullptr;
int g_iter = 0;

launch_fn launcher() {
  if (!g_launch) {
    const char *lib = std::getenv("PUMPREF_KERNEL_LIB");
    if (!lib) { std::fprintf(stderr, "PUMPREF_KERNEL_LIB not set\n"); std::exit(3); }
    void *h = dlopen(lib, RTLD_NOW | RTLD_LOCAL);
    if (!h) { std::fprintf(stderr, "dlopen %s: %s\n", lib, dlerror()); std::exit(3); }
    g_launch = (launch_fn)dlsym(h, "refcpu_launch");
    if (!g_launch) { std::fprintf(stderr, "refcpu_launch missing\n"); std::exit(3); }
  }
  return g_launch;
}

void dump(const char *name, const void *p, size_t bytes, bool append) {
  const char *dir = std::getenv("PUMPREF_DUMP");
  if (!dir) return;
  std::string path = std::string(dir) + "/" + name;
  FILE *f = std::fopen(path.c_str(), append ? "ab" : "wb");
  if (!f) return;
  std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}
template <class T> T arg(void **a, int i) { return *reinterpret_cast<T *>(a[i]); }

void dump_after(const std::string &name, void **a) {
  if (!std::getenv("PUMPREF_DUMP")) return;
  if (name.rfind("fillCoptsTopts", 0) == 0) {
    const size_t n = (size_t)NUM * (NUM - 1);
    dump("samples.f32", arg<float *>(a, 0), sizeof(float) * NUM * DIM, false);
    dump("copts.f32", arg<float *>(a, 1), sizeof(float) * n, false);
    dump("topts.f32", arg<float *>(a, 2), sizeof(float) * n, false);
  } else if (name.rfind("sampleFree", 0) == 0) {
    dump("isFreeSamples.u8", arg<bool *>(a, 3), NUM, false);
  } else if (name.rfind("freeEdges", 0) == 0) {
    const int numDisc = arg<int>(a, 4), numEdges = arg<int>(a, 7);
    dump("discMotions.f32", arg<float *>(a, 5), sizeof(float) * (size_t)numEdges * (numDisc + 1) * DIM, false);
    dump("isFreeEdges.u8", arg<bool *>(a, 6), (size_t)numEdges, false);
  } else if (name.rfind("cacheHalfspaces", 0) == 0) {
    const int numEdges = arg<int>(a, 0), maxHS = arg<int>(a, 4), W = arg<int>(a, 6);
    const size_t nhs = (size_t)numEdges * W * maxHS;
    dump("as.f32", arg<float *>(a, 7), sizeof(float) * nhs * 3, false);
    dump("bs.f32", arg<float *>(a, 8), sizeof(float) * nhs, false);
    dump("countHS.i32", arg<int *>(a, 9), sizeof(int) * (size_t)numEdges * W, false);
  } else if (name.rfind("propagateValidParticles", 0) == 0) {
    const int numNew = arg<int>(a, 0), base = arg<int>(a, 4);
    const int P = arg<int>(a, 16);
    int hdr[3] = {g_iter, numNew, base};
    dump("wavefront.i32", hdr, sizeof hdr, true);
    dump("wavefront.i32", arg<int *>(a, 3), sizeof(int) * numNew, true);  // path prev
    dump("wavefront.i32", arg<int *>(a, 2), sizeof(int) * numNew, true);  // edge
    dump("valid.u8", arg<bool *>(a, 15) + (size_t)base * P, (size_t)numNew * P, true);
    ++g_iter;
  } else if (name.rfind("calculateCP_HSMC", 0) == 0) {
    const int numNew = arg<int>(a, 0), base = arg<int>(a, 1);
    dump("pathcp.f32", arg<float *>(a, 2) + base, sizeof(float) * numNew, true);
  } else if (name.rfind("MCCP", 0) == 0) {
    const int T = arg<int>(a, 6);
    int hdr[1] = {T};
    dump("mccp_paths.f32", hdr, sizeof hdr, true);
    dump("mccp_paths.f32", arg<float *>(a, 1), sizeof(float) * (size_t)(T > 0 ? T : 0) * DIM, true);
    dump("mccp_hits.i32", arg<int *>(a, 0), sizeof(int) * 2048, true);
  }
}

}  // namespace

extern "C" {

void **__cudaRegisterFatBinary(void *) {
  static void *handle = nullptr;
  return &handle;
}
void __cudaRegisterFatBinaryEnd(void **) {}
void __cudaUnregisterFatBinary(void **) {}
char __cudaInitModule(void **) { return 1; }
void __cudaRegisterFunction(void **, const char *hostFun, char *, const char *deviceName, int,
                            uint3 *, uint3 *, dim3 *, dim3 *, int *) {
  names()[(const void *)hostFun] = deviceName;
}
void __cudaRegisterVar(void **, char *, char *, const char *, int, size_t, int, int) {}
void __cudaRegisterManagedVar(void **, void **, char *, const char *, int, size_t, int, int) {}

unsigned __cudaPushCallConfiguration(dim3 g, dim3 b, size_t shmem, struct CUstream_st *s) {
  g_cfg = Config{g, b, shmem, (void *)s};
  return 0;
}
cudaError_t __cudaPopCallConfiguration(dim3 *g, dim3 *b, size_t *shmem, void *stream) {
  *g = g_cfg.g;
  *b = g_cfg.b;
  *shmem = g_cfg.shmem;
  *(void **)stream = g_cfg.stream;
  return cudaSuccess;
}
cudaError_t __cudaGetKernel(cudaKernel_t *k, const void *hostFun) {
  *k = (cudaKernel_t)hostFun;
  return cudaSuccess;
}
// Reads n floats from dir/name into p; exits on a missing or short file.
void read_floats(const char *dir, const char *name, float *p, size_t n) {
  const std::string path = std::string(dir) + "/" + name;
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(p, sizeof(float), n, f) != n) {
    std::fprintf(stderr, "PUMPREF_BVP_FROM: cannot read %zu floats from %s\n", n, path.c_str());
    std::exit(3);
  }
  std::fclose(f);
}

cudaError_t __cudaLaunchKernel(cudaKernel_t k, dim3 g, dim3 b, void **args, size_t, cudaStream_t) {
  auto it = names().find((const void *)k);
  if (it == names().end()) return cudaErrorInvalidDeviceFunction;
  // identifier of the Itanium-mangled name "_Z<len><identifier>..."
  std::string nm = it->second;
  if (nm.rfind("_Z", 0) == 0) {
    size_t i = 2, len = 0;
    while (i < nm.size() && nm[i] >= '0' && nm[i] <= '9') len = len * 10 + (nm[i++] - '0');
    nm = nm.substr(i, len);
  }
  const char *bvp_from = std::getenv("PUMPREF_BVP_FROM");
  if (bvp_from && nm == "fillCoptsTopts") {
    const size_t n = (size_t)NUM * (NUM - 1);
    read_floats(bvp_from, "copts.f32", arg<float *>(args, 1), n);
    read_floats(bvp_from, "topts.f32", arg<float *>(args, 2), n);
  } else if (launcher()(it->second.c_str(), g.x, g.y, g.z, b.x, b.y, b.z, args)) {
    return cudaErrorLaunchFailure;
  }
  dump_after(nm, args);
  return cudaSuccess;
}

cudaError_t cudaMalloc(void **p, size_t n) {
  size_t extra = 64;
  // the particle tables (Tmax x numMCParticles x 3 floats, hardCoded.cuh)
  if (n == sizeof(float) * 100 * 2048 * 3) {
    int rows = 0, parts = 0;
    refsupport_table_tmajor(&rows, &parts);
    if (rows > 100) extra = sizeof(float) * (size_t)(rows - 100) * parts * 3 + 64;
  }
  void *q = std::malloc(n + extra);
  if (!q) return cudaErrorMemoryAllocation;
  std::memset(q, 0xFF, n + extra);  // never-written device memory reads as NaN / -1
  *p = q;
  return cudaSuccess;
}
cudaError_t cudaFree(void *p) {
  std::free(p);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind) {
  std::memmove(dst, src, n);
  if (src == (const void *)xcombTime) {
    int rows = 0, parts = 0;
    const float *ext = refsupport_table_tmajor(&rows, &parts);
    if (rows > 100)
      std::memcpy((char *)dst + n, ext + (size_t)100 * parts * 3,
                  sizeof(float) * (size_t)(rows - 100) * parts * 3);
  }
  return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaPeekAtLastError(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "fake runtime error"; }
cudaError_t cudaGetDeviceCount(int *c) {
  *c = 1;
  return cudaSuccess;
}

}  // extern "C"
