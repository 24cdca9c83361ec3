/*
 * Runs the reference's own GPU kernels, compiled by nvcc as the reference's
 * Makefile compiles them (-O3 -rdc=true, nvcc's default multiply-add
 * contraction, CUDA's pow), on inputs read from files, and writes their
 * outputs, so that the library can be compared with the reference's GPU
 * program and not only with its CPU build.
 *
 * Test infrastructure only (oracle/refgpu/build_ref_gpu.sh builds it on the
 * GPU machine from the reference sources staged by stage_ref.sh;
 * compare_ref_gpu.py drives it).  The reference's main() (mainPUMP.cu) is not
 * linked; this program launches each kernel with the launch shape
 * mainPUMP.cu / PUMP.cu / collisionProbability.cu use:
 *
 *   bvp         fillCoptsTopts   (2pBVP.cu:133-150, launched as mainPUMP.cu:293-298)
 *   sample_free sampleFree       (sampler.cu:61-88, mainPUMP.cu:430-436)
 *   free_edges  freeEdges        (collisionCheck.cu:5-37, mainPUMP.cu:443-451)
 *   halfspaces  setupAsBs + cacheHalfspaces (hsmc.cu:10-99, 201-211, mainPUMP.cu:466-497)
 *   hsmc        propagateValidParticles + calculateCP_HSMC (PUMP.cu:613-655, 745-758,
 *               launched as PUMP.cu:94-143)
 *   mccp        MCCP             (collisionProbability.cu:39-92, launched as :11-16)
 *
 * Every input file's size is checked against the sizes given on the command
 * line before anything is launched, and every index a kernel forms from them
 * stays inside the buffers (the caller keeps path times below the particle
 * table's 400 rows and dense paths at most Tmax = 100 states).  Each kernel is
 * run `reps` times and timed with CUDA events; the times are printed as one
 * JSON line.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "2pBVP.cuh"
#include "PUMP.cuh"
#include "collisionCheck.cuh"
#include "hardCoded.cuh"
#include "hsmc.cuh"
#include "sampler.cuh"

// particle tables of ref_support.cpp (the stand-in for the absent hardCoded.cu)
extern "C" const float *refsupport_table_tmajor(int *rows, int *particles);

// MCCP is defined in collisionProbability.cu; its header declares only the host wrapper
__global__ void MCCP(int *isCollision, float *path, float *xcomb, float offsetMult,
                     float *obstacles, int obstaclesCount, int T, float *debugOutput);

namespace {

#define CHECK(x)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) {                                                       \
      std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x,               \
                   cudaGetErrorString(e_));                                        \
      std::exit(3);                                                                \
    }                                                                              \
  } while (0)

[[noreturn]] void die(const char *msg, const char *arg = "") {
  std::fprintf(stderr, "ref_gpu: %s %s\n", msg, arg);
  std::exit(2);
}

template <class T>
std::vector<T> read_file(const char *path, size_t n) {
  FILE *f = std::fopen(path, "rb");
  if (!f) die("cannot open", path);
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (size < 0 || (size_t)size != n * sizeof(T)) {
    std::fprintf(stderr, "ref_gpu: %s has %ld bytes, expected %zu\n", path, size, n * sizeof(T));
    std::exit(2);
  }
  std::vector<T> v(n);
  if (n && std::fread(v.data(), sizeof(T), n, f) != n) die("short read", path);
  std::fclose(f);
  return v;
}

template <class T>
void write_file(const char *path, const T *p, size_t n) {
  FILE *f = std::fopen(path, "wb");
  if (!f) die("cannot create", path);
  if (n && std::fwrite(p, sizeof(T), n, f) != n) die("short write", path);
  std::fclose(f);
}

template <class T>
T *to_device(const std::vector<T> &v) {
  T *d = nullptr;
  CHECK(cudaMalloc(&d, sizeof(T) * (v.size() ? v.size() : 1)));
  if (!v.empty()) CHECK(cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return d;
}

template <class T>
std::vector<T> to_host(const T *d, size_t n) {
  std::vector<T> v(n);
  if (n) CHECK(cudaMemcpy(v.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost));
  return v;
}

// bool arrays as bytes (0 or 1), as the device holds them
std::vector<unsigned char> bools_to_host(const bool *d, size_t n) {
  std::vector<unsigned char> v(n);
  if (n) CHECK(cudaMemcpy(v.data(), d, n, cudaMemcpyDeviceToHost));
  for (auto &x : v) x = x ? 1 : 0;
  return v;
}

long long arg_ll(const char *s) { return std::strtoll(s, nullptr, 10); }

// Runs fn() reps times between events; prints {"kernel": ms list}.
template <class F>
void timed(const char *name, int reps, F fn) {
  cudaEvent_t a, b;
  CHECK(cudaEventCreate(&a));
  CHECK(cudaEventCreate(&b));
  std::string out = std::string("{\"kernel\": \"") + name + "\", \"ms\": [";
  for (int r = 0; r < reps; ++r) {
    CHECK(cudaEventRecord(a));
    fn();
    CHECK(cudaEventRecord(b));
    CHECK(cudaEventSynchronize(b));
    CHECK(cudaGetLastError());
    float ms = 0;
    CHECK(cudaEventElapsedTime(&ms, a, b));
    char buf[32];
    std::snprintf(buf, sizeof buf, "%s%.5f", r ? ", " : "", ms);
    out += buf;
  }
  out += "]}";
  std::printf("%s\n", out.c_str());
  CHECK(cudaEventDestroy(a));
  CHECK(cudaEventDestroy(b));
}

int grid_for(long long items, int block) {
  const long long g = (items + block - 1) / block;
  if (g < 1 || g >= 2147483647LL) die("grid out of range");
  return (int)g;
}

// bvp <samples[NUM*6]> <copts_out> <topts_out> <reps>
int cmd_bvp(char **a) {
  const auto s = read_file<float>(a[0], (size_t)NUM * DIM);
  float *d_s = to_device(s), *d_c = nullptr, *d_t = nullptr;
  const size_t np = (size_t)NUM * (NUM - 1);
  CHECK(cudaMalloc(&d_c, sizeof(float) * np));
  CHECK(cudaMalloc(&d_t, sizeof(float) * np));
  const int block = 192;
  const int grid = grid_for((long long)NUM * NUM, block);
  timed("fillCoptsTopts", (int)arg_ll(a[3]), [&] {
    fillCoptsTopts<<<grid, block>>>(d_s, d_c, d_t, 5.0f);
  });
  write_file(a[1], to_host(d_c, np).data(), np);
  write_file(a[2], to_host(d_t, np).data(), np);
  return 0;
}

// sample_free <obs[n*12]> <n> <samples[NUM*6]> <free_out u8[NUM]>
int cmd_sample_free(char **a) {
  const int nobs = (int)arg_ll(a[1]);
  const auto obs = read_file<float>(a[0], (size_t)nobs * 2 * DIM);
  const auto s = read_file<float>(a[2], (size_t)NUM * DIM);
  float *d_o = to_device(obs), *d_s = to_device(s);
  bool *d_f = nullptr;
  CHECK(cudaMalloc(&d_f, NUM));
  sampleFree<<<grid_for(NUM, 192), 192>>>(d_o, nobs, d_s, d_f, nullptr);
  CHECK(cudaDeviceSynchronize());
  const auto out = bools_to_host(d_f, NUM);
  write_file(a[3], out.data(), out.size());
  return 0;
}

// free_edges <obs> <n> <disc[E*(numDisc+1)*6]> <E> <numDisc> <free_out u8[E]> <reps>
int cmd_free_edges(char **a) {
  const int nobs = (int)arg_ll(a[1]);
  const long long E = arg_ll(a[3]);
  const int numDisc = (int)arg_ll(a[4]);
  if (E < 1 || E * (numDisc + 1) * DIM >= 2147483647LL) die("edge count out of the reference's int range");
  const auto obs = read_file<float>(a[0], (size_t)nobs * 2 * DIM);
  const auto disc = read_file<float>(a[2], (size_t)E * (numDisc + 1) * DIM);
  float *d_o = to_device(obs), *d_d = to_device(disc);
  bool *d_f = nullptr;
  CHECK(cudaMalloc(&d_f, E));
  const int block = 192;
  timed("freeEdges", (int)arg_ll(a[6]), [&] {
    freeEdges<<<grid_for(E, block), block>>>(d_o, nobs, nullptr, nullptr, numDisc, d_d, d_f, (int)E,
                                             nullptr);
  });
  const auto out = bools_to_host(d_f, E);
  write_file(a[5], out.data(), out.size());
  return 0;
}

// halfspaces <obs> <n> <disc> <isfree u8[E]> <E> <W> <maxHS> <maxd2> <as_out> <bs_out> <count_out> <reps>
int cmd_halfspaces(char **a) {
  const int nobs = (int)arg_ll(a[1]);
  const long long E = arg_ll(a[4]);
  const int W = (int)arg_ll(a[5]), maxHS = (int)arg_ll(a[6]);
  const float maxd2 = std::strtof(a[7], nullptr);
  if (2 * DIM * nobs > 1024) die("more boxes than cacheHalfspaces' shared-memory stage holds");
  const long long hsCount = E * W * maxHS;
  if (E < 1 || hsCount * 3 >= 2147483647LL) die("half-space count out of the reference's int range");
  const auto obs = read_file<float>(a[0], (size_t)nobs * 2 * DIM);
  const auto disc = read_file<float>(a[2], (size_t)E * W * DIM);
  const auto fr = read_file<unsigned char>(a[3], (size_t)E);
  std::vector<char> frb(E);
  for (long long i = 0; i < E; ++i) frb[i] = fr[i] ? 1 : 0;
  float *d_o = to_device(obs), *d_d = to_device(disc);
  bool *d_f = nullptr;
  CHECK(cudaMalloc(&d_f, E));
  CHECK(cudaMemcpy(d_f, frb.data(), E, cudaMemcpyHostToDevice));
  float *d_as = nullptr, *d_bs = nullptr;
  int *d_cnt = nullptr;
  CHECK(cudaMalloc(&d_as, sizeof(float) * 3 * hsCount));
  CHECK(cudaMalloc(&d_bs, sizeof(float) * hsCount));
  CHECK(cudaMalloc(&d_cnt, sizeof(int) * E * W));
  // the reference leaves the counts of non-free edges unwritten (hsmc.cu:30-31)
  CHECK(cudaMemset(d_cnt, 0, sizeof(int) * E * W));
  setupAsBs<<<grid_for(hsCount, 1024), 1024>>>((int)hsCount, d_bs, d_as);
  CHECK(cudaDeviceSynchronize());
  timed("cacheHalfspaces", (int)arg_ll(a[11]), [&] {
    cacheHalfspaces<<<grid_for(E * W, 1024), 1024, nobs * 2 * DIM * sizeof(float)>>>(
        (int)E, d_d, d_f, nobs, maxHS, d_o, W, d_as, d_bs, d_cnt, nullptr, maxd2);
  });
  write_file(a[8], to_host(d_as, 3 * hsCount).data(), 3 * hsCount);
  write_file(a[9], to_host(d_bs, hsCount).data(), hsCount);
  write_file(a[10], to_host(d_cnt, E * W).data(), E * W);
  return 0;
}

// hsmc <edge i32[M]> <prev i32[M]> <M> <base> <as> <bs> <E> <W> <maxHS> <times f32[base]>
//      <topts f32[E]> <valid u8[base*P]> <P> <offsetMult> <valid_out u8[M*P]> <cp_out f32[M]> <reps>
int cmd_hsmc(char **a) {
  const long long M = arg_ll(a[2]), base = arg_ll(a[3]), E = arg_ll(a[6]);
  const int W = (int)arg_ll(a[7]), maxHS = (int)arg_ll(a[8]), P = (int)arg_ll(a[12]);
  const float offsetMult = std::strtof(a[13], nullptr);
  if (M < 1 || base < 1 || P < 1 || (base + M) * P >= 2147483647LL || E * W * maxHS * 3 >= 2147483647LL)
    die("sizes out of the reference's int range");
  const auto edge = read_file<int>(a[0], M), prev = read_file<int>(a[1], M);
  const auto as = read_file<float>(a[4], (size_t)E * W * maxHS * 3);
  const auto bs = read_file<float>(a[5], (size_t)E * W * maxHS);
  const auto times = read_file<float>(a[9], base);
  const auto topts = read_file<float>(a[10], E);
  const auto valid = read_file<unsigned char>(a[11], (size_t)base * P);
  int rows = 0, pmc = 0;
  const float *tab = refsupport_table_tmajor(&rows, &pmc);
  // every index the kernel forms stays in its buffers
  for (long long i = 0; i < M; ++i) {
    if (edge[i] < 0 || edge[i] >= E || prev[i] < 0 || prev[i] >= base) die("wavefront index out of range");
    const float t_end = times[prev[i]] + topts[edge[i]];
    if (!(times[prev[i]] >= 0) || !(t_end < 0.05f * (rows - 1))) die("path time past the particle table");
  }
  if (P > pmc) die("more HSMC particles than the table holds");
  std::vector<float> tv(tab, tab + (size_t)rows * pmc * 3);
  std::vector<char> vb((size_t)(base + M) * P, 1);
  for (size_t i = 0; i < valid.size(); ++i) vb[i] = valid[i] ? 1 : 0;
  int *d_e = to_device(edge), *d_p = to_device(prev);
  float *d_as = to_device(as), *d_bs = to_device(bs), *d_ti = to_device(times), *d_to = to_device(topts),
        *d_tab = to_device(tv);
  bool *d_v = nullptr;
  CHECK(cudaMalloc(&d_v, vb.size()));
  CHECK(cudaMemcpy(d_v, vb.data(), vb.size(), cudaMemcpyHostToDevice));
  float *d_cp = nullptr;
  CHECK(cudaMalloc(&d_cp, sizeof(float) * (base + M)));
  const int block = 512;
  timed("propagateValidParticles+calculateCP_HSMC", (int)arg_ll(a[16]), [&] {
    propagateValidParticles<<<grid_for(M * P, block), block>>>(
        (int)M, W, d_e, d_p, (int)base, d_as, d_bs, nullptr, d_ti, d_to, 0.05f, maxHS, d_tab,
        offsetMult, pmc, d_v, P, nullptr);
    calculateCP_HSMC<<<grid_for(M, block), block>>>((int)M, (int)base, d_cp, d_v, P);
  });
  const auto out = bools_to_host(d_v + (size_t)base * P, (size_t)M * P);
  write_file(a[14], out.data(), out.size());
  write_file(a[15], to_host(d_cp, base + M).data() + base, M);
  return 0;
}

// mccp <obs> <n> <paths f32[sum T*6]> <lens i32[k]> <k> <offsetMult> <hits_out i32[k]> <reps>
int cmd_mccp(char **a) {
  const int nobs = (int)arg_ll(a[1]), k = (int)arg_ll(a[4]);
  const float offsetMult = std::strtof(a[5], nullptr);
  const auto obs = read_file<float>(a[0], (size_t)nobs * 2 * DIM);
  const auto lens = read_file<int>(a[3], k);
  size_t total = 0;
  for (int i = 0; i < k; ++i) {
    if (lens[i] < 3 || lens[i] > Tmax) die("dense path length outside 3 .. Tmax");
    total += lens[i];
  }
  const auto paths = read_file<float>(a[2], total * DIM);
  float *d_o = to_device(obs), *d_path = to_device(paths);
  std::vector<float> xc(xcomb, xcomb + (size_t)numMCParticles * Tmax * DIM / 2);
  float *d_x = to_device(xc);
  int *d_hit = nullptr;
  CHECK(cudaMalloc(&d_hit, sizeof(int) * numMCParticles));
  std::vector<int> hits(k);
  const int block = 64;
  timed("MCCP", (int)arg_ll(a[7]), [&] {
    size_t off = 0;
    for (int i = 0; i < k; ++i) {
      MCCP<<<grid_for(numMCParticles, block), block>>>(d_hit, d_path + off * DIM, d_x, offsetMult, d_o,
                                                       nobs, lens[i], nullptr);
      off += lens[i];
    }
  });
  size_t off = 0;
  for (int i = 0; i < k; ++i) {
    MCCP<<<grid_for(numMCParticles, block), block>>>(d_hit, d_path + off * DIM, d_x, offsetMult, d_o, nobs,
                                                     lens[i], nullptr);
    const auto h = to_host(d_hit, numMCParticles);
    int s = 0;
    for (int p = 0; p < numMCParticles; ++p) s += h[p];
    hits[i] = s;
    off += lens[i];
  }
  write_file(a[6], hits.data(), hits.size());
  return 0;
}

struct Cmd {
  const char *name;
  int nargs;
  int (*fn)(char **);
};
const Cmd kCmds[] = {{"bvp", 4, cmd_bvp},
                     {"sample_free", 4, cmd_sample_free},
                     {"free_edges", 7, cmd_free_edges},
                     {"halfspaces", 12, cmd_halfspaces},
                     {"hsmc", 17, cmd_hsmc},
                     {"mccp", 8, cmd_mccp}};

}  // namespace

int main(int argc, char **argv) {
  if (argc >= 2)
    for (const Cmd &c : kCmds)
      if (!std::strcmp(argv[1], c.name)) {
        if (argc != 2 + c.nargs) die("wrong argument count for", c.name);
        return c.fn(argv + 2);
      }
  std::fprintf(stderr, "usage: ref_gpu_N%d {bvp|sample_free|free_edges|halfspaces|hsmc|mccp} ...\n", NUM);
  return 2;
}
