// rn and the edges from the rn superset in one cooperative launch.
//
// After the pair pass, the rn selection is a string of small dependent
// steps: the superset in pair order, three radix-select passes over it, the
// ordered compaction of the pairs below rn, the adjacency row starts and the
// read-back pack.  As separate launches each step is a few microseconds of
// latency on a few megabytes.  Here one block per SM runs them all, with a
// grid barrier between dependent steps; a cooperative launch keeps every
// block resident, so the barriers always complete, and each barrier wait is
// bounded all the same (past the bound the kernel sets its error word and
// returns, and the host reports PUMP_ERR_TIMEOUT).
//
// The superset comes either as per-warp masks over the pair matrix
// (bvp_precise.cu; the entries' costs and times are read from the pair
// arrays) or already contiguous (*n_in entries).  The
// select and the compaction give the values and order of the full radix
// select and the full compaction (select.cu) whenever the superset holds
// rank k; the pack's ok flag says whether it does.
#pragma once
#include <cuda/atomic>

#include "common.cuh"
#include "ctx.h"

namespace pump {
namespace {

constexpr int kFinishThreads = 1024;
constexpr int kFinishWarps = kFinishThreads / 32;
constexpr int kFinishChunk = 2 * kFinishThreads;  // masks per scan chunk
constexpr int kFinishBatch = 8;                   // loads in flight per thread
constexpr int kFinishBatchA = 4;                  // the same, gathering the superset
constexpr long long kBarrierSpin = 1ll << 22;  // polls (each with a 100 ns sleep)

template <class TSup>
struct RnFinish {
  // the pair pass's superset masks (non-null: nmasks warp masks,
  // masks_per_row per row of the pair matrix, the costs in copts) or a
  // contiguous superset of *n_in entries already in sup_idx and sup_c
  const uint32_t *masks;
  long long nmasks;
  int masks_per_row;
  const float *copts;
  const unsigned long long *n_in;
  uint32_t *sup_idx;
  float *sup_c;
  TSup tsup;  // the optimal time of superset entry q (pair id, pair (i, j))
  long long cap, k, max_edges;
  int N;
  int *e_src, *e_dst;
  float *e_copt, *e_topt;
  int *go_start;                  // may be null
  unsigned int *hist;             // 3 x 2048 words, zero at launch
  unsigned long long *partial;    // 2 x gridDim.x words
  unsigned int *bar;              // barrier count and generation, zero at launch
  unsigned long long *n_sup;      // out: the superset's size
  const int *err_in;              // an earlier pass's wait-bound error word, or null
  int *error;                     // this kernel's
  RnEdgesPack *pack;
  long long spin_limit;
};

// Sense-counting grid barrier of a cooperative launch: false when the wait
// gave up (the error word is set; every block then returns).
__device__ bool finish_barrier(unsigned int *bar, int *error, long long spin_limit) {
  using ref_t = cuda::atomic_ref<unsigned int, cuda::thread_scope_device>;
  __shared__ int s_ok;
  __syncthreads();  // the block's writes are ordered before thread 0's fence
  if (threadIdx.x == 0) {
    __threadfence();
    ref_t gen(bar[1]);
    const unsigned int g = gen.load(cuda::memory_order_acquire);
    int ok = 1;
    if (ref_t(bar[0]).fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
      ref_t(bar[0]).store(0u, cuda::memory_order_relaxed);
      gen.store(g + 1u, cuda::memory_order_release);
    } else {
      long long spins = 0;
      while (gen.load(cuda::memory_order_acquire) == g) {
        if (++spins > spin_limit || *(volatile int *)error) {
          ok = 0;
          atomicExch(error, 1);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Block-wide sum (every thread gets it).
__device__ unsigned long long finish_block_sum(unsigned long long v) {
  __shared__ unsigned long long s_w[kFinishWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) s_w[warp] = v;
  __syncthreads();
  unsigned long long t = 0;
#pragma unroll
  for (int w = 0; w < kFinishWarps; ++w) t += s_w[w];
  return t;
}

// Block-wide exclusive scan of one value per thread; *total = the sum.
__device__ unsigned int finish_block_scan(unsigned int v, unsigned int *total) {
  __shared__ unsigned int s_w[kFinishWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  __syncthreads();
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  unsigned int before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < kFinishWarps; ++w) {
    const unsigned int c = s_w[w];
    before += w < warp ? c : 0u;
    all += c;
  }
  *total = all;
  return before + incl - v;
}

// Position of the k-th (from 0) set bit of m (k < popc(m)).
__device__ __forceinline__ int nth_set_bit(uint32_t m, int k) {
  int pos = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1) {
    const int c = __popc(m & ((1u << step) - 1u));
    if (k >= c) {
      k -= c;
      m >>= step;
      pos += step;
    }
  }
  return pos;
}

// The slice [*q0, *q1) of n items for this block.
__device__ __forceinline__ void finish_slice(long long n, long long *q0, long long *q1) {
  const long long B = gridDim.x, b = blockIdx.x;
  *q0 = n * b / B;
  *q1 = n * (b + 1) / B;
}

template <class TSup>
__global__ void __launch_bounds__(kFinishThreads) rn_finish_kernel(const RnFinish<TSup> a) {
  __shared__ unsigned int s_hist[2048];
  __shared__ unsigned int s_off[kFinishChunk + 1];
  __shared__ uint32_t s_m[kFinishChunk];
  __shared__ unsigned int s_wcnt[kFinishWarps];
  __shared__ uint32_t s_prefix, s_mask;
  __shared__ unsigned long long s_k;
  const int tid = threadIdx.x;
  const int B = gridDim.x, b = blockIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const unsigned int lt = (1u << lane) - 1u;
  for (int q = tid; q < 2048; q += kFinishThreads) s_hist[q] = 0u;
  __syncthreads();
  // ---- the superset, contiguous and in pair order; its first radix pass
  // (the top 11 key bits) is counted as it is gathered
  unsigned long long total = 0;
  if (a.masks) {
    const long long per = (a.nmasks + B - 1) / B;
    const long long t0 = (long long)b * per;
    const long long t1 = t0 + per < a.nmasks ? t0 + per : a.nmasks;
    unsigned long long s = 0;
    for (long long t = t0 + tid; t < t1; t += kFinishThreads) s += __popc(__ldg(&a.masks[t]));
    s = finish_block_sum(s);
    if (tid == 0) a.partial[b] = s;
    if (!finish_barrier(a.bar, a.error, a.spin_limit)) return;
    unsigned long long before = 0;
    for (int j = tid; j < B; j += kFinishThreads) {
      const unsigned long long v = __ldcg(&a.partial[j]);
      before += j < b ? v : 0ull;
      total += v;
    }
    before = finish_block_sum(before);
    total = finish_block_sum(total);
    unsigned long long run = before;
    for (long long c0 = t0; c0 < t1; c0 += kFinishChunk) {
      const int cn = (int)(t1 - c0 < kFinishChunk ? t1 - c0 : kFinishChunk);
      // the chunk's masks and the exclusive offsets of their entries, two
      // masks per thread
      unsigned int v[2], sum = 0;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int q = tid * 2 + u;
        const uint32_t m = q < cn ? __ldg(&a.masks[c0 + q]) : 0u;
        if (q < cn) s_m[q] = m;
        v[u] = __popc(m);
        sum += v[u];
      }
      unsigned int chunk = 0;
      unsigned int ex = finish_block_scan(sum, &chunk);
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int q = tid * 2 + u;
        if (q < cn) s_off[q] = ex;
        ex += v[u];
      }
      if (tid == 0) s_off[cn] = chunk;
      __syncthreads();
      // entry e of the chunk: the mask whose range holds e (the last with
      // offset <= e), its (e - offset)-th set bit, the pair number
      for (unsigned int e0 = 0; e0 < chunk; e0 += kFinishThreads * kFinishBatchA) {
        uint32_t vi[kFinishBatchA], vc[kFinishBatchA];
#pragma unroll
        for (int u = 0; u < kFinishBatchA; ++u) {
          const unsigned int e = e0 + u * kFinishThreads + tid;
          if (e < chunk) {
            int lo = 0, hi = cn;
            while (hi - lo > 1) {
              const int mid = (lo + hi) >> 1;
              if (s_off[mid] <= e) lo = mid; else hi = mid;
            }
            const int bit = nth_set_bit(s_m[lo], (int)(e - s_off[lo]));
            const long long t = c0 + lo;
            const long long row = t / a.masks_per_row;
            const long long col = (t - row * a.masks_per_row) * 32 + bit;
            const long long idx = row * (a.N - 1) + col;
            vi[u] = (uint32_t)idx;
            vc[u] = __ldcg(reinterpret_cast<const uint32_t *>(a.copts) + idx);
          }
        }
#pragma unroll
        for (int u = 0; u < kFinishBatchA; ++u) {
          const unsigned int e = e0 + u * kFinishThreads + tid;
          const unsigned long long pos = run + e;
          if (e < chunk && (long long)pos < a.cap) {
            a.sup_idx[pos] = vi[u];
            reinterpret_cast<uint32_t *>(a.sup_c)[pos] = vc[u];
          }
          const uint32_t bin = e < chunk ? key_of_bits(vc[u]) >> 21 : 0xFFFFFFFFu;
          const unsigned int peers = __match_any_sync(0xffffffffu, bin);
          if (e < chunk && lane == __ffs(peers) - 1) atomicAdd(&s_hist[bin], __popc(peers));
        }
      }
      run += chunk;
      __syncthreads();
    }
    for (int q = tid; q < 2048; q += kFinishThreads)
      if (s_hist[q]) atomicAdd(&a.hist[q], s_hist[q]);
    if (!finish_barrier(a.bar, a.error, a.spin_limit)) return;
  } else {
    total = *a.n_in;
  }
  const long long n = (long long)total < a.cap ? (long long)total : a.cap;
  long long q0, q1;
  finish_slice(n, &q0, &q1);
  const uint32_t *sup_bits = reinterpret_cast<const uint32_t *>(a.sup_c);
  // ---- rank k among the superset's costs: three radix passes (11, 11, 10
  // bits of the order key), each block adding its slice to the pass's
  // histogram, then every block picking the same bin from it
  if (tid == 0) {
    s_prefix = 0u;
    s_mask = 0u;
    s_k = (unsigned long long)a.k;
  }
  __syncthreads();
#pragma unroll 1
  for (int pass = 0; pass < 3; ++pass) {
    const int shift = pass == 0 ? 21 : (pass == 1 ? 10 : 0);
    const int nb = pass == 2 ? 1024 : 2048;
    unsigned int *gh = a.hist + pass * 2048;
    const uint32_t prefix = s_prefix, mask = s_mask;
    if (pass > 0 || !a.masks) {  // (the gather counted the first pass)
      for (int q = tid; q < nb; q += kFinishThreads) s_hist[q] = 0u;
      __syncthreads();
      for (long long b0 = q0; b0 < q1; b0 += (long long)kFinishThreads * kFinishBatch) {
        uint32_t key[kFinishBatch];
#pragma unroll
        for (int u = 0; u < kFinishBatch; ++u) {
          const long long q = b0 + u * kFinishThreads + tid;
          key[u] = q < q1 ? key_of_bits(__ldcg(&sup_bits[q])) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kFinishBatch; ++u) {
          const long long q = b0 + u * kFinishThreads + tid;
          const bool in = q < q1 && (key[u] & mask) == prefix;
          const uint32_t bin = in ? (key[u] >> shift) & (nb - 1) : 0xFFFFFFFFu;
          const unsigned int peers = __match_any_sync(0xffffffffu, bin);
          if (in && lane == __ffs(peers) - 1) atomicAdd(&s_hist[bin], __popc(peers));
        }
      }
      __syncthreads();
      for (int q = tid; q < nb; q += kFinishThreads)
        if (s_hist[q]) atomicAdd(&gh[q], s_hist[q]);
      if (!finish_barrier(a.bar, a.error, a.spin_limit)) return;
    }
    // the pick: nb / kFinishThreads bins per thread, scanned; the thread
    // holding rank k narrows the prefix
    const int per = nb / kFinishThreads;
    unsigned int v[2] = {0u, 0u}, sum = 0;
    for (int u = 0; u < per; ++u) {
      v[u] = __ldcg(&gh[tid * per + u]);
      sum += v[u];
    }
    unsigned int all = 0;
    const unsigned int ex = finish_block_scan(sum, &all);
    const unsigned long long kk = s_k;
    __syncthreads();
    if (kk >= ex && kk < (unsigned long long)ex + sum) {
      unsigned long long c = ex;
      for (int u = 0; u < per; ++u) {
        if (kk < c + v[u]) {
          s_prefix = prefix | ((uint32_t)(tid * per + u) << shift);
          s_mask = mask | ((uint32_t)(nb - 1) << shift);
          s_k = kk - c;
          break;
        }
        c += v[u];
      }
    }
    __syncthreads();
  }
  const uint32_t rn_bits = bits_of_key(s_prefix);
  const float rn = __uint_as_float(rn_bits);
  // ---- the edges: superset entries with cost < rn, in superset order.  Each
  // warp takes a contiguous part of the block's slice: it counts, and after
  // the barrier compacts, its own part.
  const long long len = q1 - q0;
  const long long w0 = q0 + len * warp / kFinishWarps, w1 = q0 + len * (warp + 1) / kFinishWarps;
  unsigned int cnt = 0;
  for (long long b0 = w0; b0 < w1; b0 += 32 * kFinishBatch) {
    float c[kFinishBatch];
#pragma unroll
    for (int u = 0; u < kFinishBatch; ++u) {
      const long long q = b0 + u * 32 + lane;
      c[u] = q < w1 ? __ldcg(&a.sup_c[q]) : rn;
    }
#pragma unroll
    for (int u = 0; u < kFinishBatch; ++u) cnt += c[u] < rn;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0) s_wcnt[warp] = cnt;
  __syncthreads();
  unsigned long long mine = 0, wbase = 0;
  for (int w = 0; w < kFinishWarps; ++w) {
    mine += s_wcnt[w];
    wbase += w < warp ? s_wcnt[w] : 0u;
  }
  if (tid == 0) a.partial[B + b] = mine;
  if (!finish_barrier(a.bar, a.error, a.spin_limit)) return;
  unsigned long long before = 0, edges = 0;
  for (int j = tid; j < B; j += kFinishThreads) {
    const unsigned long long v = __ldcg(&a.partial[B + j]);
    before += j < b ? v : 0ull;
    edges += v;
  }
  before = finish_block_sum(before);
  edges = finish_block_sum(edges);
  unsigned long long run = before + wbase;
  for (long long b0 = w0; b0 < w1; b0 += 32 * kFinishBatch) {
    float c[kFinishBatch];
    uint32_t id[kFinishBatch];
#pragma unroll
    for (int u = 0; u < kFinishBatch; ++u) {
      const long long q = b0 + u * 32 + lane;
      const bool valid = q < w1;
      c[u] = valid ? __ldcg(&a.sup_c[q]) : rn;
      id[u] = valid ? __ldcg(&a.sup_idx[q]) : 0u;
    }
    // the optimal times of the batch's edges, loaded together
    float t[kFinishBatch];
    int ii[kFinishBatch], jj[kFinishBatch];
#pragma unroll
    for (int u = 0; u < kFinishBatch; ++u) {
      const long long q = b0 + u * 32 + lane;
      const uint32_t i = id[u] / (uint32_t)(a.N - 1), r = id[u] - i * (uint32_t)(a.N - 1);
      ii[u] = (int)i;
      jj[u] = (int)r + (r >= i ? 1 : 0);
      t[u] = q < w1 && c[u] < rn ? a.tsup.at(q, id[u], ii[u], jj[u]) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < kFinishBatch; ++u) {
      const long long q = b0 + u * 32 + lane;
      const bool f = q < w1 && c[u] < rn;
      const unsigned int bal = __ballot_sync(0xffffffffu, f);
      const unsigned long long pos = run + __popc(bal & lt);
      if (f && (long long)pos < a.max_edges) {
        a.e_src[pos] = ii[u];
        a.e_dst[pos] = jj[u];
        a.e_copt[pos] = c[u];
        a.e_topt[pos] = t[u];
      }
      run += __popc(bal);
    }
  }
  if (!finish_barrier(a.bar, a.error, a.spin_limit)) return;
  // ---- adjacency row starts (edges sorted by source) and the pack
  const long long E = (long long)edges < a.max_edges ? (long long)edges : a.max_edges;
  if (a.go_start) {
    for (long long e = (long long)b * kFinishThreads + tid; e <= E;
         e += (long long)B * kFinishThreads) {
      const int prev = e > 0 ? __ldcg(&a.e_src[e - 1]) : -1;
      const int cur = e < E ? __ldcg(&a.e_src[e]) : a.N;
      for (int r = prev + 1; r <= cur; ++r) a.go_start[r] = (int)e;
    }
  }
  if (b == 0 && tid == 0) {
    *a.n_sup = total;
    RnEdgesPack pk;
    pk.rn_bits = rn_bits;
    pk.ok = (long long)total > a.k && (long long)total <= a.cap;
    pk.edges = edges;
    pk.error = (a.err_in && *a.err_in) || *(volatile int *)a.error;
    pk.pad = 0;
    *a.pack = pk;
  }
}

}  // namespace
}  // namespace pump
