// Path refinement: the objective J = cost + lambda * bound of a returned path,
// its adjoint with respect to the intermediate nodes, and a gradient descent
// over many paths whose loop is captured into a CUDA graph (include/pump.h
// states the objective).  One CTA per path:
//   1. segments: the binary64 optimal time tau_i (precise.cuh), the cost, the
//      cost's partial derivatives and dtau/dx by the implicit function theorem;
//   2. segment start times (warp scan of tau);
//   3. waypoints: one warp per segment, its waypoints in order, lanes over the
//      boxes (staged in shared memory); the bound's partial derivatives with
//      respect to each waypoint's position, velocity and noise scale are
//      warp-reduced and pushed back to the segment's two nodes, its tau and
//      its start time;
//   4. start-time adjoints to earlier taus (suffix scan), taus to nodes.
// Every sum runs in a fixed order (no floating-point atomics), so results
// are the same from run to run.
// Binary64 only for the optimal time; everything else binary32.  This
// translation unit is compiled with multiply-add contraction.
#include <math.h>
#include <string.h>

#include "common.cuh"
#include "ctx.h"
#include "precise.cuh"

namespace pump {
namespace {

constexpr int kMaxSeg = PUMP_REFINE_MAX_NODES - 1;
constexpr int kRefThreads = 256;
constexpr int kRefWarps = kRefThreads / 32;
constexpr float kEpsV = 1e-12f;  // added to v.v (a waypoint at rest)
constexpr float kEpsD = 1e-12f;  // added to a.a under the square root

enum Mode { kPlain = 0, kStep = 1, kAccept = 2 };

struct Work {
  float *J, *cost, *bound, *grad;  // kPlain outputs (may be null)
  float *x_cur, *x_trial;          // descent state (node rows)
  float *J_cur, *eta, *g2;         // descent state per path
  float step0;                     // first step length in state units
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Cubic Hermite basis at s: position weights of p0, p1, tau v0, tau v1 and
// velocity weights of (p0 - p1) / tau, v0, v1 (the trajectory of pathPoint,
// 2pBVP.cu:117-131, at t = s tau).
struct Basis {
  float h0, h1, h2, h3, g0, g1, g2;
  __device__ explicit Basis(float s) {
    const float s2 = s * s, s3 = s2 * s;
    h0 = 2.0f * s3 - 3.0f * s2 + 1.0f;
    h1 = -2.0f * s3 + 3.0f * s2;
    h2 = s3 - 2.0f * s2 + s;
    h3 = s3 - s2;
    g0 = 6.0f * s2 - 6.0f * s;
    g1 = 3.0f * s2 - 4.0f * s + 1.0f;
    g2 = 3.0f * s2 - 2.0f * s;
  }
};

template <bool Grad, int M>
__global__ void __launch_bounds__(kRefThreads) refine_kernel(pump_refine_args a, Work w) {
  extern __shared__ float s_obs[];  // per box: lo[0..2], hi[0..2]
  __shared__ float s_tau[kMaxSeg], s_T0[kMaxSeg], s_taubar[kMaxSeg], s_Tbar[kMaxSeg];
  __shared__ float s_dtau[kMaxSeg * 12];  // dtau_i / d(x_i, x_{i+1})
  __shared__ float s_g[kMaxSeg * 12];     // partial dJ / d(x_i, x_{i+1}) of segment i at fixed tau_i
  __shared__ float s_xbar[(kMaxSeg + 1) * 6];
  __shared__ float s_sum[2];
  __shared__ float s_red[2 * kRefWarps];
  __shared__ int s_accept;

  const int path = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int off = a.d_node_offset[path], n = a.d_node_count[path];
  if (n < 2 || n > PUMP_REFINE_MAX_NODES || off < 0 || off + n > a.n_nodes) {
    if (M == kPlain && tid == 0) {
      if (w.J) w.J[path] = __int_as_float(0x7fc00000);
      if (w.cost) w.cost[path] = __int_as_float(0x7fc00000);
      if (w.bound) w.bound[path] = __int_as_float(0x7fc00000);
    }
    return;
  }
  const float lam = a.d_lambda[path];
  const float *x = (M == kPlain ? a.d_nodes : (M == kStep ? w.x_cur : w.x_trial)) + (size_t)off * 6;
  const int nseg = n - 1;

  for (int i = tid; i < a.num_obstacles; i += kRefThreads) {
    const float *b = a.d_obstacles + (size_t)i * 12;
    s_obs[i * 6 + 0] = b[0];
    s_obs[i * 6 + 1] = b[1];
    s_obs[i * 6 + 2] = b[2];
    s_obs[i * 6 + 3] = b[6];
    s_obs[i * 6 + 4] = b[7];
    s_obs[i * 6 + 5] = b[8];
  }

  // 1. segments (thread per segment)
  float csum = 0.0f;
  for (int i = tid; i < nseg; i += kRefThreads) {
    float x0[6], x1[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
      x0[d] = x[i * 6 + d];
      x1[d] = x[i * 6 + 6 + d];
    }
    double td, cd;
    precise_tau(x0, x1, a.tmax, &td, &cd);
    const float t = (float)td;
    s_tau[i] = t;
    csum += (float)cd;
    if (Grad) {
      // dA/dx of A0 = 12|D|^2, A1 = -12 D.S, A2 = 4(v0.v0 + v0.v1 + v1.v1),
      // A3 = 2g(v0z - v1z) with D = p1 - p0, S = v0 + v1
      float dA0[12], dA1[12], dA2[12];
      float A0 = 0.0f, A1 = 0.0f, A2 = 0.0f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float D = x1[d] - x0[d], S = x0[3 + d] + x1[3 + d];
        A0 += D * D;
        A1 += D * S;
        A2 += x0[3 + d] * x0[3 + d] + x0[3 + d] * x1[3 + d] + x1[3 + d] * x1[3 + d];
        dA0[d] = -24.0f * D;
        dA0[6 + d] = 24.0f * D;
        dA0[3 + d] = 0.0f;
        dA0[9 + d] = 0.0f;
        dA1[d] = 12.0f * S;
        dA1[6 + d] = -12.0f * S;
        dA1[3 + d] = -12.0f * D;
        dA1[9 + d] = -12.0f * D;
        dA2[d] = 0.0f;
        dA2[6 + d] = 0.0f;
        dA2[3 + d] = 4.0f * (2.0f * x0[3 + d] + x1[3 + d]);
        dA2[9 + d] = 4.0f * (2.0f * x1[3 + d] + x0[3 + d]);
      }
      A0 *= 12.0f;
      A1 *= -12.0f;
      A2 *= 4.0f;
      const float r1 = 1.0f / t, r2 = r1 * r1, r3 = r2 * r1, r4 = r2 * r2, r5 = r4 * r1;
      const float Ft = 12.0f * A0 * r5 + 6.0f * A1 * r4 + 2.0f * A2 * r3;  // c''(tau)
      const bool clamped = td >= (double)a.tmax;
      const float g2 = 2.0f * PUMP_G;
#pragma unroll
      for (int m = 0; m < 12; ++m) {
        const float dA3 = m == 5 ? g2 : (m == 11 ? -g2 : 0.0f);
        s_g[i * 12 + m] = dA0[m] * r3 + dA1[m] * r2 + dA2[m] * r1 + dA3;
        const float Fx = -3.0f * dA0[m] * r4 - 2.0f * dA1[m] * r3 - dA2[m] * r2;
        s_dtau[i * 12 + m] = clamped ? 0.0f : -Fx / Ft;
      }
    }
  }
  csum = warp_sum(csum);
  if (lane == 0) s_red[warp] = csum;
  __syncthreads();
  if (tid == 0) {
    float c = 0.0f;
    for (int k = 0; k < kRefWarps; ++k) c += s_red[k];
    s_sum[0] = c;
  }

  // 2. segment start times T0[i] = tau_0 + .. + tau_{i-1}
  if (warp == 0) {
    float carry = 0.0f;
    for (int base = 0; base < nseg; base += 32) {
      const float v = base + lane < nseg ? s_tau[base + lane] : 0.0f;
      float inc = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
      }
      if (base + lane < nseg) s_T0[base + lane] = carry + inc - v;
      carry += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
  __syncthreads();

  // 3. waypoints: warp per segment, its W waypoints in order, lanes over boxes
  const float om = a.offset_mult, sf2 = a.sigma_floor * a.sigma_floor;
  float bsum = 0.0f;
  for (int i = warp; i < nseg; i += kRefWarps) {
    float x0[6], x1[6];
#pragma unroll
    for (int d = 0; d < 6; ++d) {
      x0[d] = x[i * 6 + d];
      x1[d] = x[i * 6 + 6 + d];
    }
    const float t = s_tau[i], rt = 1.0f / t, T0 = s_T0[i];
    float acc[12];
#pragma unroll
    for (int m = 0; m < 12; ++m) acc[m] = 0.0f;
    float tb_acc = 0.0f, Tb_acc = 0.0f;
    for (int k = 0; k < a.W; ++k) {
      const float s = (float)k / (float)a.W;
      const Basis B(s);
      float p[3], v[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        p[d] = B.h0 * x0[d] + B.h1 * x1[d] + t * (B.h2 * x0[3 + d] + B.h3 * x1[3 + d]);
        v[d] = B.g0 * (x0[d] - x1[d]) * rt + B.g1 * x0[3 + d] + B.g2 * x1[3 + d];
      }
      const float u = (T0 + s * t) / a.dt;
      float V, dVdT;
      if (!(u < (float)(a.T_rows - 1))) {
        V = (float)a.d_pos_var[a.T_rows - 1];
        dVdT = 0.0f;
      } else {
        const int j = (int)floorf(u);
        const float v0 = (float)a.d_pos_var[j], v1 = (float)a.d_pos_var[j + 1];
        V = v0 + (u - (float)j) * (v1 - v0);
        dVdT = (v1 - v0) / a.dt;
      }
      const float S = om * sqrtf(V + sf2), invS = 1.0f / S;
      const float vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + kEpsV, ivv = 1.0f / vv;
      float gp[3] = {0.0f, 0.0f, 0.0f}, gv[3] = {0.0f, 0.0f, 0.0f}, gS = 0.0f;
      for (int o = lane; o < a.num_obstacles; o += 32) {
        const float *bx = &s_obs[o * 6];
        float r[3];
        bool inside[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float lo = bx[d], hi = bx[3 + d];
          r[d] = fminf(fmaxf(p[d], lo), hi) - p[d];
          inside[d] = p[d] >= lo && p[d] <= hi;
        }
        const float beta = (r[0] * v[0] + r[1] * v[1] + r[2] * v[2]) * ivv;
        float av[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) av[d] = r[d] - beta * v[d];
        const float dist = sqrtf(av[0] * av[0] + av[1] * av[1] + av[2] * av[2] + kEpsD);
        const float z = dist * invS;
        bsum += 0.5f * erfcf(z * 0.70710678118654752f);
        if (Grad) {
          const float zb = -0.39894228040143268f * expf(-0.5f * z * z);  // -phi(z)
          gS -= zb * z * invS;
          const float sc = zb * invS / dist;
          float abar[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) abar[d] = sc * av[d];
          const float betabar = -(abar[0] * v[0] + abar[1] * v[1] + abar[2] * v[2]);
          const float vvbar = -betabar * beta * ivv;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float rbar = abar[d] + betabar * v[d] * ivv;
            gv[d] += -beta * abar[d] + betabar * r[d] * ivv + 2.0f * vvbar * v[d];
            if (!inside[d]) gp[d] -= rbar;
          }
        }
      }
      if (Grad) {
        // every lane ends with the same sums (xor butterfly)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          gp[d] = warp_sum(gp[d]) * lam;
          gv[d] = warp_sum(gv[d]) * lam;
        }
        gS = warp_sum(gS) * lam;
        const float Tb = gS * om * om * 0.5f * invS * dVdT;  // dB/dS dS/dV dV/dT
        float tb = s * Tb;
        const float gr = B.g0 * rt;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          acc[d] += B.h0 * gp[d] + gr * gv[d];
          acc[6 + d] += B.h1 * gp[d] - gr * gv[d];
          acc[3 + d] += t * B.h2 * gp[d] + B.g1 * gv[d];
          acc[9 + d] += t * B.h3 * gp[d] + B.g2 * gv[d];
          tb += (B.h2 * x0[3 + d] + B.h3 * x1[3 + d]) * gp[d];
          tb -= B.g0 * (x0[d] - x1[d]) * rt * rt * gv[d];
        }
        tb_acc += tb;
        Tb_acc += Tb;
      }
    }
    if (Grad && lane == 0) {
#pragma unroll
      for (int m = 0; m < 12; ++m) s_g[i * 12 + m] += acc[m];
      s_taubar[i] = tb_acc;
      s_Tbar[i] = Tb_acc;
    }
  }
  bsum = warp_sum(bsum);
  if (lane == 0) s_red[kRefWarps + warp] = bsum;
  __syncthreads();
  if (tid == 0) {
    float b = 0.0f;
    for (int k = 0; k < kRefWarps; ++k) b += s_red[kRefWarps + k];
    s_sum[1] = b;
  }

  // 4. start-time adjoints (tau_j collects Tbar of every later segment), then
  // node rows: row r gets segment r's x0 part and segment r-1's x1 part
  if (Grad) {
    if (warp == 0) {
      float carry = 0.0f;  // sum of Tbar over segments after the chunk
      for (int top = nseg; top > 0; top -= 32) {
        const int i = top - 1 - lane;
        const float v = i >= 0 ? s_Tbar[i] : 0.0f;
        float inc = v;  // sum over segments i .. top-1
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float u = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += u;
        }
        if (i >= 0) s_taubar[i] += carry + inc - v;
        carry += __shfl_sync(0xffffffffu, inc, 31);
      }
    }
    __syncthreads();
    for (int e = tid; e < n * 6; e += kRefThreads) {
      const int r = e / 6, d = e - 6 * (e / 6);
      float g = 0.0f;
      if (r < nseg) g += s_g[r * 12 + d] + s_taubar[r] * s_dtau[r * 12 + d];
      if (r >= 1) g += s_g[(r - 1) * 12 + 6 + d] + s_taubar[r - 1] * s_dtau[(r - 1) * 12 + 6 + d];
      s_xbar[e] = g;
    }
  }
  __syncthreads();

  const float J = s_sum[0] + lam * s_sum[1];
  if (M == kPlain) {
    if (tid == 0) {
      if (w.J) w.J[path] = J;
      if (w.cost) w.cost[path] = s_sum[0];
      if (w.bound) w.bound[path] = s_sum[1];
    }
    if (Grad && w.grad)
      for (int r = tid; r < n * 6; r += kRefThreads)
        w.grad[(size_t)off * 6 + r] = (r < 6 || r >= (n - 1) * 6) ? 0.0f : s_xbar[r];
  } else if (M == kStep) {
    // |g|^2 and max |g| over the intermediate rows, then the trial point
    float g2 = 0.0f, gm = 0.0f;
    for (int r = 6 + tid; r < (n - 1) * 6; r += kRefThreads) {
      g2 += s_xbar[r] * s_xbar[r];
      gm = fmaxf(gm, fabsf(s_xbar[r]));
    }
    g2 = warp_sum(g2);
    gm = warp_max(gm);
    if (lane == 0) {
      s_red[warp] = g2;
      s_red[kRefWarps + warp] = gm;
    }
    __syncthreads();
    if (tid == 0) {
      float G2 = 0.0f, GM = 0.0f;
      for (int k = 0; k < kRefWarps; ++k) {
        G2 += s_red[k];
        GM = fmaxf(GM, s_red[kRefWarps + k]);
      }
      float eta = w.eta[path];
      if (!(eta > 0.0f)) eta = GM > 0.0f ? w.step0 / GM : 0.0f;
      w.eta[path] = eta;
      w.g2[path] = G2;
      w.J_cur[path] = J;
      s_red[0] = eta;
    }
    __syncthreads();
    const float eta = s_red[0];
    float *xt = w.x_trial + (size_t)off * 6;
    for (int r = tid; r < n * 6; r += kRefThreads)
      xt[r] = (r < 6 || r >= (n - 1) * 6) ? x[r] : x[r] - eta * s_xbar[r];
  } else {  // kAccept: Armijo test of the trial point
    if (tid == 0) {
      const float eta = w.eta[path], Jc = w.J_cur[path];
      const bool ok = J <= Jc - 1e-4f * eta * w.g2[path];  // false for NaN
      s_accept = ok;
      if (ok) {
        w.J_cur[path] = J;
        w.eta[path] = 2.0f * eta;
      } else {
        w.eta[path] = 0.5f * eta;
      }
    }
    __syncthreads();
    if (s_accept) {
      float *xc = w.x_cur + (size_t)off * 6;
      for (int r = tid; r < n * 6; r += kRefThreads) xc[r] = x[r];
    }
  }
}

pump_status_t check_args(const pump_refine_args *a, const char *fn) {
  if (!a || a->n_paths < 0 || (a->n_paths > 0 && (!a->d_nodes || !a->d_node_offset ||
                                                   !a->d_node_count || !a->d_lambda ||
                                                   !a->d_pos_var)) ||
      a->n_nodes < 0 || a->W < 1 || a->W > PUMP_REFINE_MAX_W || !(a->tmax > 0) ||
      a->num_obstacles < 0 || a->num_obstacles > PUMP_REFINE_MAX_OBSTACLES ||
      (a->num_obstacles > 0 && !a->d_obstacles) || !(a->offset_mult > 0) || a->T_rows < 2 ||
      !(a->dt > 0) || !(a->sigma_floor >= 0))
    return set_error(PUMP_ERR_BAD_INPUT, "%s: bad arguments", fn);
  return PUMP_OK;
}

template <bool Grad, int M>
pump_status_t launch(const pump_refine_args &a, const Work &w, cudaStream_t stream) {
  const size_t smem = (size_t)a.num_obstacles * 6 * sizeof(float);
  PUMP_TRY(smem_attr((const void *)refine_kernel<Grad, M>, smem));
  refine_kernel<Grad, M><<<a.n_paths, kRefThreads, smem, stream>>>(a, w);
  return launch_status("refine_kernel");
}

}  // namespace
}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_refine_fwd(const pump_refine_args *a, float *d_J, float *d_cost,
                                         float *d_bound, pump_stream_t stream) {
  PUMP_TRY(check_args(a, "pump_refine_fwd"));
  if (a->n_paths == 0) return PUMP_OK;
  Work w{};
  w.J = d_J;
  w.cost = d_cost;
  w.bound = d_bound;
  return launch<false, kPlain>(*a, w, (cudaStream_t)stream);
}

extern "C" pump_status_t pump_refine_bwd(const pump_refine_args *a, float *d_grad, float *d_J,
                                         pump_stream_t stream) {
  PUMP_TRY(check_args(a, "pump_refine_bwd"));
  if (a->n_paths > 0 && !d_grad) return set_error(PUMP_ERR_BAD_INPUT, "pump_refine_bwd: null gradient");
  if (a->n_paths == 0) return PUMP_OK;
  Work w{};
  w.J = d_J;
  w.grad = d_grad;
  return launch<true, kPlain>(*a, w, (cudaStream_t)stream);
}

extern "C" pump_status_t pump_refine_paths(pump_ctx *ctx, const pump_refine_args *a, int iters,
                                           float *d_nodes_out, float *d_J, pump_stream_t stream) {
  if (!ctx || iters < 0 || (a && a->n_paths > 0 && !d_nodes_out))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_refine_paths: bad arguments");
  PUMP_TRY(check_args(a, "pump_refine_paths"));
  if (a->n_paths == 0) return PUMP_OK;
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  const size_t rows = (size_t)a->n_nodes * 6, np = (size_t)a->n_paths;
  void *scr = nullptr;
  PUMP_TRY(c->scratch(Ctx::kRefine, sizeof(float) * (rows + 3 * np), &scr));
  Work w{};
  w.x_cur = d_nodes_out;
  w.x_trial = (float *)scr;
  w.J_cur = w.x_trial + rows;
  w.eta = w.J_cur + np;
  w.g2 = w.eta + np;
  w.step0 = 0.01f;

  // graph key: everything the captured launches bake in
  unsigned char key[sizeof(Ctx::GraphCache::key)];
  size_t kl = 0;
  auto put = [&](const void *p, size_t n) { memcpy(key + kl, p, n); kl += n; };
  put(a, sizeof *a);
  put(&iters, sizeof iters);
  put(&d_nodes_out, sizeof d_nodes_out);
  put(&d_J, sizeof d_J);
  put(&scr, sizeof scr);
  static_assert(sizeof(pump_refine_args) + sizeof(int) + 3 * sizeof(void *) <= sizeof(key),
                "graph key");
  cudaStream_t s = (cudaStream_t)stream;
  Ctx::GraphCache &gc = c->refine_graph;
  if (!(gc.exec && gc.key_len == kl && memcmp(gc.key, key, kl) == 0)) {
    if (gc.exec) {
      cudaGraphExecDestroy(gc.exec);
      gc.exec = nullptr;
      gc.key_len = 0;
    }
    // set the kernels' shared-memory limits outside the capture
    const size_t smem = (size_t)a->num_obstacles * 6 * sizeof(float);
    PUMP_TRY(smem_attr((const void *)refine_kernel<true, kStep>, smem));
    PUMP_TRY(smem_attr((const void *)refine_kernel<false, kAccept>, smem));
    PUMP_TRY(smem_attr((const void *)refine_kernel<false, kPlain>, smem));
    cudaStream_t cs = nullptr;
    PUMP_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    pump_status_t st = cuda_status(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal),
                                   "cudaStreamBeginCapture");
    if (st == PUMP_OK) {
      if (d_nodes_out != a->d_nodes)
        cudaMemcpyAsync(d_nodes_out, a->d_nodes, sizeof(float) * rows, cudaMemcpyDeviceToDevice, cs);
      cudaMemsetAsync(w.eta, 0, sizeof(float) * np, cs);
      for (int it = 0; it < iters; ++it) {
        refine_kernel<true, kStep><<<a->n_paths, kRefThreads, smem, cs>>>(*a, w);
        refine_kernel<false, kAccept><<<a->n_paths, kRefThreads, smem, cs>>>(*a, w);
      }
      if (d_J) {
        if (iters == 0) {
          Work wj{};
          wj.J = d_J;
          pump_refine_args a0 = *a;
          a0.d_nodes = d_nodes_out;
          refine_kernel<false, kPlain><<<a->n_paths, kRefThreads, smem, cs>>>(a0, wj);
        } else {
          cudaMemcpyAsync(d_J, w.J_cur, sizeof(float) * np, cudaMemcpyDeviceToDevice, cs);
        }
      }
      cudaGraph_t graph = nullptr;
      cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      st = cuda_status(ce, "cudaStreamEndCapture");
      if (st == PUMP_OK) {
        st = cuda_status(cudaGraphInstantiate(&gc.exec, graph, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(graph);
      }
    }
    cudaStreamDestroy(cs);
    if (st != PUMP_OK) {
      gc.exec = nullptr;
      return st;
    }
    memcpy(gc.key, key, kl);
    gc.key_len = kl;
  }
  return cuda_status(cudaGraphLaunch(gc.exec, s), "cudaGraphLaunch");
}
