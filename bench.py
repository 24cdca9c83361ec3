#!/usr/bin/env python3
"""Benchmark of the PUMP hot path on one GB300 (or N replicas under torchrun).

Metric (the reference's headline, quoted at NUM=4000): plan ms, edges/s
through BVP + CC + MC-CP, queries/s.  Workload ("indoor4000"): N = 4000
Halton samples in pos [0,1]^3 x vel [-1,1]^3, 40 boxes (30 walls of a 4 x 4
room grid + 10 boxes), noise multiplier 2e-3, CP target 0.01, eta 2, 1024
HSMC particles, 9 waypoints per edge, closed-form binary64 2pBVP (the
configuration's "FP64 bisection"); synthetic, seeded.

One step = one planning query's hot path:
  value: the device-resident kernels of the query -- all N(N-1) pair BVPs,
         the rn selection, edge compaction and waypoints, sample and edge
         collision checks (E edges), and the HSMC propagation of every
         exploration wavefront of the query (sum M expansions x 1024
         particles, half-spaces derived in the kernel): the query's own HSMC
         launches replayed from its exploration trace with the stored parent
         paths' real start times and particle masks -- launched back to back
         on resident buffers, timed with CUDA events on the launching stream;
         the L2 is flushed (512 MB write) between steps.  Units per step:
         N(N-1) + E + sum M.
  e2e:   the same units through pump_plan() with host buffers: host problem
         in, path out, every host<->device copy and the host search logic
         inside the timed region; ms_per_step of e2e is the plan latency.
The headline uses the precision BVP (the configuration's binary64 root).
The same workload is also reported in the two arithmetics that are bit-exact
with a build of the reference: "parity" (the reference's host arithmetic,
as its CPU build computes) and "parity_gpu" (the pair matrix as the
reference's own GPU kernel computes it), each with its device pipeline, plan
latency and (parity) batched vs plain queries/s.
The CPU baseline is the C oracle (the reference's algorithm restated,
OpenMP over all host cores) timed on one whole query.

--impl reference times that CPU path alone: the reference's CPU
implementation of this path (the C oracle, a restatement pinned bit for bit
to the reference's own code built for the CPU), one whole query per step on
all host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "plan ms @NUM=4000; edges/s (BVP+CC+MC-CP); batched vs plain queries/s @CP"
UNIT = "edges/s"
WORKLOAD = "indoor4000"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--num", type=int, default=4000)
    ap.add_argument("--mode", default="precision", choices=["precision", "parity", "parity_gpu"])
    ap.add_argument("--particles", type=int, default=1024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-refine", action="store_true", help="skip the path-refinement workload")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the records of the two bit-exact arithmetics")
    ap.add_argument("--no-large", action="store_true", help="skip the large configuration (N = 32000)")
    ap.add_argument("--batch", type=int, default=256, help="queries of the batched workload (0: skip)")
    ap.add_argument("--workers", type=int, default=0,
                    help="batched-mode workers (0: the host cores less two, at most 14)")
    return ap.parse_args()


def aggregate(dist, units, total_ms, device="cpu"):
    """Replicas: every rank plans its own query (no data-path collective);
    the job's throughput is the units of all ranks over the slowest rank's
    time.  Returns (sum of units, max of each time in total_ms)."""
    if dist is None:
        return units, list(total_ms)
    import torch
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(x) for x in total_ms], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return u.item(), t.tolist()


def workload(args, query):
    from pump_gb300 import workloads
    obs = workloads.indoor(1000 * 1 + query)
    return dict(N=args.num, obstacles=obs, offset_mult=np.float32(2e-3), cp=0.01, eta=2.0,
                num_disc=8, P=args.particles)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("LOCAL_RANK", "0"),
                                          "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline
def cpu_query(args, query=0):
    """One whole query of the workload through the C oracle (the reference's
    algorithm restated on the CPU, OpenMP over all host cores); returns
    (edges/s, seconds, detail)."""
    from oracle import pyoracle as O
    from pump_gb300 import workloads
    O.build()
    w = workload(args, query)
    N = w["N"]
    tables = O.particle_tables(O.DEFAULT_SEED, 2048, 400)
    t0 = time.perf_counter()
    r = O.plan(N, w["obstacles"], workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI,
               w["offset_mult"], w["cp"], w["eta"], numDisc=w["num_disc"], P=w["P"], tables=tables)
    dt = time.perf_counter() - t0
    units = N * (N - 1) + int(r["numEdges"]) + int(r["numConsidered"])
    detail = {"cores": os.cpu_count() or 1,
              "sample": "one whole query (N=%d: %d pair BVPs with the reference's bisection, "
                        "%d edges checked, %d HSMC expansions x %d particles, solution search "
                        "and smoothing) in %.1f s" % (N, N * (N - 1), int(r["numEdges"]),
                                                       int(r["numConsidered"]), w["P"], dt),
              "units": units, "success": int(r["success"])}
    return units / dt, dt, detail


# ------------------------------------------------------------------ ours
# pump_batch_groups for the grouped form of the batch: a group is launched
# at 16 waiting queries, when every worker is waiting, or after 200 us
GROUPS = (16, 200)


def measure_queries(args, lib, L, ctx, mode):
    """Batched vs plain queries/s on the batched workload (256 queries, N
    log-uniform in [500, 8000], 5-100 boxes, init/goal in free space, CP
    target in {0.001, 0.01, 0.05}, eta in {1, 2, 4}, 4-32 waypoints per edge
    by edge length).  Plain: one pump_plan
    after another on one stream; batched: pump_plan_batch, each worker
    driving its own query's search loop; grouped: pump_plan_batch with the
    search loops of waiting queries run in groups (pump_batch_groups).  A
    query counts only when it returns a path whose Monte Carlo CP is below
    its target."""
    from pump_gb300 import workloads
    qs = workloads.batch_queries(args.batch)
    keep = []
    pbs = (lib.Problem * len(qs))()
    for k, q in enumerate(qs):
        pb = pbs[k]
        L.pump_problem_defaults(C.byref(pb))
        obs = np.ascontiguousarray(q["obstacles"], np.float32)
        keep.append(obs)
        pb.N, pb.num_obstacles, pb.obstacles = q["N"], obs.shape[0], obs.ctypes.data
        for d in range(6):
            pb.init[d], pb.goal[d] = q["init"][d], q["goal"][d]
            pb.lo[d], pb.hi[d] = workloads.LO[d], workloads.HI[d]
        pb.offset_mult, pb.cp_target, pb.cp_factor = float(q["offset_mult"]), q["cp"], q["eta"]
        pb.bvp_mode = Query.MODES[mode]
        pb.num_disc, pb.disc_len, pb.disc_min = q["num_disc"], q["disc_len"], q["disc_min"]
    paths = {}

    def results(tag):
        paths[tag] = np.zeros((len(qs), 400, 6), np.float32)
        res = (lib.PlanResult * len(qs))()
        for k in range(len(qs)):
            res[k].path, res[k].path_cap = paths[tag][k].ctypes.data, 400
        return res

    def ok(res, sts):
        return sum(1 for k in range(len(qs)) if sts[k] == lib.PUMP_OK and res[k].success
                   and res[k].soln_cp < pbs[k].cp_target)
    # a worker sweep on the GB300 machine (16 host cores, 128 uneven queries):
    # 4 -> 1646, 8 -> 1934, 16 -> 1806, 32 -> 1598 q/s; past about 8 the GPU is
    # saturated and more threads only contend
    workers = args.workers or max(1, min(14, (os.cpu_count() or 8) - 2))
    # warm both paths on every query (contexts, particle tables, and the
    # autotuner's first call of each shape class, which neither timed run pays)
    res = results("warm")
    sts = (C.c_int * len(qs))()
    for k in range(len(qs)):
        sts[k] = L.pump_plan(ctx.handle, C.byref(pbs[k]), C.byref(res[k]), None)
    L.pump_plan_batch(0, pbs, res, sts, len(qs), workers)
    # each form timed three times (the median is reported: a batch of 256
    # queries takes under 0.1 s, and single runs vary by several percent)
    res_p, sts_p = results("plain"), (C.c_int * len(qs))()
    tp = []
    for _ in range(3):
        t0 = time.perf_counter()
        for k in range(len(qs)):
            sts_p[k] = L.pump_plan(ctx.handle, C.byref(pbs[k]), C.byref(res_p[k]), None)
        tp.append(time.perf_counter() - t0)
    t_plain = statistics.median(tp)
    res_b, sts_b = results("batched"), (C.c_int * len(qs))()
    tb = []
    for _ in range(3):
        t0 = time.perf_counter()
        lib.check(L.pump_plan_batch(0, pbs, res_b, sts_b, len(qs), workers))
        tb.append(time.perf_counter() - t0)
    t_batch = statistics.median(tb)
    # the grouped form: the search loops of up to 16 waiting queries run as
    # one launch of the loop graph (pump_batch_groups)
    res_g, sts_g = results("grouped"), (C.c_int * len(qs))()
    tg = []
    try:
        L.pump_batch_groups(*GROUPS)
        lib.check(L.pump_plan_batch(0, pbs, res_g, sts_g, len(qs), workers))  # its graphs
        for _ in range(3):
            t0 = time.perf_counter()
            lib.check(L.pump_plan_batch(0, pbs, res_g, sts_g, len(qs), workers))
            tg.append(time.perf_counter() - t0)
    finally:
        L.pump_batch_groups(1, 100)
    t_group = statistics.median(tg)
    # identical results: status, solution index, CP and cost bits, and the
    # returned path's states bit for bit
    f32 = lambda x: np.float32(x).view(np.uint32)  # noqa: E731

    def same_as_plain(res_b, sts_b, tag):
        return all(res_p[k].success == res_b[k].success and res_p[k].soln_path_idx == res_b[k].soln_path_idx
                   and sts_p[k] == sts_b[k] and res_p[k].path_len == res_b[k].path_len
                   and f32(res_p[k].soln_cp) == f32(res_b[k].soln_cp)
                   and f32(res_p[k].soln_cost) == f32(res_b[k].soln_cost)
                   and np.array_equal(paths["plain"][k][: res_p[k].path_len].view(np.uint32),
                                      paths[tag][k][: res_b[k].path_len].view(np.uint32))
                   for k in range(len(qs)))
    same = same_as_plain(res_b, sts_b, "batched")
    ok_p, ok_b, ok_g = ok(res_p, sts_p), ok(res_b, sts_b), ok(res_g, sts_g)
    return {"workload": "batch256: N log-uniform [500, 8000], 5-100 boxes, noise 1e-3, waypoints "
                        "per edge by edge length (at most 0.025 apart, 4 to 32)",
            "bvp": mode, "queries": len(qs), "met_cp_target": ok_b, "workers": workers,
            "plain_queries_per_s": ok_p / t_plain, "batched_queries_per_s": ok_b / t_batch,
            "batched_over_plain": (ok_b / t_batch) / (ok_p / t_plain) if ok_p else None,
            "plain_s": t_plain, "batched_s": t_batch, "plain_s_runs": tp, "batched_s_runs": tb,
            "identical_results": bool(same),
            "grouped": {"max_group": GROUPS[0], "window_us": GROUPS[1],
                        "queries_per_s": ok_g / t_group, "s_runs": tg,
                        "identical_results": bool(same_as_plain(res_g, sts_g, "grouped"))}}


def measure_refine(args, lib, L, ctx, torch):
    """Path refinement over 1024 returned paths (8-40 nodes each) on a
    config-1-style indoor map (40 boxes, noise multiplier 2e-3): the paths are
    the returned paths of 64 planning queries (N=1000, random free init/goal),
    each resampled at 16 node counts; lambda log-uniform in [0.1, 100].
    Times one objective+adjoint launch over all paths and the 30-step
    descent (a captured CUDA graph), then judges every refined path with the
    Monte Carlo CP over 4096 particles: accepted only if CP <= 0.01 and its
    cost drops."""
    from pump_gb300 import workloads
    rng = np.random.Generator(np.random.MT19937(3000))
    obs = workloads.indoor(1001).astype(np.float32)
    nq = 64
    pbs = (lib.Problem * nq)()
    for k in range(nq):
        pb = pbs[k]
        L.pump_problem_defaults(C.byref(pb))
        pb.N, pb.num_obstacles, pb.obstacles = 1000, obs.shape[0], obs.ctypes.data
        a, b = workloads.free_point(rng, obs), workloads.free_point(rng, obs)
        for d in range(6):
            pb.init[d], pb.goal[d] = a[d], b[d]
            pb.lo[d], pb.hi[d] = workloads.LO[d], workloads.HI[d]
        pb.offset_mult, pb.cp_target, pb.cp_factor, pb.bvp_mode = 2e-3, 0.01, 2.0, 1
    dense = np.zeros((nq, 400, 6), np.float32)
    res = (lib.PlanResult * nq)()
    for k in range(nq):
        res[k].path, res[k].path_cap = dense[k].ctypes.data, 400
    sts = (C.c_int * nq)()
    lib.check(L.pump_plan_batch(0, pbs, res, sts, nq, os.cpu_count() or 4))
    src = [dense[k][:res[k].path_len] for k in range(nq) if sts[k] == lib.PUMP_OK and res[k].path_len >= 8]
    rows, offs, cnts = [], [], []
    total = 0
    for q in range(1024):
        d = src[q % len(src)]
        n = int(rng.integers(8, min(40, d.shape[0]) + 1))
        idx = np.round(np.linspace(0, d.shape[0] - 1, n)).astype(int)
        rows.append(d[idx])
        offs.append(total)
        cnts.append(n)
        total += n
    nodes = np.concatenate(rows).astype(np.float32)
    offs, cnts = np.asarray(offs, np.int32), np.asarray(cnts, np.int32)
    lam = np.exp(rng.uniform(np.log(0.1), np.log(100.0), 1024)).astype(np.float32)

    def dev(x):
        return torch.from_numpy(np.ascontiguousarray(x).copy()).cuda()
    keep = [dev(nodes), dev(offs), dev(cnts), dev(lam), dev(obs)]
    var = torch.empty(400, dtype=torch.float64, device="cuda")
    lib.check(L.pump_position_variance(400, var.data_ptr(), None))
    a = lib.RefineArgs()
    a.d_nodes, a.n_nodes = keep[0].data_ptr(), nodes.shape[0]
    a.d_node_offset, a.d_node_count, a.n_paths = keep[1].data_ptr(), keep[2].data_ptr(), 1024
    a.d_lambda, a.W, a.tmax = keep[3].data_ptr(), 8, 5.0
    a.d_obstacles, a.num_obstacles, a.offset_mult = keep[4].data_ptr(), obs.shape[0], 2e-3
    a.d_pos_var, a.T_rows, a.dt, a.sigma_floor = var.data_ptr(), 400, 0.05, 1e-3
    grad = torch.empty(nodes.size, dtype=torch.float32, device="cuda")
    J = torch.empty(1024, dtype=torch.float32, device="cuda")
    out = torch.empty(nodes.size, dtype=torch.float32, device="cuda")
    Jo = torch.empty(1024, dtype=torch.float32, device="cuda")

    def event_ms(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ts = []
        for _ in range(reps):
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)
    sh = torch.cuda.current_stream().cuda_stream
    t_bwd = event_ms(lambda: lib.check(L.pump_refine_bwd(C.byref(a), grad.data_ptr(), J.data_ptr(), sh)), 10)
    iters = 30
    t_desc = event_ms(lambda: lib.check(L.pump_refine_paths(ctx.handle, C.byref(a), iters, out.data_ptr(),
                                                             Jo.data_ptr(), sh)), 5)
    torch.cuda.synchronize()
    J0, J1 = J.cpu().numpy(), Jo.cpu().numpy()
    refined = out.cpu().numpy().reshape(-1, 6)
    table = torch.empty(400 * 4096 * 3, dtype=torch.float32, device="cuda")
    lib.check(L.pump_particle_tables(0x9E3779B97F4A7C15, 4096, 400, table.data_ptr(), None, None))
    torch.cuda.synchronize()

    def judge(x):
        cp, cost, ln = (np.zeros(1024, t) for t in (np.float32, np.float32, np.int32))
        lib.check(L.pump_path_cp(ctx.handle, np.ascontiguousarray(x).ctypes.data, offs.ctypes.data,
                                 cnts.ctypes.data, 1024, 1, table.data_ptr(), 4096, 400, 2e-3,
                                 keep[4].data_ptr(), obs.shape[0], cp.ctypes.data, cost.ctypes.data,
                                 ln.ctypes.data, None))
        return cp, cost
    t0 = time.perf_counter()
    cp0, c0 = judge(nodes)
    cp1, c1 = judge(refined)
    t_judge = (time.perf_counter() - t0) / 2
    valid0 = (cp0 >= 0) & (cp0 <= 0.01)
    acc = valid0 & (cp1 >= 0) & (cp1 <= 0.01) & (c1 < c0)
    terms = int(np.sum(cnts - 1)) * 8 * obs.shape[0]
    return {"workload": "refine1024: 1024 returned paths x 8-40 nodes, indoor map (40 boxes), "
                        "noise 2e-3, lambda log-uniform [0.1, 100], 8 waypoints per segment",
            "objective_adjoint_ms": t_bwd, "paths_per_s": 1024 / (t_bwd / 1e3),
            "waypoint_box_terms_per_s": terms / (t_bwd / 1e3),
            "descent_iters": iters, "descent_ms": t_desc,
            "J_reduction_median": float(np.median(1 - J1 / J0)),
            "judge_ms": t_judge * 1e3, "judge_particles": 4096,
            "paths_meeting_target_before": int(valid0.sum()),
            "accepted": int(acc.sum()),
            "cost_reduction_median_accepted": float(np.median(1 - c1[acc] / c0[acc])) if acc.any() else None}


# Throughput probe of the binary64 FMA pipe, the denominator of the pair
# BVP's FP64 roofline (the peaks file holds HBM copy and bf16 GEMM figures
# only): eight independent DFMA chains per thread, 8 blocks of 256 threads
# per SM, 2 flops per DFMA.  A benchmark aid, not part of the library: it is
# compiled here into the build directory on first use.
FP64_PROBE_SRC = r"""
#include <cuda_runtime.h>
__global__ void __launch_bounds__(256) dfma_kernel(int iters, double seed, double *sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-9 + k;
  const double m = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 42.0) sink[0] = s;  // keeps the chains live; never true
}
extern "C" int fp64_probe_launch(int blocks, int iters, double *sink, void *stream) {
  dfma_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, 1.0, sink);
  return (int)cudaGetLastError();
}
"""


def fp64_peak_tflops(torch):
    from pump_gb300.build import OUT, nvcc
    so = os.path.join(OUT, "libfp64probe.so")
    if not os.path.exists(so):
        src = os.path.join(OUT, "fp64probe.cu")
        with open(src, "w") as f:
            f.write(FP64_PROBE_SRC)
        subprocess.run([nvcc(), "-shared", "-Xcompiler", "-fPIC", "-O3", "-gencode",
                        "arch=compute_103a,code=sm_103a", src, "-o", so], check=True)
    P = C.CDLL(so)
    P.fp64_probe_launch.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    blocks = torch.cuda.get_device_properties(0).multi_processor_count * 8
    sink = torch.empty(1, dtype=torch.float64, device="cuda")
    sh = torch.cuda.current_stream().cuda_stream
    iters = 4096
    assert P.fp64_probe_launch(blocks, iters // 8, sink.data_ptr(), sh) == 0
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    assert P.fp64_probe_launch(blocks, iters, sink.data_ptr(), sh) == 0
    b.record()
    b.synchronize()
    return 2.0 * 8.0 * iters * blocks * 256 / (a.elapsed_time(b) * 1e-3) / 1e12


class Query:
    """One planning problem through the C ABI on one context and stream:
    plan() runs pump_plan; pipeline() times the device-resident kernels of
    the same query (see the module docstring)."""

    MODES = {"parity": 0, "precision": 1, "parity_gpu": 2}

    def __init__(self, lib, L, ctx, torch, w, mode):
        from pump_gb300 import workloads
        self.lib, self.L, self.ctx, self.torch, self.w = lib, L, ctx, torch, w
        self.mode = self.MODES[mode]
        self.obs = np.ascontiguousarray(w["obstacles"], np.float32)
        pb = lib.Problem()
        L.pump_problem_defaults(C.byref(pb))
        pb.N, pb.num_disc, pb.num_hsmc = w["N"], w["num_disc"], w["P"]
        # the Monte Carlo CP uses at least as many particles as HSMC
        pb.num_mc = max(w.get("num_mc", pb.num_mc), w["P"])
        pb.max_paths = w.get("max_paths", 0)
        pb.num_obstacles, pb.obstacles = self.obs.shape[0], self.obs.ctypes.data
        for k in range(6):
            pb.init[k], pb.goal[k] = workloads.INIT[k], workloads.GOAL[k]
            pb.lo[k], pb.hi[k] = workloads.LO[k], workloads.HI[k]
        pb.offset_mult, pb.cp_target, pb.cp_factor = float(w["offset_mult"]), w["cp"], w["eta"]
        pb.bvp_mode = self.mode
        self.pb = pb
        self.path = np.zeros((pb.table_rows, 6), np.float32)

    def plan(self, trace=False, paths_cap=0):
        """One pump_plan call; with trace, also the exploration trace, and
        with paths_cap >= the stored paths, their times and particle masks
        (with the trace, every HSMC launch's inputs)."""
        lib, pb = self.lib, self.pb
        res = lib.PlanResult()
        res.path, res.path_cap = self.path.ctypes.data, pb.table_rows
        if trace:
            self.trace_buf = np.zeros(self.trace_cap, np.int32)
            res.wf_trace, res.wf_trace_cap = self.trace_buf.ctypes.data, self.trace_buf.size
        if paths_cap:
            self.ptime = np.zeros(paths_cap, np.float32)
            self.pvalid = np.zeros(paths_cap * ((pb.num_hsmc + 31) // 32), np.uint32)
            res.path_time, res.path_valid, res.path_state_cap = (self.ptime.ctypes.data,
                                                                 self.pvalid.ctypes.data, paths_cap)
        st = self.L.pump_plan(self.ctx.handle, C.byref(pb), C.byref(res), None)
        if st not in (lib.PUMP_OK, lib.PUMP_ERR_NO_SOLUTION):
            lib.check(st)
        return res

    def pipeline(self, steps, warmup, flush, clocks=None):
        """Device-resident kernels of one query per step; returns the timing
        record.  HSMC replays the query's own launches: its (parent, edge)
        trace with the stored parents' real times and particle masks."""
        torch, lib, L, w = self.torch, self.lib, self.L, self.w
        stream = torch.cuda.current_stream()
        sh = stream.cuda_stream
        res0 = self.plan()
        self.trace_cap = 2 * int(res0.num_considered) + 2
        res0 = self.plan(trace=True, paths_cap=max(1, int(res0.num_paths)))
        assert res0.wf_trace_len == 2 * res0.num_considered, "exploration trace truncated"
        N, P, W = w["N"], w["P"], w["num_disc"] + 1
        E = int(res0.num_edges)
        nobs = self.obs.shape[0]
        sizes = [int(res0.wavefront_sizes[i]) for i in range(min(res0.iterations, 32))]
        sizes = [x for x in sizes if x > 0]
        trace = self.trace_buf[: res0.wf_trace_len].reshape(-1, 2).copy()
        M_total = int(trace.shape[0])
        units = N * (N - 1) + E + M_total
        words = (P + 31) // 32
        base = int(res0.num_paths)

        def dev(a):
            return torch.from_numpy(np.ascontiguousarray(a).copy()).cuda()

        def empty(n, dt):
            return torch.empty(int(max(n, 1)), dtype=dt, device="cuda")

        f6 = lambda v: (C.c_float * 6)(*[float(x) for x in v])  # noqa: E731
        pb = self.pb
        d_s = empty(N * 6, torch.float32)
        lib.check(L.pump_halton_samples(N, f6(pb.lo), f6(pb.hi), f6(pb.init), f6(pb.goal),
                                        d_s.data_ptr(), sh))
        d_obs = dev(self.obs)
        npairs = N * (N - 1)
        d_c, d_t = empty(npairs, torch.float32), empty(npairs, torch.float32)
        rn_idx = int(np.float32((N - 1) * N) * np.float32(0.05))
        cap = rn_idx
        d_src, d_dst = empty(cap, torch.int32), empty(cap, torch.int32)
        d_ce, d_te = empty(cap, torch.float32), empty(cap, torch.float32)
        d_go = empty(N + 1, torch.int32)
        d_disc = empty(cap * W * 6, torch.float32)
        d_fs, d_fe = empty(N, torch.uint8), empty(cap, torch.uint8)
        maxHS = min(nobs, 5)
        Pmc, T = int(pb.num_mc), int(pb.table_rows)
        d_tab = empty(T * Pmc * 3, torch.float32)
        lib.check(L.pump_particle_tables(pb.seed, Pmc, T, d_tab.data_ptr(), None, sh))
        # parents: the stored paths' masks and times; new paths go after them
        valid = np.zeros((base + max(sizes + [1])) * words, np.uint32)
        valid[: base * words] = self.pvalid[: base * words]
        d_valid = dev(valid.view(np.int32))
        d_times = dev(self.ptime[:base])
        d_cp = empty(base + max(sizes + [1]), torch.float32)
        d_err = empty(1, torch.int32).zero_()
        offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        d_prev = dev(trace[:, 0].astype(np.int32))
        d_edge = dev(trace[:, 1].astype(np.int32))
        maxd2 = float(np.float32(0.1 * np.float64(w["offset_mult"]) ** 2))
        rn = C.c_float(0)
        Eo = C.c_longlong(0)
        launches = {"n": 0}
        ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
        kernel_ms = {}
        mode = self.mode

        def timed(name, fn, nk):
            a, b = ev(), ev()
            a.record(stream)
            fn()
            b.record(stream)
            kernel_ms.setdefault(name, []).append((a, b))
            launches["n"] += nk

        stage = (C.c_float * 3)()
        stage_ms = {}
        # our kernels per pump_roadmap call: in the precision arithmetic the
        # samples with the rn bracket and the pair kernel staging the
        # superset; otherwise the pair kernel, the bracket and the superset's
        # count, scan and emit; then the finishing kernel (select, edges, row
        # starts, pack)
        roadmap_launches = 2 + 1 if mode == lib.PUMP_BVP_PRECISION else 5 + 1

        def roadmap():
            lib.check(L.pump_roadmap(self.ctx.handle, d_s.data_ptr(), N, 5.0, mode, rn_idx, cap,
                                     d_c.data_ptr(), d_t.data_ptr(), d_src.data_ptr(),
                                     d_dst.data_ptr(), d_ce.data_ptr(), d_te.data_ptr(),
                                     d_go.data_ptr(), C.byref(rn), C.byref(Eo), stage, sh))
            for name, v in zip(("rn_bracket", "bvp_pairs", "rn_edges"), stage):
                stage_ms.setdefault(name, []).append(float(v))

        def step():
            timed("roadmap", roadmap, roadmap_launches)
            timed("discretize", lambda: lib.check(L.pump_discretize_edges(
                d_s.data_ptr(), d_src.data_ptr(), d_dst.data_ptr(), d_te.data_ptr(), Eo.value, W - 1,
                mode, d_disc.data_ptr(), sh)), 1)
            timed("sample_free", lambda: lib.check(L.pump_sample_free(
                d_obs.data_ptr(), nobs, d_s.data_ptr(), N, d_fs.data_ptr(), sh)), 1)
            timed("free_edges", lambda: lib.check(L.pump_free_edges(
                d_obs.data_ptr(), nobs, d_disc.data_ptr(), Eo.value, W - 1, d_fe.data_ptr(), sh)), 1)

            # half-spaces derived inside the HSMC kernel from the boxes (the planner's path)
            def hsmc_all():
                for it, m in enumerate(sizes):
                    o = int(offs[it])
                    lib.check(L.pump_hsmc_propagate_boxes(
                        m, W, d_edge.data_ptr() + 4 * o, d_prev.data_ptr() + 4 * o, E, base,
                        d_obs.data_ptr(), nobs, d_disc.data_ptr(), maxd2, maxHS, d_times.data_ptr(),
                        d_te.data_ptr(), 0.05, d_tab.data_ptr(), Pmc, T, float(w["offset_mult"]),
                        d_valid.data_ptr(), P, d_cp.data_ptr(), d_err.data_ptr(), sh))
            timed("hsmc", hsmc_all, len(sizes))

        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        assert Eo.value == E, (Eo.value, E)
        assert int(d_err.item()) == 0
        kernel_ms.clear()
        launches["n"] = 0
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        step_ms = []
        for _ in range(steps):
            flush.fill_(1.0)
            a, b = ev(), ev()
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            step_ms.append(a.elapsed_time(b))
        torch.cuda.synchronize()
        ks = {k: sum(a.elapsed_time(b) for a, b in v) / steps for k, v in kernel_ms.items()}
        # the pair kernel and the stages around it, from the library's own
        # events on the same stream (the timed steps' calls only)
        ks.update({k: sum(v[-steps:]) / steps for k, v in stage_ms.items()})
        return {"units": units, "E": E, "M": M_total, "W": W, "maxHS": maxHS, "sizes": sizes,
                "step_ms": step_ms, "kernel_ms": ks, "launches": launches["n"],
                "per_step_units": {"pairs": npairs, "edges": E, "expansions": M_total}}

    def e2e(self, reps):
        """pump_plan latencies (host problem in, path out)."""
        out, res = [], None
        for _ in range(max(1, reps)):
            t0 = time.perf_counter()
            res = self.plan()
            out.append((time.perf_counter() - t0) * 1e3)
        return out, res


def run_ours(args):
    import torch
    from pump_gb300 import lib
    from pump_gb300.build import build as build_lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    build_lib()
    L = lib.load()
    torch.cuda.set_device(local)
    ctx = lib.Context(local)
    w = workload(args, rank)
    N, P = w["N"], w["P"]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    q = Query(lib, L, ctx, torch, w, args.mode)
    if dist:
        dist.barrier()
    clocks = ClockSampler()
    pipe = q.pipeline(args.steps, args.warmup, flush, clocks)
    # e2e: pump_plan with host buffers (includes roadmap + online + search)
    e2e_ms, plan_res = q.e2e(args.steps)
    clk = clocks.stop()
    if dist:
        dist.barrier()
    units, E, M_total, W = pipe["units"], pipe["E"], pipe["M"], pipe["W"]
    all_units, (tot, tot_e2e) = aggregate(dist, units, [sum(pipe["step_ms"]), sum(e2e_ms)], "cuda")
    ks = pipe["kernel_ms"]
    out = None
    if rank == 0:
        value = all_units * args.steps / (tot / 1e3)
        e2e_value = all_units * max(1, args.steps) / (tot_e2e / 1e3)
        # the dominant kernel: "roadmap" is the whole pump_roadmap call, whose
        # stages (the pair kernel among them) are listed on their own
        dom = max((k for k in ks if k != "roadmap"), key=ks.get)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded indoor map, Halton samples)",
            "config": {"workload": WORKLOAD, "N": N, "obstacles": int(q.obs.shape[0]),
                       "hsmc_particles": P, "waypoints_per_edge": W, "noise_mult": 2e-3,
                       "cp_target": 0.01, "eta": 2, "bvp": args.mode, "edges": E,
                       "expansions": M_total, "units_per_step": units,
                       "l2": "flushed between steps (512 MB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "plan_ms": statistics.median(e2e_ms),
            "plan_stage_ms": {"roadmap": plan_res.ms_roadmap, "online": plan_res.ms_online,
                              "explore": plan_res.ms_explore, "search": plan_res.ms_search},
            "edges_per_s": {"bvp": N * (N - 1) / (ks["bvp_pairs"] / 1e3),
                            "cc": E / (ks["free_edges"] / 1e3),
                            "hsmc": M_total / (ks["hsmc"] / 1e3)},
            "kernel_ms": {k: round(v, 4) for k, v in ks.items()},
            "dominant_kernel": dom,
            "queries_per_s_plain": 1e3 / statistics.median(e2e_ms),
            "solution": {"success": int(plan_res.success), "cp": plan_res.soln_cp,
                         "cost": plan_res.soln_cost, "paths": plan_res.num_paths},
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(plan_res.h2d_bytes),
                    "d2h_bytes_per_step": int(plan_res.d2h_bytes)},
            "gpu_launches": pipe["launches"],
            "clocks": clk,
        }
        out["roofline"] = roofline(dom, ks, N, E, M_total, W, pipe["maxHS"], P, args.mode,
                                   fp64_peak_tflops(torch), float(clk.get("sm_mhz") or 2070.0))
        if args.batch > 0:
            out["queries_per_s"] = measure_queries(args, lib, L, ctx, args.mode)
        # the two arithmetics that are bit-exact with a build of the reference,
        # on the same workload
        if not args.no_parity and args.mode == "precision":
            out["parity"] = mode_record(lib, L, ctx, torch, w, "parity", args, flush, batch=args.batch)
            out["parity_gpu"] = mode_record(lib, L, ctx, torch, w, "parity_gpu", args, flush, batch=0,
                                            steps=2, warmup=1)
        if not args.no_large and args.mode == "precision":
            try:
                out["large"] = large_record(lib, L, ctx, torch, flush)
            except lib.PumpError as e:  # reported, not fatal to the headline
                out["large"] = {"config": {"workload": "large32000"}, "error": str(e)}
        if not args.no_refine:
            out["refine"] = measure_refine(args, lib, L, ctx, torch)
        if not args.no_cpu_baseline:
            v, _dt, det = cpu_query(args, 0)
            out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": det["cores"], "kind": "port",
                                   "sample": det["sample"]}
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return out


BIT_EXACT_AGAINST = {
    "parity": "the reference program built for the CPU (x86 host arithmetic, no contraction): "
              "whole queries match tests/golden/ref_*.npz bit for bit",
    "parity_gpu": "the reference's own fillCoptsTopts on the GB300 for the pair matrix, its host "
                  "arithmetic elsewhere: whole queries match tests/golden/refgpu_*.npz bit for bit",
}


def large_record(lib, L, ctx, torch, flush):
    """The large configuration (N = 32000, 200 boxes with sides U[0.02, 0.1],
    noise 5e-3, 4096 particles for HSMC and MC CP, 16 waypoints per edge,
    CP target 0.005, eta 2, precision BVP, a path store of 2^24 paths: its
    largest wavefront holds 14.1 M new paths, past the reference's 2 N
    sqrt(N) = 11.4 M): one step of the device pipeline after one warm-up,
    and the plan latency.  The reference cannot run it
    unmodified (its sample count is a compile-time array size and its
    particle tables hold 2048 particles), so it has no CPU baseline here."""
    from pump_gb300 import workloads
    cfg = workloads.CONFIGS["cfg4"]
    w = dict(N=cfg["N"], obstacles=cfg["obstacles"](0), offset_mult=np.float32(cfg["offset_mult"]),
             cp=cfg["cp"], eta=cfg["eta"], num_disc=cfg["num_disc"], P=cfg["num_hsmc"],
             num_mc=cfg["num_mc"], max_paths=cfg["max_paths"])
    q = Query(lib, L, ctx, torch, w, "precision")
    pipe = q.pipeline(1, 1, flush)
    e2e_ms, res = q.e2e(2)
    ks = pipe["kernel_ms"]
    N, E = w["N"], pipe["E"]
    return {"config": {"workload": "large32000", "N": N, "obstacles": int(q.obs.shape[0]),
                       "hsmc_particles": w["P"], "mc_particles": w["num_mc"],
                       "waypoints_per_edge": w["num_disc"] + 1, "noise_mult": 5e-3, "cp_target": 0.005,
                       "eta": 2, "bvp": "precision", "edges": E, "expansions": pipe["M"]},
            "value": pipe["units"] / (pipe["step_ms"][0] / 1e3), "unit": UNIT,
            "ms_per_step": pipe["step_ms"][0],
            "kernel_ms": {k: round(v, 3) for k, v in ks.items()},
            "edges_per_s": {"bvp": N * (N - 1) / (ks["bvp_pairs"] / 1e3), "cc": E / (ks["free_edges"] / 1e3),
                            "hsmc": pipe["M"] / (ks["hsmc"] / 1e3) if ks.get("hsmc") else None},
            "plan_ms": statistics.median(e2e_ms),
            "plan_stage_ms": {"roadmap": res.ms_roadmap, "online": res.ms_online,
                              "explore": res.ms_explore, "search": res.ms_search},
            "e2e": {"value": pipe["units"] * len(e2e_ms) / (sum(e2e_ms) / 1e3), "unit": UNIT,
                    "h2d_bytes_per_step": int(res.h2d_bytes), "d2h_bytes_per_step": int(res.d2h_bytes)},
            "solution": {"success": int(res.success), "cp": res.soln_cp, "cost": res.soln_cost,
                         "paths": res.num_paths, "iterations": res.iterations}}


def mode_record(lib, L, ctx, torch, w, mode, args, flush, batch, steps=None, warmup=None):
    """The same workload in one of the bit-exact arithmetics: the device
    pipeline's edges/s, the plan latency (e2e edges/s) and, with batch > 0,
    batched vs plain queries/s."""
    steps = steps or args.steps
    warmup = warmup or args.warmup
    q = Query(lib, L, ctx, torch, w, mode)
    pipe = q.pipeline(steps, warmup, flush)
    e2e_ms, res = q.e2e(steps)
    ks = pipe["kernel_ms"]
    rec = {"bvp": mode, "bit_exact_against": BIT_EXACT_AGAINST[mode],
           "value": pipe["units"] * steps / (sum(pipe["step_ms"]) / 1e3), "unit": UNIT,
           "ms_per_step": sum(pipe["step_ms"]) / steps,
           "kernel_ms": {k: round(v, 4) for k, v in ks.items()},
           "plan_ms": statistics.median(e2e_ms),
           "e2e": {"value": pipe["units"] * len(e2e_ms) / (sum(e2e_ms) / 1e3), "unit": UNIT,
                   "h2d_bytes_per_step": int(res.h2d_bytes), "d2h_bytes_per_step": int(res.d2h_bytes)},
           "edges": pipe["E"], "expansions": pipe["M"],
           "solution": {"success": int(res.success), "cp": res.soln_cp, "cost": res.soln_cost,
                        "paths": res.num_paths}}
    if batch > 0:
        rec["queries_per_s"] = measure_queries(args, lib, L, ctx, mode)
    return rec


# Binary64 flops per ordered pair of the 2pBVP kernels (a fused multiply-add
# counts two), counted from the kernels' source and confirmed by ncu's
# instruction mix on this workload (per pair: 10 DFMA, 6 DADD, 2 DMUL):
#  precision: coefficient assembly in float-float on the FP32 pipe; binary64
#             only for the six coefficients (hi + lo), the Newton residual
#             Q(x) and step, and the cost at the root;
#  parity:    40 per binary64 cost evaluation (23 additions, 15
#             multiplications, one division, one scaling) x 23 evaluations
#             per pair (the mean over 20,000 pairs of this workload's
#             samples) + 20 for the pair's hoisted coefficients, the kernel's
#             work before its evaluations moved to float-float; now most
#             evaluations are binary32 arithmetic and the kernel is rated by
#             instruction issue (below), this figure kept as the
#             arithmetic a binary64 evaluation would do.
# the reference's GPU kernel evaluates the same binary64 expression as its
# CPU build (one cost: 40 operations; topt: 23 cost pairs less the shared ones)
BVP_FP64_FLOPS_PER_PAIR = {"precision": 28.0, "parity": 40.0 * 23 + 20.0,
                           "parity_gpu": 40.0 * 23 + 20.0}
# ncu smsp__inst_executed.sum of one parity pair-kernel launch at N = 1000
# (999,000 pairs), per pair; the same for the reference-GPU arithmetic's
# pair kernel
BVP_PARITY_WARP_INST_PER_PAIR = 395849939 / 999000
BVP_REFGPU_WARP_INST_PER_PAIR = 416223561 / 999000
# The precision kernel is bound by instruction issue, not by one pipe: warp
# instructions executed per pair on this workload (ncu smsp__inst_executed.sum
# over one launch of the N = 4000 workload's pair kernel, the one marking the
# rn superset, / its pairs), and DRAM bytes per launch
# (dram__bytes_read.sum + dram__bytes_write.sum of the same launch).
BVP_PRECISION_WARP_INST_PER_PAIR = 703111934 / 15996000
# ncu smsp__inst_executed.sum on indoor4000: the edge check (pair-queue
# kernel) at block size 128, the autotuner's choice there (64 and 256 differ
# by under 0.3 %), per edge; the waypoint kernel (thread per edge, block size
# 128), per waypoint
FREE_EDGES_WARP_INST_PER_EDGE_N4000 = 88103877 / 799800
DISCRETIZE_WARP_INST_PER_WAYPOINT = 18258294 / (799800 * 9)
BVP_PRECISION_DRAM_BYTES_N4000 = 0.16e6 + 69.18e6
SMSP_PER_SM = 4
NUM_SMS = 152


def roofline(dom, ks, N, E, M, W, H, P, mode, fp64_tflops, sm_mhz):
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    src = "measured" if "hbm_gbs" in peaks else "fallback"
    # algorithmic HBM bytes per launch of the memory-bound kernels
    algo = {
        "discretize": 16.0 * E + 24.0 * W * E,                # edge in, waypoints out
        "free_edges": 24.0 * W * E + E,                       # waypoints in, mask out
        # per new path: edge and parent ids, time, parent mask in, mask out, the edge's waypoints
        "hsmc": M * (8 + 4 + 2 * 4 * ((P + 31) // 32) + 24.0 * W),
    }
    table = {}
    for k, b in algo.items():
        if k in ks and ks[k] > 0:
            a = b / (ks[k] / 1e3) / 1e9
            table[k] = {"bound": "hbm", "achieved_gbs": round(a, 1), "frac": round(a / hbm, 4)}
    # rn and the edges no longer stream the cost array (the pair kernel marks
    # the superset): the stage is bound by its launches' latency
    if "rn_edges" in ks:
        table["rn_edges"] = {"bound": "latency", "ms": round(ks["rn_edges"] + ks.get("rn_bracket", 0.0), 4),
                             "note": "bracket launch + cooperative finishing kernel + the call's read-back"}
    pairs = N * (N - 1)
    t_bvp = ks["bvp_pairs"] / 1e3
    fp64 = BVP_FP64_FLOPS_PER_PAIR[mode] * pairs / t_bvp / 1e12
    table["bvp_pairs_fp64"] = {"bound": "fp64", "achieved_tflops": round(fp64, 4),
                               "frac": round(fp64 / fp64_tflops, 4),
                               "flops_per_pair": BVP_FP64_FLOPS_PER_PAIR[mode]}
    issue_peak = NUM_SMS * SMSP_PER_SM * sm_mhz * 1e6 / 1e9  # warp instructions, G/s
    if mode == "precision" and N == 4000:
        issue = BVP_PRECISION_WARP_INST_PER_PAIR * pairs / t_bvp / 1e9
        table["bvp_pairs"] = {"bound": "issue", "achieved_ginst": round(issue, 1),
                              "frac": round(issue / issue_peak, 4)}
    inst_pp = {"parity": BVP_PARITY_WARP_INST_PER_PAIR,
               "parity_gpu": BVP_REFGPU_WARP_INST_PER_PAIR}.get(mode)
    if inst_pp is not None:
        issue = inst_pp * pairs / t_bvp / 1e9
        table["bvp_pairs"] = {"bound": "issue", "achieved_ginst": round(issue, 1),
                              "frac": round(issue / issue_peak, 4),
                              "inst_per_pair": round(inst_pp, 1)}
    if mode == "precision" and N == 4000:
        for k, units, per in (("free_edges", E, FREE_EDGES_WARP_INST_PER_EDGE_N4000),
                              ("discretize", E * W, DISCRETIZE_WARP_INST_PER_WAYPOINT)):
            if ks.get(k, 0) > 0:
                g = per * units / (ks[k] / 1e3) / 1e9
                table[k + "_issue"] = {"bound": "issue", "achieved_ginst": round(g, 1),
                                       "frac": round(g / issue_peak, 4),
                                       "warp_inst_per_unit": round(per, 2)}
    if dom == "bvp_pairs" and mode == "precision" and N == 4000:
        return {"kernel": dom, "bound": "issue", "achieved": issue, "peak": issue_peak,
                "unit": "G warp-instructions/s", "frac": issue / issue_peak,
                "traffic": BVP_PRECISION_DRAM_BYTES_N4000,
                "peak_source": "152 SMs x 4 schedulers x 1 warp instruction per clock at the "
                               "SM clock sampled during the timed region (%.0f MHz)" % sm_mhz,
                "inst_per_pair": BVP_PRECISION_WARP_INST_PER_PAIR,
                "fp64_pipe": table["bvp_pairs_fp64"], "all": table}
    if dom == "bvp_pairs" and inst_pp is not None:
        return {"kernel": dom, "bound": "issue", "achieved": issue, "peak": issue_peak,
                "unit": "G warp-instructions/s", "frac": issue / issue_peak, "traffic": None,
                "peak_source": "152 SMs x 4 schedulers x 1 warp instruction per clock at the "
                               "SM clock sampled during the timed region (%.0f MHz)" % sm_mhz,
                "inst_per_pair": inst_pp, "all": table}
    if dom == "bvp_pairs":
        return {"kernel": dom, "bound": "fp64", "achieved": fp64, "peak": fp64_tflops,
                "unit": "TFLOP/s", "frac": fp64 / fp64_tflops, "traffic": None,
                "peak_source": "measured live (bench.py's DFMA probe: FP64 FMA pipe; the "
                               "driver's peak file holds only HBM and bf16 figures)",
                "flops_per_pair": BVP_FP64_FLOPS_PER_PAIR[mode], "all": table}
    t = ks[dom] / 1e3
    ach = algo.get(dom, 0.0) / t / 1e9
    return {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
            "frac": ach / hbm, "traffic": None, "peak_source": src, "all": table}


def run_reference(args):
    """The reference's CPU path of this workload (C oracle), one whole query
    per step; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    vals, secs = [], []
    det = None
    for k in range(args.warmup + args.steps):
        v, dt, det = cpu_query(args, 0)
        if k >= args.warmup:
            vals.append(v)
            secs.append(dt)
    v = statistics.median(vals)
    w = workload(args, 0)
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "impl": "reference", "data": "synthetic (seeded indoor map, Halton samples)",
            "config": {"workload": WORKLOAD, "N": w["N"], "obstacles": int(w["obstacles"].shape[0]),
                       "hsmc_particles": w["P"], "waypoints_per_edge": w["num_disc"] + 1,
                       "noise_mult": 2e-3, "cp_target": 0.01, "eta": 2,
                       "bvp": "reference finite-difference bisection"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": det["cores"], "kind": "port",
                             "sample": det["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
