"""Compares the library's parity-mode kernels with the reference's own GPU
kernels on the same inputs, stage by stage, and times both.

Test infrastructure, run on the GPU machine:
    bash oracle/refgpu/build_ref_gpu.sh && python oracle/refgpu/compare_ref_gpu.py OUTDIR

The reference side is oracle/_ref/ref_gpu_N<N> (ref_gpu_main.cu: the
reference's kernels compiled by nvcc as its Makefile compiles them).  The
library's parity arithmetic is the reference's algorithm with every operation
rounded once and no multiply-add contraction; nvcc contracts the reference's
device code and evaluates its pow() calls with CUDA's binary64 pow.  This
script counts where that changes a result, for the two benchmark problems:

  cfg0  N = 1000, 10 random boxes, 10 waypoints per edge, 128 particles
  cfg1  N = 4000, indoor map (40 boxes), 9 waypoints per edge, 1024 particles

Stages (each compared on identical inputs; the downstream stages take the
library's parity roadmap and waypoints, which equal the reference's host
code bit for bit, as inputs to both sides):
  bvp          copts/topts of every ordered pair (fillCoptsTopts)
  rn, edges    the 5 % cost quantile and the edge set each side's costs give
  sample_free  sampleFree
  free_edges   freeEdges
  halfspaces   setupAsBs + cacheHalfspaces (as, bs, counts)
  hsmc         propagateValidParticles + calculateCP_HSMC over a wavefront of
               new paths on random free edges, random parent masks and times
  mccp         MCCP over dense polyline paths (at the problem's noise
               multiplier and at 0.3, where particles do hit boxes)

Writes OUTDIR/compare.json (counts and times), OUTDIR/refgpu_bvp_N<N>.npz
(the reference GPU's pair times and costs: SHA-256 of the whole arrays, a
strided subset, rn and the edge count; committed as tests/golden/) and
OUTDIR/refgpu_bvp_diff_N<N>.npz (the pairs where the reference GPU differs
from the parity arithmetic, from which tests/golden/make_golden.py rebuilds
the whole arrays).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

STRIDE = 97


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ulp_diff(a, b):
    """|a - b| in units in the last place of binary32 (ordered-integer distance)."""
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


def mismatch(a, b):
    """Elements whose bytes differ (1-byte flags or 4-byte words)."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.size == b.size and a.dtype.itemsize == b.dtype.itemsize
    view = np.uint8 if a.dtype.itemsize == 1 else np.uint32
    return int(np.count_nonzero(a.view(view) != b.view(view)))


class Ref:
    def __init__(self, N, tmp):
        self.exe = os.path.join(ROOT, "oracle", "_ref", "ref_gpu_N%d" % N)
        if not os.path.exists(self.exe):
            raise SystemExit("missing %s (run oracle/refgpu/build_ref_gpu.sh)" % self.exe)
        self.tmp = tmp
        self.k = 0

    def file(self, arr=None, name=None):
        self.k += 1
        p = os.path.join(self.tmp, "%s_%d.bin" % (name or "f", self.k))
        if arr is not None:
            np.ascontiguousarray(arr).tofile(p)
        return p

    def run(self, *args):
        r = subprocess.run([self.exe] + [str(a) for a in args], capture_output=True, text=True,
                           timeout=1200)
        if r.returncode != 0:
            raise RuntimeError("ref_gpu %s failed (%d): %s %s" % (args[0], r.returncode, r.stdout, r.stderr))
        times = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
        return times


def med(times):
    if not times:
        return None
    ms = times[0]["ms"]
    return float(np.median(ms[1:] if len(ms) > 1 else ms))


def polyline_paths(rng, k, lo=20, hi=100):
    """k dense paths of lo..hi states: straight runs between random points in
    [0,1]^3 at most 0.02 apart (velocities zero; MCCP reads positions only)."""
    rows, lens = [], []
    for _ in range(k):
        T = int(rng.integers(lo, hi + 1))
        pts = rng.uniform(0.05, 0.95, (4, 3))
        s = np.linspace(0, 3, T)
        seg = np.minimum(s.astype(int), 2)
        f = (s - seg)[:, None]
        pos = pts[seg] * (1 - f) + pts[seg + 1] * f
        X = np.zeros((T, 6), np.float32)
        X[:, :3] = pos
        rows.append(X)
        lens.append(T)
    return np.concatenate(rows), np.asarray(lens, np.int32)


def compare(cfg_name, out_dir, torch, lib, L, ctx, ref):
    from oracle import pyoracle as O
    from pump_gb300 import workloads
    cfg = workloads.CONFIGS[cfg_name]
    N, W, P = cfg["N"], cfg["num_disc"] + 1, cfg["num_hsmc"]
    obs = np.ascontiguousarray(cfg["obstacles"](0), np.float32)
    nobs = obs.shape[0]
    om = np.float32(cfg["offset_mult"])
    maxHS = min(nobs, 5)
    maxd2 = np.float32(0.1 * np.float64(om) ** 2)
    sh = torch.cuda.current_stream().cuda_stream
    rng = np.random.Generator(np.random.MT19937(4242 + N))

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a).copy()).cuda()

    def empty(n, dt):
        return torch.empty(int(max(n, 1)), dtype=dt, device="cuda")

    def ev_ms(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    res = {"N": N, "obstacles": nobs, "W": W, "P": P, "offset_mult": float(om)}
    samples = O.halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    f_s = ref.file(samples, "samples")

    # ---- pair BVP
    f_c, f_t = ref.file(name="copts"), ref.file(name="topts")
    t_ref = ref.run("bvp", f_s, f_c, f_t, 2)
    rc = np.fromfile(f_c, np.float32)
    rt = np.fromfile(f_t, np.float32)
    d_s = dev(samples)
    npairs = N * (N - 1)
    d_c, d_t = empty(npairs, torch.float32), empty(npairs, torch.float32)
    t_ours = ev_ms(lambda: lib.check(L.pump_bvp_pairs(d_s.data_ptr(), N, 5.0, 0, d_c.data_ptr(),
                                                      d_t.data_ptr(), sh)), 2)
    oc, ot = d_c.cpu().numpy(), d_t.cpu().numpy()
    t_prec = ev_ms(lambda: lib.check(L.pump_bvp_pairs(d_s.data_ptr(), N, 5.0, 1, d_c.data_ptr(),
                                                      d_t.data_ptr(), sh)), 3)
    mc = oc.view(np.uint32) != rc.view(np.uint32)
    mt = ot.view(np.uint32) != rt.view(np.uint32)
    rel_c = np.abs(oc.astype(np.float64) - rc) / np.maximum(np.abs(rc.astype(np.float64)), 1e-30)
    res["bvp"] = {"pairs": npairs, "copt_mismatch": int(mc.sum()), "topt_mismatch": int(mt.sum()),
                  "pairs_either": int((mc | mt).sum()),
                  "copt_max_ulp": int(ulp_diff(oc, rc).max()), "topt_max_ulp": int(ulp_diff(ot, rt).max()),
                  "copt_max_rel": float(rel_c.max()),
                  "copt_mismatch_same_topt": int((mc & ~mt).sum()),
                  "ms_reference_gpu": med(t_ref), "ms_parity": t_ours, "ms_precision": t_prec}
    # ---- rn and edges from each side's costs
    k = int(np.float32((N - 1) * N) * np.float32(0.05))
    rn_ref = np.partition(rc, k)[k]
    rn_our = np.partition(oc, k)[k]
    e_ref = np.flatnonzero(rc < rn_ref)
    e_our = np.flatnonzero(oc < rn_our)
    res["rn_edges"] = {"k": k, "rn_reference_gpu": float(rn_ref), "rn_parity": float(rn_our),
                       "rn_equal": bool(rn_ref.view(np.uint32) == rn_our.view(np.uint32)),
                       "edges_reference_gpu": int(e_ref.size), "edges_parity": int(e_our.size),
                       "edges_only_in_reference": int(np.setdiff1d(e_ref, e_our).size),
                       "edges_only_in_parity": int(np.setdiff1d(e_our, e_ref).size),
                       "edge_topt_mismatch": int(np.count_nonzero(
                           rt[np.intersect1d(e_ref, e_our)].view(np.uint32)
                           != ot[np.intersect1d(e_ref, e_our)].view(np.uint32)))}
    i_idx = (np.arange(0, npairs, STRIDE, dtype=np.int64))
    # the pairs where the reference GPU differs from the parity arithmetic (which
    # the CPU build of the reference reproduces): with them the reference GPU's
    # whole arrays can be rebuilt on a machine without a GPU
    diff = np.flatnonzero(mc | mt).astype(np.int64)
    np.savez_compressed(os.path.join(out_dir, "refgpu_bvp_diff_N%d.npz" % N), idx=diff,
                        copts=rc[diff], topts=rt[diff], copts_sha=sha(rc), topts_sha=sha(rt))
    np.savez_compressed(os.path.join(out_dir, "refgpu_bvp_N%d.npz" % N),
                        copts_sha=sha(rc), topts_sha=sha(rt), stride=STRIDE,
                        copts_strided=rc[i_idx], topts_strided=rt[i_idx],
                        rn=np.float32(rn_ref), num_edges=np.int64(e_ref.size), k=np.int64(k))

    # ---- common downstream inputs: the parity roadmap and waypoints
    lib.check(L.pump_bvp_pairs(d_s.data_ptr(), N, 5.0, 0, d_c.data_ptr(), d_t.data_ptr(), sh))
    cap = k
    d_src, d_dst = empty(cap, torch.int32), empty(cap, torch.int32)
    d_ce, d_te = empty(cap, torch.float32), empty(cap, torch.float32)
    d_go = empty(N + 1, torch.int32)
    rn = C.c_float(0)
    Ec = C.c_longlong(0)
    lib.check(L.pump_roadmap_edges(ctx.handle, d_c.data_ptr(), d_t.data_ptr(), N, k, cap, d_src.data_ptr(),
                                   d_dst.data_ptr(), d_ce.data_ptr(), d_te.data_ptr(), d_go.data_ptr(),
                                   C.byref(rn), C.byref(Ec), sh))
    E = int(Ec.value)
    d_disc = empty(E * W * 6, torch.float32)
    lib.check(L.pump_discretize_edges(d_s.data_ptr(), d_src.data_ptr(), d_dst.data_ptr(), d_te.data_ptr(),
                                      E, W - 1, 0, d_disc.data_ptr(), sh))
    torch.cuda.synchronize()
    disc = d_disc.cpu().numpy()[: E * W * 6]
    topt_e = d_te.cpu().numpy()[:E]
    f_obs, f_disc = ref.file(obs, "obs"), ref.file(disc, "disc")
    d_obs = dev(obs)

    # ---- sample free
    f_sf = ref.file(name="sfree")
    ref.run("sample_free", f_obs, nobs, f_s, f_sf)
    d_fs = empty(N, torch.uint8)
    lib.check(L.pump_sample_free(d_obs.data_ptr(), nobs, d_s.data_ptr(), N, d_fs.data_ptr(), sh))
    res["sample_free"] = {"samples": N, "mismatch": mismatch(np.fromfile(f_sf, np.uint8),
                                                             d_fs.cpu().numpy()[:N])}
    # ---- edge check
    f_fe = ref.file(name="efree")
    t_ref = ref.run("free_edges", f_obs, nobs, f_disc, E, W - 1, f_fe, 5)
    d_fe = empty(E, torch.uint8)
    t_ours = ev_ms(lambda: lib.check(L.pump_free_edges(d_obs.data_ptr(), nobs, d_disc.data_ptr(), E, W - 1,
                                                       d_fe.data_ptr(), sh)), 5)
    fe_ref = np.fromfile(f_fe, np.uint8)
    fe_our = d_fe.cpu().numpy()[:E]
    res["free_edges"] = {"edges": E, "free_reference_gpu": int(fe_ref.sum()), "mismatch": mismatch(fe_ref, fe_our),
                         "ms_reference_gpu": med(t_ref), "ms_parity": t_ours}
    # ---- half-spaces
    hs = E * W * maxHS
    f_as, f_bs, f_cnt = ref.file(name="as"), ref.file(name="bs"), ref.file(name="cnt")
    f_fr = ref.file(fe_our, "isfree")
    t_ref = ref.run("halfspaces", f_obs, nobs, f_disc, f_fr, E, W, maxHS, repr(float(maxd2)),
                    f_as, f_bs, f_cnt, 3)
    r_as, r_bs = np.fromfile(f_as, np.float32), np.fromfile(f_bs, np.float32)
    r_cnt = np.fromfile(f_cnt, np.int32)
    d_as, d_bs, d_cnt = empty(3 * hs, torch.float32), empty(hs, torch.float32), empty(E * W, torch.int32)
    t_ours = ev_ms(lambda: lib.check(L.pump_cache_halfspaces(
        d_obs.data_ptr(), nobs, d_disc.data_ptr(), d_fe.data_ptr(), E, W, maxHS, float(maxd2),
        d_as.data_ptr(), d_bs.data_ptr(), d_cnt.data_ptr(), sh)), 3)
    o_as, o_bs, o_cnt = d_as.cpu().numpy()[: 3 * hs], d_bs.cpu().numpy()[:hs], d_cnt.cpu().numpy()[: E * W]
    res["halfspaces"] = {"waypoints": E * W, "stored_reference_gpu": int(r_cnt.sum()),
                         "count_mismatch": mismatch(r_cnt, o_cnt), "a_mismatch": mismatch(r_as, o_as),
                         "b_mismatch": mismatch(r_bs, o_bs),
                         "a_max_ulp": int(ulp_diff(r_as, o_as).max()), "b_max_ulp": int(ulp_diff(r_bs, o_bs).max()),
                         "ms_reference_gpu": med(t_ref), "ms_parity": t_ours}
    # ---- HSMC over a synthetic wavefront on free edges (the reference's half-spaces as input)
    free_idx = np.flatnonzero(fe_our)
    M = 4000 if N <= 1000 else 30000
    base = 256
    edge = rng.choice(free_idx, M).astype(np.int32)
    prev = rng.integers(0, base, M).astype(np.int32)
    times = rng.uniform(0.0, 8.0, base).astype(np.float32)
    assert float((times[prev] + topt_e[edge]).max()) < 0.05 * 399
    valid = (rng.random((base, P)) < 0.97).astype(np.uint8)
    f_vo, f_cp = ref.file(name="vout"), ref.file(name="cp")
    t_ref = ref.run("hsmc", ref.file(edge, "edge"), ref.file(prev, "prev"), M, base, f_as, f_bs, E, W, maxHS,
                    ref.file(times, "times"), ref.file(topt_e, "topte"), ref.file(valid, "valid"), P,
                    repr(float(om)), f_vo, f_cp, 5)
    r_valid = np.fromfile(f_vo, np.uint8).reshape(M, P)
    r_cp = np.fromfile(f_cp, np.float32)
    words = (P + 31) // 32
    packed = np.zeros((base + M, words), np.uint32)
    bits = np.packbits(valid, axis=1, bitorder="little")
    pad = np.zeros((base, words * 4), np.uint8)
    pad[:, : bits.shape[1]] = bits
    packed[:base] = pad.view(np.uint32).reshape(base, words)
    d_valid = dev(packed.reshape(-1).view(np.int32))
    d_tab = empty(400 * 2048 * 3, torch.float32)
    lib.check(L.pump_particle_tables(C.c_uint64(0x9E3779B97F4A7C15), 2048, 400, d_tab.data_ptr(), None, sh))
    d_edge, d_prev, d_times, d_te2 = dev(edge), dev(prev), dev(times), dev(topt_e)
    d_ras, d_rbs = dev(r_as), dev(r_bs)
    d_cp = empty(base + M, torch.float32)
    d_err = empty(1, torch.int32).zero_()
    t_ours = ev_ms(lambda: lib.check(L.pump_hsmc_propagate(
        M, W, d_edge.data_ptr(), d_prev.data_ptr(), E, base, d_ras.data_ptr(), d_rbs.data_ptr(), maxHS,
        d_times.data_ptr(), d_te2.data_ptr(), C.c_float(0.05), d_tab.data_ptr(), 2048, 400, C.c_float(om),
        d_valid.data_ptr(), P, d_cp.data_ptr(), d_err.data_ptr(), None, sh)), 5)
    o_words = d_valid.cpu().numpy().view(np.uint32).reshape(base + M, words)[base:]
    o_valid = np.unpackbits(o_words.view(np.uint8).reshape(M, -1), axis=1, bitorder="little")[:, :P]
    o_cp = d_cp.cpu().numpy()[base: base + M]
    res["hsmc"] = {"new_paths": M, "particles": P, "particle_mismatch": int((o_valid != r_valid).sum()),
                   "paths_with_mismatch": int((o_valid != r_valid).any(axis=1).sum()),
                   "cp_mismatch": mismatch(o_cp, r_cp), "device_error": int(d_err.cpu().item()),
                   "invalid_particles_reference_gpu": int((r_valid == 0).sum()),
                   "ms_reference_gpu": med(t_ref), "ms_parity": t_ours}
    # ---- MC CP over dense paths
    paths, lens = polyline_paths(rng, 64)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int32)
    d_paths, d_offs, d_lens = dev(paths), dev(offs), dev(lens)
    d_hits, d_mcp = empty(64, torch.int32), empty(64, torch.float32)
    res["mccp"] = []
    for mult in (float(om), 0.3):
        f_h = ref.file(name="hits")
        t_ref = ref.run("mccp", f_obs, nobs, ref.file(paths, "paths"), ref.file(lens, "lens"), 64, repr(mult),
                        f_h, 3)
        r_hits = np.fromfile(f_h, np.int32)
        t_ours = ev_ms(lambda: lib.check(L.pump_mc_cp(
            d_paths.data_ptr(), d_offs.data_ptr(), d_lens.data_ptr(), 64, d_tab.data_ptr(), 2048, 400,
            C.c_float(mult), d_obs.data_ptr(), nobs, d_hits.data_ptr(), d_mcp.data_ptr(), None, sh)), 3)
        o_hits = d_hits.cpu().numpy()[:64]
        res["mccp"].append({"paths": 64, "offset_mult": mult, "hits_reference_gpu": int(r_hits.sum()),
                            "paths_with_hit_mismatch": int((o_hits != r_hits).sum()),
                            "max_hit_diff": int(np.abs(o_hits - r_hits).max()),
                            "ms_reference_gpu_64_launches": med(t_ref), "ms_parity_one_launch": t_ours})
    return res


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.getcwd(), "refgpu_compare")
    os.makedirs(out_dir, exist_ok=True)
    import torch
    from pump_gb300 import lib
    from pump_gb300.build import build
    build()
    L = lib.load()
    torch.cuda.set_device(0)
    ctx = lib.Context(0)
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name in (sys.argv[2:] or ["cfg0", "cfg1"]):
            N = __import__("pump_gb300.workloads", fromlist=["CONFIGS"]).CONFIGS[name]["N"]
            out[name] = compare(name, out_dir, torch, lib, L, ctx, Ref(N, tmp))
            print(json.dumps({name: out[name]}), flush=True)
    ctx.close()
    with open(os.path.join(out_dir, "compare.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
