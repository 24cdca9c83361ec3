"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs the reference PUMP program built for the CPU by oracle/build_ref.sh
(oracle/_ref/pump_ref_N<N>, the reference's own main() and kernels) on the
problems below and records what it produced: its stage outputs (dumped by
the stand-in runtime at every kernel launch), the exploration trace, the
solution it prints and the path.txt it writes.  Large arrays are stored as
a strided subset plus a SHA-256 of the whole array.

Run from the repository root (needs the reference sources and gcc/nvcc):
    bash oracle/build_ref.sh && python tests/golden/make_golden.py
and for the N = 4000 benchmark problem (1024 HSMC particles):
    PUMPREF_NUMS=4000:1024 bash oracle/build_ref.sh && python tests/golden/make_golden.py indoor4000
and the same problems with the pair BVPs of the reference's own GPU kernel
(the diff files written by oracle/refgpu/compare_ref_gpu.py on the GPU):
    python tests/golden/make_golden.py refgpu DIFF_DIR
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from pump_gb300 import workloads  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(ROOT, "oracle", "_ref")
REFERENCE_DIR = os.environ.get("PUMP_REFERENCE_DIR",
                               os.path.join(os.path.dirname(ROOT), "reference"))
REFERENCE_INPUT = os.path.join(REFERENCE_DIR, "input.txt")
STRIDE = 97


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_ref(N, input_path, cp, eta, dump, P=128, bvp_from=None):
    tag = "N%d" % N if P == 128 else "N%d_P%d" % (N, P)
    env = dict(os.environ)
    if bvp_from:
        env["PUMPREF_BVP_FROM"] = bvp_from
    env["PUMPREF_KERNEL_LIB"] = os.path.join(REF, "libpumpref_cpu_%s.so" % tag)
    env["PUMPREF_DUMP"] = dump
    exe = os.path.join(REF, "pump_ref_%s" % tag)
    r = subprocess.run([exe, input_path, str(cp), str(eta)], cwd=dump, env=env,
                       capture_output=True, text=True, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return r.stdout


def parse_wavefront(path):
    wf = np.fromfile(path, np.int32) if os.path.exists(path) else np.zeros(0, np.int32)
    i, sizes, trace = 0, [], []
    while i < wf.size:
        _, n, _ = wf[i:i + 3]
        prev, edge = wf[i + 3:i + 3 + n], wf[i + 3 + n:i + 3 + 2 * n]
        trace.append(np.stack([prev, edge], 1).reshape(-1))
        sizes.append(int(n))
        i += 3 + 2 * n
    tr = np.concatenate(trace) if trace else np.zeros(0, np.int32)
    return np.asarray(sizes, np.int32), tr.astype(np.int32)


def read_problem(path):
    """Fields of a reference input file, in the order mainPUMP.cu:160-221 reads them."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.strtof.restype = ctypes.c_float
    libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    fields = open(path).read().split(",")
    # decimal -> binary32 directly, as the reference's stringstream >> float does
    vals = [libc.strtof(v.strip().encode(), None) if v.strip() else 0.0 for v in fields[:26]]
    nobs = int(fields[25].strip())
    vals += [libc.strtof(v.strip().encode(), None) for v in fields[26:26 + 12 * nobs]]
    init, goal, lo, hi = (np.float32(vals[6 * i:6 * i + 6]) for i in range(4))
    om = np.float32(vals[24])
    obs = np.float32(vals[26:26 + 12 * nobs]).reshape(nobs, 12)
    return dict(init=init, goal=goal, lo=lo, hi=hi, offset_mult=om, obstacles=obs)


def case(name, N, input_path, cp, eta, full, roadmap=True, P=128, stride=STRIDE, bvp_from=None):
    """One fixture.  P: the reference build's HSMC particle count
    (oracle/build_ref.sh entry N:P); stride: of the strided subsets;
    bvp_from: a directory with the pair arrays of the reference's GPU kernel
    (copts.f32, topts.f32) that the run uses instead of computing them."""
    with tempfile.TemporaryDirectory() as d:
        out = run_ref(N, input_path, cp, eta, d, P, bvp_from)
        f = lambda n, t: np.fromfile(os.path.join(d, n), t)  # noqa: E731
        g = {"prob_" + k: np.asarray(v) for k, v in read_problem(input_path).items()}
        g["N"], g["cp_target"], g["cp_factor"] = np.array(N), np.float32(cp), np.float32(eta)
        g["hsmc_particles"], g["stride"] = np.array(P), np.array(stride)
        samples = f("samples.f32", np.float32).reshape(N, 6)
        copts, topts = f("copts.f32", np.float32), f("topts.f32", np.float32)
        disc = f("discMotions.f32", np.float32)
        free_e, free_s = f("isFreeEdges.u8", np.uint8), f("isFreeSamples.u8", np.uint8)
        a, b = f("as.f32", np.float32), f("bs.f32", np.float32)
        g["samples"] = samples
        for key, arr in (("copts", copts), ("topts", topts), ("disc", disc), ("as", a), ("bs", b)):
            g[key + "_sha"] = np.array(sha(arr))
            if roadmap or key in ("as", "bs"):
                g[key + "_sub"] = arr if full else arr[::stride].copy()
        g["free_edges_bits"] = np.packbits(free_e)
        g["free_edges_n"] = np.array(free_e.size)
        g["free_samples"] = free_s
        sizes, trace = parse_wavefront(os.path.join(d, "wavefront.i32"))
        g["wavefront_sizes"] = sizes
        g["wavefront_trace"] = trace
        g["pathcp"] = f("pathcp.f32", np.float32) if os.path.exists(os.path.join(d, "pathcp.f32")) \
            else np.zeros(0, np.float32)
        m = re.search(r"rnIdx is (\d+)", out)
        g["rn_idx"] = np.array(int(m.group(1)))
        m = re.search(r"cutoff is ([0-9.eE+-]+) at", out)
        g["rn_printed"] = np.array(float(m.group(1)))
        m = re.search(r"number of goal paths found = (\d+) with a total number of paths = (\d+) of (\d+)", out)
        g["goal_paths"], g["num_paths"], g["num_considered"] = (np.array(int(x)) for x in m.groups())
        success = "SUCCESS" in out
        g["success"] = np.array(int(success))
        if success:
            m = re.search(r"Solution path = (\d+) with cp = ([0-9.eE+-]+) and cost = ([0-9.eE+-]+)", out)
            g["soln_idx"] = np.array(int(m.group(1)))
            g["soln_cp_printed"] = np.array(float(m.group(2)))
            g["soln_cost_printed"] = np.array(float(m.group(3)))
            nodes = {}
            for mm in re.finditer(r"Path (\d+): cost = [^,]+, time = [^,]+, cp = ([0-9.eE+-]+) vs "
                                  r"[0-9.eE+-]+ est, nodes = \[([0-9, ]+)\]", out):
                nodes[int(mm.group(1))] = [int(x) for x in mm.group(3).split(",")]
            g["soln_nodes"] = np.asarray(nodes[int(g["soln_idx"])][::-1], np.int32)
            g["path_txt"] = np.array(open(os.path.join(d, "path.txt")).read())
        ctrl = os.path.join(d, "discretizedPath.txt")
        if os.path.exists(ctrl):
            g["ctrl_txt"] = np.array(open(ctrl).read())
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **g)
        meta = {k: (v.tolist() if v.size < 8 else "array%s" % (v.shape,)) for k, v in g.items()}
        print(name, json.dumps(meta)[:400])


def gpu_pairs(N, diff_path, out_dir):
    """The pair arrays of the reference's own fillCoptsTopts run on the GPU
    (oracle/refgpu/compare_ref_gpu.py): the parity arithmetic's arrays (the
    CPU build of the reference computes them; the oracle reproduces them bit
    for bit) with the pairs listed in diff_path replaced, checked against the
    SHA-256 of the GPU's whole arrays; written to out_dir/copts.f32 and
    topts.f32."""
    from oracle import pyoracle as O
    s = O.halton_samples(N, workloads.INIT, workloads.GOAL, workloads.LO, workloads.HI)
    c, t = O.bvp_pairs(s)
    d = np.load(diff_path)
    c[d["idx"]] = d["copts"]
    t[d["idx"]] = d["topts"]
    assert sha(c) == str(d["copts_sha"]) and sha(t) == str(d["topts_sha"]), "diff does not rebuild the GPU arrays"
    c.tofile(os.path.join(out_dir, "copts.f32"))
    t.tofile(os.path.join(out_dir, "topts.f32"))
    return out_dir


def main():
    only = sys.argv[1:]
    tmp = tempfile.mkdtemp()
    if only and only[0] == "refgpu":
        # whole queries of the reference program whose pair BVPs are those of its
        # own GPU kernel: python tests/golden/make_golden.py refgpu DIFF_DIR, where
        # DIFF_DIR holds refgpu_bvp_diff_N1000.npz and refgpu_bvp_diff_N4000.npz
        # written by oracle/refgpu/compare_ref_gpu.py on the GPU machine
        diff_dir = only[1]
        g1000 = gpu_pairs(1000, os.path.join(diff_dir, "refgpu_bvp_diff_N1000.npz"),
                          tempfile.mkdtemp(dir=tmp))
        obs = workloads.random_boxes(10, 0)
        for om, tag in ((1e-3, "1e-3"), (0.3, "0.3")):
            p = os.path.join(tmp, "boxes10_noise%s.txt" % tag)
            workloads.write_input(p, obs, om)
            case("refgpu_N1000_boxes10_noise" + tag, 1000, p, 0.01, 2, full=False, roadmap=False,
                 bvp_from=g1000)
        g4000 = gpu_pairs(4000, os.path.join(diff_dir, "refgpu_bvp_diff_N4000.npz"),
                          tempfile.mkdtemp(dir=tmp))
        p = os.path.join(tmp, "indoor4000.txt")
        workloads.write_input(p, workloads.indoor(1000), 2e-3)
        case("refgpu_N4000_indoor_P1024", 4000, p, 0.01, 2, full=False, roadmap=False, P=1024,
             stride=9973, bvp_from=g4000)
        return
    if only == ["indoor4000"]:
        # the benchmark problem: N = 4000, indoor map (40 boxes), noise 2e-3,
        # 1024 HSMC particles (the reference built with numHSMCParticles = 1024:
        # bash oracle/build_ref.sh with PUMPREF_NUMS=4000:1024)
        p = os.path.join(tmp, "indoor4000.txt")
        workloads.write_input(p, workloads.indoor(1000), 2e-3)
        case("ref_N4000_indoor_P1024", 4000, p, 0.01, 2, full=False, roadmap=False, P=1024, stride=9973)
        return
    obs = workloads.random_boxes(10, 0)
    p_low = os.path.join(tmp, "boxes10_noise1e-3.txt")
    p_high = os.path.join(tmp, "boxes10_noise0.3.txt")
    workloads.write_input(p_low, obs, 1e-3)
    workloads.write_input(p_high, obs, 0.3)
    case("ref_N64_input", 64, REFERENCE_INPUT, 0.01, 2, full=True)
    case("ref_N1000_input", 1000, REFERENCE_INPUT, 0.01, 2, full=False)
    # same samples as the reference's input.txt case: roadmap arrays by hash only
    case("ref_N1000_boxes10_noise1e-3", 1000, p_low, 0.01, 2, full=False, roadmap=False)
    case("ref_N1000_boxes10_noise0.3", 1000, p_high, 0.01, 2, full=False, roadmap=False)


if __name__ == "__main__":
    main()
