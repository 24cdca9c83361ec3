"""The drop-in command line and the failure paths, on the GPU.

The reference's `./pump <input> <cp> <eta>` writes path.txt and
discretizedPath.txt (PUMP.cu:553-594); the library's `pump` must write the
same bytes for the same input.  The reference's capacity cliffs (its
maxPathCount, PUMP.cu:62-76, and the particle table's horizon,
PUMP.cu:637-638) end a query with PUMP_ERR_CAPACITY here, and every bounded
device wait ends with PUMP_ERR_TIMEOUT and leaves the context usable.  No
test here faults or hangs the GPU: the failures are made on purpose with
small capacities and a wait on a word that nothing publishes.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from helpers import dev, empty, host, ptr, stream
from test_gpu_plan import make_problem, run_plan

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,flags", [("ref_N1000_input", []),
                                        ("ref_N1000_boxes10_noise0.3", []),
                                        ("refgpu_N1000_boxes10_noise1e-3", ["--gpu-arith"])])
def test_cli_writes_the_reference_files(name, flags, gpu, pumplib, goldens, tmp_path):
    """The command line on an input file holding the golden problem (written
    in the reference's format; every value parses back to the same binary32):
    path.txt and discretizedPath.txt byte for byte, and the printed solution
    line, as the reference wrote and printed them."""
    from pump_gb300 import workloads
    from pump_gb300.build import CLI
    g = goldens[name]
    inp = tmp_path / "input.txt"
    workloads.write_input(str(inp), g["prob_obstacles"], float(g["prob_offset_mult"]),
                          init=g["prob_init"], goal=g["prob_goal"], lo=g["prob_lo"], hi=g["prob_hi"])
    env = dict(os.environ, PUMP_NUM=str(int(g["N"])))
    r = subprocess.run([CLI, str(inp), "%g" % float(g["cp_target"]), "%g" % float(g["cp_factor"])] + flags,
                       cwd=tmp_path, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "discretizedPath.txt").read_text() == str(g["ctrl_txt"])
    if int(g["success"]):
        assert (tmp_path / "path.txt").read_text() == str(g["path_txt"])
        m = re.search(r"Solution path = (\d+) with cp = (\S+) and cost = (\S+)", r.stdout)
        assert m and int(m.group(1)) == int(g["soln_idx"])
        assert m.group(2) == "%g" % float(g["soln_cp_printed"])
        assert m.group(3) == "%g" % float(g["soln_cost_printed"])
    m = re.search(r"number of goal paths found = (\d+) with a total number of paths = (\d+) of (\d+)",
                  r.stdout)
    assert m and tuple(int(x) for x in m.groups()) == (int(g["goal_paths"]), int(g["num_paths"]),
                                                       int(g["num_considered"]))


def test_capacity_max_paths(gpu, pumplib, goldens):
    """The stored-path capacity (the reference's maxPathCount, which also
    sizes the wavefront): a cap below the paths the query stores ends it with
    PUMP_ERR_CAPACITY; a cap above every wavefront changes nothing."""
    torch, ctx = gpu
    g = goldens["ref_N1000_boxes10_noise1e-3"]
    L = pumplib.load()
    pb, _obs = make_problem(pumplib, g, max_paths=200)
    st, res, _p, _n = run_plan(pumplib, ctx, pb)
    assert st == pumplib.PUMP_ERR_CAPACITY
    assert b"maxPathCount 200" in L.pump_last_error()
    pb, _obs = make_problem(pumplib, g, max_paths=int(g["num_considered"]) + 64)
    st, res, path, nodes = run_plan(pumplib, ctx, pb)
    assert st == pumplib.PUMP_OK and res.num_paths == int(g["num_paths"])
    assert np.array_equal(nodes, g["soln_nodes"])


def test_capacity_particle_table_horizon(gpu, pumplib, goldens):
    """A particle table too short for the query's path times (1 s here) ends
    the query with PUMP_ERR_CAPACITY instead of reading past the table."""
    torch, ctx = gpu
    g = goldens["ref_N1000_boxes10_noise1e-3"]
    pb, _obs = make_problem(pumplib, g, table_rows=20)
    st, _res, _p, _n = run_plan(pumplib, ctx, pb)
    assert st == pumplib.PUMP_ERR_CAPACITY
    assert b"particle table" in pumplib.load().pump_last_error()


def test_bounded_wait_gives_up_and_context_stays_usable(gpu, pumplib):
    """The look-back wait on a status word that nothing publishes ends
    through its bound (PUMP_ERR_TIMEOUT), for a short and a longer bound;
    afterwards the same context and stream compute a compaction correctly."""
    torch, ctx = gpu
    L = pumplib.load()
    for limit in (0, 1000, 100_000):
        assert L.pump_selftest_wait(ctx.handle, limit, stream(torch)) == pumplib.PUMP_ERR_TIMEOUT
        assert b"gave up" in L.pump_last_error()
    assert L.pump_selftest_wait(ctx.handle, -1, stream(torch)) == pumplib.PUMP_ERR_BAD_INPUT
    rng = np.random.default_rng(9)
    N = 200_003
    flags = (rng.random(N) < 0.4).astype(np.uint8)
    d_f = dev(torch, flags)
    d_a, d_n = empty(torch, N, torch.int32), empty(torch, 1, torch.int32)
    pumplib.check(L.pump_frontier_compact(ctx.handle, ptr(d_f), N, ptr(d_a), ptr(d_n), stream(torch)))
    n = int(host(d_n)[0])
    assert n == int(flags.sum()) and np.array_equal(host(d_a, n), np.flatnonzero(flags).astype(np.int32))
