"""The C ABI library without a GPU: it loads, exports every function
include/pump.h declares, rejects bad arguments before touching the device,
and reads the reference's input format like mainPUMP.cu:152-230."""
import ctypes as C
import os

import numpy as np


def test_exports_every_header_function(pumplib):
    L = pumplib.load()
    names = pumplib.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert missing == []
    assert b"sm_103a" in L.pump_version()


def test_status_strings(pumplib):
    L = pumplib.load()
    for s in range(7):
        assert L.pump_status_string(s)
    assert L.pump_status_string(99) == b"unknown status"


def test_bad_arguments_rejected_on_host(pumplib):
    L = pumplib.load()
    assert L.pump_bvp_pairs(None, 1, 5.0, 0, None, None, None) == pumplib.PUMP_ERR_BAD_INPUT
    assert L.pump_bvp_pairs(None, 10, 5.0, 7, None, None, None) == pumplib.PUMP_ERR_BAD_INPUT
    assert L.pump_free_edges(None, 3, None, 10, 8, None, None) == pumplib.PUMP_ERR_BAD_INPUT
    assert L.pump_hsmc_propagate(1, 9, None, None, 10, 0, None, None, 5, None, None, 0.05, None,
                                 2048, 400, 1.0, None, 128, None, None, None, None) == pumplib.PUMP_ERR_BAD_INPUT
    assert L.pump_select_kth(None, None, 10, 3, None, None) == pumplib.PUMP_ERR_BAD_INPUT
    assert L.pump_plan(None, None, None, None) == pumplib.PUMP_ERR_BAD_INPUT
    assert b"pump_plan" in L.pump_last_error()


def test_defaults_match_reference(pumplib):
    L = pumplib.load()
    pb = pumplib.Problem()
    L.pump_problem_defaults(C.byref(pb))
    # mainPUMP.cu:51-72, hardCoded.cuh:12-13, obstacles.cu:3-10
    assert (pb.N, pb.num_disc, pb.num_hsmc, pb.num_mc) == (1000, 8, 128, 2048)
    assert np.float32(pb.offset_mult) == np.float32(0.5)
    assert list(pb.lo) == [0.0, 0.0, np.float32(0.01), -1.0, -1.0, -0.5]
    obs = np.ctypeslib.as_array(C.cast(pb.obstacles, C.POINTER(C.c_float)), (pb.num_obstacles * 12,))
    assert pb.num_obstacles == 3 and np.float32(obs[6]) == np.float32(0.45)


def test_read_input_format(pumplib, tmp_path):
    from pump_gb300 import workloads
    L = pumplib.load()
    obs = workloads.random_boxes(7, 3)
    p = tmp_path / "problem.txt"
    workloads.write_input(str(p), obs, 2e-3)
    with open(p, "a") as f:
        f.write("\ntrailing text is not read\n")
    pb = pumplib.Problem()
    L.pump_problem_defaults(C.byref(pb))
    assert L.pump_read_input(str(p).encode(), C.byref(pb)) == 0
    assert pb.num_obstacles == 7
    got = np.ctypeslib.as_array(C.cast(pb.obstacles, C.POINTER(C.c_float)), (7 * 12,)).reshape(7, 12)
    assert np.array_equal(got, obs)
    assert np.float32(pb.offset_mult) == np.float32(2e-3)
    assert list(pb.init) == [np.float32(x) for x in workloads.INIT]
    assert L.pump_read_input(b"/nonexistent/file.txt", C.byref(pb)) == pumplib.PUMP_ERR_BAD_INPUT


def test_cli_usage_message(pumplib):
    import subprocess
    from pump_gb300.build import CLI
    assert os.path.exists(CLI)
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode != 0 and "Must specify an online setting filename" in r.stdout
