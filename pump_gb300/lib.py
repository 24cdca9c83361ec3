"""ctypes binding of libpump (include/pump.h).

This is the harness-side view of the C ABI that tests and benchmarks call;
the library itself is C++/CUDA.  ``load()`` fails loudly when the compiled
library is missing: there is no Python or CPU fallback for any entry point.
Device buffers are passed as integer addresses (for example a torch CUDA
tensor's ``data_ptr()``) and streams as ``cudaStream_t`` handles (for torch,
``torch.cuda.current_stream().cuda_stream``).
"""
from __future__ import annotations

import ctypes as C
import os
import re
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libpump.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "pump.h")

PUMP_OK = 0
PUMP_ERR_BAD_INPUT = 1
PUMP_ERR_CAPACITY = 2
PUMP_ERR_TIMEOUT = 3
PUMP_ERR_CUDA = 4
PUMP_ERR_NO_SOLUTION = 5
PUMP_ERR_NO_MEMORY = 6
PUMP_BVP_PARITY = 0
PUMP_BVP_PRECISION = 1
PUMP_BVP_PARITY_GPU = 2

_lock = threading.Lock()
_lib = None

vp = C.c_void_p
i32 = C.c_int
i64 = C.c_longlong
f32 = C.c_float


class PumpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class Problem(C.Structure):
    _fields_ = [
        ("N", i32), ("num_disc", i32), ("num_hsmc", i32), ("num_mc", i32), ("table_rows", i32),
        ("num_obstacles", i32), ("obstacles", vp),
        ("init", f32 * 6), ("goal", f32 * 6), ("lo", f32 * 6), ("hi", f32 * 6),
        ("offset_mult", f32), ("cp_target", f32), ("cp_factor", f32), ("seed", C.c_uint64),
        ("bvp_mode", i32), ("samples", vp), ("refine_iters", i32), ("refine_lambda", f32),
        ("max_paths", i32), ("disc_len", f32), ("disc_min", i32),
    ]


class RefineArgs(C.Structure):
    _fields_ = [
        ("d_nodes", vp), ("n_nodes", i32), ("d_node_offset", vp), ("d_node_count", vp),
        ("n_paths", i32), ("d_lambda", vp), ("W", i32), ("tmax", f32), ("d_obstacles", vp),
        ("num_obstacles", i32), ("offset_mult", f32), ("d_pos_var", vp), ("T_rows", i32),
        ("dt", f32), ("sigma_floor", f32),
    ]


class PlanResult(C.Structure):
    _fields_ = [
        ("rn", f32), ("num_edges", i64), ("iterations", i32), ("num_paths", i32),
        ("num_considered", i32), ("goal_paths", i32), ("success", i32), ("soln_path_idx", i32),
        ("soln_cp", f32), ("soln_cost", f32), ("path_len", i32), ("path", vp), ("path_cap", i32),
        ("nodes", vp), ("nodes_cap", i32), ("num_nodes", i32),
        ("ms_roadmap", C.c_double), ("ms_online", C.c_double), ("ms_explore", C.c_double),
        ("ms_search", C.c_double), ("ms_total", C.c_double), ("wavefront_sizes", i32 * 32),
        ("wf_trace", vp), ("wf_trace_cap", i64), ("wf_trace_len", i64),
        ("h2d_bytes", i64), ("d2h_bytes", i64),
        ("ctrl_path", vp), ("ctrl_cap", i32), ("ctrl_len", i32),
        ("refine_cp", f32), ("refine_cost", f32), ("refined", i32),
        ("ms_explore_wait", C.c_double), ("ms_wait", C.c_double), ("num_waits", i32),
        ("path_time", vp), ("path_valid", vp), ("path_state_cap", i32),
    ]


_SIGS = {
    "pump_status_string": (C.c_char_p, [i32]),
    "pump_last_error": (C.c_char_p, []),
    "pump_version": (C.c_char_p, []),
    "pump_ctx_create": (i32, [i32, C.POINTER(vp)]),
    "pump_ctx_destroy": (i32, [vp]),
    "pump_bvp_pairs": (i32, [vp, i32, f32, i32, vp, vp, vp]),
    "pump_bvp_batch": (i32, [vp, vp, i32, f32, i32, vp, vp, vp]),
    "pump_select_kth": (i32, [vp, vp, i64, i64, C.POINTER(f32), vp]),
    "pump_build_edges": (i32, [vp, vp, vp, i32, f32, i64, vp, vp, vp, vp, vp, C.POINTER(i64), vp]),
    "pump_roadmap_edges": (i32, [vp, vp, vp, i32, i64, i64, vp, vp, vp, vp, vp, C.POINTER(f32),
                                 C.POINTER(i64), vp]),
    "pump_roadmap": (i32, [vp, vp, i32, f32, i32, i64, i64, vp, vp, vp, vp, vp, vp, vp,
                           C.POINTER(f32), C.POINTER(i64), vp, vp]),
    "pump_discretize_edges": (i32, [vp, vp, vp, vp, i64, i32, i32, vp, vp]),
    "pump_sample_free": (i32, [vp, i32, vp, i32, vp, vp]),
    "pump_free_edges": (i32, [vp, i32, vp, i64, i32, vp, vp]),
    "pump_cache_halfspaces": (i32, [vp, i32, vp, vp, i64, i32, i32, f32, vp, vp, vp, vp]),
    "pump_cache_halfspaces_sparse": (i32, [vp, i32, vp, vp, i64, i32, i32, f32, vp, vp, vp, vp]),
    "pump_particle_tables": (i32, [C.c_uint64, i32, i32, vp, vp, vp]),
    "pump_hsmc_propagate": (i32, [i32, i32, vp, vp, i64, i32, vp, vp, i32, vp, vp, f32, vp, i32,
                                  i32, f32, vp, i32, vp, vp, vp, vp]),
    "pump_hsmc_propagate_boxes": (i32, [i32, i32, vp, vp, i64, i32, vp, i32, vp, f32, i32, vp, vp,
                                        f32, vp, i32, i32, f32, vp, i32, vp, vp, vp]),
    "pump_tune_enable": (None, [i32]),
    "pump_search_graph": (None, [i32]),
    "pump_batch_groups": (None, [i32, i32]),
    "pump_tune_reset": (None, []),
    "pump_tune_report": (i32, [C.c_char_p, C.c_size_t]),
    "pump_mc_cp": (i32, [vp, vp, vp, i32, vp, i32, i32, f32, vp, i32, vp, vp, vp, vp]),
    "pump_frontier_compact": (i32, [vp, vp, i32, vp, vp, vp]),
    "pump_frontier_compact_noalloc": (i32, [vp, i32, vp, vp, vp]),
    "pump_selftest_wait": (i32, [vp, i64, vp]),
    "pump_halton_samples": (i32, [i32, vp, vp, vp, vp, vp, vp]),
    "pump_disc_offsets": (i32, [vp, vp, vp, i64, f32, i32, i32, vp, C.POINTER(i64), vp]),
    "pump_discretize_edges_off": (i32, [vp, vp, vp, vp, i64, vp, i32, i32, vp, vp]),
    "pump_free_edges_off": (i32, [vp, i32, vp, vp, i64, i32, vp, vp]),
    "pump_hsmc_propagate_boxes_off": (i32, [i32, i32, vp, vp, i64, i32, vp, i32, vp, vp, f32, i32, vp,
                                            vp, f32, vp, i32, i32, f32, vp, i32, vp, vp, vp]),
    "pump_problem_defaults": (None, [C.POINTER(Problem)]),
    "pump_read_input": (i32, [C.c_char_p, C.POINTER(Problem)]),
    "pump_plan": (i32, [vp, C.POINTER(Problem), C.POINTER(PlanResult), vp]),
    "pump_plan_batch": (i32, [i32, vp, vp, vp, i32, i32]),
    "pump_position_variance": (i32, [i32, vp, vp]),
    "pump_path_cp": (i32, [vp, vp, vp, vp, i32, i32, vp, i32, i32, f32, vp, i32, vp, vp, vp, vp]),
    "pump_refine_fwd": (i32, [C.POINTER(RefineArgs), vp, vp, vp, vp]),
    "pump_refine_bwd": (i32, [C.POINTER(RefineArgs), vp, vp, vp]),
    "pump_refine_paths": (i32, [vp, C.POINTER(RefineArgs), i32, vp, vp, vp]),
}


def header_functions(path=HEADER):
    """Names of the functions include/pump.h declares."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pump_[a-z0-9_]+)\s*\(", text)))


def load(path=LIB_PATH):
    """Loads libpump.so (built by ``pump_gb300.build.build()``)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError("libpump.so is not built (%s); run __graft_entry__.build()" % path)
            L = C.CDLL(path)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status):
    if status != PUMP_OK:
        L = load()
        raise PumpError(status, "%s: %s" % (L.pump_status_string(status).decode(),
                                             L.pump_last_error().decode()))
    return status


class Context:
    """Owns a pump_ctx on one device."""

    def __init__(self, device=0):
        self.lib = load()
        h = vp()
        check(self.lib.pump_ctx_create(device, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.pump_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
