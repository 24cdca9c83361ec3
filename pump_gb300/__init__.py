"""pump_gb300: GB300-native (sm_103a) PUMP planner hot path.

The product is the C ABI in include/pump.h implemented by CUDA kernels and a
C++ host runtime (``pump_gb300/csrc``), built by ``pump_gb300.build`` into
``pump_gb300/_build``: ``libpump.so`` and the ``pump`` command-line program.
``pump_gb300.lib`` is the ctypes view of that ABI used by tests and
benchmarks.
"""
