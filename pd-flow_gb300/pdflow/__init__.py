"""Python view of the GB300-native PD-Flow scene-flow solver.

The compute path is the CUDA library libpdflow_gb300.so (sm_103a) behind the
C ABI of include/pdflow.h; this package binds it with ctypes and adds the
seeded synthetic scene generator used by the tests and the benchmark.
"""
from ._lib import (BatchSolver, ERR_ARG, ERR_CUDA, ERR_NO_DEVICE, ERR_OOM, ERR_STATE, ERR_TIMEOUT, OK, ExtensionMissing,
                   MixedBatch, Net, Params, PD_flow, PDFlowError, Solver, default_params, device_to_host, exported_symbols,
                   gemm_bf16, library_path, load, load_weights, render_frames)

__all__ = ["Solver", "BatchSolver", "MixedBatch", "Net", "PD_flow", "Params", "PDFlowError", "ExtensionMissing", "default_params",
           "load", "library_path", "exported_symbols", "gemm_bf16", "device_to_host", "render_frames", "load_weights", "OK", "ERR_ARG", "ERR_OOM",
           "ERR_CUDA", "ERR_STATE", "ERR_TIMEOUT", "ERR_NO_DEVICE"]
