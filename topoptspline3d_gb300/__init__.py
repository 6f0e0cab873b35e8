"""GB300-native topology-optimisation hot path (spline density, multigrid
elasticity solve, sensitivity filter, OC update) behind a C ABI.

The compute path is ``libtopo_gb300.so`` (hand-written CUDA for sm_103a); this
package builds and loads it and exposes a thin ctypes front end.
"""
from .capi import Problem, TopoError, load, lib_path  # noqa: F401
from . import workloads  # noqa: F401

__all__ = ["Problem", "TopoError", "load", "lib_path", "workloads"]
