"""CPU FP64 oracle for the topology-optimisation hot path (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this package.  It restates the reference operators (see topo_oracle.cpp for the
file:line citations) and is never used by the product library.
"""
from .oracle import Oracle, build_oracle, ORACLE_LIB  # noqa: F401
