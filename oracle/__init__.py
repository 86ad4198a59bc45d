"""CPU FP64 oracle for the TwoPIScalar Kadanoff-Baym step (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may use
this package; the product (libkb2pi and its Python host mirror) never does.
"""
from .pyoracle import Oracle, OracleParams, build_oracle, ENGINE_FULL, ENGINE_ORBIT, ENGINE_OCTANT  # noqa: F401
from .pyoracle import PEXP_LO, PEXP_NLO_QUANTUM, PEXP_NLO_CLASSICAL, PEXP_NINV_LO, PEXP_NINV_NLO  # noqa: F401
