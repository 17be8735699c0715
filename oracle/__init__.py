"""CPU oracle of the DG residual path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` import this package, and only as the
reference results / the timed CPU baseline.  It builds every problem with its own set-up code (oracle_setup.c) and never
imports or loads the library under test; the library's residual path never calls it.
"""
from .oracle_py import Oracle, Problem, build_oracle, load_oracle, nodes, ORACLE_LIB  # noqa: F401
