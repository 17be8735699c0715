"""CPU oracle of the DG residual path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of ``bench.py`` import this package, and
only as the checker / the timed CPU baseline.  The library's residual path never calls it.
"""
from .oracle_py import Oracle, load_oracle, ORACLE_LIB  # noqa: F401
