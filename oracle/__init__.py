"""CPU oracle for the GPU local push solvers (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this package, as the checker and as the timed CPU baseline.  The
product (``faster-local-solver-for-gdes_gb300/``) never imports it.
"""
