"""CPU oracle for the Feel++ assembly path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package: it is the checker and the timed CPU
baseline, never part of the product path.
"""
