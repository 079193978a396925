"""CPU restatement of the reference algorithm (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, as the checker.  The shipped library never
imports it.
"""
