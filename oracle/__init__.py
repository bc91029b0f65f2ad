"""FP64 CPU oracle of the SIMP hot path (test infrastructure only).

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py``: it is the checker, never part of the product path.
"""
