"""FP64 CPU oracle for the qdyn hot path (test infrastructure only).

Loaded by the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg, never by the engine itself.
"""
