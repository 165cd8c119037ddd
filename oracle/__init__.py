"""CPU oracle for the CheFSI hot path (test infrastructure; never imported by the product).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline use it.
"""
