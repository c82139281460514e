"""CPU oracle for the GB300 Apriori engine: test infrastructure, never on the product path.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this package. ``miner`` restates ET-Miner's CPU mining route in numpy; the
timed CPU baseline runs its per-candidate counting over all host cores in
spawned processes.
"""
