"""CPU oracle of the reference MLS-MPM substep. TEST INFRASTRUCTURE ONLY.

Imported by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of bench.py, always as the
checker or as the timed CPU baseline; the product package never imports it.
"""
