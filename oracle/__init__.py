"""CPU oracle for the batched forward-dynamics path (test infrastructure only).

Only tests/, the smoke check of __graft_entry__ and bench.py's CPU-baseline and
reference legs may import this package, and only as the checker or as the
timed CPU baseline -- never as the thing measured on the GPU or shipped.
"""
