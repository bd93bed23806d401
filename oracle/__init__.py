"""CPU oracle of the PatchMatch hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this package, as the
checker or as the timed CPU baseline. See pm_oracle.h for the parity status.
"""
