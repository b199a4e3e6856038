"""Test oracle: a CPU restatement of the reference RK-DG method.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package, as the reference for results (and the timed CPU baseline); the product never
imports it.
"""
