"""TEST INFRASTRUCTURE: the CPU FP64 oracle (checker) of the reference step.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference
arm import this package. The product package never does.
"""
