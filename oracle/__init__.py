"""TEST INFRASTRUCTURE: the CPU oracle and the reference emulator.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.  The GPU library never does.
"""
