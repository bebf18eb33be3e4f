"""CPU oracle for the GPU file-system path.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package, as the checker.  The product never imports it.
"""
