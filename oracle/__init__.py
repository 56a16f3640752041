"""CPU oracle for the RTM hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product package rtm_gpu_gb300 never does.
"""
