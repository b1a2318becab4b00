"""CPU oracle for the Hermite4 hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, as the checker; the product library never does.
"""
