"""CPU oracle for parity tests — test infrastructure, not part of the product.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
