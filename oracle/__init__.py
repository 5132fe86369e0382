"""ORACLE — test infrastructure only (CPU restatements of the reference).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this package; the product (cudadecon_gb300) never does.
"""
