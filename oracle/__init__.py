"""The oracle: CPU restatements of the reference's SOCS path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this package;
the product never does.
"""
