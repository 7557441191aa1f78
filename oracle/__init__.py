"""Oracle (test infrastructure only): CPU restatement of the reference path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
load this package.  The product (fastbact_gb300) never imports it.
"""
