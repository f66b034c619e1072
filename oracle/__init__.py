"""ORACLE -- test infrastructure only: the CPU checker for the GPU product.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package.  See grns_oracle.c for the C restatement of the
reference library and oracle.py for the Python access layer.
"""
