"""FP64 CPU oracle for the MGBF filtering pipeline -- test infrastructure only.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg.  Parity with the reference is unpinned: see mgbf_oracle.h.
"""
