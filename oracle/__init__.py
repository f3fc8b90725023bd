"""CPU oracle for the TwoChNRG iteration (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, as the checker; the product path never imports it.
"""
