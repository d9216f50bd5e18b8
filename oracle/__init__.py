"""CPU oracle for the RBF-FD hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, always as the checker.  The product library never imports it.
"""
