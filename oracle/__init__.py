"""ORACLE: CPU restatement of the reference SymX second-order path (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this
package, and only as the checker; the product package never imports it.
"""
