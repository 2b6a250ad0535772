"""ORACLE — test infrastructure, not part of the product.

CPU restatements of the reference algorithms on the hot path, used only by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
checker.  The product (fluxpy_gb300) never imports this package.
"""
